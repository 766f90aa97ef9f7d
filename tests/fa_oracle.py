"""Oracle-side feature-alignment loop body (grid_hex_meshing.cpp:3855-3869) composed from the
CPU oracle: projection (signed_distance_pseudonormal + curve point_line_projection), one
slim_m_opt iteration and the weight schedule.  TEST INFRASTRUCTURE ONLY."""
import numpy as np

import oracle_py as O


def curve_targets(TV, curves, closed, lines, line_curve, V):
    """dirty_graph_projection LINE branch (grid_hex_meshing.cpp:3963-4025)."""
    origin = np.zeros((len(lines), 3))
    axis = np.zeros((len(lines), 3))
    for i, (v, c) in enumerate(zip(lines, line_curve)):
        curve = curves[c]
        n = len(curve)
        ln = n if closed[c] else n - 1
        best = None
        for j in range(ln):
            a, b = TV[curve[j]], TV[curve[(j + 1) % n]]
            pv, _ = O.point_line_projection(a, b, V[v])
            d = np.linalg.norm(V[v] - pv)
            if best is None or d < best[0]:
                t = (b - a) / np.linalg.norm(b - a)
                best = (d, pv, t)
        origin[i], axis[i] = best[1], best[2]
    return origin, axis


def fa_steps(p, iters, lamda0=0.05, weight_opt=0.001):
    V = p["V"].copy()
    lam = lamda0
    info = None
    for _ in range(iters):
        S, I, Cc, N = O.signed_distance(p["TV"], p["TF"], V[p["regular"]])
        dis = (N * Cc).sum(1)
        if len(p["lines"]):
            org, ax = curve_targets(p["TV"], p["curves"], p["closed"], p["lines"], p["line_curve"], V)
        else:
            org = ax = np.zeros((0, 3))
        prob = O.SlimProblem(V, p["H"], ids_T=p["regular"], normal_T=N, dis_T=dis, lamda_T=lam,
                             ids_L=p["lines"], Axa_L=ax, origin_L=org, lamda_L=lam, lamda_C=lam,
                             weight_opt=weight_opt)
        V, aL, info = O.slim_m_opt(prob, 1)
        lam = min(lamda0 * max(info["energy_quality"] / info["energy_soft"] * lam, 1.0), 1e16)
    return V, info, lam
