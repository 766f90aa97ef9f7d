"""Oracle-side feature-alignment loop body (grid_hex_meshing.cpp:3855-3869) composed from the
CPU oracle: projection (signed_distance_pseudonormal of the regular vertices, the curve
point_line_projection of the line vertices, corner vertices tied to their target corners), one
slim_m_opt iteration and the weight schedule.  TEST INFRASTRUCTURE ONLY."""
import numpy as np

import oracle_py as O


def curve_targets(TV, curves, closed, lines, line_curve, V):
    """dirty_graph_projection LINE branch (grid_hex_meshing.cpp:3963-4025)."""
    return O.curve_targets(V, lines, line_curve, TV, curves, closed)


def fa_steps(p, iters, lamda0=0.05, weight_opt=0.001):
    V = p["V"].copy()
    lam = lamda0
    info = None
    corners = p.get("corners", np.zeros(0, np.int32))
    cpos = p.get("corner_pos", np.zeros((0, 3))) if len(corners) else np.zeros((0, 3))
    for _ in range(iters):
        S, I, Cc, N = O.signed_distance(p["TV"], p["TF"], V[p["regular"]])
        dis = (N * Cc).sum(1)
        if len(p["lines"]):
            org, ax = curve_targets(p["TV"], p["curves"], p["closed"], p["lines"], p["line_curve"], V)
        else:
            org = ax = np.zeros((0, 3))
        prob = O.SlimProblem(V, p["H"], ids_T=p["regular"], normal_T=N, dis_T=dis, lamda_T=lam,
                             ids_L=p["lines"], Axa_L=ax, origin_L=org, lamda_L=lam,
                             ids_C=corners, C_=cpos, lamda_C=lam, weight_opt=weight_opt)
        V, aL, info = O.slim_m_opt(prob, 1)
        lam = min(lamda0 * max(info["energy_quality"] / info["energy_soft"] * lam, 1.0), 1e16)
    return V, info, lam
