"""The seeded workload generators (CPU only): the cube-minus-cylinder feature workload's mesh,
target surface and feature sets, and one oracle feature-alignment iteration on a small copy."""
import numpy as np


def test_cube_minus_cylinder_mesh_and_features():
    from hexopt import meshgen, workloads
    import oracle_py as O
    p = workloads.cube_minus_cylinder()
    V, H = p["V"], p["H"]
    assert H.shape == (262_144, 8)
    # every corner tet of the unjittered mesh is positively oriented
    V0, H0, sets = meshgen.cube_minus_cylinder_hex()
    q = O.scaled_jacobian(V0, H0)
    assert q["min"] > 0.7 and q["inverted"] == 0
    # boundary vertices are not jittered; the jitter of the others is within 0.1 h
    b = sets["boundary"]
    assert np.array_equal(V[b], V0[b])
    assert np.abs(V[~b] - V0[~b]).max() <= 0.1 / 64 + 1e-15
    # 8 corners at the cube corners, line vertices on their curves' lines
    assert np.array_equal(np.sort(V[p["corners"]], 0), np.sort(p["corner_pos"], 0))
    assert set(np.unique(p["line_curve"])) == set(range(14))
    TV, curves = p["TV"], p["curves"]
    for v, c in zip(p["lines"], p["line_curve"]):
        x = V[v]
        if c < 12:  # a cube edge: two coordinates in {0, 1}
            assert np.sum(np.isclose(x, 0) | np.isclose(x, 1)) >= 2
        else:      # a hole circle at z = 0 or 1
            assert abs(np.hypot(x[0] - 0.5, x[1] - 0.5) - 0.25) < 1e-12 and x[2] in (0.0, 1.0)
    # regular vertices: boundary minus lines and corners
    assert len(p["regular"]) + len(p["lines"]) + len(p["corners"]) == int(b.sum())
    # the target is a closed 2-manifold: every edge is shared by exactly two triangles
    F = p["TF"]
    E = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), 1)
    _, cnt = np.unique(E, axis=0, return_counts=True)
    assert len(F) == 23_040 and np.all(cnt == 2)
    # the curves run along the target's edges: consecutive curve vertices share a triangle edge
    ekeys = set(map(tuple, E.tolist()))
    for c, closed in zip(curves, p["closed"]):
        n = len(c) if closed else len(c) - 1
        for j in range(n):
            a, b2 = int(c[j]), int(c[(j + 1) % len(c)])
            assert (min(a, b2), max(a, b2)) in ekeys


def test_cube_minus_cylinder_oracle_iteration_lowers_the_energy():
    import fa_oracle
    import oracle_py as O
    from hexopt import workloads
    p = workloads.cube_minus_cylinder(n=12, n_r=4, n_z=12)
    V1, info, lam = fa_oracle.fa_steps(p, 1)
    prob = O.SlimProblem(p["V"], p["H"], weight_opt=0.001)
    e0 = O.slim_energy(prob, p["V"])[2]
    e1 = O.slim_energy(prob, V1)[2]
    assert e1 < e0 and info["step"] > 0 and lam > 0.05
