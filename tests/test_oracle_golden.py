"""The CPU oracle against the golden vectors produced by the reference's own code
(tests/golden/make_golden.py).  These pins are what lets the GPU tests trust the oracle."""
import numpy as np
import pytest

from conftest import load_golden


def test_scaled_jacobian_matches_reference(oracle):
    z = load_golden("scaled_jacobian")
    r = oracle.scaled_jacobian(z["V"], z["H"])
    np.testing.assert_allclose(r["V_Js"], z["V_Js"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(r["H_Js"], z["H_Js"], rtol=0, atol=1e-14)
    assert np.array_equal(r["H_Js"] < 0, z["H_Js"] < 0)           # inversion flags, bit-exact
    assert r["inverted"] == int(z["stats"][3]) > 0
    np.testing.assert_allclose([r["min"], r["ave"], r["dev"]], z["stats"][:3], rtol=1e-13)


@pytest.mark.parametrize("cube", [1, 0])
def test_reference_shapes_and_gradient_operator(oracle, cube):
    z = load_golden(f"grad_ref_cube{cube}")
    RT, Dg = oracle.grad_ref(z["V"], z["H"], z["h_flag"], cube)
    np.testing.assert_allclose(RT, z["RT"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(Dg, z["Dg"], rtol=1e-12, atol=1e-12)


def test_closed_form_of_the_cube_gradient_operator(oracle):
    """For cube-target hexes J_t = E_t R_k^-1 / cbrt(6 vol_t) (unit cube-corner edges R_k)."""
    z = load_golden("grad_ref_cube1")
    V, H = z["V"], z["H"].astype(np.int64)
    T = np.array([[0, 3, 4, 1], [1, 0, 5, 2], [2, 1, 6, 3], [3, 2, 7, 0],
                  [4, 7, 5, 0], [5, 4, 6, 1], [6, 5, 7, 2], [7, 6, 4, 3]])
    ref = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    X = V + np.random.default_rng(0).normal(0, 0.01, V.shape)
    Dg = z["Dg"]
    for h in np.nonzero(z["h_flag"])[0][:20]:
        for k in range(8):
            t = 8 * h + k
            P = V[H[h, T[k]]]
            E0 = (P[1:] - P[0]).T
            Rk = (ref[T[k, 1:]] - ref[T[k, 0]]).T
            s = np.cbrt(np.linalg.det(E0))
            Q = X[H[h, T[k]]]
            J_closed = (Q[1:] - Q[0]).T @ np.linalg.inv(Rk) / s
            J_op = Q.T @ Dg[t]
            np.testing.assert_allclose(J_op, J_closed, rtol=1e-11, atol=1e-11)


def test_tet_energy_matches_reference(oracle):
    z = load_golden("tet_energy")
    prob = oracle.SlimProblem(z["V"], z["H"])
    _, Et, _, _ = oracle.slim_energy(prob, z["X"])
    np.testing.assert_allclose(Et, z["E_tet"], rtol=1e-12)


def test_flip_avoiding_step_bound_matches_reference(oracle):
    z = load_golden("max_step")
    assert oracle.max_step(z["V"], z["D"], z["H"]) == pytest.approx(float(z["max_step"][0]), rel=1e-12)


def _problem(oracle, z):
    return oracle.SlimProblem(z["V"], z["H"], h_flag=z.get("h_flag"), energy=int(z.get("energy", 2)),
                              cube=bool(int(z.get("cube", 1))), weight_opt=float(z.get("weight_opt", 0.001)),
                              exp_factor=1.0, ids_C=z["ids_C"], C_=z["C_"],
                              lamda_C=float(z["lamda_C"]), ids_T=z["ids_T"], normal_T=z["normal_T"],
                              dis_T=z["dis_T"], lamda_T=float(z["lamda_T"]), ids_L=z["ids_L"], Axa_L=z["Axa_L"],
                              origin_L=z["origin_L"], lamda_L=float(z["lamda_L"]))


@pytest.mark.parametrize("name", ["slim_fa_1", "slim_fa_3", "slim_fa_strong", "slim_fa_hflag", "slim_cube0"])
def test_slim_m_opt_matches_reference(oracle, name):
    z = load_golden(name)
    Vo, aL, info = oracle.slim_m_opt(_problem(oracle, z), int(z["iters"]))
    diag = np.linalg.norm(z["V"].max(0) - z["V"].min(0))
    assert np.abs(Vo - z["V_o"]).max() <= 1e-12 * diag
    np.testing.assert_allclose([info["energy"], info["energy_quality"], info["energy_soft"]], z["out"], rtol=1e-11)


@pytest.mark.parametrize("energy", range(6))
def test_slim_energies_match_reference(oracle, energy):
    """ARAP, LOG_ARAP, SYMMETRIC_DIRICHLET, CONFORMAL, EXP_CONFORMAL, EXP_SYMMETRIC_DIRICHLET: the
    weights and energies of update_weights_and_closest_rotations / compute_energy_with_jacobians
    (slim_m.cpp:260-350, 868-913).  slim_precompute resets SLIMData::exp_factor to 1
    (slim_m.cpp:1125), so the exponential energies run with factor 1."""
    z = load_golden(f"slim_energy_{energy}")
    Vo, aL, info = oracle.slim_m_opt(_problem(oracle, z), int(z["iters"]))
    diag = np.linalg.norm(z["V"].max(0) - z["V"].min(0))
    assert np.abs(Vo - z["V_o"]).max() <= 1e-11 * diag
    np.testing.assert_allclose([info["energy"], info["energy_quality"], info["energy_soft"]], z["out"], rtol=1e-10)


def test_projection_term_matches_reference(oracle):
    """Tetralize_Set::projection: lamda_projection |x_b - bc|^2 (slim_m.cpp:600-610, 740-745)."""
    z = load_golden("slim_projection")
    prob = oracle.SlimProblem(z["V"], z["H"], weight_opt=float(z["weight_opt"]), b=z["b"], bc=z["bc"],
                              lamda_projection=float(z["lamda_projection"]))
    Vo, aL, info = oracle.slim_m_opt(prob, int(z["iters"]))
    diag = np.linalg.norm(z["V"].max(0) - z["V"].min(0))
    assert np.abs(Vo - z["V_o"]).max() <= 1e-11 * diag
    np.testing.assert_allclose([info["energy"], info["energy_quality"], info["energy_soft"]], z["out"], rtol=1e-10)


@pytest.mark.parametrize("name", ["signed_distance", "signed_distance_cyl"])
def test_signed_distance_pseudonormal_matches_reference(oracle, name):
    z = load_golden(name)
    S, I, Cc, N = oracle.signed_distance(z["TV"], z["TF"], z["P"])
    np.testing.assert_allclose(S, z["S"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(Cc, z["C"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(N, z["N"], rtol=0, atol=1e-13)


def test_hausdorff_matches_reference(oracle):
    z = load_golden("hausdorff")
    np.testing.assert_allclose(oracle.hausdorff(z["V0"], z["F0"], z["V1"], z["F1"]), z["out"], rtol=1e-13)
    np.testing.assert_allclose(oracle.hausdorff(z["V0"], z["F0"], z["BV"], z["BF"]), z["out_b"], rtol=1e-13)


def test_known_answers(oracle):
    """Hand-derivable cases: a regular grid has SJ = 1 and SD energy 6 per tet, and SLIM leaves
    it in place; a corner tet scaled by s keeps J = I; a mesh is at Hausdorff distance 0 from
    itself; point-triangle distances in face / edge / vertex regions."""
    from hexopt import meshgen
    V, H = meshgen.grid_hex(3)
    r = oracle.scaled_jacobian(V, H)
    assert np.allclose(r["V_Js"], 1.0) and r["inverted"] == 0
    prob = oracle.SlimProblem(V, H, weight_opt=1.0)
    tot, Et, _, _ = oracle.slim_energy(prob, V)
    assert np.allclose(Et, 6.0)
    Vo, _, info = oracle.slim_m_opt(prob, 1)
    assert np.abs(Vo - V).max() < 1e-12
    _, Dg = oracle.grad_ref(V * 7.0, H)
    J = np.einsum("tjb,tjc->tbc", (V * 7.0)[H.astype(np.int64)[:, [0, 3, 4, 1]]].repeat(8, 0)[:8], Dg[:8])
    assert np.allclose(J[0], np.eye(3))
    CV, CF, _ = meshgen.cylinder_surface()
    assert oracle.hausdorff(CV, CF, CV, CF)[1] == 0.0
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float)
    F = np.array([[0, 1, 2]], np.int32)
    P = np.array([[0.2, 0.2, 0.5], [0.5, -0.3, 0.0], [-0.3, -0.4, 0.0]])
    S, I, Cc, N = oracle.signed_distance(tri, F, P)
    np.testing.assert_allclose(np.abs(S), [0.5, 0.3, 0.5], atol=1e-15)
    d = oracle.point_face_distance(P, tri, F)
    np.testing.assert_allclose(d, [0.5, 0.3, 0.5], atol=1e-15)
