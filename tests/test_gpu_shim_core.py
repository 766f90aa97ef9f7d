"""The drop-in shim's conversions run against the library: hexopt_shim_core.h, which
hexopt_reference_shim.cpp calls with the plain arrays of SLIMData / Tetralize_Set, compiled here
into a small harness (tests/shim_core_harness.cpp) and fed what the shim would build:

- the 8-tets-per-hex list of slim_m_opt's callers (hexes recovered from it; a malformed list is
  refused);
- the reference tets ts.RT as compute_referenceMesh writes them -- cubes and own-shape hexes
  (h_flag), and edge-averaged cuboids (cube = false) -- against the reference's slim_m_opt;
- a start V_init other than V (the operator at V, the iterations from V_init) against the oracle;
- the gluing solve of glueInternalNodes: per-hex copies glued by V_ranges, boundary copies held
  by known_value_post, the adaptive slim_solve2 branch, CONFORMAL energy -- against the
  reference's own pipeline2 (the glued positions are the means of each vertex's copies).
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG, ROOT, load_golden

pytestmark = pytest.mark.gpu

HEX_TETRA = np.array([[0, 3, 4, 1], [1, 0, 5, 2], [2, 1, 6, 3], [3, 2, 7, 0],
                      [4, 7, 5, 0], [5, 4, 6, 1], [6, 5, 7, 2], [7, 6, 4, 3]])
_d = C.POINTER(C.c_double)
_i32 = C.POINTER(C.c_int32)
_u32 = C.POINTER(C.c_uint32)


def p(a, t):
    return None if a is None else a.ctypes.data_as(t)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    import build
    lib = build.build()
    out = str(tmp_path_factory.mktemp("shim_core") / "libshimcore.so")
    libdir = os.path.dirname(lib)
    cmd = ["g++", "-std=c++17", "-O2", "-shared", "-fPIC", f"-I{os.path.join(ROOT, 'include')}",
           f"-I{os.path.join(PKG, 'shim')}", os.path.join(ROOT, "tests", "shim_core_harness.cpp"),
           f"-L{libdir}", "-lhexopt_gpu", f"-Wl,-rpath,{libdir}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    L = C.CDLL(out)
    L.harness_slim.argtypes = [C.c_int64, _d, _d, C.c_int64, _i32, _d, C.c_int, C.c_double, C.c_int,
                               C.c_int64, _i32, _d, C.c_double, C.c_int64, _i32, _d, _d, C.c_double,
                               C.c_int64, _i32, _d, _d, C.c_double, C.c_int, _d, _d, C.c_char_p, C.c_int]
    L.harness_glue.argtypes = [C.c_int64, _d, C.c_int64, _i32, _d, C.c_int64, _u32, C.c_int64, _d, C.c_double,
                               C.c_int, C.c_double, C.c_int, _d, _i32, _d, C.c_char_p, C.c_int]
    L.harness_hexes_from_tets.argtypes = [_i32, C.c_int64, _u32]
    return L


def tets_of(H):
    return np.ascontiguousarray(H.astype(np.int32)[:, HEX_TETRA].reshape(-1, 4))


def diag_of(V):
    return float(np.linalg.norm(V.max(0) - V.min(0)))


def run_slim(L, V, H, RT, z, iters, weight_opt, V_o=None, energy=2):
    T = tets_of(H)
    e3 = np.zeros((0, 3))
    ei = np.zeros(0, np.int32)
    g = lambda k, d: np.ascontiguousarray(z.get(k, d))
    ids_C, C_, ids_T, nT_, dT, ids_L, aL, oL = (g("ids_C", ei).astype(np.int32), g("C_", e3), g("ids_T", ei).astype(np.int32),
                                              g("normal_T", e3), g("dis_T", np.zeros(0)), g("ids_L", ei).astype(np.int32),
                                              g("Axa_L", e3), g("origin_L", e3))
    out = np.empty_like(V)
    o3 = np.empty(3)
    err = C.create_string_buffer(512)
    Vc = np.ascontiguousarray(V)
    Vo = Vc if V_o is None else np.ascontiguousarray(V_o)
    R = None if RT is None else np.ascontiguousarray(RT)
    rc = L.harness_slim(len(V), p(Vc, _d), p(Vo, _d), len(T), p(T, _i32), p(R, _d), energy, weight_opt, 0,
                        len(ids_C), p(ids_C, _i32), p(C_, _d), float(z.get("lamda_C", 0.0)),
                        len(ids_T), p(ids_T, _i32), p(nT_, _d), p(dT, _d), float(z.get("lamda_T", 0.0)),
                        len(ids_L), p(ids_L, _i32), p(aL, _d), p(oL, _d), float(z.get("lamda_L", 0.0)),
                        iters, p(out, _d), p(o3, _d), err, len(err))
    assert rc == 0, err.value.decode()
    return out, o3


def test_hexes_from_tets_and_malformed_lists(harness):
    from hexopt import meshgen
    V, H = meshgen.grid_hex(3)
    T = tets_of(H)
    Hb = np.empty_like(H)
    assert harness.harness_hexes_from_tets(p(T, _i32), len(T), p(Hb, _u32)) == 0
    assert np.array_equal(Hb, H)
    T2 = T.copy()
    T2[5, 2] += 1
    assert harness.harness_hexes_from_tets(p(T2, _i32), len(T2), p(Hb, _u32)) != 0


@pytest.mark.parametrize("name,cube", [("slim_fa_hflag", 1), ("slim_cube0", 0)])
def test_reference_tets_match_reference(harness, oracle, name, cube):
    """ts.RT handed over as the reference builds it: cube and own-shape hexes (h_flag), or
    edge-averaged cuboids, against the reference's slim_m_opt on the same tets."""
    z = load_golden(name)
    RT, _ = oracle.grad_ref(z["V"], z["H"], z.get("h_flag"), cube)
    w = float(z.get("weight_opt", 0.001))
    Vg, o3 = run_slim(harness, z["V"], z["H"], RT, z, int(z["iters"]), w)
    err = np.abs(Vg - z["V_o"]).max() / diag_of(z["V"])
    assert err <= 1e-6, err
    np.testing.assert_allclose(o3[:2], z["out"][:2], rtol=1e-6)


def test_start_other_than_v(harness, oracle):
    """slim_precompute(V, F, V_init, ...) with V_init != V: the operator at V, the iterations from
    V_init (as the oracle's SlimProblem UV)."""
    z = load_golden("slim_fa_1")
    rng = np.random.default_rng(3)
    Vi = z["V"] + rng.normal(0, 0.01, z["V"].shape)
    RT, _ = oracle.grad_ref(z["V"], z["H"], None, 1)
    Vg, o3 = run_slim(harness, z["V"], z["H"], RT, z, 1, 0.001, V_o=Vi)
    prob = oracle.SlimProblem(z["V"], z["H"], UV=Vi, ids_C=z["ids_C"], C_=z["C_"], lamda_C=float(z["lamda_C"]),
                              ids_T=z["ids_T"], normal_T=z["normal_T"], dis_T=z["dis_T"], lamda_T=float(z["lamda_T"]),
                              ids_L=z["ids_L"], Axa_L=z["Axa_L"], origin_L=z["origin_L"], lamda_L=float(z["lamda_L"]))
    Vo, _, info = oracle.slim_m_opt(prob, 1)
    assert np.abs(Vg - Vo).max() <= 1e-6 * diag_of(z["V"])
    assert o3[0] == pytest.approx(info["energy"], rel=1e-6)


def rigid_cubes(BV, H, boundary):
    """rigidDeformCubes (optimization.cpp:456-494): each hex with no boundary corner becomes the
    unit cube Procrustes-fitted (scaling, no reflection) to its corners; the others keep them."""
    ref = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], float)
    out = BV[H.astype(np.int64)].copy()
    for h in range(len(H)):
        if boundary[H[h]].any():
            continue
        Y = out[h]
        Xc, Yc = ref - ref.mean(0), Y - Y.mean(0)
        s = (np.linalg.norm(Yc) / 8) / (np.linalg.norm(Xc) / 8)
        U, S, Vt = np.linalg.svd((Xc * s).T @ Yc)
        R = U @ Vt
        if np.linalg.det(R) < 0:
            Vt[-1] *= -1
            R = U @ Vt
        t = Y.mean(0) - s * R.T @ ref.mean(0)
        out[h] = s * ref @ R + t
    return out


@pytest.mark.parametrize("name", ["untangle_a", "untangle_b", "untangle_box"])
def test_glue_setup_matches_reference_pipeline2(harness, oracle, name):
    z = load_golden(name)
    BV, H, bnd = z["V"], z["H"].astype(np.int64), z["boundary"].astype(bool)
    nv = len(BV)
    cubes = rigid_cubes(BV, H, bnd)
    # copies numbered vertex by vertex, interior vertices first (glueInternalNodes' mappedV order)
    order = np.concatenate([np.nonzero(~bnd)[0], np.nonzero(bnd)[0]])
    counts = np.bincount(H.ravel(), minlength=nv)
    start = np.zeros(nv, np.int64)
    start[order] = np.concatenate([[0], np.cumsum(counts[order])[:-1]])
    fill = start.copy()
    copy_of = np.empty(H.shape, np.int64)
    for h in range(len(H)):
        for c in range(8):
            v = H[h, c]
            copy_of[h, c] = fill[v]
            fill[v] += 1
    nc = 8 * len(H)
    Vc = np.empty((nc, 3))
    Vc[copy_of.ravel()] = cubes.reshape(-1, 3)
    V_ranges = np.ascontiguousarray((np.cumsum(counts[order]) - 1).astype(np.uint32))
    post_index = int(counts[~bnd].sum())
    T = tets_of(copy_of)
    RT, _ = oracle.grad_ref(BV, H, None, 0)  # compute_referenceMesh(BV, mesh.Hs, ..., false)
    RT = np.ascontiguousarray(RT)
    post = np.ascontiguousarray(Vc[post_index:])
    out = np.empty_like(Vc)
    it, mj = C.c_int32(), C.c_double()
    err = C.create_string_buffer(512)
    rc = harness.harness_glue(nc, p(Vc, _d), len(T), p(T, _i32), p(RT, _d), len(V_ranges), p(V_ranges, _u32),
                              post_index, p(post, _d), 1e4, 3, float(z["weight_opt"]), 50, p(out, _d), C.byref(it),
                              C.byref(mj), err, len(err))
    assert rc == 0, err.value.decode()
    glued = np.array([out[start[v]:start[v] + counts[v]].mean(0) for v in range(nv)])
    e = np.abs(glued - z["V_o"]).max() / diag_of(BV)
    print(f"\n[{name} via the shim's setup] max|dX|/diag {e:.3e}, {it.value} iterations, min J {mj.value:.6f}")
    assert e <= max(1e-6, 3 * float(z["spread"]))
