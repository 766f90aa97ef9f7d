"""Generate the golden fixtures that pin the oracle: seeded small inputs run through the
reference's OWN FP64 code (oracle/_ref/libhexopt_ref.so, built from the reference sources by
`make -C oracle ref`).  Run in a container that has the reference tree:

    make -C oracle ref && python tests/golden/make_golden.py [group ...]

Writes tests/golden/*.npz (every group when none is named; groups: base, energies, shapes,
untangle, smoothing, projection).  The
fixtures are committed; the reference build is not.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "feature-preserving-octree-hex-meshing_gb300"))

import oracle_py as O  # noqa: E402
from hexopt import meshgen  # noqa: E402

_d = C.POINTER(C.c_double)
_i32 = C.POINTER(C.c_int32)
_u32 = C.POINTER(C.c_uint32)
_u8 = C.POINTER(C.c_uint8)


def p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


def jittered_grid(n, sigma, seed, inverted=0):
    V, H = meshgen.grid_hex(n)
    b = meshgen.grid_boundary_mask(n)
    V = meshgen.jitter(V, ~b, 1.0 / n, seed, sigma=sigma)
    if inverted:
        rng = np.random.default_rng(seed + 1)
        inner = np.nonzero(~b)[0]
        pick = rng.choice(inner, size=inverted, replace=False)
        V[pick] += rng.normal(0, 0.9 / n, size=(inverted, 3))
    return V, H, b


def feature_constraints(V, n, lam=0.05):
    """Tangent planes onto a sphere for the boundary, the 8 box corners as corners and the
    x-edge at y=z=0 as a feature line; the same synthetic constraint kinds feature_alignment
    feeds slim_m_opt."""
    b = meshgen.grid_boundary_mask(n)
    k, j, i = np.meshgrid(np.arange(n + 1), np.arange(n + 1), np.arange(n + 1), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    corner = ((i == 0) | (i == n)) & ((j == 0) | (j == n)) & ((k == 0) | (k == n))
    line = (j == 0) & (k == 0) & ~corner
    reg = b & ~corner & ~line
    ids_C = np.nonzero(corner)[0].astype(np.int32)
    C_ = V[ids_C].copy()
    ids_L = np.nonzero(line)[0].astype(np.int32)
    Axa_L = np.tile([1.0, 0.0, 0.0], (len(ids_L), 1))
    origin_L = np.column_stack([V[ids_L, 0], np.zeros(len(ids_L)), np.zeros(len(ids_L))])
    ids_T = np.nonzero(reg)[0].astype(np.int32)
    c = np.array([0.5, 0.5, 0.5])
    nrm = V[ids_T] - c
    nrm /= np.linalg.norm(nrm, axis=1)[:, None]
    tgt = c + 0.62 * nrm
    dis_T = (nrm * tgt).sum(1)
    return dict(ids_C=ids_C, C_=C_, lamda_C=lam, ids_T=ids_T, normal_T=nrm, dis_T=dis_T, lamda_T=lam,
                ids_L=ids_L, Axa_L=Axa_L, origin_L=origin_L, lamda_L=lam)


def ref_slim(V, H, fc, iters, weight_opt=0.001, h_flag=None, energy=2, cube=1):
    R = O.ref()
    Vo = np.empty_like(V)
    out = np.empty(3)
    hf = None if h_flag is None else np.ascontiguousarray(h_flag, np.uint8)
    R.ref_slim_m_opt(len(V), p(V, _d), len(H), p(H, _u32), p(hf, _u8), cube, energy, weight_opt,
                     len(fc["ids_C"]), p(fc["ids_C"], _i32), p(np.ascontiguousarray(fc["C_"]), _d), fc["lamda_C"],
                     len(fc["ids_T"]), p(fc["ids_T"], _i32), p(np.ascontiguousarray(fc["normal_T"]), _d),
                     p(np.ascontiguousarray(fc["dis_T"]), _d), fc["lamda_T"],
                     len(fc["ids_L"]), p(fc["ids_L"], _i32), p(np.ascontiguousarray(fc["Axa_L"]), _d),
                     p(np.ascontiguousarray(fc["origin_L"]), _d), fc["lamda_L"], iters, p(Vo, _d), p(out, _d))
    return Vo, out


def energies():
    """slim_m_opt with each SLIM_ENERGY (global_types.h:58-66): ARAP, LOG_ARAP, SYMMETRIC_DIRICHLET,
    CONFORMAL, EXP_CONFORMAL, EXP_SYMMETRIC_DIRICHLET, 2 iterations on a jittered 4^3 grid with the
    feature-alignment constraint kinds."""
    for e in range(6):
        V, H, _ = jittered_grid(4, 0.1, 70 + e)
        fc = feature_constraints(V, 4, 0.05)
        Vo, o3 = ref_slim(V, H, fc, 2, energy=e)
        np.savez_compressed(os.path.join(HERE, f"slim_energy_{e}.npz"), V=V, H=H, iters=2, energy=e, V_o=Vo,
                            out=o3, **{k: np.asarray(v) for k, v in fc.items()})
        print("energy", e, o3)


def shapes():
    """slim_m_opt with compute_referenceMesh(cube = false): edge-averaged cuboid reference shapes,
    on a stretched box grid (cells 0.4 x 0.25 x 0.5) with own-shape hexes mixed in."""
    V, H = meshgen.grid_hex(5, 4, 3, hi=(2.0, 1.0, 1.5))
    b = meshgen.grid_boundary_mask(5, 4, 3)
    V = meshgen.jitter(V, ~b, 0.3, 80, sigma=0.1)
    hflag = np.ones(len(H), np.uint8)
    hflag[::7] = 0
    fc = dict(ids_C=np.zeros(0, np.int32), C_=np.zeros((0, 3)), lamda_C=0.0,
              ids_T=np.zeros(0, np.int32), normal_T=np.zeros((0, 3)), dis_T=np.zeros(0), lamda_T=0.0,
              ids_L=np.zeros(0, np.int32), Axa_L=np.zeros((0, 3)), origin_L=np.zeros((0, 3)), lamda_L=0.0)
    Vo, o3 = ref_slim(V, H, fc, 2, h_flag=hflag, cube=0, weight_opt=1.0)
    np.savez_compressed(os.path.join(HERE, "slim_cube0.npz"), V=V, H=H, h_flag=hflag, iters=2, V_o=Vo, out=o3,
                        weight_opt=1.0, cube=0, **{k: np.asarray(v) for k, v in fc.items()})
    print("cube0", o3)


def untangle():
    """optimization::pipeline2 (rigidDeformCubes + glueInternalNodes, the adaptive gluing solve
    with CONFORMAL energy and cuboid reference shapes) on jittered grids with inverted hexes and the
    boundary held: one solved in 1 iteration, one in 2, one that runs all 50 iterations without
    untangling, and a stretched box grid."""
    R = O.ref()
    R.ref_pipeline2.argtypes = [C.c_int64, _d, C.c_int64, _u32, _u8, C.c_double, _d, _d]
    cases = [("untangle_a", 5, 0.2, 1, None), ("untangle_b", 5, 0.25, 0, None), ("untangle_c", 5, 0.2, 2, None),
             ("untangle_box", (6, 4, 3), 0.22, 3, (2.0, 1.0, 1.5))]
    for name, n, sig, seed, hi in cases:
        if hi is None:
            V, H = meshgen.grid_hex(n)
            b = meshgen.grid_boundary_mask(n)
            V = meshgen.jitter(V, ~b, 1.0 / n, seed, sigma=sig)
        else:
            V, H = meshgen.grid_hex(*n, hi=hi)
            b = meshgen.grid_boundary_mask(*n)
            V = meshgen.jitter(V, ~b, min(hi[0] / n[0], hi[1] / n[1], hi[2] / n[2]), seed, sigma=sig)
        bb = np.ascontiguousarray(b.astype(np.uint8))
        Vo = np.empty_like(V)
        out = np.empty(4)
        R.ref_pipeline2(len(V), p(V, _d), len(H), p(H, _u32), p(bb, _u8), 1.0, p(Vo, _d), p(out, _d))
        # the reference's own spread under 1e-15 relative input noise (4 trials): the adaptive
        # solve's growing glue weight makes long runs sensitive to rounding
        diag = np.linalg.norm(V.max(0) - V.min(0))
        spread, jspread = 0.0, 0.0
        for k in range(4):
            Vn = np.ascontiguousarray(V * (1 + np.random.default_rng(k).normal(0, 1e-15, V.shape)))
            Vk = np.empty_like(V)
            ok = np.empty(4)
            R.ref_pipeline2(len(V), p(Vn, _d), len(H), p(H, _u32), p(bb, _u8), 1.0, p(Vk, _d), p(ok, _d))
            spread = max(spread, float(np.abs(Vk - Vo).max() / diag))
            jspread = max(jspread, abs(float(ok[1] - out[1])))
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), V=V, H=H, boundary=bb, weight_opt=1.0, V_o=Vo, out=out,
                            spread=spread, minJ_spread=jspread)
        print(name, out, "spread", spread, jspread)


def smoothing():
    """The smoothing stage: 3 rounds of cube reference shapes + 5 iterations of the modified
    igl::slim (slim_opt_igl, M = weight_opt / 2), no soft constraints."""
    R = O.ref()
    R.ref_smoothing.argtypes = [C.c_int64, _d, C.c_int64, _u32, C.c_double, C.c_int, C.c_int, _d, _d]
    V, H, _ = jittered_grid(5, 0.15, 90)
    Vo = np.empty_like(V)
    out = np.empty(3)
    R.ref_smoothing(len(V), p(V, _d), len(H), p(H, _u32), 1.0, 3, 5, p(Vo, _d), p(out, _d))
    np.savez_compressed(os.path.join(HERE, "smoothing.npz"), V=V, H=H, weight_opt=1.0, outer=3, inner=5, V_o=Vo,
                        out=out)
    print("smoothing", out)


def projection():
    """slim_m_opt with the projection term (ts.projection, b / bc, lamda_projection) on a
    jittered grid: the boundary vertices pulled onto a sphere-ish target, 2 iterations."""
    R = O.ref()
    R.ref_slim_m_opt_proj.argtypes = [C.c_int64, _d, C.c_int64, _u32, C.c_double, C.c_int64, _i32, _d, C.c_double,
                                      C.c_int, _d, _d]
    V, H, b = jittered_grid(4, 0.1, 95)
    ids = np.ascontiguousarray(np.nonzero(b)[0][::2].astype(np.int32))
    c = np.array([0.5, 0.5, 0.5])
    nrm = V[ids] - c
    bc = np.ascontiguousarray(c + nrm * (0.6 / np.linalg.norm(nrm, axis=1))[:, None])
    Vo = np.empty_like(V)
    out = np.empty(3)
    R.ref_slim_m_opt_proj(len(V), p(V, _d), len(H), p(H, _u32), 0.001, len(ids), p(ids, _i32), p(bc, _d), 1e3, 2,
                          p(Vo, _d), p(out, _d))
    np.savez_compressed(os.path.join(HERE, "slim_projection.npz"), V=V, H=H, b=ids, bc=bc, lamda_projection=1e3,
                        weight_opt=0.001, iters=2, V_o=Vo, out=out)
    print("projection", out)


def main(groups):
    if "projection" in groups:
        projection()
    if "smoothing" in groups:
        smoothing()
    if "untangle" in groups:
        untangle()
    if "energies" in groups:
        energies()
    if "shapes" in groups:
        shapes()
    if "base" in groups:
        base()


def base():
    R = O.ref()
    out = {}
    # 1. scaled Jacobian on a jittered 5^3 grid with a few tangled vertices
    V, H, _ = jittered_grid(5, 0.2, 11, inverted=6)
    vj = np.empty(8 * len(H)); hj = np.empty(len(H)); o4 = np.empty(4)
    R.ref_scaled_jacobian(len(V), p(V, _d), len(H), p(H, _u32), p(vj, _d), p(hj, _d), p(o4, _d))
    np.savez_compressed(os.path.join(HERE, "scaled_jacobian.npz"), V=V, H=H, V_Js=vj, H_Js=hj, stats=o4)
    out["scaled_jacobian"] = o4

    # 2. reference shapes + gradient operator, cube and own-shape hexes, cube flag on/off
    V, H, _ = jittered_grid(3, 0.15, 12, inverted=1)
    hflag = np.ones(len(H), np.uint8)
    hflag[::5] = 0
    for cube in (1, 0):
        RT = np.empty((8 * len(H), 4, 3)); Dg = np.empty((8 * len(H), 4, 3))
        R.ref_grad(len(V), p(V, _d), len(H), p(H, _u32), p(hflag, _u8), cube, p(RT, _d), p(Dg, _d))
        np.savez_compressed(os.path.join(HERE, f"grad_ref_cube{cube}.npz"), V=V, H=H, h_flag=hflag, RT=RT, Dg=Dg)

    # 3. slim_m_opt in the feature-alignment configuration (SYMMETRIC_DIRICHLET, weight 1e-3)
    for name, n, sigma, seed, iters, lam in (("slim_fa_1", 5, 0.12, 21, 1, 0.05),
                                               ("slim_fa_3", 5, 0.12, 22, 3, 0.05),
                                               ("slim_fa_strong", 4, 0.1, 23, 2, 50.0)):
        V, H, _ = jittered_grid(n, sigma, seed)
        fc = feature_constraints(V, n, lam)
        Vo, o3 = ref_slim(V, H, fc, iters)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), V=V, H=H, iters=iters, V_o=Vo, out=o3,
                            **{k: np.asarray(v) for k, v in fc.items()})
        out[name] = o3

    # 3b. own-shape (h_flag = 0) hexes mixed in, no soft constraints
    V, H, _ = jittered_grid(4, 0.12, 24)
    hflag = np.ones(len(H), np.uint8)
    hflag[::3] = 0
    fc = feature_constraints(V, 4, 0.05)
    Vo, o3 = ref_slim(V, H, fc, 2, h_flag=hflag)
    np.savez_compressed(os.path.join(HERE, "slim_fa_hflag.npz"), V=V, H=H, h_flag=hflag, iters=2, V_o=Vo, out=o3,
                        **{k: np.asarray(v) for k, v in fc.items()})

    # 4. per-tet energies at perturbed positions
    V, H, b = jittered_grid(4, 0.1, 31)
    X = meshgen.jitter(V, ~b, 0.25, 32, sigma=0.05)
    Et = np.empty(8 * len(H))
    R.ref_tet_energy(len(V), p(V, _d), p(X, _d), len(H), p(H, _u32), 2, 0.001, p(Et, _d))
    np.savez_compressed(os.path.join(HERE, "tet_energy.npz"), V=V, X=X, H=H, E_tet=Et)

    # 5. flip-avoiding step bound
    rng = np.random.default_rng(41)
    V, H, _ = jittered_grid(4, 0.1, 42)
    D = rng.normal(0, 0.2, size=V.shape)
    ms = np.empty(1)
    R.ref_max_step(len(V), p(V, _d), p(D, _d), len(H), p(H, _u32), p(ms, _d))
    np.savez_compressed(os.path.join(HERE, "max_step.npz"), V=V, D=D, H=H, max_step=ms)

    # 6. closest point + pseudonormal on a small superellipsoid and on the cylinder
    TV, TF = meshgen.superellipsoid(3000, exponent=4.0, radius=0.5)
    P = np.random.default_rng(51).uniform(-0.1, 1.1, size=(600, 3))
    S = np.empty(len(P)); I = np.empty(len(P), np.int32); Cc = np.empty((len(P), 3)); N = np.empty((len(P), 3))
    R.ref_signed_distance(len(TV), p(TV, _d), len(TF), p(TF, _i32), len(P), p(P, _d), p(S, _d), p(I, _i32),
                          p(Cc, _d), p(N, _d))
    np.savez_compressed(os.path.join(HERE, "signed_distance.npz"), TV=TV, TF=TF, P=P, S=S, I=I, C=Cc, N=N)
    CV, CF, _ = meshgen.cylinder_surface()
    P = np.random.default_rng(52).uniform(-0.7, 0.7, size=(400, 3))
    S = np.empty(len(P)); I = np.empty(len(P), np.int32); Cc = np.empty((len(P), 3)); N = np.empty((len(P), 3))
    R.ref_signed_distance(len(CV), p(CV, _d), len(CF), p(CF, _i32), len(P), p(P, _d), p(S, _d), p(I, _i32),
                          p(Cc, _d), p(N, _d))
    np.savez_compressed(os.path.join(HERE, "signed_distance_cyl.npz"), TV=CV, TF=CF, P=P, S=S, I=I, C=Cc, N=N)

    # 7. two-sided vertex-sampled Hausdorff: cylinder vs a jittered copy, and vs a hex boundary
    CV2 = CV + np.random.default_rng(61).normal(0, 0.01, size=CV.shape)
    o3 = np.empty(3)
    R.ref_hausdorff(len(CV), p(CV, _d), len(CF), p(CF, _i32), len(CV2), p(CV2, _d), len(CF), p(CF, _i32), p(o3, _d))
    HV, HH, _, _ = meshgen.cylinder_hex(n_core=4, n_ring=3, n_z=6)
    HQ = meshgen.hex_boundary_quads(HH)
    used = np.unique(HQ)
    remap = -np.ones(len(HV), np.int64)
    remap[used] = np.arange(len(used))
    BV = np.ascontiguousarray(HV[used])
    BF = np.ascontiguousarray(meshgen.quads_to_tris(remap[HQ]))
    o3b = np.empty(3)
    R.ref_hausdorff(len(CV), p(CV, _d), len(CF), p(CF, _i32), len(BV), p(BV, _d), len(BF), p(BF, _i32), p(o3b, _d))
    np.savez_compressed(os.path.join(HERE, "hausdorff.npz"), V0=CV, F0=CF, V1=CV2, F1=CF, out=o3,
                        BV=BV, BF=BF, out_b=o3b)
    for k, v in out.items():
        print(k, v)
    print("hausdorff", o3, o3b)


if __name__ == "__main__":
    main(sys.argv[1:] or ["base", "energies", "shapes", "untangle", "smoothing", "projection"])
