"""ctypes binding of the CPU oracle (libhexopt_oracle.so) and, when it has been built here, of the
reference harness (_ref/libhexopt_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
arm, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libhexopt_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libhexopt_ref.so")

SYMMETRIC_DIRICHLET = 2

_d = C.POINTER(C.c_double)
_i32 = C.POINTER(C.c_int32)
_u32 = C.POINTER(C.c_uint32)
_u8 = C.POINTER(C.c_uint8)
_i64 = C.POINTER(C.c_int64)


def build_oracle() -> str:
    """Compile the oracle with make (idempotent)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return ORACLE_SO


def _p(a, t):
    return a.ctypes.data_as(t) if a is not None else None


class orc_slim_problem(C.Structure):
    _fields_ = [
        ("nv", C.c_int64), ("nh", C.c_int64),
        ("V", _d), ("UV", _d), ("H", _u32), ("h_flag", _u8),
        ("cube", C.c_int), ("energy", C.c_int), ("weight_opt", C.c_double), ("exp_factor", C.c_double),
        ("nC", C.c_int64), ("ids_C", _i32), ("C", _d), ("lamda_C", C.c_double),
        ("nT", C.c_int64), ("ids_T", _i32), ("normal_T", _d), ("dis_T", _d), ("lamda_T", C.c_double),
        ("nL", C.c_int64), ("ids_L", _i32), ("Axa_L", _d), ("origin_L", _d), ("lamda_L", C.c_double),
        ("projection", C.c_int), ("nB", C.c_int64), ("b", _i32), ("bc", _d), ("lamda_projection", C.c_double),
    ]


class orc_slim_result(C.Structure):
    _fields_ = [("energy", C.c_double), ("energy_quality", C.c_double), ("energy_soft", C.c_double),
                ("cg_iters", C.c_int), ("cg_error", C.c_double), ("max_step", C.c_double),
                ("step", C.c_double), ("halvings", C.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        L = C.CDLL(ORACLE_SO)
        L.orc_scaled_jacobian.argtypes = [C.c_int64, _d, C.c_int64, _u32, _d, _d, _d, _d, _d, _i64]
        L.orc_reference_mesh.argtypes = [_d, C.c_int64, _u32, _u8, C.c_int, _d]
        L.orc_grad_ref.argtypes = [_d, C.c_int64, _u32, _d, _d]
        L.orc_slim_m_opt.argtypes = [C.POINTER(orc_slim_problem), C.c_int, _d, _d, C.POINTER(orc_slim_result)]
        L.orc_slim_m_opt.restype = C.c_int
        L.orc_slim_energy.argtypes = [C.POINTER(orc_slim_problem), _d, _d, _d, _d, _d]
        L.orc_slim_energy.restype = C.c_double
        L.orc_slim_energy_grad.argtypes = [C.POINTER(orc_slim_problem), _d, _d, _d]
        L.orc_max_step.argtypes = [C.c_int64, _d, _d, C.c_int64, _u32]
        L.orc_max_step.restype = C.c_double
        L.orc_tree_build.argtypes = [C.c_int64, _d, C.c_int64, _i32]
        L.orc_tree_build.restype = C.c_void_p
        L.orc_tree_free.argtypes = [C.c_void_p]
        L.orc_signed_distance.argtypes = [C.c_void_p, C.c_int64, _d, _d, _i32, _d, _d]
        L.orc_point_line_projection.argtypes = [_d, _d, _d, _d, _d]
        L.orc_curve_targets.argtypes = [C.c_int64, _d, _i32, _i32, _d, _i64, _i32, _u8, _d, _d]
        L.orc_hausdorff.argtypes = [C.c_int64, _d, C.c_int64, _i32, C.c_int64, _d, C.c_int64, _i32, _d, _d, _d]
        L.orc_point_face_distance.argtypes = [C.c_int64, _d, C.c_int64, _d, C.c_int64, _i32, _d]
        _lib = L
    return _lib


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def scaled_jacobian(V, H):
    V = _f64(V); H = np.ascontiguousarray(H, dtype=np.uint32)
    nh = len(H)
    vj = np.empty(8 * nh); hj = np.empty(nh)
    mn, av, dv = C.c_double(), C.c_double(), C.c_double()
    ninv = C.c_int64()
    lib().orc_scaled_jacobian(len(V), _p(V, _d), nh, _p(H, _u32), _p(vj, _d), _p(hj, _d),
                              C.byref(mn), C.byref(av), C.byref(dv), C.byref(ninv))
    return dict(V_Js=vj, H_Js=hj, min=mn.value, ave=av.value, dev=dv.value, inverted=ninv.value)


def grad_ref(V, H, h_flag=None, cube=True):
    V = _f64(V); H = np.ascontiguousarray(H, dtype=np.uint32)
    nt = 8 * len(H)
    RT = np.empty((nt, 4, 3)); Dg = np.empty((nt, 4, 3))
    hf = None if h_flag is None else np.ascontiguousarray(h_flag, dtype=np.uint8)
    lib().orc_reference_mesh(_p(V, _d), len(H), _p(H, _u32), _p(hf, _u8), int(cube), _p(RT, _d))
    lib().orc_grad_ref(_p(V, _d), len(H), _p(H, _u32), _p(RT, _d), _p(Dg, _d))
    return RT, Dg


class SlimProblem:
    """Inputs of one slim_m_opt call (feature-alignment form)."""

    def __init__(self, V, H, UV=None, h_flag=None, cube=True, energy=SYMMETRIC_DIRICHLET, weight_opt=0.001,
                 exp_factor=1.0, ids_C=None, C_=None, lamda_C=0.0, ids_T=None, normal_T=None, dis_T=None,
                 lamda_T=0.0, ids_L=None, Axa_L=None, origin_L=None, lamda_L=0.0, b=None, bc=None,
                 lamda_projection=0.0):
        self.V = _f64(V)
        self.UV = _f64(V if UV is None else UV)
        self.H = np.ascontiguousarray(H, dtype=np.uint32)
        self.h_flag = None if h_flag is None else np.ascontiguousarray(h_flag, dtype=np.uint8)
        self.cube, self.energy, self.weight_opt, self.exp_factor = cube, energy, weight_opt, exp_factor
        e3 = np.zeros((0, 3))
        ei = np.zeros(0, np.int32)
        self.ids_C = np.ascontiguousarray(ei if ids_C is None else ids_C, dtype=np.int32)
        self.C = _f64(e3 if C_ is None else C_).reshape(-1, 3)
        self.ids_T = np.ascontiguousarray(ei if ids_T is None else ids_T, dtype=np.int32)
        self.normal_T = _f64(e3 if normal_T is None else normal_T).reshape(-1, 3)
        self.dis_T = _f64(np.zeros(0) if dis_T is None else dis_T)
        self.ids_L = np.ascontiguousarray(ei if ids_L is None else ids_L, dtype=np.int32)
        self.Axa_L = _f64(e3 if Axa_L is None else Axa_L).reshape(-1, 3)
        self.origin_L = _f64(e3 if origin_L is None else origin_L).reshape(-1, 3)
        self.lamda_C, self.lamda_T, self.lamda_L = lamda_C, lamda_T, lamda_L
        self.b = None if b is None else np.ascontiguousarray(b, dtype=np.int32)
        self.bc = None if bc is None else _f64(bc).reshape(-1, 3)
        self.lamda_projection = lamda_projection

    def struct(self):
        s = orc_slim_problem()
        s.nv, s.nh = len(self.V), len(self.H)
        s.V, s.UV, s.H, s.h_flag = _p(self.V, _d), _p(self.UV, _d), _p(self.H, _u32), _p(self.h_flag, _u8)
        s.cube, s.energy, s.weight_opt, s.exp_factor = int(self.cube), self.energy, self.weight_opt, self.exp_factor
        s.nC, s.ids_C, s.C, s.lamda_C = len(self.ids_C), _p(self.ids_C, _i32), _p(self.C, _d), self.lamda_C
        s.nT, s.ids_T, s.normal_T, s.dis_T, s.lamda_T = (len(self.ids_T), _p(self.ids_T, _i32),
                                                         _p(self.normal_T, _d), _p(self.dis_T, _d), self.lamda_T)
        s.nL, s.ids_L, s.Axa_L, s.origin_L, s.lamda_L = (len(self.ids_L), _p(self.ids_L, _i32), _p(self.Axa_L, _d),
                                                         _p(self.origin_L, _d), self.lamda_L)
        s.projection, s.nB = 0, 0
        if self.b is not None:
            s.projection, s.nB, s.b, s.bc = 1, len(self.b), _p(self.b, _i32), _p(self.bc, _d)
            s.lamda_projection = self.lamda_projection
        return s


def slim_m_opt(prob: SlimProblem, iters: int):
    s = prob.struct()
    Vo = np.empty_like(prob.V)
    aL = np.empty(max(1, len(prob.ids_L)))
    r = orc_slim_result()
    lib().orc_slim_m_opt(C.byref(s), int(iters), _p(Vo, _d), _p(aL, _d), C.byref(r))
    return Vo, aL[:len(prob.ids_L)], dict(energy=r.energy, energy_quality=r.energy_quality,
                                           energy_soft=r.energy_soft, cg_iters=r.cg_iters, cg_error=r.cg_error,
                                           max_step=r.max_step, step=r.step, halvings=r.halvings)


def slim_energy(prob: SlimProblem, X, a_L=None):
    s = prob.struct()
    X = _f64(X)
    aL = None if a_L is None else _f64(a_L)
    Et = np.empty(8 * len(prob.H))
    eq, es = C.c_double(), C.c_double()
    tot = lib().orc_slim_energy(C.byref(s), _p(X, _d), _p(aL, _d), _p(Et, _d), C.byref(eq), C.byref(es))
    return tot, Et, eq.value, es.value


def slim_energy_grad(prob: SlimProblem, X, a_L=None):
    s = prob.struct()
    X = _f64(X)
    aL = None if a_L is None else _f64(a_L)
    G = np.empty_like(X)
    lib().orc_slim_energy_grad(C.byref(s), _p(X, _d), _p(aL, _d), _p(G, _d))
    return G


def max_step(X, D, H):
    X = _f64(X); D = _f64(D); H = np.ascontiguousarray(H, dtype=np.uint32)
    return lib().orc_max_step(len(X), _p(X, _d), _p(D, _d), len(H), _p(H, _u32))


def signed_distance(TV, TF, P):
    TV = _f64(TV); TF = np.ascontiguousarray(TF, dtype=np.int32); P = _f64(P)
    t = lib().orc_tree_build(len(TV), _p(TV, _d), len(TF), _p(TF, _i32))
    n = len(P)
    S = np.empty(n); I = np.empty(n, np.int32); Cc = np.empty((n, 3)); N = np.empty((n, 3))
    lib().orc_signed_distance(t, n, _p(P, _d), _p(S, _d), _p(I, _i32), _p(Cc, _d), _p(N, _d))
    lib().orc_tree_free(t)
    return S, I, Cc, N


def point_line_projection(v1, v2, v):
    v1, v2, v = _f64(v1), _f64(v2), _f64(v)
    pv = np.empty(3); t = C.c_double()
    lib().orc_point_line_projection(_p(v1, _d), _p(v2, _d), _p(v, _d), _p(pv, _d), C.byref(t))
    return pv, t.value


def curve_targets(X, lines, line_curve, TV, curves, closed):
    """LINE branch of dirty_graph_projection: (origin, axis) of each line vertex on its curve."""
    X, TV = _f64(X), _f64(TV)
    lines = np.ascontiguousarray(lines, dtype=np.int32)
    line_curve = np.ascontiguousarray(line_curve, dtype=np.int32)
    ptr = np.ascontiguousarray(np.concatenate([[0], np.cumsum([len(c) for c in curves])]), dtype=np.int64)
    vs = np.ascontiguousarray(np.concatenate([np.asarray(c, np.int32) for c in curves]) if len(curves)
                              else np.zeros(1, np.int32), dtype=np.int32)
    cl = np.ascontiguousarray(np.asarray(closed, np.uint8).reshape(-1) if len(closed) else np.zeros(1, np.uint8))
    n = len(lines)
    org = np.zeros((n, 3)); ax = np.zeros((n, 3))
    if n:
        lib().orc_curve_targets(n, _p(X, _d), _p(lines, _i32), _p(line_curve, _i32), _p(TV, _d), _p(ptr, _i64),
                                _p(vs, _i32), _p(cl, _u8), _p(org, _d), _p(ax, _d))
    return org, ax


def hausdorff(V0, F0, V1, F1):
    V0, V1 = _f64(V0), _f64(V1)
    F0 = np.ascontiguousarray(F0, dtype=np.int32); F1 = np.ascontiguousarray(F1, dtype=np.int32)
    dg, mx, av = C.c_double(), C.c_double(), C.c_double()
    lib().orc_hausdorff(len(V0), _p(V0, _d), len(F0), _p(F0, _i32), len(V1), _p(V1, _d), len(F1), _p(F1, _i32),
                        C.byref(dg), C.byref(mx), C.byref(av))
    return dg.value, mx.value, av.value


def point_face_distance(P, V, F):
    P, V = _f64(P), _f64(V)
    F = np.ascontiguousarray(F, dtype=np.int32)
    d = np.empty(len(P))
    lib().orc_point_face_distance(len(P), _p(P, _d), len(V), _p(V, _d), len(F), _p(F, _i32), _p(d, _d))
    return d


# ------------------------------------------------------------------ reference harness (here only)
_ref = None


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_SO)
        L.ref_scaled_jacobian.argtypes = [C.c_int64, _d, C.c_int64, _u32, _d, _d, _d]
        L.ref_grad.argtypes = [C.c_int64, _d, C.c_int64, _u32, _u8, C.c_int, _d, _d]
        L.ref_slim_m_opt.argtypes = [C.c_int64, _d, C.c_int64, _u32, _u8, C.c_int, C.c_int, C.c_double,
                                     C.c_int64, _i32, _d, C.c_double,
                                     C.c_int64, _i32, _d, _d, C.c_double,
                                     C.c_int64, _i32, _d, _d, C.c_double, C.c_int, _d, _d]
        L.ref_tet_energy.argtypes = [C.c_int64, _d, _d, C.c_int64, _u32, C.c_int, C.c_double, _d]
        L.ref_max_step.argtypes = [C.c_int64, _d, _d, C.c_int64, _u32, _d]
        L.ref_signed_distance.argtypes = [C.c_int64, _d, C.c_int64, _i32, C.c_int64, _d, _d, _i32, _d, _d]
        L.ref_hausdorff.argtypes = [C.c_int64, _d, C.c_int64, _i32, C.c_int64, _d, C.c_int64, _i32, _d]
        _ref = L
    return _ref
