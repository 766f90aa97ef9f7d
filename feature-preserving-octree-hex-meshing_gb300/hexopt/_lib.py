"""ctypes binding of libhexopt_gpu.so (the C ABI declared in include/hexopt_gpu.h).

Loading fails loudly when the library is missing or no CUDA device is present: there is no
CPU path behind this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhexopt_gpu.so")

FP64, MIXED = 0, 1
SYMMETRIC_DIRICHLET = 2

_d = C.POINTER(C.c_double)
_i32 = C.POINTER(C.c_int32)
_u32 = C.POINTER(C.c_uint32)
_u8 = C.POINTER(C.c_uint8)
_i64 = C.POINTER(C.c_int64)
_vp = C.c_void_p


class Quality(C.Structure):
    _fields_ = [("min_Jacobian", C.c_double), ("ave_Jacobian", C.c_double), ("deviation_Jacobian", C.c_double),
                ("n_inverted", C.c_int64)]


class SlimParams(C.Structure):
    _fields_ = [("energy", C.c_int), ("precision", C.c_int), ("weight_opt", C.c_double),
                ("exp_factor", C.c_double), ("cg_max_iter", C.c_int), ("cg_tol", C.c_double),
                ("ls_candidates", C.c_int), ("cube", C.c_int), ("cg_refine", C.c_int), ("variant", C.c_int)]


class SlimReport(C.Structure):
    _fields_ = [("energy", C.c_double), ("energy_quality", C.c_double), ("energy_soft", C.c_double),
                ("cg_error", C.c_double), ("max_step", C.c_double), ("step", C.c_double),
                ("cg_iters", C.c_int32), ("halvings", C.c_int32), ("status", C.c_int32), ("pad", C.c_int32)]


class FaReport(C.Structure):
    _fields_ = [("slim", SlimReport), ("quality", Quality), ("lamda", C.c_double),
                ("hausdorff_diag", C.c_double), ("hausdorff_max", C.c_double), ("hausdorff_ave", C.c_double)]


class AdaptiveReport(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("converged", C.c_int32), ("min_Jacobian", C.c_double),
                ("ave_Jacobian", C.c_double), ("energy", C.c_double), ("energy_quality", C.c_double),
                ("energy_soft", C.c_double), ("lamda_glue", C.c_double), ("status", C.c_int32), ("pad", C.c_int32)]


class UntangleReport(C.Structure):
    _fields_ = [("success", C.c_int32), ("iterations", C.c_int32), ("min_Jacobian", C.c_double),
                ("ave_Jacobian", C.c_double), ("energy", C.c_double), ("lamda_glue", C.c_double)]


class AABB(C.Structure):
    _fields_ = [("min", C.c_double * 3), ("max", C.c_double * 3)]


class Ray(C.Structure):
    _fields_ = [("o", C.c_double * 3), ("d", C.c_double * 3), ("dRcp", C.c_double * 3), ("mint", C.c_double),
                ("maxt", C.c_double)]


# name -> (restype, argtypes)
SIGNATURES = {
    "hexopt_create": (C.c_int, [C.POINTER(_vp), C.c_int]),
    "hexopt_destroy": (None, [_vp]),
    "hexopt_last_error": (C.c_char_p, [_vp]),
    "hexopt_sync": (C.c_int, [_vp]),
    "hexopt_set_ordering": (C.c_int, [_vp, C.c_int]),
    "hexopt_upload_meshes": (C.c_int, [_vp, C.c_int, _i64, _i64, _d, _u32, _u8]),
    "hexopt_set_positions": (C.c_int, [_vp, _d]),
    "hexopt_get_positions": (C.c_int, [_vp, _d]),
    "hexopt_set_positions_async": (C.c_int, [_vp, _d]),
    "hexopt_get_positions_async": (C.c_int, [_vp, _d]),
    "hexopt_num_vertices": (C.c_int64, [_vp]),
    "hexopt_num_hexes": (C.c_int64, [_vp]),
    "hexopt_num_meshes": (C.c_int, [_vp]),
    "hexopt_scaled_jacobian": (C.c_int, [_vp, _d, _d, C.POINTER(Quality)]),
    "hexopt_set_corners": (C.c_int, [_vp, _i64, _i32, _d]),
    "hexopt_set_tangents": (C.c_int, [_vp, _i64, _i32, _d, _d]),
    "hexopt_set_lines": (C.c_int, [_vp, _i64, _i32, _d, _d]),
    "hexopt_set_weights": (C.c_int, [_vp, _d, _d, _d]),
    "hexopt_set_projection": (C.c_int, [_vp, _i64, _i32, _d, _d]),
    "hexopt_set_glue": (C.c_int, [_vp, _i64, _i64, _i32, _d]),
    "hexopt_set_fixed": (C.c_int, [_vp, _i64, _i32]),
    "hexopt_slim_solve_adaptive": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.POINTER(AdaptiveReport)]),
    "hexopt_untangle": (C.c_int, [_vp, C.POINTER(SlimParams), _u8, C.c_int, C.POINTER(UntangleReport)]),
    "hexopt_get_tangents": (C.c_int, [_vp, _d, _d]),
    "hexopt_get_lines": (C.c_int, [_vp, _d, _d]),
    "hexopt_set_reference_hexes": (C.c_int, [_vp, _d]),
    "hexopt_set_reference_tets": (C.c_int, [_vp, _d]),
    "hexopt_slim_precompute": (C.c_int, [_vp, C.POINTER(SlimParams)]),
    "hexopt_slim_iterate": (C.c_int, [_vp, C.c_int, C.POINTER(SlimReport)]),
    "hexopt_slim_m_opt": (C.c_int, [_vp, C.POINTER(SlimParams), C.c_int, C.POINTER(SlimReport)]),
    "hexopt_get_curve_params": (C.c_int, [_vp, _d]),
    "hexopt_smoothing": (C.c_int, [_vp, C.POINTER(SlimParams), C.c_int, C.c_int, C.POINTER(SlimReport)]),
    "hexopt_set_target": (C.c_int, [_vp, C.c_int, C.c_int64, _d, C.c_int64, _i32]),
    "hexopt_signed_distance": (C.c_int, [_vp, C.c_int, C.c_int64, _d, _d, _i32, _d, _d]),
    "hexopt_set_feature_sets": (C.c_int, [_vp, _i64, _i32, _i64, _i32, _i32, _i64, _i64, _i32, _u8]),
    "hexopt_project_features": (C.c_int, [_vp]),
    "hexopt_query_stats": (C.c_int, [_vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "hexopt_set_query_budget": (C.c_int, [_vp, C.c_int]),
    "hexopt_hausdorff": (C.c_int, [_vp, C.c_int64, _d, C.c_int64, _i32, C.c_int64, _d, C.c_int64, _i32, _d, _d, _d]),
    "hexopt_hausdorff_uniform": (C.c_int, [_vp, C.c_int64, _d, C.c_int64, _i32, C.c_int64, _d, C.c_int64, _i32,
                                           C.c_int64, C.c_uint64, _d, _d, _d, _d, _d]),
    "hexopt_set_surface": (C.c_int, [_vp, C.c_int, C.c_int64, _i32]),
    "hexopt_hausdorff_meshes": (C.c_int, [_vp, _d, _d, _d]),
    "hexopt_point_face_distance": (C.c_int, [_vp, C.c_int64, _d, C.c_int64, _d, C.c_int64, _i32, _d]),
    "hexopt_point_face_distance_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                                     C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_char_p,
                                                     C.c_size_t]),
    "hexopt_fa_begin": (C.c_int, [_vp, C.POINTER(SlimParams), C.c_double, C.c_double]),
    "hexopt_feature_alignment_step": (C.c_int, [_vp, C.c_int, C.POINTER(FaReport)]),
    "hexopt_feature_alignment_step_get": (C.c_int, [_vp, C.c_int, C.POINTER(FaReport), _d]),
    "hexopt_use_graph": (C.c_int, [_vp, C.c_int]),
    "hexopt_energy_fwd": (C.c_int, [_vp, _d, _d]),
    "hexopt_energy_bwd": (C.c_int, [_vp, _d]),
    "hexopt_set_block_size": (C.c_int, [_vp, C.c_int, C.c_int]),
    "hexopt_autotune": (C.c_int, [_vp]),
    "hexopt_get_tuning": (C.c_int, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                    C.POINTER(C.c_int)]),
    "hexopt_launch_count": (C.c_int64, [_vp]),
    "hexopt_timer_start": (C.c_int, [_vp]),
    "hexopt_timer_stop": (C.c_int, [_vp, _d]),
    "hexopt_time_stage": (C.c_int, [_vp, C.c_int, C.c_int, _d]),
    "hexopt_write_hex_mesh": (C.c_int, [C.c_char_p, C.c_int, C.c_int64, _d, C.c_int64, _u32, _u8]),
    "hexopt_read_hex_mesh": (C.c_int, [C.c_char_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), _d, _u32]),
    "hexopt_aabb_merge": (None, [C.POINTER(AABB), C.POINTER(AABB)]),
    "hexopt_aabb_squared_distance": (C.c_double, [C.POINTER(AABB), _d]),
    "hexopt_aabb_ray_intersect": (C.c_int, [C.POINTER(AABB), C.POINTER(Ray), _d, _d]),
    "hexopt_aabb_largest_axis": (C.c_int, [C.POINTER(AABB)]),
    "hexopt_aabb_surface_area": (C.c_double, [C.POINTER(AABB)]),
}

_lib = None


def load(path: str = LIB_PATH):
    """dlopen the library and declare every entry point (no device is touched)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"libhexopt_gpu.so not built ({path}); run build() first")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def ptr(a, t):
    return None if a is None else a.ctypes.data_as(t)


class HexoptError(RuntimeError):
    pass


def write_hex_mesh(path, V, H, fmt="mesh", boundary=None):
    """A hex mesh as the reference writes it: fmt "mesh" (MEDIT) or "vtk" (legacy ASCII, with the
    boundary flags as point data).  Host only."""
    L = load()
    V = np.ascontiguousarray(V, np.float64); H = np.ascontiguousarray(H, np.uint32)
    b = None if boundary is None else np.ascontiguousarray(np.asarray(boundary, np.uint8))
    rc = L.hexopt_write_hex_mesh(os.fsencode(path), 0 if fmt == "mesh" else 1, len(V), ptr(V, _d), len(H),
                                 ptr(H, _u32), ptr(b, _u8))
    if rc != 0:
        raise HexoptError(f"write_hex_mesh failed ({rc}): {path}")


def read_hex_mesh(path):
    """(V, H) of a MEDIT .mesh file's Vertices / Hexahedra blocks.  Host only."""
    L = load()
    nv, nh = C.c_int64(0), C.c_int64(0)
    rc = L.hexopt_read_hex_mesh(os.fsencode(path), C.byref(nv), C.byref(nh), None, None)
    if rc != 0:
        raise HexoptError(f"read_hex_mesh failed ({rc}): {path}")
    V = np.empty((nv.value, 3)); H = np.empty((nh.value, 8), np.uint32)
    rc = L.hexopt_read_hex_mesh(os.fsencode(path), C.byref(nv), C.byref(nh), ptr(V, _d), ptr(H, _u32))
    if rc != 0:
        raise HexoptError(f"read_hex_mesh failed ({rc}): {path}")
    return V, H


def point_face_distance_noalloc(P_dev: int, np_: int, V_dev: int, nv: int, F_dev: int, nf: int, dist_dev: int,
                                device: int = 0, stream: int = 0):
    """hexopt_point_face_distance_noalloc on raw device addresses (P_dev np_ x 3 doubles, V_dev
    nv x 3 doubles, F_dev nf x 3 int32, dist_dev np_ doubles) on `stream` (a cudaStream_t as an
    int, 0 = legacy default stream); no device allocation.  Raises HexoptError with the library's
    message on failure."""
    L = load()
    buf = C.create_string_buffer(512)
    rc = L.hexopt_point_face_distance_noalloc(device, C.c_void_p(stream or None), np_, C.c_void_p(P_dev), nv,
                                              C.c_void_p(V_dev), nf, C.c_void_p(F_dev), C.c_void_p(dist_dev), buf,
                                              len(buf))
    if rc != 0:
        raise HexoptError(f"point_face_distance_noalloc failed ({rc}): {buf.value.decode(errors='replace')}")


class Context:
    """Owns one hexopt_ctx (one CUDA stream and one batch of meshes in HBM)."""

    def __init__(self, device: int = 0):
        self.L = load()
        h = _vp()
        rc = self.L.hexopt_create(C.byref(h), device)
        if rc != 0:
            raise HexoptError(f"hexopt_create failed ({rc}): no CUDA device or driver")
        self.h = h
        self.nv = []
        self.nh = []

    def close(self):
        if getattr(self, "h", None):
            self.L.hexopt_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _ck(self, rc, what):
        if rc != 0:
            msg = self.L.hexopt_last_error(self.h)
            raise HexoptError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")

    # ---- meshes
    def set_ordering(self, mode=2):
        """Device order of the next upload: 0 caller order, 1 Morton, 2 (default) Morton unless the
        caller's numbering is already coherent.  True / False mean 1 / 0."""
        mode = int(mode) if not isinstance(mode, bool) else int(mode)
        self._ck(self.L.hexopt_set_ordering(self.h, mode), "set_ordering")

    def upload(self, meshes, h_flag=None):
        """meshes: list of (V (nv,3) float64, H (nh,8) uint32)."""
        nv = np.array([len(V) for V, _ in meshes], np.int64)
        nh = np.array([len(H) for _, H in meshes], np.int64)
        V = np.ascontiguousarray(np.concatenate([m[0] for m in meshes]), np.float64)
        H = np.ascontiguousarray(np.concatenate([m[1] for m in meshes]), np.uint32)
        hf = None if h_flag is None else np.ascontiguousarray(h_flag, np.uint8)
        self._ck(self.L.hexopt_upload_meshes(self.h, len(meshes), ptr(nv, _i64), ptr(nh, _i64), ptr(V, _d),
                                             ptr(H, _u32), ptr(hf, _u8)), "upload_meshes")
        self.nv, self.nh = list(nv), list(nh)
        return self

    @property
    def n_meshes(self):
        return len(self.nv)

    def set_positions(self, V):
        V = np.ascontiguousarray(V, np.float64)
        self._ck(self.L.hexopt_set_positions(self.h, ptr(V, _d)), "set_positions")

    def get_positions(self):
        out = np.empty((int(sum(self.nv)), 3))
        self._ck(self.L.hexopt_get_positions(self.h, ptr(out, _d)), "get_positions")
        return out

    def set_positions_async(self, V):
        """Queue an upload of V (C-contiguous float64, nv x 3): V must stay alive and unchanged
        until sync() returns (page-locked memory lets the copy overlap the computation)."""
        if not (isinstance(V, np.ndarray) and V.dtype == np.float64 and V.flags.c_contiguous):
            raise ValueError("set_positions_async needs a C-contiguous float64 array")
        self._ck(self.L.hexopt_set_positions_async(self.h, ptr(V, _d)), "set_positions_async")

    def get_positions_async(self, out):
        """Queue a download of the positions into out (C-contiguous float64, nv x 3), complete
        after sync()."""
        if not (isinstance(out, np.ndarray) and out.dtype == np.float64 and out.flags.c_contiguous):
            raise ValueError("get_positions_async needs a C-contiguous float64 array")
        self._ck(self.L.hexopt_get_positions_async(self.h, ptr(out, _d)), "get_positions_async")

    def scaled_jacobian(self, per_corner=False):
        NH = int(sum(self.nh))
        vj = np.empty(8 * NH) if per_corner else None
        hj = np.empty(NH)
        q = (Quality * self.n_meshes)()
        self._ck(self.L.hexopt_scaled_jacobian(self.h, ptr(vj, _d), ptr(hj, _d), q), "scaled_jacobian")
        qs = [dict(min=x.min_Jacobian, ave=x.ave_Jacobian, dev=x.deviation_Jacobian, inverted=x.n_inverted) for x in q]
        return vj, hj, qs

    # ---- constraints (lists per mesh)
    @staticmethod
    def _cat(lists, dtype, width=None):
        counts = np.array([len(x) for x in lists], np.int64)
        if width:
            arr = np.concatenate([np.asarray(x, dtype).reshape(-1, width) for x in lists]) if counts.sum() else np.zeros((0, width), dtype)
        else:
            arr = np.concatenate([np.asarray(x, dtype).ravel() for x in lists]) if counts.sum() else np.zeros(0, dtype)
        return counts, np.ascontiguousarray(arr)

    def set_corners(self, ids, C_):
        n, i = self._cat(ids, np.int32)
        _, c = self._cat(C_, np.float64, 3)
        self._ck(self.L.hexopt_set_corners(self.h, ptr(n, _i64), ptr(i, _i32), ptr(c, _d)), "set_corners")

    def set_tangents(self, ids, normal, dis):
        n, i = self._cat(ids, np.int32)
        _, nn = self._cat(normal, np.float64, 3)
        _, d = self._cat(dis, np.float64)
        self._ck(self.L.hexopt_set_tangents(self.h, ptr(n, _i64), ptr(i, _i32), ptr(nn, _d), ptr(d, _d)), "set_tangents")

    def set_lines(self, ids, axis, origin):
        n, i = self._cat(ids, np.int32)
        _, ax = self._cat(axis, np.float64, 3)
        _, o = self._cat(origin, np.float64, 3)
        self._ck(self.L.hexopt_set_lines(self.h, ptr(n, _i64), ptr(i, _i32), ptr(ax, _d), ptr(o, _d)), "set_lines")

    def set_weights(self, lamda_C, lamda_T, lamda_L):
        f = lambda x: np.ascontiguousarray(np.broadcast_to(np.asarray(x, np.float64), (self.n_meshes,)))
        a, b, c = f(lamda_C), f(lamda_T), f(lamda_L)
        self._ck(self.L.hexopt_set_weights(self.h, ptr(a, _d), ptr(b, _d), ptr(c, _d)), "set_weights")

    def set_projection(self, ids, bc, lamda=None):
        """Tetralize_Set::b / bc per mesh with weight lamda_projection (scalar or per mesh)."""
        n, i = self._cat(ids, np.int32)
        _, c = self._cat(bc, np.float64, 3)
        lp = None if lamda is None else np.ascontiguousarray(np.broadcast_to(np.asarray(lamda, np.float64),
                                                                            (self.n_meshes,)))
        self._ck(self.L.hexopt_set_projection(self.h, ptr(n, _i64), ptr(i, _i32), ptr(c, _d), ptr(lp, _d)),
                 "set_projection")

    def set_glue(self, groups, lamda=None):
        """groups: per mesh a list of vertex-id arrays (each a group of copies glued together)."""
        ng = np.array([len(gs) for gs in groups], np.int64)
        ptrs, vs = [], []
        for gs in groups:
            o = 0
            ptrs.append(0)
            for g in gs:
                o += len(g)
                ptrs.append(o)
                vs.append(np.asarray(g, np.int32))
        ptrs = np.ascontiguousarray(ptrs, np.int64)
        vs = np.ascontiguousarray(np.concatenate(vs) if vs else np.zeros(1, np.int32), np.int32)
        lg = None if lamda is None else np.ascontiguousarray(np.broadcast_to(np.asarray(lamda, np.float64),
                                                                            (self.n_meshes,)))
        self._ck(self.L.hexopt_set_glue(self.h, ptr(ng, _i64), ptr(ptrs, _i64), ptr(vs, _i32), ptr(lg, _d)),
                 "set_glue")

    def set_fixed(self, ids):
        n, i = self._cat(ids, np.int32)
        self._ck(self.L.hexopt_set_fixed(self.h, ptr(n, _i64), ptr(i, _i32)), "set_fixed")

    def slim_solve_adaptive(self, type_=1, schedule=2, max_iter=50):
        """slim_solve2 (schedule 2) / slim_solve (schedule 1) with iter_num = -1."""
        rep = (AdaptiveReport * self.n_meshes)()
        self._ck(self.L.hexopt_slim_solve_adaptive(self.h, int(type_), int(schedule), int(max_iter), rep),
                 "slim_solve_adaptive")
        return [dict(iterations=r.iterations, converged=bool(r.converged), min_J=r.min_Jacobian,
                     ave_J=r.ave_Jacobian, energy=r.energy, energy_quality=r.energy_quality,
                     energy_soft=r.energy_soft, lamda_glue=r.lamda_glue, status=r.status) for r in rep]

    def untangle(self, boundary, max_iter=50, energy=3, weight_opt=1.0, **kw):
        """optimization::pipeline2 on the context's hex meshes (positions = the boundary-projected
        BV, boundary = one flag per vertex); energy defaults to CONFORMAL, the Tetralize_Set
        default the reference's gluing runs with.  Positions are replaced by the glued ones."""
        p = self.params(energy=energy, weight_opt=weight_opt, **kw)
        b = np.ascontiguousarray(np.asarray(boundary, np.uint8).reshape(-1))
        rep = (UntangleReport * self.n_meshes)()
        self._ck(self.L.hexopt_untangle(self.h, C.byref(p), ptr(b, _u8), int(max_iter), rep), "untangle")
        return [dict(success=bool(r.success), iterations=r.iterations, min_J=r.min_Jacobian, ave_J=r.ave_Jacobian,
                     energy=r.energy, lamda_glue=r.lamda_glue) for r in rep]

    def get_tangents(self, total):
        n = np.empty((total, 3)); d = np.empty(total)
        self._ck(self.L.hexopt_get_tangents(self.h, ptr(n, _d), ptr(d, _d)), "get_tangents")
        return n, d

    def get_lines(self, total):
        a = np.empty((total, 3)); o = np.empty((total, 3))
        self._ck(self.L.hexopt_get_lines(self.h, ptr(a, _d), ptr(o, _d)), "get_lines")
        return a, o

    # ---- SLIM
    def set_reference_hexes(self, P8=None):
        """Reference corners of every hex (n_hexes x 8 x 3) for compute_referenceMesh; None = the
        positions at the precompute."""
        P = None if P8 is None else np.ascontiguousarray(P8, np.float64).reshape(-1, 8, 3)
        self._ck(self.L.hexopt_set_reference_hexes(self.h, ptr(P, _d)), "set_reference_hexes")

    def set_reference_tets(self, RT=None):
        """compute_referenceMesh's reference tets (n_hexes*8 x 4 x 3); None = the default shapes."""
        R = None if RT is None else np.ascontiguousarray(RT, np.float64).reshape(-1, 4, 3)
        self._ck(self.L.hexopt_set_reference_tets(self.h, ptr(R, _d)), "set_reference_tets")

    @staticmethod
    def params(precision=FP64, weight_opt=0.001, energy=SYMMETRIC_DIRICHLET, exp_factor=1.0, cg_max_iter=20,
               cg_tol=1e-8, ls_candidates=1, cube=1, cg_refine=10, variant=0):
        return SlimParams(energy, precision, weight_opt, exp_factor, cg_max_iter, cg_tol, ls_candidates, cube,
                          cg_refine, variant)

    def slim_m_opt(self, iters, **kw):
        p = self.params(**kw)
        rep = (SlimReport * self.n_meshes)()
        self._ck(self.L.hexopt_slim_m_opt(self.h, C.byref(p), int(iters), rep), "slim_m_opt")
        return [_rep(r) for r in rep]

    def slim_precompute(self, **kw):
        p = self.params(**kw)
        self._ck(self.L.hexopt_slim_precompute(self.h, C.byref(p)), "slim_precompute")

    def slim_iterate(self, iters):
        rep = (SlimReport * self.n_meshes)()
        self._ck(self.L.hexopt_slim_iterate(self.h, int(iters), rep), "slim_iterate")
        return [_rep(r) for r in rep]

    def smoothing(self, outer=3, inner=5, **kw):
        """The smoothing stage: outer rounds of cube shapes + inner modified-igl::slim iterations."""
        p = self.params(**kw)
        rep = (SlimReport * self.n_meshes)()
        self._ck(self.L.hexopt_smoothing(self.h, C.byref(p), int(outer), int(inner), rep), "smoothing")
        return [_rep(r) for r in rep]

    def curve_params(self, total):
        a = np.empty(max(total, 1))
        self._ck(self.L.hexopt_get_curve_params(self.h, ptr(a, _d)), "get_curve_params")
        return a[:total]

    # ---- projection
    def set_target(self, mesh, TV, TF):
        TV = np.ascontiguousarray(TV, np.float64); TF = np.ascontiguousarray(TF, np.int32)
        self._ck(self.L.hexopt_set_target(self.h, mesh, len(TV), ptr(TV, _d), len(TF), ptr(TF, _i32)), "set_target")

    def signed_distance(self, mesh, P):
        P = np.ascontiguousarray(P, np.float64)
        n = len(P)
        S = np.empty(n); I = np.empty(n, np.int32); Cc = np.empty((n, 3)); N = np.empty((n, 3))
        self._ck(self.L.hexopt_signed_distance(self.h, mesh, n, ptr(P, _d), ptr(S, _d), ptr(I, _i32), ptr(Cc, _d),
                                               ptr(N, _d)), "signed_distance")
        return S, I, Cc, N

    def set_feature_sets(self, regular, lines, line_curve, curves, closed):
        """regular / lines / line_curve: per-mesh lists; curves: per-mesh list of polylines
        (arrays of target vertex ids); closed: per-mesh list of bools."""
        nr, r = self._cat(regular, np.int32)
        nl, li = self._cat(lines, np.int32)
        _, lc = self._cat(line_curve, np.int32)
        ncv = np.array([len(c) for c in curves], np.int64)
        ptrs = []
        vs = []
        for cs in curves:
            o = 0
            p_ = [0]
            for c in cs:
                o += len(c)
                p_.append(o)
                vs.append(np.asarray(c, np.int32))
            ptrs.extend(p_)
        ptrs = np.asarray(ptrs, np.int64)
        vs = np.ascontiguousarray(np.concatenate(vs) if vs else np.zeros(0, np.int32), np.int32)
        cl = np.ascontiguousarray(np.concatenate([np.asarray(c, np.uint8) for c in closed]) if sum(map(len, closed)) else np.zeros(1, np.uint8))
        self._ck(self.L.hexopt_set_feature_sets(self.h, ptr(nr, _i64), ptr(r, _i32), ptr(nl, _i64), ptr(li, _i32),
                                                ptr(lc, _i32), ptr(ncv, _i64), ptr(ptrs, _i64), ptr(vs, _i32),
                                                ptr(cl, _u8)), "set_feature_sets")

    def project_features(self):
        self._ck(self.L.hexopt_project_features(self.h), "project_features")

    def set_query_budget(self, pops=0):
        self._ck(self.L.hexopt_set_query_budget(self.h, int(pops)), "set_query_budget")

    def query_stats(self):
        """(queries handed to the cooperative pass, candidate leaves, exact fallbacks) of the last
        BVH query pass."""
        w, c, f = C.c_int64(), C.c_int64(), C.c_int64()
        self._ck(self.L.hexopt_query_stats(self.h, C.byref(w), C.byref(c), C.byref(f)), "query_stats")
        return w.value, c.value, f.value

    # ---- Hausdorff
    def hausdorff(self, V0, F0, V1, F1):
        V0 = np.ascontiguousarray(V0, np.float64); V1 = np.ascontiguousarray(V1, np.float64)
        F0 = np.ascontiguousarray(F0, np.int32); F1 = np.ascontiguousarray(F1, np.int32)
        dg, mx, av = C.c_double(), C.c_double(), C.c_double()
        self._ck(self.L.hexopt_hausdorff(self.h, len(V0), ptr(V0, _d), len(F0), ptr(F0, _i32), len(V1), ptr(V1, _d),
                                         len(F1), ptr(F1, _i32), C.byref(dg), C.byref(mx), C.byref(av)), "hausdorff")
        return dg.value, mx.value, av.value

    def hausdorff_uniform(self, V0, F0, V1, F1, n_samples=10_000, seed=0, return_samples=False):
        """Two-sided Hausdorff over n_samples area-uniform device samples of each surface:
        (diag, max, ave), plus the two sample arrays when asked."""
        V0 = np.ascontiguousarray(V0, np.float64); V1 = np.ascontiguousarray(V1, np.float64)
        F0 = np.ascontiguousarray(F0, np.int32); F1 = np.ascontiguousarray(F1, np.int32)
        dg, mx, av = C.c_double(), C.c_double(), C.c_double()
        S0 = np.empty((n_samples, 3)) if return_samples else None
        S1 = np.empty((n_samples, 3)) if return_samples else None
        self._ck(self.L.hexopt_hausdorff_uniform(self.h, len(V0), ptr(V0, _d), len(F0), ptr(F0, _i32), len(V1),
                                                 ptr(V1, _d), len(F1), ptr(F1, _i32), int(n_samples), int(seed),
                                                 C.byref(dg), C.byref(mx), C.byref(av), ptr(S0, _d), ptr(S1, _d)),
                 "hausdorff_uniform")
        out = (dg.value, mx.value, av.value)
        return out + (S0, S1) if return_samples else out

    def set_surface(self, mesh, F):
        F = np.ascontiguousarray(F, np.int32)
        self._ck(self.L.hexopt_set_surface(self.h, mesh, len(F), ptr(F, _i32)), "set_surface")

    def hausdorff_meshes(self):
        n = self.n_meshes
        dg, mx, av = np.empty(n), np.empty(n), np.empty(n)
        self._ck(self.L.hexopt_hausdorff_meshes(self.h, ptr(dg, _d), ptr(mx, _d), ptr(av, _d)), "hausdorff_meshes")
        return dg, mx, av

    def point_face_distance(self, P, V, F):
        P = np.ascontiguousarray(P, np.float64); V = np.ascontiguousarray(V, np.float64)
        F = np.ascontiguousarray(F, np.int32)
        d = np.empty(len(P))
        self._ck(self.L.hexopt_point_face_distance(self.h, len(P), ptr(P, _d), len(V), ptr(V, _d), len(F),
                                                   ptr(F, _i32), ptr(d, _d)), "point_face_distance")
        return d

    # ---- feature alignment
    def fa_begin(self, lamda0=0.05, hausdorff_ratio_t=0.005, **kw):
        p = self.params(**kw)
        self._ck(self.L.hexopt_fa_begin(self.h, C.byref(p), lamda0, hausdorff_ratio_t), "fa_begin")

    def fa_step(self, hausdorff=False, report=True, out=None):
        """One feature-alignment step.  out (C-contiguous float64, nv x 3): also queue the download
        of the step's positions in the same call, overlapped with the step's quality and
        Hausdorff passes; complete after sync()."""
        rep = (FaReport * self.n_meshes)() if report else None
        if out is None:
            self._ck(self.L.hexopt_feature_alignment_step(self.h, int(bool(hausdorff)), rep), "feature_alignment_step")
        else:
            if not (isinstance(out, np.ndarray) and out.dtype == np.float64 and out.flags.c_contiguous):
                raise ValueError("fa_step(out=...) needs a C-contiguous float64 array")
            self._ck(self.L.hexopt_feature_alignment_step_get(self.h, int(bool(hausdorff)), rep, ptr(out, _d)),
                     "feature_alignment_step_get")
        if not report:
            return None
        out = []
        for r in rep:
            d = _rep(r.slim)
            d.update(min_J=r.quality.min_Jacobian, ave_J=r.quality.ave_Jacobian, inverted=r.quality.n_inverted,
                     lamda=r.lamda, hausdorff_diag=r.hausdorff_diag, hausdorff_max=r.hausdorff_max,
                     hausdorff_ave=r.hausdorff_ave)
            out.append(d)
        return out

    def use_graph(self, on=True):
        """True / 1: replay each step as a CUDA graph (line-search rounds as a WHILE node); 2: the
        same with fixed line-search launches (profilable per kernel); False / 0: eager."""
        self._ck(self.L.hexopt_use_graph(self.h, 2 if on == 2 else int(bool(on))), "use_graph")

    # ---- adjoint
    def energy_fwd(self, X=None):
        Xc = None if X is None else np.ascontiguousarray(X, np.float64)
        E = np.empty(self.n_meshes)
        self._ck(self.L.hexopt_energy_fwd(self.h, ptr(Xc, _d), ptr(E, _d)), "energy_fwd")
        return E

    def energy_bwd(self):
        G = np.empty((int(sum(self.nv)), 3))
        self._ck(self.L.hexopt_energy_bwd(self.h, ptr(G, _d)), "energy_bwd")
        return G

    # ---- tuning
    def set_block_size(self, kind, threads):
        self._ck(self.L.hexopt_set_block_size(self.h, kind, threads), "set_block_size")

    def autotune(self):
        self._ck(self.L.hexopt_autotune(self.h), "autotune")
        a, b, v, c = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        self.L.hexopt_get_tuning(self.h, C.byref(a), C.byref(b), C.byref(v), C.byref(c))
        return dict(hex_block=a.value, vertex_block=b.value, vertex_items=v.value, ls_candidates=c.value)

    def sync(self):
        self._ck(self.L.hexopt_sync(self.h), "sync")

    def timer_start(self):
        self._ck(self.L.hexopt_timer_start(self.h), "timer_start")

    def timer_stop(self):
        ms = C.c_double()
        self._ck(self.L.hexopt_timer_stop(self.h, C.byref(ms)), "timer_stop")
        return ms.value

    def time_stage(self, stage, reps=20):
        ms = C.c_double()
        self._ck(self.L.hexopt_time_stage(self.h, stage, reps, C.byref(ms)), "time_stage")
        return ms.value

    def launch_count(self):
        return int(self.L.hexopt_launch_count(self.h))


def _rep(r):
    return dict(energy=r.energy, energy_quality=r.energy_quality, energy_soft=r.energy_soft, cg_error=r.cg_error,
                max_step=r.max_step, step=r.step, cg_iters=r.cg_iters, halvings=r.halvings, status=r.status)
