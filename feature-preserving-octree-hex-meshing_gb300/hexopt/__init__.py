"""hexopt -- GB300 (sm_103a) implementation of the octree hex mesher's geometric-optimisation hot
path, driven through the C ABI of libhexopt_gpu.so.

The module-level functions mirror the reference entry points they replace:

    scaled_jacobian(V, H)                      bool scaled_jacobian(Mesh&, Mesh_Quality&)   global_functions.h:81
    slim_m_opt(problem, iters, ...)            optimization::slim_m_opt(Tetralize_Set&, ...)  optimization.h:32
    signed_distance_pseudonormal(P, TV, TF)    igl::signed_distance_pseudonormal via build_aabb_tree
    compute(V0, F0, V1, F1)                    void compute(const Mesh&, const Mesh&, diag, max, ave)
                                                                                            metro_hausdorff.h:37
    hausdorff_uniform(V0, F0, V1, F1, n)       the same check over n area-uniform samples per surface
Everything runs on the GPU; a missing library or device raises instead of falling back.
"""
from ._lib import FP64, MIXED, SYMMETRIC_DIRICHLET, Context, HexoptError, load, read_hex_mesh, write_hex_mesh  # noqa: F401
from . import meshgen  # noqa: F401

_ctx = None


def _context():
    global _ctx
    if _ctx is None:
        _ctx = Context(0)
    return _ctx


def scaled_jacobian(V, H):
    """Mesh_Quality of a hex mesh: min/ave/deviation of the per-hex minimum corner scaled
    Jacobian, per-corner V_Js and per-hex H_Js, and the number of inverted hexes."""
    c = _context()
    c.upload([(V, H)])
    vj, hj, q = c.scaled_jacobian(per_corner=True)
    return dict(min_Jacobian=q[0]["min"], ave_Jacobian=q[0]["ave"], deviation_Jacobian=q[0]["dev"],
                V_Js=vj, H_Js=hj, n_inverted=q[0]["inverted"])


def slim_m_opt(V, H, iters, h_flag=None, ids_C=(), C=(), lamda_C=0.0, ids_T=(), normal_T=(), dis_T=(),
               lamda_T=0.0, ids_L=(), Axa_L=(), origin_L=(), lamda_L=0.0, weight_opt=0.001,
               precision=FP64, **kw):
    """slim_precompute + `iters` fixed SLIM iterations on the 8 corner tets of every hex, with
    the Feature_Constraints soft terms.  Returns (V_o, a_L, report)."""
    import numpy as np
    c = _context()
    c.upload([(V, H)], h_flag=h_flag)
    c.set_corners([ids_C], [np.asarray(C, float).reshape(-1, 3)])
    c.set_tangents([ids_T], [np.asarray(normal_T, float).reshape(-1, 3)], [dis_T])
    c.set_lines([ids_L], [np.asarray(Axa_L, float).reshape(-1, 3)], [np.asarray(origin_L, float).reshape(-1, 3)])
    c.set_weights(lamda_C, lamda_T, lamda_L)
    rep = c.slim_m_opt(iters, weight_opt=weight_opt, precision=precision, **kw)
    return c.get_positions(), c.curve_params(len(ids_L)), rep[0]


def signed_distance_pseudonormal(P, TV, TF):
    """S, I, C, N of igl::signed_distance_pseudonormal against the triangle mesh (TV, TF)."""
    import numpy as np
    c = _context()
    V, H = meshgen.grid_hex(1)  # a context needs a mesh; the query does not use it
    c.upload([(V, H)])
    c.set_target(0, TV, TF)
    return c.signed_distance(0, np.asarray(P, float))


def compute(V0, F0, V1, F1):
    """Two-sided vertex-sampled Hausdorff (diag, max, ave) as metro_hausdorff's compute()."""
    return _context().hausdorff(V0, F0, V1, F1)


def hausdorff_uniform(V0, F0, V1, F1, n_samples=10_000, seed=0, ctx=None):
    """Two-sided Hausdorff over n_samples area-uniform samples of each surface instead of the
    vertices, sampled and evaluated on the device (hexopt_hausdorff_uniform): the sample distance
    is PointDistanceEP minimised over the other surface, and the rules are those of the vertex mode
    (metro_hausdorff.cpp:358-506).  Returns (diag, max, ave)."""
    c = ctx or _context()
    return c.hausdorff_uniform(V0, F0, V1, F1, n_samples=n_samples, seed=seed)
