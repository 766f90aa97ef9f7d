"""The benchmark / parity workloads: seeded synthetic inputs of the shapes and sizes the
optimiser is measured on, and the calls that load them into a Context.

  grid_superellipsoid(n)  structured n^3 grid of the unit cube, interior Gaussian jitter, boundary
                          vertices tied by tangent planes to a triangulated superellipsoid
                          (exponent 4, float32 coordinates) -- n = 128 is the 2.1M-hex workload.
  cylinder()              O-grid hex mesh of the r = 0.5, h = 1 cylinder; the two cap circles are
                          feature curves (64 x 8 target triangulation, 1152 triangles).
  grid_batch(n_meshes)    the batching workload: jittered structured grids with per-axis dims
                          drawn from [12, 96], each tied to its own superellipsoid (exponent in
                          [2, 6], 20k-200k triangles); 256 meshes is the ~40M-hex batch.
  adjoint_problem(n)      the differentiation workload: the n^3 grid with 100 x squared
                          closest-point distance of the boundary vertices as corner terms.
  cube_minus_cylinder()   the mid-size feature workload: the unit cube minus the centred r = 0.25
                          z-axis through-hole, 262,144 hexes, 12 cube edges + 2 hole circles as
                          feature curves with the 8 cube corners, uniform +/-0.1h jitter of the
                          interior vertices, a 23k-triangle target of the same solid.
"""
from __future__ import annotations

import numpy as np

from . import meshgen


def boundary_surface(H):
    """Triangles of the hex mesh boundary (quads split 0-1-2 / 2-3-0)."""
    return meshgen.quads_to_tris(meshgen.hex_boundary_quads(H))


def grid_superellipsoid(n=128, sigma=0.2, seed=0, n_tri=200_000, exponent=4.0):
    V, H = meshgen.grid_hex(n)
    b = meshgen.grid_boundary_mask(n)
    V = meshgen.jitter(V, ~b, 1.0 / n, seed, sigma=sigma)
    TV, TF = meshgen.superellipsoid(n_tri, exponent=exponent, radius=0.5)
    regular = np.nonzero(b)[0].astype(np.int32)
    return dict(name=f"grid{n}_superellipsoid", V=V, H=H, TV=TV, TF=TF, regular=regular,
                lines=np.zeros(0, np.int32), line_curve=np.zeros(0, np.int32), curves=[], closed=[],
                corners=np.zeros(0, np.int32), surface=meshgen.quads_to_tris(meshgen.grid_boundary_quads(n)))


def grid_box_superellipsoid(dims, sigma, seed, n_tri, exponent):
    """One mesh of the batch: an nx x ny x nz grid of the unit cube (jitter in units of the
    smallest cell edge) tied to a superellipsoid of the given exponent."""
    nx, ny, nz = (int(d) for d in dims)
    V, H = meshgen.grid_hex(nx, ny, nz)
    b = meshgen.grid_boundary_mask(nx, ny, nz)
    V = meshgen.jitter(V, ~b, 1.0 / max(nx, ny, nz), seed, sigma=sigma)
    TV, TF = meshgen.superellipsoid(n_tri, exponent=exponent, radius=0.5)
    regular = np.nonzero(b)[0].astype(np.int32)
    return dict(name=f"grid{nx}x{ny}x{nz}_se{exponent:.2f}", V=V, H=H, TV=TV, TF=TF, regular=regular,
                lines=np.zeros(0, np.int32), line_curve=np.zeros(0, np.int32), curves=[], closed=[],
                corners=np.zeros(0, np.int32),
                surface=meshgen.quads_to_tris(meshgen.grid_boundary_quads(nx, ny, nz)))


def grid_batch(n_meshes=256, seed=0, dmin=12, dmax=96, sigma=0.15, tri_min=20_000, tri_max=200_000):
    """The batching workload (seeded): per mesh, per-axis dims uniform in [dmin, dmax], Gaussian
    jitter sigma * h, and a superellipsoid target with exponent uniform in [2, 6] and a
    triangle count uniform in [tri_min, tri_max]."""
    rng = np.random.default_rng(seed)
    out = []
    for m in range(n_meshes):
        dims = rng.integers(dmin, dmax + 1, 3)
        exponent = float(rng.uniform(2.0, 6.0))
        n_tri = int(rng.integers(tri_min, tri_max + 1))
        out.append(grid_box_superellipsoid(dims, sigma, seed * 100003 + m, n_tri, exponent))
    return out


def adjoint_problem(n=96, sigma=0.2, seed=0, n_tri=200_000, weight=100.0):
    """The differentiation workload: grid_superellipsoid(n) whose boundary vertices carry corner
    terms weight * |x - cp(x)|^2 (cp = closest point on the target, recomputed wherever the
    energy is evaluated); no tangent-plane or line terms."""
    p = grid_superellipsoid(n, sigma=sigma, seed=seed, n_tri=n_tri)
    p = dict(p, name=f"grid{n}_adjoint", corners=p["regular"], regular=np.zeros(0, np.int32), weight=weight)
    return p


def cylinder(n_core=8, n_ring=6, n_z=16):
    V, H, bmask, caps = meshgen.cylinder_hex(n_core=n_core, n_ring=n_ring, n_z=n_z)
    TV, TF, curves = meshgen.cylinder_surface()
    lines = np.concatenate(caps).astype(np.int32)
    line_curve = np.concatenate([np.zeros(len(caps[0])), np.ones(len(caps[1]))]).astype(np.int32)
    on_line = np.zeros(len(V), bool)
    on_line[lines] = True
    regular = np.nonzero(bmask & ~on_line)[0].astype(np.int32)
    return dict(name="cylinder", V=V, H=H, TV=TV, TF=TF, regular=regular, lines=lines, line_curve=line_curve,
                curves=[np.asarray(c, np.int32) for c in curves], closed=[True, True],
                corners=np.zeros(0, np.int32), surface=boundary_surface(H))


def cube_minus_cylinder(n=64, n_r=16, n_z=64, jitter=0.1, seed=0, target=(24, 12, 48)):
    """The unit cube minus the centred z-axis through-cylinder of radius 0.25 as a structured
    O-grid hex mesh (4 n n_r n_z hexes; 262,144 at the defaults), interior vertices jittered
    uniformly in [-jitter h, +jitter h] per coordinate (h = 1/n, seeded).  Feature curves: the 12
    cube edges and the 2 hole circles of the target (a 23,040-triangle triangulation of the same
    solid at another resolution); the hex vertices on them are line vertices, the 8 cube corners
    are corner vertices tied to the target's corners, every other boundary vertex gets a tangent
    plane."""
    V, H, sets = meshgen.cube_minus_cylinder_hex(n, n_r, n_z)
    b = sets["boundary"]
    V = meshgen.jitter(V, ~b, 1.0 / n, seed, uniform=jitter)
    TV, TF, curves, closed, tcorners = meshgen.cube_minus_cylinder_surface(*target)
    special = np.zeros(len(V), bool)
    special[sets["lines"]] = True
    special[sets["corners"]] = True
    regular = np.nonzero(b & ~special)[0].astype(np.int32)
    return dict(name=f"cube_minus_cylinder_{len(H)}", V=V, H=H, TV=TV, TF=TF, regular=regular,
                lines=sets["lines"], line_curve=sets["line_curve"], curves=curves, closed=closed,
                corners=sets["corners"].astype(np.int32), corner_pos=TV[tcorners],
                surface=boundary_surface(H))


def load(ctx, problems, with_surface=True):
    """Upload a batch of problems and their targets / feature sets into ctx."""
    ctx.upload([(p["V"], p["H"]) for p in problems])
    ctx.set_corners([p["corners"] for p in problems],
                    [p["corner_pos"] if len(p["corners"]) else np.zeros((0, 3)) for p in problems])
    for m, p in enumerate(problems):
        ctx.set_target(m, p["TV"], p["TF"])
    ctx.set_feature_sets([p["regular"] for p in problems], [p["lines"] for p in problems],
                         [p["line_curve"] for p in problems], [p["curves"] for p in problems],
                         [p["closed"] for p in problems])
    if with_surface:
        for m, p in enumerate(problems):
            ctx.set_surface(m, p["surface"])
    return ctx
