"""The benchmark / parity workloads: seeded synthetic inputs of the shapes and sizes the
optimiser is measured on, and the calls that load them into a Context.

  grid_superellipsoid(n)  structured n^3 grid of the unit cube, interior Gaussian jitter, boundary
                          vertices tied by tangent planes to a triangulated superellipsoid
                          (exponent 4, float32 coordinates) -- n = 128 is the 2.1M-hex workload.
  cylinder()              O-grid hex mesh of the r = 0.5, h = 1 cylinder; the two cap circles are
                          feature curves (64 x 8 target triangulation, 1152 triangles).
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


def load(ctx, problems, with_surface=True):
    """Upload a batch of problems and their targets / feature sets into ctx."""
    ctx.upload([(p["V"], p["H"]) for p in problems])
    ctx.set_corners([p["corners"] for p in problems], [p["TV"][:0] if len(p["corners"]) == 0 else None for p in problems])
    for m, p in enumerate(problems):
        ctx.set_target(m, p["TV"], p["TF"])
    ctx.set_feature_sets([p["regular"] for p in problems], [p["lines"] for p in problems],
                         [p["line_curve"] for p in problems], [p["curves"] for p in problems],
                         [p["closed"] for p in problems])
    if with_surface:
        for m, p in enumerate(problems):
            ctx.set_surface(m, p["surface"])
    return ctx
