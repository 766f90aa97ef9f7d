"""Seeded synthetic inputs for the optimiser: structured hex grids, jitter, boundary
identification and triangulated target surfaces.

The reference meshes its inputs with an octree pipeline that is outside the accelerated path;
these generators stand in for its output with meshes of the same kind (pure-hex, corner order of
``hex_ref_shape`` in global_types.h:208-218) and the shapes the workloads name.
"""
from __future__ import annotations

import numpy as np

# Corner order of a hex (global_types.h:208-218, hex_ref_shape).
HEX_REF = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                    [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=np.int64)


def grid_hex(nx: int, ny: int | None = None, nz: int | None = None,
             lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)):
    """Structured nx*ny*nz hex grid over the box [lo, hi].

    Returns V (nv, 3) float64 and H (nh, 8) uint32 in the reference corner order; vertex
    (i, j, k) has id i + (nx+1) * (j + (ny+1) * k).
    """
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    xs = np.linspace(lo[0], hi[0], nx + 1)
    ys = np.linspace(lo[1], hi[1], ny + 1)
    zs = np.linspace(lo[2], hi[2], nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    V = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    H = np.empty((i.size, 8), dtype=np.uint32)
    for c, (di, dj, dk) in enumerate(HEX_REF):
        H[:, c] = (i + di) + (nx + 1) * ((j + dj) + (ny + 1) * (k + dk))
    return V, H


def grid_boundary_mask(nx: int, ny: int | None = None, nz: int | None = None):
    """Boolean mask of the vertices of grid_hex(nx, ny, nz) that lie on the box surface."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    b = (i == 0) | (i == nx) | (j == 0) | (j == ny) | (k == 0) | (k == nz)
    return b.ravel()


def jitter(V: np.ndarray, movable: np.ndarray, h: float, seed: int, sigma: float | None = None,
           uniform: float | None = None) -> np.ndarray:
    """Seeded jitter of the movable vertices: Gaussian with std sigma*h, or uniform in
    [-uniform*h, +uniform*h] per coordinate."""
    rng = np.random.default_rng(seed)
    out = V.copy()
    n = int(movable.sum())
    if sigma is not None:
        d = rng.normal(0.0, sigma * h, size=(n, 3))
    else:
        d = rng.uniform(-uniform * h, uniform * h, size=(n, 3))
    out[movable] += d
    return out


def cube_sphere_surface(m: int):
    """Triangulated surface of the cube [-1, 1]^3 with m x m quads per face (12 m^2 triangles),
    outward oriented.  Returns P (nv, 3), F (nf, 3) int32."""
    idx = -np.ones((m + 1, m + 1, m + 1), dtype=np.int64)
    g = np.arange(m + 1)
    I, J, K = np.meshgrid(g, g, g, indexing="ij")
    surf = (I == 0) | (I == m) | (J == 0) | (J == m) | (K == 0) | (K == m)
    n = int(surf.sum())
    idx[surf] = np.arange(n)
    P = np.stack([I[surf], J[surf], K[surf]], axis=1).astype(np.float64) * (2.0 / m) - 1.0
    faces = []
    a = np.arange(m)
    A, B = np.meshgrid(a, a, indexing="ij")
    A, B = A.ravel(), B.ravel()
    for axis in range(3):
        for side in (0, m):
            def vid(u, v, axis=axis, side=side):
                c = [None, None, None]
                c[axis] = np.full_like(u, side)
                o = [d for d in range(3) if d != axis]
                c[o[0]] = u
                c[o[1]] = v
                return idx[c[0], c[1], c[2]]
            q0, q1, q2, q3 = vid(A, B), vid(A + 1, B), vid(A + 1, B + 1), vid(A, B + 1)
            t = np.concatenate([np.stack([q0, q1, q2], 1), np.stack([q0, q2, q3], 1)])
            faces.append(t)
    F = np.concatenate(faces).astype(np.int64)
    # orient outward
    e1 = P[F[:, 1]] - P[F[:, 0]]
    e2 = P[F[:, 2]] - P[F[:, 0]]
    nrm = np.cross(e1, e2)
    cen = P[F].mean(axis=1)
    flip = (nrm * cen).sum(1) < 0
    F[flip] = F[flip][:, [0, 2, 1]]
    return P, F.astype(np.int32)


def superellipsoid(n_tri_target: int = 200_000, exponent: float = 4.0, radius: float = 0.5,
                   center=(0.5, 0.5, 0.5), float32: bool = True):
    """Triangulated superellipsoid |x|^e + |y|^e + |z|^e = r^e: a cube-sphere lattice pushed
    radially onto the surface.  ~n_tri_target triangles; coordinates rounded to float32 when
    asked (the stored precision of the target)."""
    m = max(2, int(round(np.sqrt(n_tri_target / 12.0))))
    P, F = cube_sphere_surface(m)
    s = (np.abs(P) ** exponent).sum(1) ** (1.0 / exponent)
    Q = P * (radius / s)[:, None] + np.asarray(center)[None, :]
    if float32:
        Q = Q.astype(np.float32).astype(np.float64)
    return Q, F


def cylinder_surface(radius=0.5, height=1.0, segments=64, rings=8, center=(0.0, 0.0, 0.0)):
    """Closed cylinder: `segments` side segments x `rings` rings, fan-triangulated caps
    (64 x 8 gives 578 vertices / 1152 triangles).  Returns V, F (outward) and the vertex ids of
    the two cap circles (the sharp feature curves)."""
    th = np.arange(segments) * (2 * np.pi / segments)
    zs = np.linspace(-height / 2, height / 2, rings + 1)
    ring = np.stack([radius * np.cos(th), radius * np.sin(th)], 1)
    V = [np.column_stack([ring, np.full(segments, z)]) for z in zs]
    V = np.concatenate(V)
    bot_c = len(V)
    top_c = len(V) + 1
    V = np.concatenate([V, [[0, 0, -height / 2], [0, 0, height / 2]]]) + np.asarray(center)
    F = []
    for r in range(rings):
        for s in range(segments):
            a = r * segments + s
            b = r * segments + (s + 1) % segments
            c = (r + 1) * segments + (s + 1) % segments
            d = (r + 1) * segments + s
            F.append([a, b, c])
            F.append([a, c, d])
    for s in range(segments):
        F.append([bot_c, (s + 1) % segments, s])
        F.append([top_c, rings * segments + s, rings * segments + (s + 1) % segments])
    F = np.asarray(F, dtype=np.int32)
    curves = [np.arange(segments), rings * segments + np.arange(segments)]
    return V, F, curves


def cylinder_hex(radius=0.5, height=1.0, n_core=8, n_ring=6, n_z=16):
    """O-grid ("butterfly") hex mesh of a cylinder: a square core of n_core^2 columns surrounded by
    four blocks of n_core x n_ring columns blended onto the circle, extruded in n_z layers.
    Returns V, H, the boundary mask and the ids of the vertices on the two cap circles."""
    c = n_core
    a = radius * 0.45
    g = np.linspace(-a, a, c + 1)
    ids: dict = {}
    pts: list = []

    def nid(xy):
        key = (round(float(xy[0]), 12), round(float(xy[1]), 12))
        if key not in ids:
            ids[key] = len(pts)
            pts.append(key)
        return ids[key]

    def rot(xy, s):  # exact quarter turns
        x, y = xy
        for _ in range(s):
            x, y = -y, x
        return (x, y)

    quads = []
    core = [[nid((g[i], g[j])) for j in range(c + 1)] for i in range(c + 1)]
    for i in range(c):
        for j in range(c):
            quads.append([core[i][j], core[i + 1][j], core[i + 1][j + 1], core[i][j + 1]])
    for s in range(4):
        blk = []
        for t in range(c + 1):
            inner = (a, g[t])
            ang = np.arctan2(inner[1], inner[0])
            outer = (radius * np.cos(ang), radius * np.sin(ang))
            col = []
            for r in range(n_ring + 1):
                w = r / n_ring
                xy = inner if r == 0 else ((1 - w) * inner[0] + w * outer[0], (1 - w) * inner[1] + w * outer[1])
                col.append(nid(rot(xy, s)))
            blk.append(col)
        for t in range(c):
            for r in range(n_ring):
                quads.append([blk[t][r], blk[t + 1][r], blk[t + 1][r + 1], blk[t][r + 1]])
    P2 = np.asarray(pts, dtype=np.float64)
    Q = np.asarray(quads, dtype=np.int64)
    e1 = P2[Q[:, 1]] - P2[Q[:, 0]]
    e2 = P2[Q[:, 3]] - P2[Q[:, 0]]
    cr = e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]
    Q[cr < 0] = Q[cr < 0][:, [0, 3, 2, 1]]
    n2 = len(P2)
    zs = np.linspace(-height / 2, height / 2, n_z + 1)
    V = np.concatenate([np.column_stack([P2, np.full(n2, z)]) for z in zs])
    H = np.empty((len(Q) * n_z, 8), dtype=np.uint32)
    for k in range(n_z):
        blk = slice(k * len(Q), (k + 1) * len(Q))
        H[blk, :4] = Q + k * n2
        H[blk, 4:] = Q + (k + 1) * n2
    rim2 = np.abs(np.hypot(P2[:, 0], P2[:, 1]) - radius) < 1e-9
    bmask = np.zeros(len(V), bool)
    for k in range(n_z + 1):
        bmask[k * n2:(k + 1) * n2] |= rim2
    bmask[:n2] = True
    bmask[n_z * n2:] = True
    caps = [np.nonzero(rim2)[0], n_z * n2 + np.nonzero(rim2)[0]]
    return V, H, bmask, caps


def area_samples(V: np.ndarray, F: np.ndarray, n: int, seed: int) -> np.ndarray:
    """n points uniformly distributed by area over a triangle mesh (seeded)."""
    rng = np.random.default_rng(seed)
    a = np.linalg.norm(np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]]), axis=1)
    f = rng.choice(len(F), size=n, p=a / a.sum())
    r1 = np.sqrt(rng.random(n))
    r2 = rng.random(n)
    w0, w1, w2 = 1 - r1, r1 * (1 - r2), r1 * r2
    return w0[:, None] * V[F[f, 0]] + w1[:, None] * V[F[f, 1]] + w2[:, None] * V[F[f, 2]]


def hex_boundary_quads(H: np.ndarray) -> np.ndarray:
    """Boundary quads of a hex mesh (faces used by one hex), in the hex_face_table corner order
    (global_types.h:154-161), as an (nq, 4) array of vertex ids."""
    HF = np.array([[0, 1, 2, 3], [4, 7, 6, 5], [0, 4, 5, 1], [0, 3, 7, 4], [3, 2, 6, 7], [1, 5, 6, 2]])
    Q = H[:, HF].reshape(-1, 4).astype(np.int64)
    key = np.sort(Q, axis=1)
    _, inv, cnt = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    return Q[cnt[inv.ravel()] == 1]


def grid_boundary_quads(nx: int, ny: int | None = None, nz: int | None = None) -> np.ndarray:
    """Boundary quads of grid_hex(nx, ny, nz) directly from the grid structure (same faces and
    corner order as hex_boundary_quads, without the global face matching)."""
    ny = nx if ny is None else ny
    nz = nx if nz is None else nz
    _, H = grid_hex(nx, ny, nz)
    HF = np.array([[0, 1, 2, 3], [4, 7, 6, 5], [0, 4, 5, 1], [0, 3, 7, 4], [3, 2, 6, 7], [1, 5, 6, 2]])
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    out = []
    for f, sel in ((0, k == 0), (1, k == nz - 1), (2, j == 0), (4, j == ny - 1), (3, i == 0), (5, i == nx - 1)):
        out.append(H[sel][:, HF[f]].astype(np.int64))
    return np.concatenate(out)


def quads_to_tris(Q: np.ndarray) -> np.ndarray:
    """Split boundary quads into (0,1,2), (2,3,0) (grid_hex_meshing.cpp:4290-4313)."""
    return np.concatenate([Q[:, [0, 1, 2]], Q[:, [2, 3, 0]]]).astype(np.int32)


def _ogrid_square_minus_disc(n: int, n_r: int, radius: float, center=(0.5, 0.5)):
    """2-D O-grid of the unit square minus a centred disc: 4n columns around the hole (n per
    square side, uniform in angle on the circle and in arc length on the square), n_r rings from
    the circle (ring 0) to the square (ring n_r), each column a straight blend of the two.
    Vertex (t, j) has id j * 4n + t.  Returns P (4n (n_r+1), 2) and Q (4n n_r, 4), counter-
    clockwise."""
    cx, cy = center
    t = np.arange(4 * n)
    side, u = t // n, (t % n) / n
    outer = np.empty((4 * n, 2))
    outer[side == 0] = np.stack([np.ones((side == 0).sum()), u[side == 0]], 1)
    outer[side == 1] = np.stack([1 - u[side == 1], np.ones((side == 1).sum())], 1)
    outer[side == 2] = np.stack([np.zeros((side == 2).sum()), 1 - u[side == 2]], 1)
    outer[side == 3] = np.stack([u[side == 3], np.zeros((side == 3).sum())], 1)
    th = -np.pi / 4 + (np.pi / 2) * (t / n)
    inner = np.stack([cx + radius * np.cos(th), cy + radius * np.sin(th)], 1)
    w = (np.arange(n_r + 1) / n_r)[:, None, None]
    P = ((1 - w) * inner[None] + w * outer[None]).reshape(-1, 2)  # ring n_r is the square exactly
    j, tt = np.meshgrid(np.arange(n_r), t, indexing="ij")
    j, tt = j.ravel(), tt.ravel()
    t1 = (tt + 1) % (4 * n)
    Q = np.stack([j * 4 * n + tt, (j + 1) * 4 * n + tt, (j + 1) * 4 * n + t1, j * 4 * n + t1], 1)
    e1 = P[Q[:, 1]] - P[Q[:, 0]]
    e2 = P[Q[:, 3]] - P[Q[:, 0]]
    cr = e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]
    Q[cr < 0] = Q[cr < 0][:, [0, 3, 2, 1]]
    return P, Q.astype(np.int64)


def cube_minus_cylinder_hex(n: int = 64, n_r: int = 16, n_z: int = 64, radius: float = 0.25):
    """Structured multi-block hex mesh of the unit cube minus the centred z-axis through-cylinder
    of the given radius: the 2-D O-grid of _ogrid_square_minus_disc (4n columns, n_r rings)
    extruded in n_z layers, 4 n n_r n_z hexes (n = 64, n_r = 16, n_z = 64: 262,144).

    Returns V, H and a dict of vertex sets: 'boundary' (mask), 'corners' (8 ids: square corner
    columns at z = 0 and 1), 'lines' with 'line_curve' (vertices on the 12 cube edges and the
    2 hole circles, corners excluded; curve ids follow cube_minus_cylinder_surface's curves)."""
    P2, Q = _ogrid_square_minus_disc(n, n_r, radius)
    n2 = len(P2)
    zs = np.linspace(0.0, 1.0, n_z + 1)
    V = np.concatenate([np.column_stack([P2, np.full(n2, z)]) for z in zs])
    H = np.empty((len(Q) * n_z, 8), dtype=np.uint32)
    for k in range(n_z):
        blk = slice(k * len(Q), (k + 1) * len(Q))
        H[blk, :4] = Q + k * n2
        H[blk, 4:] = Q + (k + 1) * n2
    T = 4 * n

    def vid(t, j, k):
        return k * n2 + j * T + (np.asarray(t) % T)

    bmask = np.zeros(len(V), bool)
    for k in range(n_z + 1):
        bmask[vid(np.arange(T), 0, k)] = True
        bmask[vid(np.arange(T), n_r, k)] = True
    bmask[:n2] = True
    bmask[n_z * n2:] = True
    corners = np.array([vid(s * n, n_r, k) for k in (0, n_z) for s in range(4)], np.int64)
    lines, lcurve = [], []
    # curves 0-3: vertical cube edges at the square corners s * n
    for s in range(4):
        lines.append(vid(s * n, n_r, np.arange(1, n_z)))
        lcurve.append(np.full(n_z - 1, s))
    # curves 4-11: horizontal cube edges, side s at z = 0 (4 + s) and z = 1 (8 + s)
    for zi, k in enumerate((0, n_z)):
        for s in range(4):
            lines.append(vid(s * n + np.arange(1, n), n_r, k))
            lcurve.append(np.full(n - 1, 4 + 4 * zi + s))
    # curves 12, 13: the hole circles at z = 0 and z = 1 (closed)
    for zi, k in enumerate((0, n_z)):
        lines.append(vid(np.arange(T), 0, k))
        lcurve.append(np.full(T, 12 + zi))
    return V, H, dict(boundary=bmask, corners=corners, lines=np.concatenate(lines).astype(np.int32),
                      line_curve=np.concatenate(lcurve).astype(np.int32))


def cube_minus_cylinder_surface(n: int = 24, n_r: int = 12, n_z: int = 48, radius: float = 0.25):
    """Triangulated surface of the unit cube minus the centred z-axis cylinder: the boundary of
    cube_minus_cylinder_hex(n, n_r, n_z) (24 / 12 / 48: 23,040 triangles), quads split 0-1-2 /
    2-3-0, vertices compacted.  Returns TV, TF, the 14 feature curves as target-vertex chains
    (0-3 vertical cube edges, 4-11 horizontal cube edges, 12-13 hole circles), their closed
    flags, and the 8 cube corners' target-vertex ids."""
    V, H, sets = cube_minus_cylinder_hex(n, n_r, n_z, radius)
    F = quads_to_tris(hex_boundary_quads(H))
    used = np.unique(F)
    remap = -np.ones(len(V), np.int64)
    remap[used] = np.arange(len(used))
    TV = V[used]
    TF = remap[F].astype(np.int32)
    n2 = 4 * n * (n_r + 1)
    T = 4 * n

    def vid(t, j, k):
        return remap[k * n2 + j * T + (np.asarray(t) % T)]

    curves = [vid(s * n, n_r, np.arange(n_z + 1)) for s in range(4)]
    for k in (0, n_z):
        for s in range(4):
            curves.append(vid(s * n + np.arange(n + 1), n_r, k))
    for k in (0, n_z):
        curves.append(vid(np.arange(T), 0, k))
    closed = [False] * 12 + [True, True]
    corners = np.array([vid(s * n, n_r, k) for k in (0, n_z) for s in range(4)], np.int64)
    return TV, TF, [np.asarray(c, np.int32) for c in curves], closed, corners
