"""GPU BVH queries on adversarial geometry against the CPU oracle.

The GPU traversal screens leaves in FP32 and evaluates in FP64 only the leaves whose FP32 lower
bound is within the smallest FP32 upper bound seen.  These cases aim at the places where the FP32
bounds are least sure: obtuse, thin and tiny triangles, queries within a hair of an edge line or
a vertex, queries exactly in a triangle's plane, and the vertex wedges where PointDistanceEP
follows the first failing edge test instead of the nearest feature.  Each result has to match
the oracle's exact FP64 search: point-to-surface distance (PointDistanceEP, the Hausdorff metric)
and closest point (the projection metric) to 1e-12 absolute on a unit-sized surface.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import build
    build.build()
    import hexopt
    c = hexopt.Context(0)
    yield c
    c.close()


def crumpled_soup(rng, n=36):
    """Height-field grid with random diagonals and a fifth of the vertices pulled 97-99.9% of the
    way to a neighbour (slivers, needles and obtuse angles), plus free-standing obtuse triangles."""
    x, y = np.meshgrid(np.linspace(0, 1, n), np.linspace(0, 1, n), indexing="ij")
    z = 0.04 * rng.standard_normal(x.shape)
    V = np.stack([x, y, z], -1).reshape(-1, 3)
    idx = lambda i, j: i * n + j  # noqa: E731
    F = []
    for i in range(n - 1):
        for j in range(n - 1):
            a, b, c, d = idx(i, j), idx(i + 1, j), idx(i + 1, j + 1), idx(i, j + 1)
            if rng.random() < 0.5:
                F += [(a, b, c), (a, c, d)]
            else:
                F += [(a, b, d), (b, c, d)]
    V = V.copy()
    pull = rng.choice(n * n, n * n // 5, replace=False)
    for v in pull:
        i, j = divmod(int(v), n)
        i2, j2 = min(max(i + rng.integers(-1, 2), 0), n - 1), min(max(j + rng.integers(-1, 2), 0), n - 1)
        t = rng.uniform(0.97, 0.999)
        V[v] = V[v] + t * (V[idx(i2, j2)] - V[v])
    # free-standing obtuse triangles (apex near the midpoint of the long edge)
    extra = []
    for k in range(200):
        p0 = rng.uniform(0, 1, 3); e = rng.normal(size=3); e /= np.linalg.norm(e)
        L = rng.uniform(0.01, 0.1)
        p1 = p0 + L * e
        off = rng.normal(size=3); off -= off.dot(e) * e; off /= np.linalg.norm(off)
        p2 = p0 + rng.uniform(0.3, 0.7) * L * e + rng.uniform(1e-4, 0.05) * L * off
        extra.append((p0, p1, p2))
    base = len(V)
    V = np.concatenate([V, np.array(extra).reshape(-1, 3)])
    F = np.array(F + [(base + 3 * k, base + 3 * k + 1, base + 3 * k + 2) for k in range(len(extra))], np.int32)
    return V, F


def hard_queries(rng, V, F, m=6000):
    """Points near edge lines, near vertices, in the plane, in vertex wedges, and at random."""
    P = []
    f = rng.integers(0, len(F), m)
    T = V[F[f]]
    nrm = np.cross(T[:, 1] - T[:, 0], T[:, 2] - T[:, 0])
    nl = np.linalg.norm(nrm, axis=1, keepdims=True)
    nrm = np.where(nl > 0, nrm / np.maximum(nl, 1e-300), 0.0)
    k = rng.integers(0, 3, m)
    a, b = T[np.arange(m), k], T[np.arange(m), (k + 1) % 3]
    e = b - a
    el = np.linalg.norm(e, axis=1, keepdims=True)
    inplane = np.cross(nrm, e / np.maximum(el, 1e-300))
    t = rng.uniform(-0.2, 1.2, (m, 1))
    eps = (10.0 ** rng.uniform(-12, -4, (m, 1))) * rng.choice([-1, 1], (m, 1)) * el
    h = rng.choice([0.0, 1e-9, 1e-3, 0.02, 0.2], (m, 1)) * rng.choice([-1, 1], (m, 1))
    P.append(a + t * e + eps * inplane + h * nrm)                         # near an edge line
    c = T[np.arange(m), k]
    out = -(T[:, 0] + T[:, 1] + T[:, 2] - 3 * c)                         # away from the centroid
    P.append(c + rng.uniform(0, 0.05, (m, 1)) * out + rng.uniform(-0.01, 0.01, (m, 1)) * nrm)  # vertex wedges
    bc = rng.dirichlet([1, 1, 1], m)
    P.append(np.einsum("mi,mij->mj", bc, T))                              # in the plane, inside
    P.append(rng.uniform(-0.3, 1.3, (m, 3)))                              # anywhere
    return np.concatenate(P)


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_point_face_distance_adversarial(ctx, oracle, seed):
    rng = np.random.default_rng(seed)
    V, F = crumpled_soup(rng)
    P = hard_queries(rng, V, F)
    d = ctx.point_face_distance(P, V, F)
    ref = oracle.point_face_distance(P, V, F)
    err = np.abs(d - ref)
    assert err.max() <= 1e-12, (int(err.argmax()), float(err.max()))


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_closest_point_adversarial(ctx, oracle, seed):
    from hexopt import meshgen
    rng = np.random.default_rng(10 + seed)
    V, F = crumpled_soup(rng)
    P = hard_queries(rng, V, F)
    ctx.upload([meshgen.grid_hex(1)])
    ctx.set_target(0, V, F)
    S, I, Cc, N = ctx.signed_distance(0, P)
    So, Io, Co, No = oracle.signed_distance(V, F, P)
    # distance and closest point everywhere; the queries sit on shared edges and vertices on
    # purpose, where several faces are exactly equally close and either is a correct answer, so
    # sign and pseudonormal are compared where the two searches picked the same face
    # (at a tie each face's own formula rounds the shared closest point slightly differently)
    assert np.abs(np.abs(S) - np.abs(So)).max() <= 1e-12
    same = I == Io
    assert same.mean() > 0.5
    assert np.abs(Cc - Co)[same].max() <= 1e-12
    assert np.abs(Cc - Co)[~same].max(initial=0) <= 1e-9
    np.testing.assert_allclose(S[same], So[same], rtol=0, atol=1e-12)
    np.testing.assert_allclose(N[same], No[same], rtol=0, atol=1e-12)
    assert (np.sign(S) == np.sign(So)).mean() > 0.99
