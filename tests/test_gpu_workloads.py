"""The differentiation, batching and uniform-sample Hausdorff workloads at test sizes.

- Adjoint through the projection: symmetric Dirichlet + 100 x squared closest-point distance of
  the boundary vertices (corner terms at the closest points of the evaluation point).  The
  gradient must match FP64 central differences (h = 1e-6, closest points recomputed at every
  perturbed point) within 1e-4 relative over the seeded coordinates (|g_fd - g| / |g| of the
  sampled vectors), and each coordinate within 1e-3.  The differences are Richardson-extrapolated
  from h and h/2: near-degenerate tets of the jittered grid give |J^-1|^2 third derivatives
  large enough that a single central difference at h = 1e-6 carries ~1e-4 of truncation error.
- Batching: meshes of uneven size with their own targets, advanced together by the
  feature-alignment step, give each mesh the result of running it alone.  Float atomics make the
  vertex sums order-dependent and the truncated CG + line search amplify that to a few 1e-9 after
  two steps, so positions are compared to 1e-7 (a tenth of the 1e-6 x diagonal parity bar) and
  the reported scalars to 1e-7 relative, instead of bit equality.
- Uniform-sample Hausdorff: the GPU sample distances against the oracle's on the same samples.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hx():
    import build
    build.build()
    import hexopt
    return hexopt


def test_adjoint_through_projection_matches_central_differences(hx):
    from hexopt import workloads
    p = workloads.adjoint_problem(20, n_tri=20000)
    V, b = p["V"], p["corners"]
    ctx = hx.Context(0)
    try:
        ctx.upload([(V, p["H"])])
        ctx.set_target(0, p["TV"], p["TF"])
        C = ctx.signed_distance(0, V[b])[2]
        ctx.set_corners([b], [C])
        ctx.set_weights(p["weight"], 0.0, 0.0)
        ctx.slim_precompute(precision=hx.FP64, weight_opt=0.001)
        ctx.energy_fwd(V)
        G = ctx.energy_bwd()
        scale = float(np.sqrt(np.mean(G ** 2)))
        slot = {int(v): k for k, v in enumerate(b)}
        rng = np.random.default_rng(7)
        # half the coordinates on boundary vertices (the projection term), half anywhere
        vs = np.concatenate([rng.choice(b, 60, replace=False), rng.choice(len(V), 60, replace=False)])
        h = 1e-6
        worst = 0.0
        gf, ga = [], []
        for v in vs:
            ax = int(rng.integers(0, 3))
            def central(step):
                fd = []
                for sgn in (1.0, -1.0):
                    Vp = V.copy()
                    Vp[v, ax] += sgn * step
                    if int(v) in slot:
                        Cp = C.copy()
                        Cp[slot[int(v)]] = ctx.signed_distance(0, Vp[v:v + 1])[2][0]
                        ctx.set_corners([b], [Cp])
                    fd.append(ctx.energy_fwd(Vp)[0])
                    if int(v) in slot:
                        ctx.set_corners([b], [C])
                return (fd[0] - fd[1]) / (2 * step)
            g_fd = (4 * central(h / 2) - central(h)) / 3
            gf.append(g_fd)
            ga.append(G[v, ax])
            worst = max(worst, abs(g_fd - G[v, ax]) / max(abs(G[v, ax]), 1e-2 * scale))
        gf, ga = np.array(gf), np.array(ga)
        assert np.linalg.norm(gf - ga) / np.linalg.norm(ga) <= 1e-4
        assert worst <= 1e-3, worst
    finally:
        ctx.close()


def test_batch_of_uneven_meshes_equals_individual_runs(hx):
    from hexopt import workloads
    probs = workloads.grid_batch(4, seed=3, dmin=5, dmax=14, tri_min=2000, tri_max=6000)
    def run(ps, steps=2):
        ctx = hx.Context(0)
        try:
            workloads.load(ctx, ps)
            ctx.fa_begin(lamda0=0.05, precision=hx.FP64, weight_opt=0.001)
            for _ in range(steps):
                reps = ctx.fa_step(hausdorff=True)
            return ctx.get_positions(), reps
        finally:
            ctx.close()
    Vb, rb = run(probs)
    off = 0
    for m, p in enumerate(probs):
        Vm, rm = run([p])
        n = len(p["V"])
        np.testing.assert_allclose(Vb[off:off + n], Vm, rtol=0, atol=1e-7)
        for k in ("min_J", "energy", "hausdorff_max"):
            assert rb[m][k] == pytest.approx(rm[0][k], rel=1e-7, abs=1e-12), (m, k)
        off += n


def test_uniform_sample_hausdorff_matches_oracle(hx, oracle):
    """Device-drawn area-uniform samples: their distances to the other surface against the
    oracle's on the same samples, and the samples themselves against a numpy restatement of the
    SplitMix64 draw (the same faces and barycentric weights)."""
    from hexopt import workloads
    p = workloads.cylinder()
    V0, F0 = p["TV"], p["TF"]
    V1, F1 = p["V"], p["surface"]
    ctx = hx.Context(0)
    try:
        D, mx, ave, S0, S1 = ctx.hausdorff_uniform(V0, F0, V1, F1, n_samples=10_000, seed=5, return_samples=True)
    finally:
        ctx.close()
    np.testing.assert_allclose(S0, splitmix_samples(V0, F0, 10_000, 5), rtol=0, atol=1e-12)
    np.testing.assert_allclose(S1, splitmix_samples(V1, F1, 10_000, 5 + 3 * 10_000), rtol=0, atol=1e-12)
    d0 = oracle.point_face_distance(S0, V1, F1)
    d1 = oracle.point_face_distance(S1, V0, F0)
    k0, k1 = d0[d0 < D], d1[d1 < D]
    assert mx == pytest.approx(max(k0.max(), k1.max()), rel=1e-12)
    assert ave == pytest.approx(max(k0.mean(), k1.mean()), rel=1e-12)


def splitmix_samples(V, F, n, seed):
    """The device's sampling rule in numpy (test restatement)."""
    M = np.uint64(0xFFFFFFFFFFFFFFFF)

    def mix(x):
        with np.errstate(over="ignore"):
            z = (x + np.uint64(0x9E3779B97F4A7C15)) & M
            z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & M
            z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & M
            return z ^ (z >> np.uint64(31))
    i = np.arange(n, dtype=np.uint64)
    base = np.uint64(seed) + np.uint64(3) * i
    u = [(mix(base + np.uint64(k)) >> np.uint64(11)).astype(np.float64) / 9007199254740992.0 for k in range(3)]
    e1 = V[F[:, 1]] - V[F[:, 0]]
    e2 = V[F[:, 2]] - V[F[:, 0]]
    area = np.linalg.norm(np.cross(e1, e2), axis=1)
    cdf = np.cumsum(area)
    f = np.searchsorted(cdf, u[0] * cdf[-1], side="right")
    r1 = np.sqrt(u[1])
    w0, w1, w2 = 1 - r1, r1 * (1 - u[2]), r1 * u[2]
    return w0[:, None] * V[F[f, 0]] + w1[:, None] * V[F[f, 1]] + w2[:, None] * V[F[f, 2]]

def _shuffled(p, seed):
    """The same problem with its vertices and hexes renumbered at random (and every id remapped)."""
    rng = np.random.default_rng(seed)
    nv, nh = len(p["V"]), len(p["H"])
    vp = rng.permutation(nv)          # new vertex i is old vertex vp[i]
    inv = np.empty(nv, np.int64)
    inv[vp] = np.arange(nv)
    hp = rng.permutation(nh)
    q = dict(p)
    q["V"] = p["V"][vp]
    q["H"] = inv[p["H"][hp].astype(np.int64)].astype(np.uint32)
    for k in ("regular", "lines", "corners"):
        q[k] = inv[np.asarray(p[k], np.int64)].astype(np.int32)
    q["surface"] = inv[np.asarray(p["surface"], np.int64)].astype(np.int32)
    return q, vp


@pytest.mark.parametrize("morton", [1, 0, 2])
def test_shuffled_numbering_gives_the_same_result(hx, morton):
    """The optimiser's result does not depend on how the caller numbers vertices and hexes: a
    randomly renumbered cube-minus-cylinder mesh (features, corners, Hausdorff surface remapped)
    gives the positions of the original numbering after 2 feature-alignment steps, with the
    device's Morton ordering on (both numberings reach the same device order), off, and chosen
    by the numbering's coherence."""
    from hexopt import workloads
    p = workloads.cube_minus_cylinder(n=16, n_r=6, n_z=12)
    q, vp = _shuffled(p, 11)

    def run(pr):
        ctx = hx.Context(0)
        try:
            ctx.set_ordering(morton)
            workloads.load(ctx, [pr])
            ctx.fa_begin(lamda0=0.05, precision=hx.FP64, weight_opt=0.001)
            for _ in range(2):
                r = ctx.fa_step(hausdorff=True)[0]
            vj = ctx.scaled_jacobian(per_corner=True)[0]
            return ctx.get_positions(), r, vj
        finally:
            ctx.close()
    Va, ra, vja = run(p)
    Vb, rb, vjb = run(q)
    d = float(np.linalg.norm(p["V"].max(0) - p["V"].min(0)))
    assert np.abs(Vb - Va[vp]).max() <= 1e-9 * d
    assert rb["min_J"] == pytest.approx(ra["min_J"], abs=1e-9)
    assert rb["hausdorff_max"] == pytest.approx(ra["hausdorff_max"], rel=1e-9)
    assert np.isclose(np.sort(vjb), np.sort(vja), atol=1e-9).all()


def test_adjoint_96_all_coordinates_match_central_differences(hx):
    """The differentiation workload at full size: the 96^3 grid (884,736 hexes), symmetric
    Dirichlet over the corner tets + 100 x squared closest-point distance of the boundary vertices,
    FP64.  All 1,000 seeded coordinates are checked, none dropped: each against a fourth-order
    central difference (-f(x+2h) + 8f(x+h) - 8f(x-h) + f(x-2h)) / 12h, with h refined from 1e-6 by
    factors of 4 until two successive estimates agree to 1e-6 relative (vertices of nearly flat tets,
    whose energy varies on a scale far below 1e-6, need the smaller steps).  Aggregate relative
    error |g_fd - g| / |g| <= 1e-4."""
    from hexopt import workloads
    p = workloads.adjoint_problem(96)
    V, b = p["V"], p["corners"]
    ctx = hx.Context(0)
    try:
        ctx.upload([(V, p["H"])])
        ctx.set_target(0, p["TV"], p["TF"])
        C = ctx.signed_distance(0, V[b])[2]
        ctx.set_corners([b], [C])
        ctx.set_weights(p["weight"], 0.0, 0.0)
        ctx.slim_precompute(precision=hx.FP64, weight_opt=0.001)
        ctx.energy_fwd(V)
        G = ctx.energy_bwd()
        slot = {int(v): k for k, v in enumerate(b)}
        rng = np.random.default_rng(1234)
        coords = rng.choice(len(V) * 3, size=1000, replace=False)

        def f(v, ax, dx):
            Vp = V.copy()
            Vp[v, ax] += dx
            if v in slot:
                Cp = C.copy()
                Cp[slot[v]] = ctx.signed_distance(0, Vp[v:v + 1])[2][0]
                ctx.set_corners([b], [Cp])
            e = ctx.energy_fwd(Vp)[0]
            if v in slot:
                ctx.set_corners([b], [C])
            return e

        def d4(v, ax, h):
            return (-f(v, ax, 2 * h) + 8 * f(v, ax, h) - 8 * f(v, ax, -h) + f(v, ax, -2 * h)) / (12 * h)

        gf, ga, steps = [], [], []
        for c in coords:
            v, ax = divmod(int(c), 3)
            h = 1e-6
            prev = d4(v, ax, h)
            for _ in range(4):
                h /= 4
                cur = d4(v, ax, h)
                done = abs(cur - prev) <= 1e-6 * max(abs(cur), 1e-12)
                prev = cur
                if done:
                    break
            gf.append(prev)
            ga.append(G[v, ax])
            steps.append(h)
    finally:
        ctx.close()
    gf, ga = np.array(gf), np.array(ga)
    rel = float(np.linalg.norm(gf - ga) / np.linalg.norm(ga))
    print(f"\n[adjoint 96^3] aggregate rel err {rel:.3e} over {len(gf)} coordinates; "
          f"steps used: {sorted(set(steps))}")
    assert rel <= 1e-4


@pytest.mark.parametrize("graph", [False, True])
def test_async_position_transfers_match_synchronous(hx, graph):
    """Streaming positions through the optimiser with the asynchronous transfers (uploads and
    downloads on the copy stream, overlapping the steps; one synchronisation at the end) gives,
    step for step, the positions of the synchronous set_positions / fa_step / get_positions
    sequence, with and without graph replay, whether the download is a call of its own or is
    queued inside the step's call (fa_step(out=...), staged beside the step's tail), and when each
    step's input is the previous step's download.  Page-locked buffers (torch) and pageable numpy
    buffers both work."""
    import torch
    from hexopt import workloads
    p = workloads.grid_superellipsoid(n=16, n_tri=4000)
    rng = np.random.default_rng(3)
    h = 1.0 / 16
    inputs = [np.ascontiguousarray(p["V"] + (0.02 * h * k) * rng.standard_normal(p["V"].shape) *
                                   np.isin(np.arange(len(p["V"])), p["regular"], invert=True)[:, None])
              for k in range(4)]
    ctx = hx.Context(0)
    try:
        workloads.load(ctx, [p])
        ctx.use_graph(graph)
        ctx.fa_begin(lamda0=0.05, precision=hx.FP64, weight_opt=0.001)
        ref = []
        for V in inputs:
            ctx.set_positions(V)
            ctx.fa_step(hausdorff=True, report=False)
            ref.append(ctx.get_positions())
        for pinned in (True, False):
            if pinned:
                ins = [torch.from_numpy(V).pin_memory().numpy() for V in inputs]
                outs = [torch.empty(V.shape, dtype=torch.float64).pin_memory().numpy() for V in inputs]
            else:
                ins = [V.copy() for V in inputs]
                outs = [np.empty_like(V) for V in inputs]
            d = float(np.linalg.norm(p["V"].max(0) - p["V"].min(0)))
            # the download queued by a separate call after the step, then inside the step's own
            # call (staged once the line search has applied the step, beside the step's tail)
            for fused in (False, True):
                ctx.fa_begin(lamda0=0.05, precision=hx.FP64, weight_opt=0.001)
                for out in outs:
                    out.fill(np.nan)
                for V, out in zip(ins, outs):
                    ctx.set_positions_async(V)
                    if fused:
                        ctx.fa_step(hausdorff=True, report=False, out=out)
                    else:
                        ctx.fa_step(hausdorff=True, report=False)
                        ctx.get_positions_async(out)
                ctx.sync()
                for k, (a, b) in enumerate(zip(outs, ref)):
                    assert np.abs(a - b).max() <= 1e-9 * d, (pinned, fused, k, float(np.abs(a - b).max()))
            # chained as the end-to-end loop runs it: each step's input is the previous download
            ctx.fa_begin(lamda0=0.05, precision=hx.FP64, weight_opt=0.001)
            chain = ins[0].copy() if not pinned else torch.from_numpy(ins[0].copy()).pin_memory().numpy()
            got = []
            for _ in range(3):
                ctx.set_positions_async(chain)
                ctx.fa_step(hausdorff=True, report=False, out=chain)
                ctx.sync()
                got.append(chain.copy())
            ctx.fa_begin(lamda0=0.05, precision=hx.FP64, weight_opt=0.001)
            ctx.set_positions(ins[0])
            for k in range(3):
                ctx.fa_step(hausdorff=True, report=False)
                want = ctx.get_positions()
                assert np.abs(got[k] - want).max() <= 1e-9 * d, (pinned, "chained", k, float(np.abs(got[k] - want).max()))
    finally:
        ctx.close()
