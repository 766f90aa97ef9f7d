"""hexopt_point_face_distance_noalloc against the allocating hexopt_point_face_distance.

Two calls in a row on caller-owned device arrays (two different surfaces and point sets) must
give the allocating entry point's distances bit for bit, the second call must leave the device's
free memory unchanged (every buffer it needs is pre-allocated here, and its own scratch is the
static array set up by the first call), and a surface over the static scratch's limit must be
rejected with a message naming the sizes, before any device work.  Collected last (own file);
it passes alone and after the rest of the suite.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_FACES = 1 << 18


@pytest.fixture(scope="module")
def env():
    import build
    build.build()
    import torch
    import hexopt
    from hexopt import _lib
    ctx = hexopt.Context(0)
    yield torch, hexopt, _lib, ctx
    ctx.close()


def _case(meshgen, kind, seed):
    rng = np.random.default_rng(seed)
    if kind == "superellipsoid":
        V, F = meshgen.superellipsoid(20000)
        P = rng.uniform(-0.3, 1.3, (30000, 3))
    else:
        V, F = meshgen.cylinder_surface()[:2]
        P = rng.normal(0.0, 0.6, (20000, 3))
    return np.ascontiguousarray(V, np.float64), np.ascontiguousarray(F, np.int32), np.ascontiguousarray(P, np.float64)


def test_noalloc_matches_allocating_entry_point(env):
    torch, hexopt, _lib, ctx = env
    from hexopt import meshgen
    cases = [_case(meshgen, "superellipsoid", 1), _case(meshgen, "cylinder", 2)]
    dev = torch.device("cuda", 0)
    bufs = []
    for V, F, P in cases:  # every device buffer up front
        bufs.append(dict(V=torch.from_numpy(V).to(dev), F=torch.from_numpy(F).to(dev), P=torch.from_numpy(P).to(dev),
                         D=torch.full((len(P),), -1.0, dtype=torch.float64, device=dev)))
    stream = torch.cuda.current_stream(dev).cuda_stream
    torch.cuda.synchronize(dev)

    def call(b):
        _lib.point_face_distance_noalloc(b["P"].data_ptr(), b["P"].shape[0], b["V"].data_ptr(), b["V"].shape[0],
                                         b["F"].data_ptr(), b["F"].shape[0], b["D"].data_ptr(), device=0,
                                         stream=stream)

    before = torch.cuda.mem_get_info(dev)[0]
    call(bufs[0])  # first call on the device: sets the static scratch up
    torch.cuda.synchronize(dev)
    free0 = torch.cuda.mem_get_info(dev)[0]
    # the static scratch is reserved by this first call under lazy module loading, or was already
    # when the library was loaded under eager loading; report which
    print(f"\nfirst no-alloc call changed free device memory by {(before - free0) / 2**20:.1f} MiB")
    call(bufs[1])
    call(bufs[0])
    torch.cuda.synchronize(dev)
    free1 = torch.cuda.mem_get_info(dev)[0]
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes across no-alloc calls"
    for (V, F, P), b in zip(cases, bufs):
        want = ctx.point_face_distance(P, V, F)
        got = b["D"].cpu().numpy()
        assert np.array_equal(got, want), float(np.abs(got - want).max())


def test_noalloc_rejects_oversize_surface(env):
    torch, hexopt, _lib, ctx = env
    dev = torch.device("cuda", 0)
    tiny = torch.zeros(16, dtype=torch.float64, device=dev)
    with pytest.raises(_lib.HexoptError, match=r"262145 faces exceed the static scratch \(80 MiB, up to 262144"):
        # rejected on the host from the sizes alone; the small buffer is never read
        _lib.point_face_distance_noalloc(tiny.data_ptr(), 1, tiny.data_ptr(), 3, tiny.data_ptr(), MAX_FACES + 1,
                                         tiny.data_ptr(), device=0, stream=0)
