"""The untangling and smoothing stages against the reference's own optimization::pipeline2 (tests/golden/
untangle_*.npz, made by oracle/_ref): rigidDeformCubes, then the adaptive gluing solve of
glueInternalNodes -- per-hex vertex copies, boundary copies held, glue weight schedule of
slim_solve2, CONFORMAL energy, edge-averaged cuboid reference shapes -- until the glued mesh's
minimum scaled Jacobian is > 0 or 50 iterations.  The success flag must match exactly, the glued
positions within 1e-6 of the bbox diagonal and the minimum scaled Jacobian within 1e-6 -- or,
where the reference itself moves further under 1e-15 relative input noise (the fixture records
that spread; the case that runs all 50 iterations, its glue weight grown to ~1e9, moves by ~6e-3
of the diagonal), within three times the reference's own spread."""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hx():
    import build
    build.build()
    import hexopt
    return hexopt


def diag_of(V):
    return float(np.linalg.norm(V.max(0) - V.min(0)))


@pytest.mark.parametrize("name", ["untangle_a", "untangle_b", "untangle_c", "untangle_box"])
def test_untangle_matches_reference_pipeline2(hx, name):
    z = load_golden(name)
    ctx = hx.Context(0)
    try:
        ctx.upload([(z["V"], z["H"])])
        rep = ctx.untangle(z["boundary"], weight_opt=float(z["weight_opt"]))[0]
        Vg = ctx.get_positions()
    finally:
        ctx.close()
    err = np.abs(Vg - z["V_o"]).max() / diag_of(z["V"])
    print(f"\n[{name}] max|dX|/diag {err:.3e}  success {rep['success']}/{bool(z['out'][0])}  "
          f"minJ {rep['min_J']:.8f}/{z['out'][1]:.8f}  iterations {rep['iterations']}")
    assert rep["success"] == bool(z["out"][0])
    assert abs(rep["min_J"] - z["out"][1]) <= max(1e-6, 3 * float(z["minJ_spread"]))
    assert err <= max(1e-6, 3 * float(z["spread"]))


def test_untangle_batch_equals_individual_runs(hx):
    """Meshes of a batch untangle independently: each stops at its own iteration."""
    zs = [load_golden(n) for n in ("untangle_a", "untangle_b", "untangle_box")]
    ctx = hx.Context(0)
    try:
        ctx.upload([(z["V"], z["H"]) for z in zs])
        reps = ctx.untangle(np.concatenate([z["boundary"] for z in zs]), weight_opt=1.0)
        Vb = ctx.get_positions()
    finally:
        ctx.close()
    off = 0
    for z, r in zip(zs, reps):
        n = len(z["V"])
        assert r["success"] == bool(z["out"][0])
        assert np.abs(Vb[off:off + n] - z["V_o"]).max() <= 1e-6 * diag_of(z["V"])
        off += n


def test_smoothing_matches_reference(hx):
    """The smoothing stage (3 rounds of cube shapes + 5 iterations of the modified igl::slim,
    M = weight_opt / 2) against the reference's own slim_opt_igl loop."""
    z = load_golden("smoothing")
    ctx = hx.Context(0)
    try:
        ctx.upload([(z["V"], z["H"])])
        ctx.smoothing(int(z["outer"]), int(z["inner"]), weight_opt=float(z["weight_opt"]), precision=hx.FP64)
        Vg = ctx.get_positions()
        q = ctx.scaled_jacobian()[2][0]
    finally:
        ctx.close()
    err = np.abs(Vg - z["V_o"]).max() / diag_of(z["V"])
    print(f"\n[smoothing] max|dX|/diag {err:.3e}  minJ {q['min']:.8f}/{z['out'][1]:.8f}")
    assert err <= 1e-6
    assert abs(q["min"] - z["out"][1]) <= 1e-6


def test_projection_term_matches_reference(hx):
    """Tetralize_Set::projection with lamda_projection 1e3 against the reference's slim_m_opt."""
    z = load_golden("slim_projection")
    ctx = hx.Context(0)
    try:
        ctx.upload([(z["V"], z["H"])])
        ctx.set_projection([z["b"]], [z["bc"]], float(z["lamda_projection"]))
        rep = ctx.slim_m_opt(int(z["iters"]), precision=hx.FP64, weight_opt=float(z["weight_opt"]))
        Vg = ctx.get_positions()
    finally:
        ctx.close()
    err = np.abs(Vg - z["V_o"]).max() / diag_of(z["V"])
    assert err <= 1e-6, err
    np.testing.assert_allclose([rep[0]["energy"], rep[0]["energy_quality"], rep[0]["energy_soft"]], z["out"], rtol=1e-6)
