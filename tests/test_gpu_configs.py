"""Parity of the feature-alignment loop at the sizes the optimiser is measured on, against the
oracle's loop (tests/fa_oracle.py: the CPU restatement of the reference's FP64 path).

- 64^3 jittered grid (262,144 hexes) tied to a 200k-triangle superellipsoid, 3 iterations, in
  plain FP64 and in mixed precision.
- The cube-minus-cylinder workload (262,144 hexes; 12 cube edges and 2 hole circles as feature
  curves, 8 corners, U(+/-0.1h) jitter), 3 iterations in plain FP64 and in mixed precision.

Bars (the criteria the optimiser is held to):
  FP64 positions        within 1e-6 of the bbox diagonal (max over vertices)
  minimum scaled J      within 1e-4 (both modes)
  Hausdorff max         within 1e-5 of the bbox diagonal (both modes)
  weight schedule       lamda within 1e-6 relative (FP64)
  mixed positions       5e-5 of the diagonal on both workloads; lamda 1e-3 relative (64^3 grid)
                        and 1e-4 (cube minus cylinder).  Mixed precision rounds the local step's
                        coefficients at FP32 resolution, and the FP64 path itself moves by
                        ~1e-5 of the diagonal after 3 iterations when its input is perturbed at
                        that resolution (2^-24 h, printed by the tests): the truncated
                        20-iteration CG and the line search amplify such perturbations.  The
                        mixed result also moves from run to run (the float atomics of the
                        element scatter sum in launch order): 5e-6 to 2e-5 of the diagonal
                        on the cube minus cylinder over repeated runs.  The mixed bars sit a few
                        times above both.
Each test prints the measured errors.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def diag_of(V):
    return float(np.linalg.norm(V.max(0) - V.min(0)))


@pytest.fixture(scope="module")
def hx():
    import build
    build.build()
    import hexopt
    return hexopt


_oracle_runs = {}


def oracle_loop(name, p, iters):
    """The oracle loop's positions, last report and schedule weight, with the oracle's scaled
    Jacobian and two-sided Hausdorff of the result (cached per workload)."""
    if name not in _oracle_runs:
        import fa_oracle
        import oracle_py as O
        O.build_oracle()
        Vo, info, lam = fa_oracle.fa_steps(p, iters)
        sj = O.scaled_jacobian(Vo, p["H"])
        haus = O.hausdorff(p["TV"], p["TF"], Vo, p["surface"])
        _oracle_runs[name] = dict(V=Vo, info=info, lam=lam, min_J=sj["min"], haus=haus)
    return _oracle_runs[name]


def run_gpu(hx, p, iters, precision, V0=None):
    from hexopt import workloads
    ctx = hx.Context(0)
    try:
        workloads.load(ctx, [p])
        if V0 is not None:
            ctx.set_positions(V0)
        ctx.fa_begin(lamda0=0.05, precision=precision, weight_opt=0.001)
        for _ in range(iters):
            r = ctx.fa_step(hausdorff=True)[0]
        return ctx.get_positions(), r
    finally:
        ctx.close()


def check(name, p, Vg, r, ref, pos_bar, lam_rel):
    d = diag_of(p["V"])
    pos = float(np.abs(Vg - ref["V"]).max() / d)
    dj = abs(r["min_J"] - ref["min_J"])
    dh = abs(r["hausdorff_max"] - ref["haus"][1]) / ref["haus"][0]
    dl = abs(r["lamda"] - ref["lam"]) / ref["lam"]
    de = abs(r["energy"] - ref["info"]["energy"]) / abs(ref["info"]["energy"])
    print(f"\n[{name}] max|dX|/diag {pos:.3e}  |d minJ| {dj:.3e}  |d Hausdorff|/diag {dh:.3e}  "
          f"lamda rel {dl:.3e}  energy rel {de:.3e}  (minJ {r['min_J']:.6f}, cg_iters {r['cg_iters']}, "
          f"cg_error {r['cg_error']:.3e})")
    assert pos <= pos_bar, (name, pos)
    assert dj <= 1e-4, (name, dj)
    assert dh <= 1e-5, (name, dh)
    assert dl <= lam_rel, (name, dl)


@pytest.fixture(scope="module")
def grid64():
    from hexopt import workloads
    return workloads.grid_superellipsoid(64, sigma=0.2, seed=0, n_tri=200_000)


@pytest.fixture(scope="module")
def c2():
    from hexopt import workloads
    return workloads.cube_minus_cylinder()


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_feature_alignment_grid64_vs_oracle(hx, grid64, mode):
    ref = oracle_loop("grid64", grid64, 3)
    Vg, r = run_gpu(hx, grid64, 3, hx.FP64 if mode == "fp64" else hx.MIXED)
    if mode == "mixed":  # the FP64 path's own response to an input perturbed at FP32 resolution
        noise = np.random.default_rng(1).normal(0, 2.0 ** -24 / 64, grid64["V"].shape)
        Vn, rn = run_gpu(hx, grid64, 3, hx.FP64, V0=grid64["V"] + noise)
        print(f"\n[grid64 fp64, input noise 2^-24 h] max|dX|/diag {np.abs(Vn - ref['V']).max() / diag_of(grid64['V']):.3e}"
              f"  lamda rel {abs(rn['lamda'] - ref['lam']) / ref['lam']:.3e}")
    check(f"grid64 {mode}", grid64, Vg, r, ref, 1e-6 if mode == "fp64" else 5e-5, 1e-6 if mode == "fp64" else 1e-3)


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_feature_alignment_cube_minus_cylinder_vs_oracle(hx, c2, mode):
    ref = oracle_loop("c2", c2, 3)
    Vg, r = run_gpu(hx, c2, 3, hx.FP64 if mode == "fp64" else hx.MIXED)
    if mode == "mixed":  # the FP64 path's own response to an input perturbed at FP32 resolution
        # interior vertices only: the constrained ones start on their targets, where the soft
        # energy is ~0 and the weight schedule (Eq / Es) reacts to any perturbation of them
        h = 1.0 / 64
        free = np.ones(len(c2["V"]), bool)
        for k in ("corners", "lines", "regular"):
            free[np.asarray(c2[k], np.int64)] = False
        noise = np.random.default_rng(2).normal(0, 2.0 ** -24 * h, c2["V"].shape) * free[:, None]
        Vn, rn = run_gpu(hx, c2, 3, hx.FP64, V0=c2["V"] + noise)
        print(f"\n[cube_minus_cylinder fp64, input noise 2^-24 h] max|dX|/diag "
              f"{np.abs(Vn - ref['V']).max() / diag_of(c2['V']):.3e}  lamda rel {abs(rn['lamda'] - ref['lam']) / ref['lam']:.3e}")
    check(f"cube_minus_cylinder {mode}", c2, Vg, r, ref, 1e-6 if mode == "fp64" else 5e-5,
          1e-6 if mode == "fp64" else 1e-4)
