"""FP32 accuracy against the FP64 oracle, per synthetic config and arithmetic.

Traveltimes: two shots of each isotropic config (the first and a middle one,
on their own windows) solved by the engine in FP32 and by the oracle in FP64
on the same 1-pass schedule; the error is |T32 - T64| / T64 over the
window's interior nodes with T64 > 0. The reference and IEEE arithmetics
round every traveltime to FP32 as it is formed, so the error accumulates
along a sweep: their RMS stays within 1e-5 but isolated nodes of the layered
models exceed 1e-5 in the maximum. The compensated arithmetic carries the
times as FP32 pairs and meets 1e-5 in the maximum as well.

Gradient (the full 1701 x 351 model with 3 faults, two shots, 400
receivers, observed picks from the FP64 oracle on the true model plus 2 ms
Gaussian noise): the engine's misfit gradient against
  * the FP64 adjoint of the FP64 misfit (branches of its own),
  * the FP64 adjoint that follows the engine's own branch codes
    (sf_batch_tape_codes), the same discrete scheme evaluated in FP64,
  * central finite differences of the FP64 misfit on 32 seeded cells
    (slowness steps of 1e-6 relative), which also check the FP64 adjoint.
The compensated arithmetic meets 1e-3 against all three. The reference
arithmetic does not: its traveltimes drift by ~1e-5 relative (a few 1e-5 s),
and the adjoint's coefficients depend on differences of neighbouring times
(a few ms), so they err by up to ~1%; the test pins the current figures so
that a regression shows.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pick(shots, k):
    s = shots[k]
    return (float(s[0]), float(s[1])) + ((int(s[2]), int(s[3])) if len(s) > 2 else ())


@pytest.mark.parametrize("cfg", [1, 2, 4, 5])
def test_fp32_traveltimes_vs_fp64_per_config(oracle, engine_lib, cuda, cfg):
    from seisfat2d_gb300 import Engine, synthetic
    w = getattr(synthetic, f"config{cfg}")()
    shots = [_pick(w.shots, 0), _pick(w.shots, len(w.shots) // 2)]
    S = oracle.expand_boundary(w.slowness)
    nxx, nzz = S.shape
    T64s = []
    for s in shots:
        c0 = s[2] if len(s) > 2 else 0
        nc = s[3] if len(s) > 3 else nxx - c0
        T64s.append(oracle.solve_f64(S, w.dx, w.dz, s[0], s[1], c0=c0, ncols=nc)[0])
    for arith in ("reference", "ieee", "compensated"):
        e = Engine(w.nx, w.nz, w.dx, w.dz)
        e.set_arithmetic(arith)
        e.set_slowness(w.slowness)
        e.batch_forward(shots, np.zeros(0, np.float32), np.zeros(0, np.float32), keep_tables=True)
        errs = []
        for k, s in enumerate(shots):
            c0 = s[2] if len(s) > 2 else 0
            nc = s[3] if len(s) > 3 else nxx - c0
            T32 = e.batch_table(k, nc).astype(np.float64)
            inner = T64s[k][3:nc - 3, 3:nzz - 3]
            m = inner > 0
            errs.append((np.abs(T32[3:nc - 3, 3:nzz - 3] - inner) / np.where(m, inner, 1.0))[m])
        err = np.concatenate(errs)
        mx, rms = float(err.max()), float(np.sqrt(np.mean(err * err)))
        print(f"config {cfg} ({w.name}), {arith} arithmetic, {err.size} nodes of 2 shots: "
              f"max rel {mx:.2e}, RMS rel {rms:.2e}")
        assert rms <= 1e-5
        if arith == "compensated":
            assert mx <= 1e-5
        del e


def test_vti_traveltimes_vs_fp64_config3(oracle, engine_lib, cuda):
    """The anisotropic two-pass solve (1601 x 401, two of the 100 shots)
    against the FP64 anisotropic oracle (both solves and the qP field in
    FP64, from the same quantised stiffness). The qP pass takes the direction
    of the first solve from central differences of its traveltimes, so FP32
    rounding of those times also tilts the qP slowness: the reference and
    IEEE arithmetics reach a few 1e-4 at isolated nodes. The compensated
    arithmetic forms the differences from its pairs and meets 1e-5."""
    from seisfat2d_gb300 import Engine, synthetic
    w = synthetic.config3()
    S = oracle.expand_boundary(w.slowness)
    nxx, nzz = S.shape
    codes, mm = [], []
    for c in w.cij:
        cd, mn, mx = oracle.compress(oracle.expand_boundary(c))
        codes.append(cd)
        mm += [mn, mx]
    mm = np.array(mm, np.float32)
    shots = [_pick(w.shots, 0), _pick(w.shots, len(w.shots) // 2)]
    T64s = [oracle.shot_ani_f64(S, w.dx, w.dz, s[0], s[1], (codes, mm)) for s in shots]
    for arith in ("reference", "ieee", "compensated"):
        e = Engine(w.nx, w.nz, w.dx, w.dz)
        e.set_arithmetic(arith)
        e.set_slowness(w.slowness)
        e.set_stiffness_codes(codes, mm)
        e.batch_forward(shots, np.zeros(0, np.float32), np.zeros(0, np.float32), ani=True, keep_tables=True)
        errs = []
        for k in range(len(shots)):
            inner = T64s[k][3:-3, 3:-3]
            m = inner > 0
            T32 = e.batch_table(k, nxx).astype(np.float64)
            errs.append((np.abs(T32[3:-3, 3:-3] - inner) / np.where(m, inner, 1.0))[m])
        err = np.concatenate(errs)
        mx, rms = float(err.max()), float(np.sqrt(np.mean(err * err)))
        print(f"config 3 (VTI), {arith} arithmetic, {err.size} nodes of 2 shots: max rel {mx:.2e}, RMS rel {rms:.2e}")
        if arith == "compensated":
            assert mx <= 1e-5
        else:
            assert rms <= 3e-5 and mx <= 1e-3  # pinned (measured about 1e-5 RMS, 3.4e-4 max)
        del e


def config4_gradient_case(oracle, nshots=2, seed=44):
    """Model, shots (the first and a middle one of the 100), receivers and
    observed picks (FP64 oracle on the true model + N(0, 2 ms))."""
    from seisfat2d_gb300 import synthetic
    w = synthetic.config4()
    shots = [_pick(w.shots, 0), _pick(w.shots, len(w.shots) // 2)][:nshots]
    St = oracle.expand_boundary(w.extra["true_slowness"])
    rng = np.random.default_rng(seed)
    tobs = np.array([oracle.picks_f64(oracle.solve_f64(St, w.dx, w.dz, s[0], s[1])[0], w.dx, w.dz, w.rx, w.rz)
                     for s in shots])
    tobs = tobs + rng.normal(0.0, w.extra["noise_sigma"], tobs.shape)
    return w, shots, tobs


@pytest.mark.parametrize("arith", ["compensated", "reference"])
def test_gradient_config4_vs_fp64_and_finite_differences(oracle, engine_lib, cuda, arith):
    from seisfat2d_gb300 import Engine
    w, shots, tobs = config4_gradient_case(oracle)
    S = oracle.expand_boundary(w.slowness)
    nxx, nzz = S.shape
    e = Engine(w.nx, w.nz, w.dx, w.dz)
    e.set_arithmetic(arith)
    e.set_slowness(w.slowness)
    e.batch_forward(shots, w.rx, w.rz, keep_tape=True)
    codes = [e.tape_codes(b, nxx) for b in range(len(shots))]  # before the adjoint consumes the tape
    J, g32 = e.misfit_gradient(tobs.astype(np.float32))
    g32 = g32.astype(np.float64)
    g64 = oracle.fp64_misfit_gradients(S, w.dx, w.dz, shots, w.rx, w.rz, tobs)
    gsb = oracle.fp64_misfit_gradients(S, w.dx, w.dz, shots, w.rx, w.rz, tobs, follow=codes)
    rl = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    e_ind, e_sb, e_ties = rl(g32, g64), rl(g32, gsb), rl(gsb, g64)
    # 32 seeded cells with a gradient above 1% of the largest
    rng = np.random.default_rng(32)
    inner = np.zeros((nxx, nzz), bool)
    inner[3:-3, 3:-3] = True
    cand = np.argwhere(inner & (np.abs(g64) >= 1e-2 * np.abs(g64).max()))
    cells = [(int(i), int(j)) for j, i in cand[rng.choice(len(cand), 32, replace=False)]]
    D, _, _ = oracle.fd_misfit_f64(S, w.dx, w.dz, shots, w.rx, w.rz, tobs, cells, rel=1e-6)
    at = lambda g: np.array([g[j, i] for i, j in cells])
    fd64 = np.abs(at(g64) - D) / np.abs(D)
    fd32 = np.abs(at(g32) - D) / np.abs(D)
    print(f"config 4 gradient, {arith} arithmetic, 2 shots x 400 receivers: relative L2 vs FP64 adjoint "
          f"{e_ind:.2e}, vs FP64 adjoint on the engine's branches {e_sb:.2e} (the two FP64 adjoints differ by "
          f"{e_ties:.2e}); 32 cells vs central differences of the FP64 misfit: engine median {np.median(fd32):.2e} "
          f"max {fd32.max():.2e}, FP64 adjoint max {fd64.max():.2e}")
    assert fd64.max() <= 1e-4  # the FP64 adjoint is the derivative of the FP64 misfit
    if arith == "compensated":
        assert e_sb <= 1e-3 and e_ind <= 1e-3 and fd32.max() <= 1e-3
    else:
        # pinned: FP32 traveltime rounding through the tape coefficients (measured 4.1e-2 / 5.0e-2 / 1.1e-1)
        assert e_sb <= 6e-2 and e_ind <= 8e-2 and np.median(fd32) <= 3e-2
