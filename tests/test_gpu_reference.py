"""Pin the oracle and the engine to the reference's own kernels, run on the
GPU from cubins compiled from the reference sources (oracle/build_ref.py).

The reference is built by nvcc with FMA contraction on, the engine and the
oracle evaluate every FP32 operation with one rounding, so the comparison is
to 1e-5 relative (the benchmark spec's tolerance); the measured maximum is printed.
"""
import numpy as np
import pytest

from helpers import rel_err, smooth_model

pytestmark = pytest.mark.gpu


def _ref():
    from oracle import refkernels
    if not refkernels.available():
        pytest.skip("reference cubins not built on this machine")
    return refkernels


@pytest.mark.parametrize("nx,nz,sx,sz", [(40, 20, 0.0, 0.0), (20, 40, 93.0, 211.0), (120, 50, 555.0, 0.0),
                                         (300, 252, 1000.0, 500.0), (251, 61, 1234.0, 17.0)])
def test_engine_and_oracle_match_reference_kernels(oracle, engine_lib, cuda, nx, nz, sx, sz):
    ref = _ref()
    from seisfat2d_gb300 import Engine
    m = smooth_model(nx, nz, 10.0, seed=nx + nz, noise=0.02)
    S = oracle.expand_boundary(m)
    Tr, ms = ref.solve(S, 10.0, 10.0, sx, sz)
    e = Engine(nx, nz, 10.0, 10.0)
    e.set_slowness(m)
    T = e.time_propagation(sx, sz)
    To = oracle.solve_f32(S, 10.0, 10.0, sx, sz)
    assert np.array_equal(T, To)
    err = rel_err(T, Tr).max()
    print(f"{nx}x{nz}: max rel diff engine vs reference kernels = {err:.3e}; "
          f"bitwise-equal nodes {np.mean(T == Tr):.4f}")
    assert err <= 1e-5


def test_anisotropic_matches_reference_kernels(oracle, engine_lib, cuda):
    ref = _ref()
    from seisfat2d_gb300 import Engine
    from seisfat2d_gb300.synthetic import thomsen_stiffness
    nx, nz = 60, 30
    rng = np.random.default_rng(5)
    m = smooth_model(nx, nz, 10.0, seed=9)
    vp = 1.0 / m.astype(np.float64)
    cij = [c.astype(np.float32) for c in thomsen_stiffness(vp, vp / np.sqrt(3), 1000.0,
                                                          rng.uniform(0, .25, (nx, nz)),
                                                          rng.uniform(-.05, .15, (nx, nz)), 0.0)]
    S = oracle.expand_boundary(m)
    codes, mm = [], []
    for c in cij:
        cd, mn, mx = oracle.compress(oracle.expand_boundary(c))
        codes.append(cd)
        mm += [mn, mx]
    mm = np.array(mm, np.float32)
    Tr, _ = ref.solve(S, 10.0, 10.0, 300.0, 0.0, ani=(codes, mm))
    e = Engine(nx, nz, 10.0, 10.0)
    e.set_slowness(m)
    e.set_stiffness_codes(codes, mm)
    T = e.time_propagation(300.0, 0.0, ani=True)
    err = rel_err(T, Tr).max()
    print(f"ANI: max rel diff vs reference kernels = {err:.3e}")
    assert err <= 1e-5
