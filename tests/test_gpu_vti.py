"""Anisotropic (VTI) adjoint through the C ABI: sf_batch_forward with ani = 1
and SF_KEEP_TAPE tapes the second (qP) solve; sf_batch_misfit_gradient gives
dJ/dS and sf_batch_stiffness_gradient dJ/dC11, dJ/dC13. All three equal the
oracle's FP32 restatement bit for bit (same tapes, the qP derivative factors
in FP32, each operation rounded once, shot sums in FP64 in caller order); the oracle's
stiffness gradients match central differences of the misfit
(tests/test_oracle.py)."""
import numpy as np
import pytest

from helpers import smooth_model

pytestmark = pytest.mark.gpu


def vti_case(oracle, nx=64, nz=34, seed=5):
    from seisfat2d_gb300.synthetic import thomsen_stiffness
    rng = np.random.default_rng(seed)
    m = smooth_model(nx, nz, 10.0, seed=seed)
    vp = 1.0 / m.astype(np.float64)
    cij = thomsen_stiffness(vp, vp / np.sqrt(3.0), 1000.0, rng.uniform(0.0, 0.25, (nx, nz)),
                            rng.uniform(-0.05, 0.15, (nx, nz)))
    codes, mm = [], []
    for c in cij:
        cd, mn, mx = oracle.compress(oracle.expand_boundary(c.astype(np.float32)))
        codes.append(cd)
        mm += [mn, mx]
    return m, codes, np.array(mm, np.float32)


@pytest.mark.parametrize("arith", ["ieee", "reference", "compensated"])
def test_vti_gradient_bitexact_vs_oracle(oracle, engine_lib, cuda, arith):
    from seisfat2d_gb300 import Engine
    m, codes, mm = vti_case(oracle)
    e = Engine(m.shape[0], m.shape[1], 10.0, 10.0)
    e.set_arithmetic(arith)
    e.set_slowness(m)
    e.set_stiffness_codes(codes, mm)
    oracle.set_arith(arith)
    try:
        S = oracle.expand_boundary(m)
        rx = np.arange(15.0, 620.0, 20.0).astype(np.float32)
        rz = np.full_like(rx, 20.0)
        shots = [(120.0, 0.0), (400.0, 30.0, 10, 50), (520.0, 60.0), (300.0, 150.0, 5, 45)]
        pk = e.batch_forward(shots, rx, rz, ani=True, keep_tape=True)
        tobs = (np.nan_to_num(pk) * np.float32(1.02) + np.float32(0.003)).astype(np.float32)
        J, g = e.misfit_gradient(tobs)
        g11, g13 = e.stiffness_gradient()
        Jo, go, po, _, g11o, g13o = oracle.batch_misfit_gradient(S, 10.0, 10.0, shots, rx, rz, tobs,
                                                                 ani=(codes, mm))
        assert np.array_equal(pk, po, equal_nan=True)
        assert abs(J - Jo) <= 1e-12 * abs(Jo)
        for name, a, b in (("S", g, go), ("C11", g11, g11o), ("C13", g13, g13o)):
            print(f"{arith} dJ/d{name}: max |engine - oracle| = {np.abs(a - b).max():.3e}, max |oracle| = "
                  f"{np.abs(b).max():.3e}")
            assert np.abs(b).max() > 0
            assert np.array_equal(a, b)
    finally:
        oracle.set_arith("ieee")


def test_vti_adjoint_state(oracle, engine_lib, cuda):
    """The stiffness gradient exists only after the adjoint of an anisotropic
    taped batch; an isotropic batch afterwards withdraws it."""
    from seisfat2d_gb300 import Engine, EngineError
    m, codes, mm = vti_case(oracle, nx=40, nz=20, seed=6)
    e = Engine(m.shape[0], m.shape[1], 10.0, 10.0)
    e.set_slowness(m)
    e.set_stiffness_codes(codes, mm)
    rx = np.arange(15.0, 380.0, 30.0).astype(np.float32)
    rz = np.zeros_like(rx)
    with pytest.raises(EngineError):
        e.stiffness_gradient()
    pk = e.batch_forward([(100.0, 0.0), (250.0, 0.0)], rx, rz, ani=True, keep_tape=True)
    e.misfit_gradient(pk + np.float32(0.01))
    g11, g13 = e.stiffness_gradient()
    assert np.abs(g11).max() > 0
    pk = e.batch_forward([(100.0, 0.0)], rx, rz, keep_tape=True)
    e.misfit_gradient(pk + np.float32(0.01))
    with pytest.raises(EngineError):
        e.stiffness_gradient()
