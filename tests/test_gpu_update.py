"""Device tomography update through the C ABI (sf_smooth_model,
sf_update_slowness): bit-identical to the oracle's restatement of the
reference's model_smoothing / smooth_matrix and Tomography_ISO::model_update."""
import numpy as np
import pytest

from helpers import smooth_model

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("stdv,samples", [(5.0, 11), (2.0, 5), (0.0, 7), (3.0, 1)])
def test_smooth_model_bitexact(oracle, engine_lib, cuda, stdv, samples):
    from seisfat2d_gb300 import Engine
    nx, nz = 83, 41
    e = Engine(nx, nz, 10.0, 10.0)
    f = np.random.default_rng(samples).standard_normal((nx, nz)).astype(np.float32)
    got = e.smooth_model(f, stdv, samples)
    ref = oracle.model_smoothing(f, stdv, samples)
    assert np.array_equal(got, ref), np.abs(got - ref).max()
    dev = cuda.from_numpy(f).cuda()
    out = cuda.empty_like(dev)
    e.smooth_model(dev, stdv, samples, out=out)
    cuda.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("samples", [0, 9])
def test_update_slowness_bitexact(oracle, engine_lib, cuda, samples):
    from seisfat2d_gb300 import Engine
    nx, nz = 64, 30
    m = smooth_model(nx, nz, 10.0, seed=4)
    e = Engine(nx, nz, 10.0, 10.0)
    e.set_slowness(m)
    S0 = e.get_slowness()
    g = np.random.default_rng(7).standard_normal((e.nxx, e.nzz)).astype(np.float32)
    dS = e.update_slowness(g, -2e-6, stdv=4.0, samples=samples)
    Sref, dSref = oracle.update_slowness(S0, g, nx, nz, -2e-6, 4.0, samples)
    assert np.array_equal(dS, dSref)
    assert np.array_equal(e.get_slowness(), Sref)
    # device gradient, second update on top of the first
    e.update_slowness(cuda.from_numpy(g).cuda(), -2e-6, stdv=4.0, samples=samples, want_dS=False)
    Sref2, _ = oracle.update_slowness(Sref, g, nx, nz, -2e-6, 4.0, samples)
    assert np.array_equal(e.get_slowness(), Sref2)


def test_even_samples_rejected(engine_lib, cuda):
    from seisfat2d_gb300 import Engine, EngineError
    e = Engine(20, 10, 10.0, 10.0)
    with pytest.raises(EngineError):
        e.smooth_model(np.zeros((20, 10), np.float32), 2.0, 4)
