"""Failure detection on the GPU, without a fault: a short in-kernel wait limit
(sf_set_wait_limit) and a launch whose strips wait for a handoff tag no strip
writes (sf_test_stall_next_batch). Every wait gives up after the limit, the
kernel finishes, the call reports SF_ERR_TIMEOUT, and the same context then
runs the next batches (forward, taped forward and gradient) bit for bit as
before."""
import time

import numpy as np
import pytest

from helpers import smooth_model, surface_receivers

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("arith", ["reference", "compensated"])
def test_stalled_batch_times_out_and_the_context_recovers(oracle, engine_lib, cuda, arith):
    from seisfat2d_gb300 import Engine, EngineError
    from seisfat2d_gb300._lib import SF_ERR_TIMEOUT
    nx, nz = 140, 120  # 126 padded rows: four strips, three of which wait on the strip above
    m = smooth_model(nx, nz, 10.0, seed=61, noise=0.02)
    e = Engine(nx, nz, 10.0, 10.0)
    e.set_arithmetic(arith)
    e.set_slowness(m)
    e.set_wait_limit(0.05)
    rx, rz = surface_receivers(nx, 10.0, step=4)
    shots = [(150.0, 0.0), (700.0, 30.0), (1200.0, 0.0, 40, 90)]
    pk0 = e.batch_forward(shots, rx, rz)
    tobs = (np.nan_to_num(pk0) + np.float32(0.01)).astype(np.float32)
    e.batch_forward(shots, rx, rz, keep_tape=True)
    J0, g0 = e.misfit_gradient(tobs)
    e.test_stall_next_batch()
    t0 = time.perf_counter()
    with pytest.raises(EngineError) as ei:
        e.batch_forward(shots, rx, rz)
    dt = time.perf_counter() - t0
    assert ei.value.status == SF_ERR_TIMEOUT
    print(f"{arith}: the stalled batch returned SF_ERR_TIMEOUT after {1e3 * dt:.1f} ms (limit 50 ms per wait)")
    assert dt < 5.0
    # the context keeps working: same picks, same misfit and gradient
    assert np.array_equal(e.batch_forward(shots, rx, rz), pk0, equal_nan=True)
    e.batch_forward(shots, rx, rz, keep_tape=True)
    J1, g1 = e.misfit_gradient(tobs)
    assert J1 == J0 and np.array_equal(g1, g0)
    # and the plain solve after another stalled one
    e.test_stall_next_batch()
    with pytest.raises(EngineError) as ei:
        e.time_propagation(700.0, 30.0)
    assert ei.value.status == SF_ERR_TIMEOUT
    oracle.set_arith(arith)
    try:
        assert np.array_equal(e.time_propagation(700.0, 30.0),
                              oracle.solve_f32(oracle.expand_boundary(m), 10.0, 10.0, 700.0, 30.0))
    finally:
        oracle.set_arith("ieee")


def test_wait_limit_arguments(engine_lib, cuda):
    from seisfat2d_gb300 import Engine, EngineError
    e = Engine(40, 20, 10.0, 10.0)
    e.set_wait_limit(0.0)
    e.set_wait_limit(60.0)
    for bad in (-1.0, 61.0, float("nan")):
        with pytest.raises(EngineError):
            e.set_wait_limit(bad)
