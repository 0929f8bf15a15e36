"""Planned batches through the C ABI: an eager planned iteration, its replay
from the context's CUDA graph, a caller-captured torch CUDA graph and the
autotuned launch shape all give the bits of the per-call batch API
(sf_batch_forward + sf_batch_misfit_gradient), which the oracle pins; the
misfit gradient also equals the oracle's threaded FP32 restatement."""
import numpy as np
import pytest

from helpers import smooth_model, surface_receivers

pytestmark = pytest.mark.gpu

SHOTS = [(120.0, 0.0), (400.0, 30.0, 10, 45), (650.0, 80.0), (333.0, 200.0, 0, 50), (50.0, 0.0, 0, 30)]


def make(nx=72, nz=40, seed=5, arith="reference"):
    from seisfat2d_gb300 import Engine
    m = smooth_model(nx, nz, 10.0, seed=seed, noise=0.02)
    e = Engine(nx, nz, 10.0, 10.0)
    e.set_arithmetic(arith)
    e.set_slowness(m)
    rx, rz = surface_receivers(nx, 10.0, step=3)
    rz = rz + 10.0
    return e, m, rx, rz


def observed(e, rx, rz, seed=1):
    pk = e.batch_forward(SHOTS, rx, rz)
    rng = np.random.default_rng(seed)
    return (pk + rng.normal(0.0, 0.01, pk.shape)).astype(np.float32)


def eager(e, rx, rz, tobs):
    pk = e.batch_forward(SHOTS, rx, rz, keep_tape=True)
    J, g = e.misfit_gradient(tobs)
    return pk, J, g


def dev_buffers(torch, e, tobs):
    dev = torch.device("cuda", 0)
    return dict(t_obs=torch.from_numpy(tobs).to(dev),
                picks=torch.empty(tobs.shape, dtype=torch.float32, device=dev),
                grad=torch.empty((e.nxx, e.nzz), dtype=torch.float32, device=dev),
                misfit=torch.empty(1, dtype=torch.float64, device=dev))


@pytest.mark.parametrize("arith", ["reference", "ieee", "compensated"])
def test_plan_iteration_equals_batch_calls(oracle, engine_lib, cuda, arith):
    e, m, rx, rz = make(arith=arith)
    tobs = observed(e, rx, rz)
    pk0, J0, g0 = eager(e, rx, rz, tobs)
    e.plan_batch(SHOTS, rx, rz)
    b = dev_buffers(cuda, e, tobs)
    for _ in range(2):
        e.plan_iteration(**b)
        cuda.cuda.synchronize()
        e.synchronize()
        assert np.array_equal(b["picks"].cpu().numpy(), pk0, equal_nan=True)
        assert np.array_equal(b["grad"].cpu().numpy(), g0)
        assert float(b["misfit"].item()) == J0
    oracle.set_arith(arith)
    try:
        Jo, go, po, _ = oracle.batch_misfit_gradient(oracle.expand_boundary(m), 10.0, 10.0, SHOTS, rx, rz, tobs)
    finally:
        oracle.set_arith("ieee")
    assert np.array_equal(po, pk0, equal_nan=True)
    assert np.array_equal(go, g0)
    assert abs(Jo - J0) <= 1e-12 * abs(Jo)  # FP64 sums of the same terms in another order


def test_plan_graph_replays_and_model_updates(engine_lib, cuda):
    e, m, rx, rz = make()
    tobs = observed(e, rx, rz)
    models = [m, (m * 1.01).astype(np.float32), m, (m * 0.98).astype(np.float32)]
    refs = []
    for mm in models:  # the per-call API on each model
        e.set_slowness(mm)
        refs.append(eager(e, rx, rz, tobs))
    e.plan_batch(SHOTS, rx, rz)
    b = dev_buffers(cuda, e, tobs)
    for rep, (mm, (pk, J, g)) in enumerate(zip(models, refs)):
        e.set_slowness(mm)  # the graph reads the context's slowness in place
        e.plan_graph_launch(**b)
        cuda.cuda.synchronize()
        e.synchronize()
        assert np.array_equal(b["picks"].cpu().numpy(), pk, equal_nan=True), rep
        assert np.array_equal(b["grad"].cpu().numpy(), g), rep
        assert float(b["misfit"].item()) == J, rep
    # new pointers: the graph is captured again
    b2 = dev_buffers(cuda, e, tobs)
    e.plan_graph_launch(**b2)
    cuda.cuda.synchronize()
    assert np.array_equal(b2["grad"].cpu().numpy(), refs[-1][2])


def test_plan_in_caller_captured_torch_graph(engine_lib, cuda):
    torch = cuda
    e, m, rx, rz = make(seed=9)
    tobs = observed(e, rx, rz)
    pk0, J0, g0 = eager(e, rx, rz, tobs)
    e.plan_batch(SHOTS, rx, rz)
    b = dev_buffers(torch, e, tobs)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        e.plan_iteration(stream=s, **b)  # configure outside the capture
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=s):
        e.plan_iteration(stream=s, **b)
    for _ in range(3):
        b["grad"].fill_(0.0)
        b["picks"].fill_(0.0)
        graph.replay()
        torch.cuda.synchronize()
        e.synchronize()
        assert np.array_equal(b["picks"].cpu().numpy(), pk0, equal_nan=True)
        assert np.array_equal(b["grad"].cpu().numpy(), g0)
        assert float(b["misfit"].item()) == J0


def test_plan_autotune_keeps_bits(engine_lib, cuda):
    e, m, rx, rz = make(nx=120, nz=70, seed=11)
    tobs = observed(e, rx, rz)
    pk0, J0, g0 = eager(e, rx, rz, tobs)
    e.plan_batch(SHOTS, rx, rz)
    b = dev_buffers(cuda, e, tobs)
    w, g, ms = e.plan_autotune(reps=2, **b)
    assert w in (1, 2, 4) and g >= 0 and ms > 0
    assert e.get_launch() == (w, g)
    e.plan_iteration(**b)
    cuda.cuda.synchronize()
    e.synchronize()
    assert np.array_equal(b["grad"].cpu().numpy(), g0)
    assert np.array_equal(b["picks"].cpu().numpy(), pk0, equal_nan=True)


def test_plan_state_errors_and_kernel_times(engine_lib, cuda):
    from seisfat2d_gb300 import EngineError
    e, m, rx, rz = make()
    tobs = observed(e, rx, rz)
    b = dev_buffers(cuda, e, tobs)
    with pytest.raises(EngineError):
        e.plan_iteration(**b)  # no plan yet
    e.plan_batch(SHOTS, rx, rz)
    e.batch_forward(SHOTS, rx, rz)  # another batch ends the plan
    with pytest.raises(EngineError):
        e.plan_iteration(**b)
    e.set_kernel_timing(True)
    e.batch_forward(SHOTS, rx, rz, keep_tape=True)
    e.misfit_gradient(tobs)
    t = e.kernel_times()
    assert set(t) == {"forward", "residual", "adjoint", "gather"}
    assert all(v > 0 for v in t.values())
    e.batch_forward(SHOTS, rx, rz)
    assert set(e.kernel_times()) == {"forward"}
    e.set_kernel_timing(False)
    e.batch_forward(SHOTS, rx, rz)
    assert e.kernel_times() == {}
