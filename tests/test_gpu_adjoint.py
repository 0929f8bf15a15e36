"""GPU adjoint-state gradient through the C ABI.

The engine's FP32 gradient equals the oracle's FP32 restatement bit for bit
(same tape, same summation order, shot sums in FP64); it agrees with the
FP64 adjoint to 1e-3 relative (L2), and the FP64 adjoint with central finite
differences of the FP64 misfit.
"""
import numpy as np
import pytest

from helpers import smooth_model, surface_receivers

pytestmark = pytest.mark.gpu


def setup(nx=70, nz=36, seed=3, noise=0.02, arith="ieee"):
    from seisfat2d_gb300 import Engine
    m = smooth_model(nx, nz, 10.0, seed=seed, noise=noise)
    e = Engine(nx, nz, 10.0, 10.0)
    e.set_arithmetic(arith)
    e.set_slowness(m)
    return e, m


@pytest.mark.parametrize("arith", ["ieee", "reference", "compensated"])
def test_adjoint_bitexact_vs_oracle(oracle, engine_lib, cuda, arith):
    e, m = setup(arith=arith)
    oracle.set_arith(arith)
    try:
        S = oracle.expand_boundary(m)
        rx, rz = surface_receivers(e.nx, 10.0, step=3)
        rz = rz + 10.0
        shots = [(120.0, 0.0), (400.0, 30.0, 10, 45), (650.0, 80.0), (333.0, 200.0, 0, 50)]
        pk = e.batch_forward(shots, rx, rz, keep_tape=True)
        rng = np.random.default_rng(0)
        pg = rng.standard_normal(pk.shape).astype(np.float32)
        pg[np.isnan(pk)] = np.nan
        g = e.batch_adjoint(pg)
        go, po = oracle.batch_gradient(S, 10.0, 10.0, shots, rx, rz, pg)
        assert np.array_equal(pk, po, equal_nan=True)
        assert np.array_equal(g, go), np.abs(g - go).max()
        assert np.abs(g).max() > 0
    finally:
        oracle.set_arith("ieee")


def test_adjoint_follows_changed_batches(oracle, engine_lib, cuda):
    """One context, batches in turn: the same batch twice, then other shots
    (other windows), other receivers, both changed, and the first batch
    again. The gather's shot lists and the seed table are kept between
    adjoints while the shots and receivers stay the same; every gradient
    must still equal the oracle's for its own batch."""
    e, m = setup(nx=80, nz=40, seed=12, arith="ieee")
    oracle.set_arith("ieee")
    S = oracle.expand_boundary(m)
    rx1, rz1 = surface_receivers(e.nx, 10.0, step=3)
    rx2, rz2 = surface_receivers(e.nx, 10.0, step=4)
    rz2 = rz2 + 20.0
    sh1 = [(120.0, 0.0), (400.0, 30.0, 10, 45), (650.0, 80.0)]
    sh2 = [(300.0, 10.0, 5, 40), (700.0, 0.0), (150.0, 50.0, 0, 30), (500.0, 0.0)]
    rng = np.random.default_rng(5)
    for shots, rx, rz in [(sh1, rx1, rz1), (sh1, rx1, rz1), (sh2, rx1, rz1), (sh1, rx2, rz2),
                          (sh2, rx2, rz2), (sh1, rx1, rz1)]:
        pk = e.batch_forward(shots, rx, rz, keep_tape=True)
        pg = rng.standard_normal(pk.shape).astype(np.float32)
        pg[np.isnan(pk)] = np.nan
        g = e.batch_adjoint(pg)
        go, po = oracle.batch_gradient(S, 10.0, 10.0, shots, rx, rz, pg)
        assert np.array_equal(pk, po, equal_nan=True)
        assert np.array_equal(g, go), np.abs(g - go).max()


def test_adjoint_fp32_vs_fp64(oracle, engine_lib, cuda):
    e, m = setup(nx=90, nz=50, seed=8, noise=0.0)
    S = oracle.expand_boundary(m)
    rx, rz = surface_receivers(e.nx, 10.0, step=2)
    shots = [(150.0, 0.0), (600.0, 0.0), (880.0, 0.0)]
    pk = e.batch_forward(shots, rx, rz, keep_tape=True)
    pg = np.where(np.isnan(pk), np.nan, np.cos(np.arange(pk.size).reshape(pk.shape) * 0.1)).astype(np.float32)
    g = e.batch_adjoint(pg).astype(np.float64)
    g64, _ = oracle.batch_gradient(S, 10.0, 10.0, shots, rx, rz, pg.astype(np.float64), fp64=True)
    rel = np.linalg.norm(g - g64) / np.linalg.norm(g64)
    print(f"relative L2 error FP32 adjoint vs FP64 adjoint: {rel:.2e}")
    assert rel <= 1e-3


def test_misfit_gradient_is_adjoint_of_residuals(oracle, engine_lib, cuda):
    e, m = setup(nx=60, nz=30, seed=4)
    rx, rz = surface_receivers(e.nx, 10.0, step=2)
    shots = [(100.0, 0.0), (450.0, 0.0)]
    pk = e.batch_forward(shots, rx, rz, keep_tape=True)
    tobs = (pk + 0.01 * np.sin(np.arange(pk.size).reshape(pk.shape))).astype(np.float32)
    J, g = e.misfit_gradient(tobs)
    r = (pk - tobs).astype(np.float64)
    assert abs(J - 0.5 * np.nansum(r * r)) <= 1e-6 * abs(J)
    e.batch_forward(shots, rx, rz, keep_tape=True)
    g2 = e.batch_adjoint(np.where(np.isnan(pk), np.nan, pk - tobs).astype(np.float32))
    assert np.array_equal(g, g2)


def test_adjoint_needs_tape_and_consumes_it(engine_lib, cuda):
    from seisfat2d_gb300._lib import SF_ERR_STATE
    from seisfat2d_gb300 import EngineError
    e, m = setup(nx=40, nz=20)
    rx, rz = surface_receivers(e.nx, 10.0, step=4)
    pk = e.batch_forward([(100.0, 0.0)], rx, rz)
    with pytest.raises(EngineError) as ex:
        e.batch_adjoint(np.zeros_like(pk))
    assert ex.value.status == SF_ERR_STATE
    pk = e.batch_forward([(100.0, 0.0)], rx, rz, keep_tape=True)
    e.batch_adjoint(np.zeros_like(pk))
    with pytest.raises(EngineError):
        e.batch_adjoint(np.zeros_like(pk))


def test_autograd_wrapper_matches_adjoint(engine_lib, cuda):
    import torch
    from seisfat2d_gb300.autograd import EikonalPicks
    e, m = setup(nx=50, nz=30, seed=9)
    rx, rz = surface_receivers(e.nx, 10.0, step=3)
    shots = [(100.0, 0.0), (300.0, 50.0)]
    S = torch.tensor(e.get_slowness(), device="cuda", requires_grad=True)
    picks = EikonalPicks.apply(S, e, shots, rx, rz)
    w = torch.linspace(-1, 1, picks.numel(), device="cuda").reshape(picks.shape)
    loss = torch.nansum(picks * w)
    loss.backward()
    e.set_slowness(S.detach(), padded=True)
    e.batch_forward(shots, rx, rz, keep_tape=True)
    pg = torch.where(torch.isnan(picks), torch.nan, w).detach().cpu().numpy()
    g = e.batch_adjoint(pg)
    assert np.array_equal(S.grad.cpu().numpy(), g)


@pytest.mark.parametrize("arith", ["ieee", "reference"])
def test_strip_loop_forms_same_bits(oracle, engine_lib, cuda, arith):
    """The general and the interior-block strip loops give the same picks,
    misfit and gradient (isotropic taped batch) and the same anisotropic
    picks; SF_LOOP_AUTO takes the interior form for a batch of equal windows
    that runs at once and the general one for uneven windows."""
    from seisfat2d_gb300.synthetic import thomsen_stiffness
    e, m = setup(nx=150, nz=70, seed=9, arith=arith)
    rx, rz = surface_receivers(e.nx, 10.0, step=3)
    shots = [(150.0, 0.0), (700.0, 40.0), (1200.0, 10.0)]
    vp = 1.0 / m.astype(np.float64)
    rng = np.random.default_rng(1)
    e.set_stiffness([c.astype(np.float32) for c in thomsen_stiffness(vp, vp / np.sqrt(3.0), 1000.0,
                                                                     rng.uniform(0, .2, vp.shape),
                                                                     rng.uniform(-.05, .1, vp.shape))])
    res = {}
    for mode in ("general", "interior"):
        e.set_strip_loop(mode)
        pk = e.batch_forward(shots, rx, rz, keep_tape=True)
        assert e.strip_loop() == (mode, mode == "interior")
        J, g = e.misfit_gradient(pk + np.float32(0.01))
        pa = e.batch_forward(shots, rx, rz, ani=True)
        res[mode] = (pk, J, g, pa)
    a, b = res["general"], res["interior"]
    assert np.array_equal(a[0], b[0], equal_nan=True) and a[1] == b[1]
    assert np.array_equal(a[2], b[2]) and np.abs(a[2]).max() > 0
    assert np.array_equal(a[3], b[3], equal_nan=True)
    e.set_strip_loop("auto")
    e.batch_forward(shots, rx, rz)
    assert e.strip_loop() == ("auto", True)
    e.batch_forward([(150.0, 0.0, 0, 90), (700.0, 0.0, 40, 110)], rx, rz)
    assert e.strip_loop() == ("auto", False)


@pytest.mark.parametrize("arith", ["ieee", "reference"])
def test_strip_loop_forms_same_bits_windows(engine_lib, cuda, arith):
    """Forced interior-block loops on windowed shots (offsets, widths from too
    narrow for any interior block to wide, sources near window edges) give
    the general loops' bits: picks, tables, misfit, gradient."""
    e, m = setup(nx=160, nz=80, seed=12, arith=arith)
    rx, rz = surface_receivers(e.nx, 10.0, step=2)
    shots = [(200.0, 0.0, 10, 30), (500.0, 60.0, 30, 44), (900.0, 20.0, 50, 90), (1300.0, 150.0, 100, 66),
             (1500.0, 0.0, 0, 166)]
    res = {}
    for mode in ("general", "interior"):
        e.set_strip_loop(mode)
        pk = e.batch_forward(shots, rx, rz, keep_tables=True)
        tabs = [e.batch_table(k, s[3]) for k, s in enumerate(shots)]
        pk2 = e.batch_forward(shots, rx, rz, keep_tape=True)
        J, g = e.misfit_gradient(np.nan_to_num(pk2) + np.float32(0.02))
        res[mode] = (pk, tabs, pk2, J, g)
    a, b = res["general"], res["interior"]
    assert np.array_equal(a[0], b[0], equal_nan=True) and np.array_equal(a[2], b[2], equal_nan=True)
    for ta, tb in zip(a[1], b[1]):
        assert np.array_equal(ta, tb)
    assert a[3] == b[3] and np.array_equal(a[4], b[4]) and np.abs(a[4]).max() > 0


@pytest.mark.parametrize("warps", [2, 4])
def test_fused_gather_same_bits(engine_lib, cuda, warps):
    """The gather inside the reverse-sweep launch (tiles started as the last
    reverse sweep finishes them) gives the separate gather's bits, eagerly
    and from a replayed CUDA graph of the planned iteration."""
    e, m = setup(nx=150, nz=90, seed=21)
    e.set_launch(warps, 0)
    rx, rz = surface_receivers(e.nx, 10.0, step=3)
    shots = [(150.0, 0.0), (700.0, 40.0, 20, 100), (1200.0, 10.0), (400.0, 300.0, 0, 80), (1000.0, 0.0, 60, 96)]
    res = {}
    for fused in (False, True):
        e.set_fused_gather(fused)
        pk = e.batch_forward(shots, rx, rz, keep_tape=True)
        J, g = e.misfit_gradient(np.nan_to_num(pk) + np.float32(0.01))
        assert e.fused_gather() == (fused, fused)
        res[fused] = (pk, J, g)
    assert res[False][1] == res[True][1] and np.array_equal(res[False][2], res[True][2])
    assert np.abs(res[True][2]).max() > 0
    # planned iteration replayed from a graph, fused
    dev = cuda.device("cuda", 0)
    tobs = cuda.from_numpy(np.nan_to_num(res[True][0]) + np.float32(0.01)).to(dev)
    picks = cuda.empty(tobs.shape, dtype=cuda.float32, device=dev)
    grad = cuda.empty((e.nxx, e.nzz), dtype=cuda.float32, device=dev)
    e.set_fused_gather(True)
    e.plan_batch(shots, rx, rz)
    for _ in range(3):
        e.plan_graph_launch(picks, t_obs=tobs, grad=grad)
        e.synchronize()
        assert e.fused_gather() == (True, True)
        assert np.array_equal(grad.cpu().numpy(), res[False][2])


def test_autograd_backward_refuses_a_replaced_tape(engine_lib, cuda):
    """Two forwards on one engine before the backward: the first forward's
    backward would differentiate the second batch's tape, so it raises; the
    second's backward equals the direct adjoint."""
    import torch
    from seisfat2d_gb300.autograd import EikonalPicks
    e, m = setup(nx=50, nz=30, seed=9)
    rx, rz = surface_receivers(e.nx, 10.0, step=3)
    S = torch.tensor(e.get_slowness(), device="cuda", requires_grad=True)
    p1 = EikonalPicks.apply(S, e, [(100.0, 0.0)], rx, rz)
    p2 = EikonalPicks.apply(S, e, [(100.0, 0.0), (300.0, 50.0)], rx, rz)
    with pytest.raises(RuntimeError, match="tape belongs to a later call"):
        torch.nansum(p1).backward(retain_graph=True)
    S.grad = None
    torch.nansum(p2).backward()
    e.batch_forward([(100.0, 0.0), (300.0, 50.0)], rx, rz, keep_tape=True)
    pg = np.where(np.isnan(p2.detach().cpu().numpy()), np.nan, 1.0).astype(np.float32)
    assert np.array_equal(S.grad.cpu().numpy(), e.batch_adjoint(pg))
    # a pick gradient of the wrong size never reaches the device
    e.batch_forward([(100.0, 0.0)], rx, rz, keep_tape=True)
    with pytest.raises(ValueError, match="taped batch of 1 shots"):
        e.batch_adjoint(np.zeros((2, len(rx)), np.float32))
