"""GPU parity of the forward solver against the oracle, through the C ABI.

FP32 traveltimes must equal the oracle's FP32 restatement bit for bit (same
IEEE operations in the same order, every node), in both arithmetics; picks
likewise. Sources sit at integer metres so the near-source offsets are exact
(the reference arithmetic squares them with CUDA's powf, which the oracle
cannot restate bit for bit; arbitrary positions are checked against the
reference's own kernels in test_gpu_reference.py). The FP64 oracle bounds the
FP32 error at 1e-5 relative.
"""
import numpy as np
import pytest

from helpers import rel_err, smooth_model, surface_receivers

pytestmark = pytest.mark.gpu

SHAPES = [(40, 20), (20, 40), (61, 33), (33, 200), (200, 33), (100, 100), (37, 70)]


@pytest.fixture(params=["reference", "ieee", "compensated"])
def arith(request, oracle):
    oracle.set_arith(request.param)
    yield request.param
    oracle.set_arith("ieee")


def make_engine(nx, nz, dx, dz, model, arith="ieee"):
    from seisfat2d_gb300 import Engine
    e = Engine(nx, nz, dx, dz)
    e.set_arithmetic(arith)
    e.set_slowness(model)
    return e


@pytest.mark.parametrize("nx,nz", SHAPES)
def test_plain_bitexact_vs_oracle(oracle, engine_lib, cuda, arith, nx, nz):
    dx, dz = 10.0, 10.0
    m = smooth_model(nx, nz, dx, seed=nx * 7 + nz, noise=0.03)
    S = oracle.expand_boundary(m)
    e = make_engine(nx, nz, dx, dz, m, arith)
    srcs = [(0.0, 0.0), ((nx - 1) * dx, 0.0), (0.0, (nz - 1) * dz), ((nx - 1) * dx, (nz - 1) * dz),
            (float(round(nx * 4.37)), float(round(nz * 3.11)))]  # integer metres: exact offsets
    for sx, sz in srcs:
        T = e.time_propagation(sx, sz)
        To = oracle.solve_f32(S, dx, dz, sx, sz)
        assert np.array_equal(T, To), (sx, sz, np.abs(T - To).max())


def test_plain_dx_neq_dz(oracle, engine_lib, cuda, arith):
    nx, nz, dx, dz = 90, 50, 12.5, 7.5
    m = smooth_model(nx, nz, 10.0, seed=11, noise=0.02)
    S = oracle.expand_boundary(m)
    e = make_engine(nx, nz, dx, dz, m, arith)
    T = e.time_propagation(500.0, 30.0)
    assert np.array_equal(T, oracle.solve_f32(S, dx, dz, 500.0, 30.0))


@pytest.mark.parametrize("nx,nz", [(300, 252), (252, 300)])
def test_plain_reproduces_reference_skipped_cells(oracle, engine_lib, cuda, arith, nx, nz):
    # min(nxx, nzz) - 2 = 256: the reference's launch leaves one cell per sweep untouched
    m = smooth_model(nx, nz, 10.0, seed=5)
    S = oracle.expand_boundary(m)
    si, sj = oracle.skip_cells(S.shape[0], S.shape[1])
    assert (si >= 0).all()
    e = make_engine(nx, nz, 10.0, 10.0, m, arith)
    T = e.time_propagation(1000.0, 500.0)
    assert np.array_equal(T, oracle.solve_f32(S, 10.0, 10.0, 1000.0, 500.0, order=0))


@pytest.mark.parametrize("mode", ["reference", "ieee", "compensated"])
def test_fp32_within_1e5_of_fp64(oracle, engine_lib, cuda, mode):
    nx, nz = 301, 101
    m = smooth_model(nx, nz, 10.0, seed=21)
    S = oracle.expand_boundary(m)
    e = make_engine(nx, nz, 10.0, 10.0, m, mode)
    T = e.time_propagation(1500.0, 0.0)
    T64, _ = oracle.solve_f64(S, 10.0, 10.0, 1500.0, 0.0, passes=1)
    inner = (slice(1, -1), slice(1, -1))
    # the compensated pairs keep the FP32 field within a few ulps of FP64
    assert rel_err(T[inner], T64[inner]).max() <= (3e-7 if mode == "compensated" else 1e-5)


@pytest.mark.parametrize("warps,gang", [(1, 0), (1, 1), (1, 2), (2, 0), (4, 3), (8, 0), (16, 16), (3, 5)])
def test_launch_shapes_same_bits(oracle, engine_lib, cuda, arith, warps, gang):
    nx, nz = 150, 140
    m = smooth_model(nx, nz, 10.0, seed=31, noise=0.02)
    S = oracle.expand_boundary(m)
    e = make_engine(nx, nz, 10.0, 10.0, m, arith)
    e.set_launch(warps=warps, gang_warps=gang)
    if arith == "compensated" and warps > 8:
        # its second traveltime ring leaves shared memory for 8 warps per CTA
        from seisfat2d_gb300._lib import EngineError, SF_ERR_ARG
        with pytest.raises(EngineError) as ei:
            e.time_propagation(700.0, 100.0)
        assert ei.value.status == SF_ERR_ARG
        return
    T = e.time_propagation(700.0, 100.0)
    assert np.array_equal(T, oracle.solve_f32(S, 10.0, 10.0, 700.0, 100.0))


def test_picks_plain_and_batched(oracle, engine_lib, cuda, arith):
    import torch
    nx, nz = 120, 50
    m = smooth_model(nx, nz, 10.0, seed=41)
    S = oracle.expand_boundary(m)
    e = make_engine(nx, nz, 10.0, 10.0, m, arith)
    rx, rz = surface_receivers(nx, 10.0, step=3)
    rz = rz + 7.0
    Td = torch.zeros((e.nxx, e.nzz), dtype=torch.float32, device="cuda")
    e.time_propagation(333.0, 12.0, out=Td)
    pk = e.compute_seismogram(Td, rx, rz)
    To = oracle.solve_f32(S, 10.0, 10.0, 333.0, 12.0)
    po = oracle.picks(To, 10.0, 10.0, rx, rz)
    assert np.array_equal(pk, po)
    pb = e.batch_forward([(333.0, 12.0)], rx, rz)
    assert np.array_equal(pb[0], po)


def test_batched_windows_equal_plain_per_window(oracle, engine_lib, cuda, arith):
    nx, nz = 300, 70
    m = smooth_model(nx, nz, 10.0, seed=51, noise=0.02)
    S = oracle.expand_boundary(m)
    e = make_engine(nx, nz, 10.0, 10.0, m, arith)
    rng = np.random.default_rng(3)
    shots = []
    for k in range(23):
        sx = float(int(rng.uniform(0, (nx - 1) * 10.0)))
        sidx = int((sx + 5.0) / 10.0) + 3
        c0 = max(0, sidx - int(rng.integers(5, 120)))
        c1 = min(e.nxx, sidx + int(rng.integers(5, 120)))
        shots.append((sx, float(int(rng.uniform(0, 200.0))), c0, c1 - c0))
    shots.append((1500.0, 0.0, 0, 0))  # full width
    rx, rz = surface_receivers(nx, 10.0, step=2)
    pk = e.batch_forward(shots, rx, rz, keep_tables=True)
    for b, (sx, sz, c0, nc) in enumerate(shots):
        ncols = nc if nc > 0 else e.nxx - c0
        Tb = e.batch_table(b, ncols)
        To, po = oracle.shot(S, 10.0, 10.0, sx, sz, rx, rz, c0=c0, ncols=ncols)
        assert np.array_equal(Tb, To), b
        assert np.array_equal(pk[b], po, equal_nan=True), b


def test_batched_many_shots_grid_smaller_than_batch(oracle, engine_lib, cuda, arith):
    nx, nz = 200, 90
    m = smooth_model(nx, nz, 10.0, seed=61)
    S = oracle.expand_boundary(m)
    e = make_engine(nx, nz, 10.0, 10.0, m, arith)
    e.set_launch(warps=1, gang_warps=1)  # one warp per shot: every strip in turn
    shots = [(float(5.0 * (k % 398)), 0.0) for k in range(400)]
    rx, rz = surface_receivers(nx, 10.0, step=4)
    pk = e.batch_forward(shots, rx, rz)
    for b in (0, 57, 199, 399):
        _, po = oracle.shot(S, 10.0, 10.0, shots[b][0], 0.0, rx, rz)
        assert np.array_equal(pk[b], po, equal_nan=True)


def test_anisotropic_bitexact(oracle, engine_lib, cuda, arith):
    from seisfat2d_gb300.synthetic import thomsen_stiffness
    nx, nz = 90, 45
    rng = np.random.default_rng(7)
    vp = 1.0 / smooth_model(nx, nz, 10.0, seed=71)
    eps = rng.uniform(0.0, 0.25, (nx, nz))
    dl = rng.uniform(-0.05, 0.15, (nx, nz))
    cij = [c.astype(np.float32) for c in thomsen_stiffness(vp, vp / np.sqrt(3), 1000.0, eps, dl, 0.0)]
    m = (1.0 / vp).astype(np.float32)
    e = make_engine(nx, nz, 10.0, 10.0, m, arith)
    e.set_stiffness(cij)
    S = oracle.expand_boundary(m)
    codes, mm = [], []
    for c in cij:
        cd, mn, mx = oracle.compress(oracle.expand_boundary(c))
        codes.append(cd)
        mm += [mn, mx]
    mm = np.array(mm, np.float32)
    for (sx, sz) in [(450.0, 0.0), (0.0, 200.0), (890.0, 440.0)]:
        T = e.time_propagation(sx, sz, ani=True)
        To, _ = oracle.shot(S, 10.0, 10.0, sx, sz, ani=(codes, mm))
        assert np.array_equal(T, To), (sx, sz)
    rx, rz = surface_receivers(nx, 10.0, step=2)
    pk = e.batch_forward([(450.0, 0.0), (123.0, 60.0, 5, 50)], rx, rz, ani=True)
    _, po = oracle.shot(S, 10.0, 10.0, 123.0, 60.0, rx, rz, c0=5, ncols=50, ani=(codes, mm))
    assert np.array_equal(pk[1], po, equal_nan=True)


def test_errors_are_status_codes(engine_lib, cuda):
    from seisfat2d_gb300 import Engine, EngineError
    from seisfat2d_gb300._lib import SF_ERR_RANGE, SF_ERR_STATE
    e = Engine(50, 30, 10.0, 10.0)
    e.set_slowness(np.full((50, 30), 1 / 2000.0, np.float32))
    with pytest.raises(EngineError) as ex:
        e.time_propagation(-100.0, 0.0)
    assert ex.value.status == SF_ERR_RANGE
    with pytest.raises(EngineError) as ex:
        e.batch_forward([(100.0, 0.0, 40, 30)], np.zeros(1, np.float32), np.zeros(1, np.float32))
    assert ex.value.status == SF_ERR_RANGE
    with pytest.raises(EngineError) as ex:
        e.time_propagation(100.0, 0.0, ani=True)
    assert ex.value.status == SF_ERR_STATE
    with pytest.raises(EngineError) as ex:
        e.batch_adjoint(np.zeros((1, 1), np.float32))
    assert ex.value.status == SF_ERR_STATE
    # the context stays usable after refusals
    T = e.time_propagation(250.0, 0.0)
    assert np.isfinite(T).all()
