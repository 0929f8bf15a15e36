"""The least-squares Kirchhoff operators through the C ABI
(sf_forward_convolution, sf_kirchhoff_image_forward,
sf_kirchhoff_angle_forward): the convolution bit-identical to the oracle's
direct FP64 restatement of the reference's FFT product, the forward operators
within rounding of the oracle's exactly summed traces and of the reference's
own forward kernels (which add with atomics in no fixed order), repeatable bit
for bit, and adjoint to the migration kernels (dot-product test)."""
import numpy as np
import pytest

from helpers import smooth_model

pytestmark = pytest.mark.gpu

DT, AP = 0.002, 40.0


def case(oracle, nx=48, nz=30, seed=3, nt=250):
    m = smooth_model(nx, nz, 10.0, seed=seed)
    S = oracle.expand_boundary(m)
    xs = np.array([55.0, 200.0, 330.0], np.float32)
    xr = np.arange(5.0, 470.0, 35.0).astype(np.float32)
    Ts = np.stack([oracle.solve_f32(S, 10.0, 10.0, float(x), 0.0) for x in xs])
    Tr = np.stack([oracle.solve_f32(S, 10.0, 10.0, float(x), 0.0) for x in xr])
    rng = np.random.default_rng(seed)
    return m, S, xs, xr, Ts, Tr, rng


def engine(m):
    from seisfat2d_gb300 import Engine
    e = Engine(m.shape[0], m.shape[1], 10.0, 10.0)
    e.set_slowness(m)
    return e


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-30))


def test_forward_convolution_bitexact_vs_oracle(oracle, engine_lib, cuda):
    from seisfat2d_gb300 import Engine
    e = Engine(20, 10, 10.0, 10.0)
    tr = np.random.default_rng(1).standard_normal((7, 400)).astype(np.float32)
    got = e.forward_convolution(tr, 0.002, 20.0)
    assert np.abs(got).max() > 0
    assert np.array_equal(got, oracle.forward_convolution(tr, 0.002, 20.0))
    dev = cuda.from_numpy(tr).cuda()
    out = cuda.empty_like(dev)
    e.forward_convolution(dev, 0.002, 20.0, out=out)
    cuda.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), got)


@pytest.mark.parametrize("max_off", [1000.0, 200.0])
def test_image_forward_vs_oracle_and_reference(oracle, engine_lib, cuda, max_off):
    m, S, xs, xr, Ts, Tr, rng = case(oracle)
    e = engine(m)
    nt = 250
    img = rng.standard_normal((m.shape[0], m.shape[1])).astype(np.float32)
    dTs, dTr = cuda.from_numpy(Ts).cuda(), cuda.from_numpy(Tr).cuda()
    got = e.kirchhoff_image_forward(dTs, dTr, xs, xr, img, nt, DT, AP, max_off)
    orc = oracle.kirchhoff_image_forward(S, Ts, Tr, xs, xr, img, nt, DT, 10.0, 10.0, AP, max_off)
    far = np.abs(xs[:, None] - xr[None, :]) >= max_off
    assert not got[far].any()
    assert np.abs(orc).max() > 0
    print(f"max offset {max_off}: |engine - oracle| / max|oracle| = {rel(got, orc):.2e}")
    assert rel(got, orc) <= 2e-5
    # repeatable bit for bit, host and device buffers alike
    again = e.kirchhoff_image_forward(dTs, dTr, xs, xr, cuda.from_numpy(img).cuda(), nt, DT, AP, max_off)
    dev = cuda.zeros((len(xs), len(xr), nt), dtype=cuda.float32, device="cuda")
    e.kirchhoff_image_forward(dTs, dTr, xs, xr, cuda.from_numpy(img).cuda(), nt, DT, AP, max_off, out=dev)
    cuda.cuda.synchronize()
    assert np.array_equal(got, again) and np.array_equal(dev.cpu().numpy(), got)
    from oracle import refkernels
    if not refkernels.available():
        pytest.skip("reference kernels not built")
    ref = refkernels.kirchhoff_forward(S, Ts, Tr, xs, xr, img, nt, DT, 10.0, 10.0, AP, max_off)
    print(f"|engine - reference kernel| / max = {rel(got, ref)}, |oracle - reference| / max = {rel(orc, ref):.2e}")
    assert rel(got, ref) <= 2e-5


def test_angle_forward_vs_oracle_and_reference(oracle, engine_lib, cuda):
    m, S, xs, xr, Ts, Tr, rng = case(oracle, seed=5)
    e = engine(m)
    nt, max_off, max_ang, da = 250, 400.0, 60.0, 2.0
    na, nc, _, _ = oracle.angle_bins(xs, xr, max_ang, da)
    g = rng.standard_normal((nc, na, m.shape[1])).astype(np.float32)
    dTs, dTr = cuda.from_numpy(Ts).cuda(), cuda.from_numpy(Tr).cuda()
    got = e.kirchhoff_angle_forward(dTs, dTr, xs, xr, g, nt, DT, AP, max_off, max_ang, da)
    orc = oracle.kirchhoff_angle_forward(S, Ts, Tr, xs, xr, g, nt, DT, 10.0, 10.0, AP, max_off, max_ang, da)
    assert np.abs(orc).max() > 0
    print(f"|engine - oracle| / max|oracle| = {rel(got, orc):.2e}")
    assert rel(got, orc) <= 2e-5
    assert np.array_equal(got, e.kirchhoff_angle_forward(dTs, dTr, xs, xr, g, nt, DT, AP, max_off, max_ang, da))
    from oracle import refkernels
    if not refkernels.available():
        pytest.skip("reference kernels not built")
    ref = refkernels.kirchhoff_forward(S, Ts, Tr, xs, xr, g, nt, DT, 10.0, 10.0, AP, max_off, max_ang, da)
    print(f"|engine - reference kernel| / max = {rel(got, ref):.2e}")
    assert rel(got, ref) <= 2e-5


def test_forward_in_chunks(oracle, engine_lib, cuda):
    """A grid of more than 4096 cells with few traces splits each trace's
    cells over several CTAs whose partial traces are summed in chunk order."""
    m, S, xs, xr, Ts, Tr, rng = case(oracle, nx=140, nz=60, seed=9)
    e = engine(m)
    xs, xr, Ts, Tr = xs[:1], xr[:2], Ts[:1], Tr[:2]
    img = rng.standard_normal((140, 60)).astype(np.float32)
    nt = 400
    dTs, dTr = cuda.from_numpy(Ts).cuda(), cuda.from_numpy(Tr).cuda()
    got = e.kirchhoff_image_forward(dTs, dTr, xs, xr, img, nt, DT, AP, 1e4)
    orc = oracle.kirchhoff_image_forward(S, Ts, Tr, xs, xr, img, nt, DT, 10.0, 10.0, AP, 1e4)
    print(f"|engine - oracle| / max|oracle| = {rel(got, orc):.2e}")
    assert np.abs(orc).max() > 0 and rel(got, orc) <= 2e-5
    assert np.array_equal(got, e.kirchhoff_image_forward(dTs, dTr, xs, xr, img, nt, DT, AP, 1e4))


def test_forward_and_migration_are_adjoint(oracle, engine_lib, cuda):
    """<F m, d> = <m, F^T d> with F^T the migration kernels
    (sf_kirchhoff_image, sf_kirchhoff_angle_gathers), image and angle domain."""
    m, S, xs, xr, Ts, Tr, rng = case(oracle, seed=11)
    e = engine(m)
    nt, max_off, max_ang, da = 250, 400.0, 60.0, 2.0
    dTs, dTr = cuda.from_numpy(Ts).cuda(), cuda.from_numpy(Tr).cuda()
    d = rng.standard_normal((len(xs), len(xr), nt)).astype(np.float32)
    img = rng.standard_normal((m.shape[0], m.shape[1])).astype(np.float32)
    Fm = e.kirchhoff_image_forward(dTs, dTr, xs, xr, img, nt, DT, AP, max_off)
    Ftd = e.kirchhoff_image(dTs, dTr, xs, xr, d, DT, AP, max_off)
    lhs, rhs = np.dot(Fm.ravel().astype(np.float64), d.ravel()), np.dot(img.ravel().astype(np.float64), Ftd.ravel())
    print(f"image domain: <Fm, d> = {lhs:.6e}, <m, F^T d> = {rhs:.6e}")
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs))
    Gt = e.kirchhoff_angle_gathers(dTs, dTr, xs, xr, d, DT, AP, max_off, max_ang, da)
    g = rng.standard_normal(Gt.shape).astype(np.float32)
    Fg = e.kirchhoff_angle_forward(dTs, dTr, xs, xr, g, nt, DT, AP, max_off, max_ang, da)
    lhs, rhs = np.dot(Fg.ravel().astype(np.float64), d.ravel()), np.dot(g.ravel().astype(np.float64), Gt.ravel())
    print(f"angle domain: <Fg, d> = {lhs:.6e}, <g, F^T d> = {rhs:.6e}")
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs))


def test_forward_rejects_bad_arguments(oracle, engine_lib, cuda):
    from seisfat2d_gb300 import EngineError
    m, S, xs, xr, Ts, Tr, rng = case(oracle)
    e = engine(m)
    dTs, dTr = cuda.from_numpy(Ts).cuda(), cuda.from_numpy(Tr).cuda()
    img = np.zeros((m.shape[0], m.shape[1]), np.float32)
    with pytest.raises(EngineError):
        e.kirchhoff_image_forward(dTs, dTr, xs, xr, img, 0, DT, AP, 100.0)
    with pytest.raises(EngineError):
        e.kirchhoff_image_forward(dTs, dTr, xs, xr, img, 10, -1.0, AP, 100.0)
    with pytest.raises(EngineError):  # one source: no CMP spacing
        e.kirchhoff_angle_forward(dTs, dTr, xs[:1], xr, np.zeros(10, np.float32), 10, DT, AP, 100.0, 60.0, 2.0)
    with pytest.raises(EngineError):  # histogram larger than shared memory
        e.kirchhoff_image_forward(dTs, dTr, xs, xr, img, 60000, DT, AP, 100.0)
