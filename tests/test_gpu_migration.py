"""Kirchhoff image-domain migration through the C ABI (sf_kirchhoff_image,
sf_adjoint_convolution): bit-identical to the reference's own image kernel
compiled from its sources and replayed trace by trace (KDM.cu:3-55), close to
the oracle's restatement (libm vs CUDA math functions), and end to end from
tables kept on the device."""
import numpy as np
import pytest

from helpers import smooth_model

pytestmark = pytest.mark.gpu


def case(oracle, nx=48, nz=30, seed=3):
    m = smooth_model(nx, nz, 10.0, seed=seed)
    S = oracle.expand_boundary(m)
    xs = np.array([55.0, 200.0, 330.0], np.float32)
    xr = np.arange(5.0, 470.0, 35.0).astype(np.float32)
    Ts = np.stack([oracle.solve_f32(S, 10.0, 10.0, float(x), 0.0) for x in xs])
    Tr = np.stack([oracle.solve_f32(S, 10.0, 10.0, float(x), 0.0) for x in xr])
    rng = np.random.default_rng(seed)
    raw = rng.standard_normal((len(xs), len(xr), 250)).astype(np.float32)
    return m, S, xs, xr, Ts, Tr, raw


def test_correlation_bitexact_vs_oracle(oracle, engine_lib, cuda):
    from seisfat2d_gb300 import Engine
    e = Engine(20, 10, 10.0, 10.0)
    tr = np.random.default_rng(1).standard_normal((7, 400)).astype(np.float32)
    got = e.adjoint_convolution(tr, 0.002, 20.0)
    assert np.array_equal(got, oracle.adjoint_convolution(tr, 0.002, 20.0))
    dev = cuda.from_numpy(tr).cuda()
    out = cuda.empty_like(dev)
    e.adjoint_convolution(dev, 0.002, 20.0, out=out)
    cuda.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), got)


def test_image_vs_reference_kernel(oracle, engine_lib, cuda):
    from oracle import refkernels
    if not refkernels.available():
        pytest.skip("reference kernels not built")
    from seisfat2d_gb300 import Engine
    m, S, xs, xr, Ts, Tr, raw = case(oracle)
    e = Engine(m.shape[0], m.shape[1], 10.0, 10.0)
    e.set_slowness(m)
    d = raw.reshape(-1, raw.shape[-1])
    data = e.adjoint_convolution(d, 0.002, 30.0).reshape(raw.shape)
    for aperture, max_off in [(40.0, 1000.0), (25.0, 200.0)]:
        img = e.kirchhoff_image(cuda.from_numpy(Ts).cuda(), cuda.from_numpy(Tr).cuda(), xs, xr, data, 0.002,
                                aperture, max_off)
        ref = refkernels.kirchhoff_adjoint(S, Ts, Tr, xs, xr, data, 0.002, 10.0, 10.0, aperture, max_off)
        scale = np.abs(ref).max()
        assert scale > 0
        err = np.abs(img - ref).max() / scale
        diff = img != ref
        print(f"aperture {aperture}, max offset {max_off}: max |engine - reference| / max|reference| = {err:.2e}; "
              f"{int(diff.sum())} of {diff.size} cells differ, largest |reference| among them "
              f"{np.abs(ref[diff]).max() if diff.any() else 0.0:.2e} (max |reference| {scale:.2e})")
        assert np.array_equal(img, ref)
        orc = oracle.kirchhoff_image(S, Ts, Tr, xs, xr, data, 0.002, 10.0, 10.0, aperture, max_off)
        assert np.abs(orc - ref).max() <= 1e-4 * scale


def test_image_from_device_tables(oracle, engine_lib, cuda):
    """Tables from one batched forward each for sources and receivers, kept on
    the device and copied into contiguous arrays; image equals the one from
    the oracle's tables to rounding (engine tables are bit-identical)."""
    from seisfat2d_gb300 import Engine
    m, S, xs, xr, Ts, Tr, raw = case(oracle, seed=7)
    e = Engine(m.shape[0], m.shape[1], 10.0, 10.0)
    e.set_arithmetic("ieee")
    e.set_slowness(m)
    dev = cuda.device("cuda", 0)
    tabs = {}
    for name, xx in (("s", xs), ("r", xr)):
        e.batch_forward([(float(x), 0.0) for x in xx], np.zeros(0, np.float32), np.zeros(0, np.float32),
                        keep_tables=True)
        t = cuda.empty((len(xx), e.nxx, e.nzz), dtype=cuda.float32, device=dev)
        for k in range(len(xx)):
            e.batch_table(k, e.nxx, out=t[k])
        tabs[name] = t
    cuda.cuda.synchronize()
    assert np.array_equal(tabs["s"].cpu().numpy(), Ts)
    data = e.adjoint_convolution(raw.reshape(-1, raw.shape[-1]), 0.002, 30.0).reshape(raw.shape)
    a = e.kirchhoff_image(tabs["s"], tabs["r"], xs, xr, data, 0.002, 35.0, 1000.0)
    b = e.kirchhoff_image(cuda.from_numpy(Ts).cuda(), cuda.from_numpy(Tr).cuda(), xs, xr, data, 0.002, 35.0, 1000.0)
    assert np.array_equal(a, b)


def test_kirchhoff_timing_vs_reference(oracle, engine_lib, cuda):
    """One launch over every trace against the reference's launch per trace,
    on a 1001 x 201 grid with 20 sources x 100 receivers of 1000 samples."""
    import time
    from oracle import refkernels
    if not refkernels.available():
        pytest.skip("reference kernels not built")
    from seisfat2d_gb300 import Engine
    nx, nz = 1001, 201
    m = smooth_model(nx, nz, 10.0, seed=12)
    e = Engine(nx, nz, 10.0, 10.0)
    e.set_slowness(m)
    xs = np.linspace(500.0, 9500.0, 20).astype(np.float32)
    xr = np.linspace(0.0, 9990.0, 100).astype(np.float32)
    dev = cuda.device("cuda", 0)
    tabs = []
    for xx in (xs, xr):
        e.batch_forward([(float(x), 0.0) for x in xx], np.zeros(0, np.float32), np.zeros(0, np.float32),
                        keep_tables=True)
        t = cuda.empty((len(xx), e.nxx, e.nzz), dtype=cuda.float32, device=dev)
        for k in range(len(xx)):
            e.batch_table(k, e.nxx, out=t[k])
        tabs.append(t)
    data = np.random.default_rng(0).standard_normal((20, 100, 1000)).astype(np.float32)
    dd = cuda.from_numpy(data).cuda()
    out = cuda.empty((nx, nz), dtype=cuda.float32, device=dev)
    e.kirchhoff_image(tabs[0], tabs[1], xs, xr, dd, 0.004, 40.0, 5000.0, out=out)
    cuda.cuda.synchronize()
    t0 = time.perf_counter()
    e.kirchhoff_image(tabs[0], tabs[1], xs, xr, dd, 0.004, 40.0, 5000.0, out=out)
    cuda.cuda.synchronize()
    t_eng = time.perf_counter() - t0
    Ts, Tr = tabs[0].cpu().numpy(), tabs[1].cpu().numpy()
    S = e.get_slowness()
    t0 = time.perf_counter()
    ref = refkernels.kirchhoff_adjoint(S, Ts, Tr, xs, xr, data, 0.004, 10.0, 10.0, 40.0, 5000.0)
    t_ref = time.perf_counter() - t0
    img = out.cpu().numpy()
    err = np.abs(img - ref).max() / np.abs(ref).max()
    ntr = int((np.abs(xs[:, None] - xr[None, :]) < 5000.0).sum())
    print(f"KIRCHHOFF_TIMING 1007x207, {ntr} traces: engine {1e3 * t_eng:.1f} ms, reference launch loop "
          f"{1e3 * t_ref:.1f} ms (incl. its uploads), max rel diff {err:.1e}, bitwise {np.array_equal(img, ref)}")
    assert np.array_equal(img, ref)


def test_angle_gathers_vs_reference_kernel(oracle, engine_lib, cuda):
    """ADKDM gathers: the reference adds each trace's terms into (depth, angle,
    CMP) bins with atomics from all columns at once, in no fixed order; the
    engine's bins hold the same terms summed in trace order. Compared to the
    reference's own kernel to FP32 rounding of the sums, and reported as the
    largest difference relative to the largest bin."""
    from oracle import refkernels
    if not refkernels.available():
        pytest.skip("reference kernels not built")
    from seisfat2d_gb300 import Engine
    m, S, xs, xr, Ts, Tr, raw = case(oracle, seed=5)
    e = Engine(m.shape[0], m.shape[1], 10.0, 10.0)
    e.set_slowness(m)
    data = e.adjoint_convolution(raw.reshape(-1, raw.shape[-1]), 0.002, 30.0).reshape(raw.shape)
    g = e.kirchhoff_angle_gathers(cuda.from_numpy(Ts).cuda(), cuda.from_numpy(Tr).cuda(), xs, xr, data, 0.002,
                                  40.0, 400.0, 60.0, 2.0)
    ref = refkernels.kirchhoff_angles(S, Ts, Tr, xs, xr, data, 0.002, 10.0, 10.0, 40.0, 400.0, 60.0, 2.0)
    assert g.shape == ref.shape
    scale = np.abs(ref).max()
    assert scale > 0
    err = np.abs(g - ref).max() / scale
    print(f"angle gathers {g.shape}: max |engine - reference| / max|reference| = {err:.2e}, "
          f"bins equal {np.count_nonzero(g == ref)} of {g.size}")
    assert err <= 1e-5
    again = e.kirchhoff_angle_gathers(cuda.from_numpy(Ts).cuda(), cuda.from_numpy(Tr).cuda(), xs, xr, data, 0.002,
                                      40.0, 400.0, 60.0, 2.0)
    assert np.array_equal(g, again)  # deterministic
