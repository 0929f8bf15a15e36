"""CPU checks of the oracle itself: the restated launch schedule, the FP64
modes, analytic known answers and the quantisation."""
import numpy as np
import pytest

from helpers import layered, rel_err, smooth_model


def coverage(nxx, nzz, nthreads=256):
    """Which interior cells the reference's per-level launches reach
    (modeling.cu:123-159, restated with numpy for the test)."""
    total = nxx + nzz - 2
    mn, mx = min(nxx, nzz), max(nxx, nzz)
    res = []
    for sweep in range(4):
        zd = -1 if sweep in (2, 3) else 1
        xd = -1 if sweep in (0, 2) else 1
        cov = np.zeros((nzz, nxx), np.int32)
        for level in range(total):
            if sweep == 0:
                zo = 0 if level < nxx else level - nxx + 1
                xo = level if level < nxx else nxx - 1
            elif sweep == 1:
                zo = nzz - level - 1 if level < nzz else 0
                xo = 0 if level < nzz else level - nzz + 1
            elif sweep == 2:
                zo = level if level < nzz else nzz - 1
                xo = nxx - 1 if level < nzz else nxx - 1 - (level - nzz + 1)
            else:
                zo = nzz - 1 if level < nxx else nzz - 1 - (level - nxx + 1)
                xo = nxx - level - 1 if level < nxx else 0
            n = level + 1 if level < mn else (total - level if level >= mx else total - mn - mx + level)
            e = np.arange(((n + nthreads - 1) // nthreads) * nthreads)
            i, j = zo + zd * e, xo + xd * e
            m = (i > 0) & (i < nzz - 1) & (j > 0) & (j < nxx - 1)
            np.add.at(cov, (i[m], j[m]), 1)
        res.append(cov)
    return res


@pytest.mark.parametrize("nxx,nzz", [(26, 16), (16, 26), (23, 23), (300, 258), (258, 300), (514, 258)])
def test_skip_cells_match_launch_coverage(oracle, nxx, nzz):
    si, sj = oracle.skip_cells(nxx, nzz)
    cov = coverage(nxx, nzz)
    for s in range(4):
        inner = cov[s][1:-1, 1:-1]
        assert inner.max() <= 1, "a level launch never updates a cell twice"
        miss = np.argwhere(inner == 0) + 1
        assert len(miss) <= 1
        if len(miss):
            assert (si[s], sj[s]) == tuple(miss[0])
        else:
            assert si[s] == -1 and sj[s] == -1
    has_skip = (min(nxx, nzz) - 2) % 256 == 0
    assert (si >= 0).any() == has_skip


@pytest.mark.parametrize("nx,nz", [(40, 20), (20, 40), (57, 33), (252, 20), (20, 252)])
def test_launch_order_equals_loop_order(oracle, nx, nz):
    S = oracle.expand_boundary(smooth_model(nx, nz, 10.0, seed=nx + nz, noise=0.02))
    for (sx, sz) in [(0.0, 0.0), ((nx - 1) * 10.0, (nz - 1) * 10.0), (nx * 4.3, nz * 6.1)]:
        Ta = oracle.solve_f32(S, 10.0, 10.0, sx, sz, order=0)
        Tb = oracle.solve_f32(S, 10.0, 10.0, sx, sz, order=1)
        assert np.array_equal(Ta, Tb)


def test_launch_order_equals_loop_order_with_skipped_cells(oracle):
    nx, nz = 252, 30  # nzz = 36, nxx = 258: min-2 = 34 (no skip) -> use nzz = 258 below
    S = oracle.expand_boundary(smooth_model(40, 252, 10.0, seed=3))  # nxx = 46, nzz = 258
    si, sj = oracle.skip_cells(S.shape[0], S.shape[1])
    assert (si < 0).all()
    S = oracle.expand_boundary(smooth_model(300, 252, 10.0, seed=4))  # nzz = 258 -> skips
    si, sj = oracle.skip_cells(S.shape[0], S.shape[1])
    assert (si >= 0).all()
    Ta = oracle.solve_f32(S, 10.0, 10.0, 1234.0, 20.0, order=0)
    Tb = oracle.solve_f32(S, 10.0, 10.0, 1234.0, 20.0, order=1)
    assert np.array_equal(Ta, Tb)


def test_fp32_matches_fp64_schedule(oracle):
    S = oracle.expand_boundary(smooth_model(201, 81, 10.0, seed=7))
    T32 = oracle.solve_f32(S, 10.0, 10.0, 1000.0, 0.0)
    T64, n = oracle.solve_f64(S, 10.0, 10.0, 1000.0, 0.0, passes=1)
    assert n == 1
    inner = (slice(3, -3), slice(3, -3))
    assert rel_err(T32[inner], T64[inner]).max() < 1e-5


def test_homogeneous_first_order_error_bound(oracle):
    nx, nz, h, v = 121, 61, 10.0, 2000.0
    S = oracle.expand_boundary(np.full((nx, nz), 1.0 / v, np.float32))
    sx, sz = 600.0, 0.0
    T, _ = oracle.solve_f64(S, h, h, sx, sz, passes=1)
    x = (np.arange(nx + 6) - 3) * h
    z = (np.arange(nz + 6) - 3) * h
    Ta = np.hypot(x[:, None] - sx, z[None, :] - sz) / v
    inner = (slice(3, -3), slice(3, -3))
    err = np.abs(T[inner] - Ta[inner])
    # first-order scheme: error grows like log(r) * h / v at most a few cells' time
    assert err.max() < 4 * h / v
    far = Ta[inner] > 20 * h / v
    assert (err[far] / Ta[inner][far]).max() < 0.05


def analytic_head_wave(v, z, x):
    """Flat-layer refraction times (src/functions.py:23-33, restated)."""
    out = np.zeros((len(z), len(x)))
    for n in range(len(z)):
        out[n] = x / v[n + 1]
        for i in range(n + 1):
            ang = np.arcsin(v[i] / v[n + 1])
            out[n] += 2.0 * z[i] * np.cos(ang) / v[i]
    return out


def test_two_layer_head_wave(oracle):
    nx, nz, h = 401, 61, 10.0
    v = [1500.0, 3000.0]
    S = oracle.expand_boundary(layered(nx, nz, h, v, [200.0]))
    T, _ = oracle.solve_f64(S, h, h, 0.0, 0.0, passes=0, tol=0.0)
    x = np.arange(nx) * h
    head = analytic_head_wave(np.array(v), np.array([200.0]), x)[0]
    direct = x / v[0]
    first = np.minimum(head, direct)
    Tsurf = T[3:-3, 3]
    far = x > 1500.0
    assert (np.abs(Tsurf[far] - first[far]) / first[far]).max() < 0.02


def test_compress_deterministic_and_decodes_within_step(oracle):
    rng = np.random.default_rng(0)
    f = rng.uniform(1e9, 9e9, (50, 40)).astype(np.float32)
    c1, mn1, mx1 = oracle.compress(f)
    c2, mn2, mx2 = oracle.compress(f)
    assert np.array_equal(c1, c2) and mn1 == mn2 and mx1 == mx2
    assert mn1 == f.min() and mx1 == f.max()
    dec = mn1 + (c1.astype(np.float32) - 1.0) * (mx1 - mn1) / 65534.0
    assert np.abs(dec - f).max() <= (mx1 - mn1) / 65534.0 * 1.01
    z = np.zeros((10, 10), np.float32)
    cz, mnz, mxz = oracle.compress(z)
    assert (cz == 1).all() and mnz == 0.0 and mxz == 0.0


def numpy_cubic2d(T, i, j, xd, zd):
    def c1d(P, t):
        return P[1] + 0.5 * t * (P[2] - P[0] + t * (2 * P[0] - 5 * P[1] + 4 * P[2] - P[3] +
                                                    t * (3 * (P[1] - P[2]) + P[3] - P[0])))
    p = [c1d([T[j + a - 1, i + b - 1] for b in range(4)], zd) for a in range(4)]
    return c1d(p, xd)


def test_picks_match_independent_cubic(oracle):
    S = oracle.expand_boundary(smooth_model(80, 40, 10.0, seed=9))
    T = oracle.solve_f32(S, 10.0, 10.0, 300.0, 0.0)
    rng = np.random.default_rng(1)
    rx = rng.uniform(0, 790.0, 50).astype(np.float32)
    rz = rng.uniform(0, 390.0, 50).astype(np.float32)
    pk = oracle.picks(T, 10.0, 10.0, rx, rz)
    for r in range(50):
        i = int((rz[r] + 5.0) / 10.0) + 3
        j = int((rx[r] + 5.0) / 10.0) + 3
        x0 = np.floor((rx[r] + 5.0) / 10.0) * 10.0
        z0 = np.floor((rz[r] + 5.0) / 10.0) * 10.0
        ref = numpy_cubic2d(T.astype(np.float64), i, j, (rx[r] - x0) / 10.0, (rz[r] - z0) / 10.0)
        assert abs(pk[r] - ref) <= 1e-5 * abs(ref) + 1e-6


def test_window_solve_is_crop_solve(oracle):
    S = oracle.expand_boundary(smooth_model(120, 40, 10.0, seed=5))
    c0, nc = 30, 60
    Tw = oracle.solve_f32(S, 10.0, 10.0, 600.0, 0.0, c0=c0, ncols=nc)
    assert Tw.shape == (nc, S.shape[1])
    T, pk = oracle.shot(S, 10.0, 10.0, 600.0, 0.0, c0=c0, ncols=nc)
    assert np.array_equal(T, Tw)


def golden_cases():
    import glob
    import os
    return sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "*.npz")))


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: p.split("/")[-1][:-4])
def test_oracle_matches_reference_kernel_golden_vectors(oracle, path):
    """Golden vectors: the reference's own kernels run on a GB300 (see
    tests/golden/make_golden.py). In reference arithmetic (FP32 init, nvcc's
    FMA sites) the oracle reproduces them bit for bit; in IEEE arithmetic
    (every operation rounded once, FP64 init) to the 1e-5 relative tolerance."""
    d = np.load(path)
    S, dx, dz, sx, sz = d["S"], float(d["dx"]), float(d["dz"]), float(d["sx"]), float(d["sz"])
    try:
        for mode in ("reference", "ieee"):
            oracle.set_arith(mode)
            if "codes" in d:
                T, _ = oracle.shot(S, dx, dz, sx, sz, ani=(list(d["codes"]), d["mm"]))
            else:
                T = oracle.solve_f32(S, dx, dz, sx, sz, order=0)
            if mode == "reference":
                assert np.array_equal(T, d["T_ref"])
            else:
                assert rel_err(T, d["T_ref"]).max() <= 1e-4
    finally:
        oracle.set_arith("ieee")
    assert len(golden_cases()) >= 7


def test_fp64_adjoint_matches_finite_differences(oracle):
    """Central differences of the FP64 misfit on 32 seeded interior cells
    (cells where the difference quotient is stable under halving h)."""
    nx, nz, h = 48, 26, 10.0
    m = smooth_model(nx, nz, h, seed=12, noise=0.03)
    S = oracle.expand_boundary(m).astype(np.float32)
    rx = (np.arange(2, nx - 2, 2) * h).astype(np.float32)
    rz = np.full_like(rx, 20.0)
    shots = [(120.0, 0.0), (300.0, 60.0)]
    tobs = np.zeros((len(shots), len(rx)))

    def misfit(Sm):
        _, pk = oracle.batch_gradient(Sm, h, h, shots, rx, rz, np.zeros((len(shots), len(rx))), fp64=True)
        r = pk - tobs
        return 0.5 * np.nansum(r * r), r

    J0, r0 = misfit(S)
    g, _ = oracle.batch_gradient(S, h, h, shots, rx, rz, r0, fp64=True)
    rng = np.random.default_rng(5)
    cells = [(int(rng.integers(4, nx + 2)), int(rng.integers(4, nz + 2))) for _ in range(32)]
    ok = 0
    for (j, i) in cells:
        vals = []
        for eps in (1e-3, 5e-4):
            d = eps * float(S[j, i])
            Sp, Sn = S.astype(np.float64).copy(), S.astype(np.float64).copy()
            Sp[j, i] += d
            Sn[j, i] -= d
            # the oracle's FP64 path reads FP32 slowness: perturb in FP64 via a scaled model
            Jp, _ = misfit(Sp.astype(np.float32))
            Jn, _ = misfit(Sn.astype(np.float32))
            dp = float(Sp.astype(np.float32)[j, i]) - float(Sn.astype(np.float32)[j, i])
            vals.append((Jp - Jn) / dp)
        fd = vals[0]
        scale = max(abs(fd), abs(g[j, i]), 1e-12 * abs(J0) + 1e-30)
        if abs(vals[0] - vals[1]) <= 1e-3 * scale and abs(fd - g[j, i]) <= 1e-3 * scale:
            ok += 1
    assert ok >= 28, ok


def test_threaded_batch_gradient_matches_per_shot_path(oracle):
    """orc_batch_gradient_f32 (one shot per thread, FP64 ordered sum) equals
    the per-shot tape/seed/adjoint path and its misfit the FP64 sum of the
    FP32 residuals."""
    rng = np.random.default_rng(0)
    S = oracle.expand_boundary((1.0 / rng.uniform(1500, 3000, (60, 40))).astype(np.float32))
    shots = [(100.0, 0.0), (300.0, 50.0, 10, 40), (500.0, 20.0), (250.0, 0.0, 0, 35)]
    rx = np.linspace(0, 590, 25).astype(np.float32)
    rz = np.full(25, 5.0, np.float32)
    tobs = rng.normal(0.2, 0.02, (len(shots), 25)).astype(np.float32)
    tobs[1, 3] = np.nan
    J, g, pk, used = oracle.batch_misfit_gradient(S, 10.0, 10.0, shots, rx, rz, tobs)
    _, pk2 = oracle.batch_gradient(S, 10.0, 10.0, shots, rx, rz, np.zeros_like(tobs))
    pg = (pk2 - tobs).astype(np.float32)
    g2, _ = oracle.batch_gradient(S, 10.0, 10.0, shots, rx, rz, pg)
    assert used >= 1
    assert np.array_equal(pk, pk2, equal_nan=True)
    assert np.array_equal(g, g2)
    r = pg.astype(np.float64)
    assert J == pytest.approx(0.5 * np.nansum(r * r), rel=1e-13)


def test_smoothing_kernel_and_update(oracle):
    """Restated model_smoothing / smooth_matrix (inversion.cpp:347-447): the
    normalised kernel sums to 1 and is symmetric, a unit impulse spreads into
    the kernel, stdv 0 is the identity, and the update without smoothing is
    S += scale * grad on the interior only."""
    k = oracle.smooth_kernel(5.0, 11)
    assert abs(float(k.sum(dtype=np.float64)) - 1.0) < 1e-5
    assert np.array_equal(k, k.T) and np.array_equal(k, k[::-1, ::-1])
    m = np.zeros((30, 20), np.float32)
    m[12, 9] = 1.0
    s = oracle.model_smoothing(m, 5.0, 11)
    assert np.array_equal(s[7:18, 4:15], k)
    r = np.random.default_rng(1).standard_normal((17, 13)).astype(np.float32)
    assert np.array_equal(oracle.model_smoothing(r, 0.0, 7), r)
    nx, nz, nb = 12, 9, 3
    S = np.random.default_rng(2).uniform(2e-4, 6e-4, (nx + 2 * nb, nz + 2 * nb)).astype(np.float32)
    g = np.random.default_rng(3).standard_normal(S.shape).astype(np.float32)
    Sn, dS = oracle.update_slowness(S, g, nx, nz, -1e-5)
    inner = (slice(nb, nb + nx), slice(nb, nb + nz))
    assert np.array_equal(dS, (np.float32(-1e-5) * g[inner]).astype(np.float32))
    assert np.array_equal(Sn[inner], (S[inner] + dS).astype(np.float32))
    Sn[inner] = S[inner]
    assert np.array_equal(Sn, S)  # the pad ring keeps its values


def test_kirchhoff_correlation_matches_fft_form(oracle):
    """The direct FP64 cross-correlation restates Migration::adjoint_convolution
    (migration.cu:173-228): zero-padded FFT, product A conj(B), unnormalised
    inverse (FFTW), shift nw/2 + nw/10."""
    dt, fmax, nt = 0.002, 25.0, 300
    w = oracle.kirchhoff_wavelet(fmax, dt)
    nw = len(w)
    assert nw > 4 and nw % 2 == 0
    tr = np.random.default_rng(5).standard_normal((3, nt)).astype(np.float32)
    got = oracle.adjoint_convolution(tr, dt, fmax)
    nfft = 1
    while nfft < nt + nw - 1:
        nfft *= 2
    W = np.fft.rfft(np.concatenate([w.astype(np.float64), np.zeros(nfft - nw)]))
    shift = nw // 2 + nw // 10
    for q in range(3):
        A = np.fft.rfft(np.concatenate([tr[q].astype(np.float64), np.zeros(nfft - nt)]))
        c = np.fft.irfft(A * np.conj(W), nfft) * nfft
        ref = np.zeros(nt)
        ref[shift:] = c[:nt - shift]
        assert np.allclose(got[q], ref.astype(np.float32), rtol=1e-6, atol=1e-6 * np.abs(ref).max())


def test_kirchhoff_image_is_linear_in_the_traces(oracle):
    rng = np.random.default_rng(2)
    nx, nz, nb = 24, 16, 3
    S = oracle.expand_boundary((1.0 / rng.uniform(1800, 2500, (nx, nz))).astype(np.float32))
    xs = np.array([60.0, 150.0], np.float32)
    xr = np.array([30.0, 90.0, 170.0], np.float32)
    Ts = np.stack([oracle.solve_f32(S, 10.0, 10.0, float(x), 0.0) for x in xs])
    Tr = np.stack([oracle.solve_f32(S, 10.0, 10.0, float(x), 0.0) for x in xr])
    d = rng.standard_normal((2, 3, 200)).astype(np.float32)
    a = oracle.kirchhoff_image(S, Ts, Tr, xs, xr, d, 0.001, 10.0, 10.0, 30.0, 1000.0)
    b = oracle.kirchhoff_image(S, Ts, Tr, xs, xr, 2 * d, 0.001, 10.0, 10.0, 30.0, 1000.0)
    assert np.isfinite(a).all() and np.abs(a).max() > 0
    assert np.array_equal(b, 2 * a)
    c = oracle.kirchhoff_image(S, Ts, Tr, xs, xr, d, 0.001, 10.0, 10.0, 30.0, 50.0)  # offset cut
    assert not np.array_equal(a, c)


def test_kirchhoff_forward_convolution_matches_fft_form(oracle):
    """The direct FP64 convolution restates Migration::forward_convolution
    (migration.cu:230-261): zero-padded FFT, product A B, unnormalised
    inverse, output sample t read at t + nw/2 + nw/10."""
    dt, fmax, nt = 0.002, 25.0, 300
    w = oracle.kirchhoff_wavelet(fmax, dt)
    nw = len(w)
    tr = np.random.default_rng(6).standard_normal((3, nt)).astype(np.float32)
    got = oracle.forward_convolution(tr, dt, fmax)
    nfft = 1
    while nfft < nt + nw - 1:
        nfft *= 2
    W = np.fft.rfft(np.concatenate([w.astype(np.float64), np.zeros(nfft - nw)]))
    shift = nw // 2 + nw // 10
    for q in range(3):
        A = np.fft.rfft(np.concatenate([tr[q].astype(np.float64), np.zeros(nfft - nt)]))
        c = np.fft.irfft(A * W, nfft) * nfft
        ref = c[shift:shift + nt]
        assert np.allclose(got[q], ref.astype(np.float32), rtol=1e-6, atol=1e-6 * np.abs(ref).max())


def _kirchhoff_case(oracle, seed=2, nx=24, nz=16):
    rng = np.random.default_rng(seed)
    S = oracle.expand_boundary((1.0 / rng.uniform(1800, 2500, (nx, nz))).astype(np.float32))
    xs = np.array([60.0, 150.0], np.float32)
    xr = np.array([30.0, 90.0, 170.0], np.float32)
    Ts = np.stack([oracle.solve_f32(S, 10.0, 10.0, float(x), 0.0) for x in xs])
    Tr = np.stack([oracle.solve_f32(S, 10.0, 10.0, float(x), 0.0) for x in xr])
    return rng, S, xs, xr, Ts, Tr


def test_kirchhoff_forward_is_the_adjoint_of_the_image(oracle):
    """<F m, d> = <m, F^T d> for the image-domain forward operator (the
    least-squares variant's demigration, migration.cu:485-570) and the
    migration kernel (:398-483): the same weights and samples."""
    rng, S, xs, xr, Ts, Tr = _kirchhoff_case(oracle)
    nt, dt = 200, 0.001
    m = rng.standard_normal((S.shape[0] - 6, S.shape[1] - 6)).astype(np.float32)
    d = rng.standard_normal((2, 3, nt)).astype(np.float32)
    Fm = oracle.kirchhoff_image_forward(S, Ts, Tr, xs, xr, m, nt, dt, 10.0, 10.0, 30.0, 1000.0)
    Ftd = oracle.kirchhoff_image(S, Ts, Tr, xs, xr, d, dt, 10.0, 10.0, 30.0, 1000.0)
    lhs = float(np.dot(Fm.ravel().astype(np.float64), d.ravel()))
    rhs = float(np.dot(m.ravel().astype(np.float64), Ftd.ravel()))
    assert abs(Fm).max() > 0
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs))
    # traces beyond max_offset stay zero
    cut = oracle.kirchhoff_image_forward(S, Ts, Tr, xs, xr, m, nt, dt, 10.0, 10.0, 30.0, 50.0)
    far = np.abs(xs[:, None] - xr[None, :]) >= 50.0
    assert not cut[far].any() and cut[~far].any()


def test_kirchhoff_angle_forward_bins(oracle):
    """Angle-domain forward operator: a gather that is one in a single
    (CMP, angle) bin and zero elsewhere feeds only the traces of that CMP;
    the sum over all bins equals the image-domain operator on an image of
    ones (every cell lands in exactly one angle bin below max_angle)."""
    rng, S, xs, xr, Ts, Tr = _kirchhoff_case(oracle, seed=4)
    nt, dt = 200, 0.001
    na, nc, mn, dcmp = oracle.angle_bins(xs, xr, 90.0, 2.0)
    nz = S.shape[1] - 6
    ones = np.ones((nc, na, nz), np.float32)
    a = oracle.kirchhoff_angle_forward(S, Ts, Tr, xs, xr, ones, nt, dt, 10.0, 10.0, 30.0, 1000.0, 90.0, 2.0)
    img = oracle.kirchhoff_image_forward(S, Ts, Tr, xs, xr, np.ones((S.shape[0] - 6, nz), np.float32), nt, dt,
                                         10.0, 10.0, 30.0, 1000.0)
    assert np.abs(a).max() > 0
    assert np.allclose(a, img, rtol=1e-5, atol=1e-6 * np.abs(img).max())
    one = np.zeros_like(ones)
    one[1, 3, :] = 1.0
    b = oracle.kirchhoff_angle_forward(S, Ts, Tr, xs, xr, one, nt, dt, 10.0, 10.0, 30.0, 1000.0, 90.0, 2.0)
    cmp_bin = ((0.5 * (xs[:, None] + xr[None, :]) - mn) / dcmp).astype(int)
    assert not b[cmp_bin != 1].any()


def _vti_case(oracle, seed=8, nx=36, nz=22, dh=10.0, eps_max=0.2):
    from helpers import smooth_model
    from seisfat2d_gb300.synthetic import thomsen_stiffness
    rng = np.random.default_rng(seed)
    m = smooth_model(nx, nz, dh, seed=seed)
    vp = 1.0 / m.astype(np.float64)
    eps = rng.uniform(0.05, eps_max, (nx, nz))
    dlt = rng.uniform(-0.05, 0.1, (nx, nz))
    cij = thomsen_stiffness(vp, vp / np.sqrt(3.0), 1000.0, eps, dlt)
    codes, mm = [], []
    for c in cij:
        cd, mn, mx = oracle.compress(oracle.expand_boundary(c.astype(np.float32)))
        codes.append(cd)
        mm += [mn, mx]
    S = oracle.expand_boundary(m)
    shots = [(95.0, 0.0), (260.0, 0.0)]
    rx = np.arange(5.0, 355.0, 20.0).astype(np.float32)
    rz = np.zeros_like(rx)
    return rng, S, codes, np.array(mm, np.float32), shots, rx, rz


def test_vti_gradient_matches_finite_differences(oracle):
    """The anisotropic adjoint (second solve taped, each shot's gradient with
    respect to its qP slowness times dSq/dC11, dSq/dC13 with the first
    solve's directions held fixed) against central differences of the misfit
    along smooth perturbations of the C11 and C13 codes. The first solve sees
    S only, so for the stiffnesses the held directions are exact."""
    rng, S, codes, mm, shots, rx, rz = _vti_case(oracle)
    nxx, nzz = S.shape
    _, p0 = None, None
    t_obs = oracle.batch_misfit_gradient(S, 10.0, 10.0, shots, rx, rz, np.zeros((2, len(rx))),
                                         ani=(codes, mm))[2] * np.float32(1.01)
    J0, gS, _, _, g11, g13 = oracle.batch_misfit_gradient(S, 10.0, 10.0, shots, rx, rz, t_obs, ani=(codes, mm))
    assert J0 > 0 and np.abs(g11).max() > 0 and np.abs(g13).max() > 0
    xx, zz = np.meshgrid(np.arange(nxx), np.arange(nzz), indexing="ij")
    bump = np.exp(-((xx - 0.5 * nxx) ** 2 + (zz - 0.6 * nzz) ** 2) / (2 * 6.0 ** 2))
    for which, g in ((0, g11), (1, g13)):
        mn, mx = float(mm[2 * which]), float(mm[2 * which + 1])
        step = (np.float32(mx) - np.float32(mn)) / np.float32(65534)
        d = np.rint(400 * bump).astype(np.int64)
        base = codes[which].astype(np.int64)
        Js = []
        for sgn in (1, -1):
            cd = list(codes)
            cd[which] = np.clip(base + sgn * d, 1, 65535).astype(np.uint16)
            Js.append(oracle.batch_misfit_gradient(S, 10.0, 10.0, shots, rx, rz, t_obs, ani=(cd, mm))[0])
        dC = d * float(step)
        pred = float(np.sum(g.astype(np.float64) * dC))
        fd = (Js[0] - Js[1]) / 2.0
        print(f"C{'11' if which == 0 else '13'}: finite difference {fd:.6e}, adjoint {pred:.6e}")
        assert abs(fd - pred) <= 0.03 * abs(fd)


def test_vti_gradient_isotropic_limit(oracle):
    """With isotropic stiffness the qP pass returns S (to rounding), so the
    anisotropic gradient with respect to S equals the isotropic one to
    rounding."""
    from helpers import smooth_model
    from seisfat2d_gb300.synthetic import thomsen_stiffness
    m = smooth_model(30, 18, 10.0, seed=12)
    vp = 1.0 / m.astype(np.float64)
    cij = thomsen_stiffness(vp, vp / np.sqrt(3.0), 1000.0, np.zeros_like(vp), np.zeros_like(vp))
    codes, mm = [], []
    for c in cij:
        cd, mn, mx = oracle.compress(oracle.expand_boundary(c.astype(np.float32)))
        codes.append(cd)
        mm += [mn, mx]
    S = oracle.expand_boundary(m)
    shots = [(80.0, 0.0), (210.0, 0.0)]
    rx = np.arange(5.0, 295.0, 15.0).astype(np.float32)
    rz = np.zeros_like(rx)
    t_obs = np.full((2, len(rx)), 0.05, np.float32)
    Ji, gi, _, _ = oracle.batch_misfit_gradient(S, 10.0, 10.0, shots, rx, rz, t_obs)
    Ja, ga, _, _, g11, g13 = oracle.batch_misfit_gradient(S, 10.0, 10.0, shots, rx, rz, t_obs,
                                                          ani=(codes, np.array(mm, np.float32)))
    assert abs(Ja - Ji) <= 1e-4 * Ji
    # the pad copies the edge cells, so a tie between a pad cell and its
    # edge cell may go either way (the qP pass keeps S on the pad and rounds
    # inside): compare the gradients folded onto the model cells
    def fold(g, nb=3):
        nxx, nzz = g.shape
        out = np.zeros((nxx - 2 * nb, nzz - 2 * nb))
        xi = np.clip(np.arange(nxx) - nb, 0, nxx - 2 * nb - 1)
        zi = np.clip(np.arange(nzz) - nb, 0, nzz - 2 * nb - 1)
        np.add.at(out, (xi[:, None], zi[None, :]), g.astype(np.float64))
        return out
    fa, fi = fold(ga), fold(gi)
    assert np.abs(fa - fi).max() <= 2e-3 * np.abs(fi).max()


def test_vti_factors_fp32_vs_fp64(oracle):
    """The qP pass's derivative factors are computed in FP32 (each operation
    rounded once). On a solved VTI field they agree with the same formulas
    evaluated in FP64 from the same inputs to a few FP32 ulps."""
    from helpers import smooth_model
    from seisfat2d_gb300.synthetic import thomsen_stiffness
    rng = np.random.default_rng(21)
    m = smooth_model(48, 30, 10.0, seed=21)
    vp = 1.0 / m.astype(np.float64)
    cij = thomsen_stiffness(vp, vp / np.sqrt(3.0), 1000.0, rng.uniform(0.0, 0.25, vp.shape),
                            rng.uniform(-0.05, 0.15, vp.shape))
    codes, mm = [], []
    for c in cij:
        cd, mn, mx = oracle.compress(oracle.expand_boundary(c.astype(np.float32)))
        codes.append(cd)
        mm += [mn, mx]
    mm = np.array(mm, np.float32)
    S = oracle.expand_boundary(m)
    T = oracle.solve_f32(S, 10.0, 10.0, 230.0, 40.0)
    init, sIdx, sIdz = oracle.init_block_f32(S, 230.0, 40.0, 10.0, 10.0, 3)
    fS, f11, f13 = oracle.qp_factors(T, S, 10.0, 10.0, sIdz, sIdx, codes, mm)

    # FP64 restatement from the same FP32 inputs (decoded stiffness as the oracle decodes it)
    nb = 3
    ncols, nzz = T.shape
    dec = [(mm[2 * q] + (codes[q].astype(np.float32) - np.float32(1.0)) * (mm[2 * q + 1] - mm[2 * q])
            / np.float32(65534.0)).astype(np.float32).astype(np.float64) for q in range(6)]
    c11, c13, c15, c33, c35, c55 = dec
    Td = T.astype(np.float64)
    sl = (slice(nb, ncols - nb), slice(nb, nzz - nb))
    dTz = 0.5 * (Td[nb:ncols - nb, nb + 1:nzz - nb + 1] - Td[nb:ncols - nb, nb - 1:nzz - nb - 1]) / 10.0
    dTx = 0.5 * (Td[nb + 1:ncols - nb + 1, nb:nzz - nb] - Td[nb - 1:ncols - nb - 1, nb:nzz - nb]) / 10.0
    nrm = np.sqrt(dTx * dTx + dTz * dTz)
    px, pz = dTx / nrm, dTz / nrm
    c11, c13, c15, c33, c35, c55 = (c[sl] for c in (c11, c13, c15, c33, c35, c55))
    Gxx = c11 * px * px + c55 * pz * pz + 2.0 * c15 * px * pz
    Gzz = c55 * px * px + c33 * pz * pz + 2.0 * c35 * px * pz
    Gxz = c15 * px * px + c35 * pz * pz + (c13 + c55) * px * pz
    h = 0.5 * (Gxx - Gzz)
    r = np.sqrt(h * h + Gxz * Gxz)
    lam = 0.5 * (Gxx + Gzz) + r
    vx = np.where(h >= 0.0, h + r, Gxz)
    vz = np.where(h >= 0.0, Gxz, r - h)
    nv = np.sqrt(vx * vx + vz * vz)
    vx, vz = vx / nv, vz / nv
    fs = np.sqrt(c33 / lam)
    sq = S.astype(np.float64)[sl] * fs
    e11 = -0.5 * sq * px * px * vx * vx / lam
    e13 = -sq * px * pz * vx * vz / lam
    keep = np.ones(fs.shape, bool)
    keep[sIdx - nb, sIdz - nb] = False  # the source node keeps (1, 0, 0)
    for got, want in ((fS, fs), (f11, e11), (f13, e13)):
        g = got[sl].astype(np.float64)[keep]
        w = want[keep]
        err = np.abs(g - w).max() / np.abs(w).max()
        print(f"max |FP32 - FP64| / max |FP64| = {err:.2e}")
        assert err <= 2e-6


@pytest.mark.parametrize("stdv,samples", [(5.0, 11), (2.0, 5), (3.0, 3), (0.0, 7), (1.5, 1), (4.0, 15)])
def test_smoothing_matches_reference_code(oracle, stdv, samples):
    """The oracle's model_smoothing restatement equals the reference's own
    Inversion::model_smoothing / smooth_matrix (src/inversion/inversion.cpp:
    347-447, compiled from the reference source by oracle/build_ref.py) bit
    for bit. Skipped where the reference sources are absent."""
    import ctypes as C
    from oracle import build_ref
    lib = build_ref.build_inversion_host()
    if lib is None:
        pytest.skip("reference sources not present")
    L = C.CDLL(lib)
    L.ref_model_smoothing.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float]
    rng = np.random.default_rng(samples)
    for nx, nz in ((37, 23), (64, 9)):
        m = rng.standard_normal((nx, nz)).astype(np.float32) * np.float32(1e-5)
        ref = np.ascontiguousarray(m.copy())
        L.ref_model_smoothing(ref.ctypes.data, nx, nz, samples, stdv)
        ours = oracle.model_smoothing(m, stdv, samples)
        assert np.array_equal(ours, ref), np.abs(ours - ref).max()
        assert np.array_equal(ref, m) == (stdv == 0.0 or samples == 1)


def _ref_modeling_host():
    import ctypes as C
    from oracle import build_ref
    lib = build_ref.build_modeling_host()
    if lib is None:
        pytest.skip("reference sources not present")
    L = C.CDLL(lib)
    L.ref_expand_boundary.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int]
    L.ref_compression.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    return L


@pytest.mark.parametrize("nx,nz", [(40, 20), (17, 33), (1, 5)])
def test_padding_matches_reference_code(oracle, nx, nz):
    """The oracle's expand_boundary (the padding behind every golden vector and
    the engine's sf_set_slowness) equals the reference's own
    Modeling::expand_boundary (src/modeling/modeling.cu:204-232, compiled from
    the reference sources) bit for bit."""
    L = _ref_modeling_host()
    nb = 3
    m = np.random.default_rng(nx * nz).uniform(2e-4, 7e-4, (nx, nz)).astype(np.float32)
    ref = np.zeros((nx + 2 * nb, nz + 2 * nb), np.float32)
    L.ref_expand_boundary(np.ascontiguousarray(m).ctypes.data, ref.ctypes.data, nx, nz, nb)
    assert np.array_equal(oracle.expand_boundary(m), ref)


def test_quantisation_matches_reference_code(oracle):
    """The oracle's Cij quantisation equals the reference's own
    Modeling::compression (modeling.cu:264-279, compiled single-threaded)
    for varying fields: same range and same codes. A constant field makes the
    reference divide 0 by 0; both decode to the constant, so only the range is
    compared there."""
    import ctypes as C
    from seisfat2d_gb300.synthetic import thomsen_stiffness
    L = _ref_modeling_host()
    rng = np.random.default_rng(7)
    vp = rng.uniform(1500.0, 4500.0, (50, 30))
    cij = thomsen_stiffness(vp, vp / np.sqrt(3.0), 1000.0, rng.uniform(0.0, 0.25, vp.shape),
                            rng.uniform(-0.05, 0.15, vp.shape), tilt_deg=20.0)
    cij.append(np.full(vp.shape, 3.5e9))
    for k, c in enumerate(cij):
        f = oracle.expand_boundary(c.astype(np.float32))
        codes, mn, mx = oracle.compress(f)
        ref = np.zeros(f.size, np.uint16)
        rmx, rmn = C.c_float(), C.c_float()
        L.ref_compression(np.ascontiguousarray(f).ctypes.data, ref.ctypes.data, f.size, C.byref(rmx),
                          C.byref(rmn))
        assert (mn, mx) == (rmn.value, rmx.value)
        if mx > mn:
            assert np.array_equal(codes.ravel(), ref), k


def test_picks_match_reference_code(oracle):
    """The oracle's picks (receiver stencil + Catmull-Rom rule) equal the
    reference's own compute_seismogram host loop and cubic2d
    (modeling.cu:161-194, admin.cpp:121-133, compiled from the reference
    sources) bit for bit, for receivers whose 4x4 stencil lies inside the
    field (the reference reads outside it otherwise; the oracle and the engine
    return NaN there). Runs without a GPU only: the reference's copy of the
    device field must fail to leave the given field in place."""
    import ctypes as C
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("needs a machine without a GPU")
    L = _ref_modeling_host()
    L.ref_compute_seismogram.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_void_p,
                                         C.c_void_p, C.c_int, C.c_void_p]
    nx, nz, nb = 60, 30, 3
    for dx, dz in ((10.0, 10.0), (12.5, 7.5)):
        S = oracle.expand_boundary(np.full((nx, nz), 1.0 / 2000.0, np.float32))
        T = oracle.solve_f32(S, dx, dz, 0.37 * nx * dx, 0.2 * nz * dz)
        rng = np.random.default_rng(int(dx * 10))
        rx = rng.uniform(0.0, (nx - 1) * dx, 300).astype(np.float32)
        rz = rng.uniform(0.0, (nz - 1) * dz, 300).astype(np.float32)
        ours = oracle.picks(T, dx, dz, rx, rz)
        ref = np.zeros(300, np.float32)
        Tc = np.ascontiguousarray(T.copy())
        L.ref_compute_seismogram(Tc.ctypes.data, nx, nz, nb, dx, dz, rx.ctypes.data, rz.ctypes.data, 300,
                                 ref.ctypes.data)
        ok = ~np.isnan(ours)
        assert ok.sum() > 200
        assert np.array_equal(Tc, T)
        assert np.array_equal(ours[ok], ref[ok])


@pytest.mark.parametrize("fmax,dt", [(25.0, 2e-3), (30.0, 1e-3), (12.5, 4e-3), (45.0, 5e-4)])
def test_wavelet_matches_reference_code(oracle, fmax, dt):
    """The oracle's Ricker wavelet equals the reference's own
    Migration::set_wavelet (src/migration/migration.cu:54-71, compiled from the
    reference sources) bit for bit: length and samples."""
    import ctypes as C
    from oracle import build_ref
    lib = build_ref.build_migration_host()
    if lib is None:
        pytest.skip("reference sources not present")
    L = C.CDLL(lib)
    L.ref_set_wavelet.argtypes = [C.c_float, C.c_float, C.c_void_p, C.c_int]
    L.ref_set_wavelet.restype = C.c_int
    ref = np.zeros(4096, np.float32)
    nw = L.ref_set_wavelet(fmax, dt, ref.ctypes.data, ref.size)
    ours = oracle.kirchhoff_wavelet(fmax, dt)
    assert nw > 0 and len(ours) == nw
    assert np.array_equal(ours, ref[:nw])
