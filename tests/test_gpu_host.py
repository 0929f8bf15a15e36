"""The C++ drop-in (Modeling/Eikonal_ISO/Eikonal_ANI/Geometry/admin and
Tomography_ISO) driven by parameters.txt, end to end on the GPU: the output
files of modeling.exe, traveltime_tables.exe and inversion.exe."""
import os
import subprocess

import numpy as np
import pytest

from helpers import smooth_model, write_case

pytestmark = pytest.mark.gpu


def run(exe, p):
    r = subprocess.run([exe, p], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


@pytest.mark.parametrize("batch", [False, True])
def test_modeling_exe_matches_oracle(oracle, cuda, exes, tmp_path, batch):
    nx, nz, dx, dz = 80, 40, 10.0, 10.0
    m = smooth_model(nx, nz, dx, seed=17, noise=0.02)
    shots = [(100.0, 0.0), (400.0, 50.0), (700.0, 10.0)]
    recs = [(float(x), 20.0) for x in range(0, 790, 15)]
    p = write_case(str(tmp_path), nx, nz, dx, dz, m, shots, recs, batch=batch)
    run(exes["modeling.exe"], p)
    oracle.set_arith("reference")
    try:
        S = oracle.expand_boundary(m)
        rx = np.array([r[0] for r in recs], np.float32)
        rz = np.array([r[1] for r in recs], np.float32)
        for k, (sx, sz) in enumerate(shots):
            out = np.fromfile(os.path.join(str(tmp_path), f"out_eikonal_iso_nStations{len(recs)}_shot_{k + 1}.bin"),
                              np.float32)
            _, po = oracle.shot(S, dx, dz, sx, sz, rx, rz)
            assert np.array_equal(out, po, equal_nan=True)
    finally:
        oracle.set_arith("ieee")


def test_modeling_exe_compensated_arithmetic(oracle, cuda, exes, tmp_path):
    """parameters.txt `eikonal_arithmetic = compensated`: the driver's picks
    equal the oracle's compensated restatement bit for bit."""
    nx, nz, dx, dz = 90, 50, 10.0, 10.0
    m = smooth_model(nx, nz, dx, seed=19, noise=0.02)
    shots = [(150.0, 0.0), (620.0, 35.0)]
    recs = [(float(x), 10.0) for x in range(0, 890, 20)]
    p = write_case(str(tmp_path), nx, nz, dx, dz, m, shots, recs, batch=True)
    with open(p, "a") as f:
        f.write("eikonal_arithmetic = compensated\n")
    run(exes["modeling.exe"], p)
    oracle.set_arith("compensated")
    try:
        S = oracle.expand_boundary(m)
        rx = np.array([r[0] for r in recs], np.float32)
        rz = np.array([r[1] for r in recs], np.float32)
        for k, (sx, sz) in enumerate(shots):
            out = np.fromfile(os.path.join(str(tmp_path), f"out_eikonal_iso_nStations{len(recs)}_shot_{k + 1}.bin"),
                              np.float32)
            _, po = oracle.shot(S, dx, dz, sx, sz, rx, rz)
            assert np.array_equal(out, po, equal_nan=True)
    finally:
        oracle.set_arith("ieee")


def test_modeling_exe_anisotropic(oracle, cuda, exes, tmp_path):
    from seisfat2d_gb300.synthetic import thomsen_stiffness
    nx, nz, dx, dz = 60, 30, 10.0, 10.0
    rng = np.random.default_rng(3)
    m = smooth_model(nx, nz, dx, seed=23)
    vp = 1.0 / m.astype(np.float64)
    cij = thomsen_stiffness(vp, vp / np.sqrt(3.0), 1000.0, rng.uniform(0, .2, (nx, nz)),
                            rng.uniform(-.05, .1, (nx, nz)), 10.0)
    for name, c in zip(["C11", "C13", "C15", "C33", "C35", "C55"], cij):
        c.astype(np.float32).tofile(os.path.join(str(tmp_path), f"model_{name}.bin"))
    shots = [(300.0, 0.0)]
    recs = [(float(x), 0.0) for x in range(0, 590, 10)]
    p = write_case(str(tmp_path), nx, nz, dx, dz, m, shots, recs, mtype=1)
    run(exes["modeling.exe"], p)
    oracle.set_arith("reference")
    try:
        codes, mm = [], []
        for c in cij:
            cd, mn, mx = oracle.compress(oracle.expand_boundary(c.astype(np.float32)))
            codes.append(cd)
            mm += [mn, mx]
        _, po = oracle.shot(oracle.expand_boundary(m), dx, dz, 300.0, 0.0,
                            np.array([r[0] for r in recs], np.float32), np.zeros(len(recs), np.float32),
                            ani=(codes, np.array(mm, np.float32)))
        out = np.fromfile(os.path.join(str(tmp_path), f"out_eikonal_ani_nStations{len(recs)}_shot_1.bin"), np.float32)
        assert np.array_equal(out, po, equal_nan=True)
    finally:
        oracle.set_arith("ieee")


def test_traveltime_tables_exe(oracle, cuda, exes, tmp_path):
    nx, nz, dx, dz = 50, 25, 10.0, 10.0
    m = smooth_model(nx, nz, dx, seed=29)
    shots = [(120.0, 0.0), (300.0, 0.0)]
    recs = [(40.0, 0.0), (450.0, 100.0)]
    p = write_case(str(tmp_path), nx, nz, dx, dz, m, shots, recs)
    run(exes["traveltime_tables.exe"], p)
    oracle.set_arith("reference")
    try:
        S = oracle.expand_boundary(m)
        for kind, pts in (("src", shots), ("rec", recs)):
            for k, (x, z) in enumerate(pts):
                T = np.fromfile(os.path.join(str(tmp_path), f"tab_eikonal_{kind}_{k + 1}.bin"), np.float32)
                assert np.array_equal(T.reshape(S.shape), oracle.solve_f32(S, dx, dz, x, z))
    finally:
        oracle.set_arith("ieee")


def test_inversion_exe_reduces_residual(oracle, cuda, exes, tmp_path):
    from seisfat2d_gb300.synthetic import gaussian_smooth
    nx, nz, dx, dz = 80, 30, 10.0, 10.0
    true = smooth_model(nx, nz, dx, seed=31, noise=0.0)
    start = (1.0 / gaussian_smooth(1.0 / true.astype(np.float64), 6.0)).astype(np.float32)
    shots = [(float(x), 0.0) for x in range(50, 790, 100)]
    recs = [(float(x), 0.0) for x in range(0, 790, 20)]
    d = str(tmp_path)
    p = write_case(d, nx, nz, dx, dz, start, shots, recs)
    oracle.set_arith("reference")
    try:
        St = oracle.expand_boundary(true)
        rx = np.array([r[0] for r in recs], np.float32)
        for k, (sx, sz) in enumerate(shots):
            _, po = oracle.shot(St, dx, dz, sx, sz, rx, np.zeros(len(recs), np.float32))
            po.astype(np.float32).tofile(os.path.join(d, f"obs_shot_{k + 1}.bin"))
    finally:
        oracle.set_arith("ieee")
    out = run(exes["inversion.exe"], p)
    res = np.loadtxt(os.path.join(d, "tomography_iso_convergence_3_iterations.txt"))
    print("residuo per iteration:", res)
    assert len(res) == 4 and res[-1] < res[0]
    vp = np.fromfile(os.path.join(d, f"tomography_iso_final_model_vp_{nz}x{nx}.bin"), np.float32)
    assert np.isfinite(vp).all() and vp.size == nx * nz


@pytest.mark.parametrize("migtype", [0, 1])
def test_migration_exe_matches_engine(cuda, exes, tmp_path, migtype):
    """migration.exe (image-domain or angle-domain Kirchhoff) writes what the
    engine's batched tables, correlation and imaging give through the Python
    mirror."""
    from seisfat2d_gb300 import Engine
    nx, nz, dx, dz = 60, 25, 10.0, 10.0
    m = smooth_model(nx, nz, dx, seed=21)
    shots = [(100.0, 0.0), (300.0, 0.0), (480.0, 0.0)]
    recs = [(float(x), 0.0) for x in range(0, 590, 40)]
    d = str(tmp_path)
    p = write_case(d, nx, nz, dx, dz, m, shots, recs, migtype=migtype)
    rng = np.random.default_rng(4)
    data = rng.standard_normal((len(shots), len(recs), 400)).astype(np.float32)
    for k in range(len(shots)):
        data[k].tofile(os.path.join(d, f"mig_shot_{k + 1}.bin"))  # nt x nrec, trace-major
    run(exes["migration.exe"], p)
    e = Engine(nx, nz, dx, dz)
    e.set_slowness(m)
    dev = cuda.device("cuda", 0)
    tabs = []
    for pts in (shots, recs):
        e.batch_forward(pts, np.zeros(0, np.float32), np.zeros(0, np.float32), keep_tables=True)
        t = cuda.empty((len(pts), e.nxx, e.nzz), dtype=cuda.float32, device=dev)
        for k in range(len(pts)):
            e.batch_table(k, e.nxx, out=t[k])
        tabs.append(t)
    corr = e.adjoint_convolution(data.reshape(-1, 400), 2e-3, 25.0).reshape(data.shape)
    xs, xr = [s[0] for s in shots], [r[0] for r in recs]
    if migtype == 0:
        img = np.fromfile(os.path.join(d, f"IDKDM_result_{nz}x{nx}.bin"), np.float32).reshape(nx, nz)
        ref = e.kirchhoff_image(tabs[0], tabs[1], xs, xr, corr, 2e-3, 35.0, 600.0)
    else:
        ref = e.kirchhoff_angle_gathers(tabs[0], tabs[1], xs, xr, corr, 2e-3, 35.0, 600.0, 60.0, 2.0)
        nc, na, _ = ref.shape
        img = np.fromfile(os.path.join(d, f"ADKDM_result_{nz}x{nc}x{na}.bin"), np.float32).reshape(ref.shape)
    assert np.abs(ref).max() > 0
    assert np.array_equal(img, ref)


def _seq_sum(acc, x):
    """FP32 running sum in index order, as the reference's host loops add."""
    return np.cumsum(np.concatenate([[np.float32(acc)], np.ravel(x).astype(np.float32)]), dtype=np.float32)[-1]


def least_squares_mirror(e, Ts, Tr, xs, xr, dobs, dt, fmax, aperture, max_off, max_it, angle=False, max_ang=0.0,
                         da=1.0, smooth=0.0):
    """LSKDM (LSKDM.cu:3-235) step by step on the engine's operators: FP32
    host vectors, sums in the reference's order."""
    f32 = np.float32
    EPS = f32(1e-6)
    ns, nr, nt = dobs.shape
    inside = np.abs(xs[:, None] - xr[None, :]) < max_off

    def F(model):
        if angle:
            tr = e.kirchhoff_angle_forward(Ts, Tr, xs, xr, model, nt, dt, aperture, max_off, max_ang, da)
        else:
            tr = e.kirchhoff_image_forward(Ts, Tr, xs, xr, model, nt, dt, aperture, max_off)
        return e.forward_convolution(tr.reshape(-1, nt), dt, fmax).reshape(tr.shape)

    def Ft(res):
        c = e.adjoint_convolution(res.reshape(-1, nt), dt, fmax).reshape(res.shape)
        if angle:
            return e.kirchhoff_angle_gathers(Ts, Tr, xs, xr, c, dt, aperture, max_off, max_ang, da)
        return e.kirchhoff_image(Ts, Tr, xs, xr, c, dt, aperture, max_off)

    shape = Ft(np.zeros_like(dobs)).shape
    model = np.zeros(shape, f32)
    direction = np.zeros(shape, f32)
    gold = np.zeros(shape, f32)
    residuo, it = [], 0
    while True:
        pred = F(model)
        res = np.where(np.abs(dobs) > EPS, dobs - pred, f32(0)).astype(f32)
        res[~inside] = 0
        acc = f32(0)
        for s in range(ns):
            for r in range(nr):
                if inside[s, r]:
                    acc = _seq_sum(acc, res[s, r] * res[s, r])
        g = Ft(res)
        it += 1
        residuo.append(np.sqrt(acc))
        if it > max_it:
            break
        beta = f32(_seq_sum(0, g * g) / f32(_seq_sum(0, gold * gold) + EPS))
        direction = (g + beta * direction).astype(f32)
        alpha_num = _seq_sum(0, g * direction)
        gold = g.copy()
        Fd = F(direction)
        aden = f32(0)
        for s in range(ns):
            for r in range(nr):
                if inside[s, r]:
                    aden = _seq_sum(aden, Fd[s, r] * Fd[s, r])
        alpha = f32(alpha_num / f32(aden + EPS))
        if angle:
            na = shape[1]
            fw = np.concatenate([model[:, 1:], model[:, -2:-1]], axis=1)
            bw = np.concatenate([model[:, 1:2], model[:, :-1]], axis=1)
            lap = ((fw - f32(2) * model) + bw).astype(f32)
            direction = (direction + (f32(smooth) * lap) / f32(f32(da) * f32(da))).astype(f32)
        model = (model + alpha * direction).astype(f32)
    return model, np.array(residuo, np.float32)


@pytest.mark.parametrize("migtype", [2, 3])
def test_migration_exe_least_squares(cuda, exes, tmp_path, migtype):
    """migration.exe with mig_type 2 (IDLSKDM) / 3 (ADLSKDM) writes what the
    reference's least-squares loop gives on the engine's operators, and the
    residual norm falls."""
    from seisfat2d_gb300 import Engine
    nx, nz, dx, dz = 60, 25, 10.0, 10.0
    m = smooth_model(nx, nz, dx, seed=21)
    shots = [(100.0, 0.0), (300.0, 0.0), (480.0, 0.0)]
    recs = [(float(x), 0.0) for x in range(0, 590, 40)]
    d = str(tmp_path)
    p = write_case(d, nx, nz, dx, dz, m, shots, recs, migtype=migtype)
    e = Engine(nx, nz, dx, dz)
    e.set_slowness(m)
    dev = cuda.device("cuda", 0)
    tabs = []
    for pts in (shots, recs):
        e.batch_forward(pts, np.zeros(0, np.float32), np.zeros(0, np.float32), keep_tables=True)
        t = cuda.empty((len(pts), e.nxx, e.nzz), dtype=cuda.float32, device=dev)
        for k in range(len(pts)):
            e.batch_table(k, e.nxx, out=t[k])
        tabs.append(t)
    xs = np.array([s[0] for s in shots], np.float32)
    xr = np.array([r[0] for r in recs], np.float32)
    # observed traces: a two-reflector image through the forward operator
    refl = np.zeros((nx, nz), np.float32)
    refl[:, 10] = 1.0
    refl[:, 18] = -0.5
    raw = e.kirchhoff_image_forward(tabs[0], tabs[1], xs, xr, refl, 400, 2e-3, 35.0, 600.0)
    dobs = e.forward_convolution(raw.reshape(-1, 400), 2e-3, 25.0).reshape(raw.shape)
    for k in range(len(shots)):
        dobs[k].tofile(os.path.join(d, f"mig_shot_{k + 1}.bin"))
    run(exes["migration.exe"], p)
    angle = migtype == 3
    model, res = least_squares_mirror(e, tabs[0], tabs[1], xs, xr, dobs, 2e-3, 25.0, 35.0, 600.0, 3, angle=angle,
                                      max_ang=60.0, da=2.0, smooth=0.5)
    name = "ADLSKDM" if angle else "IDLSKDM"
    dims = f"{nz}x{model.shape[0]}x{model.shape[1]}" if angle else f"{nz}x{nx}"
    out = np.fromfile(os.path.join(d, f"{name}_result_{dims}_iteration_3.bin"), np.float32).reshape(model.shape)
    conv = np.loadtxt(os.path.join(d, f"{name}_convergence_3_iterations.txt"))
    print(name, "residual norms", conv)
    assert len(conv) == 4 and conv[-1] < conv[0]
    assert np.allclose(conv, res, rtol=1e-5)
    assert np.abs(model).max() > 0
    assert np.array_equal(out, model)


def _vti_files(oracle, d, nx, nz, m, eps, dlt):
    from seisfat2d_gb300.synthetic import thomsen_stiffness
    vp = 1.0 / m.astype(np.float64)
    cij = thomsen_stiffness(vp, vp / np.sqrt(3.0), 1000.0, eps, dlt)
    for name, c in zip(["C11", "C13", "C15", "C33", "C35", "C55"], cij):
        c.astype(np.float32).tofile(os.path.join(d, f"model_{name}.bin"))
    codes, mm = [], []
    for c in cij:
        cd, mn, mx = oracle.compress(oracle.expand_boundary(c.astype(np.float32)))
        codes.append(cd)
        mm += [mn, mx]
    return codes, np.array(mm, np.float32)


def test_inversion_exe_vti_stiffness_round_trip(oracle, cuda, exes, tmp_path):
    """inv_type 1 with no iteration: the exported epsilon and delta are the
    Thomsen parameters the stiffness files were built from (get_stiffness_VTI)."""
    nx, nz = 40, 20
    rng = np.random.default_rng(2)
    m = smooth_model(nx, nz, 10.0, seed=3)
    eps = rng.uniform(0.0, 0.25, (nx, nz))
    dlt = rng.uniform(-0.05, 0.15, (nx, nz))
    d = str(tmp_path)
    _vti_files(oracle, d, nx, nz, m, eps, dlt)
    shots = [(100.0, 0.0)]
    recs = [(float(x), 0.0) for x in range(0, 390, 30)]
    p = write_case(d, nx, nz, 10.0, 10.0, m, shots, recs, aniso=True, invtype=1, maxit=0)
    np.zeros(len(recs), np.float32).tofile(os.path.join(d, "obs_shot_1.bin"))
    run(exes["inversion.exe"], p)
    ep = np.fromfile(os.path.join(d, f"tomography_vti_final_model_ep_{nz}x{nx}.bin"), np.float32).reshape(nx, nz)
    dl = np.fromfile(os.path.join(d, f"tomography_vti_final_model_dl_{nz}x{nx}.bin"), np.float32).reshape(nx, nz)
    assert np.allclose(ep, eps, atol=1e-5) and np.allclose(dl, dlt, atol=1e-4)


def test_inversion_exe_vti_reduces_residual(oracle, cuda, exes, tmp_path):
    """Anisotropic tomography (inv_type 1): observed picks from the oracle's
    two-pass solve in the true (S, epsilon, delta); the start model has a
    smoothed S and epsilon, delta off by a constant. The residual falls and the
    three models are written."""
    from seisfat2d_gb300.synthetic import gaussian_smooth
    nx, nz = 70, 30
    true = smooth_model(nx, nz, 10.0, seed=31, noise=0.0)
    eps_t = np.full((nx, nz), 0.12)
    dlt_t = np.full((nx, nz), 0.05)
    d = str(tmp_path)
    codes, mm = _vti_files(oracle, d, nx, nz, true, eps_t, dlt_t)
    shots = [(float(x), 0.0) for x in range(50, 690, 80)]
    recs = [(float(x), 0.0) for x in range(0, 690, 15)]
    St = oracle.expand_boundary(true)
    rx = np.array([r[0] for r in recs], np.float32)
    for k, (sx, sz) in enumerate(shots):
        _, po = oracle.shot(St, 10.0, 10.0, sx, sz, rx, np.zeros(len(recs), np.float32), ani=(codes, mm))
        po.astype(np.float32).tofile(os.path.join(d, f"obs_shot_{k + 1}.bin"))
    start = (1.0 / gaussian_smooth(1.0 / true.astype(np.float64), 4.0)).astype(np.float32)
    _vti_files(oracle, d, nx, nz, start, eps_t - 0.08, dlt_t + 0.04)
    p = write_case(d, nx, nz, 10.0, 10.0, start, shots, recs, aniso=True, invtype=1, maxit=3)
    run(exes["inversion.exe"], p)
    res = np.loadtxt(os.path.join(d, "tomography_vti_convergence_3_iterations.txt"))
    print("VTI residuo per iteration:", res)
    assert len(res) == 4 and res[-1] < 0.9 * res[0]
    ep = np.fromfile(os.path.join(d, f"tomography_vti_final_model_ep_{nz}x{nx}.bin"), np.float32)
    dl = np.fromfile(os.path.join(d, f"tomography_vti_final_model_dl_{nz}x{nx}.bin"), np.float32)
    vp = np.fromfile(os.path.join(d, f"tomography_vti_final_model_vp_{nz}x{nx}.bin"), np.float32)
    assert ep.size == dl.size == vp.size == nx * nz
    assert np.isfinite(ep).all() and np.isfinite(dl).all() and np.isfinite(vp).all()
    print("mean epsilon", ep.mean(), "mean delta", dl.mean())
