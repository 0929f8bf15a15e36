"""Pin the oracle and the engine to the reference's own kernels, run on the
GPU from cubins compiled from the reference sources (oracle/build_ref.py).

In reference arithmetic (the engine's default) the engine reproduces the
reference's traveltimes bit for bit; in IEEE arithmetic (every operation
rounded once, FP64 initialisation) the maximum relative difference is printed
and bounded.
"""
import numpy as np
import pytest

from helpers import rel_err, smooth_model

pytestmark = pytest.mark.gpu


def _ref():
    from oracle import refkernels
    if not refkernels.available():
        pytest.skip("reference cubins not built on this machine")
    return refkernels


@pytest.mark.parametrize("nx,nz,sx,sz,noise", [(40, 20, 0.0, 0.0, 0.02), (20, 40, 93.0, 211.0, 0.05),
                                               (120, 50, 555.0, 0.0, 0.0), (300, 252, 1000.0, 500.0, 0.02),
                                               (251, 61, 1234.0, 17.0, 0.08), (90, 90, 450.0, 300.0, 0.1)])
def test_engine_matches_reference_kernels_bitwise(oracle, engine_lib, cuda, nx, nz, sx, sz, noise):
    ref = _ref()
    from seisfat2d_gb300 import Engine
    m = smooth_model(nx, nz, 10.0, seed=nx + nz, noise=noise)
    S = oracle.expand_boundary(m)
    Tr, ms = ref.solve(S, 10.0, 10.0, sx, sz)
    e = Engine(nx, nz, 10.0, 10.0)
    assert e.get_arithmetic() == "reference"
    e.set_slowness(m)
    T = e.time_propagation(sx, sz)
    print(f"{nx}x{nz} noise {noise}: reference-arithmetic nodes equal to the reference kernels: "
          f"{np.mean(T == Tr):.6f}, max rel diff {rel_err(T, Tr).max():.2e}")
    assert np.array_equal(T, Tr)
    oracle.set_arith("reference")
    try:
        assert np.array_equal(oracle.solve_f32(S, 10.0, 10.0, sx, sz), Tr)
    finally:
        oracle.set_arith("ieee")
    e.set_arithmetic("ieee")
    Ti = e.time_propagation(sx, sz)
    print(f"   IEEE arithmetic: max rel diff {rel_err(Ti, Tr).max():.2e}, rms {np.sqrt(np.mean(rel_err(Ti, Tr)**2)):.2e}")


def test_anisotropic_matches_reference_kernels(oracle, engine_lib, cuda):
    ref = _ref()
    from seisfat2d_gb300 import Engine
    from seisfat2d_gb300.synthetic import thomsen_stiffness
    nx, nz = 60, 30
    rng = np.random.default_rng(5)
    m = smooth_model(nx, nz, 10.0, seed=9)
    vp = 1.0 / m.astype(np.float64)
    cij = [c.astype(np.float32) for c in thomsen_stiffness(vp, vp / np.sqrt(3), 1000.0,
                                                          rng.uniform(0, .25, (nx, nz)),
                                                          rng.uniform(-.05, .15, (nx, nz)), 0.0)]
    S = oracle.expand_boundary(m)
    codes, mm = [], []
    for c in cij:
        cd, mn, mx = oracle.compress(oracle.expand_boundary(c))
        codes.append(cd)
        mm += [mn, mx]
    mm = np.array(mm, np.float32)
    Tr, _ = ref.solve(S, 10.0, 10.0, 300.0, 0.0, ani=(codes, mm))
    e = Engine(nx, nz, 10.0, 10.0)
    e.set_slowness(m)
    e.set_stiffness_codes(codes, mm)
    T = e.time_propagation(300.0, 0.0, ani=True)
    print(f"ANI: nodes equal to the reference kernels {np.mean(T == Tr):.6f}")
    assert np.array_equal(T, Tr)


def test_engine_matches_golden_vectors(oracle, engine_lib, cuda):
    import glob
    import os
    from seisfat2d_gb300 import Engine
    files = sorted(glob.glob(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "*.npz")))
    assert files
    for f in files:
        d = np.load(f)
        S = d["S"]
        nxx, nzz = S.shape
        e = Engine(nxx - 6, nzz - 6, float(d["dx"]), float(d["dz"]))
        e.set_slowness(S, padded=True)
        ani = "codes" in d
        if ani:
            e.set_stiffness_codes(list(d["codes"]), d["mm"])
        T = e.time_propagation(float(d["sx"]), float(d["sz"]), ani=ani)
        print(os.path.basename(f), f"nodes equal to the reference kernels {np.mean(T == d['T_ref']):.6f}")
        assert np.array_equal(T, d["T_ref"])


def test_reference_solver_timing_config2(oracle, engine_lib, cuda):
    """Times the reference's own per-shot solver (its kernels, its launch
    sequence) and the engine's per-shot drop-in on the 2007 x 507 padded grid;
    prints ms/shot for the record and checks the two agree to 1e-5."""
    ref = _ref()
    import time

    from seisfat2d_gb300 import Engine
    from seisfat2d_gb300.synthetic import config2
    w = config2()
    S = oracle.expand_boundary(w.slowness)
    Tr, ms_ref = ref.solve(S, w.dx, w.dz, 10000.0, 0.0, repeats=3)
    e = Engine(w.nx, w.nz, w.dx, w.dz)
    e.set_slowness(w.slowness)
    Td = cuda.empty((e.nxx, e.nzz), dtype=cuda.float32, device="cuda")
    e.time_propagation(10000.0, 0.0, out=Td)
    cuda.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(3):
        e.time_propagation(10000.0, 0.0, out=Td)
    cuda.cuda.synchronize()
    ms_ours = (time.perf_counter() - t0) / 3 * 1e3
    T = Td.cpu().numpy()
    print(f"\nREFERENCE_TIMING cfg2 2007x507: reference solver {ms_ref:.3f} ms/shot, "
          f"engine per-shot drop-in {ms_ours:.3f} ms/shot, equal nodes {np.mean(T == Tr):.6f}")
    assert np.array_equal(T, Tr)


def test_random_tiny_cases_bitwise(oracle, engine_lib, cuda):
    """Seeded random tiny grids (contrasts 500-6000 m/s, fractional source
    positions, uneven spacings, tilted anisotropy): the engine in reference
    arithmetic equals the reference's kernels on every node."""
    ref = _ref()
    from seisfat2d_gb300 import Engine
    from seisfat2d_gb300.synthetic import thomsen_stiffness
    rng = np.random.default_rng(2026)
    bad = 0
    for c in range(160):
        nx, nz = int(rng.integers(5, 16)), int(rng.integers(5, 16))
        dx = float(rng.choice([5.0, 7.5, 10.0, 12.5, 3.3]))
        dz = float(rng.choice([5.0, 7.5, 10.0, 12.5, 4.1]))
        v = rng.uniform(500.0, 6000.0, (nx, nz))
        m = (1.0 / v).astype(np.float32)
        S = oracle.expand_boundary(m)
        sx = float(rng.uniform(0, (nx - 1) * dx))
        sz = float(rng.uniform(0, (nz - 1) * dz))
        e = Engine(nx, nz, dx, dz)
        e.set_slowness(m)
        ani = None
        if c >= 120:
            cij = thomsen_stiffness(v, v / np.sqrt(3.0), 1000.0, rng.uniform(0.0, 0.3, (nx, nz)),
                                    rng.uniform(-0.1, 0.2, (nx, nz)), float(rng.uniform(-45, 45)))
            codes, mm = [], []
            for q in cij:
                cd, mn, mx = oracle.compress(oracle.expand_boundary(q.astype(np.float32)))
                codes.append(cd)
                mm += [mn, mx]
            ani = (codes, np.array(mm, np.float32))
            e.set_stiffness_codes(*ani)
        Tr, _ = ref.solve(S, dx, dz, sx, sz, ani=ani)
        T = e.time_propagation(sx, sz, ani=ani is not None)
        bad += not np.array_equal(T, Tr)
        e.close()
    print(f"random tiny cases differing from the reference kernels: {bad} of 160")
    assert bad == 0


def test_anisotropic_config3_full_grid_matches_reference_kernels(oracle, engine_lib, cuda):
    """The 1601 x 401 VTI workload (1607 x 407 padded), one shot, against the
    reference's own two-pass kernels on every node; the FP64 anisotropic
    oracle gives the error of both FP32 fields."""
    ref = _ref()
    from seisfat2d_gb300 import Engine
    from seisfat2d_gb300.synthetic import config3
    w = config3()
    S = oracle.expand_boundary(w.slowness)
    codes, mm = [], []
    for c in w.cij:
        cd, mn, mx = oracle.compress(oracle.expand_boundary(c))
        codes.append(cd)
        mm += [mn, mx]
    mm = np.array(mm, np.float32)
    sx, sz = float(w.shots[50][0]), float(w.shots[50][1])
    Tr, ms_ref = ref.solve(S, w.dx, w.dz, sx, sz, ani=(codes, mm))
    e = Engine(w.nx, w.nz, w.dx, w.dz)
    e.set_slowness(w.slowness)
    e.set_stiffness_codes(codes, mm)
    T = e.time_propagation(sx, sz, ani=True)
    T64 = oracle.shot_ani_f64(S, w.dx, w.dz, sx, sz, (codes, mm))
    inner = (slice(3, -3), slice(3, -3))
    er = rel_err(T[inner], T64[inner])
    print(f"\nVTI 1607x407 shot at x={sx:.1f} m: nodes equal to the reference kernels {np.mean(T == Tr):.6f} "
          f"(reference solver {ms_ref:.1f} ms); vs the FP64 oracle: max rel {er.max():.2e}, "
          f"RMS {np.sqrt(np.mean(er ** 2)):.2e}")
    assert np.array_equal(T, Tr)
