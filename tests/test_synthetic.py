"""The seeded synthetic workloads have the sizes, spacings, geometries and
value ranges of the five benchmark configurations, and a seed reproduces
them exactly (the bench and the tests stand on these inputs)."""
import numpy as np
import pytest

from seisfat2d_gb300 import synthetic

NB = 3


def _vel(w, key=None):
    s = w.slowness if key is None else w.extra[key]
    return 1.0 / s.astype(np.float64)


def test_config1_gradient_model_and_geometry():
    w = synthetic.config1()
    assert (w.nx, w.nz, w.dx, w.dz) == (1001, 201, 10.0, 10.0)
    assert w.slowness.shape == (1001, 201) and w.slowness.dtype == np.float32
    v = _vel(w)
    assert np.allclose(v[:, :20], 1500.0, rtol=1e-6)           # water to 200 m
    assert v.min() >= 1500.0 - 1e-3 and v.max() <= 4000.0 + 300.0 + 1e-3
    assert w.shots == [(5000.0, 0.0)]
    assert np.array_equal(w.rx, np.arange(1001, dtype=np.float32) * 10.0) and not w.rz.any()


def test_config2_layers_and_geometry():
    w = synthetic.config2()
    assert (w.nx, w.nz, w.dx) == (2001, 501, 10.0)
    v = _vel(w)
    assert v.min() >= 1500.0 - 1e-3 and v.max() <= 4500.0 + 1e-3
    assert len(np.unique(np.round(v, 3))) <= 6
    assert [s[0] for s in w.shots] == [100.0 * k for k in range(200)] and all(s[1] == 0.0 for s in w.shots)
    assert np.array_equal(w.rx, np.arange(800, dtype=np.float32) * 25.0)


def test_config3_thomsen_fields():
    w = synthetic.config3()
    assert (w.nx, w.nz, w.dx) == (1601, 401, 10.0) and len(w.shots) == 100
    e, d = w.extra["eps"], w.extra["delta"]
    assert e.min() >= 0.0 and e.max() <= 0.25 + 1e-6
    assert d.min() >= -0.05 - 1e-6 and d.max() <= 0.15 + 1e-6
    c11, c13, c15, c33, c35, c55 = (c.astype(np.float64) for c in w.cij)
    vp = _vel(w)
    assert np.allclose(c33, 1000.0 * vp ** 2, rtol=1e-6)
    assert np.allclose(c55, c33 / 3.0, rtol=1e-5)              # vs = vp / sqrt(3)
    assert np.allclose(c11, c33 * (1.0 + 2.0 * e), rtol=1e-5)
    assert not c15.any() and not c35.any()                     # no tilt


def test_config4_layers_faults_start_model():
    w = synthetic.config4()
    assert (w.nx, w.nz, w.dx) == (1701, 351, 10.0) and len(w.shots) == 100 and len(w.rx) == 400
    vt = _vel(w, "true_slowness")
    assert vt.min() >= 1500.0 - 1e-3 and vt.max() <= 4500.0 + 1e-3
    v0 = _vel(w)
    assert v0.std() < vt.std()                                 # start model = truth smoothed
    assert w.extra["noise_sigma"] == 0.002


def test_config5_uneven_windows():
    w = synthetic.config5()
    assert (w.nx, w.nz, w.dx) == (4001, 1001, 5.0) and len(w.shots) == 1000
    nxx = w.nx + 2 * NB
    for k, (sx, sz, c0, nc) in enumerate(w.shots):
        assert sx == 20.0 * k and sz == 0.0
        assert 0 <= c0 and c0 + nc <= nxx
        assert c0 <= int(round(sx / w.dx)) + NB < c0 + nc       # the source lies in its window
        full = (c0 > 0) and (c0 + nc < nxx)
        if full:                                               # unclipped windows are 2-8 km wide
            assert 2000.0 <= (nc - 2) * w.dx <= 8000.0 + 2 * w.dx
    widths = np.array([s[3] for s in w.shots])
    assert widths.min() < widths.max()                          # uneven


@pytest.mark.parametrize("cfg", [1, 4])
def test_seed_reproduces_the_workload(cfg):
    a = synthetic.CONFIGS[cfg]()
    b = synthetic.CONFIGS[cfg]()
    assert np.array_equal(a.slowness, b.slowness) and a.shots == b.shots
    c = synthetic.CONFIGS[cfg](seed=a.seed + 100)
    assert not np.array_equal(a.slowness, c.slowness)
