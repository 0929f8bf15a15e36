"""Seeded synthetic workloads with the shapes of the five benchmark configs.

The reference ships no data (its inputs/ folders are empty), so every model,
geometry and observed-pick set here is generated from a recorded numpy seed.
Models are returned as slowness ``(nx, nz)`` float32 arrays (z fastest, the
reference's ``nz x nx`` binary layout).
"""
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    nx: int
    nz: int
    dx: float
    dz: float
    slowness: np.ndarray            # (nx, nz) float32
    shots: list                     # (sx, sz) or (sx, sz, c0, ncols)
    rx: np.ndarray
    rz: np.ndarray
    seed: int
    cij: list = field(default=None)  # six (nx, nz) float32 fields (anisotropic)
    extra: dict = field(default_factory=dict)


def _smooth1d(a, sigma_samples, axis):
    if sigma_samples <= 0:
        return a
    r = int(3 * sigma_samples) + 1
    k = np.exp(-0.5 * (np.arange(-r, r + 1) / sigma_samples) ** 2)
    k /= k.sum()
    pad = [(0, 0)] * a.ndim
    pad[axis] = (r, r)
    ap = np.pad(a, pad, mode="edge")
    out = np.zeros_like(a, dtype=np.float64)
    n = a.shape[axis]
    for q, w in enumerate(k):
        sl = [slice(None)] * a.ndim
        sl[axis] = slice(q, q + n)
        out += w * ap[tuple(sl)]
    return out


def gaussian_smooth(a, sigma_samples):
    """Separable Gaussian smoothing with edge padding."""
    out = np.asarray(a, np.float64)
    for ax in range(out.ndim):
        out = _smooth1d(out, sigma_samples, ax)
    return out


def gradient_model(nx, nz, dh, rng, water=200.0, v0=1800.0, v1=4000.0, anomaly=300.0, sigma=250.0):
    """Water layer, then a linear gradient, plus a seeded Gaussian anomaly."""
    x = np.arange(nx) * dh
    z = np.arange(nz) * dh
    zmax = z[-1]
    vp = np.where(z[None, :] < water, 1500.0,
                  v0 + (v1 - v0) * np.clip((z[None, :] - water) / max(zmax - water, 1.0), 0, 1))
    vp = np.broadcast_to(vp, (nx, nz)).copy()
    ax = rng.uniform(0.2, 0.8) * x[-1]
    az = rng.uniform(water + 0.2 * (zmax - water), water + 0.8 * (zmax - water))
    sign = rng.choice([-1.0, 1.0])
    bump = sign * anomaly * np.exp(-((x[:, None] - ax) ** 2 + (z[None, :] - az) ** 2) / (2 * sigma ** 2))
    vp = vp + np.where(z[None, :] >= water, bump, 0.0)
    return vp


def layered_model(nx, nz, dh, rng, nlayers, vmin=1500.0, vmax=4500.0, perturb=50.0, nfaults=0,
                  throw=(50.0, 150.0)):
    """Layers with smoothly perturbed interfaces, optionally cut by dipping
    normal faults that drop the hanging wall by a seeded throw."""
    x = np.arange(nx) * dh
    z = np.arange(nz) * dh
    zmax = z[-1]
    vels = np.linspace(vmin, vmax, nlayers)
    base = np.linspace(0, zmax, nlayers + 1)[1:-1]
    tops = []
    for b in base:
        noise = rng.standard_normal(nx)
        noise = _smooth1d(noise, 100.0 / dh * 5, 0)
        noise = noise / (np.abs(noise).max() + 1e-12) * perturb
        tops.append(b + noise)
    tops = np.array(tops)  # (nlayers-1, nx)
    shift = np.zeros((nx, nz))
    for _ in range(nfaults):
        xf = rng.uniform(0.1, 0.9) * x[-1]
        dip = np.radians(rng.uniform(55.0, 80.0)) * rng.choice([-1.0, 1.0])
        t = rng.uniform(*throw)
        side = x[:, None] > xf + z[None, :] / np.tan(dip)
        shift += np.where(side, t, 0.0)
    zz = z[None, :] - shift  # depth in the unfaulted frame
    layer = np.zeros((nx, nz), np.int64)
    for k in range(tops.shape[0]):
        layer += (zz >= tops[k][:, None]).astype(np.int64)
    return vels[layer]


def thomsen_stiffness(vp, vs, rho, eps, dlt, tilt_deg=0.0):
    """Rotated 2D VTI stiffness (C11, C13, C15, C33, C35, C55) in Pa from
    Thomsen parameters, following the formulas of src/functions.py:72-109 of
    the reference (restated here, not imported)."""
    c33 = rho * vp ** 2
    c55 = rho * vs ** 2
    c11 = c33 * (1.0 + 2.0 * eps)
    c13 = np.sqrt((c33 - c55) ** 2 + 2.0 * dlt * c33 * (c33 - c55)) - c55
    c15 = np.zeros_like(c33)
    c35 = np.zeros_like(c33)
    th = np.radians(tilt_deg)
    if th == 0.0:
        return [c11, c13, c15, c33, c35, c55]
    c, s = np.cos(th), np.sin(th)
    s2, c2 = np.sin(2 * th), np.cos(2 * th)
    M = np.array([[c * c, s * s, s2], [s * s, c * c, -s2], [-0.5 * s2, 0.5 * s2, c2]])
    C = np.array([[c11, c13, c15], [c13, c33, c35], [c15, c35, c55]])
    R = np.einsum("ab,bc...,dc->ad...", M, C, M)
    return [R[0, 0], R[0, 1], R[0, 2], R[1, 1], R[1, 2], R[2, 2]]


def config1(seed=1):
    rng = np.random.default_rng(seed)
    nx, nz, dh = 1001, 201, 10.0
    vp = gradient_model(nx, nz, dh, rng)
    rx = np.arange(0, nx) * dh
    return Workload("cfg1_plain_iso_1001x201", nx, nz, dh, dh, (1.0 / vp).astype(np.float32),
                    [(5000.0, 0.0)], rx.astype(np.float32), np.zeros(nx, np.float32), seed)


def config2(seed=2, nshots=200):
    rng = np.random.default_rng(seed)
    nx, nz, dh = 2001, 501, 10.0
    vp = layered_model(nx, nz, dh, rng, 6)
    shots = [(100.0 * k, 0.0) for k in range(nshots)]
    rx = (np.arange(800) * 25.0).astype(np.float32)
    return Workload("cfg2_batched_iso_2001x501_200shots", nx, nz, dh, dh, (1.0 / vp).astype(np.float32),
                    shots, rx, np.zeros(800, np.float32), seed)


def config3(seed=3, nshots=100):
    rng = np.random.default_rng(seed)
    nx, nz, dh = 1601, 401, 10.0
    vp = gradient_model(nx, nz, dh, rng)
    sig = 200.0 / dh
    e = gaussian_smooth(rng.standard_normal((nx, nz)), sig)
    d = gaussian_smooth(rng.standard_normal((nx, nz)), sig)
    e = (e - e.min()) / (e.max() - e.min()) * 0.25
    d = (d - d.min()) / (d.max() - d.min()) * 0.20 - 0.05
    vs = vp / np.sqrt(3.0)
    cij = [c.astype(np.float32) for c in thomsen_stiffness(vp, vs, 1000.0, e, d)]
    shots = [(float(x), 0.0) for x in np.linspace(0.0, (nx - 1) * dh, nshots)]
    rx = (np.arange(0, nx, 2) * dh).astype(np.float32)
    return Workload("cfg3_vti_1601x401_100shots", nx, nz, dh, dh, (1.0 / vp).astype(np.float32), shots,
                    rx, np.zeros(len(rx), np.float32), seed, cij=cij,
                    extra={"eps": e.astype(np.float32), "delta": d.astype(np.float32)})


def config4(seed=4, nshots=100, nrec=400):
    rng = np.random.default_rng(seed)
    nx, nz, dh = 1701, 351, 10.0
    vp = layered_model(nx, nz, dh, rng, 6, nfaults=3)
    start = gaussian_smooth(vp, 500.0 / dh)
    shots = [(float(x), 0.0) for x in np.linspace(0.0, (nx - 1) * dh, nshots)]
    rx = np.linspace(0.0, (nx - 1) * dh, nrec).astype(np.float32)
    return Workload("cfg4_adjoint_1701x351_100shots_400rec", nx, nz, dh, dh,
                    (1.0 / start).astype(np.float32), shots, rx, np.zeros(nrec, np.float32), seed,
                    extra={"true_slowness": (1.0 / vp).astype(np.float32), "noise_sigma": 0.002})


def config5(seed=5, nshots=1000):
    rng = np.random.default_rng(seed)
    nx, nz, dh = 4001, 1001, 5.0
    vp = layered_model(nx, nz, dh, rng, 8, nfaults=6)
    start = gaussian_smooth(vp, 500.0 / dh)
    nb = 3
    nxx = nx + 2 * nb
    shots = []
    for k in range(nshots):
        sx = 20.0 * k
        width = rng.uniform(2000.0, 8000.0)
        c_lo = int(np.floor((sx - width / 2) / dh)) + nb
        c_hi = int(np.ceil((sx + width / 2) / dh)) + nb
        c_lo = max(0, c_lo)
        c_hi = min(nxx, c_hi + 1)
        shots.append((sx, 0.0, c_lo, c_hi - c_lo))
    rx = (np.arange(0, nx, 5) * dh).astype(np.float32)
    return Workload("cfg5_uneven_4001x1001_1000shots", nx, nz, dh, dh, (1.0 / start).astype(np.float32),
                    shots, rx, np.zeros(len(rx), np.float32), seed,
                    extra={"true_slowness": (1.0 / vp).astype(np.float32), "noise_sigma": 0.002})


CONFIGS = {1: config1, 2: config2, 3: config3, 4: config4, 5: config5}
