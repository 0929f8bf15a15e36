"""Small seeded models and geometries shared by the tests."""
import numpy as np


def smooth_model(nx, nz, dh, seed=0, vmin=1500.0, vmax=3500.0, noise=0.0):
    """Depth gradient plus a Gaussian bump and optional seeded noise:
    returns slowness (nx, nz) float32."""
    rng = np.random.default_rng(seed)
    x = np.arange(nx) * dh
    z = np.arange(nz) * dh
    v = vmin + (vmax - vmin) * (z[None, :] / max(z[-1], 1.0)) + 0 * x[:, None]
    cx, cz = rng.uniform(0.3, 0.7) * x[-1], rng.uniform(0.3, 0.7) * z[-1]
    v = v + 300.0 * np.exp(-((x[:, None] - cx) ** 2 + (z[None, :] - cz) ** 2) / (2 * (0.15 * x[-1] + dh) ** 2))
    if noise:
        v = np.maximum(v * (1.0 + noise * rng.standard_normal(v.shape)), 300.0)
    return (1.0 / v).astype(np.float32)


def layered(nx, nz, dh, vels, tops):
    z = np.arange(nz) * dh
    v = np.full((nx, nz), vels[0], np.float64)
    for k, t in enumerate(tops):
        v[:, z >= t] = vels[k + 1]
    return (1.0 / v).astype(np.float32)


def surface_receivers(nx, dh, step=1):
    rx = (np.arange(0, nx, step) * dh).astype(np.float32)
    return rx, np.zeros_like(rx)


def rel_err(a, b, floor=1e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)
