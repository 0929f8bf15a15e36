"""Small seeded models and geometries shared by the tests."""
import os

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


# parameters.txt of the C++ drivers, with the keys of the reference's run/parameters.txt
PARAMS = """#--------------------------------------------------------------
# Model paramenters
x_samples = {nx}                       # <int>
z_samples = {nz}                       # <int>

x_spacing = {dx}                       # [m] <float>
z_spacing = {dz}                       # [m] <float>

slowness_file = {d}/slowness.bin
Cijkl_folder = {d}/model_
SPS = {d}/sps.txt
RPS = {d}/rps.txt
modeling_type = {mtype}
modeling_output_folder = {d}/out_
batch_shots = {batch}
quiet = true
inv_type = {invtype}
inv_max_it = {maxit}
smooth_per_iteration = true
gaussian_filter_stdv = 2.0
gaussian_filter_samples = 5
inv_residuo_folder = {d}/
inv_output_folder = {d}/
inv_data_folder = {d}/
inv_data_prefix = obs_shot_
anisotropy = {aniso}
mig_tables_folder = {d}/tab_
mig_type = {migtype}
mig_max_angle = 60
mig_angle_spacing = 2.0
time_samples = 400
time_spacing = 2e-3
max_frequency = 25.0
mig_aperture = 35
mig_max_offset = 600
mig_data_folder = {d}/
mig_data_prefix = mig_shot_
mig_seismic_folder = {d}/
mig_max_iteration = 3
mig_residuo_folder = {d}/
mig_smooth_lambda = 0.5
"""


def write_case(d, nx, nz, dx, dz, m, shots, recs, mtype=0, batch=False, aniso=False, migtype=0, invtype=0,
               maxit=3):
    m.astype(np.float32).tofile(os.path.join(d, "slowness.bin"))
    with open(os.path.join(d, "sps.txt"), "w") as f:
        f.write("".join(f"{x},{z}\n" for x, z in shots))
    with open(os.path.join(d, "rps.txt"), "w") as f:
        f.write("".join(f"{x},{z}\n" for x, z in recs))
    p = os.path.join(d, "parameters.txt")
    with open(p, "w") as f:
        f.write(PARAMS.format(nx=nx, nz=nz, dx=dx, dz=dz, d=d, mtype=mtype, batch="true" if batch else "false",
                              aniso="true" if aniso else "false", migtype=migtype, invtype=invtype,
                              maxit=maxit))
    return p
