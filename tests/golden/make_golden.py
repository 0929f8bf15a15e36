"""Generate the golden vectors of tests/golden/ by running the reference's own
kernels (oracle/build_ref.py cubins, replayed by oracle/ref_harness.cpp) on a
GB300 on small seeded cases.

Usage (needs a GPU and the cubins built from the reference sources):
    python tests/golden/make_golden.py --out tests/golden

Each case file ``<name>.npz`` holds the inputs (padded slowness, spacing,
source, optional quantised Cij codes and their ranges) and the reference's
traveltime field ``T_ref`` (nxx, nzz).
"""
import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from helpers import smooth_model  # noqa: E402
from oracle import oracle as O  # noqa: E402
from oracle import refkernels  # noqa: E402
from seisfat2d_gb300.synthetic import thomsen_stiffness  # noqa: E402

CASES = [
    # name, nx, nz, dx, dz, sx, sz, noise, ani
    ("iso_40x20_corner", 40, 20, 10.0, 10.0, 0.0, 0.0, 0.02, False),
    ("iso_20x40_interior", 20, 40, 10.0, 10.0, 93.0, 211.0, 0.02, False),
    ("iso_61x33_dxdz", 61, 33, 12.5, 7.5, 400.0, 10.0, 0.03, False),
    ("iso_120x50_surface", 120, 50, 10.0, 10.0, 555.0, 0.0, 0.0, False),
    ("iso_300x252_skipped_cells", 300, 252, 10.0, 10.0, 1000.0, 500.0, 0.0, False),
    ("ani_60x30_vti", 60, 30, 10.0, 10.0, 300.0, 0.0, 0.0, True),
    ("ani_45x45_tilt", 45, 45, 10.0, 10.0, 220.0, 100.0, 0.0, True),
    ("s_iso_96x48_n30", 96, 48, 5.0, 5.0, 237.5, 0.0, 0.30, False),
    ("s_iso_80x30_dxdz", 80, 30, 7.0, 12.0, 100.0, 0.0, 0.15, False),
    ("s_ani_60x40_tilt_n", 60, 40, 10.0, 10.0, 290.0, 10.0, 0.10, True),
]

# rougher inputs that exercise the edge-update branches and the comparisons
SEARCH_CASES = [
    ("s_iso_64x40_n10", 64, 40, 10.0, 10.0, 310.0, 5.0, 0.10, False),
    ("s_iso_40x64_n20", 40, 64, 10.0, 10.0, 190.0, 333.0, 0.20, False),
    ("s_iso_80x30_dxdz", 80, 30, 7.0, 12.0, 100.0, 0.0, 0.15, False),
    ("s_iso_50x50_n05", 50, 50, 10.0, 10.0, 0.0, 490.0, 0.05, False),
    ("s_iso_96x48_n30", 96, 48, 5.0, 5.0, 237.5, 0.0, 0.30, False),
    ("s_iso_70x35_dxdz2", 70, 35, 12.5, 6.25, 431.0, 87.0, 0.10, False),
    ("s_ani_60x40_tilt_n", 60, 40, 10.0, 10.0, 290.0, 10.0, 0.10, True),
    ("s_ani_50x50_tilt_n", 50, 50, 10.0, 10.0, 10.0, 250.0, 0.05, True),
]


def make_case(name, nx, nz, dx, dz, sx, sz, noise, ani):
    m = smooth_model(nx, nz, 10.0, seed=nx * 31 + nz, noise=noise)
    S = O.expand_boundary(m)
    out = dict(S=S, dx=np.float32(dx), dz=np.float32(dz), sx=np.float32(sx), sz=np.float32(sz))
    anix = None
    if ani:
        rng = np.random.default_rng(nx + nz)
        vp = 1.0 / m.astype(np.float64)
        eps = rng.uniform(0.0, 0.25, (nx, nz))
        dl = rng.uniform(-0.05, 0.15, (nx, nz))
        tilt = (20.0 if name.startswith("ani") else 35.0) if "tilt" in name else 0.0
        cij = thomsen_stiffness(vp, vp / np.sqrt(3.0), 1000.0, eps, dl, tilt)
        codes, mm = [], []
        for c in cij:
            cd, mn, mx = O.compress(O.expand_boundary(c.astype(np.float32)))
            codes.append(cd)
            mm += [mn, mx]
        out["codes"] = np.stack(codes)
        out["mm"] = np.array(mm, np.float32)
        anix = (codes, out["mm"])
    T, _ = refkernels.solve(S, dx, dz, sx, sz, ani=anix)
    out["T_ref"] = T
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.dirname(os.path.abspath(__file__)))
    ap.add_argument("--search", action="store_true", help="the rough cases instead")
    a = ap.parse_args()
    os.makedirs(a.out, exist_ok=True)
    for c in (SEARCH_CASES if a.search else CASES):
        d = make_case(*c)
        np.savez_compressed(os.path.join(a.out, c[0] + ".npz"), **d)
        print("wrote", c[0])


if __name__ == "__main__":
    main()
