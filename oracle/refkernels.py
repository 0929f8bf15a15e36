"""Run the reference's own kernels (test infrastructure; see build_ref.py)."""
import ctypes as C
import os

import numpy as np

from . import build_ref

_h = None


def available():
    return build_ref.available()


def _handle(device=0):
    global _h
    if _h is None:
        path = build_ref.build_harness()
        h = C.CDLL(path)
        h.ref_open.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
        h.ref_solve.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_float, C.c_float, C.c_float,
                                C.c_float, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.POINTER(C.c_double), C.c_int]
        rc = h.ref_open(build_ref.cubin_path("modeling").encode(),
                        build_ref.cubin_path("eikonal_ani").encode(), device)
        if rc != 0:
            raise RuntimeError(f"ref_open failed ({rc})")
        _h = h
    return _h


def solve(S_padded, dx, dz, sx, sz, ani=None, nb=3, repeats=1):
    """Reference time_propagation on a padded (nxx, nzz) slowness.
    ani: (codes[6] padded uint16, mm[12]) or None. Returns (T, ms)."""
    h = _handle()
    S = np.ascontiguousarray(S_padded, np.float32)
    nxx, nzz = S.shape
    T = np.zeros_like(S)
    ms = C.c_double()
    if ani is not None:
        codes = [np.ascontiguousarray(c, np.uint16) for c in ani[0]]
        arr = (C.c_void_p * 6)(*[c.ctypes.data for c in codes])
        mm = np.ascontiguousarray(ani[1], np.float32)
        cp, mp = C.cast(arr, C.c_void_p), C.c_void_p(mm.ctypes.data)
    else:
        cp, mp = None, None
    rc = h.ref_solve(nxx, nzz, nb, C.c_void_p(S.ctypes.data), dx, dz, sx, sz, 1 if ani is not None else 0,
                     cp, mp, C.c_void_p(T.ctypes.data), C.byref(ms), repeats)
    if rc != 0:
        raise RuntimeError(f"ref_solve failed ({rc})")
    return T, ms.value


def init(S_padded, dx, dz, sx, sz, nb=3):
    """The reference's time_set + time_init field (no sweeps)."""
    h = _handle()
    h.ref_init.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_float, C.c_float, C.c_float,
                           C.c_float, C.c_void_p]
    S = np.ascontiguousarray(S_padded, np.float32)
    T = np.zeros_like(S)
    rc = h.ref_init(S.shape[0], S.shape[1], nb, C.c_void_p(S.ctypes.data), dx, dz, sx, sz,
                    C.c_void_p(T.ctypes.data))
    if rc != 0:
        raise RuntimeError(f"ref_init failed ({rc})")
    return T


def kirchhoff_adjoint(S_padded, Ts, Tr, xsrc, xrec, data, dt, dx, dz, aperture, max_offset, nb=3):
    """The reference's IDKDM trace loop (KDM.cu:3-55) with its own
    image_domain_adjoint_kernel on correlated traces data (nsrc, nrec, nt);
    tables (n, nxx, nzz). Returns the (nx, nz) image."""
    h = _handle()
    if not getattr(h, "_kirch", False):
        h.ref_kirchhoff_open.argtypes = [C.c_char_p]
        h.ref_kirchhoff_adjoint.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 3 + [C.c_int, C.c_int] + \
            [C.c_void_p] * 3 + [C.c_int] + [C.c_float] * 5 + [C.c_void_p]
        rc = h.ref_kirchhoff_open(build_ref.cubin_path("migration").encode())
        if rc != 0:
            raise RuntimeError(f"ref_kirchhoff_open failed ({rc})")
        h._kirch = True
    S = np.ascontiguousarray(S_padded, np.float32)
    nxx, nzz = S.shape
    Ts = np.ascontiguousarray(Ts, np.float32)
    Tr = np.ascontiguousarray(Tr, np.float32)
    xs = np.ascontiguousarray(xsrc, np.float32)
    xr = np.ascontiguousarray(xrec, np.float32)
    d = np.ascontiguousarray(data, np.float32)
    img = np.zeros((nxx - 2 * nb, nzz - 2 * nb), np.float32)
    rc = h.ref_kirchhoff_adjoint(nxx, nzz, nb, S.ctypes.data, Ts.ctypes.data, Tr.ctypes.data, len(xs), len(xr),
                                 xs.ctypes.data, xr.ctypes.data, d.ctypes.data, d.shape[-1], dt, dx, dz, aperture,
                                 max_offset, img.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"ref_kirchhoff_adjoint failed ({rc})")
    return img


def kirchhoff_angles(S_padded, Ts, Tr, xsrc, xrec, data, dt, dx, dz, aperture, max_offset, max_angle, da, nb=3):
    """The reference's ADKDM trace loop with its own angle_domain_adjoint_kernel;
    returns gathers (ncmp, nang, nz). CMP bins as Migration::set_gathers with
    the largest CMP started from the first pair's (the reference leaves it
    uninitialised)."""
    h = _handle()
    if not getattr(h, "_kirch", False):
        h.ref_kirchhoff_open.argtypes = [C.c_char_p]
        if h.ref_kirchhoff_open(build_ref.cubin_path("migration").encode()) != 0:
            raise RuntimeError("ref_kirchhoff_open failed")
        h.ref_kirchhoff_adjoint.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 3 + [C.c_int, C.c_int] + \
            [C.c_void_p] * 3 + [C.c_int] + [C.c_float] * 5 + [C.c_void_p]
        h._kirch = True
    h.ref_kirchhoff_angles.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 3 + [C.c_int, C.c_int] + \
        [C.c_void_p] * 3 + [C.c_int] + [C.c_float] * 6 + [C.c_int, C.c_int, C.c_float, C.c_float, C.c_void_p]
    xs = np.ascontiguousarray(xsrc, np.float32)
    xr = np.ascontiguousarray(xrec, np.float32)
    f32 = np.float32
    d = f32(0.5) * min(f32(xs[1] - xs[0]), f32(xr[1] - xr[0]))
    cmps = (f32(0.5) * (xs[:, None] + xr[None, :])).astype(np.float32)
    mn, mx = f32(min(f32(1e6), cmps.min())), f32(cmps.max())
    na = int(f32(max_angle) / f32(da)) + 1
    nc = int(f32(mx - mn) / d) + 1
    S = np.ascontiguousarray(S_padded, np.float32)
    nxx, nzz = S.shape
    Ts = np.ascontiguousarray(Ts, np.float32)
    Tr = np.ascontiguousarray(Tr, np.float32)
    dd = np.ascontiguousarray(data, np.float32)
    g = np.zeros((nc, na, nzz - 2 * nb), np.float32)
    rc = h.ref_kirchhoff_angles(nxx, nzz, nb, S.ctypes.data, Ts.ctypes.data, Tr.ctypes.data, len(xs), len(xr),
                                xs.ctypes.data, xr.ctypes.data, dd.ctypes.data, dd.shape[-1], dt, dx, dz, aperture,
                                max_offset, da, na, nc, float(mn), float(d), g.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"ref_kirchhoff_angles failed ({rc})")
    return g


def kirchhoff_forward(S_padded, Ts, Tr, xsrc, xrec, model, nt, dt, dx, dz, aperture, max_offset, max_angle=None,
                      da=None, nb=3):
    """The reference's least-squares forward operator per trace
    (LSKDM.cu:52-90) with its own image_domain_forward_kernel (model (nx, nz))
    or, with max_angle and da, angle_domain_forward_kernel (model = gathers
    (ncmp, nang, nz)); returns raw traces (nsrc, nrec, nt)."""
    h = _handle()
    if not getattr(h, "_kirch", False):
        h.ref_kirchhoff_open.argtypes = [C.c_char_p]
        if h.ref_kirchhoff_open(build_ref.cubin_path("migration").encode()) != 0:
            raise RuntimeError("ref_kirchhoff_open failed")
        h.ref_kirchhoff_adjoint.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 3 + [C.c_int, C.c_int] + \
            [C.c_void_p] * 3 + [C.c_int] + [C.c_float] * 5 + [C.c_void_p]
        h._kirch = True
    h.ref_kirchhoff_forward.argtypes = [C.c_int] * 4 + [C.c_void_p] * 3 + [C.c_int, C.c_int] + [C.c_void_p] * 3 + \
        [C.c_size_t, C.c_int] + [C.c_float] * 6 + [C.c_int, C.c_float, C.c_float, C.c_void_p]
    xs = np.ascontiguousarray(xsrc, np.float32)
    xr = np.ascontiguousarray(xrec, np.float32)
    S = np.ascontiguousarray(S_padded, np.float32)
    nxx, nzz = S.shape
    m = np.ascontiguousarray(model, np.float32)
    angle = max_angle is not None
    na, mn, d = 0, 0.0, 1.0
    if angle:
        f32 = np.float32
        d = f32(0.5) * min(f32(xs[1] - xs[0]), f32(xr[1] - xr[0]))
        cmps = (f32(0.5) * (xs[:, None] + xr[None, :])).astype(np.float32)
        mn = f32(min(f32(1e6), cmps.min()))
        na = int(f32(max_angle) / f32(da)) + 1
    out = np.zeros((len(xs), len(xr), int(nt)), np.float32)
    Ts = np.ascontiguousarray(Ts, np.float32)
    Tr = np.ascontiguousarray(Tr, np.float32)
    rc = h.ref_kirchhoff_forward(1 if angle else 0, nxx, nzz, nb, S.ctypes.data, Ts.ctypes.data, Tr.ctypes.data,
                                 len(xs), len(xr), xs.ctypes.data, xr.ctypes.data, m.ctypes.data, m.size, int(nt),
                                 dt, dx, dz, aperture, max_offset, float(da or 1.0), na, float(mn), float(d),
                                 out.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"ref_kirchhoff_forward failed ({rc})")
    return out
