"""ctypes view of the CPU oracle (test infrastructure: tests/, the smoke entry
and the bench's CPU-baseline leg only).

Arrays follow the reference's layout: a padded field of ``nzz`` rows (z) by
``nxx`` columns (x) is stored z-fastest, i.e. a numpy array of shape
``(nxx, nzz)`` in C order (``a[j, i]`` is row ``i``, column ``j``).
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
u16p = np.ctypeslib.ndpointer(np.uint16, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
IP = C.POINTER(C.c_int)


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            path = _build.build()
        L = C.CDLL(path)
        L.orc_expand_boundary.argtypes = [f32p, C.c_int, C.c_int, C.c_int, f32p]
        L.orc_reduce_boundary.argtypes = [f32p, C.c_int, C.c_int, C.c_int, f32p]
        L.orc_skip_cells.argtypes = [C.c_int, C.c_int, i32p, i32p]
        L.orc_source_index.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, IP, IP]
        L.orc_init_block_f64.argtypes = [f32p, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                         C.c_int, C.c_int, C.c_int, f64p]
        L.orc_solve_f32.argtypes = [C.c_int, C.c_int, f32p, C.c_int, C.c_float, C.c_float, C.c_int,
                                    C.c_int, f32p, f32p, C.c_int, C.c_int]
        L.orc_solve_f64.argtypes = [C.c_int, C.c_int, f32p, C.c_int, C.c_double, C.c_double, C.c_int,
                                    C.c_int, f64p, f64p, C.c_int, C.c_double, C.c_int]
        L.orc_solve_f64.restype = C.c_int
        L.orc_compress.argtypes = [f32p, C.c_int, u16p, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.orc_qslowness_f32.argtypes = [C.c_int, C.c_int, C.c_int, f32p, f32p, C.c_int, C.c_float,
                                        C.c_float, C.c_int, C.c_int, C.c_void_p * 6, f32p, f32p]
        L.orc_picks_f32.argtypes = [f32p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int,
                                    f32p, f32p, C.c_int, f32p]
        L.orc_shot_f32.argtypes = [C.c_int, C.c_int, C.c_int, f32p, C.c_float, C.c_float, C.c_int,
                                   C.c_int, C.c_float, C.c_float, C.c_int, C.c_void_p * 6, f32p,
                                   C.c_void_p, f32p, f32p, C.c_int, C.c_void_p]
        L.orc_shot_f32.restype = C.c_int
        L.orc_batch_f32.argtypes = [C.c_int, C.c_int, C.c_int, f32p, C.c_float, C.c_float, C.c_int,
                                    f32p, f32p, i32p, i32p, C.c_int, C.c_void_p * 6, f32p, f32p,
                                    f32p, C.c_int, f32p, C.c_int]
        L.orc_batch_f32.restype = C.c_int
        L.orc_solve_tape_f32.argtypes = [C.c_int, C.c_int, f32p, C.c_int, C.c_float, C.c_float,
                                         C.c_int, C.c_int, f32p, f32p, u8p, f32p, f32p]
        L.orc_solve_tape_f64.argtypes = [C.c_int, C.c_int, f32p, C.c_int, C.c_double, C.c_double,
                                         C.c_int, C.c_int, f64p, f64p, u8p, f64p, f64p]
        L.orc_solve_follow_f64.argtypes = [C.c_int, C.c_int, f32p, C.c_int, C.c_double, C.c_double,
                                           C.c_int, C.c_int, f64p, u8p, f64p, f64p, f64p]
        L.orc_shot_ani_f64.argtypes = [C.c_int, C.c_int, C.c_int, f32p, C.c_float, C.c_float, C.c_int, C.c_int,
                                       C.c_float, C.c_float, C.c_void_p * 6, f32p, f64p]
        L.orc_shot_ani_f64.restype = C.c_int
        L.orc_picks_f64.argtypes = [f64p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int, f32p, f32p,
                                    C.c_int, f64p]
        L.orc_misfit_f64.argtypes = [C.c_int, C.c_int, C.c_int, f32p, C.c_float, C.c_float, C.c_int, f32p, f32p,
                                     i32p, i32p, f32p, f32p, C.c_int, f64p]
        L.orc_misfit_f64.restype = C.c_double
        L.orc_fd_misfit_f64.argtypes = [C.c_int, C.c_int, C.c_int, f32p, C.c_float, C.c_float, C.c_int, f32p,
                                        f32p, i32p, i32p, f32p, f32p, C.c_int, f64p, C.c_int, i32p, i32p,
                                        C.c_double, f32p, f32p, f64p, f64p, C.c_int]
        L.orc_fd_misfit_f64.restype = C.c_int
        L.orc_adjoint_f32.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, u8p, f32p, f32p, f32p,
                                      f32p, f32p]
        L.orc_adjoint_f64.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, u8p, f64p, f64p, f64p,
                                      f64p, f64p]
        L.orc_pick_weights_f64.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                                           C.c_int, C.c_int, C.c_int, IP, IP, f64p]
        L.orc_pick_weights_f64.restype = C.c_int
        L.orc_init_block_f32.argtypes = [f32p, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                         C.c_int, C.c_int, C.c_int, f32p]
        L.orc_set_arith.argtypes = [C.c_int]
        L.orc_seed_lambda_f32.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int,
                                          f32p, f32p, C.c_int, f32p, f32p]
        L.orc_seed_lambda_f64.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int,
                                          f32p, f32p, C.c_int, f64p, f64p]
        L.orc_batch_gradient_f32.argtypes = [C.c_int, C.c_int, C.c_int, f32p, C.c_float, C.c_float,
                                             C.c_int, f32p, f32p, i32p, i32p, f32p, f32p, C.c_int,
                                             f32p, f32p, C.POINTER(C.c_double), f32p, C.c_int, C.c_int,
                                             C.c_void_p * 6, f32p, f32p, f32p]
        L.orc_qp_factors.argtypes = [C.c_int, C.c_int, C.c_int, f32p, f32p, C.c_int, C.c_float, C.c_float,
                                     C.c_int, C.c_int, C.c_void_p * 6, f32p, f32p, f32p, f32p]
        L.orc_batch_gradient_f32.restype = C.c_int
        L.orc_smooth_kernel.argtypes = [C.c_float, C.c_int, f32p]
        L.orc_model_smoothing.argtypes = [f32p, C.c_int, C.c_int, C.c_float, C.c_int, f32p]
        L.orc_kirchhoff_wavelet.argtypes = [C.c_float, C.c_float, f32p, C.c_int]
        L.orc_kirchhoff_wavelet.restype = C.c_int
        L.orc_adjoint_convolution.argtypes = [f32p, f32p, C.c_int, C.c_int, f32p, C.c_int]
        L.orc_kirchhoff_image.argtypes = [C.c_int, C.c_int, C.c_int, f32p, f32p, f32p, C.c_int, C.c_int, f32p,
                                          f32p, f32p, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                          C.c_float, f32p]
        L.orc_kirchhoff_forward.argtypes = [C.c_int, C.c_int, C.c_int, f32p, f32p, f32p, C.c_int, C.c_int, f32p,
                                            f32p, f32p, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float,
                                            C.c_float, C.c_int, C.c_float, C.c_float, C.c_float, f32p]
        L.orc_forward_convolution.argtypes = [f32p, f32p, C.c_int, C.c_int, f32p, C.c_int]
        L.orc_update_slowness.argtypes = [f32p, f32p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int,
                                          f32p]
        _lib = L
    return _lib


_arith = 0


def set_arith(mode):
    """'ieee' (every operation rounded once, FP64 init) or 'reference' (the
    reference build's FP32 init and FMAs)."""
    global _arith
    _arith = {"ieee": 0, "reference": 1, "compensated": 2}[mode] if isinstance(mode, str) else int(mode)
    lib().orc_set_arith(_arith)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def expand_boundary(model, nb=3):
    """model: (nx, nz) float32 -> padded (nx+2nb, nz+2nb)."""
    model = _f32(model)
    nx, nz = model.shape
    out = np.zeros((nx + 2 * nb, nz + 2 * nb), np.float32)
    lib().orc_expand_boundary(model, nx, nz, nb, out)
    return out


def reduce_boundary(padded, nb=3):
    padded = _f32(padded)
    nxx, nzz = padded.shape
    out = np.zeros((nxx - 2 * nb, nzz - 2 * nb), np.float32)
    lib().orc_reduce_boundary(padded, nxx - 2 * nb, nzz - 2 * nb, nb, out)
    return out


def skip_cells(ncols, nzz):
    si = np.zeros(4, np.int32)
    sj = np.zeros(4, np.int32)
    lib().orc_skip_cells(ncols, nzz, si, sj)
    return si, sj


def source_index(sx, sz, dx, dz, nb=3):
    a, b = C.c_int(), C.c_int()
    lib().orc_source_index(sx, sz, dx, dz, nb, C.byref(a), C.byref(b))
    return a.value, b.value


def init_block(S, sx, sz, dx, dz, nb=3):
    S = _f32(S)
    nzz = S.shape[1]
    sIdx, sIdz = source_index(sx, sz, dx, dz, nb)
    v = np.zeros(9, np.float64)
    lib().orc_init_block_f64(S, nzz, sx, sz, dx, dz, nb, sIdx, sIdz, v)
    return v, sIdx, sIdz


def init_block_f32(S, sx, sz, dx, dz, nb=3):
    """The 9 FP32 initial values of the current arithmetic mode."""
    S = _f32(S)
    if _arith == 1:
        sIdx, sIdz = source_index(sx, sz, dx, dz, nb)
        v = np.zeros(9, np.float32)
        lib().orc_init_block_f32(S, S.shape[1], sx, sz, dx, dz, nb, sIdx, sIdz, v)
        return v, sIdx, sIdz
    v, sIdx, sIdz = init_block(S, sx, sz, dx, dz, nb)
    return v.astype(np.float32), sIdx, sIdz


def solve_f32(S, dx, dz, sx, sz, nb=3, passes=1, order=1, c0=0, ncols=None):
    """FP32 restatement of one isotropic solve on window [c0, c0+ncols)."""
    S = _f32(S)
    nxx, nzz = S.shape
    ncols = nxx - c0 if ncols is None else ncols
    init, sIdx, sIdz = init_block_f32(S, sx, sz, dx, dz, nb)
    Sw = np.ascontiguousarray(S[c0:c0 + ncols])
    T = np.zeros((ncols, nzz), np.float32)
    lib().orc_solve_f32(nzz, ncols, Sw, nzz, dx, dz, sIdz, sIdx - c0, init, T, passes, order)
    return T


def solve_f64(S, dx, dz, sx, sz, nb=3, passes=1, tol=0.0, max_passes=50, c0=0, ncols=None):
    """FP64 solve: passes>0 runs that many passes; passes<=0 iterates to tol."""
    S = _f32(S)
    nxx, nzz = S.shape
    ncols = nxx - c0 if ncols is None else ncols
    v, sIdx, sIdz = init_block(S, sx, sz, dx, dz, nb)
    Sw = np.ascontiguousarray(S[c0:c0 + ncols])
    T = np.zeros((ncols, nzz), np.float64)
    n = lib().orc_solve_f64(nzz, ncols, Sw, nzz, dx, dz, sIdz, sIdx - c0, v, T, passes, tol,
                            max_passes)
    return T, n


def compress(field):
    """Quantise a padded field to uint16; returns (codes, vmin, vmax)."""
    field = _f32(field)
    out = np.zeros(field.shape, np.uint16)
    mx, mn = C.c_float(), C.c_float()
    lib().orc_compress(field.ravel(), field.size, out.ravel(), C.byref(mx), C.byref(mn))
    return out, mn.value, mx.value


def _codes_arg(codes):
    arr = (C.c_void_p * 6)()
    keep = []
    for k in range(6):
        c = np.ascontiguousarray(codes[k], dtype=np.uint16)
        keep.append(c)
        arr[k] = c.ctypes.data
    return arr, keep


def qslowness(T, S, dx, dz, sIdz, sIdx, codes, mm, nb=3):
    T = _f32(T)
    S = _f32(S)
    ncols, nzz = T.shape
    arr, keep = _codes_arg(codes)
    out = np.zeros_like(T)
    lib().orc_qslowness_f32(nzz, ncols, nb, T, S, nzz, dx, dz, sIdz, sIdx, arr,
                            _f32(mm), out)
    return out


def qp_factors(T, S, dx, dz, sIdz, sIdx, codes, mm, nb=3):
    """Derivative factors of the qP pass (dSq/dS, dSq/dC11, dSq/dC13) over a
    window, as the taped anisotropic forward writes them."""
    T = _f32(T)
    S = _f32(S)
    ncols, nzz = T.shape
    arr, keep = _codes_arg(codes)
    f = [np.zeros_like(T) for _ in range(3)]
    lib().orc_qp_factors(nzz, ncols, nb, T, S, nzz, dx, dz, sIdz, sIdx, arr, _f32(mm), f[0], f[1], f[2])
    return f


def picks(T, dx, dz, rx, rz, nb=3, c0=0):
    T = _f32(T)
    ncols, nzz = T.shape
    rx, rz = _f32(rx), _f32(rz)
    out = np.zeros(len(rx), np.float32)
    lib().orc_picks_f32(T, nzz, ncols, c0, dx, dz, nb, rx, rz, len(rx), out)
    return out


def shot(S, dx, dz, sx, sz, rx=None, rz=None, nb=3, c0=0, ncols=None, ani=None, want_T=True):
    """Full shot as the C-ABI runs it. ani: (codes[6], mm[12]) or None.
    Returns (T or None, picks or None)."""
    S = _f32(S)
    nxx, nzz = S.shape
    ncols = nxx - c0 if ncols is None else ncols
    T = np.zeros((ncols, nzz), np.float32) if want_T else None
    nrec = 0 if rx is None else len(rx)
    pk = np.zeros(nrec, np.float32) if nrec else None
    if ani is not None:
        arr, keep = _codes_arg(ani[0])
        mm = _f32(ani[1])
    else:
        arr, keep = (C.c_void_p * 6)(), []
        mm = np.zeros(12, np.float32)
    rxa = _f32(rx if nrec else np.zeros(1))
    rza = _f32(rz if nrec else np.zeros(1))
    rc = lib().orc_shot_f32(nzz, nxx, nb, S, dx, dz, c0, ncols, sx, sz, 1 if ani is not None else 0,
                            arr, mm, T.ctypes.data if T is not None else None, rxa, rza, nrec,
                            pk.ctypes.data if pk is not None else None)
    if rc != 0:
        raise ValueError("source outside the window")
    return T, pk


def batch_picks(S, dx, dz, sx, sz, c0, ncols, rx, rz, nb=3, ani=None, nthreads=0):
    """CPU baseline: all shots, picks only. Returns (picks, threads_used)."""
    S = _f32(S)
    nxx, nzz = S.shape
    ns = len(sx)
    out = np.zeros((ns, len(rx)), np.float32)
    if ani is not None:
        arr, keep = _codes_arg(ani[0])
        mm = _f32(ani[1])
    else:
        arr, keep = (C.c_void_p * 6)(), []
        mm = np.zeros(12, np.float32)
    used = lib().orc_batch_f32(nzz, nxx, nb, S, dx, dz, ns, _f32(sx), _f32(sz),
                               np.ascontiguousarray(c0, np.int32),
                               np.ascontiguousarray(ncols, np.int32), 1 if ani is not None else 0,
                               arr, mm, _f32(rx), _f32(rz), len(rx), out, nthreads)
    return out, used


def batch_misfit_gradient(S, dx, dz, shots, rx, rz, t_obs, nb=3, nthreads=0, ani=None):
    """FP32 oracle of sf_batch_misfit_gradient, one shot per thread.
    shots: (sx, sz) or (sx, sz, c0, ncols). Returns (misfit, grad (nxx, nzz),
    picks (nshots, nrec), threads_used). ani: (codes[6], mm[12]) for the
    anisotropic two-pass scheme; then grad is dJ/dS and the return value has
    two more entries, dJ/dC11 and dJ/dC13 (nxx, nzz)."""
    S = _f32(S)
    nxx, nzz = S.shape
    ns = len(shots)
    sx = _f32([s[0] for s in shots])
    sz = _f32([s[1] for s in shots])
    c0 = np.array([int(s[2]) if len(s) > 2 else 0 for s in shots], np.int32)
    nc = np.array([int(s[3]) if len(s) > 3 and s[3] > 0 else nxx - int(c0[k]) for k, s in enumerate(shots)],
                  np.int32)
    picks = np.zeros((ns, len(rx)), np.float32)
    grad = np.zeros((nxx, nzz), np.float32)
    mis = C.c_double()
    g11 = np.zeros((nxx, nzz), np.float32)
    g13 = np.zeros((nxx, nzz), np.float32)
    if ani is not None:
        arr, keep = _codes_arg(ani[0])
        mm = _f32(ani[1])
    else:
        arr, keep = (C.c_void_p * 6)(), []
        mm = np.zeros(12, np.float32)
    used = lib().orc_batch_gradient_f32(nzz, nxx, nb, S, dx, dz, ns, sx, sz, c0, nc, _f32(rx), _f32(rz),
                                        len(rx), _f32(np.asarray(t_obs).reshape(ns, len(rx))), picks,
                                        C.byref(mis), grad, nthreads, 1 if ani is not None else 0, arr, mm,
                                        g11, g13)
    if used < 0:
        raise ValueError("a source lies outside its window")
    if ani is not None:
        return mis.value, grad, picks, used, g11, g13
    return mis.value, grad, picks, used


def smooth_kernel(stdv, samples):
    k = np.zeros(samples * samples, np.float32)
    lib().orc_smooth_kernel(stdv, samples, k)
    return k.reshape(samples, samples)  # [x, z]


def model_smoothing(model, stdv, samples):
    """The reference's model_smoothing of an (nx, nz) field."""
    m = _f32(model)
    out = np.zeros_like(m)
    lib().orc_model_smoothing(m, m.shape[0], m.shape[1], stdv, samples, out)
    return out


def update_slowness(S, grad, nx, nz, scale, stdv=0.0, samples=0, nb=3):
    """Tomography_ISO::model_update on a copy of the padded slowness S;
    returns (S_new, dS)."""
    Sn = _f32(S).copy()
    dS = np.zeros((nx, nz), np.float32)
    lib().orc_update_slowness(Sn, _f32(grad), nx, nz, nb, scale, stdv, samples, dS)
    return Sn, dS


def kirchhoff_wavelet(fmax, dt):
    w = np.zeros(1 << 16, np.float32)
    nw = lib().orc_kirchhoff_wavelet(fmax, dt, w, len(w))
    if nw < 0:
        raise ValueError("wavelet too long")
    return w[:nw].copy()


def adjoint_convolution(traces, dt, fmax):
    """Migration::adjoint_convolution of (ntr, nt) traces."""
    a = _f32(traces)
    w = kirchhoff_wavelet(fmax, dt)
    out = np.zeros_like(a)
    lib().orc_adjoint_convolution(a.ravel(), out.ravel(), a.shape[0], a.shape[1], w, len(w))
    return out


def kirchhoff_image(S, Ts, Tr, xsrc, xrec, data, dt, dx, dz, aperture, max_offset, nb=3):
    """Image-domain Kirchhoff migration; S (nxx, nzz), Ts (nsrc, nxx, nzz),
    Tr (nrec, nxx, nzz), data (nsrc, nrec, nt). Returns the (nx, nz) image."""
    S = _f32(S)
    nxx, nzz = S.shape
    img = np.zeros((nxx - 2 * nb, nzz - 2 * nb), np.float32)
    d = _f32(data)
    lib().orc_kirchhoff_image(nxx, nzz, nb, S, _f32(Ts).ravel(), _f32(Tr).ravel(), len(xsrc), len(xrec),
                              _f32(xsrc), _f32(xrec), d.ravel(), d.shape[-1], dt, dx, dz, aperture, max_offset,
                              img)
    return img


def forward_convolution(traces, dt, fmax):
    """Migration::forward_convolution of (ntr, nt) traces."""
    a = _f32(traces)
    w = kirchhoff_wavelet(fmax, dt)
    out = np.zeros_like(a)
    lib().orc_forward_convolution(a.ravel(), out.ravel(), a.shape[0], a.shape[1], w, len(w))
    return out


def angle_bins(xsrc, xrec, max_angle, da):
    """(nang, ncmp, min CMP, CMP spacing) of Migration::set_gathers
    (migration.cu:73-97), the largest CMP started from the first pair's."""
    f32 = np.float32
    xs, xr = _f32(xsrc), _f32(xrec)
    d = f32(0.5) * min(f32(xs[1] - xs[0]), f32(xr[1] - xr[0]))
    cmps = (f32(0.5) * (xs[:, None] + xr[None, :])).astype(np.float32)
    mn, mx = f32(min(f32(1e6), cmps.min())), f32(cmps.max())
    return int(f32(max_angle) / f32(da)) + 1, int(f32(mx - mn) / d) + 1, float(mn), float(d)


def kirchhoff_image_forward(S, Ts, Tr, xsrc, xrec, image, nt, dt, dx, dz, aperture, max_offset, nb=3):
    """Image-domain forward operator: image (nx, nz) -> traces (nsrc, nrec, nt),
    each sample's terms summed in FP64 and rounded once."""
    S = _f32(S)
    nxx, nzz = S.shape
    out = np.zeros((len(xsrc), len(xrec), int(nt)), np.float32)
    lib().orc_kirchhoff_forward(nxx, nzz, nb, S, _f32(Ts).ravel(), _f32(Tr).ravel(), len(xsrc), len(xrec),
                                _f32(xsrc), _f32(xrec), _f32(image).ravel(), int(nt), dt, dx, dz, aperture,
                                max_offset, 0, 1.0, 0.0, 1.0, out)
    return out


def kirchhoff_angle_forward(S, Ts, Tr, xsrc, xrec, gathers, nt, dt, dx, dz, aperture, max_offset, max_angle, da,
                            nb=3):
    """Angle-domain forward operator: gathers (ncmp, nang, nz) -> traces."""
    S = _f32(S)
    nxx, nzz = S.shape
    na, nc, mn, d = angle_bins(xsrc, xrec, max_angle, da)
    g = _f32(gathers)
    assert g.shape == (nc, na, nzz - 2 * nb), (g.shape, (nc, na, nzz - 2 * nb))
    out = np.zeros((len(xsrc), len(xrec), int(nt)), np.float32)
    lib().orc_kirchhoff_forward(nxx, nzz, nb, S, _f32(Ts).ravel(), _f32(Tr).ravel(), len(xsrc), len(xrec),
                                _f32(xsrc), _f32(xrec), g.ravel(), int(nt), dt, dx, dz, aperture, max_offset, na, da,
                                mn, d, out)
    return out


def solve_tape(S, dx, dz, sx, sz, nb=3, c0=0, ncols=None, fp64=False, follow=None):
    """Forward with tape. Returns (T, code, c1, c2, sIdz, sIdx_loc); tape arrays
    have shape (4, ncols, nzz). fp64 with follow (codes (4, ncols, nzz) of an
    FP32 tape): the FP64 solve takes those branches instead of its own."""
    S = _f32(S)
    nxx, nzz = S.shape
    ncols = nxx - c0 if ncols is None else ncols
    v, sIdx, sIdz = init_block(S, sx, sz, dx, dz, nb)
    Sw = np.ascontiguousarray(S[c0:c0 + ncols])
    code = np.zeros((4, ncols, nzz), np.uint8)
    if fp64 and follow is not None:
        code = np.ascontiguousarray(follow, np.uint8).reshape(4, ncols, nzz).copy()
        T = np.zeros((ncols, nzz), np.float64)
        c1 = np.zeros((4, ncols, nzz), np.float64)
        c2 = np.zeros_like(c1)
        lib().orc_solve_follow_f64(nzz, ncols, Sw, nzz, dx, dz, sIdz, sIdx - c0, v, code, T, c1, c2)
    elif fp64:
        T = np.zeros((ncols, nzz), np.float64)
        c1 = np.zeros((4, ncols, nzz), np.float64)
        c2 = np.zeros_like(c1)
        lib().orc_solve_tape_f64(nzz, ncols, Sw, nzz, dx, dz, sIdz, sIdx - c0, v, T, code, c1, c2)
    else:
        T = np.zeros((ncols, nzz), np.float32)
        c1 = np.zeros((4, ncols, nzz), np.float32)
        c2 = np.zeros_like(c1)
        init, _, _ = init_block_f32(S, sx, sz, dx, dz, nb)
        lib().orc_solve_tape_f32(nzz, ncols, Sw, nzz, dx, dz, sIdz, sIdx - c0, init, T, code, c1, c2)
    return T, code, c1, c2, sIdz, sIdx - c0


def init_dist(sx, sz, dx, dz, nb=3):
    sIdx, sIdz = source_index(sx, sz, dx, dz, nb)
    d = np.zeros(9)
    for b in range(3):
        for a in range(3):
            zi, xi = sIdz + a - 1, sIdx + b - 1
            ddx = float(xi - nb) * float(np.float32(dx)) - float(np.float32(sx))
            ddz = float(zi - nb) * float(np.float32(dz)) - float(np.float32(sz))
            d[a + 3 * b] = np.sqrt(ddx * ddx + ddz * ddz)
    return d


def adjoint(tape, lam, dist, fp64=False, grad=None):
    """Reverse sweeps. tape = (code, c1, c2, sIdz, sIdx_loc); lam: adjoint of the
    final T (ncols, nzz). Returns (grad, lam_init)."""
    code, c1, c2, sIdz, sloc = tape
    ncols, nzz = code.shape[1], code.shape[2]
    dt = np.float64 if fp64 else np.float32
    lam = np.ascontiguousarray(lam, dtype=dt).copy()
    g = np.zeros((ncols, nzz), dt) if grad is None else np.ascontiguousarray(grad, dtype=dt)
    fn = lib().orc_adjoint_f64 if fp64 else lib().orc_adjoint_f32
    fn(nzz, ncols, sIdz, sloc, np.ascontiguousarray(code), np.ascontiguousarray(c1, dt),
       np.ascontiguousarray(c2, dt), np.ascontiguousarray(dist, dt), lam, g)
    return g, lam


def pick_weights(x, z, dx, dz, nzz, ncols, nb=3, c0=0):
    """Returns (i, j_local, w[4,4]) or None; w[a, b] weights node (i-1+b, j-1+a)."""
    i, j = C.c_int(), C.c_int()
    w = np.zeros(16)
    rc = lib().orc_pick_weights_f64(x, z, dx, dz, nb, nzz, ncols, c0, C.byref(i), C.byref(j), w)
    if rc:
        return None
    return i.value, j.value, w.reshape(4, 4)


def seed_lambda(ncols, nzz, dx, dz, rx, rz, pg, c0=0, nb=3, fp64=False):
    """Adjoint seed of one shot window from its pick gradients (receivers in
    order, the engine's tap order and rounding)."""
    rx, rz = _f32(rx), _f32(rz)
    if fp64:
        lam = np.zeros((ncols, nzz), np.float64)
        lib().orc_seed_lambda_f64(nzz, ncols, c0, dx, dz, nb, rx, rz, len(rx),
                                  np.ascontiguousarray(pg, np.float64), lam)
    else:
        lam = np.zeros((ncols, nzz), np.float32)
        lib().orc_seed_lambda_f32(nzz, ncols, c0, dx, dz, nb, rx, rz, len(rx), _f32(pg), lam)
    return lam


def batch_gradient(S, dx, dz, shots, rx, rz, pick_grad, nb=3, fp64=False, follow=None):
    """Oracle of sf_batch_adjoint: per shot (window) tape + seed + reverse
    sweeps, shot gradients summed in FP64 in shot order onto the padded grid.
    Returns (grad (nxx, nzz), picks (nshots, nrec)). fp64 with follow (one
    code array (4, ncols, nzz) per shot, e.g. an FP32 engine's tape codes):
    the FP64 adjoint of the same branch pattern."""
    S = _f32(S)
    nxx, nzz = S.shape
    total = np.zeros((nxx, nzz), np.float64)
    picks_out = np.zeros((len(shots), len(rx)), np.float64 if fp64 else np.float32)
    for b, s in enumerate(shots):
        sx, sz = s[0], s[1]
        c0 = int(s[2]) if len(s) > 2 else 0
        nc = int(s[3]) if len(s) > 3 and s[3] > 0 else nxx - c0
        T, code, c1, c2, sIdz, sloc = solve_tape(S, dx, dz, sx, sz, nb, c0, nc, fp64=fp64,
                                                 follow=None if follow is None else follow[b])
        if fp64:
            pk = np.full(len(rx), np.nan)
            for r in range(len(rx)):
                pw = pick_weights(rx[r], rz[r], dx, dz, nzz, nc, nb, c0)
                if pw is not None:
                    i, j, w = pw
                    pk[r] = sum(w[a, bb] * T[j + a - 1, i + bb - 1] for a in range(4) for bb in range(4))
        else:
            pk = picks(T, dx, dz, rx, rz, nb, c0)
        picks_out[b] = pk
        lam = seed_lambda(nc, nzz, dx, dz, rx, rz, pick_grad[b], c0, nb, fp64)
        d = init_dist(sx, sz, dx, dz, nb)
        g, _ = adjoint((code, c1, c2, sIdz, sloc), lam, d, fp64=fp64)
        total[c0:c0 + nc] += g.astype(np.float64)
    return (total if fp64 else total.astype(np.float32)), picks_out


def picks_f64(T, dx, dz, rx, rz, nb=3, c0=0):
    """FP64 picks of an FP64 window field (ncols, nzz)."""
    T = np.ascontiguousarray(T, np.float64)
    ncols, nzz = T.shape
    out = np.zeros(len(rx), np.float64)
    lib().orc_picks_f64(T, nzz, ncols, c0, dx, dz, nb, _f32(rx), _f32(rz), len(rx), out)
    return out


def _shot_arrays(shots, nxx):
    sx = _f32([s[0] for s in shots])
    sz = _f32([s[1] for s in shots])
    c0 = np.array([int(s[2]) if len(s) > 2 else 0 for s in shots], np.int32)
    nc = np.array([int(s[3]) if len(s) > 3 and s[3] > 0 else nxx - int(c0[k]) for k, s in enumerate(shots)],
                  np.int32)
    return sx, sz, c0, nc


def misfit_f64(S, dx, dz, shots, rx, rz, t_obs, nb=3):
    """FP64 misfit 0.5 sum (p - t_obs)^2 of the FP64 1-pass solves (own branches)."""
    S = _f32(S)
    nxx, nzz = S.shape
    sx, sz, c0, nc = _shot_arrays(shots, nxx)
    tobs = np.ascontiguousarray(np.asarray(t_obs, np.float64).reshape(len(shots), len(rx)))
    return lib().orc_misfit_f64(nzz, nxx, nb, S, dx, dz, len(shots), sx, sz, c0, nc, _f32(rx), _f32(rz),
                                len(rx), tobs)


def fd_misfit_f64(S, dx, dz, shots, rx, rz, t_obs, cells, rel=1e-5, nb=3, nthreads=0):
    """Central finite differences of misfit_f64 on padded cells [(i, j), ...]
    (row i, column j): returns (dJ/dS per cell, (J+ - J-) values, threads)."""
    S = _f32(S)
    nxx, nzz = S.shape
    sx, sz, c0, nc = _shot_arrays(shots, nxx)
    tobs = np.ascontiguousarray(np.asarray(t_obs, np.float64).reshape(len(shots), len(rx)))
    ci = np.ascontiguousarray([c[0] for c in cells], np.int32)
    cj = np.ascontiguousarray([c[1] for c in cells], np.int32)
    n = len(cells)
    sp, sm = np.zeros(n, np.float32), np.zeros(n, np.float32)
    jp, jm = np.zeros(n), np.zeros(n)
    used = lib().orc_fd_misfit_f64(nzz, nxx, nb, S, dx, dz, len(shots), sx, sz, c0, nc, _f32(rx), _f32(rz),
                                   len(rx), tobs, n, ci, cj, rel, sp, sm, jp, jm, nthreads)
    d = (jp - jm) / (sp.astype(np.float64) - sm.astype(np.float64))
    return d, jp - jm, used


def shot_ani_f64(S, dx, dz, sx, sz, ani, nb=3, c0=0, ncols=None):
    """The two-pass anisotropic shot in FP64 (FP64 first solve, qP field and
    second solve); ani = (codes[6], mm[12]). Returns T (ncols, nzz) float64."""
    S = _f32(S)
    nxx, nzz = S.shape
    ncols = nxx - c0 if ncols is None else ncols
    arr, keep = _codes_arg(ani[0])
    T = np.zeros((ncols, nzz), np.float64)
    if lib().orc_shot_ani_f64(nzz, nxx, nb, S, dx, dz, c0, ncols, sx, sz, arr, _f32(ani[1]), T) != 0:
        raise ValueError("source outside the window")
    return T


def fp64_misfit_gradients(S, dx, dz, shots, rx, rz, t_obs, follow=None, nb=3):
    """FP64 adjoint-state gradients of the FP64 misfit 0.5 sum (p - t_obs)^2
    (p the FP64 picks) of a batch of shot windows, summed in shot order onto
    the padded grid (nxx, nzz): the FP64 solves take their own branches, or
    with follow (one code array (4, ncols, nzz) per shot, e.g. an FP32
    engine's sf_batch_tape_codes) the branches those codes name."""
    S = _f32(S)
    nxx, nzz = S.shape
    g = np.zeros((nxx, nzz))
    tobs = np.asarray(t_obs, np.float64).reshape(len(shots), len(rx))
    for b, s in enumerate(shots):
        c0 = int(s[2]) if len(s) > 2 else 0
        nc = int(s[3]) if len(s) > 3 and s[3] > 0 else nxx - c0
        T, code, c1, c2, sIdz, sloc = solve_tape(S, dx, dz, s[0], s[1], nb, c0, nc, fp64=True,
                                                 follow=None if follow is None else follow[b])
        p = picks_f64(T, dx, dz, rx, rz, nb, c0)
        lam = seed_lambda(nc, nzz, dx, dz, rx, rz, p - tobs[b], c0, nb, fp64=True)
        gb, _ = adjoint((code, c1, c2, sIdz, sloc), lam, init_dist(s[0], s[1], dx, dz, nb), fp64=True)
        g[c0:c0 + nc] += gb
    return g
