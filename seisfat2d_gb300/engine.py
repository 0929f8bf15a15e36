"""Python mirror of the engine's C ABI (used by the tests, the bench and the
autograd wrapper). Every call goes through ``libseisfat2d.so``.

Arrays use the reference layout: a padded field of ``nzz`` rows by ``nxx``
columns, z fastest, is a ``(nxx, nzz)`` array (``a[j, i]`` = row i, column j);
a model is ``(nx, nz)``. numpy arrays are host buffers, CUDA torch tensors are
device buffers.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import (SF_KEEP_TABLES, SF_KEEP_TAPE, SF_LAYOUT_MODEL, SF_LAYOUT_PADDED, SF_MEM_DEVICE,
                   SF_MEM_HOST, EngineError, sf_shot)

try:  # torch is optional for host-buffer use
    import torch
except Exception:  # pragma: no cover
    torch = None


def _is_dev(a):
    return torch is not None and isinstance(a, torch.Tensor) and a.is_cuda


def _ptr(a, dtype=np.float32):
    """(pointer, mem kind, keepalive) of a numpy array or torch tensor."""
    if _is_dev(a):
        if not a.is_contiguous():
            raise ValueError("device tensor must be contiguous")
        return C.c_void_p(a.data_ptr()), SF_MEM_DEVICE, a
    if torch is not None and isinstance(a, torch.Tensor):
        a = a.detach().numpy()
    arr = np.ascontiguousarray(a, dtype=dtype)
    return C.c_void_p(arr.ctypes.data), SF_MEM_HOST, arr


def _stream_ptr(stream):
    if stream is None:
        return None
    if torch is not None and isinstance(stream, torch.cuda.Stream):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


class Engine:
    """One padded model grid on one device (``sf_ctx``)."""

    def __init__(self, nx, nz, dx, dz, device=0):
        self.L = _lib.load()
        self._ctx = C.c_void_p()
        st = self.L.sf_ctx_create(C.byref(self._ctx), int(nx), int(nz), float(dx), float(dz),
                                  int(device))
        if st != 0:
            raise EngineError(st, "sf_ctx_create: " + self.L.sf_status_string(st).decode())
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        self.L.sf_ctx_dims(self._ctx, C.byref(a), C.byref(b), C.byref(c))
        self.nx, self.nz, self.dx, self.dz = int(nx), int(nz), float(dx), float(dz)
        self.nxx, self.nzz, self.nb = a.value, b.value, c.value
        self.device = device
        # the tape of the last taped batch: a counter that every call which
        # replaces or consumes the tape advances, and the batch's (shots,
        # receivers), so an adjoint can be checked against the forward it
        # differentiates
        self.tape_generation = 0
        self.tape_shape = None

    def _tape_changed(self, shape=None):
        self.tape_generation += 1
        self.tape_shape = shape

    def close(self):
        if self._ctx:
            self.L.sf_ctx_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        if st != 0:
            msg = self.L.sf_ctx_last_error(self._ctx)
            raise EngineError(st, f"{what}: {msg.decode() if msg else ''}")

    # -------------------------------------------------------------- models
    def set_slowness(self, s, padded=False):
        p, mem, keep = _ptr(s)
        self._check(self.L.sf_set_slowness(self._ctx, p, SF_LAYOUT_PADDED if padded else SF_LAYOUT_MODEL,
                                           mem), "sf_set_slowness")

    def get_slowness(self):
        out = np.zeros((self.nxx, self.nzz), np.float32)
        self._check(self.L.sf_get_slowness(self._ctx, C.c_void_p(out.ctypes.data), SF_MEM_HOST),
                    "sf_get_slowness")
        return out

    def set_stiffness(self, cij):
        arr = (C.c_void_p * 6)()
        keep = []
        mem = None
        for q in range(6):
            p, m, k = _ptr(cij[q])
            arr[q] = p.value
            keep.append(k)
            mem = m
        self._check(self.L.sf_set_stiffness(self._ctx, arr, mem), "sf_set_stiffness")

    def set_stiffness_codes(self, codes, minmax):
        arr = (C.c_void_p * 6)()
        keep = []
        for q in range(6):
            c = np.ascontiguousarray(codes[q], dtype=np.uint16)
            keep.append(c)
            arr[q] = c.ctypes.data
        mm = np.ascontiguousarray(minmax, dtype=np.float32)
        self._check(self.L.sf_set_stiffness_codes(self._ctx, arr, C.c_void_p(mm.ctypes.data),
                                                  SF_MEM_HOST), "sf_set_stiffness_codes")

    # -------------------------------------------------------------- per shot
    def time_propagation(self, sx, sz, ani=False, out=None, stream=None):
        """One shot on the whole grid; returns (nxx, nzz) traveltimes."""
        if out is None:
            out = np.zeros((self.nxx, self.nzz), np.float32)
        p, mem, keep = _ptr(out)
        self._tape_changed()
        self._check(self.L.sf_time_propagation(self._ctx, 1 if ani else 0, float(sx), float(sz), p, mem,
                                               _stream_ptr(stream)), "sf_time_propagation")
        return out

    def compute_seismogram(self, T_dev, rx, rz, out=None, stream=None):
        rx = np.ascontiguousarray(rx, np.float32)
        rz = np.ascontiguousarray(rz, np.float32)
        if out is None:
            out = np.zeros(len(rx), np.float32)
        p, mem, keep = _ptr(out)
        self._check(self.L.sf_compute_seismogram(self._ctx, C.c_void_p(T_dev.data_ptr()),
                                                 C.c_void_p(rx.ctypes.data), C.c_void_p(rz.ctypes.data),
                                                 len(rx), p, mem, _stream_ptr(stream)),
                    "sf_compute_seismogram")
        return out

    # -------------------------------------------------------------- batches
    @staticmethod
    def shot_table(shots):
        """shots: iterable of (sx, sz) or (sx, sz, c0, ncols)."""
        shots = list(shots)
        arr = (sf_shot * len(shots))()
        for k, s in enumerate(shots):
            sx, sz = float(s[0]), float(s[1])
            c0 = int(s[2]) if len(s) > 2 else 0
            nc = int(s[3]) if len(s) > 3 else 0
            arr[k] = sf_shot(sx, sz, c0, nc)
        return arr

    def batch_forward(self, shots, rx, rz, ani=False, keep_tape=False, keep_tables=False, out=None,
                      stream=None):
        """All shots in one persistent launch; returns picks (nshots, nrec)."""
        tab = shots if isinstance(shots, C.Array) else self.shot_table(shots)
        rx = np.ascontiguousarray(rx, np.float32)
        rz = np.ascontiguousarray(rz, np.float32)
        ns, nr = len(tab), len(rx)
        if out is None:
            out = np.zeros((ns, nr), np.float32)
        p, mem, keep = _ptr(out)
        flags = (SF_KEEP_TAPE if keep_tape else 0) | (SF_KEEP_TABLES if keep_tables else 0)
        self._tape_changed((ns, nr) if keep_tape else None)
        self._check(self.L.sf_batch_forward(self._ctx, 1 if ani else 0, tab, ns,
                                            C.c_void_p(rx.ctypes.data), C.c_void_p(rz.ctypes.data), nr,
                                            p, mem, flags, _stream_ptr(stream)), "sf_batch_forward")
        return out

    def batch_table(self, shot, ncols, out=None, stream=None):
        if out is None:
            out = np.zeros((ncols, self.nzz), np.float32)
        p, mem, keep = _ptr(out)
        self._check(self.L.sf_batch_table(self._ctx, int(shot), p, mem, _stream_ptr(stream)),
                    "sf_batch_table")
        return out

    def _check_adjoint_args(self, per_shot, out, what):
        """The C ABI cannot see buffer sizes: check them against the taped
        batch (without one the C call reports SF_ERR_STATE)."""
        if self.tape_shape is None:
            return
        n = int(np.prod(per_shot.shape)) if hasattr(per_shot, "shape") else len(per_shot)
        if n != self.tape_shape[0] * self.tape_shape[1]:
            raise ValueError(f"{what}: {n} values for a taped batch of {self.tape_shape[0]} shots x "
                             f"{self.tape_shape[1]} receivers")
        if out is not None and tuple(out.shape) != (self.nxx, self.nzz):
            raise ValueError(f"{what}: output of shape {tuple(out.shape)}, expected {(self.nxx, self.nzz)}")

    def batch_adjoint(self, pick_grad, out=None, stream=None):
        self._check_adjoint_args(pick_grad, out, "batch_adjoint")
        if out is None:
            out = np.zeros((self.nxx, self.nzz), np.float32)
        pg, pmem, k1 = _ptr(pick_grad)
        p, mem, k2 = _ptr(out)
        self._tape_changed()  # the reverse sweeps consume the tape
        self._check(self.L.sf_batch_adjoint(self._ctx, pg, pmem, p, mem, _stream_ptr(stream)),
                    "sf_batch_adjoint")
        return out

    def tape_codes(self, shot, ncols, stream=None):
        """Branch codes (4, ncols, nzz) of one shot of the last taped batch:
        [sweep, window column, row], the oracle's tape layout."""
        out = np.zeros((4, ncols, self.nzz), np.uint8)
        self._check(self.L.sf_batch_tape_codes(self._ctx, int(shot), C.c_void_p(out.ctypes.data), SF_MEM_HOST,
                                               _stream_ptr(stream)), "sf_batch_tape_codes")
        return out

    def stiffness_gradient(self, stream=None):
        """dJ/dC11 and dJ/dC13 (each (nxx, nzz)) of the last adjoint of an
        anisotropic taped batch."""
        g11 = np.zeros((self.nxx, self.nzz), np.float32)
        g13 = np.zeros_like(g11)
        self._check(self.L.sf_batch_stiffness_gradient(self._ctx, C.c_void_p(g11.ctypes.data),
                                                       C.c_void_p(g13.ctypes.data), SF_MEM_HOST,
                                                       _stream_ptr(stream)), "sf_batch_stiffness_gradient")
        return g11, g13

    def misfit_gradient(self, t_obs, out=None, stream=None, want_misfit=True):
        """Misfit 1/2 sum (pick - t_obs)^2 of the taped batch and its slowness
        gradient (padded (nxx, nzz)). With want_misfit False and a device
        ``out`` the call only enqueues work on ``stream`` (misfit is None)."""
        self._check_adjoint_args(t_obs, out, "misfit_gradient")
        if out is None:
            out = np.zeros((self.nxx, self.nzz), np.float32)
        po, omem, k1 = _ptr(t_obs)
        p, mem, k2 = _ptr(out)
        mis = C.c_double()
        self._tape_changed()  # the reverse sweeps consume the tape
        self._check(self.L.sf_batch_misfit_gradient(self._ctx, po, omem, C.byref(mis) if want_misfit else None,
                                                    p, mem, _stream_ptr(stream)), "sf_batch_misfit_gradient")
        return (mis.value if want_misfit else None), out

    # ------------------------------------------------------- model update
    def smooth_model(self, field, stdv, samples, out=None, stream=None):
        """The reference's Gaussian model smoothing of an (nx, nz) field."""
        if out is None:
            out = np.zeros((self.nx, self.nz), np.float32)
        pi, mem, k1 = _ptr(field)
        po, _, k2 = _ptr(out)
        self._check(self.L.sf_smooth_model(self._ctx, pi, po, float(stdv), int(samples), mem, _stream_ptr(stream)),
                    "sf_smooth_model")
        return out

    def update_slowness(self, grad, scale, stdv=0.0, samples=0, want_dS=True, stream=None):
        """S += smooth(scale * grad) on the model interior; returns dS (nx, nz)."""
        pg, gmem, k1 = _ptr(grad)
        dS = np.zeros((self.nx, self.nz), np.float32) if want_dS else None
        pd = C.c_void_p(dS.ctypes.data) if want_dS else None
        self._check(self.L.sf_update_slowness(self._ctx, pg, gmem, float(scale), float(stdv), int(samples), pd,
                                              0, _stream_ptr(stream)), "sf_update_slowness")
        return dS

    # ----------------------------------------------------------- migration
    def adjoint_convolution(self, traces, dt, fmax, out=None, stream=None):
        """The reference's wavelet cross-correlation of (ntr, nt) traces."""
        pi, mem, k1 = _ptr(traces)
        shape = tuple(traces.shape)
        if out is None:
            out = np.zeros(shape, np.float32)
        po, _, k2 = _ptr(out)
        self._check(self.L.sf_adjoint_convolution(self._ctx, pi, po, int(shape[0]), int(shape[1]), float(dt),
                                                  float(fmax), mem, _stream_ptr(stream)), "sf_adjoint_convolution")
        return out

    def kirchhoff_image(self, Ts, Tr, xsrc, xrec, data, dt, aperture, max_offset, out=None, stream=None):
        """Image-domain Kirchhoff migration. Ts (nsrc, nxx, nzz) and Tr
        (nrec, nxx, nzz) are CUDA tensors of padded tables; data (nsrc, nrec,
        nt) correlated traces; returns the (nx, nz) image."""
        xs = np.ascontiguousarray(xsrc, np.float32)
        xr = np.ascontiguousarray(xrec, np.float32)
        pts = self._dev_ptr(Ts, "Ts")
        ptr = self._dev_ptr(Tr, "Tr")
        pd, dmem, k1 = _ptr(data)
        if out is None:
            out = np.zeros((self.nx, self.nz), np.float32)
        po, omem, k2 = _ptr(out)
        nt = int(data.shape[-1])
        self._check(self.L.sf_kirchhoff_image(self._ctx, pts, ptr, len(xs), len(xr), C.c_void_p(xs.ctypes.data),
                                              C.c_void_p(xr.ctypes.data), pd, dmem, nt, float(dt), float(aperture),
                                              float(max_offset), po, omem, _stream_ptr(stream)),
                    "sf_kirchhoff_image")
        return out

    def kirchhoff_angle_gathers(self, Ts, Tr, xsrc, xrec, data, dt, aperture, max_offset, max_angle, da,
                                stream=None):
        """Angle-domain Kirchhoff migration; returns gathers (ncmp, nang, nz)."""
        xs = np.ascontiguousarray(xsrc, np.float32)
        xr = np.ascontiguousarray(xrec, np.float32)
        na, nc = C.c_int(), C.c_int()
        args = (C.c_void_p(xs.ctypes.data), C.c_void_p(xr.ctypes.data))
        self._check(self.L.sf_kirchhoff_angle_gathers(self._ctx, None, None, len(xs), len(xr), *args, None, 0, 1,
                                                      1.0, float(aperture), float(max_offset), float(max_angle),
                                                      float(da), None, 0, C.byref(na), C.byref(nc), None),
                    "sf_kirchhoff_angle_gathers")
        out = np.zeros((nc.value, na.value, self.nz), np.float32)
        pd, dmem, k1 = _ptr(data)
        self._check(self.L.sf_kirchhoff_angle_gathers(self._ctx, self._dev_ptr(Ts, "Ts"), self._dev_ptr(Tr, "Tr"),
                                                      len(xs), len(xr), *args, pd, dmem, int(data.shape[-1]),
                                                      float(dt), float(aperture), float(max_offset),
                                                      float(max_angle), float(da), C.c_void_p(out.ctypes.data), 0,
                                                      None, None, _stream_ptr(stream)),
                    "sf_kirchhoff_angle_gathers")
        return out

    def forward_convolution(self, traces, dt, fmax, out=None, stream=None):
        """The reference's wavelet convolution (Migration::forward_convolution)
        of (ntr, nt) traces."""
        pi, mem, k1 = _ptr(traces)
        shape = tuple(traces.shape)
        if out is None:
            out = np.zeros(shape, np.float32)
        po, _, k2 = _ptr(out)
        self._check(self.L.sf_forward_convolution(self._ctx, pi, po, int(shape[0]), int(shape[1]), float(dt),
                                                  float(fmax), mem, _stream_ptr(stream)), "sf_forward_convolution")
        return out

    def kirchhoff_image_forward(self, Ts, Tr, xsrc, xrec, image, nt, dt, aperture, max_offset, out=None,
                                stream=None):
        """Image-domain Kirchhoff forward operator (the least-squares
        variant's demigration): image (nx, nz) -> traces (nsrc, nrec, nt)."""
        xs = np.ascontiguousarray(xsrc, np.float32)
        xr = np.ascontiguousarray(xrec, np.float32)
        pm, mmem, k1 = _ptr(image)
        if out is None:
            out = np.zeros((len(xs), len(xr), int(nt)), np.float32)
        po, omem, k2 = _ptr(out)
        self._check(self.L.sf_kirchhoff_image_forward(self._ctx, self._dev_ptr(Ts, "Ts"), self._dev_ptr(Tr, "Tr"),
                                                      len(xs), len(xr), C.c_void_p(xs.ctypes.data),
                                                      C.c_void_p(xr.ctypes.data), pm, mmem, int(nt), float(dt),
                                                      float(aperture), float(max_offset), po, omem,
                                                      _stream_ptr(stream)),
                    "sf_kirchhoff_image_forward")
        return out

    def kirchhoff_angle_forward(self, Ts, Tr, xsrc, xrec, gathers, nt, dt, aperture, max_offset, max_angle, da,
                                out=None, stream=None):
        """Angle-domain Kirchhoff forward operator: gathers (ncmp, nang, nz)
        -> traces (nsrc, nrec, nt)."""
        xs = np.ascontiguousarray(xsrc, np.float32)
        xr = np.ascontiguousarray(xrec, np.float32)
        pm, mmem, k1 = _ptr(gathers)
        if out is None:
            out = np.zeros((len(xs), len(xr), int(nt)), np.float32)
        po, omem, k2 = _ptr(out)
        self._check(self.L.sf_kirchhoff_angle_forward(self._ctx, self._dev_ptr(Ts, "Ts"), self._dev_ptr(Tr, "Tr"),
                                                      len(xs), len(xr), C.c_void_p(xs.ctypes.data),
                                                      C.c_void_p(xr.ctypes.data), pm, mmem, int(nt), float(dt),
                                                      float(aperture), float(max_offset), float(max_angle),
                                                      float(da), po, omem, _stream_ptr(stream)),
                    "sf_kirchhoff_angle_forward")
        return out

    # -------------------------------------------------------- planned batches
    def plan_batch(self, shots, rx, rz, stream=None):
        """Fix an isotropic batch (shots as for batch_forward) for
        plan_iteration / plan_graph_launch / plan_autotune."""
        tab = shots if isinstance(shots, C.Array) else self.shot_table(shots)
        rx = np.ascontiguousarray(rx, np.float32)
        rz = np.ascontiguousarray(rz, np.float32)
        self._check(self.L.sf_plan_batch(self._ctx, tab, len(tab), C.c_void_p(rx.ctypes.data),
                                         C.c_void_p(rz.ctypes.data), len(rx), _stream_ptr(stream)),
                    "sf_plan_batch")
        self._plan = (len(tab), len(rx))

    @staticmethod
    def _dev_ptr(t, what):
        if t is None:
            return None
        if not _is_dev(t) or not t.is_contiguous():
            raise ValueError(f"{what} must be a contiguous CUDA tensor")
        return C.c_void_p(t.data_ptr())

    def _plan_args(self, t_obs, picks, misfit, grad):
        return (self._dev_ptr(t_obs, "t_obs"), self._dev_ptr(picks, "picks"), self._dev_ptr(misfit, "misfit"),
                self._dev_ptr(grad, "grad"))

    def plan_iteration(self, picks, t_obs=None, grad=None, misfit=None, stream=None):
        """Enqueue one iteration of the planned batch (device tensors only):
        picks (nshots, nrec) f32; with t_obs, grad (nxx, nzz) f32 and
        optionally misfit (1,) f64."""
        a = self._plan_args(t_obs, picks, misfit, grad)
        self._tape_changed(self._plan if t_obs is None else None)  # with t_obs the tape is consumed
        self._check(self.L.sf_plan_iteration(self._ctx, *a, _stream_ptr(stream)), "sf_plan_iteration")

    def plan_graph_launch(self, picks, t_obs=None, grad=None, misfit=None, stream=None):
        """The same iteration replayed from the context's CUDA graph."""
        a = self._plan_args(t_obs, picks, misfit, grad)
        self._tape_changed(self._plan if t_obs is None else None)
        self._check(self.L.sf_plan_graph_launch(self._ctx, *a, _stream_ptr(stream)), "sf_plan_graph_launch")

    def plan_autotune(self, picks, t_obs=None, grad=None, misfit=None, reps=3, stream=None):
        """Pick the fastest launch shape for the planned batch; returns
        (warps_per_cta, gang_warps, ms_per_iteration)."""
        a = self._plan_args(t_obs, picks, misfit, grad)
        w, g, ms = C.c_int(), C.c_int(), C.c_float()
        self._tape_changed(self._plan if t_obs is None else None)
        self._check(self.L.sf_plan_autotune(self._ctx, *a, int(reps), _stream_ptr(stream), C.byref(w), C.byref(g),
                                            C.byref(ms)), "sf_plan_autotune")
        return w.value, g.value, ms.value

    # ------------------------------------------------------------ timing
    KERNELS = ("forward", "residual", "adjoint", "gather")

    def set_kernel_timing(self, enable=True):
        self._check(self.L.sf_set_kernel_timing(self._ctx, 1 if enable else 0), "sf_set_kernel_timing")

    def kernel_times(self):
        """{kernel: ms} of the latest launch of each batched kernel since the
        previous query (kernels not launched are left out)."""
        ms = (C.c_float * 4)()
        self._check(self.L.sf_kernel_times(self._ctx, ms, 4), "sf_kernel_times")
        return {k: float(v) for k, v in zip(self.KERNELS, ms) if v >= 0.0}

    def synchronize(self, stream=None):
        self._check(self.L.sf_synchronize(self._ctx, _stream_ptr(stream)), "sf_synchronize")

    def set_wait_limit(self, seconds):
        """Time limit of the in-kernel waits (0: the default, about 2 s)."""
        self._check(self.L.sf_set_wait_limit(self._ctx, float(seconds)), "sf_set_wait_limit")

    def test_stall_next_batch(self):
        """Test of the timeout path: the next forward launch's strips wait for
        a handoff tag nothing writes (sf_test_stall_next_batch)."""
        self._check(self.L.sf_test_stall_next_batch(self._ctx), "sf_test_stall_next_batch")

    ARITHMETICS = {"reference": _lib.SF_ARITH_REFERENCE, "ieee": _lib.SF_ARITH_IEEE,
                   "compensated": _lib.SF_ARITH_COMPENSATED}

    def set_arithmetic(self, mode):
        """'reference' (the reference build's FP32 arithmetic), 'ieee' (every
        operation rounded once) or 'compensated' (traveltimes carried as FP32
        pairs; see sf_set_arithmetic)."""
        self._check(self.L.sf_set_arithmetic(self._ctx, self.ARITHMETICS[mode]), "sf_set_arithmetic")

    def get_arithmetic(self):
        v = C.c_int()
        self.L.sf_get_arithmetic(self._ctx, C.byref(v))
        return {m: k for k, m in self.ARITHMETICS.items()}[v.value]

    def set_launch(self, warps=0, gang_warps=0):
        """warps per CTA (0 keeps it) and warps per shot (0: automatic)."""
        self._check(self.L.sf_set_launch(self._ctx, int(warps), int(gang_warps)), "sf_set_launch")

    def set_strip_loop(self, mode):
        """'auto', 'general' or 'interior' (sf_set_strip_loop)."""
        m = {"auto": -1, "general": 0, "interior": 1}[mode]
        self._check(self.L.sf_set_strip_loop(self._ctx, m), "sf_set_strip_loop")

    def set_fused_gather(self, enable):
        self._check(self.L.sf_set_fused_gather(self._ctx, 1 if enable else 0), "sf_set_fused_gather")

    def fused_gather(self):
        """(enabled, whether the last adjoint ran the gather inside its launch)."""
        e, last = C.c_int(), C.c_int()
        self._check(self.L.sf_get_fused_gather(self._ctx, C.byref(e), C.byref(last)), "sf_get_fused_gather")
        return bool(e.value), bool(last.value)

    def strip_loop(self):
        """(mode, whether the last batch ran the interior-block form)."""
        m, last = C.c_int(), C.c_int()
        self._check(self.L.sf_get_strip_loop(self._ctx, C.byref(m), C.byref(last)), "sf_get_strip_loop")
        return {-1: "auto", 0: "general", 1: "interior"}[m.value], bool(last.value)

    def get_launch(self):
        a, b = C.c_int(), C.c_int()
        self.L.sf_get_launch(self._ctx, C.byref(a), C.byref(b))
        return a.value, b.value
