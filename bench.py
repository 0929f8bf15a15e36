"""Benchmark of the batched eikonal engine on one GB300 (or N, one process per
GPU under torchrun, shots sharded across ranks).

Default workload (forward + adjoint): 100 surface shots on the 1701 x 351
(1707 x 357 padded) synthetic faulted layered model at 10 m, 400 receivers.
A step is one tomography iteration of the batch: the taped forward of every
shot with its 400 picks in one persistent launch, the pick residuals against
observed picks and the FP64 misfit, the reverse (adjoint) sweeps of every
shot in one persistent launch and the deterministic gather of the slowness
gradient. ``--config 2`` / ``--config 3`` time the forward batch alone (200
isotropic shots on 2001 x 501; 100 VTI shots on 1601 x 401). Prints ONE JSON
line (rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config 2|3|4|5]
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "eikonal+adjoint shots/s batched vs plain at \u22641e-5 rel err; HBM GB/s"
UNIT = "shots/s"
# algorithmic bytes per padded window cell and shot
BYTES_PER_CELL_FWD = 48       # 4 sweeps x (S 4 B + T read 4 B + T write 4 B)
BYTES_PER_CELL_FWD_ANI = 120  # 2 x 48 + qP pass (6 x 2 B Cij + T 4 B + S 4 B + S 4 B)
BYTES_PER_CELL_ADJ = 56       # 4 sweeps x (T 4 B + lam read 4 B + lam write 4 B) + S 4 B + g 4 B
FA_CONFIGS = (4, 5)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=4)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--warps", type=int, default=0, help="warps per CTA (0: engine default)")
    ap.add_argument("--gang", type=int, default=0, help="warps per shot (0: automatic)")
    ap.add_argument("--no-fused-gather", action="store_true", help="gather in its own launch")
    ap.add_argument("--strip-loop", default="auto", choices=["auto", "general", "interior"],
                    help="strip-loop form (fixing it, or --warps/--gang, skips the autotuner)")
    ap.add_argument("--arith", default="compensated", choices=["reference", "ieee", "compensated"],
                    help="arithmetic of the timed step (the reference build's arithmetic is measured beside it)")
    ap.add_argument("--no-checks", action="store_true",
                    help="skip the checker legs (accuracy against the FP64 oracle, the reference's GPU solver)")
    ap.add_argument("--no-configs", action="store_true", help="time the --config workload only")
    ap.add_argument("--config-steps", type=int, default=5, help="timed steps of the other workloads")
    ap.add_argument("--config-warmup", type=int, default=3, help="warm-up steps of the other workloads")
    ap.add_argument("--nplain", type=int, default=8, help="shots timed one at a time for the plain solver")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """Samples nvidia-smi during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.out = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, n in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def workload(cfg):
    from seisfat2d_gb300 import synthetic
    return synthetic.CONFIGS[cfg]()


def workload_ids():
    from seisfat2d_gb300 import synthetic
    return list(synthetic.CONFIGS)


def window(s, nxx):
    c0 = int(s[2]) if len(s) > 2 else 0
    nc = int(s[3]) if len(s) > 3 and s[3] > 0 else nxx - c0
    return c0, nc


def load_traffic(name):
    """DRAM bytes per padded window cell and shot of one kernel, from its
    committed ncu summary under profiles/ (None when absent)."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_cell_shot:"):
            return float(line.split(":")[1])
    return None


class CpuPort:
    """The oracle's FP32 restatement of the reference schedule (and, for the
    forward+adjoint workload, its taped reverse sweeps) on the host cores,
    one shot per thread."""

    def __init__(self, w, fa):
        from oracle import oracle as O
        self.O, self.w, self.fa = O, w, fa
        self.S = O.expand_boundary(w.slowness)
        self.nxx = self.S.shape[0]
        self.ani = None
        if w.cij is not None:
            codes, mm = [], []
            for c in w.cij:
                cd, mn, mx = O.compress(O.expand_boundary(c))
                codes.append(cd)
                mm += [mn, mx]
            self.ani = (codes, np.array(mm, np.float32))
        self.nthreads = os.cpu_count() or 1
        # the observed picks of the GPU arm (FP64 oracle on the true model + noise)
        self.obs = fp64_observed(w, range(len(w.shots))) if fa else None

    def run(self, idx, nthreads):
        O, w = self.O, self.w
        sel = [w.shots[k] for k in idx]
        if self.fa:
            _, _, _, used = O.batch_misfit_gradient(self.S, w.dx, w.dz, sel, w.rx, w.rz, self.obs[list(idx)],
                                                    nthreads=nthreads)
            return used
        c0 = [window(s, self.nxx)[0] for s in sel]
        nc = [window(s, self.nxx)[1] for s in sel]
        _, used = O.batch_picks(self.S, w.dx, w.dz, [s[0] for s in sel], [s[1] for s in sel], c0, nc,
                                w.rx, w.rz, ani=self.ani, nthreads=nthreads)
        return used

    def calibrate(self, seconds):
        """Shots per sample so that one sample takes about `seconds` on all
        threads (at least one shot per thread, at most the whole batch)."""
        shots = self.w.shots
        t0 = time.perf_counter()
        self.run([len(shots) // 2], 1)
        one = time.perf_counter() - t0
        n = int(seconds * self.nthreads / max(one, 1e-3))
        n = max(self.nthreads, (n // self.nthreads) * self.nthreads)
        return min(n, 50 * len(shots)), one

    def sample(self, n, k=0):
        """Indices of n shots spread over the batch (the batch repeated when n exceeds it)."""
        ns = len(self.w.shots)
        if n <= ns:
            return [(q * ns // n + k) % ns for q in range(n)]
        return [(q + k) % ns for q in range(n)]

    def describe(self, n, dt):
        what = ("taped forward + picks + residuals + reverse sweeps + FP64 gradient sum" if self.fa
                else "forward + picks")
        return (f"{n} shots of {self.w.name} ({len(self.w.shots)} in the batch) per sample, one shot per thread, "
                f"{what}, {dt:.1f} s timed; oracle FP32 restatement of the reference schedule "
                f"(gcc -O3 -fopenmp)")


def cpu_baseline(w, seconds, fa):
    port = CpuPort(w, fa)
    n, one = port.calibrate(seconds)
    sel = port.sample(n)
    t0 = time.perf_counter()
    used = port.run(sel, port.nthreads)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": used, "kind": "port", "sample": port.describe(n, dt),
            "single_thread_ms_per_shot": 1e3 * one}


def run_reference(a):
    """The reference has no CPU eikonal path and no adjoint; this arm times the
    oracle's FP32 restatement of its schedule (plus the taped adjoint for the
    forward+adjoint workload) on all host cores, each step a bounded sample of
    the same workload."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    w = workload(a.config)
    fa = a.config in FA_CONFIGS
    port = CpuPort(w, fa)
    n, one = port.calibrate(a.cpu_seconds / max(1, a.steps))
    for k in range(a.warmup):
        port.run(port.sample(n, k), port.nthreads)
    done, tot, used = 0, 0.0, 1
    for k in range(a.steps):
        sel = port.sample(n, a.warmup + k)
        t0 = time.perf_counter()
        used = port.run(sel, port.nthreads)
        tot += time.perf_counter() - t0
        done += len(sel)
    v = done / tot
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * tot / max(1, a.steps),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": {"workload": w.name, "nshots": len(w.shots), "nrec": len(w.rx), "grid": [w.nx, w.nz],
                       "dh": w.dx, "step": "forward+adjoint" if fa else "forward"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": used, "kind": "port",
                             "sample": port.describe(n, tot), "single_thread_ms_per_shot": 1e3 * one},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference has no CPU eikonal path and no adjoint; this arm times the oracle's "
                    "FP32 restatement of its schedule on the host cores"}
    print(json.dumps(line), flush=True)


def fp64_observed(w, idx):
    """Observed picks of shots `idx` of a forward+adjoint workload: the FP64
    oracle's picks on the true model (1-pass FP64 solve, FP64 Catmull-Rom
    weights) plus N(0, sigma) noise seeded per shot, so any subset of the
    shots gets the same values. Synthetic input, made outside every timed
    region on the host cores (NaN where a receiver leaves the shot's window)."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import oracle as O
    St = O.expand_boundary(w.extra["true_slowness"])
    nxx = St.shape[0]

    def one(k):
        s = w.shots[k]
        c0, nc = window(s, nxx)
        T, _ = O.solve_f64(St, w.dx, w.dz, s[0], s[1], c0=c0, ncols=nc)
        p = O.picks_f64(T, w.dx, w.dz, w.rx, w.rz, c0=c0)
        return p + np.random.default_rng(w.seed * 100003 + k).normal(0.0, w.extra["noise_sigma"], p.shape)

    with ThreadPoolExecutor(max(1, os.cpu_count() or 1)) as ex:
        return np.array(list(ex.map(one, idx)), np.float32).reshape(len(idx), len(w.rx))


def stiffness_codes(w):
    from oracle import oracle as O
    codes, mm = [], []
    for c in w.cij:
        cd, mn, mx = O.compress(O.expand_boundary(c))
        codes.append(cd)
        mm += [mn, mx]
    return codes, np.array(mm, np.float32)


def accuracy_checks(eng, w, fa, ani):
    """The checker leg (after every timed region): traveltimes of two shots
    of the batch (the first and the middle one, on their windows) against the
    FP64 oracle on the same 1-pass schedule, and for forward+adjoint
    workloads their misfit gradient against the FP64 adjoint with branches of
    its own and the FP64 adjoint that follows the engine's branch codes."""
    from oracle import oracle as O
    nxx, nzz = eng.nxx, eng.nzz
    idx = [0, len(w.shots) // 2]
    shots = [w.shots[k] for k in idx]
    S = O.expand_boundary(w.slowness)
    anic = stiffness_codes(w) if ani else None
    none = np.zeros(0, np.float32)
    eng.batch_forward(shots, none, none, ani=ani, keep_tables=True)
    errs = []
    for k, s in enumerate(shots):
        c0, nc = window(s, nxx)
        T32 = eng.batch_table(k, nc).astype(np.float64)
        T64 = (O.shot_ani_f64(S, w.dx, w.dz, s[0], s[1], anic, c0=c0, ncols=nc) if ani
               else O.solve_f64(S, w.dx, w.dz, s[0], s[1], c0=c0, ncols=nc)[0])
        inner = T64[3:nc - 3, 3:nzz - 3]
        m = inner > 0
        errs.append((np.abs(T32[3:nc - 3, 3:nzz - 3] - inner) / np.where(m, inner, 1.0))[m])
    e = np.concatenate(errs)
    out = {"checker": "FP64 oracle, same 1-pass schedule" + (" (FP64 qP pass)" if ani else ""),
           "shots": idx, "arithmetic": eng.get_arithmetic(),
           "traveltime": {"max_rel": float(e.max()), "rms_rel": float(np.sqrt(np.mean(e * e))),
                          "nodes": int(e.size), "bar": 1e-5}}
    if fa:
        tobs = fp64_observed(w, idx)
        eng.batch_forward(shots, w.rx, w.rz, keep_tape=True)
        codes = [eng.tape_codes(b, window(s, nxx)[1]) for b, s in enumerate(shots)]
        _, g32 = eng.misfit_gradient(tobs)
        g32 = g32.astype(np.float64)
        t64 = tobs.astype(np.float64)
        g64 = O.fp64_misfit_gradients(S, w.dx, w.dz, shots, w.rx, w.rz, t64)
        gsb = O.fp64_misfit_gradients(S, w.dx, w.dz, shots, w.rx, w.rz, t64, follow=codes)
        rl = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
        out["gradient"] = {"rel_l2_vs_fp64": rl(g32, g64), "rel_l2_vs_fp64_same_branches": rl(g32, gsb),
                           "fp64_adjoints_differ_by": rl(gsb, g64), "bar": 1e-3,
                           "note": "same-branch: the FP64 adjoint evaluated on the engine's own branch codes "
                                   "(sf_batch_tape_codes)"}
    return out


def reference_gpu(w, nshots):
    """The reference's own per-shot GPU solver on this workload's grid: its
    kernels compiled for sm_103a from its sources, its host launch loop
    (modeling.cu:123-159, 4 x (nxx+nzz-2) launches per solve; the two-pass
    anisotropic solve for VTI) replayed by a driver-API harness; CUDA events
    around one time_propagation per shot, outside every timed region."""
    try:
        from oracle import oracle as O
        from oracle import refkernels
        if not refkernels.available():
            return {"unavailable": "reference cubins were not built (the reference sources are absent)"}
        S = O.expand_boundary(w.slowness)
        anic = stiffness_codes(w) if w.cij is not None else None
        sel = [w.shots[k * len(w.shots) // nshots] for k in range(nshots)]
        refkernels.solve(S, w.dx, w.dz, sel[0][0], sel[0][1], ani=anic)  # warm-up (module load)
        ms = [refkernels.solve(S, w.dx, w.dz, s[0], s[1], ani=anic)[1] for s in sel]
        mean = statistics.mean(ms)
        return {"kind": "reference kernels, sm_103a, launch loop replayed", "ms_per_shot": mean,
                "shots_per_s": 1e3 / mean, "shots_timed": nshots, "grid_padded": list(S.shape),
                "solve": "whole padded grid per shot (the reference has no windows)" +
                         ("; two-pass anisotropic" if anic else ""),
                "path": "time_set + time_init + eikonal_solver (modeling.cu:104-159)" +
                        (" + get_quasi_slowness + second solve (eikonal_ani.cu:33-45)" if anic else "")}
    except Exception as ex:  # the checker must not take the bench down
        return {"unavailable": f"{type(ex).__name__}: {ex}"[:200]}


def measure(cfg, a, env, arith, full, steps, warmup):
    """One workload on this rank's shard: the timed step (graph replay of the
    planned forward+adjoint iteration, or the batched forward), per-kernel
    device times, end to end through the C ABI with host buffers, and with
    `full` the plain per-shot solver. Returns the JSON fields."""
    import torch
    rank, world, local, dev, stream, dist = env
    from seisfat2d_gb300 import Engine
    from seisfat2d_gb300.shard import allreduce_gradient, shard, shard_indices
    w = workload(cfg)
    fa = cfg in FA_CONFIGS
    ani = w.cij is not None
    mine = shard_indices(len(w.shots), rank, world)
    shots = shard(w.shots, rank, world)
    nrec = len(w.rx)
    eng = Engine(w.nx, w.nz, w.dx, w.dz, device=local)
    eng.set_arithmetic(arith)
    if a.warps or a.gang:
        eng.set_launch(a.warps, a.gang)
    eng.set_strip_loop(a.strip_loop)
    eng.set_fused_gather(not a.no_fused_gather)
    if ani:
        eng.set_stiffness(w.cij)
    eng.set_slowness(w.slowness)
    tab = eng.shot_table(shots)
    picks = torch.empty((len(shots), nrec), dtype=torch.float32, device=dev)
    grad = torch.empty((eng.nxx, eng.nzz), dtype=torch.float32, device=dev) if fa else None
    misfit = torch.empty(1, dtype=torch.float64, device=dev)
    obs = torch.from_numpy(fp64_observed(w, mine)).to(dev) if fa else None
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2 (129 MB)

    def ev():
        return torch.cuda.Event(enable_timing=True)

    tuned = None
    if fa:
        # planned batch: shots and receivers stay on the device, the iteration
        # replays from the engine's CUDA graph; the autotuner picks the launch shape
        eng.plan_batch(tab, w.rx, w.rz, stream=stream)
        if not (a.warps or a.gang or a.strip_loop != "auto"):
            tuned = eng.plan_autotune(picks, t_obs=obs, grad=grad, misfit=misfit, reps=2, stream=stream)

    def step():
        if fa:
            eng.plan_graph_launch(picks, t_obs=obs, grad=grad, misfit=misfit, stream=stream)
            if dist:  # the one exchange of the sharded iteration: the gradient sum over shots
                allreduce_gradient(grad, misfit)
        else:
            eng.batch_forward(tab, w.rx, w.rz, ani=ani, out=picks, stream=stream)

    for _ in range(warmup):
        step()
    eng.synchronize(stream)
    torch.cuda.synchronize()
    # --- timed: device-resident inputs, L2 flushed between steps
    times = []
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    with Clocks(local) as clk:
        for _ in range(steps):
            flush.zero_()
            m = [ev(), ev()]
            m[0].record(stream)
            step()
            m[1].record(stream)
            m[1].synchronize()
            times.append(m[0].elapsed_time(m[1]))
    eng.synchronize(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    ms = statistics.mean(times)
    tot_ms = sum(times)
    if dist:
        t = torch.tensor([tot_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot_ms = float(t.item())
        dist.barrier()
    total_shots = len(w.shots) * steps
    value = total_shots / (tot_ms / 1e3)

    # --- per-kernel device times (CUDA events the engine records around each
    # launch on this stream), the same steps run eagerly, L2 flushed between steps
    eng.set_kernel_timing(True)
    kt = {}
    eager_ms = []
    for _ in range(steps):
        flush.zero_()
        m = [ev(), ev()]
        m[0].record(stream)
        if fa:
            eng.plan_iteration(picks, t_obs=obs, grad=grad, misfit=misfit, stream=stream)
        else:
            step()
        m[1].record(stream)
        for k, v in eng.kernel_times().items():
            kt.setdefault(k, []).append(v)
        m[1].synchronize()
        eager_ms.append(m[0].elapsed_time(m[1]))
    eng.set_kernel_timing(False)
    eng.synchronize(stream)
    kt = {k: statistics.mean(v) for k, v in kt.items()}

    # --- end to end through the C ABI with host buffers: model in, picks (+ misfit, gradient) out;
    # the buffers are pinned host memory (numpy views of pinned torch tensors)
    def pinned(shape):
        return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()
    host_picks = pinned((len(shots), nrec))
    host_grad = pinned((eng.nxx, eng.nzz))
    host_obs = None
    if fa:
        host_obs = pinned(tuple(obs.shape))
        host_obs[...] = obs.cpu().numpy()
    model = pinned(tuple(w.slowness.shape))
    model[...] = w.slowness
    e2e_times = []
    for k in range(warmup + steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.set_slowness(model)
        eng.batch_forward(tab, w.rx, w.rz, ani=ani, keep_tape=fa, out=host_picks, stream=stream)
        if fa:
            eng.misfit_gradient(host_obs, out=host_grad, stream=stream)
        t1 = time.perf_counter()
        if k >= warmup:
            e2e_times.append(t1 - t0)
    e2e_tot = sum(e2e_times)
    if dist:
        t = torch.tensor([e2e_tot], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_tot = float(t.item())
    e2e_value = total_shots / e2e_tot
    h2d = model.nbytes + len(shots) * 16 + w.rx.nbytes + w.rz.nbytes + (host_obs.nbytes if fa else 0)
    d2h = host_picks.nbytes + (host_grad.nbytes + 8 if fa else 0)

    launch_used = eng.get_launch()
    loop_used = eng.strip_loop()
    fused_used = eng.fused_gather()[1]
    plain = None
    if full:
        # --- plain: one shot at a time, spread over the batch, with the engine's
        # default launch shape (the autotuned one belongs to the batch)
        eng.set_launch(1, 0)
        eng.set_strip_loop("auto")
        nplain = max(1, min(a.nplain, len(shots)))
        sel = [shots[q * len(shots) // nplain] for q in range(nplain)]
        Tdev = torch.empty((eng.nxx, eng.nzz), dtype=torch.float32, device=dev)
        pk = torch.empty(nrec, dtype=torch.float32, device=dev)

        def plain_forward():
            for s in sel:
                eng.time_propagation(s[0], s[1], ani=ani, out=Tdev, stream=stream)
                eng.compute_seismogram(Tdev, w.rx, w.rz, out=pk, stream=stream)

        one_tabs = [eng.shot_table([s]) for s in sel]
        one_obs = [obs[q * len(shots) // nplain:q * len(shots) // nplain + 1].contiguous()
                   for q in range(nplain)] if fa else None
        pk1 = torch.empty((1, nrec), dtype=torch.float32, device=dev)

        def plain_fa():
            for q in range(nplain):
                eng.batch_forward(one_tabs[q], w.rx, w.rz, keep_tape=True, out=pk1, stream=stream)
                eng.misfit_gradient(one_obs[q], out=grad, stream=stream, want_misfit=False)

        def timed(fn):
            fn()
            torch.cuda.synchronize()
            e0, e1 = ev(), ev()
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            return e0.elapsed_time(e1) / nplain

        plain_ms = timed(plain_forward)
        plain = {"forward_ms_per_shot": plain_ms, "forward_shots_per_s": 1e3 / plain_ms,
                 "path": "sf_time_propagation + sf_compute_seismogram, one shot per call",
                 "batched_vs_plain_forward": value / world / (1e3 / plain_ms)}
        if fa:
            plain_fa_ms = timed(plain_fa)
            plain.update({
                "forward_adjoint_ms_per_shot": plain_fa_ms, "forward_adjoint_shots_per_s": 1e3 / plain_fa_ms,
                "forward_adjoint_path": "sf_batch_forward + sf_batch_misfit_gradient on a one-shot batch, per shot",
                "batched_vs_plain_forward_adjoint": value / world / (1e3 / plain_fa_ms)})
        eng.synchronize(stream)

    cells = sum(window(s, eng.nxx)[1] * eng.nzz for s in shots)
    peak, peak_kind = load_peaks()
    fwd_bpc = BYTES_PER_CELL_FWD_ANI if ani else BYTES_PER_CELL_FWD
    kname = "k_shots_tape" if fa else ("k_shots_ani" if ani else "k_shots")
    if arith == "compensated":
        kname += "_comp"  # its own capture (the lo parts add window traffic); absent ones give no traffic
    fkern = "sf::k_shots<tape>" if fa else ("sf::k_shots, sf::k_qp, sf::k_shots (solve on S, qP pass, solve on the qP slowness)"
                                            if ani else "sf::k_shots")
    stages = {"forward": {"kernel": fkern, "ms": kt["forward"],
                          "algorithmic_bytes": fwd_bpc * cells, "traffic_file": f"{kname}_cfg{cfg}.txt"}}
    if fa and "gather" in kt:
        stages["adjoint"] = {"kernel": "sf::k_adjoint", "ms": kt["adjoint"],
                             "algorithmic_bytes": (BYTES_PER_CELL_ADJ - 8) * cells,
                             "traffic_file": f"k_adjoint_cfg{cfg}.txt"}
        stages["gather"] = {"kernel": "sf::k_gather", "ms": kt["gather"], "algorithmic_bytes": 8 * cells,
                            "traffic_file": f"k_gather_cfg{cfg}.txt"}
    elif fa:
        # reverse sweeps and gather in one launch (sf_set_fused_gather)
        stages["adjoint"] = {"kernel": "sf::k_adjoint_gather (reverse sweeps + gather)", "ms": kt["adjoint"],
                             "algorithmic_bytes": BYTES_PER_CELL_ADJ * cells,
                             "traffic_file": f"k_adjoint_gather_cfg{cfg}.txt"}
    if fa:
        stages["residual"] = {"kernel": "sf::k_residual", "ms": kt["residual"],
                              "algorithmic_bytes": 3 * 4 * len(shots) * nrec, "traffic_file": None}
    for st in stages.values():
        st["achieved_gbs"] = st["algorithmic_bytes"] / (st["ms"] / 1e3) / 1e9
        st["frac"] = st["achieved_gbs"] / peak
        tpc = load_traffic(st["traffic_file"]) if st["traffic_file"] else None
        st["traffic"] = tpc * cells if tpc else None
    dom = max(stages.values(), key=lambda st: st["ms"])
    step_bytes = sum(st["algorithmic_bytes"] for st in stages.values())
    config = {"workload": w.name, "nshots": len(w.shots), "nrec": nrec, "grid": [w.nx, w.nz],
              "padded": [eng.nxx, eng.nzz], "dh": w.dx,
              "step": ("taped forward + picks, residuals + FP64 misfit, reverse sweeps, gradient gather"
                       if fa else ("VTI forward (2 solves + qP pass) + picks" if ani else "forward + picks")),
              "parallelism": f"shots sharded over {world} GPU(s)" +
                             (", FP64 gradient sum over ranks in the step" if fa and world > 1 else ""),
              "l2": "flushed between timed steps (512 MB write)",
              "launch": {"warps_per_cta": launch_used[0], "warps_per_shot": launch_used[1] or "auto",
                         "strip_loop": {"mode": loop_used[0],
                                        "form": "interior-block" if loop_used[1] else "general"},
                         **({"gather": "inside the reverse-sweep launch" if fused_used else "own launch"}
                            if fa else {}),
                         "chosen_by": "sf_plan_autotune" if tuned else (
                             "flags" if (a.warps or a.gang or a.strip_loop != "auto") else "default")},
              "timed_path": ("sf_plan_graph_launch (CUDA graph of the planned iteration)" if fa
                             else "sf_batch_forward"),
              "eager_ms_per_step": statistics.mean(eager_ms),
              "arithmetic": eng.get_arithmetic()}
    out = {
        "value": value, "ms_per_step": ms, "steps": steps, "warmup": warmup, "config": config,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "buffers": "pinned host memory", "path": "sf_set_slowness(host model) + sf_batch_forward(host picks)" +
                        (" + sf_batch_misfit_gradient(host picks in, host misfit and gradient out)" if fa else "")},
        "roofline": {"bound": "hbm", "achieved": dom["achieved_gbs"], "peak": peak, "unit": "GB/s",
                     "frac": dom["frac"], "peak_source": peak_kind, "traffic": dom["traffic"],
                     "kernel": dom["kernel"], "algorithmic_bytes": dom["algorithmic_bytes"],
                     "stages": stages, "timing": "CUDA events recorded by the engine around each launch "
                                                 "(sf_set_kernel_timing), mean over the eager steps",
                     "limiter": "latency of the sweep recurrence: each solve of a shot is 4 sweeps x "
                                "(columns + 31) dependent warp-steps, and the batch fills a fraction of the "
                                "warp slots; HBM is the bound the fraction is quoted against",
                     "step": {"algorithmic_bytes": step_bytes,
                              "achieved_gbs": step_bytes / (ms / 1e3) / 1e9,
                              "frac": step_bytes / (ms / 1e3) / 1e9 / peak}},
        "gpu_launches": steps * ((4 if "gather" in kt else 3) if fa else (3 if ani else 1)),
        "clocks": clk.summary(),
        "wall_s_timed": wall,
    }
    if plain:
        out["plain"] = plain
    if rank == 0 and not a.no_checks:
        out["accuracy"] = accuracy_checks(eng, w, fa, ani)
        out["reference_gpu"] = reference_gpu(w, 3 if full else 2)
        rg = out["reference_gpu"]
        if "ms_per_shot" in rg:
            fwd_ms = kt["forward"] / len(shots)
            rg["batched_forward_vs_reference"] = rg["ms_per_shot"] / fwd_ms
            rg["batched_step_vs_reference_forward"] = value / world / rg["shots_per_s"]
            rg["note"] = ("batched_forward_vs_reference: the reference's ms per forward shot over the batched "
                          "forward kernel's ms per shot" + ("; the step also runs the adjoint" if fa else ""))
    eng.close()
    return w, fa, out


def run_ours(a):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    env = (rank, world, local, dev, torch.cuda.current_stream(dev), dist)
    w, fa, head = measure(a.config, a, env, a.arith, True, a.steps, a.warmup)
    line = {"metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded model and geometry" + (
                "; observed picks = FP64 oracle on the true model + seeded N(0, 2 ms) noise)" if fa else ")")}
    for k in ("config", "e2e", "roofline", "plain", "gpu_launches", "clocks", "wall_s_timed", "accuracy",
              "reference_gpu"):
        if k in head:
            line[k] = head[k]
    if world == 1 and not a.no_configs:
        # the same step in the reference build's arithmetic (bit-identical to the
        # reference's kernels), and the other configs in this run's arithmetic
        brief = ("value", "ms_per_step", "steps", "warmup", "e2e", "accuracy", "reference_gpu", "clocks")
        if a.arith != "reference":
            _, _, r = measure(a.config, a, env, "reference", False, a.config_steps, a.config_warmup)
            line["reference_arithmetic"] = {k: r[k] for k in brief if k in r}
            line["reference_arithmetic"]["stages_ms"] = {k: v["ms"] for k, v in r["roofline"]["stages"].items()}
        line["configs"] = {}
        for c in sorted(workload_ids()):
            if c == a.config or c == 1:
                continue
            _, _, r = measure(c, a, env, a.arith, False, a.config_steps, a.config_warmup)
            d = {k: r[k] for k in brief if k in r}
            d["workload"] = r["config"]["workload"]
            d["step"] = r["config"]["step"]
            d["arithmetic"] = r["config"]["arithmetic"]
            d["launch"] = r["config"]["launch"]
            d["roofline"] = {k: r["roofline"][k] for k in ("kernel", "achieved", "frac", "traffic")}
            d["stages_ms"] = {k: v["ms"] for k, v in r["roofline"]["stages"].items()}
            d["gpu_launches"] = r["gpu_launches"]
            line["configs"][f"config{c}"] = d
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    if not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, a.cpu_seconds, fa)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
