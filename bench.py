"""Benchmark of the batched eikonal engine on one GB300 (or N, one process per
GPU under torchrun, shots sharded across ranks).

Workload: 200 surface shots, each a full 4-sweep isotropic solve on the
2001 x 501 (2007 x 507 padded) synthetic 6-layer model at 10 m, plus 800
receiver picks per shot; all shots in one persistent launch. A step is one
such batch. Prints ONE JSON line (rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
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

METRIC = "eikonal shots/s (batched, FP32, <=1e-5 rel err)"
UNIT = "shots/s"
BYTES_PER_CELL_FWD = 48  # 4 sweeps x (S 4 B + T read 4 B + T write 4 B)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--warps", type=int, default=0, help="warps per CTA (0: engine default)")
    ap.add_argument("--gang", type=int, default=0, help="warps per shot (0: automatic)")
    ap.add_argument("--arith", default="reference", choices=["reference", "ieee"])
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


def load_traffic(name):
    """DRAM bytes per padded cell per shot of the forward kernel from the
    committed ncu summary (profiles/), or None."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_cell_shot:"):
            return float(line.split(":")[1])
    return None


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


def cpu_baseline(w, seconds, rank):
    """The oracle's FP32 port of the reference schedule on the host cores
    (one shot per thread), on a bounded sample of the same shots."""
    from oracle import oracle as O
    S = O.expand_boundary(w.slowness)
    nthreads = os.cpu_count() or 1
    shots = w.shots
    # calibrate on one shot, then size the sample to ~`seconds` of work
    t0 = time.perf_counter()
    O.batch_picks(S, w.dx, w.dz, [shots[0][0]], [shots[0][1]], [0], [S.shape[0]], w.rx, w.rz, nthreads=1)
    one = time.perf_counter() - t0
    n = max(nthreads, int(seconds * nthreads / max(one, 1e-3)))
    n = min(n, len(shots))
    n = max(nthreads, (n // nthreads) * nthreads) if n >= nthreads else n
    sel = [shots[k * len(shots) // n] for k in range(n)]
    sx = [s[0] for s in sel]
    sz = [s[1] for s in sel]
    c0 = [s[2] if len(s) > 2 else 0 for s in sel]
    nc = [s[3] if len(s) > 3 and s[3] > 0 else S.shape[0] - (s[2] if len(s) > 2 else 0) for s in sel]
    t0 = time.perf_counter()
    _, used = O.batch_picks(S, w.dx, w.dz, sx, sz, c0, nc, w.rx, w.rz, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": used, "kind": "port",
            "sample": f"{n} of the {len(shots)} shots of {w.name}, one shot per thread, "
                      f"{dt:.1f} s, oracle FP32 restatement of the reference schedule (-O2)"}


def run_reference(a):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    w = workload(a.config)
    samples = []
    res = None
    for k in range(a.steps):
        res = cpu_baseline(w, a.cpu_seconds / max(1, a.steps) * 2, rank)
        samples.append(res["value"])
    v = statistics.median(samples)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": w.name, "nshots": len(w.shots), "nrec": len(w.rx),
                       "grid": [w.nx, w.nz], "dh": w.dx},
            "cpu_baseline": dict(res, value=v),
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference has no CPU eikonal path; this arm times the oracle's FP32 "
                    "restatement of its schedule on the host cores"}
    print(json.dumps(line), flush=True)


def run_ours(a):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from seisfat2d_gb300 import Engine
    w = workload(a.config)
    shots = w.shots[rank::world]
    nrec = len(w.rx)
    eng = Engine(w.nx, w.nz, w.dx, w.dz, device=local)
    eng.set_arithmetic(a.arith)
    if a.warps or a.gang:
        eng.set_launch(a.warps, a.gang)
    eng.set_slowness(w.slowness)
    tab = eng.shot_table(shots)
    dev = torch.device("cuda", local)
    picks = torch.empty((len(shots), nrec), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2 (129 MB)

    def step():
        eng.batch_forward(tab, w.rx, w.rz, out=picks, stream=stream)

    for _ in range(a.warmup):
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
        for _ in range(a.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
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
    total_shots = len(w.shots) * a.steps
    value = total_shots / (tot_ms / 1e3)

    # --- end to end through the C ABI with host buffers (model in, picks out)
    host_picks = np.zeros((len(shots), nrec), np.float32)
    model = np.ascontiguousarray(w.slowness)
    e2e_times = []
    for k in range(a.warmup + a.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        eng.set_slowness(model)
        eng.batch_forward(tab, w.rx, w.rz, out=host_picks, stream=stream)
        t1 = time.perf_counter()
        if k >= a.warmup:
            e2e_times.append(t1 - t0)
    e2e_tot = sum(e2e_times)
    if dist:
        t = torch.tensor([e2e_tot], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_tot = float(t.item())
    e2e_value = total_shots / e2e_tot
    h2d = model.nbytes + len(shots) * 16 + 2 * w.rx.nbytes
    d2h = host_picks.nbytes

    # --- plain per-shot drop-in (one shot at a time, one CTA) for batched vs plain
    Tdev = torch.empty((eng.nxx, eng.nzz), dtype=torch.float32, device=dev)
    nplain = min(8, len(shots))
    eng.time_propagation(shots[0][0], shots[0][1], out=Tdev, stream=stream)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    pk = torch.empty(nrec, dtype=torch.float32, device=dev)
    for s in shots[:nplain]:
        eng.time_propagation(s[0], s[1], out=Tdev, stream=stream)
        eng.compute_seismogram(Tdev, w.rx, w.rz, out=pk, stream=stream)
    e1.record(stream)
    e1.synchronize()
    plain_ms = e0.elapsed_time(e1) / nplain

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    cells = sum((s[3] if len(s) > 3 and s[3] > 0 else eng.nxx) * eng.nzz for s in shots)
    alg_bytes = BYTES_PER_CELL_FWD * cells
    peak, peak_kind = load_peaks()
    achieved = alg_bytes / (ms / 1e3) / 1e9
    tpc = load_traffic("k_shots_cfg2_forward.txt")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded model and geometry)",
        "config": {"workload": w.name, "nshots": len(w.shots), "nrec": nrec, "grid": [w.nx, w.nz],
                   "padded": [eng.nxx, eng.nzz], "dh": w.dx, "parallelism": f"shots sharded over {world} GPU(s)",
                   "l2": "flushed between timed steps (512 MB write)",
                   "launch": {"warps_per_cta": eng.get_launch()[0], "warps_per_shot": eng.get_launch()[1] or "auto"},
                   "arithmetic": eng.get_arithmetic()},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "path": "sf_set_slowness(host model) + sf_batch_forward(host picks)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": (tpc * cells) if tpc else None,
                     "algorithmic_bytes": alg_bytes, "kernel": "sf::k_shots<false>"},
        "plain": {"ms_per_shot": plain_ms, "shots_per_s": 1e3 / plain_ms,
                  "batched_vs_plain": value / world / (1e3 / plain_ms)},
        "gpu_launches": a.steps,
        "clocks": clk.summary(),
        "wall_s_timed": wall,
    }
    if not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, a.cpu_seconds, rank)
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
