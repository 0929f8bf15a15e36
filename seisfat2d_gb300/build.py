"""Build recipe of the engine library (``libseisfat2d.so``), sm_103a only.

Each CUDA translation unit is compiled in parallel with nvcc, then linked into
one shared library next to this file (git-ignored). Host code is compiled with
``-ffp-contract=off`` so host-side float arithmetic (source indices, constants,
quantisation) rounds the same way on x86-64 and aarch64.
"""
import concurrent.futures as cf
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INC = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libseisfat2d.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-O2",
]
UNITS = ["sf_engine.cu", "sf_adjoint.cu", "sf_plan.cu", "sf_update.cu", "sf_migration.cu"]
# k_shots instantiations, one object each from sf_shots_inst.cu: (tape,
# reference arithmetic, interior-block strip loops, compensated arithmetic)
KSHOTS = [(0, 0, 0, 0), (0, 0, 1, 0), (0, 1, 0, 0), (0, 1, 1, 0), (1, 0, 0, 0), (1, 0, 1, 0), (1, 1, 0, 0), (1, 1, 1, 0),
          (0, 0, 0, 1), (0, 0, 1, 1), (1, 0, 0, 1), (1, 0, 1, 1)]


def _jobs():
    """(source, extra nvcc flags, object name) of every translation unit."""
    jobs = [(u, [], u.replace(".cu", ".o")) for u in UNITS]
    for v in KSHOTS:
        tag = "".join(str(b) for b in v)
        defs = [f"-DSF_{k}={'true' if b else 'false'}" for k, b in zip(("TAPE", "REF", "INTERIOR", "COMP"), v)]
        jobs.append(("sf_shots_inst.cu", defs + [f"-DSF_KSHOTS_NAME=sf_kshots_{tag}"], f"sf_shots_{tag}.o"))
    return jobs


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _deps():
    out = []
    for d in (CSRC, INC):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h")):
                out.append(os.path.join(d, f))
    return out


def build(force=False, verbose=False, ptxas_info=False):
    """Compile the engine; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    deps = _deps()
    newest = max(os.path.getmtime(d) for d in deps)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    nvcc = _nvcc()
    extra = ["-Xptxas", "-v"] if ptxas_info else []

    def compile_unit(job):
        u, defs, oname = job
        obj = os.path.join(BUILD, oname)
        cmd = [nvcc] + NVCC_FLAGS + extra + defs + ["-I", INC, "-c", os.path.join(CSRC, u), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0 or verbose or ptxas_info:
            print(r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on " + oname)
        return obj

    jobs = _jobs()
    with cf.ThreadPoolExecutor(min(len(jobs), max(4, os.cpu_count() or 4))) as ex:
        objs = list(ex.map(compile_unit, jobs))
    tmp = LIB + ".tmp"
    subprocess.run([nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
