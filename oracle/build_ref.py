"""Recipe: the reference's own device code as a checker (test infrastructure).

Compiles the kernels of phbastosa/SeisFAT2D's modeling path -- time_set,
time_init, inner_sweep (src/modeling/modeling.cu) and get_quasi_slowness
(src/modeling/eikonal_ani.cu) -- from the reference sources where they lie,
into ``oracle/_ref/*.cubin`` (device code only, sm_103a). The reference
includes <fftw3.h> unconditionally (src/admin/admin.hpp:10) although the
modeling path never calls FFTW, which is not installed: an empty stub header
generated under ``oracle/_ref/stub`` satisfies the include.

Differences from the reference's own build line (run/program.sh:51): device
code only, ``-rdc`` off (every kernel is self-contained) and an explicit
sm_103a target; nvcc's defaults otherwise (FMA contraction on, IEEE div/sqrt).

``ref_harness.cpp`` (always built, it needs no reference source) loads those
cubins with the CUDA driver API and replays the reference's host launch loop,
so the reference's kernels run unmodified on the GPU.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("SF_REFERENCE_ROOT", "/root/reference")
OUT = os.path.join(HERE, "_ref")
BUILD = os.path.join(HERE, "_build")
CUBINS = {"modeling": "src/modeling/modeling.cu", "eikonal_ani": "src/modeling/eikonal_ani.cu"}
HARNESS_SRC = os.path.join(HERE, "ref_harness.cpp")
HARNESS = os.path.join(BUILD, "libref_harness.so")


def cubin_path(name):
    return os.path.join(OUT, name + ".cubin")


def build_cubins():
    if not os.path.isdir(os.path.join(REF, "src", "modeling")):
        return False
    stub = os.path.join(OUT, "stub")
    os.makedirs(stub, exist_ok=True)
    open(os.path.join(stub, "fftw3.h"), "w").close()
    for name, rel in CUBINS.items():
        src = os.path.join(REF, rel)
        out = cubin_path(name)
        if os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
            continue
        cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "--std=c++11",
               "-I", stub, src, "-o", out + ".tmp"]
        subprocess.run(cmd, check=True, capture_output=True)
        os.replace(out + ".tmp", out)
    return True


def build_harness():
    os.makedirs(BUILD, exist_ok=True)
    if os.path.exists(HARNESS) and os.path.getmtime(HARNESS) >= os.path.getmtime(HARNESS_SRC):
        return HARNESS
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", HARNESS_SRC,
           "-I", os.path.join(cuda, "include"), "-L", os.path.join(cuda, "lib64", "stubs"),
           "-L", os.path.join(cuda, "lib64"), "-lcuda", "-o", HARNESS + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(HARNESS + ".tmp", HARNESS)
    return HARNESS


def build():
    build_cubins()
    build_harness()


def available():
    return all(os.path.exists(cubin_path(n)) for n in CUBINS)


if __name__ == "__main__":
    print("cubins:", build_cubins(), "harness:", build_harness())
