"""Recipe: the reference's own device code as a checker (test infrastructure).

Compiles the kernels of phbastosa/SeisFAT2D's modeling path -- time_set,
time_init, inner_sweep (src/modeling/modeling.cu) and get_quasi_slowness
(src/modeling/eikonal_ani.cu) -- and its Kirchhoff imaging kernels
(src/migration/migration.cu) from the reference sources where they lie,
into ``oracle/_ref/*.cubin`` (device code only, sm_103a). The reference
includes <fftw3.h> unconditionally (src/admin/admin.hpp:10); FFTW is not
installed and no device code calls it, so a stub header of declarations
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
CUBINS = {"modeling": "src/modeling/modeling.cu", "eikonal_ani": "src/modeling/eikonal_ani.cu",
          "migration": "src/migration/migration.cu"}
# Declarations of the FFTW3 interface the reference's host code names
# (src/migration/migration.cu:173-261). Only the device code ends up in the
# cubins, but the compiler parses the host code too.
FFTW_STUB = """#pragma once
#include <cstddef>
typedef double fftw_complex[2];
typedef struct fftw_plan_opaque* fftw_plan;
#define FFTW_ESTIMATE (1U << 6)
void* fftw_malloc(size_t n);
fftw_plan fftw_plan_dft_r2c_1d(int n, double* in, fftw_complex* out, unsigned flags);
fftw_plan fftw_plan_dft_c2r_1d(int n, fftw_complex* in, double* out, unsigned flags);
void fftw_execute(const fftw_plan p);
"""
HARNESS_SRC = os.path.join(HERE, "ref_harness.cpp")
HARNESS = os.path.join(BUILD, "libref_harness.so")


def cubin_path(name):
    return os.path.join(OUT, name + ".cubin")


def build_cubins():
    if not os.path.isdir(os.path.join(REF, "src", "modeling")):
        return False
    stub = os.path.join(OUT, "stub")
    os.makedirs(stub, exist_ok=True)
    with open(os.path.join(stub, "fftw3.h"), "w") as f:
        f.write(FFTW_STUB)
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
