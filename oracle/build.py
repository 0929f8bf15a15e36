"""Build recipe for the CPU oracle (test infrastructure, never shipped).

Compiles ``eikonal_oracle.c`` into ``oracle/_build/liboracle.so`` with
``-ffp-contract=off`` so FP32 operations round once each, in source order, on
x86-64 and aarch64 alike.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")
SRC = os.path.join(HERE, "eikonal_oracle.c")


def build(force=False):
    """Compile the oracle shared library; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = [SRC, os.path.join(HERE, "eikonal_oracle.h")]
    if not force and os.path.exists(LIB) and all(
        os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps
    ):
        return LIB
    cmd = [
        "gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp",
        "-ffp-contract=off", "-fno-fast-math", "-fno-strict-aliasing",
        SRC, "-o", LIB + ".tmp", "-lm",
    ]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
