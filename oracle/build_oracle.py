"""Build the C oracle (test infrastructure) into oracle/_build/libams_oracle.so.

The oracle is compiled with -ffp-contract=off so that float expressions round
exactly as written (no fused multiply-add), which is the arithmetic contract
the CUDA kernels follow.  When the reference sources are present, the
reference harness (oracle/ref_harness) is built as well.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libams_oracle.so")


def build_oracle(force=False):
    src = os.path.join(HERE, "ams_oracle.c")
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
        os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "ams_oracle.h"))
    ):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-Wall", "-o", LIB, src, "-lm"]
    subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    sys.path.insert(0, os.path.join(HERE, "ref_harness"))
    import build_ref  # noqa: E402
    print(build_ref.build_ref(force="--force" in sys.argv))
