"""Compile the reference's own device programs into a CPU library.

Recipe: g++ on optixPathTracer.cu where it lies in the reference tree, with
the OptiX shim of oracle/ref_harness/shim first on the include path and the
reference's vendored sutil / random.h headers after it.  Output goes to
oracle/_ref/libams_ref.so (git-ignored).  Nothing is copied out of the
reference tree.  The reference tree is named by the environment variable
AMS_REFERENCE_ROOT; without it the harness is not built (available() is
False).  The fixtures it produces are committed under tests/golden/.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
LIB = os.path.join(OUT, "libams_ref.so")
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


def ref_root():
    """The reference tree named by AMS_REFERENCE_ROOT, or None."""
    r = os.environ.get("AMS_REFERENCE_ROOT")
    return r if r and os.path.exists(os.path.join(r, "optixPathTracer.cu")) else None


def available():
    return ref_root() is not None


def build_ref(force=False):
    REF = ref_root()
    if REF is None:
        return None
    os.makedirs(OUT, exist_ok=True)
    srcs = [os.path.join(HERE, "ref_harness.cpp"), os.path.join(ORACLE, "ams_oracle.c")]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
        os.path.getmtime(s) for s in srcs + [os.path.join(HERE, "shim", "optix.h")]
    ):
        return LIB
    objs = []
    common = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-w"]
    obj_o = os.path.join(OUT, "ams_oracle.o")
    subprocess.check_call(["gcc", "-std=c11", "-fopenmp", *common, "-c", srcs[1], "-o", obj_o])
    objs.append(obj_o)
    obj_h = os.path.join(OUT, "ref_harness.o")
    subprocess.check_call([
        "g++", "-std=c++17", *common,
        "-I", os.path.join(HERE, "shim"),
        "-I", REF,
        "-I", os.path.join(REF, "optix", "SDK"),
        "-I", os.path.join(REF, "optix", "SDK", "cuda"),
        "-I", ORACLE,
        "-I", CUDA_INC,
        "-c", srcs[0], "-o", obj_h,
    ])
    objs.append(obj_h)
    subprocess.check_call(["g++", "-shared", "-fopenmp", "-o", LIB, *objs, "-lm"])
    return LIB


if __name__ == "__main__":
    print(build_ref(force=True))
