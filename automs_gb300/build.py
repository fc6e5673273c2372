"""Build libams.so in-tree (automs_gb300/_build/) for sm_103a.

nvcc compiles each .cu for -gencode arch=compute_103a,code=sm_103a (the
tracer with -fmad=false, see trace.cu), g++ compiles the C-ABI host code,
and everything links into one shared library with the static CUDA runtime.
Translation units compile in parallel.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libams.so")
ROOT = os.path.dirname(HERE)
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc") if os.path.exists(
    os.path.join(CUDA_HOME, "bin", "nvcc")) else shutil.which("nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# per-file extra flags
CU_FLAGS = {
    "trace.cu": ["-fmad=false"],
}


def _sources():
    cus = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpps = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    return cus, cpps


def _deps_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(ROOT, "include", "ams.h"))
    files.append(os.path.abspath(__file__))
    return max(os.path.getmtime(f) for f in files)


def build(force=False, verbose=False):
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    if NVCC is None:
        raise RuntimeError("nvcc not found: cannot build libams.so")
    os.makedirs(BUILD, exist_ok=True)
    cus, cpps = _sources()
    jobs = []
    for f in cus:
        obj = os.path.join(BUILD, f + ".o")
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "--expt-relaxed-constexpr", *CU_FLAGS.get(f, []),
               "-I", CSRC, "-I", os.path.join(ROOT, "include"),
               "-c", os.path.join(CSRC, f), "-o", obj]
        jobs.append((cmd, obj))
    for f in cpps:
        obj = os.path.join(BUILD, f + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I", CSRC,
               "-I", os.path.join(ROOT, "include"), "-I", os.path.join(CUDA_HOME, "include"),
               "-c", os.path.join(CSRC, f), "-o", obj]
        jobs.append((cmd, obj))

    def run(job):
        cmd, obj = job
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        objs = list(ex.map(run, jobs))
    tmp = LIB + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static",
           "-Xlinker", "--no-undefined", "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
