"""Failure detection without a GPU fault: the bounded mbarrier wait that
guards every TMA / tcgen05 pipeline gives up after its limit and reports it,
and the context stays usable (tests/wait_timeout_check.cu)."""
import ctypes as C
import os
import shutil
import subprocess

import pytest
import torch

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bounded_wait_runs_out_and_reports(tmp_path):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    so = str(tmp_path / "wait_check.so")
    r = subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-shared",
                        "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "automs_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "wait_timeout_check.cu"), "-o", so],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = C.CDLL(so)
    ok, el = C.c_ulonglong(), C.c_ulonglong()
    limit = 50_000_000  # 50 ms
    assert lib.run_wait_nothing(C.c_ulonglong(limit), C.byref(ok), C.byref(el)) == 0
    assert ok.value == 0, "the wait should have given up"
    assert limit <= el.value < limit + 1_000_000_000, el.value
    # the context still works
    x = torch.arange(1024, device="cuda", dtype=torch.float32)
    assert float(x.sum()) == 1023 * 1024 / 2
