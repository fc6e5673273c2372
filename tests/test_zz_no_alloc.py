"""The allocation-free objective entry point against the regular one.

ams_objective_fwd_bwd_noalloc serves callers that cannot allocate device
memory (their own memory pool owns the device, or they run inside a stream
capture where cudaMalloc is not allowed).  It must give the same loss and
gradients as ams_objective_fwd_bwd, call after call, from its fixed scratch.
This file is collected last so that a failure here does not hide others.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _case(rng, S=8, M=96, R=700, Cc=4):
    def cn(*sh):
        return torch.as_tensor(((rng.normal(size=sh) + 1j * rng.normal(size=sh)) * 1e-4)
                               .astype(np.complex64), device="cuda")
    W = torch.as_tensor((rng.normal(size=(Cc, S)) + 1j * rng.normal(size=(Cc, S)))
                        .astype(np.complex64), device="cuda")
    phi = torch.as_tensor(rng.uniform(0, 7.0, M).astype(np.float32), device="cuda")
    drop = torch.zeros(Cc, dtype=torch.uint8, device="cuda")
    if Cc > 1:
        drop[1] = 1
    return dict(Hd=cn(S, R), Ha=cn(S, M), Hr=cn(M, R), W=W, phi=phi, drop=drop, S=S, M=M, R=R,
                C=Cc)


def _run(lib, name, c):
    P = lambda t: C.c_void_p(t.data_ptr())
    out = dict(loss=torch.empty((), device="cuda"), gW=torch.empty_like(c["W"]),
               gphi=torch.empty_like(c["phi"]),
               gY=torch.empty(c["C"], c["R"], dtype=torch.complex64, device="cuda"),
               amp=torch.empty(c["C"], c["R"], device="cuda"))
    buf = C.create_string_buffer(512)
    rc = getattr(lib, name)(
        P(c["Hd"]), P(c["Ha"]), P(c["Hr"]), P(c["phi"]), 5.2, P(c["W"]), c["S"], c["M"], c["R"],
        c["C"], 0.5, P(c["drop"]), P(out["loss"]), P(out["gW"]), P(out["gphi"]), P(out["gY"]),
        P(out["amp"]), C.c_void_p(torch.cuda.current_stream().cuda_stream), buf, 512)
    assert rc == 0, buf.value
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


def test_noalloc_matches_regular_entry_point():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from automs_gb300 import _lib
    lib = _lib.lib()
    rng = np.random.Generator(np.random.PCG64(21))
    cases = [_case(rng), _case(rng, S=16, M=300, R=2048, Cc=1)]
    for c in cases:
        ref = _run(lib, "ams_objective_fwd_bwd", c)
        for _ in range(2):  # two calls in a row share the fixed scratch
            got = _run(lib, "ams_objective_fwd_bwd_noalloc", c)
            for k in ref:
                np.testing.assert_allclose(got[k], ref[k], rtol=1e-5,
                                           atol=1e-6 * float(np.abs(ref[k]).max() + 1e-30),
                                           err_msg=k)


def test_noalloc_rejects_oversize_problem():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from automs_gb300 import _lib
    lib = _lib.lib()
    buf = C.create_string_buffer(512)
    x = torch.zeros(8, device="cuda")
    p = C.c_void_p(x.data_ptr())
    # C=64 codes over 200k Rx needs far more than the fixed scratch
    rc = lib.ams_objective_fwd_bwd_noalloc(p, None, None, None, 1.0, p, 4, 0, 200000, 64, 1.0,
                                           None, p, None, None, None, None, None, buf, 512)
    assert rc == 4
    assert b"scratch" in buf.value
