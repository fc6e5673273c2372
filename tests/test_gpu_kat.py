"""Known-answer channels through the CUDA tracer (C ABI): free space and one
mirror against their closed forms (tests/kat_scenes.py), with the same ray
set as the oracle."""
import numpy as np
import pytest
import torch

import oracle
from kat_scenes import check, kat_config

pytestmark = pytest.mark.gpu


def test_free_space_and_mirror_closed_form():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from automs_gb300 import tracer
    H = []
    for L in (0, 1):
        c = kat_config(L)
        sc = tracer.Scene(c["tris"], c["mat"], c["mat_prop"])
        res, st = sc.trace(c["src"], c["dst"], c["params"])
        torch.cuda.synchronize()
        sc.close()
        h = (res[..., 0] + 1j * res[..., 1]).cpu().numpy().astype(np.complex128)
        _, so, _ = oracle.trace_channel(c["tris"], c["mat"], c["mat_prop"], c["src"], c["dst"],
                                        c["params"], nthreads=4)
        assert st["rx_paths"] == so["rx_paths"] and st["rx_fail"] == so["rx_fail"]
        assert st["unique_paths"] == L + 1
        H.append(h)
    check(H[0], H[1], c["src"], c["dst"])
