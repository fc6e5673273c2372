"""Known-answer channels through the oracle: free space and one mirror
against their closed forms (tests/kat_scenes.py)."""
import oracle
from kat_scenes import check, kat_config


def test_free_space_and_mirror_closed_form():
    H = []
    for L in (0, 1):
        c = kat_config(L)
        h, st, paths = oracle.trace_channel(c["tris"], c["mat"], c["mat_prop"], c["src"], c["dst"],
                                            c["params"], nthreads=4)
        assert st["unique_paths"] == L + 1
        H.append(h.astype("complex128"))
    check(H[0], H[1], c["src"], c["dst"])
