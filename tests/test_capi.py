"""The C-ABI library: it loads, exports every symbol include/ams.h declares,
and rejects bad arguments with a status (no GPU needed for these)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "ams.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(ams_[a-z_0-9]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def L():
    from automs_gb300 import _lib
    return _lib.lib()


def test_every_declared_symbol_is_exported(L):
    syms = declared_symbols()
    assert "ams_trace_channel" in syms and "ams_objective_fwd_bwd" in syms
    for s in syms:
        assert hasattr(L, s), s


def test_version(L):
    assert b"sm_103a" in L.ams_version()


def test_bad_arguments_return_status(L):
    from automs_gb300._lib import TraceParams
    buf = C.create_string_buffer(256)
    assert L.ams_scene_create(None, 0, None, None, 0, None, None, buf, 256) == 1
    assert b"NULL" in buf.value
    h = C.c_void_p()
    assert L.ams_scene_create(None, 5, None, None, 1, None, C.byref(h), buf, 256) == 1
    p = TraceParams()
    assert L.ams_trace_channel(None, C.byref(p), None, 1, 1, None, 1, 1, None, None, None,
                               None, None, buf, 256) == 1
    # objective: C > 64, missing W, missing metasurface pieces
    args = [C.c_void_p(8), None, None, None, 1.0, C.c_void_p(8), 4, 0, 16, 65, 1.0, None,
            C.c_void_p(8), None, None, None, None, None, buf, 256]
    assert L.ams_objective_fwd_bwd(*args) == 1
    args[9] = 4
    args[1] = C.c_void_p(8)  # H_a without H_r / phi
    assert L.ams_objective_fwd_bwd(*args) == 1
    assert L.ams_coverage_db(None, 1, 1, -150.0, 0.0, None, None, buf, 256) == 1


def test_trace_params_validation(L):
    from automs_gb300 import tracer
    buf = C.create_string_buffer(256)
    for bad in (dict(max_reflection=6), dict(reserve_size=0), dict(reserve_size=257),
                dict(src_bptype=4), dict(dst_gridsize=0), dict(wave_len=0.0)):
        p = tracer.make_params(**bad)
        rc = L.ams_trace_channel(C.c_void_p(1), C.byref(p), C.c_void_p(8), 1, 1, C.c_void_p(8),
                                 1, 1, None, None, C.c_void_p(8), None, None, buf, 256)
        assert rc == 1, bad
