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


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes and numpy mirrors of the C structs (ams_trace_params,
    ams_stats, ams_ray_record) have the header's size and field offsets,
    printed by a program compiled against include/ams.h."""
    import shutil
    import subprocess

    import numpy as np

    from automs_gb300 import _lib, tracer
    if shutil.which("g++") is None:
        pytest.skip("g++ is missing")
    mirrors = {"ams_trace_params": _lib.TraceParams, "ams_stats": _lib.Stats}
    lines = ['#include <cstddef>', '#include <cstdio>', '#include "ams.h"', "int main() {"]
    for cname, py in mirrors.items():
        lines.append(f'  printf("{cname} %zu\\n", sizeof({cname}));')
        for f, _ in py._fields_:
            lines.append(f'  printf("{cname}.{f} %zu\\n", offsetof({cname}, {f}));')
    lines.append('  printf("ams_ray_record %zu\\n", sizeof(ams_ray_record));')
    for f in tracer.RAY_RECORD.names:
        lines.append(f'  printf("ams_ray_record.{f} %zu\\n", offsetof(ams_ray_record, {f}));')
    lines.append("  return 0;\n}")
    src = tmp_path / "layout.cpp"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    r = subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = dict(line.split() for line in subprocess.run([exe], capture_output=True,
                                                       text=True).stdout.splitlines())
    for cname, py in mirrors.items():
        assert int(got[cname]) == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(got[f"{cname}.{f}"]) == getattr(py, f).offset, (cname, f)
    assert int(got["ams_ray_record"]) == tracer.RAY_RECORD.itemsize
    for f in tracer.RAY_RECORD.names:
        assert int(got[f"ams_ray_record.{f}"]) == tracer.RAY_RECORD.fields[f][1], f
    np.testing.assert_equal(tracer.RAY_RECORD.itemsize, 72)
