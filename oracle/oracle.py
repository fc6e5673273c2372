"""ctypes front end of the C oracle and of the reference harness.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(HERE, "ref_harness"))
import build_oracle  # noqa: E402
import build_ref  # noqa: E402


class OrcParams(C.Structure):
    _fields_ = [
        ("samples_per_launch", C.c_int), ("launch_x", C.c_int), ("launch_y", C.c_int),
        ("wave_len", C.c_double), ("max_reflection", C.c_int), ("reserve_size", C.c_int),
        ("src_bptype", C.c_int), ("dst_bptype", C.c_int), ("dst_gridsize", C.c_int),
        ("src_r", C.c_float), ("dst_r", C.c_float),
        ("src_dir", C.c_float * 3), ("dst_dir", C.c_float * 3), ("strict_grid", C.c_int),
    ]


class OrcStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "rx_paths", "rx_fail", "fwd_records", "unique_records", "unique_paths",
        "rounds", "tasks", "overflow", "farfield")]


_lib = None
_ref = None
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build_oracle.build_oracle())
        _lib.orc_trace_channel.restype = C.c_int
        _lib.orc_tea4.restype = C.c_uint32
        _lib.orc_tea4.argtypes = [C.c_uint32, C.c_uint32]
        _lib.orc_rnd.restype = C.c_float
        _lib.orc_rnd.argtypes = [C.POINTER(C.c_uint32)]
        _lib.orc_rand_dir.argtypes = [C.POINTER(C.c_uint32), C.c_uint32, C.c_uint32,
                                      C.c_int, C.c_int, _f32p]
        _lib.orc_sincos.argtypes = [C.c_float, _f32p]
        _lib.orc_theta_id.restype = C.c_int
        _lib.orc_theta_id.argtypes = [C.c_float]
        _lib.orc_beampattern.restype = C.c_float
        _lib.orc_beampattern.argtypes = [_f32p, _f32p, C.c_int]
        _lib.orc_intersect_tri.restype = C.c_float
        _lib.orc_intersect_tri.argtypes = [_f32p] * 5
    return _lib


def ref_available():
    return build_ref.available()


def ref_lib():
    global _ref
    if _ref is None:
        path = build_ref.build_ref()
        if path is None:
            raise RuntimeError("reference sources are not mounted here")
        _ref = C.CDLL(path)
        _ref.ref_tea4.restype = C.c_uint32
        _ref.ref_tea4.argtypes = [C.c_uint32, C.c_uint32]
        _ref.ref_rnd.restype = C.c_float
        _ref.ref_rnd.argtypes = [C.POINTER(C.c_uint32)]
        _ref.ref_rand_dir.argtypes = [C.POINTER(C.c_uint32), C.c_uint32, C.c_uint32,
                                      C.c_int, C.c_int, _f32p]
        _ref.ref_beampattern.restype = C.c_float
        _ref.ref_beampattern.argtypes = [_f32p, _f32p, C.c_int]
        _ref.ref_image_update.argtypes = [_f32p, _f32p, _f32p]
        _ref.ref_theta_id.restype = C.c_int
        _ref.ref_theta_id.argtypes = [C.c_float]
    return _ref


def _params(p):
    o = OrcParams()
    o.samples_per_launch = int(p.get("samples_per_launch", 1))
    o.launch_x = int(p["launch_x"])
    o.launch_y = int(p["launch_y"])
    o.wave_len = float(p["wave_len"])
    o.max_reflection = int(p["max_reflection"])
    o.reserve_size = int(p.get("reserve_size", 100))
    o.src_bptype = int(p["src_bptype"])
    o.dst_bptype = int(p["dst_bptype"])
    o.dst_gridsize = int(p.get("dst_gridsize", 5))
    o.src_r = float(p.get("src_r", 0.5e-5))
    o.dst_r = float(p.get("dst_r", 0.06))
    for i in range(3):
        o.src_dir[i] = float(p["src_dir"][i])
        o.dst_dir[i] = float(p["dst_dir"][i])
    o.strict_grid = int(p.get("strict_grid", 0))
    return o


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def aabbs(pos, r):
    """cat([pos - r, pos + r], -1) in float32, as go.py:669-670 builds it."""
    pos = _c(pos, np.float32).reshape(-1, 3)
    r32 = np.float32(r)
    return np.concatenate([pos - r32, pos + r32], axis=-1).astype(np.float32)


def trace_channel(tris, mat, mat_prop, src, dst, params, nthreads=0, max_paths=1 << 20,
                  src_box=None, dst_box=None):
    """Oracle build_channel.  src [s0,s1,3], dst [n0,n1,3]; src_box / dst_box
    (float32 [n, 6]) default to pos -/+ r.  Returns (H complex64 [S,R],
    stats dict, paths int32 [P,14])."""
    L = lib()
    tris = _c(tris, np.float32).reshape(-1, 9)
    mat = _c(mat, np.int32).reshape(-1)
    mat_prop = _c(mat_prop, np.float32).reshape(-1, 19)
    src = _c(src, np.float32)
    dst = _c(dst, np.float32)
    n_src = src.size // 3
    n0, n1 = dst.shape[0], dst.shape[1]
    n_dst = n0 * n1
    src_box = (aabbs(src, params.get("src_r", 0.5e-5)) if src_box is None
               else _c(src_box, np.float32).reshape(-1, 6))
    dst_box = (aabbs(dst, params.get("dst_r", 0.06)) if dst_box is None
               else _c(dst_box, np.float32).reshape(-1, 6))
    res = np.zeros((n_src, n_dst, 2), np.float32)
    st = OrcStats()
    paths = np.zeros((max_paths, 14), np.int32)
    pp = _params(params)
    rc = L.orc_trace_channel(
        tris.ctypes.data_as(C.c_void_p), C.c_int(tris.shape[0]),
        mat.ctypes.data_as(C.c_void_p), mat_prop.ctypes.data_as(C.c_void_p),
        C.c_int(mat_prop.shape[0]), src.ctypes.data_as(C.c_void_p), C.c_int(n_src),
        dst.ctypes.data_as(C.c_void_p), C.c_int(n0), C.c_int(n1),
        src_box.ctypes.data_as(C.c_void_p), dst_box.ctypes.data_as(C.c_void_p),
        C.byref(pp), res.ctypes.data_as(C.c_void_p), C.byref(st),
        paths.ctypes.data_as(C.c_void_p), C.c_int(max_paths), C.c_int(nthreads))
    if rc != 0:
        raise RuntimeError(f"orc_trace_channel failed with status {rc}")
    stats = {k: int(getattr(st, k)) for k, _ in OrcStats._fields_}
    npaths = min(stats["unique_paths"], max_paths)
    return (res[..., 0] + 1j * res[..., 1]).astype(np.complex64), stats, paths[:npaths].copy()


def ref_trace_channel(tris, mat, mat_prop, src, dst, params, max_paths=1 << 20, src_box=None,
                      dst_box=None):
    """The reference device programs run on the CPU (oracle/_ref).  Same
    return convention as trace_channel; stats has rx_paths, rx_fail,
    fwd_records, unique_records, unique_paths, rounds.  src_box / dst_box
    (float32 [n, 6]) default to pos -/+ r."""
    R = ref_lib()
    tris = _c(tris, np.float32).reshape(-1, 9)
    mat = _c(mat, np.int32).reshape(-1)
    mat_prop = _c(mat_prop, np.float32).reshape(-1, 19)
    src = _c(src, np.float32)
    dst = _c(dst, np.float32)
    s0, s1 = src.shape[0], src.shape[1]
    n0, n1 = dst.shape[0], dst.shape[1]
    src_box = (aabbs(src, params.get("src_r", 0.5e-5)) if src_box is None
               else _c(src_box, np.float32).reshape(-1, 6))
    dst_box = (aabbs(dst, params.get("dst_r", 0.06)) if dst_box is None
               else _c(dst_box, np.float32).reshape(-1, 6))
    res = np.zeros((s0 * s1, n0 * n1, 2), np.float32)
    stats = np.zeros(2, np.uint64)
    counts = np.zeros(4, np.int64)
    paths = np.zeros((max_paths, 14), np.int32)
    sd = _c(params["src_dir"], np.float32)
    dd = _c(params["dst_dir"], np.float32)
    vp = C.c_void_p
    rc = R.ref_trace_channel(
        vp(tris.ctypes.data), C.c_int(tris.shape[0]), vp(mat.ctypes.data),
        vp(mat_prop.ctypes.data), vp(src.ctypes.data), C.c_int(s0), C.c_int(s1),
        vp(dst.ctypes.data), C.c_int(n0), C.c_int(n1),
        vp(src_box.ctypes.data), vp(dst_box.ctypes.data),
        C.c_int(int(params.get("samples_per_launch", 1))), C.c_int(int(params["launch_x"])),
        C.c_int(int(params["launch_y"])), C.c_double(float(params["wave_len"])),
        C.c_int(int(params["max_reflection"])), C.c_int(int(params.get("reserve_size", 100))),
        vp(sd.ctypes.data), vp(dd.ctypes.data), C.c_int(int(params["src_bptype"])),
        C.c_int(int(params["dst_bptype"])), C.c_int(int(params.get("dst_gridsize", 5))),
        C.c_double(float(params.get("src_r", 0.5e-5))), C.c_double(float(params.get("dst_r", 0.06))),
        vp(res.ctypes.data), vp(stats.ctypes.data), vp(counts.ctypes.data),
        vp(paths.ctypes.data), C.c_int(max_paths))
    if rc != 0:
        raise RuntimeError(f"ref_trace_channel failed with status {rc}")
    st = {"rx_paths": int(stats[0]), "rx_fail": int(stats[1]), "fwd_records": int(counts[0]),
          "unique_records": int(counts[1]), "unique_paths": int(counts[2]), "rounds": int(counts[3])}
    npaths = min(st["unique_paths"], max_paths)
    return (res[..., 0] + 1j * res[..., 1]).astype(np.complex64), st, paths[:npaths].copy()
