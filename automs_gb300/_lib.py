"""ctypes binding of libams.so (the C ABI in include/ams.h).

The library is the only compute path: if it is missing or cannot be loaded,
every entry point raises.  There is no CPU fallback.
"""
import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
_lock = threading.Lock()
_lib = None

AMS_OK = 0
STATUS = {1: "bad argument", 2: "out of device memory", 3: "CUDA error", 4: "capacity exceeded",
          6: "numeric range", 7: "internal error"}


class AmsError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"libams status {status} ({STATUS.get(status, '?')}): {msg}")
        self.status = status


class TraceParams(C.Structure):
    _fields_ = [
        ("samples_per_launch", C.c_int), ("launch_x", C.c_int), ("launch_y", C.c_int),
        ("wave_len", C.c_double), ("max_reflection", C.c_int), ("reserve_size", C.c_int),
        ("src_bptype", C.c_int), ("dst_bptype", C.c_int), ("dst_gridsize", C.c_int),
        ("src_r", C.c_float), ("dst_r", C.c_float),
        ("src_dir", C.c_float * 3), ("dst_dir", C.c_float * 3),
        ("strict_grid", C.c_int), ("log_level", C.c_int),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("rx_paths", C.c_ulonglong), ("rx_fail", C.c_ulonglong), ("fwd_records", C.c_ulonglong),
        ("unique_records", C.c_ulonglong), ("unique_paths", C.c_ulonglong),
        ("rounds", C.c_ulonglong), ("tasks", C.c_ulonglong), ("overflow", C.c_ulonglong),
        ("ms_bvh", C.c_float), ("ms_stage1", C.c_float), ("ms_stage2", C.c_float),
        ("ms_total", C.c_float), ("workspace_bytes", C.c_ulonglong),
        ("segments_fwd", C.c_ulonglong), ("segments_bwd", C.c_ulonglong),
        ("ms_stage2_kernel", C.c_float), ("acc_adds", C.c_ulonglong),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_P = C.c_void_p
_I = C.c_int
_F = C.c_float
_D = C.c_double
_S = C.c_size_t
_E = C.c_char_p

SIGNATURES = {
    "ams_version": (C.c_char_p, []),
    "ams_scene_create": (_I, [_P, _I, _P, _P, _I, _P, C.POINTER(_P), _E, _S]),
    "ams_scene_destroy": (None, [_P]),
    "ams_trace_channel": (_I, [_P, C.POINTER(TraceParams), _P, _I, _I, _P, _I, _I, _P, _P, _P,
                               C.POINTER(Stats), _P, _E, _S]),
    "ams_launch_pathtrace": (_I, [_P, _P, _I, _I, _P, _I, _I, _P, _P, _P, _I, _P, _I, _I, _I, _D,
                                  _I, _I, _P, _I, _P, _P, _I, _I, _I, _I, _D, _D,
                                  C.POINTER(Stats), _E, _S]),
    "ams_trace_export_paths": (_I, [_P, _P, _I, C.POINTER(_I), _E, _S]),
    "ams_trace_channel_export": (_I, [_P, C.POINTER(TraceParams), _P, _I, _I, _P, _I, _I, _P, _P,
                                      _P, C.POINTER(Stats), _P, C.c_ulonglong,
                                      C.POINTER(C.c_ulonglong), _P, _E, _S]),
    "ams_objective_fwd_bwd": (_I, [_P, _P, _P, _P, _F, _P, _I, _I, _I, _I, _F, _P, _P, _P, _P,
                                   _P, _P, _P, _E, _S]),
    "ams_objective_fwd_bwd_noalloc": (_I, [_P, _P, _P, _P, _F, _P, _I, _I, _I, _I, _F, _P, _P,
                                           _P, _P, _P, _P, _P, _E, _S]),
    "ams_objective_recv": (_I, [_P, _P, _P, _P, _F, _P, _I, _I, _I, _I, _P, _P, _E, _S]),
    "ams_objective_plan_create": (_I, [_P, _P, _P, _I, _I, _I, _I, _P, C.POINTER(_P), _E, _S]),
    "ams_objective_plan_fwd_bwd": (_I, [_P, _P, _F, _P, _I, _F, _P, _P, _P, _P, _P, _P, _P, _E,
                                        _S]),
    "ams_objective_plan_bytes": (C.c_ulonglong, [_P]),
    "ams_objective_plan_destroy": (None, [_P]),
    "ams_objective_status": (_I, [_P, _P, _E, _S]),
    "ams_objective_plan_create_stacked": (_I, [_P, _P, _I, _I, _I, _I, _P, C.POINTER(_P), _E, _S]),
    "ams_objective_plan_coef_fwd_bwd": (_I, [_P, _P, _P, _I, _F, _P, _P, _P, _P, _P, _P, _E, _S]),
    "ams_cgemm": (_I, [_I, _I, _I, _P, _I, _I, _P, _I, _I, _P, _I, _I, _P, _E, _S]),
    "ams_debug_inject_wait_timeout": (None, [_I]),
    "ams_coverage_db": (_I, [_P, _I, _I, _F, _F, _P, _P, _E, _S]),
    "ams_scratch_bytes": (C.c_ulonglong, []),
    "ams_gemm_bf16": (_I, [_P, _P, _I, _I, _I, _P, _I, _P, _P, _P, _E, _S]),
    "ams_mlp_create": (_I, [_P, _I, _I, C.c_ulonglong, _P, C.POINTER(_P), _E, _S]),
    "ams_mlp_destroy": (None, [_P]),
    "ams_mlp_forward": (_I, [_P, _P, _I, _P, _P, _E, _S]),
    "ams_mlp_train_step": (_I, [_P, _P, _P, _I, _F, _P, _P, _E, _S]),
    "ams_mlp_gradients": (_I, [_P, _P, _P, _I, _P, _P, _P, _E, _S]),
    "ams_mlp_params": (_I, [_P, _P, _I, C.POINTER(C.c_longlong), _P, _E, _S]),
}


def lib_path():
    return os.path.join(_HERE, "_build", "libams.so")


def lib():
    """Load libams.so, building it first if it is absent and nvcc exists."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not os.path.exists(path):
            from . import build as _build
            _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"libams.so is missing at {path}; the CUDA path cannot run")
        L = C.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def call(name, *args):
    """Call an entry point that ends with (errbuf, errlen); raise on failure."""
    buf = C.create_string_buffer(1024)
    rc = getattr(lib(), name)(*args, buf, C.sizeof(buf))
    if rc != AMS_OK:
        raise AmsError(rc, buf.value.decode(errors="replace"))
    return rc
