"""Channel tracer front end: the drop-in for build_channel / build_channels.

Mirrors go.py:623-767 (build_channel) and go.py:1135-1247 (build_channels)
with the same signatures and dict keys; the OptiX op behind them
(torch.ops.pathtrace.torch_launch_pathtrace, optixPathTracer.cpp:781-870)
is replaced by libams.so (include/ams.h).  Tensors live on the current CUDA
device; results are complex64 [n_src, n_dst].
"""
import ctypes as C

import numpy as np
import torch

from . import scenes
from ._lib import Stats, TraceParams, call, lib


def _f32(x, device="cuda"):
    return torch.as_tensor(x, dtype=torch.float32, device=device).contiguous()


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def make_params(launch_x=100, launch_y=100, wave_len=scenes.WAVE_LEN_60GHZ, max_reflection=4,
                reserve_size=100, src_bptype=2, dst_bptype=0, dst_gridsize=5, src_r=0.5e-5,
                dst_r=0.06, src_dir=(0.0, 0.0, 0.0), dst_dir=(0.0, 0.0, 0.0),
                samples_per_launch=1, strict_grid=0, log_level=0):
    p = TraceParams()
    p.samples_per_launch = int(samples_per_launch)
    p.launch_x, p.launch_y = int(launch_x), int(launch_y)
    p.wave_len = float(wave_len)
    p.max_reflection = int(max_reflection)
    p.reserve_size = int(reserve_size)
    p.src_bptype, p.dst_bptype = int(src_bptype), int(dst_bptype)
    p.dst_gridsize = int(dst_gridsize)
    p.src_r, p.dst_r = float(src_r), float(dst_r)
    sd = torch.as_tensor(src_dir, dtype=torch.float32).flatten().cpu()
    dd = torch.as_tensor(dst_dir, dtype=torch.float32).flatten().cpu()
    for i in range(3):
        p.src_dir[i] = float(sd[i])
        p.dst_dir[i] = float(dd[i])
    p.strict_grid = int(strict_grid)
    p.log_level = int(log_level)
    return p


def params_from_dict(d):
    keys = ("launch_x", "launch_y", "wave_len", "max_reflection", "reserve_size", "src_bptype",
            "dst_bptype", "dst_gridsize", "src_r", "dst_r", "src_dir", "dst_dir",
            "samples_per_launch", "strict_grid", "log_level")
    return make_params(**{k: d[k] for k in keys if k in d})


class Scene:
    """Triangles + materials with their BVH kept on the GPU across calls."""

    def __init__(self, tris, mat, mat_prop):
        lib()
        self.tris = _f32(tris).reshape(-1, 9)
        self.mat = torch.as_tensor(mat, dtype=torch.int32, device="cuda").contiguous().reshape(-1)
        self.mat_prop = _f32(mat_prop).reshape(-1, 19)
        if self.mat.numel() != self.tris.shape[0]:
            raise ValueError("mat must have one entry per triangle")
        if self.tris.shape[0] and int(self.mat.max()) >= self.mat_prop.shape[0]:
            raise ValueError("material index out of range of mat_prop")
        self._h = C.c_void_p()
        call("ams_scene_create", _ptr(self.tris), self.tris.shape[0], _ptr(self.mat),
             _ptr(self.mat_prop), self.mat_prop.shape[0], _stream(), C.byref(self._h))

    @classmethod
    def from_folder(cls, scene_folder, blackhole_buffer=(), reflector_buffer=(), door_buffer=()):
        t, m, mp = scenes.load_scene_folder(scene_folder, blackhole_buffer, reflector_buffer,
                                            door_buffer)
        return cls(t, m, mp)

    def close(self):
        if self._h:
            lib().ams_scene_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trace(self, src, dst, params, result=None, src_aabb=None, dst_aabb=None):
        """Accumulate the channel src -> dst into result [S, R, 2] float32
        (allocated zeroed if None).  src [s0, s1, 3], dst [n0, n1, 3].
        Returns (result, stats dict)."""
        if isinstance(params, dict):
            params = params_from_dict(params)
        src = _f32(src)
        dst = _f32(dst)
        if src.dim() != 3 or dst.dim() != 3 or src.shape[-1] != 3 or dst.shape[-1] != 3:
            raise ValueError("src and dst must be [n0, n1, 3]")
        s0, s1 = src.shape[0], src.shape[1]
        n0, n1 = dst.shape[0], dst.shape[1]
        if result is None:
            result = torch.zeros(s0 * s1, n0 * n1, 2, dtype=torch.float32, device="cuda")
        elif (result.dtype != torch.float32 or not result.is_cuda or not result.is_contiguous()
              or result.numel() != s0 * s1 * n0 * n1 * 2):
            raise ValueError("result must be a contiguous CUDA float32 [S, R, 2] tensor")
        sa = _f32(src_aabb) if src_aabb is not None else None
        da = _f32(dst_aabb) if dst_aabb is not None else None
        st = Stats()
        call("ams_trace_channel", self._h, C.byref(params), _ptr(src), s0, s1, _ptr(dst), n0, n1,
             _ptr(sa), _ptr(da), _ptr(result), C.byref(st), _stream())
        return result, st.as_dict()

    def trace_export(self, src, dst, params, max_records=None):
        """trace() with every backward ray of stage 2 recorded (the
        reference's EXPORT_TASKINFO dump, optixPathTracer.h:40-52): returns
        (result, stats, records) with records a numpy structured array of
        RAY_RECORD (see ams_ray_record in include/ams.h), in round, task, Rx,
        Tx order.  max_records defaults to what a first plain trace counts."""
        if isinstance(params, dict):
            params = params_from_dict(params)
        if max_records is None:
            _, st = self.trace(src, dst, params)
            max_records = st["rx_paths"] + st["rx_fail"]
            max_records = max(int(max_records * 1.5) + 1024, 1024)
        src = _f32(src)
        dst = _f32(dst)
        s0, s1 = src.shape[0], src.shape[1]
        n0, n1 = dst.shape[0], dst.shape[1]
        result = torch.zeros(s0 * s1, n0 * n1, 2, dtype=torch.float32, device="cuda")
        rec = torch.empty(int(max_records) * RAY_RECORD.itemsize, dtype=torch.uint8, device="cuda")
        n = C.c_ulonglong()
        st = Stats()
        call("ams_trace_channel_export", self._h, C.byref(params), _ptr(src), s0, s1, _ptr(dst),
             n0, n1, C.c_void_p(0), C.c_void_p(0), _ptr(result), C.byref(st), _ptr(rec),
             C.c_ulonglong(int(max_records)), C.byref(n), _stream())
        k = min(int(n.value), int(max_records))
        out = rec[:k * RAY_RECORD.itemsize].cpu().numpy().view(RAY_RECORD)
        return result, st.as_dict(), out

    def export_paths(self, max_paths=1 << 22):
        """Unique path keys of the last trace, int32 [P, 14], sorted in the
        order of the reference's std::map<Path, int> (optixPathTracer.h:28-38)."""
        n = C.c_int()
        call("ams_trace_export_paths", self._h, C.c_void_p(0), 0, C.byref(n))
        out = np.zeros((max(n.value, 1), 14), np.int32)
        call("ams_trace_export_paths", self._h, C.c_void_p(out.ctypes.data), n.value, C.byref(n))
        return sort_paths(out[: n.value])


# ams_ray_record of include/ams.h (72 bytes)
RAY_RECORD = np.dtype([("src", "<i4"), ("dst", "<i4"), ("path", "<i4"), ("traced", "<i4"),
                       ("successful", "<i4"), ("hit_cnt", "<i4"), ("launch_angle", "<f4"),
                       ("receive_angle", "<f4"), ("loss", "<f4"), ("pad0", "<f4"),
                       ("phase", "<f8"), ("hit_loss_idx", "<i4", 5), ("pad1", "<i4")])
assert RAY_RECORD.itemsize == 72


def sort_paths(paths):
    """Order path keys like operator< of optixPathTracer.h:28-38 (hit count,
    reflect mask, then the 12 matrix entries as floats)."""
    if len(paths) == 0:
        return paths
    f = paths[:, :12].view(np.float32)
    keys = [f[:, k] for k in range(11, -1, -1)] + [paths[:, 13], paths[:, 12]]
    return paths[np.lexsort(keys)]


def trace_channel(tris, mat, mat_prop, src, dst, params):
    """One-shot trace on arrays: returns (H complex64 [S, R] on the GPU, stats)."""
    sc = Scene(tris, mat, mat_prop)
    try:
        res, st = sc.trace(src, dst, params)
    finally:
        sc.close()
    return torch.complex(res[..., 0], res[..., 1]), st


def launch_pathtrace(result, src, dst, src_aabb_buffer, dst_aabb_buffer, scene_triangle_buffer,
                     mat, samples_per_launch, launch_x, launch_y, wave_len, max_reflection,
                     reserve_size, mat_prop, src_dir, dst_dir, optix_log_level, src_bptype,
                     dst_bptype, dst_gridsize, src_r, dst_r):
    """Same arguments as torch.ops.pathtrace.torch_launch_pathtrace
    (optixPathTracer.cpp:781-790); accumulates into `result` [S, R, 2].
    Unlike the reference, errors raise instead of being printed."""
    for t, name in ((result, "result"), (src, "src"), (dst, "dst"), (scene_triangle_buffer, "scene"),
                    (mat, "mat"), (mat_prop, "mat_prop")):
        if not (t.is_cuda and t.is_contiguous()):
            raise ValueError(f"{name} must be a contiguous CUDA tensor")
    sd = np.ascontiguousarray(torch.as_tensor(src_dir).cpu().numpy(), np.float32)
    dd = np.ascontiguousarray(torch.as_tensor(dst_dir).cpu().numpy(), np.float32)
    st = Stats()
    n_mat = mat_prop.numel() // 19
    call("ams_launch_pathtrace", _ptr(result), _ptr(src), src.shape[0], src.shape[1], _ptr(dst),
         dst.shape[0], dst.shape[1], _ptr(src_aabb_buffer.contiguous()),
         _ptr(dst_aabb_buffer.contiguous()), _ptr(scene_triangle_buffer),
         scene_triangle_buffer.numel() // 9, _ptr(mat), int(samples_per_launch), int(launch_x),
         int(launch_y), float(wave_len), int(max_reflection), int(reserve_size), _ptr(mat_prop),
         n_mat, C.c_void_p(sd.ctypes.data), C.c_void_p(dd.ctypes.data), int(optix_log_level),
         int(src_bptype), int(dst_bptype), int(dst_gridsize), float(src_r), float(dst_r),
         C.byref(st))
    return st.as_dict()


def build_channel(src, dst, src_dir, dst_dir, src_bptype, dst_bptype, wave_len, scene_folder,
                  max_reflection=4, dst_radius=0.06, src_radius=0.5e-5, samples_per_launch=1,
                  reserved_size=100, blackhole_buffer=[], reflector_buffer=[], door_buffer=[],
                  dst_gridsize=5, launch=(100, 100), scene=None, return_stats=False,
                  return_paths=False):
    """build_channel of go.py:623-767.  Extra keywords: `launch` (the
    reference hard-codes 100 x 100, go.py:739-740), `scene` (a prebuilt
    Scene instead of the folder), `return_stats` (also return the trace's
    counters), `return_paths` (also return its ordered path list)."""
    own = scene is None
    if own:
        scene = Scene.from_folder(scene_folder, blackhole_buffer, reflector_buffer, door_buffer)
    src = _f32(src)
    dst = _f32(dst)
    p = make_params(launch[0], launch[1], wave_len, max_reflection, reserved_size, src_bptype,
                    dst_bptype, dst_gridsize, src_radius, dst_radius, src_dir, dst_dir,
                    samples_per_launch)
    src_buffer = torch.cat([src - src_radius, src + src_radius], dim=-1)
    dst_buffer = torch.cat([dst - dst_radius, dst + dst_radius], dim=-1)
    paths = None
    try:
        res, st = scene.trace(src, dst, p, src_aabb=src_buffer, dst_aabb=dst_buffer)
        if return_paths:
            paths = scene.export_paths()
    finally:
        if own:
            scene.close()
    H = torch.complex(res[..., 0], res[..., 1])
    out = (H,) + ((st,) if return_stats else ()) + ((paths,) if return_paths else ())
    return out if len(out) > 1 else H


def build_channels(src, dst, ms_list, ap_dir, scene_folder, wave_len, max_reflection,
                   reflector_buffer=[], door_buffer=[], launch=(100, 100), details=None):
    """build_channels of go.py:1135-1247: keys src_to_dst, src_to_ms{i},
    ms{i}_to_dst, ms{i}_to_ms{j} in the reference's order; AP beam type 2,
    MS 1, Rx 0; the other metasurfaces are blackholes in each trace.  With a
    dict as `details`, details[key] = (counters, ordered path list) of each
    trace."""
    dir_no = torch.tensor([0, 0, 0], dtype=torch.float32)
    if isinstance(ap_dir, list):
        ap_dir = torch.tensor(ap_dir, dtype=torch.float32)
    n = len(ms_list)
    ch = {}
    want = details is not None
    kw = dict(reflector_buffer=reflector_buffer, door_buffer=door_buffer, launch=launch,
              return_stats=want, return_paths=want)

    def put(key, out):
        if want:
            ch[key], st, paths = out
            details[key] = (st, paths)
        else:
            ch[key] = out
    put("src_to_dst", build_channel(src, dst, ap_dir, dir_no, 2, 0, wave_len, scene_folder,
                                    max_reflection,
                                    blackhole_buffer=[ms_list[i].blackhole for i in range(n)],
                                    **kw))
    for i in range(n):
        others = [ms_list[k].blackhole for k in range(n) if k != i]
        put("src_to_ms{%d}" % i, build_channel(src, ms_list[i].pos, ap_dir, ms_list[i].recv_dir,
                                               2, 1, wave_len, scene_folder, max_reflection,
                                               blackhole_buffer=others, **kw))
        put("ms{%d}_to_dst" % i, build_channel(ms_list[i].pos, dst, ms_list[i].send_dir, dir_no,
                                               1, 0, wave_len, scene_folder, max_reflection,
                                               blackhole_buffer=others, **kw))
        for j in range(i + 1, n):
            bh = [ms_list[k].blackhole for k in range(n) if k != i and k != j]
            put("ms{%d}_to_ms{%d}" % (i, j), build_channel(
                ms_list[i].pos, ms_list[j].pos, ms_list[i].send_dir, ms_list[j].recv_dir, 1, 1,
                wave_len, scene_folder, max_reflection, blackhole_buffer=bh, **kw))
    return ch


def coverage_db(H, threshold=-150.0, offset=0.0):
    """20 log10 |sum_src H| per Rx, NaN -> threshold, clamped at threshold
    (draw_channel + amp_data_to_image, go.py:849-851, 944-964)."""
    H = H.contiguous()
    if H.dtype != torch.complex64 or not H.is_cuda:
        raise ValueError("H must be a complex64 CUDA tensor")
    S, R = H.shape
    out = torch.empty(R, dtype=torch.float32, device=H.device)
    call("ams_coverage_db", _ptr(H), S, R, float(threshold), float(offset), _ptr(out), _stream())
    return out
