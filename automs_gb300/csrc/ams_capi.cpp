// ams_capi.cpp -- host orchestration behind the C ABI of include/ams.h.
//
// Replaces optixPathTracer.cpp:70-360 (launch parameters, two-stage launch,
// host dedup and flood-fill scheduler) and :781-870 (the Torch op):
//   * the triangle BVH is built once per scene and kept across calls;
//   * the Tx/Rx sphere BVHs, path table and bitmaps live in one device
//     workspace per scene that grows to the largest call and is reused;
//   * the host loop only reads a handful of device counters per round;
//   * every failure is returned as a status with a message.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ams.h"
#include "bvh_sah.h"
#include "lbvh.h"
#include "trace.h"

namespace {

void set_err(char *buf, size_t len, const char *fmt, ...) {
  if (!buf || len == 0) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, len, fmt, ap);
  va_end(ap);
}

// Device blocks of destroyed scenes kept for the next scene on the device.
// cudaFree synchronises the whole device and cudaMalloc costs tens of
// microseconds; a caller that builds a scene per channel (as build_channel,
// go.py:679-767, does) would pay both on every call.  Blocks are kept in
// size classes per device.  A scene hands its blocks back only
// when it is destroyed, after its last call returned (every scene call
// synchronises its stream), so no GPU work still uses them.  On an
// allocation failure the device's cached blocks are released and the
// allocation retried once.
struct BlockPool {
  std::mutex mu;
  std::multimap<std::pair<int, size_t>, void *> free_blocks;
  std::vector<void *> free_pinned;  // HostCounters blocks (pinned host memory)
};
BlockPool &block_pool() {
  static BlockPool *p = new BlockPool();  // lives until the process exits
  return *p;
}
// power-of-two classes from 4 KB; from 1 MB on, sixteenths of the power of
// two above the request (at most 12.5% over: a 4.3 GB accumulator takes
// 4.8 GB, not 8 GB)
size_t size_class(size_t bytes) {
  size_t c = 4096;
  while (c < bytes) c <<= 1;
  if (c >= ((size_t)1 << 20)) {
    const size_t step = c / 16;
    c = (bytes + step - 1) / step * step;
  }
  return c;
}
cudaError_t pool_malloc(void **out, size_t bytes) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const size_t c = size_class(bytes);
  BlockPool &bp = block_pool();
  {
    std::lock_guard<std::mutex> lk(bp.mu);
    auto it = bp.free_blocks.find({dev, c});
    if (it != bp.free_blocks.end()) {
      *out = it->second;
      bp.free_blocks.erase(it);
      return cudaSuccess;
    }
  }
  e = cudaMalloc(out, c);
  if (e == cudaErrorMemoryAllocation) {
    (void)cudaGetLastError();
    std::vector<void *> rel;
    {
      std::lock_guard<std::mutex> lk(bp.mu);
      for (auto it = bp.free_blocks.begin(); it != bp.free_blocks.end();) {
        if (it->first.first == dev) { rel.push_back(it->second); it = bp.free_blocks.erase(it); }
        else ++it;
      }
    }
    for (void *q : rel) cudaFree(q);
    e = cudaMalloc(out, c);
  }
  if (e != cudaSuccess) *out = nullptr;
  return e;
}
void pool_free(void *ptr, size_t bytes, int dev) {
  if (!ptr) return;
  BlockPool &bp = block_pool();
  std::lock_guard<std::mutex> lk(bp.mu);
  bp.free_blocks.insert({{dev, size_class(bytes)}, ptr});
}

template <class T>
cudaError_t pool_malloc_pinned(T **out) {
  BlockPool &bp = block_pool();
  {
    std::lock_guard<std::mutex> lk(bp.mu);
    if (!bp.free_pinned.empty()) {
      *out = static_cast<T *>(bp.free_pinned.back());
      bp.free_pinned.pop_back();
      return cudaSuccess;
    }
  }
  return cudaMallocHost(reinterpret_cast<void **>(out), sizeof(T));
}
void pool_free_pinned(void *ptr) {
  if (!ptr) return;
  BlockPool &bp = block_pool();
  std::lock_guard<std::mutex> lk(bp.mu);
  bp.free_pinned.push_back(ptr);
}

struct Arena {
  char *base = nullptr;
  size_t cap = 0, used = 0, high = 0;
  int dev = 0;
  ~Arena() { pool_free(base, cap, dev); }
  cudaError_t ensure(size_t bytes) {
    if (bytes <= cap) return cudaSuccess;
    if (base) { pool_free(base, cap, dev); base = nullptr; cap = 0; }
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = pool_malloc(reinterpret_cast<void **>(&base), bytes);
    if (e != cudaSuccess) { base = nullptr; return e; }
    cap = size_class(bytes);
    high = std::max(high, bytes);
    return cudaSuccess;
  }
  void reset() { used = 0; }
  template <class T> T *take(size_t count) {
    size_t b = (sizeof(T) * count + 255) & ~(size_t)255;
    T *p = reinterpret_cast<T *>(base + used);
    used += b;
    return p;
  }
};

size_t al(size_t v) { return (v + 255) & ~(size_t)255; }

struct HostCounters {
  unsigned long long ctr[16];
  unsigned err;
};

}  // namespace

struct ams_scene {
  int device = 0;
  int n_tri = 0, n_mat = 0;
  float *tris = nullptr;
  int *mat = nullptr;
  float *mat_prop = nullptr;
  char *bvh_out = nullptr;
  Lbvh bvh;
  Arena ws;       // per-call workspace
  Arena tasks;    // task list of a round (grown on demand)
  int tab_log2 = 14;
  HostCounters *hc = nullptr;  // pinned
  TraceDev last{};
  bool have_last = false;
  float ms_bvh_scene = 0.f;
  cudaEvent_t k2[2] = {nullptr, nullptr};
  size_t tris_bytes = 0, mat_bytes = 0, mat_prop_bytes = 0, bvh_bytes = 0;
  ~ams_scene() {
    for (auto &e : k2)
      if (e) cudaEventDestroy(e);
    pool_free(tris, tris_bytes, device);
    pool_free(mat, mat_bytes, device);
    pool_free(mat_prop, mat_prop_bytes, device);
    pool_free(bvh_out, bvh_bytes, device);
    pool_free_pinned(hc);
  }
};

#define CK(call)                                                                         \
  do {                                                                                   \
    cudaError_t _e = (call);                                                             \
    if (_e != cudaSuccess) {                                                             \
      set_err(errbuf, errlen, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(_e),   \
              __FILE__, __LINE__);                                                       \
      return _e == cudaErrorMemoryAllocation ? AMS_ERR_OOM : AMS_ERR_CUDA;               \
    }                                                                                    \
  } while (0)

namespace {
// Timing between two recorded events, 0 when it cannot be read.  The error
// such a call returns is also left as the thread's last error, which a later
// cudaGetLastError() (after our own launches) would misreport: clear it.
float elapsed_ms(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    (void)cudaGetLastError();
    ms = 0.f;
  }
  return ms;
}
// An entry point starts with no pending error from runtime calls made
// elsewhere on this thread (its own launches are checked with
// cudaGetLastError()).
void clear_stale_error() { (void)cudaGetLastError(); }
}  // namespace

extern "C" {

const char *ams_version(void) { return "automs-gb300 0.1 (sm_103a)"; }

ams_status ams_scene_create(const float *tris, int n_tri, const int *mat, const float *mat_prop,
                            int n_mat, void *stream, ams_scene **out, char *errbuf,
                            size_t errlen) {
  clear_stale_error();
  if (!out) { set_err(errbuf, errlen, "out is NULL"); return AMS_ERR_ARG; }
  *out = nullptr;
  if (n_tri < 0 || n_mat < 0 || (n_tri > 0 && (!tris || !mat)) || (n_mat > 0 && !mat_prop) ||
      (n_tri > 0 && n_mat == 0)) {
    set_err(errbuf, errlen, "bad scene arrays (n_tri=%d, n_mat=%d)", n_tri, n_mat);
    return AMS_ERR_ARG;
  }
  if (n_tri > (1 << 28)) { set_err(errbuf, errlen, "too many triangles"); return AMS_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  ams_scene *s = new ams_scene();
  cudaGetDevice(&s->device);
  s->n_tri = n_tri;
  s->n_mat = n_mat;
  auto fail = [&](ams_status code) { delete s; return code; };
  cudaError_t e;
  if ((e = cudaEventCreate(&s->k2[0])) != cudaSuccess || (e = cudaEventCreate(&s->k2[1])) != cudaSuccess ||
      (e = pool_malloc_pinned(&s->hc)) != cudaSuccess) {
    set_err(errbuf, errlen, "cudaMallocHost: %s", cudaGetErrorString(e));
    return fail(AMS_ERR_OOM);
  }
  s->tris_bytes = sizeof(float) * 9 * (size_t)std::max(n_tri, 1);
  s->mat_bytes = sizeof(int) * (size_t)std::max(n_tri, 1);
  s->mat_prop_bytes = sizeof(float) * 19 * (size_t)std::max(n_mat, 1);
  s->bvh_bytes = lbvh_output_bytes(n_tri);
  if ((e = pool_malloc(reinterpret_cast<void **>(&s->tris), s->tris_bytes)) != cudaSuccess ||
      (e = pool_malloc(reinterpret_cast<void **>(&s->mat), s->mat_bytes)) != cudaSuccess ||
      (e = pool_malloc(reinterpret_cast<void **>(&s->mat_prop), s->mat_prop_bytes)) !=
          cudaSuccess ||
      (e = pool_malloc(reinterpret_cast<void **>(&s->bvh_out), s->bvh_bytes)) != cudaSuccess) {
    set_err(errbuf, errlen, "scene allocation: %s", cudaGetErrorString(e));
    return fail(AMS_ERR_OOM);
  }
  // host copy of the triangles: validated here, and the input of the SAH
  // builder for large scenes
  std::vector<float> ht(9 * (size_t)n_tri);
  if (n_tri > 0) {
    // material ids index mat_prop rows, vertices must be finite: check on
    // the host once (the reference accepts both and fails silently)
    // (on the caller's stream, after whatever produced the arrays there)
    std::vector<int> hm((size_t)n_tri);
    if ((e = cudaMemcpyAsync(hm.data(), mat, sizeof(int) * (size_t)n_tri, cudaMemcpyDeviceToHost,
                             st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(ht.data(), tris, sizeof(float) * 9 * (size_t)n_tri,
                             cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess) {
      set_err(errbuf, errlen, "reading the scene arrays: %s", cudaGetErrorString(e));
      return fail(AMS_ERR_CUDA);
    }
    for (int i = 0; i < n_tri; i++)
      if (hm[i] < 0 || hm[i] >= n_mat) {
        set_err(errbuf, errlen, "mat[%d] = %d is outside [0, %d)", i, hm[i], n_mat);
        return fail(AMS_ERR_ARG);
      }
    for (size_t i = 0; i < ht.size(); i++)
      if (!std::isfinite(ht[i])) {
        set_err(errbuf, errlen, "triangle %zu has a non-finite vertex coordinate", i / 9);
        return fail(AMS_ERR_ARG);
      }
    if ((e = cudaMemcpyAsync(s->tris, tris, sizeof(float) * 9 * (size_t)n_tri,
                             cudaMemcpyDeviceToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(s->mat, mat, sizeof(int) * (size_t)n_tri, cudaMemcpyDeviceToDevice,
                             st)) != cudaSuccess) {
      set_err(errbuf, errlen, "copying the scene arrays: %s", cudaGetErrorString(e));
      return fail(AMS_ERR_CUDA);
    }
  }
  if (n_mat > 0 &&
      (e = cudaMemcpyAsync(s->mat_prop, mat_prop, sizeof(float) * 19 * (size_t)n_mat,
                           cudaMemcpyDeviceToDevice, st)) != cudaSuccess) {
    set_err(errbuf, errlen, "copying mat_prop: %s", cudaGetErrorString(e));
    return fail(AMS_ERR_CUDA);
  }
  if ((e = s->ws.ensure(lbvh_scratch_bytes(n_tri) + 1024)) != cudaSuccess) {
    set_err(errbuf, errlen, "BVH scratch: %s", cudaGetErrorString(e));
    return fail(AMS_ERR_OOM);
  }
  auto t0 = std::chrono::steady_clock::now();
  if (n_tri >= AMS_SAH_MIN_TRIS) {
    // large scene: SAH hierarchy built on the host from the host copy of the
    // triangles (traversal visits 20-40% fewer nodes than with the LBVH)
    std::vector<BvhNode> hn;
    std::vector<int> hp;
    char msg[160] = {0};
    if (!sah_build_triangles(ht.data(), n_tri, hn, hp, msg, sizeof msg)) {
      set_err(errbuf, errlen, "triangle BVH build: %s", msg);
      return fail(AMS_ERR_INTERNAL);
    }
    if ((e = lbvh_from_host(s->bvh, s->tris, n_tri, hn.data(), hp.data(), s->bvh_out, st)) !=
            cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess) {
      set_err(errbuf, errlen, "triangle BVH upload: %s", cudaGetErrorString(e));
      return fail(AMS_ERR_CUDA);
    }
  } else if ((e = lbvh_build_triangles(s->bvh, s->tris, n_tri, s->ws.base, s->bvh_out, st)) !=
                 cudaSuccess ||
             (e = cudaStreamSynchronize(st)) != cudaSuccess) {
    set_err(errbuf, errlen, "triangle BVH build: %s", cudaGetErrorString(e));
    return fail(AMS_ERR_CUDA);
  }
  s->ms_bvh_scene =
      std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  *out = s;
  return AMS_OK;
}

void ams_scene_destroy(ams_scene *scene) { delete scene; }

static ams_status validate(const ams_trace_params *p, int s0, int s1, int n0, int n1,
                           char *errbuf, size_t errlen) {
  if (!p) { set_err(errbuf, errlen, "params is NULL"); return AMS_ERR_ARG; }
  if (s0 <= 0 || s1 <= 0 || n0 <= 0 || n1 <= 0) {
    set_err(errbuf, errlen, "empty src or dst array");
    return AMS_ERR_ARG;
  }
  if ((long long)s0 * s1 > (1 << 26) || (long long)n0 * n1 > (1 << 28)) {
    set_err(errbuf, errlen, "src/dst arrays too large");
    return AMS_ERR_ARG;
  }
  if (p->max_reflection < 0 || p->max_reflection > 5) {
    set_err(errbuf, errlen, "max_reflection must be in [0, 5] (32 branch slots), got %d",
            p->max_reflection);
    return AMS_ERR_ARG;
  }
  if (p->reserve_size < 1 || p->reserve_size > 256) {
    set_err(errbuf, errlen, "reserve_size must be in [1, 256], got %d", p->reserve_size);
    return AMS_ERR_ARG;
  }
  if (p->samples_per_launch < 0 || p->launch_x <= 0 || p->launch_y <= 0 ||
      (long long)p->launch_x * p->launch_y > (1LL << 31) - 1) {
    set_err(errbuf, errlen, "bad launch grid");
    return AMS_ERR_ARG;
  }
  if (p->src_bptype < 0 || p->src_bptype > 3 || p->dst_bptype < 0 || p->dst_bptype > 3) {
    set_err(errbuf, errlen, "beam pattern types must be in [0, 3]");
    return AMS_ERR_ARG;
  }
  if (p->dst_gridsize <= 0) { set_err(errbuf, errlen, "dst_gridsize must be > 0"); return AMS_ERR_ARG; }
  if (!(p->wave_len > 0.0)) { set_err(errbuf, errlen, "wave_len must be > 0"); return AMS_ERR_ARG; }
  if (!(p->src_r >= 0.f) || !(p->dst_r >= 0.f)) {
    set_err(errbuf, errlen, "radii must be >= 0");
    return AMS_ERR_ARG;
  }
  return AMS_OK;
}

}  // extern "C"

namespace {
// The trace of ams_trace_channel; with records != nullptr, every backward
// ray's record is written (one path per stage-2 item in every round).
ams_status trace_impl(ams_scene *S, const ams_trace_params *p, const float *src, int s0, int s1,
                      const float *dst, int n0, int n1, const float *src_aabb_in,
                      const float *dst_aabb_in, float *result, ams_stats *stats,
                      ams_ray_record *records, unsigned long long max_records,
                      unsigned long long *n_records, void *stream, char *errbuf,
                      size_t errlen) {
  clear_stale_error();
  if (!S) { set_err(errbuf, errlen, "scene is NULL"); return AMS_ERR_ARG; }
  ams_status v = validate(p, s0, s1, n0, n1, errbuf, errlen);
  if (v != AMS_OK) return v;
  if (!src || !dst || !result) { set_err(errbuf, errlen, "null src/dst/result"); return AMS_ERR_ARG; }
  cudaStream_t st = (cudaStream_t)stream;
  const int n_src = s0 * s1, n_dst = n0 * n1, gs = p->dst_gridsize;
  const int n0g = (n0 - 1) / gs + 1, n1g = (n1 - 1) / gs + 1, ng = n0g * n1g;
  cudaEvent_t ev[4];
  for (auto &e : ev) CK(cudaEventCreate(&e));
  struct EvGuard { cudaEvent_t *e; ~EvGuard() { for (int i = 0; i < 4; i++) cudaEventDestroy(e[i]); } } eg{ev};
  CK(cudaEventRecord(ev[0], st));

  for (int attempt = 0; attempt < 6; attempt++) {
    const unsigned tab_size = 1u << S->tab_log2;
    const int W = (int)(tab_size / 32);
    size_t need = 0;
    need += al(sizeof(float) * 6 * (size_t)n_src) + al(sizeof(float) * 6 * (size_t)n_dst);
    need += al(std::max(lbvh_scratch_bytes(n_src), lbvh_scratch_bytes(n_dst)));
    need += al(lbvh_output_bytes(n_src)) + al(lbvh_output_bytes(n_dst));
    need += al(8 * (size_t)tab_size) + al(56 * (size_t)tab_size);
    need += 3 * al(4 * (size_t)ng * W);
    need += 2 * al(4 * ((size_t)ng + 1)) + al(4 * (size_t)ng) + 2 * al(4 * (size_t)tab_size);
    need += al(16 * (size_t)n_src * n_dst);
    need += al(8 * 16) + al(4);
    need += 4096;
    CK(S->ws.ensure(need));
    S->ws.reset();
    const float *src_aabb = src_aabb_in, *dst_aabb = dst_aabb_in;
    float *sbox = src_aabb ? nullptr : S->ws.take<float>(6 * (size_t)n_src);
    float *dbox = dst_aabb ? nullptr : S->ws.take<float>(6 * (size_t)n_dst);
    char *scratch = S->ws.take<char>(std::max(lbvh_scratch_bytes(n_src), lbvh_scratch_bytes(n_dst)));
    char *tx_out = S->ws.take<char>(lbvh_output_bytes(n_src));
    char *rx_out = S->ws.take<char>(lbvh_output_bytes(n_dst));
    TraceDev P{};
    P.rec = records;
    P.rec_cap = records ? max_records : 0;
    P.rec_base = 0;
    P.tab_h = S->ws.take<unsigned long long>(tab_size);
    P.tab_key = S->ws.take<int32_t>(14 * (size_t)tab_size);
    P.T = S->ws.take<unsigned>((size_t)ng * W);
    P.N = S->ws.take<unsigned>((size_t)ng * W);
    P.S = S->ws.take<unsigned>((size_t)ng * W);
    P.cell_off = S->ws.take<int>((size_t)ng + 1);
    P.chunk_off = S->ws.take<int>((size_t)ng + 1);
    P.cell_cnt = S->ws.take<int>((size_t)ng);
    P.slot_of = S->ws.take<int>(tab_size);
    int *dense_of = S->ws.take<int>(tab_size);
    P.acc = S->ws.take<unsigned long long>(2 * (size_t)n_src * n_dst);
    P.ctr = S->ws.take<unsigned long long>(16);
    P.err = S->ws.take<unsigned>(1);

    if (!src_aabb) { CK(sphere_aabbs(src, n_src, p->src_r, sbox, st)); src_aabb = sbox; }
    if (!dst_aabb) { CK(sphere_aabbs(dst, n_dst, p->dst_r, dbox, st)); dst_aabb = dbox; }
    Lbvh tx, rx;
    CK(lbvh_build_spheres(tx, src, src_aabb, n_src, scratch, tx_out, st));
    CK(lbvh_build_spheres(rx, dst, dst_aabb, n_dst, scratch, rx_out, st));
    CK(cudaEventRecord(ev[1], st));

    P.tris = S->tris;
    P.tri_nodes = S->bvh.nodes;
    P.tri_prims = S->bvh.prims;
    P.n_tri = S->n_tri;
    P.mat = S->mat;
    P.mat_prop = S->mat_prop;
    P.tx_nodes = tx.nodes; P.tx_prims = tx.prims; P.n_src = n_src; P.src = src; P.src_r = p->src_r;
    P.rx_nodes = rx.nodes; P.rx_prims = rx.prims; P.n_dst = n_dst; P.dst = dst; P.dst_r = p->dst_r;
    P.n0_dst = n0; P.n1_dst = n1; P.n0g = n0g; P.n1g = n1g; P.ng = ng; P.gs = gs;
    P.strict_grid = p->strict_grid;
    P.L = p->max_reflection; P.reserve = p->reserve_size; P.spl = p->samples_per_launch;
    P.launch_x = p->launch_x; P.launch_y = p->launch_y;
    P.lam_f = (float)p->wave_len; P.lam_d = p->wave_len;
    P.two_pi_over_lam = 6.283185307179586 / p->wave_len;
    for (int k = 0; k < 3; k++) { P.src_dir[k] = p->src_dir[k]; P.dst_dir[k] = p->dst_dir[k]; }
    P.src_bp = p->src_bptype; P.dst_bp = p->dst_bptype;
    P.tab_mask = tab_size - 1;
    P.tab_limit = tab_size / 2;
    P.W = W;

    CK(cudaMemsetAsync(P.tab_h, 0, 8 * (size_t)tab_size, st));
    CK(cudaMemsetAsync(P.tab_key, 0, 56 * (size_t)tab_size, st));  // 0 = word not written
    CK(cudaMemsetAsync(P.T, 0, 4 * (size_t)ng * W, st));
    CK(cudaMemsetAsync(P.S, 0, 4 * (size_t)ng * W, st));
    CK(cudaMemsetAsync(P.acc, 0, 16 * (size_t)n_src * n_dst, st));
    CK(cudaMemsetAsync(P.ctr, 0, 8 * 16, st));
    CK(cudaMemsetAsync(P.err, 0, 4, st));

    // ---- stage 1
    CK(trace_stage1(P, st));
    CK(trace_count_bits(P, P.T, P.ctr + 6, st));
    CK(cudaEventRecord(ev[2], st));
    CK(cudaMemcpyAsync(S->hc->ctr, P.ctr, 128, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&S->hc->err, P.err, 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (S->hc->err & AMS_DERR_PATH_TABLE) {
      if (S->tab_log2 >= 26) {
        set_err(errbuf, errlen, "path table would exceed 2^26 slots");
        return AMS_ERR_CAPACITY;
      }
      S->tab_log2 += 2;
      continue;  // grow the path table and run again
    }
    if (S->hc->err) {
      set_err(errbuf, errlen, "stage 1 device error flags 0x%x", S->hc->err);
      return (S->hc->err & AMS_DERR_HASH) ? AMS_ERR_INTERNAL : AMS_ERR_CAPACITY;
    }
    const unsigned long long fwd_records = S->hc->ctr[0];
    const unsigned long long overflow = S->hc->ctr[1];
    const unsigned long long n_paths = S->hc->ctr[2];
    const unsigned long long unique_records = S->hc->ctr[6];

    // ---- stage 2 rounds
    unsigned long long rounds = 0, total_tasks = 0;
    float ms_k2 = 0.f;
    unsigned long long n_new = unique_records;
    if (fwd_records > 0) {
      // stage 2 on dense path ids: the bitmaps shrink from one bit per table
      // slot to one per path found
      P.n_paths = (int)n_paths;
      P.W = (int)((n_paths + 31) / 32);
      const size_t dwords = (size_t)ng * P.W;
      CK(cudaMemsetAsync(P.N, 0, 4 * dwords, st));
      CK(trace_dense_paths(P, P.T, W, dense_of, P.N, st));
      CK(cudaMemcpyAsync(P.T, P.N, 4 * dwords, cudaMemcpyDeviceToDevice, st));
      CK(trace_count_tasks(P, P.N, st));
      while (n_new > 0) {
        // per task: its (path id, slot) and at most one chunk record
        const size_t per_task = sizeof(int2) + sizeof(int4);
        if (S->tasks.cap < n_new * per_task + 512) {
          CK(cudaStreamSynchronize(st));
          CK(S->tasks.ensure(std::max<size_t>(n_new * per_task * 2 + 512, 1 << 20)));
        }
        P.task_cap = (S->tasks.cap - 512) / per_task;
        P.task_path = reinterpret_cast<int2 *>(S->tasks.base);
        P.chunk_at = reinterpret_cast<int4 *>(S->tasks.base + al(sizeof(int2) * P.task_cap));
        P.kpi = records ? 1 : trace_paths_per_item(P, n_new);
        CK(trace_make_tasks(P, P.N, st));
        CK(cudaEventRecord(S->k2[0], st));
        if (records) {
          CK(trace_stage2_export(P, n_new, st));
          P.rec_base += n_new * (unsigned long long)(gs * gs) * (unsigned long long)n_src;
        } else {
          CK(trace_stage2(P, n_new, st));
        }
        CK(cudaEventRecord(S->k2[1], st));
        CK(trace_expand(P, st));
        rounds++;
        total_tasks += n_new;
        CK(cudaMemcpyAsync(S->hc->ctr, P.ctr, 128, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(&S->hc->err, P.err, 4, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (S->hc->err) {
          set_err(errbuf, errlen, "stage 2 device error flags 0x%x", S->hc->err);
          return (S->hc->err & AMS_DERR_ACC_RANGE) ? AMS_ERR_NUMERIC : AMS_ERR_CAPACITY;
        }
        ms_k2 += elapsed_ms(S->k2[0], S->k2[1]);
        if (S->hc->ctr[5] != n_new) {
          set_err(errbuf, errlen, "task count mismatch (%llu listed, %llu expected)",
                  S->hc->ctr[5], n_new);
          return AMS_ERR_INTERNAL;
        }
        n_new = S->hc->ctr[7];
      }
      CK(trace_finalize(P, result, st));
    }
    CK(cudaEventRecord(ev[3], st));
    CK(cudaMemcpyAsync(S->hc->ctr, P.ctr, 128, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    S->last = P;
    S->have_last = true;
    if (stats) {
      memset(stats, 0, sizeof(*stats));
      stats->rx_paths = S->hc->ctr[3];
      stats->rx_fail = S->hc->ctr[4];
      stats->fwd_records = fwd_records;
      stats->unique_records = fwd_records ? unique_records : 0;
      stats->unique_paths = fwd_records ? n_paths : 0;
      stats->rounds = rounds;
      stats->tasks = total_tasks;
      stats->overflow = overflow;
      stats->ms_bvh = elapsed_ms(ev[0], ev[1]);
      stats->ms_stage1 = elapsed_ms(ev[1], ev[2]);
      stats->ms_stage2 = elapsed_ms(ev[2], ev[3]);
      stats->ms_total = elapsed_ms(ev[0], ev[3]);
      stats->workspace_bytes = S->ws.high + S->tasks.high;
      stats->segments_fwd = S->hc->ctr[8];
      stats->segments_bwd = S->hc->ctr[9];
      stats->ms_stage2_kernel = ms_k2;
      stats->acc_adds = S->hc->ctr[13];
    }
    if (n_records) *n_records = P.rec_base;
    if (p->log_level > 0) {
      const float a = elapsed_ms(ev[0], ev[1]), b = elapsed_ms(ev[1], ev[2]),
                  c = elapsed_ms(ev[2], ev[3]);
      fprintf(stderr,
              "[ams] bvh %.3f ms, stage1 %.3f ms (%llu records, %llu unique, %llu paths), "
              "stage2 %.3f ms (%llu rounds, %llu tasks), rays %llu ok / %llu failed\n",
              a, b, fwd_records, unique_records, n_paths, c, rounds, total_tasks,
              S->hc->ctr[3], S->hc->ctr[4]);
    }
    return AMS_OK;
  }
  set_err(errbuf, errlen, "path table retries exhausted");
  return AMS_ERR_CAPACITY;
}
}  // namespace

extern "C" {

ams_status ams_trace_channel(ams_scene *S, const ams_trace_params *p, const float *src, int s0,
                             int s1, const float *dst, int n0, int n1, const float *src_aabb,
                             const float *dst_aabb, float *result, ams_stats *stats,
                             void *stream, char *errbuf, size_t errlen) {
  return trace_impl(S, p, src, s0, s1, dst, n0, n1, src_aabb, dst_aabb, result, stats, nullptr, 0,
                    nullptr, stream, errbuf, errlen);
}

ams_status ams_trace_channel_export(ams_scene *S, const ams_trace_params *p, const float *src,
                                    int s0, int s1, const float *dst, int n0, int n1,
                                    const float *src_aabb, const float *dst_aabb, float *result,
                                    ams_stats *stats, ams_ray_record *records,
                                    unsigned long long max_records,
                                    unsigned long long *n_records, void *stream, char *errbuf,
                                    size_t errlen) {
  if (!records || !n_records) {
    set_err(errbuf, errlen, "records and n_records are required");
    return AMS_ERR_ARG;
  }
  *n_records = 0;
  return trace_impl(S, p, src, s0, s1, dst, n0, n1, src_aabb, dst_aabb, result, stats, records,
                    max_records, n_records, stream, errbuf, errlen);
}

ams_status ams_launch_pathtrace(float *result, const float *src, int s0, int s1, const float *dst,
                                int n0, int n1, const float *src_aabb, const float *dst_aabb,
                                const float *scene_tris, int n_tri, const int *mat,
                                int samples_per_launch, int launch_x, int launch_y,
                                double wave_len, int max_reflection, int reserve_size,
                                const float *mat_prop, int n_mat, const float *src_dir,
                                const float *dst_dir, int log_level, int src_bptype,
                                int dst_bptype, int dst_gridsize, double src_r, double dst_r,
                                ams_stats *stats, char *errbuf, size_t errlen) {
  clear_stale_error();
  if (!src_dir || !dst_dir) { set_err(errbuf, errlen, "src_dir/dst_dir are NULL"); return AMS_ERR_ARG; }
  ams_trace_params p{};
  p.samples_per_launch = samples_per_launch;
  p.launch_x = launch_x;
  p.launch_y = launch_y;
  p.wave_len = wave_len;
  p.max_reflection = max_reflection;
  p.reserve_size = reserve_size;
  p.src_bptype = src_bptype;
  p.dst_bptype = dst_bptype;
  p.dst_gridsize = dst_gridsize;
  p.src_r = (float)src_r;
  p.dst_r = (float)dst_r;
  for (int k = 0; k < 3; k++) { p.src_dir[k] = src_dir[k]; p.dst_dir[k] = dst_dir[k]; }
  p.log_level = log_level;
  ams_scene *scene = nullptr;
  ams_status s = ams_scene_create(scene_tris, n_tri, mat, mat_prop, n_mat, nullptr, &scene,
                                  errbuf, errlen);
  if (s != AMS_OK) return s;
  s = ams_trace_channel(scene, &p, src, s0, s1, dst, n0, n1, src_aabb, dst_aabb, result, stats,
                        nullptr, errbuf, errlen);
  ams_scene_destroy(scene);
  return s;
}

ams_status ams_trace_export_paths(ams_scene *S, int32_t *host_out, int max_paths, int *n_out,
                                  char *errbuf, size_t errlen) {
  clear_stale_error();
  if (!S || !n_out || (max_paths > 0 && !host_out)) {
    set_err(errbuf, errlen, "bad arguments");
    return AMS_ERR_ARG;
  }
  *n_out = 0;
  if (!S->have_last) return AMS_OK;
  const TraceDev &P = S->last;
  size_t n = (size_t)P.tab_mask + 1;
  int32_t *dev = nullptr;
  unsigned long long *cnt = nullptr;
  CK(cudaMalloc(&dev, 56 * n + 64));
  cnt = reinterpret_cast<unsigned long long *>(reinterpret_cast<char *>(dev) + 56 * n);
  ams_status rc = AMS_OK;
  unsigned long long got = 0;
  if (cudaMemset(cnt, 0, 8) != cudaSuccess || trace_export_paths(P, dev, cnt, nullptr) != cudaSuccess ||
      cudaMemcpy(&got, cnt, 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_err(errbuf, errlen, "path export failed");
    rc = AMS_ERR_CUDA;
  } else {
    size_t k = std::min<size_t>(got, (size_t)std::max(max_paths, 0));
    if (k && cudaMemcpy(host_out, dev, 56 * k, cudaMemcpyDeviceToHost) != cudaSuccess) {
      set_err(errbuf, errlen, "path copy failed");
      rc = AMS_ERR_CUDA;
    }
    *n_out = (int)got;
  }
  cudaFree(dev);
  return rc;
}

}  // extern "C"

// ------------------------------------------------------------ objective
#include <mutex>
#include <vector>

#include "objective.h"

namespace {
struct DevScratch {
  char *ptr = nullptr;
  size_t cap = 0;
};
std::mutex g_scratch_mu;
std::vector<DevScratch> g_scratch;

cudaError_t scratch_for(size_t bytes, char **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if ((int)g_scratch.size() <= dev) g_scratch.resize(dev + 1);
  DevScratch &d = g_scratch[dev];
  if (d.cap < bytes) {
    // the buffer may still be in use by earlier asynchronous calls
    if (d.ptr) {
      if ((e = cudaDeviceSynchronize()) != cudaSuccess) return e;
      cudaFree(d.ptr);
      d.ptr = nullptr;
      d.cap = 0;
    }
    size_t want = std::max(bytes, (size_t)1 << 20);
    if ((e = cudaMalloc(&d.ptr, want)) != cudaSuccess) return e;
    // the control block (arrival counter) must start at zero
    if ((e = cudaMemset(d.ptr, 0, kObjControlBytes)) != cudaSuccess) return e;
    d.cap = want;
  }
  *out = d.ptr;
  return cudaSuccess;
}

ams_status obj_validate(const float *H_d, const float *H_a, const float *H_r, const float *phi,
                        float max_phase, const float *W, int S, int M, int R, int C,
                        char *errbuf, size_t errlen) {
  if (!H_d || !W) { set_err(errbuf, errlen, "H_d and W are required"); return AMS_ERR_ARG; }
  if (S <= 0 || R <= 0 || C <= 0) {
    set_err(errbuf, errlen, "S, R and C must be positive (S=%d R=%d C=%d)", S, R, C);
    return AMS_ERR_ARG;
  }
  if (C > 64) { set_err(errbuf, errlen, "at most 64 codes per call (C=%d)", C); return AMS_ERR_ARG; }
  bool ms = H_a || H_r;
  if (ms && (!H_a || !H_r || !phi || M <= 0)) {
    set_err(errbuf, errlen, "metasurface hop needs H_a, H_r, phi and M > 0");
    return AMS_ERR_ARG;
  }
  if (ms && !(max_phase > 0.f)) { set_err(errbuf, errlen, "max_phase must be > 0"); return AMS_ERR_ARG; }
  return AMS_OK;
}
}  // namespace

extern "C" {

ams_status ams_objective_fwd_bwd(const float *H_d, const float *H_a, const float *H_r,
                                 const float *phi, float max_phase, const float *W, int S, int M,
                                 int R, int C, float w, const uint8_t *drop, float *loss,
                                 float *grad_W, float *grad_phi, float *grad_Y, float *recv_amp,
                                 void *stream, char *errbuf, size_t errlen) {
  clear_stale_error();
  ams_status v = obj_validate(H_d, H_a, H_r, phi, max_phase, W, S, M, R, C, errbuf, errlen);
  if (v != AMS_OK) return v;
  if (!loss) { set_err(errbuf, errlen, "loss output is NULL"); return AMS_ERR_ARG; }
  if (grad_phi && !H_a) { set_err(errbuf, errlen, "grad_phi needs a metasurface hop"); return AMS_ERR_ARG; }
  const bool ms = H_a != nullptr;
  ObjScratchLayout L = obj_scratch_layout(S, ms ? M : 0, R, C);
  char *scr = nullptr;
  CK(scratch_for(L.total, &scr));
  ObjArgs a{H_d, H_a, H_r, phi, W, max_phase, S, ms ? M : 0, R, C, w, drop,
            loss, grad_W, ms ? grad_phi : nullptr, recv_amp, grad_Y};
  CK(obj_run(a, scr, (cudaStream_t)stream));
  return AMS_OK;
}

ams_status ams_objective_fwd_bwd_noalloc(const float *H_d, const float *H_a, const float *H_r,
                                         const float *phi, float max_phase, const float *W, int S,
                                         int M, int R, int C, float w, const uint8_t *drop,
                                         float *loss, float *grad_W, float *grad_phi,
                                         float *grad_Y, float *recv_amp, void *stream,
                                         char *errbuf, size_t errlen) {
  clear_stale_error();
  ams_status v = obj_validate(H_d, H_a, H_r, phi, max_phase, W, S, M, R, C, errbuf, errlen);
  if (v != AMS_OK) return v;
  if (!loss) { set_err(errbuf, errlen, "loss output is NULL"); return AMS_ERR_ARG; }
  if (grad_phi && !H_a) { set_err(errbuf, errlen, "grad_phi needs a metasurface hop"); return AMS_ERR_ARG; }
  const bool ms = H_a != nullptr;
  const ObjScratchLayout L = obj_scratch_layout(S, ms ? M : 0, R, C);
  if (L.total > (size_t)AMS_OBJECTIVE_NOALLOC_MAX_SCRATCH) {
    set_err(errbuf, errlen,
            "problem needs %zu bytes of scratch, above the fixed %u bytes of the "
            "allocation-free entry point (S=%d M=%d R=%d C=%d)",
            L.total, (unsigned)AMS_OBJECTIVE_NOALLOC_MAX_SCRATCH, S, M, R, C);
    return AMS_ERR_CAPACITY;
  }
  char *scr = nullptr;
  CK(obj_noalloc_scratch(&scr));
  cudaStream_t st = (cudaStream_t)stream;
  // the control block (arrival counter) must be zero when a call starts
  CK(cudaMemsetAsync(scr, 0, kObjControlBytes, st));
  ObjArgs a{H_d, H_a, H_r, phi, W, max_phase, S, ms ? M : 0, R, C, w, drop,
            loss, grad_W, ms ? grad_phi : nullptr, recv_amp, grad_Y};
  CK(obj_run(a, scr, st));
  return AMS_OK;
}

struct ams_objective_plan {
  ObjTcPlan *p;
  int S, M, R, Cmax;
  bool stacked = false;  // made by ams_objective_plan_create_stacked (no H_a)
};

ams_status ams_objective_plan_create(const float *H_d, const float *H_a, const float *H_r, int S,
                                     int M, int R, int C_max, void *stream,
                                     ams_objective_plan **out, char *errbuf, size_t errlen) {
  clear_stale_error();
  if (!out) { set_err(errbuf, errlen, "out is NULL"); return AMS_ERR_ARG; }
  *out = nullptr;
  if (!H_d || !H_a || !H_r) {
    set_err(errbuf, errlen, "a plan needs H_d, H_a and H_r");
    return AMS_ERR_ARG;
  }
  if (S <= 0 || M <= 0 || R <= 0 || C_max <= 0 || C_max > 64) {
    set_err(errbuf, errlen, "need S, M, R > 0 and 1 <= C_max <= 64 (S=%d M=%d R=%d C_max=%d)", S,
            M, R, C_max);
    return AMS_ERR_ARG;
  }
  if ((reinterpret_cast<uintptr_t>(H_d) | reinterpret_cast<uintptr_t>(H_a) |
       reinterpret_cast<uintptr_t>(H_r)) & 7) {
    set_err(errbuf, errlen, "complex arrays must be 8-byte aligned");
    return AMS_ERR_ARG;
  }
  ObjTcPlan *tp = nullptr;
  CK(obj_tc_plan_create(H_d, H_a, H_r, S, M, R, C_max, (cudaStream_t)stream, &tp));
  *out = new ams_objective_plan{tp, S, M, R, C_max, false};
  return AMS_OK;
}

ams_status ams_objective_plan_fwd_bwd(ams_objective_plan *plan, const float *phi, float max_phase,
                                      const float *W, int C, float w, const uint8_t *drop,
                                      float *loss, float *grad_W, float *grad_phi, float *grad_Y,
                                      float *recv_amp, void *stream, char *errbuf,
                                      size_t errlen) {
  clear_stale_error();
  if (!plan || !plan->p) { set_err(errbuf, errlen, "plan is NULL"); return AMS_ERR_ARG; }
  if (!phi || !W || !loss) { set_err(errbuf, errlen, "phi, W and loss are required"); return AMS_ERR_ARG; }
  if (C <= 0 || C > plan->Cmax) {
    set_err(errbuf, errlen, "C=%d outside [1, %d] of this plan", C, plan->Cmax);
    return AMS_ERR_ARG;
  }
  if (!(max_phase > 0.f)) { set_err(errbuf, errlen, "max_phase must be > 0"); return AMS_ERR_ARG; }
  if (plan->stacked) {
    set_err(errbuf, errlen, "a stacked plan takes its coefficients: ams_objective_plan_coef_fwd_bwd");
    return AMS_ERR_ARG;
  }
  if (grad_Y && obj_tc_plan_streams(plan->p)) {
    set_err(errbuf, errlen, "grad_Y is not available from a plan made with C_max <= 2");
    return AMS_ERR_ARG;
  }
  ObjArgs a{nullptr, nullptr, nullptr, phi, W, max_phase, plan->S, plan->M, plan->R, C, w, drop,
            loss, grad_W, grad_phi, recv_amp, grad_Y};
  CK(obj_tc_run(plan->p, a, (cudaStream_t)stream));
  return AMS_OK;
}

ams_status ams_objective_plan_create_stacked(const float *H_d, const float *H_r, int S, int M,
                                             int R, int C_max, void *stream,
                                             ams_objective_plan **out, char *errbuf,
                                             size_t errlen) {
  clear_stale_error();
  if (!out) { set_err(errbuf, errlen, "out is NULL"); return AMS_ERR_ARG; }
  *out = nullptr;
  if (!H_d || !H_r) { set_err(errbuf, errlen, "a stacked plan needs H_d and H_r"); return AMS_ERR_ARG; }
  if (S <= 0 || M <= 0 || R <= 0 || C_max <= 0 || C_max > 64) {
    set_err(errbuf, errlen, "need S, M, R > 0 and 1 <= C_max <= 64 (S=%d M=%d R=%d C_max=%d)", S,
            M, R, C_max);
    return AMS_ERR_ARG;
  }
  if ((reinterpret_cast<uintptr_t>(H_d) | reinterpret_cast<uintptr_t>(H_r)) & 7) {
    set_err(errbuf, errlen, "complex arrays must be 8-byte aligned");
    return AMS_ERR_ARG;
  }
  ObjTcPlan *tp = nullptr;
  CK(obj_tc_plan_create(H_d, nullptr, H_r, S, M, R, C_max, (cudaStream_t)stream, &tp, true));
  *out = new ams_objective_plan{tp, S, M, R, C_max, true};
  return AMS_OK;
}

ams_status ams_objective_plan_coef_fwd_bwd(ams_objective_plan *plan, const float *U,
                                           const float *W, int C, float w, const uint8_t *drop,
                                           float *loss, float *grad_U, float *grad_W,
                                           float *recv_amp, void *stream, char *errbuf,
                                           size_t errlen) {
  clear_stale_error();
  if (!plan || !plan->p) { set_err(errbuf, errlen, "plan is NULL"); return AMS_ERR_ARG; }
  if (!plan->stacked) {
    set_err(errbuf, errlen, "coefficients are taken by plans from ams_objective_plan_create_stacked");
    return AMS_ERR_ARG;
  }
  if (!U || !W || !loss) { set_err(errbuf, errlen, "U, W and loss are required"); return AMS_ERR_ARG; }
  if (C <= 0 || C > plan->Cmax) {
    set_err(errbuf, errlen, "C=%d outside [1, %d] of this plan", C, plan->Cmax);
    return AMS_ERR_ARG;
  }
  ObjArgs a{nullptr, nullptr, nullptr, nullptr, W, 1.0f, plan->S, plan->M, plan->R, C, w, drop,
            loss, grad_W, nullptr, recv_amp, nullptr};
  a.U_in = U;
  a.grad_U = grad_U;
  CK(obj_tc_run(plan->p, a, (cudaStream_t)stream));
  return AMS_OK;
}

ams_status ams_cgemm(int m, int n, int k, const float *A, int lda, int opA, const float *B,
                     int ldb, int opB, float *Cm, int ldc, int accumulate, void *stream,
                     char *errbuf, size_t errlen) {
  clear_stale_error();
  if (!A || !B || !Cm || m <= 0 || n <= 0 || k <= 0 || opA < 0 || opA > 3 || opB < 0 ||
      opB > 3) {
    set_err(errbuf, errlen, "bad complex GEMM arguments (m=%d n=%d k=%d opA=%d opB=%d)", m, n, k,
            opA, opB);
    return AMS_ERR_ARG;
  }
  if (lda < (opA == 0 || opA == 3 ? k : m) || ldb < (opB == 0 || opB == 3 ? n : k) || ldc < n) {
    set_err(errbuf, errlen, "leading dimensions too small");
    return AMS_ERR_ARG;
  }
  CK(cgemm_run(m, n, k, A, lda, opA, B, ldb, opB, Cm, ldc, accumulate != 0, (cudaStream_t)stream));
  return AMS_OK;
}

unsigned long long ams_objective_plan_bytes(const ams_objective_plan *plan) {
  return plan ? (unsigned long long)obj_tc_plan_bytes(plan->p) : 0ull;
}

void ams_objective_plan_destroy(ams_objective_plan *plan) {
  if (!plan) return;
  obj_tc_plan_destroy(plan->p);
  delete plan;
}

ams_status ams_objective_recv(const float *H_d, const float *H_a, const float *H_r,
                              const float *phi, float max_phase, const float *W, int S, int M,
                              int R, int C, float *recv_amp, void *stream, char *errbuf,
                              size_t errlen) {
  clear_stale_error();
  ams_status v = obj_validate(H_d, H_a, H_r, phi, max_phase, W, S, M, R, C, errbuf, errlen);
  if (v != AMS_OK) return v;
  if (!recv_amp) { set_err(errbuf, errlen, "recv_amp is NULL"); return AMS_ERR_ARG; }
  const bool ms = H_a != nullptr;
  ObjScratchLayout L = obj_scratch_layout(S, ms ? M : 0, R, C);
  char *scr = nullptr;
  CK(scratch_for(L.total, &scr));
  ObjArgs a{H_d, H_a, H_r, phi, W, max_phase, S, ms ? M : 0, R, C, 1.0f, nullptr,
            nullptr, nullptr, nullptr, recv_amp, nullptr};
  CK(obj_run(a, scr, (cudaStream_t)stream));
  return AMS_OK;
}

ams_status ams_coverage_db(const float *H, int S, int R, float threshold, float offset, float *out,
                           void *stream, char *errbuf, size_t errlen) {
  clear_stale_error();
  if (!H || !out || S <= 0 || R <= 0) { set_err(errbuf, errlen, "bad arguments"); return AMS_ERR_ARG; }
  CK(coverage_db_run(H, S, R, threshold, offset, out, (cudaStream_t)stream));
  return AMS_OK;
}

ams_status ams_objective_status(const ams_objective_plan *plan, void *stream, char *errbuf,
                                size_t errlen) {
  clear_stale_error();
  CK(cudaStreamSynchronize((cudaStream_t)stream));
  std::vector<const unsigned *> words;
  if (plan) {
    if (!plan->p) { set_err(errbuf, errlen, "plan is NULL"); return AMS_ERR_ARG; }
    words.push_back(obj_tc_plan_status_word(plan->p));
  } else {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    {
      std::lock_guard<std::mutex> lk(g_scratch_mu);
      if ((int)g_scratch.size() > dev && g_scratch[dev].ptr)
        words.push_back(reinterpret_cast<const unsigned *>(g_scratch[dev].ptr + 48));
    }
    char *na = nullptr;
    CK(obj_noalloc_scratch(&na));
    words.push_back(reinterpret_cast<const unsigned *>(na + 48));
  }
  unsigned flags = 0;
  for (const unsigned *w : words) {
    unsigned v = 0;
    CK(cudaMemcpy(&v, w, 4, cudaMemcpyDeviceToHost));
    flags |= v;
  }
  if (flags) {
    set_err(errbuf, errlen,
            "a bounded wait of the last objective call ran out (flags 0x%x): its outputs are NaN",
            flags);
    return AMS_ERR_INTERNAL;
  }
  return AMS_OK;
}

void ams_debug_inject_wait_timeout(int calls) { obj_inject_timeouts(calls); }

unsigned long long ams_scratch_bytes(void) {
  unsigned long long t = 0;
  {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    for (auto &d : g_scratch) t += d.cap;
  }
  BlockPool &bp = block_pool();
  std::lock_guard<std::mutex> lk(bp.mu);
  for (auto &kv : bp.free_blocks) t += kv.first.second;
  return t;
}

}  // extern "C"

// -------------------------------------------------------- surrogate MLP
#include "gemm_tc.h"
#include "mlp.h"

struct ams_mlp {
  MlpDev dev;
  char *arena = nullptr;
  ~ams_mlp() {
    if (arena) cudaFree(arena);
  }
};

namespace {
ams_status mlp_check_err(ams_mlp *m, cudaStream_t st, char *errbuf, size_t errlen) {
  unsigned e = 0;
  cudaError_t ce = cudaMemcpyAsync(&e, m->dev.err, 4, cudaMemcpyDeviceToHost, st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
  if (ce != cudaSuccess) {
    set_err(errbuf, errlen, "MLP: %s", cudaGetErrorString(ce));
    return AMS_ERR_CUDA;
  }
  if (e) {
    set_err(errbuf, errlen, "tensor-core GEMM timed out waiting (flags 0x%x)", e);
    cudaMemsetAsync(m->dev.err, 0, 4, st);
    return AMS_ERR_INTERNAL;
  }
  return AMS_OK;
}
}  // namespace

extern "C" {

ams_status ams_gemm_bf16(const void *A, const void *B, int M, int N, int K, const float *bias,
                         int relu, float *C32, void *C16, void *stream, char *errbuf,
                         size_t errlen) {
  clear_stale_error();
  if (!A || !B || (!C32 && !C16)) { set_err(errbuf, errlen, "null operand"); return AMS_ERR_ARG; }
  if (M <= 0 || N <= 0 || K <= 0 || M % 128 || N % 64 || K % 64) {
    set_err(errbuf, errlen, "need M %% 128 == 0, N %% 64 == 0, K %% 64 == 0 (M=%d N=%d K=%d)", M,
            N, K);
    return AMS_ERR_ARG;
  }
  if (((uintptr_t)A | (uintptr_t)B) & 15) {
    set_err(errbuf, errlen, "A and B must be 16-byte aligned");
    return AMS_ERR_ARG;
  }
  unsigned *err = nullptr;
  CK(cudaMallocAsync((void **)&err, 4, (cudaStream_t)stream));
  CK(cudaMemsetAsync(err, 0, 4, (cudaStream_t)stream));
  GemmEpilogue ep;
  ep.bias = bias;
  ep.relu = relu != 0;
  ep.out32 = C32;
  ep.out16 = reinterpret_cast<__nv_bfloat16 *>(C16);
  ep.ldc = N;
  cudaError_t e = gemm_bf16_tc(reinterpret_cast<const __nv_bfloat16 *>(A),
                               reinterpret_cast<const __nv_bfloat16 *>(B), M, N, K, ep, err,
                               (cudaStream_t)stream);
  unsigned flags = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, err, 4, cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  cudaFreeAsync(err, (cudaStream_t)stream);
  if (e != cudaSuccess) {
    set_err(errbuf, errlen, "GEMM: %s", cudaGetErrorString(e));
    return AMS_ERR_CUDA;
  }
  if (flags) {
    set_err(errbuf, errlen, "tensor-core GEMM timed out waiting (flags 0x%x)", flags);
    return AMS_ERR_INTERNAL;
  }
  return AMS_OK;
}

ams_status ams_mlp_create(const int *dims, int n_dims, int max_batch, unsigned long long seed,
                          void *stream, ams_mlp **out, char *errbuf, size_t errlen) {
  clear_stale_error();
  if (!out || !dims || n_dims < 2 || n_dims > kMlpMaxLayers + 1 || max_batch <= 0) {
    set_err(errbuf, errlen, "bad MLP shape");
    return AMS_ERR_ARG;
  }
  *out = nullptr;
  for (int i = 0; i < n_dims; i++)
    if (dims[i] <= 0 || (i > 0 && dims[i] % 128)) {
      set_err(errbuf, errlen, "width %d = %d: widths after the input must be multiples of 128", i,
              dims[i]);
      return AMS_ERR_ARG;
    }
  ams_mlp *m = new ams_mlp();
  MlpDev &d = m->dev;
  d.L = n_dims - 1;
  for (int i = 0; i < n_dims; i++) {
    d.d[i] = dims[i];
    d.dp[i] = i == 0 ? (dims[0] + 63) / 64 * 64 : dims[i];
  }
  d.max_bp = (max_batch + 127) / 128 * 128;
  // one arena
  size_t total = 0;
  auto add = [&](size_t b) { size_t o = total; total += al(b); return o; };
  size_t off_W[kMlpMaxLayers + 1], off_b[kMlpMaxLayers + 1], off_mW[kMlpMaxLayers + 1],
      off_vW[kMlpMaxLayers + 1], off_mb[kMlpMaxLayers + 1], off_vb[kMlpMaxLayers + 1],
      off_gW[kMlpMaxLayers + 1], off_gb[kMlpMaxLayers + 1], off_Wb[kMlpMaxLayers + 1],
      off_Wt[kMlpMaxLayers + 1], off_H[kMlpMaxLayers + 1], off_dZ[kMlpMaxLayers + 1];
  size_t maxw = 0;
  for (int l = 1; l <= d.L; l++) {
    size_t n = (size_t)d.d[l] * d.dp[l - 1];
    off_W[l] = add(4 * n); off_mW[l] = add(4 * n); off_vW[l] = add(4 * n); off_gW[l] = add(4 * n);
    off_b[l] = add(4 * d.d[l]); off_mb[l] = add(4 * d.d[l]); off_vb[l] = add(4 * d.d[l]);
    off_gb[l] = add(4 * d.d[l]);
    off_Wb[l] = add(2 * n); off_Wt[l] = add(2 * n);
    off_dZ[l] = add(2 * (size_t)d.max_bp * d.dp[l]);
    maxw = std::max(maxw, (size_t)std::max(d.dp[l], d.dp[l - 1]));
  }
  for (int l = 0; l < d.L; l++) off_H[l] = add(2 * (size_t)d.max_bp * d.dp[l]);
  size_t off_tA = add(2 * (size_t)d.max_bp * maxw), off_tB = add(2 * (size_t)d.max_bp * maxw);
  size_t off_Y = add(4 * (size_t)d.max_bp * d.dp[d.L]);
  size_t off_part = add(8 * (size_t)kMlpLossParts), off_err = add(4);
  cudaError_t e = cudaMalloc(&m->arena, total);
  if (e != cudaSuccess) {
    set_err(errbuf, errlen, "MLP arena (%zu bytes): %s", total, cudaGetErrorString(e));
    delete m;
    return AMS_ERR_OOM;
  }
  char *a = m->arena;
  for (int l = 1; l <= d.L; l++) {
    d.W[l] = (float *)(a + off_W[l]); d.mW[l] = (float *)(a + off_mW[l]);
    d.vW[l] = (float *)(a + off_vW[l]); d.gW[l] = (float *)(a + off_gW[l]);
    d.b[l] = (float *)(a + off_b[l]); d.mb[l] = (float *)(a + off_mb[l]);
    d.vb[l] = (float *)(a + off_vb[l]); d.gb[l] = (float *)(a + off_gb[l]);
    d.Wb[l] = (__nv_bfloat16 *)(a + off_Wb[l]); d.Wt[l] = (__nv_bfloat16 *)(a + off_Wt[l]);
    d.dZ[l] = (__nv_bfloat16 *)(a + off_dZ[l]);
  }
  for (int l = 0; l < d.L; l++) d.H[l] = (__nv_bfloat16 *)(a + off_H[l]);
  d.tA = (__nv_bfloat16 *)(a + off_tA);
  d.tB = (__nv_bfloat16 *)(a + off_tB);
  d.Y = (float *)(a + off_Y);
  d.part = (double *)(a + off_part);
  d.err = (unsigned *)(a + off_err);
  cudaStream_t st = (cudaStream_t)stream;
  cudaMemsetAsync(d.err, 0, 4, st);
  if ((e = mlp_init(d, (uint32_t)(seed ^ (seed >> 32)), st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess) {
    set_err(errbuf, errlen, "MLP init: %s", cudaGetErrorString(e));
    delete m;
    return AMS_ERR_CUDA;
  }
  *out = m;
  return AMS_OK;
}

void ams_mlp_destroy(ams_mlp *mlp) { delete mlp; }

ams_status ams_mlp_forward(ams_mlp *m, const float *X, int B, float *Y, void *stream, char *errbuf,
                           size_t errlen) {
  clear_stale_error();
  if (!m || !X || !Y || B <= 0 || B > m->dev.max_bp) {
    set_err(errbuf, errlen, "bad MLP forward arguments (B=%d)", B);
    return AMS_ERR_ARG;
  }
  CK(mlp_forward(m->dev, X, B, Y, (cudaStream_t)stream));
  return mlp_check_err(m, (cudaStream_t)stream, errbuf, errlen);
}

ams_status ams_mlp_train_step(ams_mlp *m, const float *X, const float *T, int B, float lr,
                              float *loss, void *stream, char *errbuf, size_t errlen) {
  clear_stale_error();
  if (!m || !X || !T || B <= 0 || B > m->dev.max_bp || !(lr >= 0.f)) {
    set_err(errbuf, errlen, "bad MLP training arguments (B=%d)", B);
    return AMS_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  CK(mlp_forward(m->dev, X, B, nullptr, st));
  CK(mlp_backward(m->dev, T, B, loss, st));
  CK(mlp_adam(m->dev, lr, st));
  return mlp_check_err(m, st, errbuf, errlen);
}

// which: 0 parameters, 1 gradients, 2 Adam first moments, 3 second moments
static void mlp_param_copy(MlpDev &d, float *flat, bool to_flat, int which, cudaStream_t st) {
  size_t o = 0;
  for (int l = 1; l <= d.L; l++) {
    float *const Ws[4] = {d.W[l], d.gW[l], d.mW[l], d.vW[l]};
    float *const bs[4] = {d.b[l], d.gb[l], d.mb[l], d.vb[l]};
    float *W = Ws[which];
    float *b = bs[which];
    const size_t dp = sizeof(float) * d.dp[l - 1], dl = sizeof(float) * d.d[l - 1];
    if (to_flat)
      cudaMemcpy2DAsync(flat + o, dl, W, dp, dl, d.d[l], cudaMemcpyDeviceToDevice, st);
    else
      cudaMemcpy2DAsync(W, dp, flat + o, dl, dl, d.d[l], cudaMemcpyDeviceToDevice, st);
    o += (size_t)d.d[l] * d.d[l - 1];
    if (to_flat)
      cudaMemcpyAsync(flat + o, b, sizeof(float) * d.d[l], cudaMemcpyDeviceToDevice, st);
    else
      cudaMemcpyAsync(b, flat + o, sizeof(float) * d.d[l], cudaMemcpyDeviceToDevice, st);
    o += d.d[l];
  }
}

ams_status ams_mlp_gradients(ams_mlp *m, const float *X, const float *T, int B, float *loss,
                             float *grads, void *stream, char *errbuf, size_t errlen) {
  clear_stale_error();
  if (!m || !X || !T || !grads || B <= 0 || B > m->dev.max_bp) {
    set_err(errbuf, errlen, "bad MLP gradient arguments");
    return AMS_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  CK(mlp_forward(m->dev, X, B, nullptr, st));
  CK(mlp_backward(m->dev, T, B, loss, st));
  mlp_param_copy(m->dev, grads, true, 1, st);
  CK(cudaGetLastError());
  return mlp_check_err(m, st, errbuf, errlen);
}

ams_status ams_mlp_params(ams_mlp *m, float *params, int direction, long long *count, void *stream,
                          char *errbuf, size_t errlen) {
  if (!m || (direction != 0 && direction != 1)) {
    set_err(errbuf, errlen, "bad arguments");
    return AMS_ERR_ARG;
  }
  long long n = 0;
  for (int l = 1; l <= m->dev.L; l++) n += (long long)m->dev.d[l] * m->dev.d[l - 1] + m->dev.d[l];
  if (count) *count = n;
  if (!params) return AMS_OK;
  cudaStream_t st = (cudaStream_t)stream;
  mlp_param_copy(m->dev, params, direction == 0, 0, st);
  if (direction == 1) CK(mlp_refresh_bf16(m->dev, st));
  CK(cudaStreamSynchronize(st));
  return AMS_OK;
}

ams_status ams_mlp_adam_state(ams_mlp *m, float *m1, float *m2, long long *step, int direction,
                              void *stream, char *errbuf, size_t errlen) {
  clear_stale_error();
  if (!m || !m1 || !m2 || !step || (direction != 0 && direction != 1)) {
    set_err(errbuf, errlen, "bad arguments");
    return AMS_ERR_ARG;
  }
  if (direction == 1 && (*step < 0 || *step > 0x7fffffffLL)) {
    set_err(errbuf, errlen, "Adam step %lld out of range", *step);
    return AMS_ERR_ARG;
  }
  cudaStream_t st = (cudaStream_t)stream;
  mlp_param_copy(m->dev, m1, direction == 0, 2, st);
  mlp_param_copy(m->dev, m2, direction == 0, 3, st);
  CK(cudaGetLastError());
  if (direction == 0) *step = m->dev.step;
  else m->dev.step = (int)*step;
  CK(cudaStreamSynchronize(st));
  return AMS_OK;
}

}  // extern "C"
