// lbvh.cu -- linear BVH builder (Karras 2012, "Maximizing parallelism in
// the construction of BVHs, octrees and k-d trees"), GB300 version.
//
// Replaces the OptiX GAS builds of the reference (optixPathTracer.cpp:382-546:
// one triangle GAS, one custom-AABB GAS per sphere set) with:
//   1. centroid bounds (one CTA reduction),
//   2. 30-bit Morton codes of the centroids scaled to a cube, with the
//      primitive index in the low word (bit 30 set for primitives larger
//      than a quarter of the scene),
//   3. a sort of the keys: bitonic in shared memory up to 16,384 keys, else
//      a stable LSD radix sort (one 1024-thread CTA, 4-bit digits, warp
//      ballots for the in-tile ranks),
//   4. the Karras hierarchy, one thread per internal node,
//   5. a bottom-up refit with per-node arrival counters.
// Node layout: both children's boxes live in the parent (64 bytes per node,
// four 16-byte loads), boxes widened outward so that node culling is
// conservative.  Leaves hold one primitive; a child reference c < 0 is the
// leaf of sorted primitive ~c.
#include "ams_common.cuh"
#include "lbvh.h"

namespace {

__device__ __forceinline__ float widen_lo(float v) {
  return nextafterf(v - (1e-6f + 1e-6f * fabsf(v)), -3.0e38f);
}
__device__ __forceinline__ float widen_hi(float v) {
  return nextafterf(v + (1e-6f + 1e-6f * fabsf(v)), 3.0e38f);
}

__global__ void k_bounds(const PrimBox *boxes, int n, float *out6) {
  __shared__ float s[6][32];
  float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const PrimBox b = boxes[i];
    for (int k = 0; k < 3; k++) {
      float c = 0.5f * (b.lo[k] + b.hi[k]);
      lo[k] = fminf(lo[k], c);
      hi[k] = fmaxf(hi[k], c);
    }
  }
  for (int k = 0; k < 3; k++) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
      hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
    }
  }
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
    for (int k = 0; k < 3; k++) { s[k][w] = lo[k]; s[3 + k][w] = hi[k]; }
  __syncthreads();
  if (w == 0) {
    int nw = blockDim.x >> 5;
    for (int k = 0; k < 6; k++) {
      float v = l < nw ? s[k][l] : (k < 3 ? 3.0e38f : -3.0e38f);
      for (int o = 16; o > 0; o >>= 1) {
        float u = __shfl_xor_sync(0xffffffffu, v, o);
        v = k < 3 ? fminf(v, u) : fmaxf(v, u);
      }
      if (l == 0) out6[k] = v;
    }
  }
}

__device__ __forceinline__ uint32_t expand10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__global__ void k_morton(const PrimBox *boxes, int n, const float *b6, uint64_t *keys) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const PrimBox b = boxes[i];
  uint32_t q[3];
  // one scale for all axes (the largest centroid extent): a flat room or
  // building gets its first splits across its long sides instead of cutting
  // its 3 m height as finely as its 45 m width
  const float cube = fmaxf(fmaxf(b6[3] - b6[0], b6[4] - b6[1]), b6[5] - b6[2]);
  for (int k = 0; k < 3; k++) {
    float c = 0.5f * (b.lo[k] + b.hi[k]);
    float u = cube > 0.0f ? (c - b6[k]) / cube : 0.5f;
    u = fminf(fmaxf(u, 0.0f), 1.0f);
    q[k] = (uint32_t)fminf(u * 1024.0f, 1023.0f);
  }
  uint32_t m = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
  // Primitives larger than a quarter of the scene (floors, walls) get a bit
  // above the Morton code, so the root splits them off into their own
  // subtree instead of inflating the boxes of every node on the way to the
  // small ones around their centroids.  Culling only: results do not change.
  float bext = 0.0f, sext = 0.0f;
  for (int k = 0; k < 3; k++) {
    bext = fmaxf(bext, b.hi[k] - b.lo[k]);
    sext = fmaxf(sext, b6[3 + k] - b6[k]);
  }
  if (sext > 0.0f && bext > 0.25f * sext) m |= 1u << 30;
  keys[i] = ((uint64_t)m << 32) | (uint32_t)i;
}

// Stable LSD radix sort of 64-bit items on their upper 32 bits (30 used),
// one CTA of 1024 threads, tiles of 1024 items in order.
__global__ void __launch_bounds__(1024) k_sort(uint64_t *a, uint64_t *b, int n) {
  __shared__ int hist[16];
  __shared__ int base[16];
  __shared__ int wcnt[32][16];
  __shared__ int woff[32][16];
  const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
  const unsigned lt = (1u << lane) - 1u;
  uint64_t *in = a, *out = b;
  for (int pass = 0; pass < 8; pass++) {
    const int shift = 32 + 4 * pass;
    if (tid < 16) hist[tid] = 0;
    __syncthreads();
    for (int i = tid; i < n; i += 1024) atomicAdd(&hist[(int)((in[i] >> shift) & 15u)], 1);
    __syncthreads();
    if (tid == 0) {
      int s = 0;
      for (int v = 0; v < 16; v++) { base[v] = s; s += hist[v]; }
    }
    __syncthreads();
    for (int t0 = 0; t0 < n; t0 += 1024) {
      int i = t0 + tid;
      bool valid = i < n;
      uint64_t key = valid ? in[i] : 0ull;
      int d = valid ? (int)((key >> shift) & 15u) : 16;
      int rank = 0;
      for (int v = 0; v < 16; v++) {
        unsigned bal = __ballot_sync(0xffffffffu, d == v);
        if (d == v) rank = __popc(bal & lt);
        if (lane == 0) wcnt[w][v] = __popc(bal);
      }
      __syncthreads();
      if (tid < 16) {
        int s = 0;
        for (int ww = 0; ww < 32; ww++) { woff[ww][tid] = s; s += wcnt[ww][tid]; }
        hist[tid] = s;  // tile count of digit tid
      }
      __syncthreads();
      if (valid) out[base[d] + woff[w][d] + rank] = key;
      __syncthreads();
      if (tid < 16) base[tid] += hist[tid];
      __syncthreads();
    }
    uint64_t *t = in; in = out; out = t;
  }
  // 8 passes: the sorted data is back in `a`
}

// Up to kSmemSortMax keys: bitonic sort in shared memory, one CTA of 1024
// threads (log2(n) (log2(n) + 1) / 2 compare-exchange steps).  The keys are
// unique (primitive index in the low word), so the order equals the stable
// radix sort's.  Padding slots hold ~0, which sorts last.
constexpr int kSmemSortMax = 16384;
__global__ void __launch_bounds__(1024) k_sort_smem(uint64_t *a, int n) {
  extern __shared__ uint64_t sk[];
  int np = 1;
  while (np < n) np <<= 1;
  for (int i = threadIdx.x; i < np; i += blockDim.x) sk[i] = i < n ? a[i] : ~0ull;
  __syncthreads();
  // each step visits its np / 2 compare-exchange pairs (i, i + j) directly
  for (int k = 2; k <= np; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int q = threadIdx.x; q < (np >> 1); q += blockDim.x) {
        const int i = ((q & ~(j - 1)) << 1) | (q & (j - 1));
        const int l = i + j;
        const uint64_t x = sk[i], y = sk[l];
        const bool up = (i & k) == 0;
        if ((x > y) == up) { sk[i] = y; sk[l] = x; }
      }
      __syncthreads();
    }
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) a[i] = sk[i];
}

__device__ __forceinline__ int delta(const uint64_t *k, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  return __clzll(k[i] ^ k[j]);  // keys are unique (index in the low word)
}

__global__ void k_karras(const uint64_t *keys, int n, BvhNode *nodes, int *parent) {
  // parent[0 .. n-2]: internal nodes, parent[n-1 .. 2n-2]: leaves
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  int d = (delta(keys, n, i, i + 1) - delta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  int dmin = delta(keys, n, i, i - d);
  int lmax = 2;
  while (delta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (delta(keys, n, i, i + (l + t) * d) > dmin) l += t;
  int j = i + l * d;
  int dnode = delta(keys, n, i, j);
  int s = 0;
  int len = l;
  int t = (len + 1) >> 1;
  while (true) {
    if (delta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    if (t == 1) break;
    t = (t + 1) >> 1;
  }
  int g = i + s * d + min(d, 0);
  int lo = min(i, j), hi = max(i, j);
  int left = (lo == g) ? ~g : g;
  int right = (hi == g + 1) ? ~(g + 1) : g + 1;
  nodes[i].d = make_int4(left, right, 0, 0);
  if (left >= 0) parent[left] = i; else parent[(n - 1) + ~left] = i;
  if (right >= 0) parent[right] = i; else parent[(n - 1) + ~right] = i;
  if (i == 0) parent[0] = -1;
}

__device__ __forceinline__ void store_child(BvhNode &nd, int which, const float lo[3],
                                            const float hi[3]) {
  float wl[3], wh[3];
  for (int k = 0; k < 3; k++) { wl[k] = widen_lo(lo[k]); wh[k] = widen_hi(hi[k]); }
  if (which == 0) {
    nd.a = make_float4(wl[0], wl[1], wl[2], wh[0]);
    nd.b.x = wh[1]; nd.b.y = wh[2];
  } else {
    nd.b.z = wl[0]; nd.b.w = wl[1];
    nd.c = make_float4(wl[2], wh[0], wh[1], wh[2]);
  }
}

__global__ void k_refit(const uint64_t *keys, const PrimBox *boxes, int n, BvhNode *nodes,
                        const int *parent, int *flags, float *node_box, int *perm) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  int orig = (int)(keys[j] & 0xffffffffu);
  perm[j] = orig;
  if (n == 1) return;
  int p = parent[(n - 1) + j];
  while (p >= 0) {
    __threadfence();
    if (atomicAdd(&flags[p], 1) == 0) return;  // the sibling finishes this node
    __threadfence();
    int4 ch = nodes[p].d;
    float lo[2][3], hi[2][3];
    for (int c = 0; c < 2; c++) {
      int r = c == 0 ? ch.x : ch.y;
      if (r < 0) {
        const PrimBox b = boxes[(int)(keys[~r] & 0xffffffffu)];
        for (int k = 0; k < 3; k++) { lo[c][k] = b.lo[k]; hi[c][k] = b.hi[k]; }
      } else {
        const volatile float *nb = node_box + 6 * r;
        for (int k = 0; k < 3; k++) { lo[c][k] = nb[k]; hi[c][k] = nb[3 + k]; }
      }
    }
    BvhNode nd = nodes[p];
    store_child(nd, 0, lo[0], hi[0]);
    store_child(nd, 1, lo[1], hi[1]);
    nodes[p] = nd;
    float *ob = node_box + 6 * p;
    for (int k = 0; k < 3; k++) {
      ob[k] = fminf(lo[0][k], lo[1][k]);
      ob[3 + k] = fmaxf(hi[0][k], hi[1][k]);
    }
    p = parent[p];
  }
}

__global__ void k_tri_boxes(const float *tris, int n, PrimBox *boxes) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float *v = tris + (size_t)i * 9;
  PrimBox b;
  for (int k = 0; k < 3; k++) {
    b.lo[k] = fminf(fminf(v[k], v[3 + k]), v[6 + k]);
    b.hi[k] = fmaxf(fmaxf(v[k], v[3 + k]), v[6 + k]);
  }
  boxes[i] = b;
}

__global__ void k_aabb_boxes(const float *aabb, int n, PrimBox *boxes) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  PrimBox b;
  for (int k = 0; k < 3; k++) { b.lo[k] = aabb[6 * i + k]; b.hi[k] = aabb[6 * i + 3 + k]; }
  boxes[i] = b;
}

// sorted triangle data: v0 (w = original index), v1, v2
__global__ void k_pack_tris(const float *tris, const int *perm, int n, float4 *out) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  int o = perm[j];
  const float *v = tris + (size_t)o * 9;
  out[3 * j + 0] = make_float4(v[0], v[1], v[2], __int_as_float(o));
  out[3 * j + 1] = make_float4(v[3], v[4], v[5], 0.0f);
  out[3 * j + 2] = make_float4(v[6], v[7], v[8], 0.0f);
}

// sorted sphere data: centre (w = original index), box lo, box hi
__global__ void k_pack_spheres(const float *pos, const float *aabb, const int *perm, int n,
                               float4 *out) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  int o = perm[j];
  out[3 * j + 0] = make_float4(pos[3 * o], pos[3 * o + 1], pos[3 * o + 2], __int_as_float(o));
  out[3 * j + 1] = make_float4(aabb[6 * o], aabb[6 * o + 1], aabb[6 * o + 2], 0.0f);
  out[3 * j + 2] = make_float4(aabb[6 * o + 3], aabb[6 * o + 4], aabb[6 * o + 5], 0.0f);
}

__global__ void k_sphere_aabbs(const float *pos, int n, float r, float *aabb) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int k = 0; k < 3; k++) {
    aabb[6 * i + k] = pos[3 * i + k] - r;
    aabb[6 * i + 3 + k] = pos[3 * i + k] + r;
  }
}

inline int nblk(int n, int b) { return (n + b - 1) / b; }

}  // namespace

size_t lbvh_scratch_bytes(int n) {
  size_t s = 0;
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  s += al(sizeof(PrimBox) * (size_t)n);      // boxes
  s += al(sizeof(uint64_t) * (size_t)n) * 2;  // keys ping-pong
  s += al(sizeof(int) * (size_t)(2 * n));     // parent
  s += al(sizeof(int) * (size_t)n);           // flags
  s += al(sizeof(float) * 6 * (size_t)n);     // node boxes
  s += al(sizeof(float) * 8);                 // bounds
  return s;
}

size_t lbvh_output_bytes(int n) {
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  return al(sizeof(BvhNode) * (size_t)(n > 1 ? n - 1 : 1)) + al(sizeof(int) * (size_t)n) +
         al(sizeof(float4) * 3 * (size_t)n);
}

static cudaError_t build_common(Lbvh &out, int n, char *scratch, char *outbuf,
                                cudaStream_t st) {
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  PrimBox *boxes = (PrimBox *)scratch;
  char *p = scratch + al(sizeof(PrimBox) * (size_t)n);
  uint64_t *ka = (uint64_t *)p; p += al(sizeof(uint64_t) * (size_t)n);
  uint64_t *kb = (uint64_t *)p; p += al(sizeof(uint64_t) * (size_t)n);
  int *parent = (int *)p; p += al(sizeof(int) * (size_t)(2 * n));
  int *flags = (int *)p; p += al(sizeof(int) * (size_t)n);
  float *nbox = (float *)p; p += al(sizeof(float) * 6 * (size_t)n);
  float *b6 = (float *)p;
  out.n = n;
  out.nodes = (BvhNode *)outbuf;
  out.perm = (int *)(outbuf + al(sizeof(BvhNode) * (size_t)(n > 1 ? n - 1 : 1)));
  out.prims = (float4 *)((char *)out.perm + al(sizeof(int) * (size_t)n));
  if (n == 0) return cudaSuccess;
  k_bounds<<<1, 1024, 0, st>>>(boxes, n, b6);
  k_morton<<<nblk(n, 256), 256, 0, st>>>(boxes, n, b6, ka);
  if (n <= kSmemSortMax) {
    static size_t attr_set[AMS_MAX_DEVICES] = {0};
    cudaError_t e = ams_set_smem_atleast(attr_set, k_sort_smem, kSmemSortMax * sizeof(uint64_t));
    if (e != cudaSuccess) return e;
    int np = 1;
    while (np < n) np <<= 1;
    k_sort_smem<<<1, 1024, np * sizeof(uint64_t), st>>>(ka, n);
  } else {
    k_sort<<<1, 1024, 0, st>>>(ka, kb, n);
  }
  if (n > 1) {
    k_karras<<<nblk(n - 1, 256), 256, 0, st>>>(ka, n, out.nodes, parent);
    cudaMemsetAsync(flags, 0, sizeof(int) * (size_t)n, st);
  }
  k_refit<<<nblk(n, 256), 256, 0, st>>>(ka, boxes, n, out.nodes, parent, flags, nbox, out.perm);
  return cudaGetLastError();
}

cudaError_t lbvh_build_triangles(Lbvh &out, const float *tris, int n, char *scratch,
                                 char *outbuf, cudaStream_t st) {
  if (n > 0) k_tri_boxes<<<nblk(n, 256), 256, 0, st>>>(tris, n, (PrimBox *)scratch);
  cudaError_t e = build_common(out, n, scratch, outbuf, st);
  if (e != cudaSuccess || n == 0) return e;
  k_pack_tris<<<nblk(n, 256), 256, 0, st>>>(tris, out.perm, n, out.prims);
  return cudaGetLastError();
}

cudaError_t lbvh_build_spheres(Lbvh &out, const float *pos, const float *aabb, int n,
                               char *scratch, char *outbuf, cudaStream_t st) {
  if (n > 0) k_aabb_boxes<<<nblk(n, 256), 256, 0, st>>>(aabb, n, (PrimBox *)scratch);
  cudaError_t e = build_common(out, n, scratch, outbuf, st);
  if (e != cudaSuccess || n == 0) return e;
  k_pack_spheres<<<nblk(n, 256), 256, 0, st>>>(pos, aabb, out.perm, n, out.prims);
  return cudaGetLastError();
}

cudaError_t lbvh_from_host(Lbvh &out, const float *tris, int n, const BvhNode *h_nodes,
                           const int *h_perm, char *outbuf, cudaStream_t st) {
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  out.n = n;
  out.nodes = (BvhNode *)outbuf;
  out.perm = (int *)(outbuf + al(sizeof(BvhNode) * (size_t)(n > 1 ? n - 1 : 1)));
  out.prims = (float4 *)((char *)out.perm + al(sizeof(int) * (size_t)n));
  if (n == 0) return cudaSuccess;
  cudaError_t e;
  if (n > 1 && (e = cudaMemcpyAsync(out.nodes, h_nodes, sizeof(BvhNode) * (size_t)(n - 1),
                                    cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return e;
  if ((e = cudaMemcpyAsync(out.perm, h_perm, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice,
                           st)) != cudaSuccess)
    return e;
  k_pack_tris<<<nblk(n, 256), 256, 0, st>>>(tris, out.perm, n, out.prims);
  return cudaGetLastError();
}

cudaError_t sphere_aabbs(const float *pos, int n, float r, float *aabb, cudaStream_t st) {
  if (n > 0) k_sphere_aabbs<<<nblk(n, 256), 256, 0, st>>>(pos, n, r, aabb);
  return cudaGetLastError();
}
