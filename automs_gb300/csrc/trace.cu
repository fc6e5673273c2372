// trace.cu -- the two-stage ray-traced channel simulator on GB300.
//
// Reference behaviour (file:line of the reference):
//   stage 1, forward discovery    optixPathTracer.cu:142-190, :285-331
//   stage 2, backward verify      optixPathTracer.cu:191-273, :332-417
//   sphere capture                optixPathTracer.cu:419-445
//   beam patterns                 optixPathTracer.cu:107-136
//   dedup + flood fill            optixPathTracer.cpp:127-354
//
// GB300 design:
//   * software BVH traversal over LBVHs (lbvh.cu) with a per-thread stack;
//     node culling is conservative, primitive tests are exact, and the
//     closest hit is chosen by (t, instance, primitive), so the hit does not
//     depend on traversal order.
//   * stage 1 inserts each forward record straight into a hashed path table
//     and a (cell x path) bitmap: no record buffer, no host round trip.
//   * stage 2 works on bitmaps: a round is "list new tasks -> trace the
//     25 x S backward rays of every task -> expand successes to the 4
//     neighbour cells"; the host only reads the new-task count.
//   * channel contributions are summed exactly in 64-bit fixed point, so H is
//     bit-reproducible whatever the launch order.
//   * this file is compiled with -fmad=false: the float arithmetic of every
//     decision matches the CPU oracle bit for bit.
#include "ams_common.cuh"
#include "trace.h"

namespace {

// Largest floats not above cos((2k-1) pi / 72), k = 1..18: the 5-degree bin
// edges of theta_id = int((acos|c| / (pi/2) * 36 + 1) / 2)
// (optixPathTracer.cu:304-306).
__constant__ unsigned c_theta_thr_bits[18] = {
    0x3f7fc19fu, 0x3f7dcf54u, 0x3f79ee88u, 0x3f7426cbu, 0x3f6c835eu, 0x3f631324u,
    0x3f57e880u, 0x3f4b1934u, 0x3f3cbe35u, 0x3f2cf37au, 0x3f1bd7c9u, 0x3f098c77u,
    0x3eec6a50u, 0x3ec3ef15u, 0x3e99f61cu, 0x3e5da258u, 0x3e05a8a8u, 0x3d32aa3eu};

__device__ __forceinline__ int theta_id(float c) {
  float a = fabsf(c);
  int id = 0;
#pragma unroll
  for (int k = 0; k < 18; k++) id += (a <= __uint_as_float(c_theta_thr_bits[k])) ? 1 : 0;
  return id;
}

// ------------------------------------------------------------------- RNG
// TEA-4 (Zafar, Olano, Curtis 2010) and the Numerical Recipes LCG
// (optix/SDK/cuda/random.h:31-61)
__device__ __forceinline__ uint32_t tea4(uint32_t v0, uint32_t v1) {
  uint32_t s0 = 0;
#pragma unroll
  for (int n = 0; n < 4; n++) {
    s0 += 0x9e3779b9u;
    v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
    v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
  }
  return v0;
}
__device__ __forceinline__ float rnd(uint32_t &seed) {
  seed = 1664525u * seed + 1013904223u;
  return (float)(seed & 0x00FFFFFFu) / (float)0x01000000;
}

// sin/cos of a float angle in [0, 7): Cody-Waite reduction by pi/2 with a
// two-part constant and Taylor series to degree 17/18 in double, rounded
// once to float (correctly rounded except within ~1e-16 of a midpoint).
__device__ __forceinline__ void sincos_exact(float a, float &s_out, float &c_out) {
  double x = (double)a;
  double kd = floor(x * 0.6366197723675814 + 0.5);
  double r = (x - kd * 1.5707963267341256) - kd * 6.077100506506192e-11;
  double r2 = r * r;
  double s = 2.8114572543455206e-15;
  s = s * r2 - 7.647163731819816e-13;
  s = s * r2 + 1.6059043836821613e-10;
  s = s * r2 - 2.505210838544172e-08;
  s = s * r2 + 2.7557319223985893e-06;
  s = s * r2 - 0.0001984126984126984;
  s = s * r2 + 0.008333333333333333;
  s = s * r2 - 0.16666666666666666;
  s = s * r2 + 1.0;
  s = s * r;
  double c = 1.5619206968586225e-16;
  c = c * r2 - 4.779477332387385e-14;
  c = c * r2 + 1.1470745597729725e-11;
  c = c * r2 - 2.08767569878681e-09;
  c = c * r2 + 2.755731922398589e-07;
  c = c * r2 - 2.48015873015873e-05;
  c = c * r2 + 0.001388888888888889;
  c = c * r2 - 0.041666666666666664;
  c = c * r2 + 0.5;
  c = 1.0 - c * r2;
  int q = ((int)kd) & 3;
  double so = q == 0 ? s : (q == 1 ? c : (q == 2 ? -s : -c));
  double co = q == 0 ? c : (q == 1 ? -s : (q == 2 ? -c : s));
  s_out = (float)so;
  c_out = (float)co;
}

// rand_dir, optixPathTracer.cu:56-68
__device__ __forceinline__ af3 rand_dir(uint32_t &seed, uint32_t ix, uint32_t iy, int lx, int ly) {
  float rnd1 = (rnd(seed) + (float)ix) / (float)lx;
  float rnd2 = (rnd(seed) + (float)iy) / (float)ly;
  float theta = (2.0f * AMS_PIF) * rnd1;
  float r = sqrtf(rnd2);
  float sn, cs;
  sincos_exact(theta, sn, cs);
  float u = r * cs, v = r * sn;
  float q = sqrtf(1.0f - r * r);
  return mk3((2.0f * u) * q, (2.0f * v) * q, 1.0f - (2.0f * r) * r);
}

// get_beampattern_factor, optixPathTracer.cu:107-136; branches on the float
// cosine against cos(120 deg) and cos(75 deg), taper value in float.
__device__ __forceinline__ float beampattern(af3 d1, af3 d2, int type) {
  float c = dot3(d1, d2) / (len3(d1) * len3(d2));
  switch (type) {
    case 0: return 1.0f;
    case 1: return c < 0.0f ? 0.0f : c * 2.4495f;
    case 2: {
      if ((double)c < -0.5) return 0.1f;
      if ((double)c < 0.25881904510252074) {
        float th = acosf(c);
        float e = (2.0943951f - th) * 0.31830987f * 4.0f * 0.41299623f - 1.0f;
        return exp10f(e) * 2.4495f;
      }
      return (float)((double)c * 2.4495);
    }
    case 3: return c < 0.0f ? 0.0f : 1.4142f;
    default: return 0.0f;
  }
}

// ------------------------------------------------------------ primitives
struct RayT {
  af3 o, d;
  af3 inv;              // 1 / d clamped to +-1e30 (exact wherever it is smaller)
  float oix, oiy, oiz;  // o * inv for the node test
  int kx, ky, kz;
  float Sx, Sy, Sz;
};

__device__ __forceinline__ void ray_setup(RayT &r, af3 o, af3 d) {
  r.o = o;
  r.d = d;
  // The fused node test computes lo * inv - o * inv.  For an axis-parallel
  // ray (a zero direction component) an infinite inverse would give
  // inf - inf = NaN, or -inf for a box that reaches below 0, and cull nodes
  // the ray is inside of.  The clamp keeps every term finite; node boxes are
  // widened far beyond its rounding error.  prim_slab recovers the exact
  // inverse where the clamp applies.
  const float big = 1e30f;
  r.inv = mk3(fminf(fmaxf(1.0f / d.x, -big), big), fminf(fmaxf(1.0f / d.y, -big), big),
              fminf(fmaxf(1.0f / d.z, -big), big));
  r.oix = o.x * r.inv.x;
  r.oiy = o.y * r.inv.y;
  r.oiz = o.z * r.inv.z;
  float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  int kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
  int kx = kz + 1; if (kx == 3) kx = 0;
  int ky = kx + 1; if (ky == 3) ky = 0;
  if (comp3(d, kz) < 0.0f) { int t = kx; kx = ky; ky = t; }
  r.kx = kx; r.ky = ky; r.kz = kz;
  float dz = comp3(d, kz);
  r.Sx = comp3(d, kx) / dz;
  r.Sy = comp3(d, ky) / dz;
  r.Sz = 1.0f / dz;
}

// Watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2(1) 2013).
__device__ __forceinline__ float tri_hit(const RayT &r, af3 v0, af3 v1, af3 v2) {
  af3 A = sub3(v0, r.o), B = sub3(v1, r.o), C = sub3(v2, r.o);
  float Az_ = comp3(A, r.kz), Bz_ = comp3(B, r.kz), Cz_ = comp3(C, r.kz);
  float Ax = comp3(A, r.kx) - r.Sx * Az_;
  float Ay = comp3(A, r.ky) - r.Sy * Az_;
  float Bx = comp3(B, r.kx) - r.Sx * Bz_;
  float By = comp3(B, r.ky) - r.Sy * Bz_;
  float Cx = comp3(C, r.kx) - r.Sx * Cz_;
  float Cy = comp3(C, r.ky) - r.Sy * Cz_;
  float U = Cx * By - Cy * Bx;
  float V = Ax * Cy - Ay * Cx;
  float W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return -1.0f;
  float det = U + V + W;
  if (det == 0.0f) return -1.0f;
  float Az = r.Sz * Az_, Bz = r.Sz * Bz_, Cz = r.Sz * Cz_;
  float T = U * Az + V * Bz + W * Cz;
  return T / det;
}

// slab gate in front of the sphere program (AABB given by the caller)
// exact 1 / d from the clamped inverse (recomputed only where clamped)
__device__ __forceinline__ float exact_inv(float clamped, float d) {
  return fabsf(clamped) < 1e30f ? clamped : 1.0f / d;
}

__device__ __forceinline__ bool prim_slab(const RayT &r, float4 lo, float4 hi) {
  const float ix = exact_inv(r.inv.x, r.d.x), iy = exact_inv(r.inv.y, r.d.y),
              iz = exact_inv(r.inv.z, r.d.z);
  float tx0 = (lo.x - r.o.x) * ix, tx1 = (hi.x - r.o.x) * ix;
  float ty0 = (lo.y - r.o.y) * iy, ty1 = (hi.y - r.o.y) * iy;
  float tz0 = (lo.z - r.o.z) * iz, tz1 = (hi.z - r.o.z) * iz;
  float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
  float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
  return tn <= tf && tf >= AMS_TMIN && tn <= AMS_TMAX;
}

// __intersection__sphere, optixPathTracer.cu:419-445; t = closest approach
// D = d * (1 / |d|) is passed in: the same for every sphere of one query
__device__ __forceinline__ float sphere_hit(const RayT &r, af3 D, af3 center, float radius) {
  af3 O = sub3(center, r.o);
  float b = dot3(O, D);
  float c = dot3(O, O);
  float acc = fmaxf(5e-5f, radius * radius);
  if ((c - b * b < acc) && b > 0.0f && sqrtf(c) > radius) {
    if (b > AMS_TMIN && b < AMS_TMAX) return b;
  }
  return -1.0f;
}

struct Hit { float t; int inst; int prim; };

__device__ __forceinline__ bool better(float t, int inst, int prim, const Hit &h) {
  if (t < h.t) return true;
  if (t > h.t) return false;
  if (inst != h.inst) return inst < h.inst;
  return prim < h.prim;
}

// conservative child test: widened boxes, loosened far bound
__device__ __forceinline__ bool child_test(const RayT &r, float lx, float ly, float lz, float hx,
                                           float hy, float hz, float best, float &tn_out) {
  float tx0 = __fmaf_rn(lx, r.inv.x, -r.oix), tx1 = __fmaf_rn(hx, r.inv.x, -r.oix);
  float ty0 = __fmaf_rn(ly, r.inv.y, -r.oiy), ty1 = __fmaf_rn(hy, r.inv.y, -r.oiy);
  float tz0 = __fmaf_rn(lz, r.inv.z, -r.oiz), tz1 = __fmaf_rn(hz, r.inv.z, -r.oiz);
  float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
  float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
  tn_out = tn;
  // the o*inv form loses a little accuracy; the slack below covers it
  return tn <= __fmaf_rn(tf, 1.0001f, 1e-5f) && tf >= -1e-5f &&
         tn <= __fmaf_rn(best, 1.0001f, 1e-4f);
}

__device__ __forceinline__ af3 unit_dir(const RayT &r) { return scl3(r.d, 1.0f / len3(r.d)); }

// INST 2 (the many Rx spheres) uses the unit direction computed once per
// query; INST 1 (Tx spheres, rarely past the slab gate) computes it here
template <int INST>
__device__ __forceinline__ void test_prim(const float4 *prims, int j, const RayT &r, Hit &best,
                                          float radius, const af3 &Dq) {
  const float4 a = __ldg(prims + 3 * j);
  const float4 b = __ldg(prims + 3 * j + 1);
  const float4 c = __ldg(prims + 3 * j + 2);
  int orig = __float_as_int(a.w);
  if (INST == 0) {
    float t = tri_hit(r, mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), mk3(c.x, c.y, c.z));
    if (t > AMS_TMIN && t < AMS_TMAX && better(t, 0, orig, best)) {
      best.t = t; best.inst = 0; best.prim = orig;
    }
  } else {
    if (!prim_slab(r, b, c)) return;
    float t = sphere_hit(r, INST == 2 ? Dq : unit_dir(r), mk3(a.x, a.y, a.z), radius);
    if (t >= 0.0f && better(t, INST, orig, best)) {
      best.t = t; best.inst = INST; best.prim = orig;
    }
  }
}

#define AMS_STACK 64
#define AMS_SEG_CAP 65536  // closest-hit queries per ray before giving up

template <int INST>
__device__ void traverse(const BvhNode *nodes, const float4 *prims, int n, const RayT &r,
                         Hit &best, float radius, unsigned *err) {
  if (n <= 0) return;
  af3 Dq = mk3(0.f, 0.f, 0.f);
  if (INST == 2) Dq = unit_dir(r);
  if (n == 1) { test_prim<INST>(prims, 0, r, best, radius, Dq); return; }
  int st_node[AMS_STACK];
  float st_t[AMS_STACK];
  int sp = 0;
  int node = 0;
  while (true) {
    if ((unsigned)node >= (unsigned)(n - 1)) { atomicOr(err, AMS_DERR_BVH); return; }
    const float4 *np = reinterpret_cast<const float4 *>(nodes + node);
    const float4 a = __ldg(np), b = __ldg(np + 1), c = __ldg(np + 2);
    const int4 d = __ldg(reinterpret_cast<const int4 *>(np + 3));
    float tn0, tn1;
    bool h0 = child_test(r, a.x, a.y, a.z, a.w, b.x, b.y, best.t, tn0);
    bool h1 = child_test(r, b.z, b.w, c.x, c.y, c.z, c.w, best.t, tn1);
    if (h0 && d.x < 0) {
      if (~d.x >= n) { atomicOr(err, AMS_DERR_BVH); return; }
      test_prim<INST>(prims, ~d.x, r, best, radius, Dq);
      h0 = false;
    }
    if (h1 && d.y < 0) {
      if (~d.y >= n) { atomicOr(err, AMS_DERR_BVH); return; }
      test_prim<INST>(prims, ~d.y, r, best, radius, Dq);
      h1 = false;
    }
    if (h0 && h1) {
      int nearn = d.x, farn = d.y;
      float tfar = tn1;
      if (tn1 < tn0) { nearn = d.y; farn = d.x; tfar = tn0; }
      if (sp < AMS_STACK) {
        st_node[sp] = farn; st_t[sp] = tfar; sp++;
      } else {
        atomicOr(err, AMS_DERR_STACK);
      }
      node = nearn;
    } else if (h0) {
      node = d.x;
    } else if (h1) {
      node = d.y;
    } else {
      bool found = false;
      while (sp > 0) {
        sp--;
        if (st_t[sp] <= __fmaf_rn(best.t, 1.0001f, 1e-4f)) { node = st_node[sp]; found = true; break; }
      }
      if (!found) break;
    }
  }
}

// Backward-ray query of stage 2: optixTrace with the visibility mask of the
// scene and the Tx spheres (optixPathTracer.cpp:417-424).  On a path's last
// segment the Tx sphere is the expected hit: finding it first bounds the
// scene traversal to the segment before it instead of the wall behind the
// Tx.  Other segments end on a triangle, so the scene goes first there.  The
// result is the same lexicographic minimum in either order.
__device__ __forceinline__ Hit closest_s2(const TraceDev &P, af3 o, af3 d, bool last) {
  RayT r;
  ray_setup(r, o, d);
  Hit h;
  h.t = AMS_TMAX; h.inst = 3; h.prim = 0x7fffffff;
#pragma unroll 1
  for (int ph = 0; ph < 2; ph++) {
    if ((ph == 0) == last) traverse<1>(P.tx_nodes, P.tx_prims, P.n_src, r, h, P.src_r, P.err);
    else traverse<0>(P.tri_nodes, P.tri_prims, P.n_tri, r, h, 0.0f, P.err);
  }
  return h;
}

// ---------------------------------------------------------- image method
struct Mat34 { float m[12]; };

__device__ __forceinline__ af3 image_of(const Mat34 &M, af3 p) {
  const float *m = M.m;
  return mk3(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3] * 1.0f,
             m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7] * 1.0f,
             m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11] * 1.0f);
}

// updateImageTransform, optixPathTracer.cu:70-76 (sum order of Matrix.h:339-356)
__device__ __forceinline__ void image_update(Mat34 &M, af3 N, af3 A) {
  float n[3] = {N.x, N.y, N.z};
  float a[9];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 3; j++) {
      float p = (2.0f * n[i]) * n[j];
      a[i * 3 + j] = (i == j ? 1.0f : 0.0f) - p;
    }
  Mat34 r;
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int j = 0; j < 4; j++) {
      float s = a[i * 3] * M.m[j];
      s = s + a[i * 3 + 1] * M.m[4 + j];
      s = s + a[i * 3 + 2] * M.m[8 + j];
      r.m[i * 4 + j] = s;
    }
  float k2 = 2.0f * dot3(A, N);
  r.m[3] = r.m[3] + k2 * N.x;
  r.m[7] = r.m[7] + k2 * N.y;
  r.m[11] = r.m[11] + k2 * N.z;
  M = r;
}

__device__ __forceinline__ int32_t fbits(float f) {
  int32_t b = __float_as_int(f);
  return b == (int32_t)0x80000000 ? 0 : b;  // -0 and +0 are one key
}

// Path-key hash: word-wise FNV-1a (Fowler, Noll, Vo) in 64 bits, finished
// by an avalanche mixer; it places the key in the open-addressed table.
__device__ __forceinline__ uint64_t key_hash64(const int32_t *k) {
  uint64_t h = 0xcbf29ce484222325ull;
#pragma unroll
  for (int i = 0; i < 14; i++) h = (h ^ (uint64_t)(uint32_t)k[i]) * 0x100000001b3ull;
  return mix64(h);
}

// OR a bit into a bitmap word (a reduction: the thread does not wait)
__device__ __forceinline__ void set_bit(unsigned *word, unsigned bit) { atomicOr(word, bit); }

// Key words are stored with the sign bit flipped.  A key never holds
// 0x80000000 (-0.0 is canonicalised to +0, and the hit count and reflect
// mask are small non-negative integers), so a stored word is never 0, and a
// 0 read back from a slot is a word its claiming thread has not written yet.
#define AMS_KEY_FLIP 0x80000000u
__device__ __forceinline__ int32_t key_word(const int32_t *slot_key, int i) {
  return (int32_t)((uint32_t)__ldg(slot_key + i) ^ AMS_KEY_FLIP);
}

// Claim or find the slot of a path key; returns -1 when the table is full.
// The 64-bit hash picks the first probe; a slot belongs to the key whose
// 14 words are stored in it.  One batch of loads reads a slot's hash and
// words: a slot with the same hash whose words are all written (non-zero)
// and equal is the key's slot; one whose words are still being written is
// re-read until they are (a few instructions of the claiming thread; the
// wait is bounded); a slot holding other words is passed over.  So two
// distinct keys never share a slot, and a key never takes two.
__device__ int path_insert(const TraceDev &P, const int32_t *key) {
  const uint64_t h = key_hash64(key) | 1ull;
  uint32_t enc[14];
#pragma unroll
  for (int i = 0; i < 14; i++) enc[i] = (uint32_t)key[i] ^ AMS_KEY_FLIP;
  uint32_t slot = (uint32_t)h & P.tab_mask;
  for (uint32_t probe = 0; probe <= P.tab_mask; probe++) {
    unsigned long long old = __ldcg(P.tab_h + slot);
    uint32_t *sk = reinterpret_cast<uint32_t *>(P.tab_key) + (size_t)slot * 14;
    if (old == 0ull) old = atomicCAS(P.tab_h + slot, 0ull, (unsigned long long)h);
    if (old == 0ull) {
#pragma unroll
      for (int i = 0; i < 14; i++) __stcg(sk + i, enc[i]);
      unsigned long long occ = atomicAdd(P.ctr + 2, 1ull);
      if (occ >= P.tab_limit) atomicOr(P.err, AMS_DERR_PATH_TABLE);
      return (int)slot;
    }
    if (old == (unsigned long long)h) {
      for (int spin = 0;; spin++) {
        uint32_t w[14];
        bool full = true, same = true;
#pragma unroll
        for (int i = 0; i < 14; i++) w[i] = __ldcg(sk + i);
#pragma unroll
        for (int i = 0; i < 14; i++) {
          full &= w[i] != 0u;
          same &= w[i] == enc[i];
        }
        if (same) return (int)slot;
        if (full) break;  // another key with this hash: probe on
        if (spin > (1 << 22)) { atomicOr(P.err, AMS_DERR_HASH); return -1; }
        __nanosleep(32);
      }
    }
    slot = (slot + 1u) & P.tab_mask;
  }
  atomicOr(P.err, AMS_DERR_PATH_TABLE);
  return -1;
}

// scene triangle by original primitive index (optixPathTracer.cu:296-299)
__device__ __forceinline__ void scene_tri(const TraceDev &P, int prim, af3 &v0, af3 &v1, af3 &v2) {
  const float *v = P.tris + (size_t)prim * 9;
  v0 = mk3(__ldg(v), __ldg(v + 1), __ldg(v + 2));
  v1 = mk3(__ldg(v + 3), __ldg(v + 4), __ldg(v + 5));
  v2 = mk3(__ldg(v + 6), __ldg(v + 7), __ldg(v + 8));
}

// ---------------------------------------------------------------- stage 1
// A branch slot whose ray waits while an earlier-indexed one is traced (the
// reference's 32-entry PRD stack, optixPathTracer.cu:152-190).  Its
// remaining levels follow from the index: a reflection spawned at hit count
// hc sets bit hc - 1 as the slot's highest bit and keeps L + 1 - hc levels.
struct Slot {
  af3 o, d;
  Mat34 M;
};

__device__ __forceinline__ int slot_ttl(int L, int j) { return L - (31 - __clz(j)); }

// Image matrix of the lane's current ray: slot 0 (the primary ray) is the
// identity and is never stored; any other slot's matrix sits in one per-lane
// array (48 bytes of local memory that stay in L1; a shared-memory copy
// measured 3% slower, its 6 KB per CTA taken from L1).
struct CurMatrix {
  float *cm;  // the lane's 12 floats
  __device__ __forceinline__ Mat34 get(int cur) const {
    Mat34 M;
#pragma unroll
    for (int k = 0; k < 12; k++)
      M.m[k] = cur == 0 ? ((k == 0 || k == 5 || k == 10) ? 1.0f : 0.0f) : cm[k];
    return M;
  }
  __device__ __forceinline__ void set(const Mat34 &M) const {
#pragma unroll
    for (int k = 0; k < 12; k++) cm[k] = M.m[k];
  }
};



// Stage 1 runs as a persistent loop per warp with dynamic fetching (after
// Aila & Laine, "Understanding the efficiency of ray traversal on GPUs",
// HPG 2009).  All lanes visit BVH nodes of their own closest-hit queries
// (Rx spheres, then the scene pruned at the sphere hit) in one loop whose
// body is a single node visit, until every lane's query has ended; then all
// lanes handle their hits together and set up their next queries (the next
// segment, the next pending slot, the next sub-launch, or a launch index
// fetched from a global counter), and the next round of node visits starts.
// Lanes that finish a short ray take new work instead of idling behind the
// warp's longest ray, and the hit code runs once per round for the whole
// warp.  (Handling the hits of a subset of lanes while the others still
// traverse measured slower at every threshold tried: the hit code is long.)
// Per launch index the queries, hits and records come in the order of the
// sequential trace (slots in increasing index, which is the order
// __ffs(pending) gives because a spawned slot always has a higher index than
// its parent), so the per-thread min_hc dedup and the reserve cap see
// exactly what they see in the reference.
enum { PH_RX = 0, PH_SCENE = 1, PH_HIT = 2 };

// warp-aggregated fetch of one launch index per calling lane
__device__ __forceinline__ long long fetch_launch(unsigned long long *ctr) {
  const unsigned m = __activemask();
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(m) - 1;
  unsigned long long base = 0;
  if (lane == leader) base = atomicAdd(ctr, (unsigned long long)__popc(m));
  base = __shfl_sync(m, base, leader);
  return (long long)(base + (unsigned long long)__popc(m & ((1u << lane) - 1u)));
}

struct S1Query {
  RayT r;
  af3 Dq;  // unit direction for the sphere tests
  Hit best;
  int phase, node, sp;
};

// first node of the query's next instance, or PH_HIT; one-primitive
// instances are tested here (they have no nodes)
__device__ __forceinline__ void s1_enter(const TraceDev &P, S1Query &q, int phase) {
  q.node = 0;
  q.sp = 0;
  if (phase == PH_RX) {
    if (P.n_dst > 1) { q.phase = PH_RX; return; }
    if (P.n_dst == 1) test_prim<2>(P.rx_prims, 0, q.r, q.best, P.dst_r, q.Dq);
  }
  if (P.n_tri > 1) { q.phase = PH_SCENE; return; }
  if (P.n_tri == 1) test_prim<0>(P.tri_prims, 0, q.r, q.best, 0.0f, q.Dq);
  q.phase = PH_HIT;
}

struct S1Ray {
  long long li;
  int ix, iy, launch, res_cnt;
  uint32_t seed;
  bool capped;
  af3 spos;
  unsigned pending;
  int cur, ttl, guard;
  // path-table slot of the last record's key: the key is a function of
  // (slot, remaining levels) within one sub-launch, and consecutive records
  // along a ray mostly repeat it
  int key_cur, key_ttl, key_slot;
};

// the hit of the finished query (stage-1 closest-hit program,
// optixPathTracer.cu:285-331)
__device__ __forceinline__ void s1_hit(const TraceDev &P, S1Query &q, S1Ray &w, Slot *slots,
                                    const CurMatrix &cm, volatile int *los_slot, int *rec,
                                    unsigned long long &my_records) {
  const int L = P.L;
  if (q.best.inst == 3) { w.ttl = 0; return; }
  const af3 d = q.r.d;
  const af3 o = add3(q.r.o, scl3(d, q.best.t));
  q.r.o = o;
  if (q.best.inst == 0 && w.ttl > 1) {
    af3 v0, v1, v2;
    scene_tri(P, q.best.prim, v0, v1, v2);
    af3 N0 = nrm3(cross3(sub3(v1, v0), sub3(v2, v0)));
    af3 N = faceforward3(N0, neg3(d), N0);
    int m = __ldg(P.mat + q.best.prim);
    float ct = dot3(d, N) / (len3(N) * len3(d));
    int tid = theta_id(ct);
    bool pen = __ldg(P.mat_prop + tid + m * AMS_NBINS) < 0.0f;
    w.ttl--;
    int hc = L + 1 - w.ttl;
    int j = w.cur | (1 << (hc - 1));
    Mat34 M = cm.get(w.cur);
    af3 V = sub3(v0, image_of(M, w.spos));
    af3 Nimg = faceforward3(N0, V, N0);
    image_update(M, Nimg, v0);
    const af3 dr = sub3(d, scl3(N, 2.0f * dot3(d, N)));
    if (!pen && (w.pending & ((1u << j) - 1u)) == 0u) {
      // the current ray stops and the new slot is the lowest pending one, so
      // it is the next to be traced: continue with it at once, without
      // storing it (always the case when no material is penetrable)
      w.cur = j;
      w.guard = 0;
      q.r.d = dr;
      cm.set(M);
    } else {
      Slot &c = slots[j];
      c.o = o;
      c.d = dr;
      c.M = M;
      w.pending |= 1u << j;
      if (!pen) w.ttl = 0;
    }
  } else if (q.best.inst == 2) {
    if (w.res_cnt < P.reserve) {
      int d0 = q.best.prim / P.n1_dst, d1 = q.best.prim % P.n1_dst;
      int cell = (d0 / P.gs) * P.n1g + d1 / P.gs;
      int hc = L + 1 - w.ttl;
      int mhc = 0;
      for (int k = w.res_cnt - 1; k >= 0; k--)
        if ((rec[k] >> 3) == cell) { mhc = (rec[k] & 7) + 1; break; }
      if (mhc <= hc) {
        rec[w.res_cnt++] = cell * 8 + hc;
        int slot = w.key_slot;
        if (w.key_cur != w.cur || w.key_ttl != w.ttl) {
          // the primary ray's key depends on the hit count only (identity
          // matrix, slot 0), so the CTA keeps its slot per hit count
          slot = w.cur == 0 ? los_slot[hc] : -1;
          if (slot < 0) {
            int32_t key[14];
            const Mat34 M = cm.get(w.cur);
#pragma unroll
            for (int k = 0; k < 12; k++) key[k] = fbits(M.m[k]);
            key[12] = hc;
            key[13] = w.cur;
            slot = path_insert(P, key);
            if (w.cur == 0 && slot >= 0) los_slot[hc] = slot;
          }
          w.key_cur = w.cur;
          w.key_ttl = w.ttl;
          w.key_slot = slot;
        }
        if (slot >= 0) set_bit(P.T + (size_t)cell * P.W + (slot >> 5), 1u << (slot & 31));
        my_records++;
      }
    } else {
      w.capped = true;
    }
  }
}

// next query of the lane: the current slot's next segment, the next pending
// slot, the next sub-launch, or the next launch index.  Returns false when
// no launch index is left.
__device__ __forceinline__ bool s1_next(const TraceDev &P, S1Query &q, S1Ray &w, const Slot *slots,
                                       const CurMatrix &cm, long long n_fetch, long long tiles_y,
                                       unsigned long long &my_capped) {
  while (true) {
    if (w.ttl > 0) {
      if (++w.guard > AMS_SEG_CAP) {
        atomicOr(P.err, AMS_DERR_LOOP);
        w.ttl = 0;
        continue;
      }
      ray_setup(q.r, q.r.o, q.r.d);
      q.Dq = unit_dir(q.r);
      q.best.t = AMS_TMAX; q.best.inst = 3; q.best.prim = 0x7fffffff;
      s1_enter(P, q, PH_RX);
      return true;
    }
    if (w.pending) {
      w.cur = __ffs(w.pending) - 1;
      w.pending &= w.pending - 1u;
      q.r.o = slots[w.cur].o;
      q.r.d = slots[w.cur].d;
      cm.set(slots[w.cur].M);
      w.ttl = slot_ttl(P.L, w.cur);
      w.guard = 0;
      continue;
    }
    if (w.li >= 0 && w.launch < P.spl) {
      w.launch++;
      float rs = rnd(w.seed) * (float)P.n_src;
      uint32_t src = (uint32_t)rs;
      if (src >= (uint32_t)P.n_src) src = (uint32_t)P.n_src - 1u;
      w.spos = ld3(P.src + 3 * src);
      // slot 0 (the primary ray) starts at once: origin and direction go
      // straight into the query, and its image matrix is the identity,
      // which is never stored (CurMatrix)
      q.r.o = w.spos;
      q.r.d = rand_dir(w.seed, (uint32_t)w.ix, (uint32_t)w.iy, P.launch_x, P.launch_y);
      w.cur = 0;
      w.ttl = P.L + 1;
      w.guard = 0;
      w.pending = 0u;
      w.key_cur = -1;  // a new ray: forget the last key
      continue;
    }
    if (w.li >= 0 && w.capped) my_capped++;
    // launch indices are dealt in tiles of 4 (ix, azimuth) x 8 (iy, height)
    // cells, so lanes that fetch together trace neighbouring directions
    // (4.09 ms on coverage-128 against 4.26 ms for 1 x 32 runs of iy and
    // 4.24-4.39 ms for 8 x 4 .. 32 x 1); n_fetch counts the tiles' cells,
    // those outside the launch are skipped
    while (true) {
      const long long f = fetch_launch(P.ctr + 10);
      if (f >= n_fetch) return false;
      const long long tile = f >> 5;
      const int c = (int)(f & 31);
      const int ix = (int)(tile / tiles_y) * 4 + (c & 3);
      const int iy = (int)(tile % tiles_y) * 8 + (c >> 2);
      if (ix < P.launch_x && iy < P.launch_y) {
        w.li = f;
        w.ix = ix;
        w.iy = iy;
        break;
      }
    }
    w.seed = tea4((uint32_t)w.ix * (uint32_t)P.launch_y + (uint32_t)w.iy, 0u);
    w.launch = 0;
    w.res_cnt = 0;
    w.capped = false;
  }
}

// 8 CTAs of 128 per SM (64 registers) measured fastest among 4 to 12.
// LMAX bounds max_reflection: 2^LMAX branch slots (slot indices hold one bit
// per hit count below L).
template <int LMAX>
__global__ void __launch_bounds__(128, 8) k_stage1(TraceDev P) {
  const long long tiles_y = (P.launch_y + 7) / 8;
  const long long n_fetch = (long long)((P.launch_x + 3) / 4) * tiles_y * 32;
  unsigned long long my_records = 0, my_segs = 0, my_capped = 0;
  float curm[12];
  const CurMatrix cm{curm};
  // path-table slot of the primary ray's key per hit count (-1: not known)
  __shared__ int s_los[AMS_MAX_L + 2];
  if (threadIdx.x < AMS_MAX_L + 2) s_los[threadIdx.x] = -1;
  __syncthreads();
  int rec[AMS_MAX_RESERVE];  // cell * 8 + hit_cnt of the records kept so far
  Slot slots[1 << LMAX];     // deferred branch slots
  int st_node[AMS_STACK];
  float st_t[AMS_STACK];

  S1Ray w;
  w.li = -1; w.ix = 0; w.iy = 0; w.launch = 0; w.res_cnt = 0; w.seed = 0u; w.capped = false;
  w.spos = mk3(0.f, 0.f, 0.f); w.pending = 0u; w.cur = 0; w.ttl = 0; w.guard = 0;
  w.key_cur = -1; w.key_ttl = 0; w.key_slot = -1;
  S1Query q;
  ray_setup(q.r, mk3(0.f, 0.f, 0.f), mk3(0.f, 0.f, 1.f));
  q.Dq = mk3(0.f, 0.f, 1.f);
  q.best.t = AMS_TMAX; q.best.inst = 3; q.best.prim = 0x7fffffff;
  q.phase = PH_HIT; q.node = 0; q.sp = 0;
  bool live = s1_next(P, q, w, slots, cm, n_fetch, tiles_y, my_capped);

  while (__any_sync(0xffffffffu, live)) {
    // ---- traversal: node visits until every lane's query has ended
    while (true) {
      const bool trav = live && q.phase != PH_HIT;
      if (__ballot_sync(0xffffffffu, trav) == 0u) break;
      if (trav) {
        const bool rx = q.phase == PH_RX;
        const BvhNode *nodes = rx ? P.rx_nodes : P.tri_nodes;
        const float4 *prims = rx ? P.rx_prims : P.tri_prims;
        const int n = rx ? P.n_dst : P.n_tri;
        bool more = true;
        if ((unsigned)q.node >= (unsigned)(n - 1)) {
          atomicOr(P.err, AMS_DERR_BVH);
          more = false;
        } else {
          const float4 *np = reinterpret_cast<const float4 *>(nodes + q.node);
          const float4 a = __ldg(np), b = __ldg(np + 1), c = __ldg(np + 2);
          const int4 d = __ldg(reinterpret_cast<const int4 *>(np + 3));
          float tn0, tn1;
          bool h0 = child_test(q.r, a.x, a.y, a.z, a.w, b.x, b.y, q.best.t, tn0);
          bool h1 = child_test(q.r, b.z, b.w, c.x, c.y, c.z, c.w, q.best.t, tn1);
          // leaves: one test site for both children
          int lf0 = (h0 && d.x < 0) ? ~d.x : -1;
          int lf1 = (h1 && d.y < 0) ? ~d.y : -1;
          if (lf0 >= 0) h0 = false;
          if (lf1 >= 0) h1 = false;
          if (lf0 >= n || lf1 >= n) {
            atomicOr(P.err, AMS_DERR_BVH);
            more = false;
          } else {
#pragma unroll 1
            for (int k = 0; k < 2; k++) {
              const int lf = k == 0 ? lf0 : lf1;
              if (lf < 0) continue;
              if (rx) test_prim<2>(prims, lf, q.r, q.best, P.dst_r, q.Dq);
              else test_prim<0>(prims, lf, q.r, q.best, 0.0f, q.Dq);
            }
            if (h0 && h1) {
              int nearn = d.x, farn = d.y;
              float tfar = tn1;
              if (tn1 < tn0) { nearn = d.y; farn = d.x; tfar = tn0; }
              if (q.sp < AMS_STACK) {
                st_node[q.sp] = farn; st_t[q.sp] = tfar; q.sp++;
              } else {
                atomicOr(P.err, AMS_DERR_STACK);
              }
              q.node = nearn;
            } else if (h0) {
              q.node = d.x;
            } else if (h1) {
              q.node = d.y;
            } else {
              more = false;
              const float lim = __fmaf_rn(q.best.t, 1.0001f, 1e-4f);
              while (q.sp > 0) {
                q.sp--;
                if (st_t[q.sp] <= lim) { q.node = st_node[q.sp]; more = true; break; }
              }
            }
          }
        }
        if (!more) {
          if (rx) s1_enter(P, q, PH_SCENE);
          else q.phase = PH_HIT;
        }
      }
    }
    // ---- hits of the waiting lanes, then their next queries
    if (live && q.phase == PH_HIT) {
      my_segs++;
      s1_hit(P, q, w, slots, cm, s_los, rec, my_records);
      live = s1_next(P, q, w, slots, cm, n_fetch, tiles_y, my_capped);
    }
  }
  // block-aggregated counters
  unsigned long long rr = my_records, sg = my_segs, cp = my_capped;
  for (int off = 16; off > 0; off >>= 1) {
    rr += __shfl_xor_sync(0xffffffffu, rr, off);
    sg += __shfl_xor_sync(0xffffffffu, sg, off);
    cp += __shfl_xor_sync(0xffffffffu, cp, off);
  }
  if ((threadIdx.x & 31) == 0) {
    if (rr) atomicAdd(P.ctr + 0, rr);
    if (sg) atomicAdd(P.ctr + 8, sg);
    if (cp) atomicAdd(P.ctr + 1, cp);
  }
}

// --------------------------------------------------------------- tasks
// Dense path ids: after stage 1 the path table is final, so stage 2 numbers
// its paths 0 .. n_paths - 1 (slot_of maps back to the table) and keeps its
// bitmaps [cell][W] with W = ceil(n_paths / 32) words instead of one bit per
// table slot.  The numbering follows the order in which threads claim ids;
// nothing computed depends on it (sums are exact, lists are per cell).
__global__ void k_dense_ids(TraceDev P, int *dense_of, unsigned long long *n) {
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s <= P.tab_mask;
       s += gridDim.x * blockDim.x) {
    if (P.tab_h[s] == 0ull) continue;
    const unsigned long long id = atomicAdd(n, 1ull);
    dense_of[s] = (int)id;
    P.slot_of[id] = (int)s;
  }
}

// out[cell][dense id] = the bits of in[cell][slot] (out zeroed before)
__global__ void k_to_dense(TraceDev P, const unsigned *in, int w_in, const int *dense_of,
                           unsigned *out) {
  const long long nwords = (long long)P.ng * w_in;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nwords;
       i += (long long)gridDim.x * blockDim.x) {
    unsigned b = in[i];
    if (!b) continue;
    const int cell = (int)(i / w_in), w = (int)(i % w_in);
    while (b) {
      const int k = __ffs(b) - 1;
      b &= b - 1u;
      const int d = dense_of[w * 32 + k];
      atomicOr(out + (size_t)cell * P.W + (d >> 5), 1u << (d & 31));
    }
  }
}

// The round's tasks, listed per cell: cell c's new paths (dense ids) are
// task_path[cell_off[c] .. cell_off[c + 1]) in increasing order, cut into
// chunks of up to kpi paths: chunk_at[chunk_off[c] ..] = (cell, first
// task).  A warp per cell counts, one CTA scans, a warp per cell fills.
// tasks per cell of the first round (later rounds: k_expand counts them)
__global__ void k_cell_counts(TraceDev P, const unsigned *bits) {
  const int lane = threadIdx.x & 31;
  const int nwarp = (gridDim.x * blockDim.x) >> 5;
  for (int cell = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; cell < P.ng; cell += nwarp) {
    const unsigned *row = bits + (size_t)cell * P.W;
    int c = 0;
    for (int w = lane; w < P.W; w += 32) c += __popc(row[w]);
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) P.cell_cnt[cell] = c;
  }
}

// exclusive scans of the task and chunk counts (cell_cnt, zeroed for the
// next round's counts) into cell_off and chunk_off ([ng] = totals), and the
// round's counters reset; one CTA of 1024 threads
__global__ void __launch_bounds__(1024) k_cell_scan(TraceDev P) {
  __shared__ int wsum[32], wch[32];
  __shared__ int carry_s, ccarry_s;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  if (t == 0) { carry_s = 0; ccarry_s = 0; }
  __syncthreads();
  for (int base = 0; base < P.ng; base += 1024) {
    const int i = base + t;
    const int v = i < P.ng ? P.cell_cnt[i] : 0;
    if (i < P.ng) P.cell_cnt[i] = 0;
    const int ch = (v + P.kpi - 1) / P.kpi;
    int x = v, y = ch;
    for (int o = 1; o < 32; o <<= 1) {
      const int x2 = __shfl_up_sync(0xffffffffu, x, o);
      const int y2 = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) { x += x2; y += y2; }
    }
    if (lane == 31) { wsum[wid] = x; wch[wid] = y; }
    __syncthreads();
    int xb = 0, yb = 0;
    for (int k = 0; k < wid; k++) { xb += wsum[k]; yb += wch[k]; }
    const int carry = carry_s, ccarry = ccarry_s;
    if (i < P.ng) {
      P.cell_off[i] = carry + xb + x - v;
      P.chunk_off[i] = ccarry + yb + y - ch;
    }
    __syncthreads();
    if (t == 0) {
      int xs = 0, ys = 0;
      for (int k = 0; k < 32; k++) { xs += wsum[k]; ys += wch[k]; }
      carry_s = carry + xs;
      ccarry_s = ccarry + ys;
    }
    __syncthreads();
  }
  if (t == 0) {
    P.cell_off[P.ng] = carry_s;
    P.chunk_off[P.ng] = ccarry_s;
    P.ctr[5] = (unsigned long long)carry_s;
    P.ctr[7] = 0ull;  // new tasks, counted by k_expand after this round's stage 2
  }
}

__global__ void k_cell_fill(TraceDev P, const unsigned *bits) {
  const int lane = threadIdx.x & 31;
  const int nwarp = (gridDim.x * blockDim.x) >> 5;
  for (int cell = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; cell < P.ng; cell += nwarp) {
    const int first = P.cell_off[cell], end = P.cell_off[cell + 1];
    if (first == end) continue;
    const unsigned *row = bits + (size_t)cell * P.W;
    long long pos = first;
    for (int w0 = 0; w0 < P.W; w0 += 32) {
      const int w = w0 + lane;
      unsigned b = w < P.W ? row[w] : 0u;
      const int c = __popc(b);
      int x = c;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      long long q = pos + x - c;
      while (b) {
        const int k = __ffs(b) - 1;
        b &= b - 1u;
        const int id = w * 32 + k;
        if ((unsigned long long)q < P.task_cap)
          P.task_path[q] = make_int2(id, id < P.n_paths ? P.slot_of[id] : -1);
        else atomicOr(P.err, AMS_DERR_TASKS);
        q++;
      }
      pos += __shfl_sync(0xffffffffu, x, 31);
    }
    const int c0 = P.chunk_off[cell], c1 = P.chunk_off[cell + 1];
    for (int j = c0 + lane; j < c1; j += 32) {
      const int t0 = first + (j - c0) * P.kpi;
      if ((unsigned long long)j < P.task_cap) P.chunk_at[j] = make_int4(cell, t0, min(end, t0 + P.kpi), 0);
      else atomicOr(P.err, AMS_DERR_TASKS);
    }
  }
  // the success bits of the coming stage 2 start empty
  const long long nw = (long long)P.ng * P.W;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nw;
       i += (long long)gridDim.x * blockDim.x)
    P.S[i] = 0u;
}

// ---------------------------------------------------------------- stage 2
// One backward ray (stage-2 raygen + closest-hit programs,
// optixPathTracer.cu:191-273, :332-417): the image source of the path key in
// `slot` seen from Rx position o, traced back to Tx `s`.  Returns true with
// the contribution as 2^-56 fixed point when the ray arrives.
template <bool EXPORT = false>
__device__ __forceinline__ bool s2_ray(const TraceDev &P, int slot, int s, af3 o, af3 srcdir,
                                       af3 dstdir, unsigned &segs, unsigned long long &cre,
                                       unsigned long long &cim, ams_ray_record *rr = nullptr) {
  const int32_t *key = P.tab_key + (size_t)slot * 14;
  Mat34 M;
#pragma unroll
  for (int k = 0; k < 12; k++) M.m[k] = __int_as_float(key_word(key, k));
  const int hc = key_word(key, 12), mask = key_word(key, 13);
  const float lam = P.lam_f;
  af3 d = nrm3(sub3(image_of(M, ld3(P.src + 3 * s)), o));
  float amp = beampattern(d, dstdir, P.dst_bp);
  float xloss = 1.0f;  // exported: free-space factors only
  if (EXPORT) {
    rr->receive_angle = dot3(d, dstdir) / (len3(d) * len3(dstdir));
    rr->hit_cnt = 0;
  }
  float far = 1e6f, dd = 0.0f, dres = 0.0f;
  double D = 0.0;
  int ttl = hc + 1;
  int guard = 0;
  bool ok = false;
  while (ttl > 0) {
    if (++guard > AMS_SEG_CAP) { atomicOr(P.err, AMS_DERR_LOOP); break; }
    Hit h = closest_s2(P, o, d, ttl == 1);
    segs++;
    if (h.inst == 3) break;
    const float t = h.t;
    o = add3(o, scl3(d, t));
    dd += t;
    D += (double)t;
    if (h.inst == 0) {
      if (ttl == 1) break;
      af3 v0, v1, v2;
      scene_tri(P, h.prim, v0, v1, v2);
      af3 N0 = nrm3(cross3(sub3(v1, v0), sub3(v2, v0)));
      af3 N = faceforward3(N0, neg3(d), N0);
      int m = __ldg(P.mat + h.prim);
      float ct = dot3(d, N) / (len3(N) * len3(d));
      float loss = fabsf(__ldg(P.mat_prop + theta_id(ct) + m * AMS_NBINS));
      ttl--;
      int hcb = hc + 1 - ttl;
      int is_ref = (mask >> (hcb - 1)) & 1;
      float max_d = fmaxf(fmaxf(len3(sub3(v0, v1)), len3(sub3(v1, v2))), len3(sub3(v2, v0)));
      float fspl = 1.0f;
      if (dd > far) { fspl = lam / ((4.0f * AMS_PIF) * dres); dres = 0.0f; }
      amp *= loss * fspl;
      dres += dd;
      if (EXPORT) {
        if (rr->hit_cnt < 5) rr->hit_loss_idx[rr->hit_cnt] = theta_id(ct) + m * AMS_NBINS;
        rr->hit_cnt++;
        xloss *= fspl;
      }
      // far_dist = 2 max_d^2 / lambda, divided in double and rounded to
      // float (optixPathTracer.cu:385-389).  Its value matters only when
      // the segment is longer; a float estimate (relative error < 3e-7)
      // with a 1e-5 margin settles the common near-field case without
      // the double division (FP64 is slow on this part).
      float far_next = 1e6f;
      if (dd > ((2.0f * max_d) * max_d / lam) * 0.99999f) {
        const float fd = (float)(2.0 * (double)max_d * (double)max_d / (double)lam);
        far_next = (dd > fd) ? fd : 1e6f;
      }
      far = far_next;
      dd = 0.0f;
      if (is_ref) d = sub3(d, scl3(N, 2.0f * dot3(d, N)));
    } else if (h.inst == 1 && h.prim == s) {
      if (ttl == 1) {
        float bp = beampattern(neg3(d), srcdir, P.src_bp);
        float af = lam / ((4.0f * AMS_PIF) * (dres + dd));
        amp *= bp * af;
        ok = true;
        if (EXPORT) {
          const af3 nd = neg3(d);
          rr->launch_angle = dot3(nd, srcdir) / (len3(nd) * len3(srcdir));
          rr->loss = xloss * af;
          rr->phase = D * P.two_pi_over_lam;
        }
      }
      break;
    }
  }
  if (ok) {
    // FP64 path length -> phase, reduced mod 2 pi in FP64 (products with
    // precomputed 2 pi / lambda and 1 / (2 pi): no FP64 division per ray)
    double ph = D * P.two_pi_over_lam;
    ph = ph - 6.283185307179586 * floor(ph * 0.15915494309189535);
    float sn, cs;
    sincosf((float)ph, &sn, &cs);
    // the contribution in 2^-56 fixed point, in FP32: the limit (64) and the
    // scale (2^56) are powers of two, so the range test and the scaling are
    // exact in float and the rounding to an integer sees the same value as
    // a conversion through double would (FP64 is slow on this part)
    const float re = amp * cs, im = -amp * sn;
    if (!(fabsf(re) < (float)AMS_ACC_LIMIT && fabsf(im) < (float)AMS_ACC_LIMIT)) {
      atomicOr(P.err, AMS_DERR_ACC_RANGE);
      return false;
    }
    cre = (unsigned long long)__float2ll_rn(re * (float)AMS_ACC_SCALE);
    cim = (unsigned long long)__float2ll_rn(im * (float)AMS_ACC_SCALE);
  }
  return ok;
}

// Persistent stage 2: a warp takes an item = (a chunk of up to kpi of one
// cell's new paths, 32 consecutive (Rx within the cell, Tx) pairs, Tx
// fastest) and traces the chunk's paths one after the other; each
// lane sums its pair's contributions over the chunk in registers (exact
// 64-bit fixed point) and adds them once into the Rx-major accumulator
// acc[dst][s], so a warp's adds cover one or a few contiguous runs of Tx
// (coalesced), one atomic add per (Tx, Rx) and chunk instead of two per
// verified ray.  The lanes of an item trace the same path key from the same
// Rx to neighbouring Tx elements: nearly identical rays.  One warp per item,
// 8 per CTA: the block scheduler balances items of uneven cost (fixed
// strides over persistent warps and a fetch counter both measured slower);
// kpi is chosen per round by the host so that a round keeps several items
// per resident warp.
__global__ void __launch_bounds__(256, 5) k_stage2(TraceDev P) {
  const int S = P.n_src;
  const long long pairs = (long long)P.gs * P.gs * S;
  const long long G = (pairs + 31) / 32;
  const long long n_items = (long long)P.chunk_off[P.ng] * G;
  const int lane = threadIdx.x & 31;
  const af3 srcdir = mk3(P.src_dir[0], P.src_dir[1], P.src_dir[2]);
  const af3 dstdir = mk3(P.dst_dir[0], P.dst_dir[1], P.dst_dir[2]);
  unsigned n_ok = 0, n_fail = 0, n_segs = 0, n_adds = 0;  // n_adds: warp total
  if (blockIdx.x == 0 && threadIdx.x == 0 && n_items > (long long)gridDim.x * (blockDim.x >> 5))
    atomicOr(P.err, AMS_DERR_TASKS);  // the launch must cover every item
  {
    const long long item = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (item >= n_items) return;
    const int4 chunk = __ldg(P.chunk_at + item / G);
    const int cell = chunk.x, t0 = chunk.y, t1 = chunk.z;
    if ((unsigned)cell >= (unsigned)P.ng || t0 < 0 || t1 < t0 ||
        (unsigned long long)t1 > P.task_cap) {
      if (lane == 0) atomicOr(P.err, AMS_DERR_TASKS);
      return;
    }
    const long long pr = (long long)(item % G) * 32 + lane;
    bool act = pr < pairs;
    const int inner = act ? (int)(pr / S) : 0, s = act ? (int)(pr % S) : 0;
    const int gi = cell / P.n1g, gj = cell % P.n1g;
    const int di = inner / P.gs + gi * P.gs, dj = inner % P.gs + gj * P.gs;
    const int dst = di * P.n1_dst + dj;
    if (dst >= P.n_dst || (P.strict_grid && (di >= P.n0_dst || dj >= P.n1_dst))) act = false;
    unsigned long long sre = 0, sim = 0;
    for (int t = t0; t < t1; t++) {
      const int2 task = __ldg(P.task_path + t);
      const int path = task.x, slot = task.y;
      if ((unsigned)path >= (unsigned)P.n_paths || (unsigned)slot > P.tab_mask) {
        if (lane == 0) atomicOr(P.err, AMS_DERR_TASKS);
        break;
      }
      bool ok = false;
      if (act) {
        unsigned long long cre = 0, cim = 0;
        ok = s2_ray(P, slot, s, ld3(P.dst + 3 * dst), srcdir, dstdir, n_segs, cre, cim);
        if (ok) { sre += cre; sim += cim; n_ok++; } else { n_fail++; }
      }
      if (__any_sync(0xffffffffu, ok) && lane == 0)
        atomicOr(P.S + (size_t)cell * P.W + (path >> 5), 1u << (path & 31));
    }
    const bool add = act && (sre | sim);
    if (add) {
      unsigned long long *acc = P.acc + ((size_t)dst * S + s) * 2;
      atomicAdd(acc, sre);
      atomicAdd(acc + 1, sim);
    }
    n_adds += 2u * (unsigned)__popc(__ballot_sync(0xffffffffu, add));
  }
  for (int off = 16; off > 0; off >>= 1) {
    n_ok += __shfl_xor_sync(0xffffffffu, n_ok, off);
    n_fail += __shfl_xor_sync(0xffffffffu, n_fail, off);
    n_segs += __shfl_xor_sync(0xffffffffu, n_segs, off);
  }
  if (lane == 0) {
    if (n_adds) atomicAdd(P.ctr + 13, (unsigned long long)n_adds);
    if (n_segs) atomicAdd(P.ctr + 9, (unsigned long long)n_segs);
    if (n_ok) atomicAdd(P.ctr + 3, (unsigned long long)n_ok);
    if (n_fail) atomicAdd(P.ctr + 4, (unsigned long long)n_fail);
  }
}

// Stage 2 for rounds whose items hold one path each (kpi == 1, where the
// per-lane sums above have nothing to add up): one thread per backward ray,
// rays of all tasks laid out back to back (task-major, then Rx within the
// cell, then Tx), so no warp idles on the padding of a task's last item.
// Each verified ray adds its contribution to the Rx-major accumulator.
template <bool EXPORT>
__global__ void __launch_bounds__(256, 5) k_stage2_rays(TraceDev P) {
  const int S = P.n_src;
  const long long pairs = (long long)P.gs * P.gs * S;
  const long long n_rays = (long long)P.cell_off[P.ng] * pairs;
  const long long ray = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  if (blockIdx.x == 0 && threadIdx.x == 0 && n_rays > (long long)gridDim.x * blockDim.x)
    atomicOr(P.err, AMS_DERR_TASKS);  // the launch must cover every ray
  if (ray - lane >= n_rays) return;   // the whole warp is past the last ray
  bool valid = ray < n_rays;
  const long long t = valid ? ray / pairs : -1;
  int cell = 0, path = 0, slot = 0, inner = 0, s = 0;
  if (valid) {
    const int4 chunk = __ldg(P.chunk_at + t);
    const int2 task = __ldg(P.task_path + t);
    cell = chunk.x;
    path = task.x;
    slot = task.y;
    const long long pr = ray % pairs;
    inner = (int)(pr / S);
    s = (int)(pr % S);
    if ((unsigned)cell >= (unsigned)P.ng || (unsigned)path >= (unsigned)P.n_paths ||
        (unsigned)slot > P.tab_mask || (unsigned long long)t >= P.task_cap) {
      atomicOr(P.err, AMS_DERR_TASKS);
      valid = false;
    }
  }
  bool ok = false, traced = false;
  unsigned segs = 0;
  ams_ray_record rr;
  if (EXPORT) {
    rr.src = s; rr.dst = -1; rr.path = path; rr.traced = 0; rr.successful = 0; rr.hit_cnt = 0;
    rr.launch_angle = 0.f; rr.receive_angle = 0.f; rr.loss = 0.f; rr.pad0 = 0.f;
    rr.phase = 0.0; rr.pad1 = 0;
#pragma unroll
    for (int i = 0; i < 5; i++) rr.hit_loss_idx[i] = -1;
  }
  if (valid) {
    const int gi = cell / P.n1g, gj = cell % P.n1g;
    const int di = inner / P.gs + gi * P.gs, dj = inner % P.gs + gj * P.gs;
    const int dst = di * P.n1_dst + dj;
    if (EXPORT) rr.dst = dst;
    if (!(dst >= P.n_dst || (P.strict_grid && (di >= P.n0_dst || dj >= P.n1_dst)))) {
      traced = true;
      unsigned long long cre = 0, cim = 0;
      const af3 srcdir = mk3(P.src_dir[0], P.src_dir[1], P.src_dir[2]);
      const af3 dstdir = mk3(P.dst_dir[0], P.dst_dir[1], P.dst_dir[2]);
      ok = s2_ray<EXPORT>(P, slot, s, ld3(P.dst + 3 * dst), srcdir, dstdir, segs, cre, cim, &rr);
      if (ok) {
        unsigned long long *acc = P.acc + ((size_t)dst * S + s) * 2;
        atomicAdd(acc, cre);
        atomicAdd(acc + 1, cim);
      }
    }
  }
  if (EXPORT && valid) {
    rr.traced = traced ? 1 : 0;
    rr.successful = ok ? 1 : 0;
    const unsigned long long at = P.rec_base + (unsigned long long)ray;
    if (at < P.rec_cap) P.rec[at] = rr;
  }
  // counters and each task's success bit, one atomic per warp / task
  const unsigned okb = __ballot_sync(0xffffffffu, ok);
  const unsigned trb = __ballot_sync(0xffffffffu, traced);
  for (int off = 16; off > 0; off >>= 1) segs += __shfl_xor_sync(0xffffffffu, segs, off);
  if (lane == 0) {
    if (segs) atomicAdd(P.ctr + 9, (unsigned long long)segs);
    if (okb) {
      atomicAdd(P.ctr + 3, (unsigned long long)__popc(okb));
      atomicAdd(P.ctr + 13, 2ull * (unsigned long long)__popc(okb));  // two adds per ray
    }
    if (trb & ~okb) atomicAdd(P.ctr + 4, (unsigned long long)__popc(trb & ~okb));
  }
  const unsigned same = __match_any_sync(0xffffffffu, t);
  if (valid && (okb & same) && lane == __ffs(same) - 1)
    atomicOr(P.S + (size_t)cell * P.W + (path >> 5), 1u << (path & 31));
}

// N = (S of the 4 neighbour cells) & ~T; T |= N; S = 0 (cpp:257-300).  The
// neighbours are linear cell indices +-1 and +-n1g with only the [0, ng)
// check, exactly as the reference (so row ends wrap).
__global__ void k_expand(TraceDev P) {
  const long long nwords = (long long)P.ng * P.W;
  const long long stride = (long long)gridDim.x * blockDim.x;
  unsigned long long cnt = 0;
  for (long long wi = (long long)blockIdx.x * blockDim.x + threadIdx.x; wi < nwords; wi += stride) {
    const int cell = (int)(wi / P.W);
    const int w = (int)(wi % P.W);
    unsigned s = 0;
    const int nb[4] = {cell - 1, cell + 1, cell - P.n1g, cell + P.n1g};
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (nb[k] >= 0 && nb[k] < P.ng) s |= P.S[(size_t)nb[k] * P.W + w];
    unsigned t = P.T[wi];
    unsigned n = s & ~t;
    P.N[wi] = n;
    if (n) {
      P.T[wi] = t | n;
      atomicAdd(P.cell_cnt + cell, __popc(n));
    }
    cnt += __popc(n);
  }
  for (int off = 16; off > 0; off >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(P.ctr + 7, cnt);
}

__global__ void k_popcount(const unsigned *bits, long long n, unsigned long long *out) {
  unsigned long long c = 0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    c += __popc(bits[i]);
  for (int off = 16; off > 0; off >>= 1) c += __shfl_xor_sync(0xffffffffu, c, off);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// result[s][dst] += acc[dst][s] * 2^-56 (re, im): 32 x 32 tiles turned
// through shared memory, reads coalesced over s and writes over dst.
// Block (32, 8), grid (ceil(n_dst / 32), ceil(n_src / 32)).
__global__ void k_finalize(const unsigned long long *acc, float *result, int n_src, int n_dst) {
  __shared__ float2 tl[32][33];
  const int d0 = blockIdx.x * 32, s0 = blockIdx.y * 32;
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int d = d0 + i, s = s0 + threadIdx.x;
    float2 v = make_float2(0.f, 0.f);
    if (d < n_dst && s < n_src) {
      const unsigned long long *a = acc + ((size_t)d * n_src + s) * 2;
      v = make_float2((float)((double)(long long)a[0] * AMS_ACC_INV),
                      (float)((double)(long long)a[1] * AMS_ACC_INV));
    }
    tl[i][threadIdx.x] = v;
  }
  __syncthreads();
  for (int i = threadIdx.y; i < 32; i += blockDim.y) {
    const int s = s0 + i, d = d0 + threadIdx.x;
    if (s >= n_src || d >= n_dst) continue;
    const float2 v = tl[threadIdx.x][i];
    if (v.x != 0.f || v.y != 0.f) {
      float2 *r = reinterpret_cast<float2 *>(result) + (size_t)s * n_dst + d;
      float2 x = *r;
      x.x += v.x;
      x.y += v.y;
      *r = x;
    }
  }
}

__global__ void k_export(TraceDev P, int32_t *out, unsigned long long *n_out) {
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s <= P.tab_mask;
       s += gridDim.x * blockDim.x) {
    if (P.tab_h[s] == 0ull) continue;
    unsigned long long k = atomicAdd(n_out, 1ull);
    for (int i = 0; i < 14; i++)
      out[k * 14 + i] = (int32_t)((uint32_t)P.tab_key[(size_t)s * 14 + i] ^ AMS_KEY_FLIP);
  }
}

int grid_for(long long n, int block) {
  long long b = (n + block - 1) / block;
  const long long cap = (long long)ams_device_sms() * 16;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (int)b;
}

}  // namespace

cudaError_t trace_stage1(const TraceDev &P, cudaStream_t st) {
  // persistent: as many CTAs as are resident at once (lanes fetch launch
  // indices from ctr[10], zeroed with the other counters)
  long long n = (long long)P.launch_x * P.launch_y;
  // the smallest slot array that holds max_reflection's slots
  const int lk = P.L <= 2 ? 0 : (P.L == 3 ? 1 : 2);
  void (*const kern[3])(TraceDev) = {k_stage1<2>, k_stage1<3>, k_stage1<AMS_MAX_L>};
  static int per_sm[3][AMS_MAX_DEVICES] = {{0}};
  const int dev = ams_current_device();
  if (dev < 0) return cudaErrorInvalidDevice;
  if (per_sm[lk][dev] == 0) {
    int b = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern[lk], 128, 0);
    if (e != cudaSuccess) return e;
    per_sm[lk][dev] = b > 0 ? b : 1;
  }
  long long blocks = (long long)per_sm[lk][dev] * ams_device_sms();
  const long long need = (n + 127) / 128;
  if (blocks > need) blocks = need;
  if (blocks < 1) blocks = 1;
  kern[lk]<<<(int)blocks, 128, 0, st>>>(P);
  return cudaGetLastError();
}

namespace {
int stage2_per_sm() {
  static int per_sm[AMS_MAX_DEVICES] = {0};
  const int dev = ams_current_device();
  if (dev < 0) return 1;
  if (per_sm[dev] == 0) {
    int b = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_stage2, 256, 0) != cudaSuccess) b = 1;
    per_sm[dev] = b > 0 ? b : 1;
  }
  return per_sm[dev];
}
}  // namespace

int trace_paths_per_item(const TraceDev &P, unsigned long long n_tasks) {
  // several paths per item (fewer atomic adds) only when a round still has
  // about 32 items per resident warp with them: long items at the end of a
  // smaller round leave the GPU idle (coverage-128's first round: 9 paths
  // per item, 1.94 ms, against about 1.6 ms one thread per ray)
  const unsigned long long warps = (unsigned long long)stage2_per_sm() * ams_device_sms() * 8;
  const unsigned long long pairs = (unsigned long long)(P.gs * P.gs) * P.n_src;
  const unsigned long long work = n_tasks * ((pairs + 31) / 32);
  unsigned long long k = work / (32 * warps);
  if (k < 1) k = 1;
  if (k > 16) k = 16;
  return (int)k;
}

cudaError_t trace_dense_paths(const TraceDev &P, const unsigned *T_slots, int w_slots,
                              int *dense_of, unsigned *out, cudaStream_t st) {
  k_dense_ids<<<grid_for((long long)P.tab_mask + 1, 256), 256, 0, st>>>(P, dense_of, P.ctr + 12);
  k_to_dense<<<grid_for((long long)P.ng * w_slots, 256), 256, 0, st>>>(P, T_slots, w_slots,
                                                                      dense_of, out);
  return cudaGetLastError();
}

cudaError_t trace_count_tasks(const TraceDev &P, const unsigned *bits, cudaStream_t st) {
  k_cell_counts<<<grid_for((long long)P.ng * 32, 256), 256, 0, st>>>(P, bits);
  return cudaGetLastError();
}

cudaError_t trace_make_tasks(const TraceDev &P, const unsigned *bits, cudaStream_t st) {
  const long long threads = (long long)P.ng * 32;
  k_cell_scan<<<1, 1024, 0, st>>>(P);
  k_cell_fill<<<grid_for(threads, 256), 256, 0, st>>>(P, bits);
  return cudaGetLastError();
}

cudaError_t trace_stage2(const TraceDev &P, unsigned long long n_tasks, cudaStream_t st) {
  if (n_tasks == 0) return cudaSuccess;
  // one warp per item; the chunks number at most n_tasks / kpi + one per
  // cell (the exact count is on the device, warps beyond it return)
  const unsigned long long pairs = (unsigned long long)(P.gs * P.gs) * P.n_src;
  const unsigned long long k = (unsigned long long)P.kpi;
  unsigned long long chunks = (n_tasks + k - 1) / k + (unsigned long long)P.ng;
  if (chunks > n_tasks) chunks = n_tasks;
  if (P.kpi == 1) {  // one path per item: one thread per ray
    const unsigned long long blocks = (n_tasks * pairs + 255) / 256;
    if (blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
    k_stage2_rays<false><<<(unsigned)blocks, 256, 0, st>>>(P);
    return cudaGetLastError();
  }
  const unsigned long long items_max = chunks * ((pairs + 31) / 32);
  const unsigned long long blocks = (items_max + 7) / 8;
  if (blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
  k_stage2<<<(unsigned)blocks, 256, 0, st>>>(P);
  return cudaGetLastError();
}

cudaError_t trace_stage2_export(const TraceDev &P, unsigned long long n_tasks, cudaStream_t st) {
  if (n_tasks == 0) return cudaSuccess;
  if (P.kpi != 1) return cudaErrorInvalidValue;
  const unsigned long long pairs = (unsigned long long)(P.gs * P.gs) * P.n_src;
  const unsigned long long blocks = (n_tasks * pairs + 255) / 256;
  if (blocks > 0x7fffffffull) return cudaErrorInvalidConfiguration;
  k_stage2_rays<true><<<(unsigned)blocks, 256, 0, st>>>(P);
  return cudaGetLastError();
}

cudaError_t trace_expand(const TraceDev &P, cudaStream_t st) {
  long long n = (long long)P.ng * P.W;
  k_expand<<<grid_for(n, 256), 256, 0, st>>>(P);
  return cudaGetLastError();
}

cudaError_t trace_count_bits(const TraceDev &P, const unsigned *bits, unsigned long long *out,
                             cudaStream_t st) {
  long long n = (long long)P.ng * P.W;
  k_popcount<<<grid_for(n, 256), 256, 0, st>>>(bits, n, out);
  return cudaGetLastError();
}

cudaError_t trace_finalize(const TraceDev &P, float *result, cudaStream_t st) {
  dim3 grid((P.n_dst + 31) / 32, (P.n_src + 31) / 32), block(32, 8);
  k_finalize<<<grid, block, 0, st>>>(P.acc, result, P.n_src, P.n_dst);
  return cudaGetLastError();
}

cudaError_t trace_export_paths(const TraceDev &P, int32_t *out, unsigned long long *n_out,
                               cudaStream_t st) {
  k_export<<<grid_for((long long)P.tab_mask + 1, 256), 256, 0, st>>>(P, out, n_out);
  return cudaGetLastError();
}
