/*
 * ams_oracle.c -- CPU restatement of the AutoMS channel simulator.
 *
 * TEST INFRASTRUCTURE ONLY (see ams_oracle.h).  Compile with
 * -ffp-contract=off so that float expressions round exactly as written.
 */
#include "ams_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_PIF 3.14159265358979323846f /* M_PIf of sutil/vec_math.h:44 */
#define ORC_TMIN 1e-5f                  /* optixPathTracer.cu:98 */
#define ORC_TMAX 1e16f
#define ORC_NBINS 19 /* 19 angle bins per material, go.py:690-698 */
#define ORC_MAX_SLOTS 32

typedef struct { float x, y, z; } f3;

static inline f3 mk(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static inline f3 add(f3 a, f3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline f3 sub(f3 a, f3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline f3 scl(f3 a, float s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline f3 neg(f3 a) { return mk(-a.x, -a.y, -a.z); }
/* sutil vec_math.h:527-549: dot, cross, length, normalize */
static inline float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline f3 cross3(f3 a, f3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline float len3(f3 v) { return sqrtf(dot3(v, v)); }
static inline f3 nrm3(f3 v) { float inv = 1.0f / sqrtf(dot3(v, v)); return scl(v, inv); }
/* vec_math.h:567-570 */
static inline f3 faceforward3(f3 n, f3 i, f3 nref) { return scl(n, copysignf(1.0f, dot3(i, nref))); }
static inline f3 ld3(const float *p) { return mk(p[0], p[1], p[2]); }
static inline float comp(f3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

/* ------------------------------------------------------------------ RNG */
/* TEA with 4 rounds (Zafar, Olano, Curtis 2010), random.h:31-46 */
uint32_t orc_tea4(uint32_t v0, uint32_t v1) {
  uint32_t s0 = 0;
  for (int n = 0; n < 4; n++) {
    s0 += 0x9e3779b9u;
    v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
    v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
  }
  return v0;
}
/* Numerical Recipes LCG, 24 low bits, random.h:49-61 */
float orc_rnd(uint32_t *seed) {
  *seed = 1664525u * (*seed) + 1013904223u;
  return (float)(*seed & 0x00FFFFFFu) / (float)0x01000000;
}

/* sin/cos of a float angle in [0, 7): Cody-Waite reduction by pi/2 (two-part
 * constant) and Taylor series to degree 17/18, evaluated in double and
 * rounded once to float.  The CUDA kernels evaluate the same expression. */
static void orc_sincos_f(float a, float *s_out, float *c_out) {
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
  *s_out = (float)so;
  *c_out = (float)co;
}

void orc_sincos(float a, float out[2]) { orc_sincos_f(a, &out[0], &out[1]); }

/* rand_dir, optixPathTracer.cu:56-68 */
static f3 rand_dir(uint32_t *seed, uint32_t ix, uint32_t iy, int lx, int ly) {
  float rnd1 = (orc_rnd(seed) + (float)ix) / (float)lx;
  float rnd2 = (orc_rnd(seed) + (float)iy) / (float)ly;
  float theta = (2.0f * ORC_PIF) * rnd1;
  float r = sqrtf(rnd2);
  float sn, cs;
  orc_sincos_f(theta, &sn, &cs);
  float u = r * cs, v = r * sn;
  float q = sqrtf(1.0f - r * r);
  return mk((2.0f * u) * q, (2.0f * v) * q, 1.0f - (2.0f * r) * r);
}
void orc_rand_dir(uint32_t *seed, uint32_t ix, uint32_t iy, int lx, int ly, float out[3]) {
  f3 d = rand_dir(seed, ix, iy, lx, ly);
  out[0] = d.x; out[1] = d.y; out[2] = d.z;
}

/* ------------------------------------------------- angle bin and beams */
/* theta_id = int((acos|c| / (pi/2) * 36 + 1) / 2), optixPathTracer.cu:304-306,
 * restated as a count of 5-degree bin edges: id >= k iff
 * |c| <= cos((2k-1) pi / 72).  The thresholds are the largest floats not
 * above those cosines, so the comparison is exact in float. */
static float g_theta_thr[18];
static int g_theta_init = 0;
static void theta_init(void) {
  if (g_theta_init) return;
  for (int k = 1; k <= 18; k++) {
    double c = cos((2.0 * k - 1.0) * 3.14159265358979323846 / 72.0);
    float f = (float)c;
    if ((double)f > c) f = nextafterf(f, -1.0f);
    g_theta_thr[k - 1] = f;
  }
  g_theta_init = 1;
}
int orc_theta_id(float cos_theta) {
  theta_init();
  float a = fabsf(cos_theta);
  int id = 0;
  for (int k = 0; k < 18; k++) id += (a <= g_theta_thr[k]) ? 1 : 0;
  return id;
}

/* get_beampattern_factor, optixPathTracer.cu:107-136.  Branches are taken on
 * the float cosine against the cosines of 120 and 75 degrees; the taper value
 * is evaluated in double. */
static float beampattern(f3 d1, f3 d2, int type) {
  float c = dot3(d1, d2) / (len3(d1) * len3(d2));
  switch (type) {
  case 0: return 1.0f;
  case 1: return c < 0.0f ? 0.0f : c * 2.4495f;
  case 2: {
    if ((double)c < -0.5) return 0.1f;
    if ((double)c < 0.25881904510252074) {
      double th = acos((double)c);
      double e = (2.0 * 3.14159265358979323846 / 3.0 - th) / 3.14159265358979323846 * 4.0 *
                     0.4129962305693391 - 1.0;
      return (float)(pow(10.0, e) * 2.4495);
    }
    return (float)((double)c * 2.4495);
  }
  case 3: return c < 0.0f ? 0.0f : 1.4142f;
  default: return 0.0f;
  }
}
float orc_beampattern(const float a[3], const float b[3], int type) {
  return beampattern(ld3(a), ld3(b), type);
}

/* ------------------------------------------------------- ray primitives */
typedef struct {
  f3 o, d, inv;
  int kx, ky, kz;
  float Sx, Sy, Sz;
} ray_t;

static void ray_setup(ray_t *r, f3 o, f3 d) {
  r->o = o; r->d = d;
  r->inv = mk(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
  float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  int kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
  int kx = kz + 1; if (kx == 3) kx = 0;
  int ky = kx + 1; if (ky == 3) ky = 0;
  if (comp(d, kz) < 0.0f) { int t = kx; kx = ky; ky = t; }
  r->kx = kx; r->ky = ky; r->kz = kz;
  float dz = comp(d, kz);
  r->Sx = comp(d, kx) / dz;
  r->Sy = comp(d, ky) / dz;
  r->Sz = 1.0f / dz;
}

/* Watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2(1) 2013),
 * no back-face culling.  Returns t or -1. */
static float tri_hit(const ray_t *r, f3 v0, f3 v1, f3 v2) {
  f3 A = sub(v0, r->o), B = sub(v1, r->o), C = sub(v2, r->o);
  float Az_ = comp(A, r->kz), Bz_ = comp(B, r->kz), Cz_ = comp(C, r->kz);
  float Ax = comp(A, r->kx) - r->Sx * Az_;
  float Ay = comp(A, r->ky) - r->Sy * Az_;
  float Bx = comp(B, r->kx) - r->Sx * Bz_;
  float By = comp(B, r->ky) - r->Sy * Bz_;
  float Cx = comp(C, r->kx) - r->Sx * Cz_;
  float Cy = comp(C, r->ky) - r->Sy * Cz_;
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
  float Az = r->Sz * Az_, Bz = r->Sz * Bz_, Cz = r->Sz * Cz_;
  float T = U * Az + V * Bz + W * Cz;
  return T / det;
}
float orc_intersect_tri(const float o[3], const float d[3], const float a[3],
                        const float b[3], const float c[3]) {
  ray_t r;
  ray_setup(&r, ld3(o), ld3(d));
  float t = tri_hit(&r, ld3(a), ld3(b), ld3(c));
  return (t > ORC_TMIN && t < ORC_TMAX) ? t : -1.0f;
}

/* Slab test against a primitive AABB over the whole ray interval.  This is
 * the gate in front of the sphere program (OptiX runs the intersection
 * program only for AABBs the ray enters). */
static int slab(const ray_t *r, const float *lo, const float *hi) {
  float tx0 = (lo[0] - r->o.x) * r->inv.x, tx1 = (hi[0] - r->o.x) * r->inv.x;
  float ty0 = (lo[1] - r->o.y) * r->inv.y, ty1 = (hi[1] - r->o.y) * r->inv.y;
  float tz0 = (lo[2] - r->o.z) * r->inv.z, tz1 = (hi[2] - r->o.z) * r->inv.z;
  float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
  float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
  return tn <= tf && tf >= ORC_TMIN && tn <= ORC_TMAX;
}

int orc_prim_slab(const float o[3], const float d[3], const float lo[3], const float hi[3]) {
  ray_t r;
  ray_setup(&r, ld3(o), ld3(d));
  return slab(&r, lo, hi);
}

/* __intersection__sphere, optixPathTracer.cu:419-445.  Returns t = b or -1. */
static float sphere_hit(const ray_t *r, f3 center, float radius) {
  f3 O = sub(center, r->o);
  /* ray_dir / length(ray_dir) is ray_dir * (1 / length), vec_math.h:483-487 */
  f3 D = scl(r->d, 1.0f / len3(r->d));
  float b = dot3(O, D);
  float c = dot3(O, O);
  float acc = fmaxf(5e-5f, radius * radius);
  if ((c - b * b < acc) && b > 0.0f && sqrtf(c) > radius) {
    if (b > ORC_TMIN && b < ORC_TMAX) return b;
  }
  return -1.0f;
}

/* ------------------------------------------------------------------ BVH */
typedef struct {
  float lo[3], hi[3];
  int left, right; /* right < 0: leaf with prims [left, left - right - 1) */
} bvh_node;

typedef struct {
  bvh_node *nodes;
  int *prims;
  int n_nodes;
} bvh_t;

typedef struct { float lo[3], hi[3], c[3]; } pbox;

static float widen_lo(float v) { return nextafterf(v - (1e-6f + 1e-6f * fabsf(v)), -FLT_MAX); }
static float widen_hi(float v) { return nextafterf(v + (1e-6f + 1e-6f * fabsf(v)), FLT_MAX); }

static pbox *g_sort_boxes;
static int g_sort_axis;
static int cmp_centroid(const void *a, const void *b) {
  float ca = g_sort_boxes[*(const int *)a].c[g_sort_axis];
  float cb = g_sort_boxes[*(const int *)b].c[g_sort_axis];
  if (ca < cb) return -1;
  if (ca > cb) return 1;
  return (*(const int *)a) - (*(const int *)b);
}

static int bvh_build_rec(bvh_t *bv, pbox *boxes, int *idx, int n, int offset) {
  int me = bv->n_nodes++;
  bvh_node *nd = &bv->nodes[me];
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  float clo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, chi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int i = 0; i < n; i++) {
    pbox *b = &boxes[idx[i]];
    for (int k = 0; k < 3; k++) {
      lo[k] = fminf(lo[k], b->lo[k]); hi[k] = fmaxf(hi[k], b->hi[k]);
      clo[k] = fminf(clo[k], b->c[k]); chi[k] = fmaxf(chi[k], b->c[k]);
    }
  }
  for (int k = 0; k < 3; k++) { nd->lo[k] = widen_lo(lo[k]); nd->hi[k] = widen_hi(hi[k]); }
  if (n <= 4) {
    nd->left = offset; nd->right = -(n + 1);
    return me;
  }
  int axis = 0;
  float ext = chi[0] - clo[0];
  if (chi[1] - clo[1] > ext) { axis = 1; ext = chi[1] - clo[1]; }
  if (chi[2] - clo[2] > ext) { axis = 2; }
  g_sort_boxes = boxes; g_sort_axis = axis;
  qsort(idx, (size_t)n, sizeof(int), cmp_centroid);
  int h = n / 2;
  int l = bvh_build_rec(bv, boxes, idx, h, offset);
  int r = bvh_build_rec(bv, boxes, idx + h, n - h, offset + h);
  bv->nodes[me].left = l;
  bv->nodes[me].right = r;
  return me;
}

static void bvh_build(bvh_t *bv, pbox *boxes, int n) {
  bv->nodes = (bvh_node *)malloc(sizeof(bvh_node) * (size_t)(2 * n + 1));
  bv->prims = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  bv->n_nodes = 0;
  for (int i = 0; i < n; i++) bv->prims[i] = i;
  if (n > 0) bvh_build_rec(bv, boxes, bv->prims, n, 0);
}
static void bvh_free(bvh_t *bv) { free(bv->nodes); free(bv->prims); }

/* conservative node test: the node boxes are widened and the far bound is
 * loosened so that no primitive whose t is <= best can be culled. */
static int node_hit(const ray_t *r, const bvh_node *n, float best) {
  float tx0 = (n->lo[0] - r->o.x) * r->inv.x, tx1 = (n->hi[0] - r->o.x) * r->inv.x;
  float ty0 = (n->lo[1] - r->o.y) * r->inv.y, ty1 = (n->hi[1] - r->o.y) * r->inv.y;
  float tz0 = (n->lo[2] - r->o.z) * r->inv.z, tz1 = (n->hi[2] - r->o.z) * r->inv.z;
  float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fminf(tz0, tz1));
  float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fmaxf(tz0, tz1));
  return tn <= tf * 1.00001f + 1e-6f && tf >= 0.0f && tn <= best * 1.0001f + 1e-4f;
}

/* ---------------------------------------------------------------- scene */
typedef struct {
  const float *tris; int n_tri;
  const int *mat; const float *mat_prop; int n_mat;
  const float *src; int n_src; const float *src_lo, *src_hi;
  const float *dst; int n_dst; const float *dst_lo, *dst_hi;
  float src_r, dst_r;
  bvh_t bvh[3];
} scene_t;

typedef struct { float t; int inst; int prim; } hit_t;

static inline int better(float t, int inst, int prim, const hit_t *h) {
  if (t < h->t) return 1;
  if (t > h->t) return 0;
  if (inst != h->inst) return inst < h->inst;
  return prim < h->prim;
}

static void trav(const scene_t *S, int inst, const ray_t *r, hit_t *best) {
  const bvh_t *bv = &S->bvh[inst];
  if (bv->n_nodes == 0) return;
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const bvh_node *n = &bv->nodes[stack[--sp]];
    if (!node_hit(r, n, best->t)) continue;
    if (n->right < 0) {
      int cnt = -n->right - 1;
      for (int i = 0; i < cnt; i++) {
        int p = bv->prims[n->left + i];
        float t;
        if (inst == 0) {
          const float *v = S->tris + (size_t)p * 9;
          t = tri_hit(r, ld3(v), ld3(v + 3), ld3(v + 6));
          if (!(t > ORC_TMIN && t < ORC_TMAX)) continue;
        } else if (inst == 1) {
          if (!slab(r, S->src_lo + 3 * p, S->src_hi + 3 * p)) continue;
          t = sphere_hit(r, ld3(S->src + 3 * p), S->src_r);
          if (t < 0.0f) continue;
        } else {
          if (!slab(r, S->dst_lo + 3 * p, S->dst_hi + 3 * p)) continue;
          t = sphere_hit(r, ld3(S->dst + 3 * p), S->dst_r);
          if (t < 0.0f) continue;
        }
        if (better(t, inst, p, best)) { best->t = t; best->inst = inst; best->prim = p; }
      }
    } else {
      stack[sp++] = n->right;
      stack[sp++] = n->left;
    }
  }
}

/* optixTrace with visibility mask: bit i selects instance i (cpp:417-424) */
static hit_t closest(const scene_t *S, f3 o, f3 d, int mask) {
  ray_t r;
  ray_setup(&r, o, d);
  hit_t h = {ORC_TMAX, 3, 0x7fffffff};
  for (int i = 0; i < 3; i++)
    if (mask & (1 << i)) trav(S, i, &r, &h);
  if (h.inst == 3) h.t = -1.0f;
  return h;
}

static void tri_verts(const scene_t *S, int p, f3 *v0, f3 *v1, f3 *v2) {
  const float *v = S->tris + (size_t)p * 9;
  *v0 = ld3(v); *v1 = ld3(v + 3); *v2 = ld3(v + 6);
}

/* ------------------------------------------------------- image transform */
typedef struct { float m[12]; } mat34;

static mat34 mat_identity(void) {
  mat34 r; memset(&r, 0, sizeof(r));
  r.m[0] = 1.0f; r.m[5] = 1.0f; r.m[10] = 1.0f;
  return r;
}
/* getImage, optixPathTracer.cu:78-81 with Matrix.h:448-462 */
static f3 image_of(const mat34 *M, f3 p) {
  const float *m = M->m;
  return mk(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3] * 1.0f,
            m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7] * 1.0f,
            m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11] * 1.0f);
}
/* updateImageTransform, optixPathTracer.cu:70-76: M <- (I - 2 N N^T) M,
 * t <- t + 2 (A.N) N, summed in the order of Matrix.h:339-356 */
static void image_update(mat34 *M, f3 N, f3 A) {
  float n[3] = {N.x, N.y, N.z};
  float a[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      float p = 0.0f;
      p += (2.0f * 0.0f) * 0.0f;
      p += (2.0f * n[i]) * n[j];
      a[i * 3 + j] = (i == j ? 1.0f : 0.0f) - p;
    }
  mat34 r;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 4; j++) {
      float s = 0.0f;
      for (int k = 0; k < 3; k++) s += a[i * 3 + k] * M->m[k * 4 + j];
      r.m[i * 4 + j] = s;
    }
  float k2 = 2.0f * dot3(A, N);
  r.m[3] = r.m[3] + k2 * N.x;
  r.m[7] = r.m[7] + k2 * N.y;
  r.m[11] = r.m[11] + k2 * N.z;
  *M = r;
}

/* ------------------------------------------------------------- records */
/* ForwardRecord, optixPathTracer.h:59-62: 12 floats + hit_cnt + is_reflect
 * + dst_grid_idx, compared as 15 int32 words (cpp:168-185). */
typedef struct { int32_t w[15]; } rec_t;

typedef struct { rec_t *v; size_t n, cap; } recvec;
static void rv_push(recvec *rv, const rec_t *r) {
  if (rv->n == rv->cap) {
    rv->cap = rv->cap ? rv->cap * 2 : 1024;
    rv->v = (rec_t *)realloc(rv->v, rv->cap * sizeof(rec_t));
  }
  rv->v[rv->n++] = *r;
}

static int32_t fbits(float f) {
  int32_t b;
  memcpy(&b, &f, 4);
  if (b == (int32_t)0x80000000) b = 0; /* -0 and +0 are one key */
  return b;
}

typedef struct {
  f3 o, d;
  mat34 M;
  int ttl;
  int live;
} slot_t;

/* stage 1 for one launch index (optixPathTracer.cu:142-190) */
static void forward_thread(const scene_t *S, const orc_params *p, int n1_dst,
                           int n1g, int ix, int iy, recvec *out, uint64_t *ovf) {
  uint32_t seed = orc_tea4((uint32_t)(ix * p->launch_y + iy), 0u);
  int res_cnt = 0;
  int cap = p->reserve_size;
  int *rc_cell = (int *)malloc(sizeof(int) * (size_t)(cap > 0 ? cap : 1));
  int *rc_hc = (int *)malloc(sizeof(int) * (size_t)(cap > 0 ? cap : 1));
  int L = p->max_reflection;
  int hit_cap = 0;
  for (int launch = 0; launch < p->samples_per_launch; launch++) {
    float rs = orc_rnd(&seed) * (float)S->n_src;
    uint32_t src = (uint32_t)rs;
    if (src >= (uint32_t)S->n_src) src = (uint32_t)S->n_src - 1;
    f3 spos = ld3(S->src + 3 * src);
    slot_t slots[ORC_MAX_SLOTS];
    for (int i = 0; i < ORC_MAX_SLOTS; i++) slots[i].live = 0;
    slots[0].o = spos;
    slots[0].d = rand_dir(&seed, (uint32_t)ix, (uint32_t)iy, p->launch_x, p->launch_y);
    slots[0].M = mat_identity();
    slots[0].ttl = L + 1;
    slots[0].live = 1;
    for (int i = 0; i < ORC_MAX_SLOTS; i++) {
      if (!slots[i].live) continue;
      slot_t *s = &slots[i];
      while (s->ttl > 0) {
        hit_t h = closest(S, s->o, s->d, 5);
        if (h.inst == 3) { s->ttl = 0; break; }
        f3 dir = s->d;
        s->o = add(s->o, scl(dir, h.t));
        if (h.inst == 0 && s->ttl > 1) {
          f3 v0, v1, v2;
          tri_verts(S, h.prim, &v0, &v1, &v2);
          f3 N0 = nrm3(cross3(sub(v1, v0), sub(v2, v0)));
          f3 N = faceforward3(N0, neg(dir), N0);
          int m = S->mat[h.prim];
          float ct = dot3(dir, N) / (len3(N) * len3(dir));
          int tid = orc_theta_id(ct);
          int pen = S->mat_prop[tid + m * ORC_NBINS] < 0.0f;
          s->ttl--;
          int hc = L + 1 - s->ttl;
          int j = i | (1 << (hc - 1));
          slot_t *c = &slots[j];
          c->live = 1;
          c->ttl = s->ttl;
          c->o = s->o;
          c->d = sub(dir, scl(N, 2.0f * dot3(dir, N)));
          c->M = s->M;
          f3 V = sub(v0, image_of(&c->M, spos));
          f3 Nimg = faceforward3(N0, V, N0);
          image_update(&c->M, Nimg, v0);
          if (!pen) s->ttl = 0;
        } else if (h.inst == 2) {
          if (res_cnt < cap) {
            int d0 = h.prim / n1_dst, d1 = h.prim % n1_dst;
            int cell = (d0 / p->dst_gridsize) * n1g + d1 / p->dst_gridsize;
            int hc = L + 1 - s->ttl;
            int mhc = 0;
            for (int k = res_cnt - 1; k >= 0; k--)
              if (rc_cell[k] == cell) { mhc = rc_hc[k] + 1; break; }
            if (mhc <= hc) {
              rc_cell[res_cnt] = cell; rc_hc[res_cnt] = hc;
              rec_t r;
              for (int k = 0; k < 12; k++) r.w[k] = fbits(s->M.m[k]);
              r.w[12] = hc; r.w[13] = i; r.w[14] = cell;
              rv_push(out, &r);
              res_cnt++;
            }
          } else {
            hit_cap = 1;
          }
        }
      }
    }
  }
  if (hit_cap) *ovf += 1;
  free(rc_cell);
  free(rc_hc);
}

/* backward verification of one (path, src, dst), optixPathTracer.cu:223-271
 * and :332-417.  Returns 1 on success with the complex contribution. */
static int backward_ray(const scene_t *S, const orc_params *p, const mat34 *M,
                        int hc, int mask, int src, int dst, double *re, double *im,
                        int *farfield) {
  f3 o = ld3(S->dst + 3 * dst);
  f3 dir = nrm3(sub(image_of(M, ld3(S->src + 3 * src)), o));
  f3 dstdir = ld3(p->dst_dir), srcdir = ld3(p->src_dir);
  float amp = beampattern(dir, dstdir, p->dst_bptype);
  float lam = (float)p->wave_len;
  float far = 1e6f, dd = 0.0f, dres = 0.0f;
  double D = 0.0;
  int ttl = hc + 1;
  int ok = 0;
  while (ttl > 0) {
    hit_t h = closest(S, o, dir, 3);
    if (h.inst == 3) break;
    float t = h.t;
    o = add(o, scl(dir, t));
    dd += t;
    D += (double)t;
    if (h.inst == 0) {
      if (ttl == 1) { ttl = 0; break; }
      f3 v0, v1, v2;
      tri_verts(S, h.prim, &v0, &v1, &v2);
      f3 N0 = nrm3(cross3(sub(v1, v0), sub(v2, v0)));
      f3 N = faceforward3(N0, neg(dir), N0);
      int m = S->mat[h.prim];
      float ct = dot3(dir, N) / (len3(N) * len3(dir));
      int tid = orc_theta_id(ct);
      float loss = fabsf(S->mat_prop[tid + m * ORC_NBINS]);
      ttl--;
      int hcb = hc + 1 - ttl;
      int is_ref = (mask >> (hcb - 1)) & 1;
      float max_d = fmaxf(fmaxf(len3(sub(v0, v1)), len3(sub(v1, v2))), len3(sub(v2, v0)));
      float fspl = 1.0f;
      if (dd > far) {
        fspl = lam / ((4.0f * ORC_PIF) * dres);
        dres = 0.0f;
        *farfield = 1;
      }
      amp *= loss * fspl;
      dres += dd;
      float fd = (float)(2.0 * (double)max_d * (double)max_d / (double)lam);
      far = (dd > fd) ? fd : 1e6f;
      dd = 0.0f;
      if (is_ref) dir = sub(dir, scl(N, 2.0f * dot3(dir, N)));
    } else if (h.inst == 1 && h.prim == src) {
      if (ttl == 1) {
        float bp = beampattern(neg(dir), srcdir, p->src_bptype);
        float af = lam / ((4.0f * ORC_PIF) * (dres + dd));
        amp *= bp * af;
        ok = 1;
      }
      ttl = 0;
    }
  }
  if (!ok) return 0;
  double ph = 6.283185307179586 * D / p->wave_len;
  ph = ph - 6.283185307179586 * floor(ph / 6.283185307179586);
  *re = (double)amp * cos(ph);
  *im = -(double)amp * sin(ph);
  return 1;
}

/* ------------------------------------------------------------ dedup */
static int cmp_rec(const void *a, const void *b) {
  const int32_t *x = ((const rec_t *)a)->w, *y = ((const rec_t *)b)->w;
  for (int k = 0; k < 15; k++) {
    if (x[k] < y[k]) return -1;
    if (x[k] > y[k]) return 1;
  }
  return 0;
}
static float wf(int32_t b) { float f; memcpy(&f, &b, 4); return f; }
/* Path ordering of optixPathTracer.h:28-38 and Matrix.h:764-776 */
static int cmp_path(const void *a, const void *b) {
  const int32_t *x = (const int32_t *)a, *y = (const int32_t *)b;
  if (x[12] != y[12]) return x[12] < y[12] ? -1 : 1;
  if (x[13] != y[13]) return x[13] < y[13] ? -1 : 1;
  for (int k = 0; k < 12; k++) {
    float fx = wf(x[k]), fy = wf(y[k]);
    if (fx < fy) return -1;
    if (fx > fy) return 1;
  }
  return 0;
}

typedef struct { int cell, pid; } task_t;

int orc_trace_channel(const float *tris, int n_tri, const int *mat,
                      const float *mat_prop, int n_mat, const float *src,
                      int n_src, const float *dst, int n0_dst, int n1_dst,
                      const float *src_aabb, const float *dst_aabb,
                      const orc_params *p, float *result, orc_stats *st,
                      int32_t *paths_out, int max_paths, int nthreads) {
  if (!p || !result || !st || n_src <= 0 || n0_dst <= 0 || n1_dst <= 0) return 1;
  if (p->max_reflection < 0 || p->max_reflection > 5) return 2;
  if (p->dst_gridsize <= 0 || p->launch_x <= 0 || p->launch_y <= 0) return 3;
  memset(st, 0, sizeof(*st));
  theta_init();
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
  int n_dst = n0_dst * n1_dst;
  scene_t S;
  memset(&S, 0, sizeof(S));
  S.tris = tris; S.n_tri = n_tri; S.mat = mat; S.mat_prop = mat_prop; S.n_mat = n_mat;
  S.src = src; S.n_src = n_src; S.dst = dst; S.n_dst = n_dst;
  S.src_r = p->src_r; S.dst_r = p->dst_r;
  float *slo = (float *)malloc(sizeof(float) * 3 * (size_t)n_src);
  float *shi = (float *)malloc(sizeof(float) * 3 * (size_t)n_src);
  float *dlo = (float *)malloc(sizeof(float) * 3 * (size_t)n_dst);
  float *dhi = (float *)malloc(sizeof(float) * 3 * (size_t)n_dst);
  /* AABB buffers: cat([pos - r, pos + r], -1), go.py:669-670 */
  for (int i = 0; i < n_src; i++)
    for (int k = 0; k < 3; k++) {
      slo[3 * i + k] = src_aabb ? src_aabb[6 * i + k] : src[3 * i + k] - p->src_r;
      shi[3 * i + k] = src_aabb ? src_aabb[6 * i + 3 + k] : src[3 * i + k] + p->src_r;
    }
  for (int i = 0; i < n_dst; i++)
    for (int k = 0; k < 3; k++) {
      dlo[3 * i + k] = dst_aabb ? dst_aabb[6 * i + k] : dst[3 * i + k] - p->dst_r;
      dhi[3 * i + k] = dst_aabb ? dst_aabb[6 * i + 3 + k] : dst[3 * i + k] + p->dst_r;
    }
  S.src_lo = slo; S.src_hi = shi; S.dst_lo = dlo; S.dst_hi = dhi;
  {
    pbox *b = (pbox *)malloc(sizeof(pbox) * (size_t)(n_tri > 0 ? n_tri : 1));
    for (int i = 0; i < n_tri; i++) {
      const float *v = tris + (size_t)i * 9;
      for (int k = 0; k < 3; k++) {
        b[i].lo[k] = fminf(fminf(v[k], v[3 + k]), v[6 + k]);
        b[i].hi[k] = fmaxf(fmaxf(v[k], v[3 + k]), v[6 + k]);
        b[i].c[k] = 0.5f * (b[i].lo[k] + b[i].hi[k]);
      }
    }
    bvh_build(&S.bvh[0], b, n_tri);
    free(b);
    b = (pbox *)malloc(sizeof(pbox) * (size_t)n_src);
    for (int i = 0; i < n_src; i++)
      for (int k = 0; k < 3; k++) {
        b[i].lo[k] = slo[3 * i + k]; b[i].hi[k] = shi[3 * i + k]; b[i].c[k] = src[3 * i + k];
      }
    bvh_build(&S.bvh[1], b, n_src);
    free(b);
    b = (pbox *)malloc(sizeof(pbox) * (size_t)n_dst);
    for (int i = 0; i < n_dst; i++)
      for (int k = 0; k < 3; k++) {
        b[i].lo[k] = dlo[3 * i + k]; b[i].hi[k] = dhi[3 * i + k]; b[i].c[k] = dst[3 * i + k];
      }
    bvh_build(&S.bvh[2], b, n_dst);
    free(b);
  }
  int gs = p->dst_gridsize;
  int n0g = (n0_dst - 1) / gs + 1, n1g = (n1_dst - 1) / gs + 1, ng = n0g * n1g;

  /* ---- stage 1 */
  int nthr = 1;
#ifdef _OPENMP
  nthr = omp_get_max_threads();
#endif
  recvec *rvs = (recvec *)calloc((size_t)nthr, sizeof(recvec));
  uint64_t *ovf = (uint64_t *)calloc((size_t)nthr, sizeof(uint64_t));
  long n_launch = (long)p->launch_x * p->launch_y;
#pragma omp parallel for schedule(dynamic, 64)
  for (long li = 0; li < n_launch; li++) {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    forward_thread(&S, p, n1_dst, n1g, (int)(li / p->launch_y), (int)(li % p->launch_y),
                   &rvs[tid], &ovf[tid]);
  }
  size_t n_rec = 0;
  for (int t = 0; t < nthr; t++) { n_rec += rvs[t].n; st->overflow += ovf[t]; }
  rec_t *recs = (rec_t *)malloc(sizeof(rec_t) * (n_rec ? n_rec : 1));
  {
    size_t o = 0;
    for (int t = 0; t < nthr; t++) {
      if (rvs[t].n) memcpy(recs + o, rvs[t].v, rvs[t].n * sizeof(rec_t));
      o += rvs[t].n;
      free(rvs[t].v);
    }
  }
  free(rvs); free(ovf);
  st->fwd_records = n_rec;
  int status = 0;
  if (n_rec == 0) goto done; /* "No path found!" (cpp:148-151) */

  /* ---- dedup: unique records, then the ordered path list */
  qsort(recs, n_rec, sizeof(rec_t), cmp_rec);
  size_t nu = 0;
  for (size_t i = 0; i < n_rec; i++)
    if (nu == 0 || cmp_rec(&recs[nu - 1], &recs[i]) != 0) recs[nu++] = recs[i];
  st->unique_records = nu;
  int32_t *paths = (int32_t *)malloc(sizeof(int32_t) * 14 * nu);
  for (size_t i = 0; i < nu; i++) memcpy(paths + 14 * i, recs[i].w, 14 * sizeof(int32_t));
  qsort(paths, nu, 14 * sizeof(int32_t), cmp_path);
  size_t np = 0;
  for (size_t i = 0; i < nu; i++)
    if (np == 0 || cmp_path(paths + 14 * (np - 1), paths + 14 * i) != 0) {
      memmove(paths + 14 * np, paths + 14 * i, 14 * sizeof(int32_t));
      np++;
    }
  st->unique_paths = np;
  if (paths_out) {
    size_t k = np < (size_t)max_paths ? np : (size_t)max_paths;
    memcpy(paths_out, paths, k * 14 * sizeof(int32_t));
  }
  mat34 *pM = (mat34 *)malloc(sizeof(mat34) * np);
  for (size_t i = 0; i < np; i++)
    for (int k = 0; k < 12; k++) pM[i].m[k] = wf(paths[14 * i + k]);

  unsigned char *traced = (unsigned char *)calloc((size_t)ng * np, 1);
  task_t *tasks = (task_t *)malloc(sizeof(task_t) * nu);
  size_t nt = 0;
  for (size_t i = 0; i < nu; i++) {
    int32_t *key = recs[i].w;
    int32_t *f = (int32_t *)bsearch(key, paths, np, 14 * sizeof(int32_t), cmp_path);
    int pid = (int)((f - paths) / 14);
    int cell = key[14];
    if (!traced[(size_t)cell * np + pid]) {
      traced[(size_t)cell * np + pid] = 1;
      tasks[nt].cell = cell; tasks[nt].pid = pid; nt++;
    }
  }
  free(recs);

  double *acc = (double *)calloc((size_t)n_src * n_dst * 2, sizeof(double));
  uint64_t okc = 0, failc = 0, ffc = 0;
  for (int round = 1;; round++) {
    unsigned char *succ = (unsigned char *)calloc(nt ? nt : 1, 1);
    st->rounds++;
    st->tasks += nt;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : okc, failc, ffc)
    for (long ti = 0; ti < (long)nt; ti++) {
      int cell = tasks[ti].cell, pid = tasks[ti].pid;
      int gi = cell / n1g, gj = cell % n1g;
      int hc = paths[14 * pid + 12], mask = paths[14 * pid + 13];
      for (int s = 0; s < n_src; s++)
        for (int inner = 0; inner < gs * gs; inner++) {
          int di = inner / gs + gi * gs, dj = inner % gs + gj * gs;
          if (p->strict_grid && (di >= n0_dst || dj >= n1_dst)) continue;
          int d = di * n1_dst + dj;
          if (d >= n_dst) continue;
          double re, im;
          int ff = 0;
          if (backward_ray(&S, p, &pM[pid], hc, mask, s, d, &re, &im, &ff)) {
            ffc += (uint64_t)ff;
            size_t o = ((size_t)s * n_dst + d) * 2;
#pragma omp atomic
            acc[o] += re;
#pragma omp atomic
            acc[o + 1] += im;
            okc++;
            succ[ti] = 1;
          } else {
            failc++;
          }
        }
    }
    /* 4-neighbour expansion of successful tasks (cpp:257-300) */
    task_t *nx = (task_t *)malloc(sizeof(task_t) * (nt * 4 + 1));
    size_t nn = 0;
    for (size_t ti = 0; ti < nt; ti++) {
      if (!succ[ti]) continue;
      int c = tasks[ti].cell, pid = tasks[ti].pid;
      int nb[4] = {c - 1, c + 1, c - n1g, c + n1g};
      for (int k = 0; k < 4; k++) {
        if (nb[k] < 0 || nb[k] >= ng) continue;
        if (!traced[(size_t)nb[k] * np + pid]) {
          traced[(size_t)nb[k] * np + pid] = 1;
          nx[nn].cell = nb[k]; nx[nn].pid = pid; nn++;
        }
      }
    }
    free(succ);
    free(tasks);
    tasks = nx;
    nt = nn;
    if (nt == 0) break;
  }
  st->rx_paths = okc;
  st->rx_fail = failc;
  st->farfield = ffc;
  for (size_t i = 0; i < (size_t)n_src * n_dst * 2; i++) result[i] += (float)acc[i];
  free(acc);
  free(tasks);
  free(traced);
  free(pM);
  free(paths);
  goto cleanup;
done:
  free(recs);
cleanup:
  for (int i = 0; i < 3; i++) bvh_free(&S.bvh[i]);
  free(slo); free(shi); free(dlo); free(dhi);
  return status;
}
