/*
 * ams_oracle.h -- CPU restatement of the AutoMS ray-traced channel simulator.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it.  The product path never calls it.
 *
 * What it restates (reference file:line):
 *   - stage-1 forward discovery   optixPathTracer.cu:142-190, :285-331
 *   - stage-2 backward verify     optixPathTracer.cu:191-273, :332-417
 *   - sphere capture              optixPathTracer.cu:419-445
 *   - beam patterns               optixPathTracer.cu:107-136
 *   - host dedup + flood fill     optixPathTracer.cpp:93-360
 *   - TEA/LCG random numbers      optix/SDK/cuda/random.h:31-67
 *
 * Arithmetic contract shared with the CUDA kernels: every decision (which
 * triangle / sphere a ray hits, which cell a record lands in, path keys) is
 * made from IEEE float add/sub/mul/div/sqrt in a fixed order with no FMA
 * contraction, so the ray sets match the CUDA path bit for bit.  The path
 * length is summed in FP64 and the phase 2*pi*d/lambda is formed in FP64.
 * Triangle hits use the watertight test of Woop, Benthin and Wald (JCGT
 * 2013) because the reference's OptiX test is closed driver code.
 *
 * Parity of this oracle with the reference is pinned by oracle/ref_harness,
 * which runs the reference's own device programs on the CPU.
 */
#ifndef AMS_ORACLE_H
#define AMS_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int samples_per_launch;
  int launch_x, launch_y;
  double wave_len;
  int max_reflection;   /* <= 5 (32 branch slots, optixPathTracer.h:5) */
  int reserve_size;     /* per-thread record cap (optixPathTracer.cu:173) */
  int src_bptype, dst_bptype;
  int dst_gridsize;
  float src_r, dst_r;
  float src_dir[3], dst_dir[3];
  int strict_grid;      /* 0: reproduce the reference's row wrap at the grid edge */
} orc_params;

typedef struct {
  uint64_t rx_paths;        /* stats[0] of the reference */
  uint64_t rx_fail;         /* stats[1] */
  uint64_t fwd_records;     /* trace_count_original */
  uint64_t unique_records;  /* trace_count after unique */
  uint64_t unique_paths;    /* pathList size */
  uint64_t rounds;          /* stage-2 rounds that ran */
  uint64_t tasks;           /* (path, cell) tasks traced over all rounds */
  uint64_t overflow;        /* threads that hit the reserve cap */
  uint64_t farfield;        /* verified rays whose loss used the far-field switch
                               (optixPathTracer.cu:369-377) at least once */
} orc_stats;

/* Full build_channel: accumulates into result[n_src*n_dst*2] (re, im).
 * src_aabb/dst_aabb may be NULL (then pos -/+ r).  paths_out (optional)
 * receives the sorted unique path list as 14 words per path
 * (12 floats of the image transform, hit_cnt, is_reflect). */
int orc_trace_channel(const float *tris, int n_tri, const int *mat,
                      const float *mat_prop, int n_mat, const float *src,
                      int n_src, const float *dst, int n0_dst, int n1_dst,
                      const float *src_aabb, const float *dst_aabb,
                      const orc_params *p, float *result, orc_stats *st,
                      int32_t *paths_out, int max_paths, int nthreads);

/* Unit-level restatements exposed for tests. */
uint32_t orc_tea4(uint32_t v0, uint32_t v1);
float orc_rnd(uint32_t *seed);
void orc_rand_dir(uint32_t *seed, uint32_t ix, uint32_t iy, int launch_x,
                  int launch_y, float out[3]);
/* (sin a, cos a) of a float angle in [0, 7), correctly rounded to float
 * except within ~1e-16 of a rounding midpoint */
void orc_sincos(float a, float out[2]);
int orc_theta_id(float cos_theta);
float orc_beampattern(const float d1[3], const float d2[3], int type);
/* watertight triangle hit: returns t or -1 */
float orc_intersect_tri(const float o[3], const float d[3], const float v0[3],
                        const float v1[3], const float v2[3]);
/* slab test of a ray against a primitive AABB over [1e-5, 1e16] */
int orc_prim_slab(const float o[3], const float d[3], const float lo[3],
                  const float hi[3]);

#ifdef __cplusplus
}
#endif
#endif
