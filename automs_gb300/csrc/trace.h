// trace.h -- device-side parameter block and launchers of the channel tracer.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/ams.h"
#include "lbvh.h"

// device error flags (bits of TraceDev::err)
#define AMS_DERR_PATH_TABLE 1u    // path table full
#define AMS_DERR_HASH 2u          // a path-table slot's key words never appeared
#define AMS_DERR_STACK 4u         // traversal stack overflow
#define AMS_DERR_ACC_RANGE 8u     // contribution outside the fixed-point range
#define AMS_DERR_TASKS 16u        // task list overflow
#define AMS_DERR_BVH 32u          // BVH node index out of range
#define AMS_DERR_LOOP 64u         // a ray exceeded the segment cap

struct TraceDev {
  // scene triangles: original order [n_tri, 9] and sorted (3 float4 each)
  const float *tris;
  const BvhNode *tri_nodes;
  const float4 *tri_prims;
  int n_tri;
  const int *mat;
  const float *mat_prop;
  // Tx spheres (instance 1) and Rx spheres (instance 2)
  const BvhNode *tx_nodes;
  const float4 *tx_prims;
  int n_src;
  const float *src;  // original order [n_src, 3]
  float src_r;
  const BvhNode *rx_nodes;
  const float4 *rx_prims;
  int n_dst;
  const float *dst;  // original order [n_dst, 3]
  float dst_r;
  // Rx grid and cells
  int n0_dst, n1_dst, n0g, n1g, ng, gs;
  int strict_grid;
  // launch parameters
  int L, reserve, spl, launch_x, launch_y;
  float lam_f;
  double lam_d;
  double two_pi_over_lam;  // 2 pi / lam_d
  float src_dir[3], dst_dir[3];
  int src_bp, dst_bp;
  // path table (open addressing, slot = path id)
  unsigned long long *tab_h;
  int32_t *tab_key;  // 14 words per slot, sign bits flipped (0 = not written yet)
  unsigned tab_mask;
  unsigned tab_limit;  // occupied slots above this -> grow and retry
  // task bitmaps [ng][W]: stage 1 sets T in table-slot space (W = slots /
  // 32); stage 2 runs on dense path ids (W = ceil(n_paths / 32))
  unsigned *T;  // traced
  unsigned *N;  // new this round
  unsigned *S;  // succeeded this round
  int W;
  // stage-2 path ids: dense id -> table slot
  int *slot_of;
  int n_paths;
  // tasks of the current round per cell: dense path ids task_path[cell_off[c]
  // .. cell_off[c + 1]) of cell c, cut into chunks of up to kpi paths,
  // chunk_at[chunk_off[c] .. chunk_off[c + 1])
  int2 *task_path;  // (dense path id, table slot)
  int4 *chunk_at;   // (cell, first task, end task, 0)
  unsigned long long task_cap;  // entries of task_path and of chunk_at
  int *cell_cnt;   // [ng] tasks per cell of the coming round
  int *cell_off;   // [ng + 1]
  int *chunk_off;  // [ng + 1]
  int kpi;         // paths per stage-2 item this round
  // fixed-point channel accumulators, Rx-major: acc[(dst * n_src + s) * 2]
  unsigned long long *acc;
  // counters: 0 records, 1 overflow threads, 2 occupied slots, 3 ok rays,
  // 4 failed rays, 5 tasks this round, 6 unique records, 7 new tasks,
  // 8 stage-1 closest-hit queries, 9 stage-2 closest-hit queries,
  // 10 stage-1 launch-index fetch, 12 dense path ids, 13 int64 adds into acc
  unsigned long long *ctr;
  unsigned *err;
  // per-ray records of stage 2 (ams_trace_channel_export): record of ray r
  // of the round at rec[rec_base + r] while below rec_cap
  ams_ray_record *rec;
  unsigned long long rec_cap, rec_base;
};

cudaError_t trace_stage1(const TraceDev &P, cudaStream_t st);
// dense path ids (dense_of [slots], P.slot_of) and the stage-1 bitmap
// T_slots [ng][w_slots] turned into dense ids in `out` [ng][P.W], zeroed before
cudaError_t trace_dense_paths(const TraceDev &P, const unsigned *T_slots, int w_slots,
                              int *dense_of, unsigned *out, cudaStream_t st);
// paths per stage-2 item for a round of n_tasks tasks (set P.kpi before
// listing the round's tasks)
int trace_paths_per_item(const TraceDev &P, unsigned long long n_tasks);
// tasks per cell of the first stage-2 round (later rounds: trace_expand)
cudaError_t trace_count_tasks(const TraceDev &P, const unsigned *bits, cudaStream_t st);
// the round's task and chunk lists; also clears the success bitmap
cudaError_t trace_make_tasks(const TraceDev &P, const unsigned *bits, cudaStream_t st);
cudaError_t trace_stage2(const TraceDev &P, unsigned long long n_tasks, cudaStream_t st);
// one thread per ray, each ray's record written (P.rec; P.kpi must be 1)
cudaError_t trace_stage2_export(const TraceDev &P, unsigned long long n_tasks, cudaStream_t st);
cudaError_t trace_expand(const TraceDev &P, cudaStream_t st);
cudaError_t trace_count_bits(const TraceDev &P, const unsigned *bits, unsigned long long *out,
                             cudaStream_t st);
cudaError_t trace_finalize(const TraceDev &P, float *result, cudaStream_t st);
cudaError_t trace_export_paths(const TraceDev &P, int32_t *out_keys, unsigned long long *n_out,
                               cudaStream_t st);
