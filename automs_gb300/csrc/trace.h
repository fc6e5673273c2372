// trace.h -- device-side parameter block and launchers of the channel tracer.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

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
  // task bitmaps [ng][W] in slot space
  unsigned *T;  // traced
  unsigned *N;  // new this round
  unsigned *S;  // succeeded this round
  int W;
  // tasks of the current round per cell: slots task_slot[cell_off[c] ..
  // cell_off[c + 1]) of cell c; cells with tasks act_cells[0 .. *n_act),
  // active cell a owning stage-2 items item_off[a] .. item_off[a + 1)
  int *task_slot;
  unsigned long long task_cap;
  int *cell_off;        // [ng + 1]
  int *act_cells;       // [ng]
  long long *item_off;  // [ng + 1]
  int *n_act;
  int kpi;              // paths per stage-2 item this round
  // fixed-point channel accumulators, Rx-major: acc[(dst * n_src + s) * 2]
  unsigned long long *acc;
  // counters: 0 records, 1 overflow threads, 2 occupied slots, 3 ok rays,
  // 4 failed rays, 5 tasks this round, 6 unique records, 7 new tasks,
  // 8 stage-1 closest-hit queries, 9 stage-2 closest-hit queries,
  // 10 stage-1 launch-index fetch, 11 stage-2 item fetch
  unsigned long long *ctr;
  unsigned *err;
};

cudaError_t trace_stage1(const TraceDev &P, cudaStream_t st);
// paths per stage-2 item for a round of n_tasks tasks (set P.kpi before
// listing the round's tasks)
int trace_paths_per_item(const TraceDev &P, unsigned long long n_tasks);
cudaError_t trace_make_tasks(const TraceDev &P, const unsigned *bits, cudaStream_t st);
cudaError_t trace_stage2(const TraceDev &P, unsigned long long n_tasks, cudaStream_t st);
cudaError_t trace_expand(const TraceDev &P, cudaStream_t st);
cudaError_t trace_count_bits(const TraceDev &P, const unsigned *bits, unsigned long long *out,
                             cudaStream_t st);
cudaError_t trace_finalize(const TraceDev &P, float *result, cudaStream_t st);
cudaError_t trace_export_paths(const TraceDev &P, int32_t *out_keys, unsigned long long *n_out,
                               cudaStream_t st);
