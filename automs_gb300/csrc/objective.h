// objective.h -- launcher of the phase-map objective kernels (objective.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/ams.h"

struct ObjArgs {
  const float *Hd, *Ha, *Hr, *phi, *W;
  float max_phase;
  int S, M, R, C;
  float w;
  const uint8_t *drop;
  float *loss, *grad_W, *grad_phi, *recv_amp, *grad_Y;
  // plan evaluations with the metasurface rows' coefficient given directly
  // (U_in [C, M], instead of (W H_a) e^{j phi'}): grad_U [C, M] receives
  // dL/dU and grad_W only the H_d rows' part
  const float *U_in = nullptr;
  float *grad_U = nullptr;
};

// Byte offsets of the scratch regions for one problem size.  The first 256
// bytes are a control block at a fixed offset: a float (1/||masked||) at 0,
// three last-CTA arrival counters (uint32) at 32, 36 and 40, and a
// wait-timeout flag word at 48.  They must be zero before the first call; every call leaves the
// counters at zero again.
struct ObjScratchLayout {
  size_t U, G1, G2, part, GU, inv, Um, gw, Pp, lp, GUs, total;
};
constexpr size_t kObjControlBytes = 256;

ObjScratchLayout obj_scratch_layout(int S, int M, int R, int C);
// enqueue one evaluation on `st`; scratch must hold layout.total bytes
cudaError_t obj_run(const ObjArgs &a, char *scratch, cudaStream_t st);
cudaError_t coverage_db_run(const float *H, int S, int R, float threshold, float offset,
                            float *out, cudaStream_t st);
// Wait-timeout word: the kernels with bounded mbarrier waits set the word at
// control-block offset 48 when a wait runs out; every call on such a path
// clears it first (its first kernel, or obj_begin_call), and the call's
// outputs are then NaN.
cudaError_t obj_begin_call(unsigned *err, bool cleared, cudaStream_t st);
// test hook: the next `calls` calls on paths with bounded waits behave as if
// one of their waits had run out
void obj_inject_timeouts(int calls);
// scratch of the allocation-free entry point (objective.cu); the first call
// on a device looks up the array's device address
cudaError_t obj_noalloc_scratch(char **out);

// Evaluation plan for a fixed channel set with a metasurface hop.  Cmax > 2:
// tensor cores (tcgen05, 3xBF16 split precision); the plan holds BF16 hi/lo
// copies of [H_r; H_d] in the two layouts the forward and adjoint GEMMs read.
// Cmax <= 2: streaming kernels over a transposed FP32 copy [R][M+S] (one
// contiguous block per tile of Rx; grad_Y is not produced).  The plan owns
// its scratch.  H_d, H_a and H_r must stay valid while the plan is used;
// evaluations on one plan must not overlap.  1 <= C <= Cmax <= 64.
struct ObjTcPlan;
cudaError_t obj_tc_plan_create(const float *Hd, const float *Ha, const float *Hr, int S, int M,
                               int R, int Cmax, cudaStream_t st, ObjTcPlan **out,
                               bool force_tc = false);
cudaError_t obj_tc_run(ObjTcPlan *p, const ObjArgs &a, cudaStream_t st);
size_t obj_tc_plan_bytes(const ObjTcPlan *p);
// device address of the plan's wait-timeout word
const unsigned *obj_tc_plan_status_word(const ObjTcPlan *p);
bool obj_tc_plan_streams(const ObjTcPlan *p);
void obj_tc_plan_destroy(ObjTcPlan *p);

// C = op(A) op(B) (+ C when accumulate) for row-major complex64 matrices on
// the CUDA cores; op 0 = as is, 1 = transposed, 2 = conjugate transposed,
// 3 = conjugated.
// C is m x n, the inner dimension k; lda, ldb, ldc in complex elements.
cudaError_t cgemm_run(int m, int n, int k, const float *A, int lda, int opA, const float *B,
                      int ldb, int opB, float *C, int ldc, bool accumulate, cudaStream_t st);
