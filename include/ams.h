/*
 * ams.h -- C ABI of the AutoMS GB300 library (libams.so).
 *
 * Plain pointers and sizes only.  Pointers documented "device" are CUDA
 * device pointers (e.g. torch.Tensor.data_ptr() of a CUDA tensor); "host"
 * pointers are ordinary host memory.  Every entry point returns an
 * ams_status; on failure a message is written to errbuf (if given) and
 * nothing is thrown across the ABI.  All work is enqueued on `stream`
 * (a cudaStream_t, NULL = legacy default stream) and the call returns after
 * the stream has finished the call's work, unless stated otherwise.
 *
 * Reference interfaces replaced (microsoft/AutoMS):
 *   torch.ops.pathtrace.torch_launch_pathtrace   optixPathTracer.cpp:781-870
 *   Model.get_channel / Model.forward / backward go.py:107-245
 *   draw_channel coverage reduction             go.py:849-851, 944-964
 */
#ifndef AMS_H
#define AMS_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int ams_status;
#define AMS_OK 0
#define AMS_ERR_ARG 1       /* bad argument (null pointer, size, type) */
#define AMS_ERR_OOM 2       /* device allocation failed */
#define AMS_ERR_CUDA 3      /* CUDA runtime / launch error */
#define AMS_ERR_CAPACITY 4  /* a fixed capacity was exceeded */
#define AMS_ERR_NUMERIC 6   /* value outside the representable range */
#define AMS_ERR_INTERNAL 7  /* internal consistency check failed */

/* Library version string. */
const char *ams_version(void);

/* ------------------------------------------------------------- tracer */

/* Scene: triangles and materials, with the triangle BVH built once and kept
 * across trace calls (the reference rebuilds its OptiX structures on every
 * call, optixPathTracer.cpp:834-839).  One scene per host thread. */
typedef struct ams_scene ams_scene;

/* Launch parameters of one channel build; fields and meaning as the
 * arguments of torch_launch_pathtrace (optixPathTracer.cpp:781-790). */
typedef struct {
  int samples_per_launch; /* rays per launch index */
  int launch_x, launch_y; /* stage-1 launch grid */
  double wave_len;        /* wavelength [m] */
  int max_reflection;     /* 0..5 */
  int reserve_size;       /* per-launch-index record cap, 1..256 */
  int src_bptype, dst_bptype; /* beam pattern types 0..3 */
  int dst_gridsize;       /* Rx cell edge (cells of gs x gs Rx) */
  float src_r, dst_r;     /* sphere radii of Tx and Rx */
  float src_dir[3], dst_dir[3]; /* array boresights (host values) */
  int strict_grid;        /* 0 = reference behaviour at the grid edge */
  int log_level;          /* 0 silent, 1 per-stage timings on stderr */
} ams_trace_params;

/* Counters of one build.  rx_paths is the reference's stats[0]
 * (successful backward verifications), rx_fail its stats[1]. */
typedef struct {
  unsigned long long rx_paths, rx_fail;
  unsigned long long fwd_records;    /* records kept by stage 1 */
  unsigned long long unique_records; /* distinct (path, cell) pairs */
  unsigned long long unique_paths;   /* distinct path keys */
  unsigned long long rounds;         /* stage-2 rounds */
  unsigned long long tasks;          /* (path, cell) tasks traced */
  unsigned long long overflow;       /* launch indices that hit reserve_size */
  float ms_bvh, ms_stage1, ms_stage2, ms_total;
  unsigned long long workspace_bytes; /* device workspace high-water mark */
  unsigned long long segments_fwd;   /* closest-hit queries of stage 1 */
  unsigned long long segments_bwd;   /* closest-hit queries of stage 2 */
  float ms_stage2_kernel;            /* device time of the backward kernels */
  unsigned long long acc_adds;       /* int64 atomic adds into the fixed-point H:
                                        two per verified ray in rounds of one
                                        path per item, two per (Tx, Rx) pair
                                        and chunk of paths otherwise */
} ams_stats;

/* Create a scene from device arrays: tris [n_tri*9] float (3 vertices per
 * triangle), mat [n_tri] int32 material ids, mat_prop [n_mat*19] float
 * (angle-bin coefficients, negative = penetrable).  The arrays are copied
 * (after the work queued on `stream`); material ids outside [0, n_mat) and
 * non-finite coordinates are rejected with AMS_ERR_ARG.  The triangle
 * hierarchy is built once here: a GPU LBVH below 16,384 triangles, a
 * binned-SAH tree built on host threads from there on.  Synchronous.
 * Replaces the scene part of optixPathTracer.cpp:382-546. */
ams_status ams_scene_create(const float *tris, int n_tri, const int *mat,
                            const float *mat_prop, int n_mat, void *stream,
                            ams_scene **out, char *errbuf, size_t errlen);
/* The scene's device memory goes back to a per-device pool that the next
 * scene draws from (no cudaFree, so no device-wide synchronisation); call
 * only after the scene's last call returned. */
void ams_scene_destroy(ams_scene *scene);

/* Build the channel from src [s0*s1*3] to dst [n0*n1*3] (device float) and
 * ACCUMULATE it into result [s0*s1, n0*n1, 2] (device float, re/im
 * interleaved), as the reference op does (optixPathTracer.cu:259-264).
 * src_aabb/dst_aabb [n*6] (device) may be NULL: then pos -/+ r.
 * stats may be NULL.  A build that finds no path is status AMS_OK with
 * stats->unique_paths == 0 (the reference's "No path found!"). */
ams_status ams_trace_channel(ams_scene *scene, const ams_trace_params *p,
                             const float *src, int s0, int s1, const float *dst,
                             int n0, int n1, const float *src_aabb,
                             const float *dst_aabb, float *result,
                             ams_stats *stats, void *stream, char *errbuf,
                             size_t errlen);

/* One-shot drop-in for torch_launch_pathtrace (optixPathTracer.cpp:781-790):
 * same arguments in the same order, flattened to pointers and sizes.
 * src_dir/dst_dir are HOST float[3] (the reference dereferences them on the
 * host, optixPathTracer.cpp:827-828); every other array is device memory. */
ams_status ams_launch_pathtrace(
    float *result, const float *src, int s0, int s1, const float *dst, int n0,
    int n1, const float *src_aabb, const float *dst_aabb,
    const float *scene_tris, int n_tri, const int *mat,
    int samples_per_launch, int launch_x, int launch_y, double wave_len,
    int max_reflection, int reserve_size, const float *mat_prop, int n_mat,
    const float *src_dir, const float *dst_dir, int log_level, int src_bptype,
    int dst_bptype, int dst_gridsize, double src_r, double dst_r,
    ams_stats *stats, char *errbuf, size_t errlen);

/* One backward ray of stage 2, as the reference's EXPORT_TASKINFO build
 * records it (ExportedTaskInfo, optixPathTracer.h:40-52, filled at
 * optixPathTracer.cu:200-268, 378-413): whether it reached its Tx; the
 * cosines at the Tx (launch_angle, against src_dir) and at the Rx
 * (receive_angle, against dst_dir); loss = the product of the free-space
 * factors (far-field splits and lambda / (4 pi d)), material losses left
 * out; phase = 2 pi d / lambda of the whole path (radians, unreduced; FP64
 * here, FP32 in the reference); the Tx, the Rx, the scene hits and, per
 * hit, theta_id + 19 * material (the mat_prop entry of its loss).  Here
 * also the path id and whether the ray was traced (its Rx exists). */
typedef struct {
  int32_t src, dst, path, traced;
  int32_t successful, hit_cnt;
  float launch_angle, receive_angle, loss, pad0;
  double phase;
  int32_t hit_loss_idx[5];
  int32_t pad1;
} ams_ray_record; /* 72 bytes */

/* ams_trace_channel, and every backward ray of stage 2 written to records
 * (device, capacity max_records; rays past it are counted, not written) in
 * round order, then task order (cells in order, paths within a cell), then
 * Rx within the cell, then Tx.  *n_records receives the number of rays.
 * Slower than ams_trace_channel (one thread per ray in every round). */
ams_status ams_trace_channel_export(ams_scene *scene, const ams_trace_params *p,
                                    const float *src, int s0, int s1,
                                    const float *dst, int n0, int n1,
                                    const float *src_aabb, const float *dst_aabb,
                                    float *result, ams_stats *stats,
                                    ams_ray_record *records,
                                    unsigned long long max_records,
                                    unsigned long long *n_records, void *stream,
                                    char *errbuf, size_t errlen);

/* Path list of the scene's last build: 14 int32 words per path (12 floats
 * of the image transform, hit count, reflect mask; optixPathTracer.h:9-13),
 * unordered, into host memory.  *n_out receives the number of paths. */
ams_status ams_trace_export_paths(ams_scene *scene, int32_t *host_out,
                                  int max_paths, int *n_out, char *errbuf,
                                  size_t errlen);

/* ----------------------------------------------------------- objective */

/* Phase-map coverage objective and its adjoint (go.py:107-245, loss mode
 * "capacity") for one metasurface hop:
 *   Y = W H_d + ((W H_a) o exp(j (phi mod max_phase))) H_r     [C, R]
 *   cap = log2(1 + (|Y| + eps)^2 / 1e-9)
 *   cap' = cap with the rows where drop[c] != 0 zeroed
 *   loss = -w * sum_r max_c cap' + || cap' o (cap' != max_c cap') ||_F
 * All arrays are device memory, complex values are interleaved float pairs
 * in the reference orientation: H_d [S,R], H_a [S,M], H_r [M,R], W [C,S].
 * H_a/H_r/phi/grad_phi may be NULL (no metasurface, M ignored).  drop [C]
 * uint8 may be NULL (no dropout).  Outputs: loss [1] float, grad_W [C,S]
 * complex (dL/dRe + j dL/dIm), grad_phi [M] float, grad_Y [C,R] complex
 * (gradient with respect to Y, for callers that compose the channel
 * themselves), recv_amp [C,R] float (|Y|, Model.result of go.py:170); any of
 * them may be NULL.  The call is asynchronous on `stream`.  Scratch memory is
 * allocated internally on first use and kept across calls; calls on one
 * device must not overlap. */
ams_status ams_objective_fwd_bwd(const float *H_d, const float *H_a,
                                 const float *H_r, const float *phi,
                                 float max_phase, const float *W, int S, int M,
                                 int R, int C, float w, const uint8_t *drop,
                                 float *loss, float *grad_W, float *grad_phi,
                                 float *grad_Y, float *recv_amp, void *stream,
                                 char *errbuf, size_t errlen);

/* Allocation-free variant of ams_objective_fwd_bwd.  No counterpart in the
 * reference: it exists for callers that must not allocate device memory,
 * e.g. code that owns the whole device memory through its own pool, code
 * inside a CUDA stream capture where cudaMalloc is not allowed, or
 * latency-critical loops that cannot afford cudaMalloc's implicit
 * synchronisation.  Same arguments and results as ams_objective_fwd_bwd;
 * its scratch is a fixed array of AMS_OBJECTIVE_NOALLOC_MAX_SCRATCH bytes
 * inside the library image (held on every device that loads the library
 * until the process exits), so the call itself never allocates.  Problems
 * whose scratch would exceed that size are rejected with AMS_ERR_CAPACITY.
 * The first call on a device looks the array up for that device; make that
 * first call before any stream capture.  All calls on a device share the
 * array, so calls that overlap on the GPU (different streams, threads) race
 * and give wrong results: serialise them.  The call is asynchronous on
 * `stream`. */
#define AMS_OBJECTIVE_NOALLOC_MAX_SCRATCH (16u << 20)
ams_status ams_objective_fwd_bwd_noalloc(
    const float *H_d, const float *H_a, const float *H_r, const float *phi,
    float max_phase, const float *W, int S, int M, int R, int C, float w,
    const uint8_t *drop, float *loss, float *grad_W, float *grad_phi,
    float *grad_Y, float *recv_amp, void *stream, char *errbuf, size_t errlen);

/* Evaluation plan of ams_objective_fwd_bwd for a fixed channel set (one
 * metasurface hop) evaluated many times -- the optimizer loop of
 * optimize_model (go.py:296-336), with the reference's code_num codes or
 * with C = 1.  No single counterpart in the reference: it replaces the
 * autograd forward/backward of Model.forward (go.py:159-245) when the
 * channels are fixed.  With C_max > 2 it is the tensor-core path.  The plan converts [H_r; H_d] once into BF16 hi/lo
 * pairs (x = hi + lo, 3xBF16 products with FP32 accumulation, relative
 * error about 1e-5) in the two layouts of the forward and adjoint GEMMs
 * (tcgen05 tensor cores).  H_d, H_a, H_r must stay valid and unchanged while
 * the plan lives.  ams_objective_plan_fwd_bwd has the arguments and results
 * of ams_objective_fwd_bwd (the channels come from the plan); calls on one
 * plan must not overlap.  The plan owns about 8 (R (M+S) + (M+S) R) bytes of
 * device memory (ams_objective_plan_bytes).  A plan made with C_max <= 2
 * (and M+S <= 4096 for one code, 2048 for two) instead holds one FP32 copy
 * of [H_r; H_d] transposed to [R][M+S] and runs the single-pass streaming
 * kernels over it (each tile of Rx is one contiguous block); it does not
 * produce grad_Y (AMS_ERR_ARG). */
typedef struct ams_objective_plan ams_objective_plan;
ams_status ams_objective_plan_create(const float *H_d, const float *H_a,
                                     const float *H_r, int S, int M, int R,
                                     int C_max, void *stream,
                                     ams_objective_plan **out, char *errbuf,
                                     size_t errlen);
ams_status ams_objective_plan_fwd_bwd(ams_objective_plan *plan,
                                      const float *phi, float max_phase,
                                      const float *W, int C, float w,
                                      const uint8_t *drop, float *loss,
                                      float *grad_W, float *grad_phi,
                                      float *grad_Y, float *recv_amp,
                                      void *stream, char *errbuf,
                                      size_t errlen);
unsigned long long ams_objective_plan_bytes(const ams_objective_plan *plan);

/* Plan over a stacked channel set for several metasurfaces: H_r [M, R]
 * holds the rows of every metasurface's MS->Rx channel one after the other
 * (M = the sum of their sizes), H_d [S, R] the AP->Rx channel; tensor-core
 * mode (3xBF16) whatever C_max.  Its evaluations take the coefficient of
 * every metasurface row directly, U [C, M] complex: the sum over all
 * metasurface paths that end on that element of the path product up to it
 * (go.py:112-156; for one metasurface U = (W H_a) o e^{j phi'}), so that
 *   Y = W H_d + U H_r
 * and the loss is that of ams_objective_fwd_bwd.  Outputs: loss, grad_U
 * [C, M] (dL/dU, complex convention of grad_W), grad_W [C, S] (the H_d
 * term only), recv_amp [C, R]; any but loss may be NULL.  The caller chains
 * grad_U back through its path products (ams_cgemm). */
ams_status ams_objective_plan_create_stacked(const float *H_d, const float *H_r,
                                             int S, int M, int R, int C_max,
                                             void *stream,
                                             ams_objective_plan **out,
                                             char *errbuf, size_t errlen);
ams_status ams_objective_plan_coef_fwd_bwd(ams_objective_plan *plan,
                                           const float *U, const float *W,
                                           int C, float w, const uint8_t *drop,
                                           float *loss, float *grad_U,
                                           float *grad_W, float *recv_amp,
                                           void *stream, char *errbuf,
                                           size_t errlen);

/* C = op(A) op(B) (+ C when accumulate != 0) for row-major complex64
 * device matrices (interleaved float pairs) on the CUDA cores, FP32: op 0
 * as is, 1 transposed, 2 conjugate transposed, 3 conjugated; C is m x n, k the inner
 * dimension, lda/ldb/ldc in complex elements.  The path products between
 * metasurfaces of go.py:138-146 and their adjoints (small: C codes by the
 * metasurface sizes). */
ams_status ams_cgemm(int m, int n, int k, const float *A, int lda, int opA,
                     const float *B, int ldb, int opB, float *C, int ldc,
                     int accumulate, void *stream, char *errbuf, size_t errlen);
void ams_objective_plan_destroy(ams_objective_plan *plan);

/* Wait-timeout report of the objective.  The streaming and tensor-core
 * kernels wait on TMA copies with a 2 s limit per wait; when a wait runs out
 * the kernel drains its copies in flight, the call's outputs (loss,
 * gradients) are written as NaN, and this call reports it: it synchronises
 * `stream` and returns AMS_ERR_INTERNAL (message in errbuf) if a wait of the
 * last call on `plan` -- or, with plan == NULL, of the last
 * ams_objective_fwd_bwd / ams_objective_fwd_bwd_noalloc call on the current
 * device -- ran out, AMS_OK otherwise.  Each call clears its own report when
 * it starts.  No counterpart in the reference (whose op returns void,
 * optixPathTracer.cpp:858-860). */
ams_status ams_objective_status(const ams_objective_plan *plan, void *stream,
                                char *errbuf, size_t errlen);

/* Fault injection for tests of the error path: the next `calls` objective
 * calls that take a path with bounded waits (streaming or tensor-core
 * kernels) report one of their waits as run out, exactly as a TMA copy that
 * did not arrive in time would, without waiting less or touching the GPU's
 * state.  0 cancels.  Not for production use. */
void ams_debug_inject_wait_timeout(int calls);

/* Received amplitude |Y| [C,R] of the same model (forward only). */
ams_status ams_objective_recv(const float *H_d, const float *H_a,
                              const float *H_r, const float *phi,
                              float max_phase, const float *W, int S, int M,
                              int R, int C, float *recv_amp, void *stream,
                              char *errbuf, size_t errlen);

/* Coverage map in dB: 20 log10 |sum over Tx of H[:, r]| + offset, NaN or
 * -inf replaced by threshold, clamped below at threshold
 * (go.py:849-851, 944-964).  H [S,R] complex device, out [R] float device. */
ams_status ams_coverage_db(const float *H, int S, int R, float threshold,
                           float offset, float *out, void *stream,
                           char *errbuf, size_t errlen);

/* ------------------------------------------------------ surrogate MLP */

/* BF16 GEMM on the tensor cores (tcgen05): C = A . B^T with A [M,K], B [N,K]
 * bf16 row-major (device), FP32 accumulation; epilogue adds bias [N] (may be
 * NULL), applies ReLU if relu != 0, and stores C32 [M,N] float and/or C16
 * [M,N] bf16 (either may be NULL).  M % 128 == 0, N % 64 == 0, K % 64 == 0.
 * No counterpart in the reference (building block of the surrogate). */
ams_status ams_gemm_bf16(const void *A, const void *B, int M, int N, int K,
                         const float *bias, int relu, float *C32, void *C16,
                         void *stream, char *errbuf, size_t errlen);

/* Surrogate network that maps a placement descriptor to a coverage-gain map
 * and screens annealing candidates; it replaces the blind trials of the
 * reference's NNI tuner (physical_exp_nni_main.py:11-29).  dims[0..n_dims-1]
 * are the layer widths (input, hidden..., output); every width after the
 * input must be a multiple of 128.  ReLU between layers, MSE loss, Adam.
 * Weights are FP32 masters with BF16 copies for the tensor-core GEMMs. */
typedef struct ams_mlp ams_mlp;
ams_status ams_mlp_create(const int *dims, int n_dims, int max_batch,
                          unsigned long long seed, void *stream, ams_mlp **out,
                          char *errbuf, size_t errlen);
void ams_mlp_destroy(ams_mlp *mlp);
/* Y [B, d_out] = net(X [B, d_in]); float device arrays, B <= max_batch. */
ams_status ams_mlp_forward(ams_mlp *mlp, const float *X, int B, float *Y,
                           void *stream, char *errbuf, size_t errlen);
/* One Adam step on the batch (X, T [B, d_out]); loss (device float, may be
 * NULL) receives the mean squared error before the step. */
ams_status ams_mlp_train_step(ams_mlp *mlp, const float *X, const float *T,
                              int B, float lr, float *loss, void *stream,
                              char *errbuf, size_t errlen);
/* Gradient of the loss without a step, written to grads (device) in the
 * parameter layout below. */
ams_status ams_mlp_gradients(ams_mlp *mlp, const float *X, const float *T,
                             int B, float *loss, float *grads, void *stream,
                             char *errbuf, size_t errlen);
/* Parameters as one float array: for each layer W [d_out, d_in] row-major
 * then b [d_out].  direction 0 copies out (get), 1 copies in (set).
 * *count receives the number of floats; params may be NULL to query it. */
ams_status ams_mlp_params(ams_mlp *mlp, float *params, int direction,
                          long long *count, void *stream, char *errbuf,
                          size_t errlen);
/* Adam state for checkpoint / resume: first and second moments (device
 * float arrays of ams_mlp_params' count, same layout) and the step count.
 * direction 0 copies out, 1 copies in; with the parameters restored too,
 * training continues exactly as if it had not stopped.  The reference keeps
 * no learned state (its checkpoints are torch.save of results,
 * physical_exp_nni_model.py:152-161, and the best-loss snapshot of
 * optimize_model, go.py:320-335); this serves the surrogate. */
ams_status ams_mlp_adam_state(ams_mlp *mlp, float *m1, float *m2,
                              long long *step, int direction, void *stream,
                              char *errbuf, size_t errlen);

/* Device bytes held by the library itself: the objective's internal scratch
 * (all devices) and the blocks of destroyed scenes kept for reuse by the
 * next scene -- for leak checks. */
unsigned long long ams_scratch_bytes(void);

#ifdef __cplusplus
}
#endif
#endif
