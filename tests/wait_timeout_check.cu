// Bounded mbarrier wait (automs_gb300/csrc/tc_ptx.cuh, used by every TMA /
// tcgen05 pipeline of the library) run out on purpose, without a fault: one
// thread waits on an mbarrier that nothing arrives on, with a short limit,
// and reports whether the wait gave up and after how long.  Built by
// tests/test_gpu_wait_timeout.py with nvcc.
#include <cuda_runtime.h>

#include "tc_ptx.cuh"

__global__ void k_wait_nothing(unsigned long long limit_ns, unsigned long long *out) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned long long t0 = tc::now_ns();
    const bool ok = tc::mbar_wait(&bar, 0, limit_ns);  // phase 0 never completes
    out[0] = ok ? 1ull : 0ull;
    out[1] = tc::now_ns() - t0;
  }
}

extern "C" int run_wait_nothing(unsigned long long limit_ns, unsigned long long *ok,
                                unsigned long long *elapsed_ns) {
  unsigned long long *d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return 1;
  k_wait_nothing<<<1, 32>>>(limit_ns, d);
  unsigned long long h[2] = {2, 0};
  cudaError_t e = cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return 2;
  *ok = h[0];
  *elapsed_ns = h[1];
  return 0;
}
