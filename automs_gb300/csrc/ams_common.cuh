// ams_common.cuh -- shared device helpers for the AutoMS GB300 kernels.
//
// Arithmetic contract of the tracer (trace.cu is compiled with -fmad=false):
// every geometric decision is made from IEEE float add/sub/mul/div/sqrt in
// the order written here, so ray sets are reproducible bit for bit by the
// CPU oracle.  Vector helpers follow the operation order of the reference's
// vector library (sutil/vec_math.h:527-570, Matrix.h:339-462).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define AMS_PIF 3.14159265358979323846f
#define AMS_TMIN 1e-5f   // optixPathTracer.cu:98
#define AMS_TMAX 1e16f
#define AMS_NBINS 19     // angle bins per material (go.py:690-698)
#define AMS_MAX_L 5      // 32 branch slots (optixPathTracer.h:5)
#define AMS_MAX_RESERVE 256

// Facts of the current device, looked up once per device (up to 64 devices
// per process).
#define AMS_MAX_DEVICES 64
inline int ams_current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= AMS_MAX_DEVICES) return -1;
  return dev;
}
// multiprocessors of the current device (1 if the query fails)
inline int ams_device_sms() {
  static int sms[AMS_MAX_DEVICES] = {0};
  const int dev = ams_current_device();
  if (dev < 0) return 1;
  if (sms[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 1;
    sms[dev] = n;
  }
  return sms[dev];
}
// Raise a kernel's dynamic shared-memory limit on the current device to at
// least `bytes`; `cur` is the caller's per-kernel record of the limit set.
template <class F>
inline cudaError_t ams_set_smem_atleast(size_t (&cur)[AMS_MAX_DEVICES], F *kernel, size_t bytes) {
  const int dev = ams_current_device();
  if (dev < 0) return cudaErrorInvalidDevice;
  if (cur[dev] >= bytes) return cudaSuccess;
  cudaError_t e =
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur[dev] = bytes;
  return e;
}


struct af3 { float x, y, z; };

__device__ __forceinline__ af3 mk3(float x, float y, float z) { af3 r; r.x = x; r.y = y; r.z = z; return r; }
__device__ __forceinline__ af3 add3(af3 a, af3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ af3 sub3(af3 a, af3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ af3 scl3(af3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ af3 neg3(af3 a) { return mk3(-a.x, -a.y, -a.z); }
__device__ __forceinline__ float dot3(af3 a, af3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ af3 cross3(af3 a, af3 b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float len3(af3 v) { return sqrtf(dot3(v, v)); }
__device__ __forceinline__ af3 nrm3(af3 v) { float inv = 1.0f / sqrtf(dot3(v, v)); return scl3(v, inv); }
__device__ __forceinline__ af3 faceforward3(af3 n, af3 i, af3 nref) {
  return scl3(n, copysignf(1.0f, dot3(i, nref)));
}
__device__ __forceinline__ af3 ld3(const float *p) { return mk3(p[0], p[1], p[2]); }
__device__ __forceinline__ float comp3(af3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// 64-bit and 32-bit mixers (splitmix64 finaliser, Steele et al. 2014;
// murmur3 fmix32, Appleby) used for the path table.
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint32_t mix32(uint32_t h) {
  h ^= h >> 16; h *= 0x85ebca6bu; h ^= h >> 13; h *= 0xc2b2ae35u; h ^= h >> 16;
  return h;
}

// Fixed-point scale of the channel accumulators: contributions are summed
// exactly as int64 multiples of 2^-56 (magnitude limit 64).
#define AMS_ACC_SCALE 72057594037927936.0       // 2^56
#define AMS_ACC_INV (1.0 / 72057594037927936.0)
#define AMS_ACC_LIMIT 64.0
