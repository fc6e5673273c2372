/*
 * optix.h (shim) -- a CPU stand-in for the handful of OptiX 7 device calls
 * that the reference's device programs use, so that those programs can be
 * compiled as plain host C++ and run on the CPU as a reference oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  It is placed first on the include path of the
 * harness build (oracle/ref_harness/build_ref.py) and shadows the real
 * OptiX header.  The ray traversal itself (closest hit over triangles and
 * AABB primitives) is implemented in ref_harness.cpp; the reference's own
 * closest-hit, miss and intersection programs are called from there.
 */
#pragma once
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <cmath>
#include <algorithm>
#include <vector_types.h>
#include <vector_functions.h>

#define __global__
#define __device__
#define __host__
#define __constant__
#define __forceinline__ inline

typedef unsigned long long OptixTraversableHandle;
typedef unsigned int OptixVisibilityMask;
enum { OPTIX_RAY_FLAG_NONE = 0 };
typedef unsigned int uint;

struct ShimState {
  uint3 launch_index;
  uint3 launch_dim;
  unsigned int payload0, payload1;
  float3 ray_o, ray_d;
  float ray_tmin, ray_tmax;
  int cur_prim, cur_inst;
  float hit_t;
  int hit_prim, hit_inst;
  bool in_closest_hit;
};
extern ShimState g_shim;

inline uint3 optixGetLaunchIndex() { return g_shim.launch_index; }
inline uint3 optixGetLaunchDimensions() { return g_shim.launch_dim; }
inline unsigned int optixGetPayload_0() { return g_shim.payload0; }
inline unsigned int optixGetPayload_1() { return g_shim.payload1; }
inline float3 optixGetWorldRayOrigin() { return g_shim.ray_o; }
inline float3 optixGetWorldRayDirection() { return g_shim.ray_d; }
inline float optixGetRayTmax() { return g_shim.hit_t; }
inline unsigned int optixGetPrimitiveIndex() {
  return (unsigned int)(g_shim.in_closest_hit ? g_shim.hit_prim : g_shim.cur_prim);
}
inline unsigned int optixGetInstanceId() {
  return (unsigned int)(g_shim.in_closest_hit ? g_shim.hit_inst : g_shim.cur_inst);
}
bool optixReportIntersection(float t, unsigned int kind);
void optixTrace(OptixTraversableHandle handle, float3 o, float3 d, float tmin,
                float tmax, float time, OptixVisibilityMask mask,
                unsigned int flags, unsigned int sbt_offset,
                unsigned int sbt_stride, unsigned int miss_index,
                unsigned int &u0, unsigned int &u1);

inline float atomicAdd(float *a, float v) { float o = *a; *a = o + v; return o; }
inline unsigned long long atomicAdd(unsigned long long *a, unsigned long long v) {
  unsigned long long o = *a; *a = o + v; return o;
}

extern "C" void __closesthit__forward();
extern "C" void __closesthit__backward();
extern "C" void __miss__forward();
extern "C" void __miss__backward();
extern "C" void __intersection__sphere();
