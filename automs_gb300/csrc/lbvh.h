// lbvh.h -- linear BVH over triangles or sphere AABBs (see lbvh.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

struct PrimBox { float lo[3], hi[3]; };

// 64-byte node: a = (c0.lo.xyz, c0.hi.x), b = (c0.hi.yz, c1.lo.xy),
// c = (c1.lo.z, c1.hi.xyz), d = (child0, child1); child < 0 is leaf ~child.
struct __align__(16) BvhNode { float4 a, b, c; int4 d; };

struct Lbvh {
  int n = 0;               // primitives
  BvhNode *nodes = nullptr;  // n-1 internal nodes, root = 0
  int *perm = nullptr;     // sorted position -> original primitive index
  float4 *prims = nullptr; // 3 float4 per sorted primitive (see lbvh.cu)
};

size_t lbvh_scratch_bytes(int n);
size_t lbvh_output_bytes(int n);
cudaError_t lbvh_build_triangles(Lbvh &out, const float *tris, int n, char *scratch,
                                 char *outbuf, cudaStream_t st);
cudaError_t lbvh_build_spheres(Lbvh &out, const float *pos, const float *aabb, int n,
                               char *scratch, char *outbuf, cudaStream_t st);
// adopts a hierarchy built on the host (bvh_sah.h) for triangles already on
// the device: copies nodes and perm into outbuf (the caller keeps the host
// arrays alive until the stream has run) and packs the sorted triangles
cudaError_t lbvh_from_host(Lbvh &out, const float *tris, int n, const BvhNode *h_nodes,
                           const int *h_perm, char *outbuf, cudaStream_t st);
cudaError_t sphere_aabbs(const float *pos, int n, float r, float *aabb, cudaStream_t st);
