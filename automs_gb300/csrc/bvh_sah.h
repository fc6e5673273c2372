// bvh_sah.h -- binned-SAH hierarchy over scene triangles, built on the host.
#pragma once
#include <vector>

#include "lbvh.h"

// Scenes with at least this many triangles get the SAH hierarchy; smaller
// ones the GPU LBVH (the two trace equally fast there, and the LBVH needs no
// host round trip).
#define AMS_SAH_MIN_TRIS 16384

// Builds the hierarchy of n triangles (host array [n][9]) in the node format
// of lbvh.h: nodes[0 .. n-2] with the root at 0, child < 0 = leaf of sorted
// primitive ~child, child boxes widened outward; perm[sorted] = original
// index.  Returns false (with a message) if the tree fails its own checks.
bool sah_build_triangles(const float *tris, int n, std::vector<BvhNode> &nodes,
                         std::vector<int> &perm, char *msg, size_t msglen);
