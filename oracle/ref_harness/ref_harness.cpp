// ref_harness.cpp -- runs the reference's own device programs
// (optixPathTracer.cu: raygen stage 1/2, closest-hit forward/backward, miss,
// sphere intersection) on the CPU, with a brute-force closest-hit traversal
// standing in for OptiX, and restates the host scheduler of
// optixPathTracer.cpp:93-360 around them.
//
// TEST INFRASTRUCTURE ONLY.  It is compiled by build_ref.py straight from the
// reference sources (never copied) into oracle/_ref/libams_ref.so, and used
// in this container to pin the C oracle and to generate the golden fixtures
// under tests/golden/.
//
// Stand-ins for closed code:
//   * OptiX triangle test -> watertight test of the C oracle
//     (orc_intersect_tri), same [1e-5, 1e16] interval.
//   * OptiX AABB gate in front of __intersection__sphere -> slab test of the C
//     oracle (orc_prim_slab).
//   * closest-hit ties: smaller t, then lower instance id, then lower
//     primitive index (OptiX leaves ties unspecified).
//   * at::unique_dim over int32 rows -> std::set of rows.
#include "optix.h"  // shim, first on the include path

#include "optixPathTracer.cu"  // the reference device programs, unmodified

#include <array>
#include <climits>
#include <map>
#include <set>
#include <vector>

#include "ams_oracle.h"

ShimState g_shim;

namespace {
struct Scene {
  const float *tris = nullptr;
  int n_tri = 0;
  const float *src_aabb = nullptr;  // [n_src, 6]
  const float *dst_aabb = nullptr;  // [n_dst, 6]
  int n_src = 0, n_dst = 0;
};
Scene g_scene;

struct Best {
  float t;
  int inst, prim;
  bool found;
};
Best g_best;

bool better(float t, int inst, int prim) {
  if (!g_best.found) return true;
  if (t < g_best.t) return true;
  if (t > g_best.t) return false;
  if (inst != g_best.inst) return inst < g_best.inst;
  return prim < g_best.prim;
}
}  // namespace

bool optixReportIntersection(float t, unsigned int) {
  if (!(t > g_shim.ray_tmin && t < g_shim.ray_tmax)) return false;
  if (better(t, g_shim.cur_inst, g_shim.cur_prim)) {
    g_best = {t, g_shim.cur_inst, g_shim.cur_prim, true};
    return true;
  }
  return false;
}

void optixTrace(OptixTraversableHandle, float3 o, float3 d, float tmin,
                float tmax, float, OptixVisibilityMask mask, unsigned int,
                unsigned int sbt_offset, unsigned int, unsigned int miss_index,
                unsigned int &u0, unsigned int &u1) {
  g_shim.payload0 = u0;
  g_shim.payload1 = u1;
  g_shim.ray_o = o;
  g_shim.ray_d = d;
  g_shim.ray_tmin = tmin;
  g_shim.ray_tmax = tmax;
  g_shim.in_closest_hit = false;
  g_best = {tmax, 3, INT_MAX, false};
  const float of[3] = {o.x, o.y, o.z}, df[3] = {d.x, d.y, d.z};
  if (mask & 1u) {
    for (int p = 0; p < g_scene.n_tri; p++) {
      const float *v = g_scene.tris + (size_t)p * 9;
      float t = orc_intersect_tri(of, df, v, v + 3, v + 6);
      if (t > 0.0f && better(t, 0, p)) g_best = {t, 0, p, true};
    }
  }
  for (int inst = 1; inst <= 2; inst++) {
    if (!(mask & (1u << inst))) continue;
    const float *box = inst == 1 ? g_scene.src_aabb : g_scene.dst_aabb;
    int n = inst == 1 ? g_scene.n_src : g_scene.n_dst;
    for (int p = 0; p < n; p++) {
      if (!orc_prim_slab(of, df, box + 6 * p, box + 6 * p + 3)) continue;
      g_shim.cur_prim = p;
      g_shim.cur_inst = inst;
      __intersection__sphere();
    }
  }
  if (g_best.found) {
    g_shim.hit_t = g_best.t;
    g_shim.hit_prim = g_best.prim;
    g_shim.hit_inst = g_best.inst;
    g_shim.in_closest_hit = true;
    if (sbt_offset == RAY_TYPE_FORWARD)
      __closesthit__forward();
    else
      __closesthit__backward();
    g_shim.in_closest_hit = false;
  } else {
    if (miss_index == RAY_TYPE_FORWARD)
      __miss__forward();
    else
      __miss__backward();
  }
}

namespace {
void run_launch(unsigned int nx, unsigned int ny) {
  g_shim.launch_dim = make_uint3(nx, ny, 1);
  for (unsigned int x = 0; x < nx; x++)
    for (unsigned int y = 0; y < ny; y++) {
      g_shim.launch_index = make_uint3(x, y, 0);
      __raygen__rg();
    }
}
}  // namespace

extern "C" {

// Equivalent of torch_launch_pathtrace (optixPathTracer.cpp:781-861) with the
// scheduler of launchSubframe (:93-360).  counts_out: [records, unique
// records, unique paths, rounds].  paths_out: the ordered path list, 14 words
// per path.
int ref_trace_channel(const float *tris, int n_tri, const int *mat,
                      const float *mat_prop, const float *src, int s0, int s1,
                      const float *dst, int n0_dst, int n1_dst,
                      const float *src_aabb, const float *dst_aabb,
                      int samples_per_launch, int launch_x, int launch_y,
                      double wave_len, int max_reflection, int reserve_size,
                      const float *src_dir, const float *dst_dir,
                      int src_bptype, int dst_bptype, int dst_gridsize,
                      double src_r, double dst_r, float *result,
                      unsigned long long *stats_out, long long *counts_out,
                      int32_t *paths_out, int max_paths) {
  Params &P = params;
  std::memset(&P, 0, sizeof(P));
  P.max_reflection = max_reflection;
  P.samples_per_launch = samples_per_launch;
  P.launch_x = launch_x;
  P.launch_y = launch_y;
  P.src_bptype = src_bptype;
  P.dst_bptype = dst_bptype;
  P.dst_gridsize = dst_gridsize;
  P.result = result;
  P.mat = const_cast<int *>(mat);
  P.mat_prop = const_cast<float *>(mat_prop);
  P.wave_len = (float)wave_len;
  P.src = (float3 *)src;
  P.dst = (float3 *)dst;
  P.scene_triangle_buffer = const_cast<float *>(tris);
  P.n_src = s0 * s1;
  P.n_dst = n0_dst * n1_dst;
  P.n0_dst = n0_dst;
  P.n1_dst = n1_dst;
  P.n0_dst_grid = (n0_dst - 1) / dst_gridsize + 1;
  P.n1_dst_grid = (n1_dst - 1) / dst_gridsize + 1;
  P.n_dst_grid = P.n0_dst_grid * P.n1_dst_grid;
  P.n_scene_triangle = n_tri;
  P.reserve_size = reserve_size;
  P.src_r = (float)src_r;
  P.dst_r = (float)dst_r;
  P.src_dir = make_float3(src_dir[0], src_dir[1], src_dir[2]);
  P.dst_dir = make_float3(dst_dir[0], dst_dir[1], dst_dir[2]);

  g_scene.tris = tris;
  g_scene.n_tri = n_tri;
  g_scene.src_aabb = src_aabb;
  g_scene.dst_aabb = dst_aabb;
  g_scene.n_src = P.n_src;
  g_scene.n_dst = P.n_dst;

  const long long n_launch = (long long)launch_x * launch_y;
  std::vector<ForwardRecord> tmp((size_t)(n_launch * reserve_size));
  std::vector<int> min_hc((size_t)(n_launch * P.n_dst_grid), 0);
  std::vector<int> counts((size_t)n_launch, 0);
  unsigned long long stats[2] = {0, 0};
  P.tmp_results = tmp.data();
  P.min_hc = min_hc.data();
  P.tmp_result_counts = counts.data();
  P.stats = stats;

  // stage 1
  P.stage = 1;
  run_launch((unsigned)launch_x, (unsigned)launch_y);

  std::vector<ForwardRecord> all;
  for (long long i = 0; i < n_launch; i++)
    for (int k = 0; k < counts[i]; k++) all.push_back(tmp[(size_t)(i * reserve_size + k)]);
  counts_out[0] = (long long)all.size();
  counts_out[1] = counts_out[2] = counts_out[3] = 0;
  if (all.empty()) {
    stats_out[0] = stats_out[1] = 0;
    return 0;  // "No path found!" (cpp:148-151)
  }
  // unique over the int32 view of the records (cpp:168-185)
  std::set<std::array<int32_t, 15>> rows;
  for (auto &r : all) {
    std::array<int32_t, 15> a;
    std::memcpy(a.data(), &r, 60);
    rows.insert(a);
  }
  std::vector<ForwardRecord> uniq;
  for (auto &a : rows) {
    ForwardRecord r;
    std::memcpy(&r, a.data(), 60);
    uniq.push_back(r);
  }
  counts_out[1] = (long long)uniq.size();

  // ordered path list (cpp:195-222)
  const int grid_num = P.n_dst_grid;
  std::map<Path, int> pathListInv;
  for (auto &r : uniq) pathListInv[r.path] = 0;
  std::vector<Path> pathList;
  for (auto it = pathListInv.begin(); it != pathListInv.end(); ++it) {
    it->second = (int)pathList.size();
    pathList.push_back(it->first);
  }
  counts_out[2] = (long long)pathList.size();
  for (int i = 0; i < (int)pathList.size() && i < max_paths; i++)
    std::memcpy(paths_out + 14 * i, &pathList[i], 56);
  P.pathList = pathList.data();

  // stage-2 rounds with 4-neighbour flood fill (cpp:229-354)
  P.stage = 2;
  std::vector<std::set<int>> tracedPath(grid_num);
  std::vector<std::vector<int>> gridTraceTasks(grid_num);
  std::vector<TraceTask> traceTasks;
  std::vector<unsigned char> success;
  int rounds = 0;
  for (int round = 1;; round++) {
    if (round == 1) {
      for (auto &r : uniq) {
        int task = pathListInv[r.path];
        gridTraceTasks[r.dst_grid_idx].push_back(task);
        tracedPath[r.dst_grid_idx].insert(task);
      }
    } else {
      bool goflag = false;
      for (int i = 0; i < grid_num; i++) gridTraceTasks[i].clear();
      for (size_t i = 0; i < traceTasks.size(); i++) {
        if (!success[i]) continue;
        int path_idx = traceTasks[i].path_idx;
        int g = traceTasks[i].dst_grid_idx;
        int nb[4] = {g - 1, g + 1, g - P.n1_dst_grid, g + P.n1_dst_grid};
        for (int n : nb) {
          if (n < 0 || n >= grid_num) continue;
          if (tracedPath[n].find(path_idx) == tracedPath[n].end()) {
            goflag = true;
            gridTraceTasks[n].push_back(path_idx);
            tracedPath[n].insert(path_idx);
          }
        }
      }
      if (!goflag) break;
    }
    traceTasks.clear();
    for (int g = 0; g < grid_num; g++)
      for (int path : gridTraceTasks[g]) traceTasks.push_back(TraceTask{path, g});
    int len = (int)traceTasks.size();
    success.assign((size_t)len, 0);
    static_assert(sizeof(bool) == 1, "bool flags");
    P.traceTasks = traceTasks.data();
    P.taskSuccess = reinterpret_cast<bool *>(success.data());
    P.traceTaskLen = len;
    int ideal = len * dst_gridsize * dst_gridsize;
    int threadNum = std::min(100000000 / P.n_src, ideal);
    run_launch((unsigned)P.n_src, (unsigned)threadNum);
    rounds++;
  }
  counts_out[3] = rounds;
  stats_out[0] = stats[0];
  stats_out[1] = stats[1];
  return 0;
}

// unit-level entry points of the reference helpers
uint32_t ref_tea4(uint32_t a, uint32_t b) { return tea<4>(a, b); }
float ref_rnd(uint32_t *seed) { return rnd(*seed); }
void ref_rand_dir(uint32_t *seed, uint32_t ix, uint32_t iy, int lx, int ly,
                  float *out) {
  params.launch_x = lx;
  params.launch_y = ly;
  float3 d = rand_dir(*seed, ix, iy);
  out[0] = d.x;
  out[1] = d.y;
  out[2] = d.z;
}
float ref_beampattern(const float *a, const float *b, int type) {
  return get_beampattern_factor(make_float3(a[0], a[1], a[2]),
                                make_float3(b[0], b[1], b[2]), type);
}
void ref_image_update(float *m12, const float *n, const float *a) {
  sutil::Matrix3x4 M;
  std::memcpy(M.getData(), m12, 48);
  updateImageTransform(M, make_float3(n[0], n[1], n[2]),
                       make_float3(a[0], a[1], a[2]));
  std::memcpy(m12, M.getData(), 48);
}
int ref_theta_id(float cos_theta) {
  float theta = acosf(fabsf(cos_theta));
  return (int)((theta / (M_PIf / 2) * 36 + 1) / 2);
}

}  // extern "C"
