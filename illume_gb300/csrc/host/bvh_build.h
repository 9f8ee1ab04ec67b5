// BVH construction for one mesh (object space).
//
// * Binned SAH binary build (16 bins per axis on centroids).
// * Binary layout (Bvh2Node, 64 B): both child boxes live in the parent node.
// * 4-wide layout (Bvh4Node, 128 B): the binary tree (leaves of up to 4 triangles)
//   collapsed into nodes of up to 4 children chosen by a dynamic program that minimises
//   the summed box area of the 4-wide nodes; it shares the binary layout's triangle
//   records.
// * 8-wide layout (WideNode, 80 B): the binary tree (leaves of up to 3 triangles)
//   collapsed into nodes of up to 8 children by the same dynamic program, child slots
//   ordered by ray octant, child boxes quantised to 8 bits per axis with outward rounding.
// Triangle boxes are padded by a small absolute margin before building, so that a box
// test evaluated in FP32 never rejects a ray whose FP32 triangle test reports a hit
// (for ray origins within ~100x the mesh extent); quantisation only widens boxes.
#pragma once

#include <stdint.h>
#include <string>
#include <vector>

#include "../common/types.h"

namespace illume {

struct BuildStats {
  int bvh2_nodes = 0, bvh2_leaves = 0, bvh2_depth = 0;
  int wide_nodes = 0, wide_leaves = 0, wide_depth = 0;
  int bvh4_nodes = 0, bvh4_depth = 0;
  double sah_cost = 0.0;
  int device_built = 0;          // 1: the binary tree came from the device build
  int device_rounds = 0;         // its clustering rounds
  double device_ms = 0.0;        // and the wall time of its device part
  std::string device_fallback;   // why a requested device build fell back to the host build
};

struct MeshBvh {
  std::vector<Bvh4Node> bvh4;      // 4-wide layout over bvh2_tris
  std::vector<Bvh2Node> bvh2;
  std::vector<float4> bvh2_tris;   // 3 float4 per triangle in leaf order, .w of the first = prim id
  std::vector<WideNode> wide;
  std::vector<float4> wide_tris;
  bool root_leaf = false;
  bool has_wide = false;           // the 8-wide layout is built (on first need, Scene::ensure_wide)
  float lo[3], hi[3];              // padded object-space bounds of the mesh
  BuildStats stats;
};

// Layouts of build_mesh_bvh: the binary and 4-wide layouts (one tree, shared triangle
// records), the 8-wide quantised layout (its own tree, leaves of up to 3 triangles).
enum BuildLayouts { kLayoutBinary4 = 1, kLayoutWide = 2, kLayoutAll = 3 };

// Host threads of a BVH build: ILLUME_BUILD_THREADS if set (>= 1), else the cores (at
// most 16), unless the calling thread holds a share set by BuildThreadShare. The result
// does not depend on it.
int build_threads();

// While alive, build_threads() on this thread returns `share` (>= 1): for builds that
// run beside other builds on the same cores (one mesh per thread), so that their own
// parallel passes do not oversubscribe the cores.
class BuildThreadShare {
 public:
  explicit BuildThreadShare(int share);
  ~BuildThreadShare();
  BuildThreadShare(const BuildThreadShare&) = delete;
  BuildThreadShare& operator=(const BuildThreadShare&) = delete;

 private:
  int saved_;
};

// The share of each of the builds that run together on `builders` threads: all cores
// when at most one of `sizes` (triangles per mesh) is large enough to use more than one
// thread, else the cores divided among the builders.
int build_thread_share(const int* sizes, int count, int builders);

struct Context;

// positions: 3 floats per vertex; tris: 3 ints per triangle. With `device`, the binary
// tree is built on that context's GPU by locally-ordered clustering (bvh_device.h) and
// turned into leaves here; a device build that fails, or whose tree is deeper than the
// traversal stacks allow, is replaced by the host build (stats.device_fallback says why).
// `layouts` (BuildLayouts) selects what is built; a call for kLayoutWide alone fills only
// the 8-wide arrays and statistics of `out` (host build).
void build_mesh_bvh(const float* positions, int num_vertices, const int* tris, int num_tris, MeshBvh* out,
                    Context* device = nullptr, int layouts = kLayoutAll);

// Invariants of the built layouts (the 8-wide one when has_wide): every triangle
// referenced exactly once, every triangle inside its leaf box, every inner child box
// inside its parent's box, quantised boxes (decoded exactly) containing their contents.
// Returns false with a message on failure.
bool check_mesh_bvh(const float* positions, const int* tris, int num_tris, const MeshBvh& b, std::string* msg);

}  // namespace illume
