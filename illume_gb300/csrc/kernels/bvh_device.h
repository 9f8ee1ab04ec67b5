// Scene ingest on the device: a binary BVH over a mesh's triangle boxes built on the GPU
// by locally-ordered clustering (PLOC: D. Meister and J. Bittner, "Parallel
// Locally-Ordered Clustering for Bounding Volume Hierarchy Construction", IEEE TVCG
// 2018). The primitives are sorted by the 30-bit Morton code of their box centroids;
// then, until one cluster is left, every cluster finds the cluster within 16 positions
// of it whose merged box has the smallest surface area, mutual nearest neighbours merge
// into a new node, and the cluster list is compacted in order.
//
// No counterpart in the reference, whose tree is built on one host thread by a
// 1024-step sweep per level (src/accel/bvh.cpp:65-249, 362-395); any tree gives the
// same closest hits, since hits are decided by the triangle tests and ties go to the
// lower primitive index. The host turns the cluster tree into leaves and node layouts
// (bvh_build.cpp).
#pragma once

#include <string>
#include <vector>

namespace illume {

struct Context;

struct ClusterTree {
  int n = 0;                 // primitives; leaf node k (0 <= k < n) holds primitive prim[k]
  std::vector<int> prim;     // n
  std::vector<float> box;    // 6 floats per node (lo x, y, z, hi x, y, z), 2n - 1 nodes
  std::vector<int> child;    // inner node n + j has children child[2j], child[2j + 1]
  int root = 0;              // inner nodes are numbered after their children
  int iterations = 0;        // clustering rounds
  double device_ms = 0.0;    // wall time of the device part (upload, sort, clustering, download)
};

// boxes6: 6 floats per primitive (lo x, y, z, hi x, y, z). Runs on the context's device
// on a stream of its own and waits for it. Returns ILLUME_OK, or an error status with a
// message (device memory, or a clustering round that merged nothing).
int build_cluster_tree_device(Context* ctx, const float* boxes6, int n, ClusterTree* out, std::string* err);

}  // namespace illume
