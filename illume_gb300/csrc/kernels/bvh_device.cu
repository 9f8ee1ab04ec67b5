// Device BVH build by locally-ordered clustering (see bvh_device.h).
#include "bvh_device.h"

#include <algorithm>
#include <chrono>
#include <cstdint>

#include "../host/runtime.h"

namespace illume {

namespace {

constexpr int kRadius = 16;            // clustering window: 16 positions either side
constexpr int kNNThreads = 256;
constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;          // keys per thread per tile
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kScanThreads = 256;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

// float <-> unsigned with the same order (for atomicMin / atomicMax on floats)
__device__ __forceinline__ unsigned order_bits(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float from_order_bits(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

// bounds[0..2] = min of the centroids (order bits), bounds[3..5] = max
__global__ void __launch_bounds__(256) k_centroid_bounds(const float* box, int n, unsigned* bounds) {
  float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    for (int a = 0; a < 3; ++a) {
      const float c = 0.5f * (box[6 * (size_t)i + a] + box[6 * (size_t)i + 3 + a]);
      lo[a] = fminf(lo[a], c);
      hi[a] = fmaxf(hi[a], c);
    }
  }
  for (int off = 16; off > 0; off >>= 1)
    for (int a = 0; a < 3; ++a) {
      lo[a] = fminf(lo[a], __shfl_down_sync(0xffffffffu, lo[a], off));
      hi[a] = fmaxf(hi[a], __shfl_down_sync(0xffffffffu, hi[a], off));
    }
  if ((threadIdx.x & 31) == 0)
    for (int a = 0; a < 3; ++a) {
      atomicMin(bounds + a, order_bits(lo[a]));
      atomicMax(bounds + 3 + a, order_bits(hi[a]));
    }
}

// 10 bits of x spread to every third bit
__device__ __forceinline__ unsigned spread3(unsigned x) {
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000ffu;
  x = (x | (x << 8)) & 0x0300f00fu;
  x = (x | (x << 4)) & 0x030c30c3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

__global__ void __launch_bounds__(256) k_morton(const float* box, int n, const unsigned* bounds, unsigned* keys,
                                                int* vals) {
  float lo[3], ext[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = from_order_bits(bounds[a]);
    const float e = from_order_bits(bounds[3 + a]) - lo[a];
    ext[a] = e > 0.0f ? e : 1.0f;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    unsigned q[3];
    for (int a = 0; a < 3; ++a) {
      const float c = 0.5f * (box[6 * (size_t)i + a] + box[6 * (size_t)i + 3 + a]);
      const float u = (c - lo[a]) / ext[a] * 1024.0f;
      q[a] = (unsigned)min(1023, max(0, (int)u));
    }
    keys[i] = (spread3(q[0]) << 2) | (spread3(q[1]) << 1) | spread3(q[2]);
    vals[i] = i;
  }
}

// ---- stable LSD radix sort of (key, value) pairs, 4 bits per pass ----
// counts[d * tiles + t] = keys of tile t whose digit is d
__global__ void __launch_bounds__(kSortThreads) k_radix_count(const unsigned* keys, int n, int shift, int tiles,
                                                              int* counts) {
  __shared__ int cnt[16];
  const int t = blockIdx.x;
  if (threadIdx.x < 16) cnt[threadIdx.x] = 0;
  __syncthreads();
  for (int j = 0; j < kSortItems; ++j) {
    const int l = t * kSortTile + j * kSortThreads + threadIdx.x;
    if (l < n) atomicAdd(&cnt[(keys[l] >> shift) & 15u], 1);
  }
  __syncthreads();
  if (threadIdx.x < 16) counts[threadIdx.x * tiles + t] = cnt[threadIdx.x];
}

// offsets: exclusive scan of counts (digit-major), so that the keys of digit d in tile t
// start at offsets[d * tiles + t]; within a tile keys keep their order (warps in order,
// lanes in order), which makes every pass stable
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const unsigned* kin, const int* vin, unsigned* kout,
                                                                int* vout, int n, int shift, int tiles,
                                                                const int* offsets) {
  constexpr int kWarps = kSortThreads / 32;
  __shared__ int run[16];
  __shared__ int wcnt[kWarps][16];
  const int t = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x < 16) run[threadIdx.x] = offsets[threadIdx.x * tiles + t];
  __syncthreads();
  for (int j = 0; j < kSortItems; ++j) {
    const int l = t * kSortTile + j * kSortThreads + threadIdx.x;
    const bool valid = l < n;
    const unsigned key = valid ? kin[l] : 0u;
    const int val = valid ? vin[l] : 0;
    const int d = valid ? (int)((key >> shift) & 15u) : 16;
    int rank = 0;
    for (int dd = 0; dd < 16; ++dd) {
      const unsigned m = __ballot_sync(0xffffffffu, d == dd);
      if (d == dd) rank = __popc(m & ((1u << lane) - 1u));
      if (lane == 0) wcnt[warp][dd] = __popc(m);
    }
    __syncthreads();
    if (valid) {
      int base = run[d];
      for (int w = 0; w < warp; ++w) base += wcnt[w][d];
      kout[base + rank] = key;
      vout[base + rank] = val;
    }
    __syncthreads();
    if (threadIdx.x < 16) {
      int s = 0;
      for (int w = 0; w < kWarps; ++w) s += wcnt[w][threadIdx.x];
      run[threadIdx.x] += s;
    }
    __syncthreads();
  }
}

// ---- exclusive scan of ints; out[n] receives the total ----
__global__ void __launch_bounds__(kScanThreads) k_scan_tile(const int* in, int* out, int n, int* tile_sums) {
  __shared__ int wsum[kScanThreads / 32];
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems], s = 0;
  for (int q = 0; q < kScanItems; ++q) {
    v[q] = base + q < n ? in[base + q] : 0;
    s += v[q];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int inc = s;
  for (int off = 1; off < 32; off <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, inc, off);
    if (lane >= off) inc += y;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  int before = 0;
  for (int w = 0; w < warp; ++w) before += wsum[w];
  int run = before + inc - s;
  for (int q = 0; q < kScanItems; ++q) {
    if (base + q < n) out[base + q] = run;
    run += v[q];
  }
  if (threadIdx.x == kScanThreads - 1) tile_sums[blockIdx.x] = before + inc;
}

// one block: exclusive scan of the tile sums in place; sums[tiles] = total
__global__ void __launch_bounds__(1024) k_scan_sums(int* sums, int tiles) {
  __shared__ int wsum[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int base = 0; base < tiles; base += 1024) {
    const int i = base + threadIdx.x;
    const int v = i < tiles ? sums[i] : 0;
    int inc = v;
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, inc, off);
      if (lane >= off) inc += y;
    }
    if (lane == 31) wsum[warp] = inc;
    __syncthreads();
    int before = 0;
    for (int w = 0; w < warp; ++w) before += wsum[w];
    const int c = carry;
    if (i < tiles) sums[i] = c + before + inc - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry = c + before + inc;
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[tiles] = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_add(int* out, int n, const int* tile_sums, int tiles) {
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  const int add = tile_sums[blockIdx.x];
  for (int q = 0; q < kScanItems; ++q)
    if (base + q < n) out[base + q] += add;
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = tile_sums[tiles];
}

// ---- clustering ----
__global__ void __launch_bounds__(256) k_leaves(const float* box, const int* sorted, int n, float* node_box,
                                                int* clusters) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int p = sorted[k];
    for (int a = 0; a < 6; ++a) node_box[6 * (size_t)k + a] = box[6 * (size_t)p + a];
    clusters[k] = k;
  }
}

__device__ __forceinline__ float merged_area(const float* a, const float* b) {
  const float dx = fmaxf(a[3], b[3]) - fminf(a[0], b[0]);
  const float dy = fmaxf(a[4], b[4]) - fminf(a[1], b[1]);
  const float dz = fmaxf(a[5], b[5]) - fminf(a[2], b[2]);
  return dx * dy + dy * dz + dz * dx;
}

// nn[i] = the position j != i within kRadius of i whose merged box with i has the least
// surface area (the lowest such j on ties); -1 when i is the only cluster
__global__ void __launch_bounds__(kNNThreads) k_nearest(const int* clusters, int nc, const float* node_box, int* nn) {
  __shared__ float tile[(kNNThreads + 2 * kRadius) * 6];
  const int first = blockIdx.x * kNNThreads - kRadius;
  for (int s = threadIdx.x; s < kNNThreads + 2 * kRadius; s += kNNThreads) {
    const int j = first + s;
    if (j >= 0 && j < nc) {
      const int node = clusters[j];
      for (int a = 0; a < 6; ++a) tile[6 * s + a] = node_box[6 * (size_t)node + a];
    }
  }
  __syncthreads();
  const int i = blockIdx.x * kNNThreads + threadIdx.x;
  if (i >= nc) return;
  const float* me = tile + 6 * (threadIdx.x + kRadius);
  float best = INFINITY;
  int bj = -1;
  const int lo = max(0, i - kRadius), hi = min(nc - 1, i + kRadius);
  for (int j = lo; j <= hi; ++j) {
    if (j == i) continue;
    const float a = merged_area(me, tile + 6 * (j - first));
    if (a < best || bj < 0) {
      best = a;
      bj = j;
    }
  }
  nn[i] = bj;
}

__global__ void __launch_bounds__(256) k_pair_flags(const int* nn, int nc, int* merge, int* keep) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
    const int j = nn[i];
    const bool mutual = j >= 0 && j < nc && nn[j] == i;
    merge[i] = mutual && i < j;
    keep[i] = !(mutual && i > j);
  }
}

// merged pairs become new nodes numbered from next_node in position order; the kept
// clusters (merged nodes at their lower position) are compacted in order
__global__ void __launch_bounds__(256) k_merge(const int* clusters, int nc, const int* nn, const int* merge,
                                               const int* merge_off, const int* keep, const int* keep_off, int n,
                                               int next_node, float* node_box, int* child, int* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x) {
    if (!keep[i]) continue;
    if (merge[i]) {
      const int id = next_node + merge_off[i];
      const int a = clusters[i], b = clusters[nn[i]];
      child[2 * (size_t)(id - n)] = a;
      child[2 * (size_t)(id - n) + 1] = b;
      for (int k = 0; k < 3; ++k) {
        node_box[6 * (size_t)id + k] = fminf(node_box[6 * (size_t)a + k], node_box[6 * (size_t)b + k]);
        node_box[6 * (size_t)id + 3 + k] = fmaxf(node_box[6 * (size_t)a + 3 + k], node_box[6 * (size_t)b + 3 + k]);
      }
      out[keep_off[i]] = id;
    } else {
      out[keep_off[i]] = clusters[i];
    }
  }
}

int grid_for(int n, int threads) { return std::max(1, std::min((n + threads - 1) / threads, 4096)); }

// exclusive scan of in[0..n) into out[0..n], out[n] = total; sums: (n + tile - 1) / tile + 1 ints
void exclusive_scan(const int* in, int* out, int n, int* sums, cudaStream_t st) {
  const int tiles = (n + kScanTile - 1) / kScanTile;
  k_scan_tile<<<tiles, kScanThreads, 0, st>>>(in, out, n, sums);
  k_scan_sums<<<1, 1024, 0, st>>>(sums, tiles);
  k_scan_add<<<tiles, kScanThreads, 0, st>>>(out, n, sums, tiles);
}

}  // namespace

int build_cluster_tree_device(Context* ctx, const float* boxes6, int n, ClusterTree* out, std::string* err) {
  if (n < 1) { *err = "no primitives"; return ILLUME_ERR_INVALID; }
  if (n > (1 << 28)) { *err = "too many primitives for the device build"; return ILLUME_ERR_UNSUPPORTED; }
  ILLUME_CUDA_TRY(cudaSetDevice(ctx->device));
  struct Stream {
    cudaStream_t s = nullptr;
    ~Stream() { if (s) cudaStreamDestroy(s); }
  } stream;
  ILLUME_CUDA_TRY(cudaStreamCreateWithFlags(&stream.s, cudaStreamNonBlocking));
  cudaStream_t st = stream.s;
  const auto t0 = std::chrono::steady_clock::now();
  const int nodes = 2 * n - 1;
  const int sort_tiles = (n + kSortTile - 1) / kSortTile;
  const int count_len = 16 * sort_tiles;
  const int scan_len = std::max(count_len, n);
  const int scan_sums = (scan_len + kScanTile - 1) / kScanTile + 1;
  DevBuffer d_box, d_bounds, d_keys[2], d_vals[2], d_counts, d_offsets, d_sums, d_node_box, d_child, d_clusters[2],
      d_nn, d_merge, d_keep, d_merge_off, d_keep_off;
  int s;
#define ALLOC(buf, bytes) if ((s = (buf).alloc(ctx, (bytes))) != ILLUME_OK) { *err = last_error(); return s; }
  ALLOC(d_box, sizeof(float) * 6 * (size_t)n);
  ALLOC(d_bounds, sizeof(unsigned) * 6);
  for (int k = 0; k < 2; ++k) {
    ALLOC(d_keys[k], sizeof(unsigned) * (size_t)n);
    ALLOC(d_vals[k], sizeof(int) * (size_t)n);
    ALLOC(d_clusters[k], sizeof(int) * (size_t)n);
  }
  ALLOC(d_counts, sizeof(int) * (size_t)count_len);
  ALLOC(d_offsets, sizeof(int) * ((size_t)count_len + 1));
  ALLOC(d_sums, sizeof(int) * (size_t)scan_sums);
  ALLOC(d_node_box, sizeof(float) * 6 * (size_t)nodes);
  ALLOC(d_child, sizeof(int) * 2 * (size_t)std::max(1, n - 1));
  ALLOC(d_nn, sizeof(int) * (size_t)n);
  ALLOC(d_merge, sizeof(int) * (size_t)n);
  ALLOC(d_keep, sizeof(int) * (size_t)n);
  ALLOC(d_merge_off, sizeof(int) * ((size_t)n + 1));
  ALLOC(d_keep_off, sizeof(int) * ((size_t)n + 1));
#undef ALLOC
  // every return below waits for the stream first, so no launch of this build is still
  // in flight when its buffers are released (declared after them: destroyed before them)
  struct Drain {
    cudaStream_t s;
    ~Drain() { cudaStreamSynchronize(s); }
  } drain{st};
  ILLUME_CUDA_TRY(cudaMemcpyAsync(d_box.get(), boxes6, sizeof(float) * 6 * (size_t)n, cudaMemcpyHostToDevice, st));
  const unsigned init[6] = {0xffffffffu, 0xffffffffu, 0xffffffffu, 0u, 0u, 0u};
  ILLUME_CUDA_TRY(cudaMemcpyAsync(d_bounds.get(), init, sizeof(init), cudaMemcpyHostToDevice, st));
  k_centroid_bounds<<<grid_for(n, 256), 256, 0, st>>>(d_box.as<float>(), n, d_bounds.as<unsigned>());
  k_morton<<<grid_for(n, 256), 256, 0, st>>>(d_box.as<float>(), n, d_bounds.as<unsigned>(), d_keys[0].as<unsigned>(),
                                           d_vals[0].as<int>());
  for (int pass = 0; pass < 8; ++pass) {
    const int a = pass & 1, b = a ^ 1;
    k_radix_count<<<sort_tiles, kSortThreads, 0, st>>>(d_keys[a].as<unsigned>(), n, 4 * pass, sort_tiles,
                                                       d_counts.as<int>());
    exclusive_scan(d_counts.as<int>(), d_offsets.as<int>(), count_len, d_sums.as<int>(), st);
    k_radix_scatter<<<sort_tiles, kSortThreads, 0, st>>>(d_keys[a].as<unsigned>(), d_vals[a].as<int>(),
                                                         d_keys[b].as<unsigned>(), d_vals[b].as<int>(), n, 4 * pass,
                                                         sort_tiles, d_offsets.as<int>());
  }
  // eight passes: the sorted pairs are back in buffer 0
  k_leaves<<<grid_for(n, 256), 256, 0, st>>>(d_box.as<float>(), d_vals[0].as<int>(), n, d_node_box.as<float>(),
                                             d_clusters[0].as<int>());
  ILLUME_CUDA_TRY(cudaGetLastError());
  int nc = n, next_node = n, cur = 0, iterations = 0;
  const int max_iterations = 4096;
  while (nc > 1) {
    if (++iterations > max_iterations) {
      *err = "device BVH build: clustering did not finish";
      return ILLUME_ERR_UNSUPPORTED;
    }
    const int* cl = d_clusters[cur].as<int>();
    k_nearest<<<(nc + kNNThreads - 1) / kNNThreads, kNNThreads, 0, st>>>(cl, nc, d_node_box.as<float>(),
                                                                         d_nn.as<int>());
    k_pair_flags<<<grid_for(nc, 256), 256, 0, st>>>(d_nn.as<int>(), nc, d_merge.as<int>(), d_keep.as<int>());
    exclusive_scan(d_merge.as<int>(), d_merge_off.as<int>(), nc, d_sums.as<int>(), st);
    exclusive_scan(d_keep.as<int>(), d_keep_off.as<int>(), nc, d_sums.as<int>(), st);
    int totals[2] = {0, 0};
    ILLUME_CUDA_TRY(cudaMemcpyAsync(totals, d_merge_off.as<int>() + nc, sizeof(int), cudaMemcpyDeviceToHost, st));
    ILLUME_CUDA_TRY(cudaMemcpyAsync(totals + 1, d_keep_off.as<int>() + nc, sizeof(int), cudaMemcpyDeviceToHost, st));
    ILLUME_CUDA_TRY(cudaStreamSynchronize(st));
    const int merges = totals[0], kept = totals[1];
    if (merges < 1 || merges + kept != nc || next_node + merges > nodes) {
      *err = "device BVH build: a clustering round merged no pair";
      return ILLUME_ERR_UNSUPPORTED;
    }
    k_merge<<<grid_for(nc, 256), 256, 0, st>>>(cl, nc, d_nn.as<int>(), d_merge.as<int>(), d_merge_off.as<int>(),
                                               d_keep.as<int>(), d_keep_off.as<int>(), n, next_node,
                                               d_node_box.as<float>(), d_child.as<int>(),
                                               d_clusters[cur ^ 1].as<int>());
    ILLUME_CUDA_TRY(cudaGetLastError());
    next_node += merges;
    nc = kept;
    cur ^= 1;
  }
  if (next_node != nodes) {
    *err = "device BVH build: the tree does not hold every primitive";
    return ILLUME_ERR_UNSUPPORTED;
  }
  out->n = n;
  out->iterations = iterations;
  out->prim.resize(n);
  out->box.resize(6 * (size_t)nodes);
  out->child.resize(2 * (size_t)(n - 1));
  ILLUME_CUDA_TRY(cudaMemcpyAsync(out->prim.data(), d_vals[0].get(), sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost,
                                  st));
  ILLUME_CUDA_TRY(cudaMemcpyAsync(out->box.data(), d_node_box.get(), sizeof(float) * 6 * (size_t)nodes,
                                  cudaMemcpyDeviceToHost, st));
  if (n > 1)
    ILLUME_CUDA_TRY(cudaMemcpyAsync(out->child.data(), d_child.get(), sizeof(int) * 2 * (size_t)(n - 1),
                                    cudaMemcpyDeviceToHost, st));
  ILLUME_CUDA_TRY(cudaMemcpyAsync(&out->root, d_clusters[cur].get(), sizeof(int), cudaMemcpyDeviceToHost, st));
  ILLUME_CUDA_TRY(cudaStreamSynchronize(st));
  out->device_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return ILLUME_OK;
}

}  // namespace illume
