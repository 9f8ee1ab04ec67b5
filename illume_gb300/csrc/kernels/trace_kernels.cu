// Closest-hit kernels: the wavefront trace stage and the trace test hook.
#include <type_traits>

#include "launch.h"
#include "trace.cuh"
#include "../common/philox.cuh"
#include "../../../include/illume.h"

namespace illume {

__device__ __forceinline__ int* ev_counts(const WaveBuffers& w, int parity) { return w.counters + 2 + 16 * parity; }

// Warp-aggregated append: lanes of `mask` that pass the same `key` share one atomic.
__device__ __forceinline__ int warp_append_keyed(unsigned mask, int key, int* counters) {
  const unsigned peers = __match_any_sync(mask, key);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counters + key, __popc(peers));
  base = __shfl_sync(peers, base, leader);
  return base + __popc(peers & ((1u << lane) - 1));
}

// Trace stage of one bounce: closest hit of every queued ray, then the event class
// (escape, medium scatter before the surface, or the hit material) and an append of the
// ray's slot to that class's queue. The medium decision uses the first number of the
// path's bounce stream, as src/renderer.cu:152-157 does.
template <int KIND, bool COUNT>
__global__ void __launch_bounds__(128) k_trace(WaveBuffers w, SceneView sc, RenderKnobs k, int bounce) {
  const int parity = bounce & 1;
  const int n = w.counters[parity];
  if (blockIdx.x == 0 && threadIdx.x == 0) w.counters[parity ^ 1] = 0;
  int* counts = ev_counts(w, parity);
  const int sample_base = w.pass->sample_base;
  typename std::conditional<KIND == BVH_WIDE8, uint2, int>::type stack[kStack];
  unsigned long long my_nodes = 0, my_tris = 0;
  for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const int i = base + threadIdx.x;
    const bool valid = i < n;
    const unsigned mask = __ballot_sync(0xffffffffu, valid);
    if (!valid) continue;
    const float4 qo = w.q_orig[parity][i];
    const float4 qd = w.q_dir[parity][i];
    VisitCount vc;
    const HitRecord h = closest_hit<KIND, COUNT>(sc, v3(qo.x, qo.y, qo.z), v3(qd.x, qd.y, qd.z), k.isect, stack, &vc);
    if (COUNT) { my_nodes += vc.nodes; my_tris += vc.tris; }
    int cls;
    const int medium = __float_as_int(qd.w);
    bool scattered = false;
    if (medium >= 0 && sc.mediums[medium].active) {
      const int pid = __float_as_int(qo.w);
      const uint32_t pixel = (uint32_t)(pid % w.npix), sample = (uint32_t)(sample_base + pid / w.npix);
      const Philox4 r = philox4x32_10(pixel, sample, (uint32_t)(bounce + 1), 0u, k.seed, k.job);
      const float u = philox_unit(r.x);
      const float dist = -logf(u) / sc.mediums[medium].scattering;
      scattered = dist < h.t;
    }
    if (scattered) cls = EV_MEDIUM;
    else if (h.geom == -1) cls = EV_MISS;
    else {
      const int mat = h.geom >= 0 ? sc.instances[h.geom].material : sc.spheres[-2 - h.geom].material;
      cls = EV_SURFACE + sc.materials[mat].type;
    }
    w.hit[i] = make_float4(h.t, h.u, h.v, __int_as_float(h.prim));
    w.hit_geom[i] = h.geom;
    const int pos = warp_append_keyed(mask, cls, counts);
    w.evq[(size_t)cls * w.cap + pos] = i;
  }
  if (COUNT) {
    for (int off = 16; off > 0; off >>= 1) {
      my_nodes += __shfl_down_sync(0xffffffffu, my_nodes, off);
      my_tris += __shfl_down_sync(0xffffffffu, my_tris, off);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(w.visits, my_nodes);
      atomicAdd(w.visits + 1, my_tris);
    }
  }
}

template <int KIND>
__global__ void __launch_bounds__(128) k_trace_hook(SceneView sc, const float4* rays, int n, int isect,
                                                    illume_hit* out) {
  typename std::conditional<KIND == BVH_WIDE8, uint2, int>::type stack[kStack];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 a = rays[2 * i], b = rays[2 * i + 1];
    const HitRecord h = closest_hit<KIND>(sc, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), isect, stack);
    illume_hit o;
    o.t = h.t;
    o.u = h.geom >= 0 ? h.u : 0.0f;
    o.v = h.geom >= 0 ? h.v : 0.0f;
    o.inst = h.geom >= 0 ? h.geom : -1;
    o.prim = h.geom >= 0 ? h.prim : -1;
    o.sphere = h.geom <= -2 ? -2 - h.geom : -1;
    o.pad[0] = o.pad[1] = 0;
    out[i] = o;
  }
}

const void* trace_kernel_ptr(int bvh_kind) {
  return bvh_kind == BVH_WIDE8 ? (const void*)k_trace<BVH_WIDE8, false> : (const void*)k_trace<BVH_BINARY, false>;
}

void launch_trace(const WaveBuffers& w, const SceneView& sc, const RenderKnobs& k, int bounce, int grid,
                  cudaStream_t st, bool count_visits) {
  if (count_visits) {
    if (k.bvh_kind == BVH_WIDE8) k_trace<BVH_WIDE8, true><<<grid, 128, 0, st>>>(w, sc, k, bounce);
    else k_trace<BVH_BINARY, true><<<grid, 128, 0, st>>>(w, sc, k, bounce);
    return;
  }
  if (k.bvh_kind == BVH_WIDE8) k_trace<BVH_WIDE8, false><<<grid, 128, 0, st>>>(w, sc, k, bounce);
  else k_trace<BVH_BINARY, false><<<grid, 128, 0, st>>>(w, sc, k, bounce);
}

void launch_trace_hook(const SceneView& sc, const float* rays8, int n, int isect, int bvh_kind, void* hits,
                       cudaStream_t st) {
  if (n <= 0) return;
  const int grid = (n + 127) / 128;
  if (bvh_kind == BVH_WIDE8)
    k_trace_hook<BVH_WIDE8><<<grid, 128, 0, st>>>(sc, (const float4*)rays8, n, isect, (illume_hit*)hits);
  else
    k_trace_hook<BVH_BINARY><<<grid, 128, 0, st>>>(sc, (const float4*)rays8, n, isect, (illume_hit*)hits);
}

int kernel_grid_blocks(const void* fn, int block, int device) {
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, 0);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

}  // namespace illume
