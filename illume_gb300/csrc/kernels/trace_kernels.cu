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

// Event class of a traced ray: escape, medium scatter before the surface, or the hit
// material. The medium decision uses the first number of the path's bounce stream, as
// src/renderer.cu:152-157 does.
__device__ __forceinline__ int event_class(const WaveBuffers& w, const JobDesc& J, const SceneView& sc,
                                           const HitRecord& h, int g, int medium, int bounce) {
  if (medium >= 0 && sc.mediums[medium].active) {
    const int pid = g - J.path_base;
    const uint32_t pixel = (uint32_t)(pid % J.npix), sample = (uint32_t)(J.sample_base + pid / J.npix);
    const Philox4 r = philox4x32_10(pixel, sample, (uint32_t)(bounce + 1), 0u, J.seed, J.job);
    const float dist = -logf(philox_unit(r.x)) / sc.mediums[medium].scattering;
    if (dist < h.t) return EV_MEDIUM;
  }
  if (h.geom == -1) return EV_MISS;
  const int mat = h.geom >= 0 ? sc.instances[h.geom].material : sc.spheres[-2 - h.geom].material;
  return EV_SURFACE + sc.materials[mat].type;
}

// Trace stage of one bounce: closest hit of every queued ray in its job's scene, then
// an append of the ray's queue position to its event class's queue.
// OPT: box tests in fused multiply-add form, and warps take their next 32 rays from a
// shared counter (counters[44 + parity]) instead of a fixed grid stride, so that warps
// whose rays finish early take over the remaining work.
// PS, NF (4-wide only): see traverse_bvh4_ww.
template <int KIND, bool COUNT, int MINB = 1, bool OPT = false, bool WW = false, bool PS = false, bool NF = false,
          bool FR = false, bool SI = false>
__global__ void __launch_bounds__(128, MINB) k_trace(WaveBuffers w, RenderKnobs k, int bounce) {
  const int it = pass_iteration(w, bounce);
  const int parity = it & 1;
  const int n = w.counters[parity];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    w.counters[parity ^ 1] = 0;
    w.counters[44 + (parity ^ 1)] = 0;
  }
  int* counts = ev_counts(w, parity);
  int* fetch = w.counters + 44 + parity;
  const int lane = threadIdx.x & 31;
  typename std::conditional<KIND == BVH_WIDE8, uint2, int>::type stack[kStack];
  unsigned long long my_nodes = 0, my_tris = 0, my_slots = 0;
  int base = OPT ? 0 : blockIdx.x * blockDim.x + (threadIdx.x & ~31);
  for (;;) {
    if (OPT) {
      int b0 = 0;
      if (lane == 0) b0 = atomicAdd(fetch, 32);
      base = __shfl_sync(0xffffffffu, b0, 0);
    }
    if (base >= n) break;
    const int i = base + lane;
    if (!OPT) base += gridDim.x * blockDim.x;
    const bool valid = i < n;
    const unsigned mask = __ballot_sync(0xffffffffu, valid);
    if (!valid) continue;
    const float4 qo = w.q_orig[parity][i];
    const float4 qd = w.q_dir[parity][i];
    const int packed = __float_as_int(qd.w);
    const JobDesc& J = w.jobs[packed >> kMediumBits];
    const SceneView& sc = J.sc;
    VisitCount vc;
    const HitRecord h =
        closest_hit<KIND, COUNT, OPT, WW, false, PS, NF, FR, SI>(sc, v3(qo.x, qo.y, qo.z), v3(qd.x, qd.y, qd.z), k.isect,
                                                         stack, &vc);
    if (COUNT) {
      my_nodes += vc.nodes;
      my_tris += vc.tris;
      // node-fetch slots the warp spends on this batch: 32 lanes x its longest ray
      const unsigned longest = __reduce_max_sync(mask, (unsigned)vc.nodes);
      if (lane == __ffs(mask) - 1) my_slots += 32ull * longest;
    }
    if (vc.dropped) atomicOr(w.counters + kCounterStackDrops, 1);
    const int cls = event_class(w, J, sc, h, __float_as_int(qo.w), (packed & ((1 << kMediumBits) - 1)) - 1,
                                ray_bounce(w, parity, i, it));
    w.hit[i] = make_float4(h.t, h.u, h.v, __int_as_float(h.prim));
    w.hit_geom[i] = h.geom;
    const int pos = warp_append_keyed(mask, cls, counts);
    w.evq[(size_t)cls * w.qcap + pos] = i;
  }
  if (COUNT) {
    for (int off = 16; off > 0; off >>= 1) {
      my_nodes += __shfl_down_sync(0xffffffffu, my_nodes, off);
      my_tris += __shfl_down_sync(0xffffffffu, my_tris, off);
      my_slots += __shfl_down_sync(0xffffffffu, my_slots, off);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(w.visits, my_nodes);
      atomicAdd(w.visits + 1, my_tris);
      atomicAdd(w.visits + 2, my_slots);
    }
  }
}

// Binary-BVH trace kernel with lane refill. Each lane holds one ray at a time through a
// small state machine (idle -> next instance -> traversing -> finished); every loop
// iteration runs one while-while round for the traversing lanes, and lanes whose rays
// are finished take new rays at once (one counter fetch per warp for all idle lanes),
// so a warp no longer waits for its longest ray before taking new work.
enum { RF_IDLE = 0, RF_INSTANCE = 1, RF_TRAVERSE = 2, RF_FINISH = 3 };

template <bool COUNT>
__global__ void __launch_bounds__(128, 8) k_trace_refill(WaveBuffers w, RenderKnobs k, int bounce) {
  const unsigned FULL = 0xffffffffu;
  const int it = pass_iteration(w, bounce);
  const int parity = it & 1;
  const int n = w.counters[parity];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    w.counters[parity ^ 1] = 0;
    w.counters[44 + (parity ^ 1)] = 0;
  }
  int* counts = ev_counts(w, parity);
  int* fetch = w.counters + 44 + parity;
  const int lane = threadIdx.x & 31;
  int stack[kStack];
  int slot = -1, phase = RF_IDLE, inst = 0, cur = kEmptyEntry, leaf = kEmptyEntry, sp = 0, visits = 0;
  int job = 0;
  TraceRay r;
  MeshBest b{FLT_MAX, -1, 0.0f, 0.0f};
  HitRecord h;
  h.t = FLT_MAX; h.u = h.v = 0.0f; h.prim = -1; h.geom = -1;
  VisitCount vc;
  bool more = true;   // warp-uniform: rays may remain in the queue
  for (;;) {
    if (more) {
      const unsigned idle = __ballot_sync(FULL, phase == RF_IDLE);
      if (idle) {
        const int leader = __ffs(idle) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(fetch, __popc(idle));
        base = __shfl_sync(FULL, base, leader);
        if (base + __popc(idle) >= n) more = false;
        if (phase == RF_IDLE) {
          const int i = base + __popc(idle & ((1u << lane) - 1));
          if (i < n) {
            slot = i;
            const float4 qo = w.q_orig[parity][i], qd = w.q_dir[parity][i];
            job = __float_as_int(qd.w) >> kMediumBits;
            const SceneView& sc = w.jobs[job].sc;
            const V3 o = v3(qo.x, qo.y, qo.z), d = v3(qd.x, qd.y, qd.z);
            h.t = FLT_MAX; h.u = h.v = 0.0f; h.prim = -1; h.geom = -1;
            for (int s = 0; s < sc.num_spheres; ++s) {   // spheres (src/primitives/sphere.cu:43-77)
              const DevSphere spr = sc.spheres[s];
              const V3 l = sub(v3(spr.cx, spr.cy, spr.cz), o);
              const float sd = dot(l, d), ls = dot(l, l), rs = spr.r * spr.r;
              if (sd < 0.0f && ls > rs) continue;
              const float ms = ls - sd * sd;
              if (ms > rs) continue;
              const float q = sqrtf(rs - ms);
              const float t = ls > rs ? sd - q : sd + q;
              if (t < h.t) { h.t = t; h.geom = -2 - s; h.prim = -1; }
            }
            inst = 0;
            phase = RF_INSTANCE;
          }
        }
      }
    }
    if (__ballot_sync(FULL, phase != RF_IDLE) == 0) break;
    if (phase == RF_INSTANCE) {
      // next instance whose world box the ray enters before its best hit
      const SceneView& sc = w.jobs[job].sc;
      const float4 qo = w.q_orig[parity][slot], qd = w.q_dir[parity][slot];
      const V3 o = v3(qo.x, qo.y, qo.z), d = v3(qd.x, qd.y, qd.z);
      TraceRay wr;
      wr.o = o;
      wr.d = d;
      wr.idir = v3(safe_rcp(d.x), safe_rcp(d.y), safe_rcp(d.z));
      while (inst < sc.num_instances) {
        const DevInstance& in = sc.instances[inst];
        float te;
        if (box_hit(in.lo[0], in.lo[1], in.lo[2], in.hi[0], in.hi[1], in.hi[2], wr, h.t, te)) {
          setup_ray(r, xform(in.inv, o, 1.0f), xform(in.inv, d, 0.0f), k.isect);
          b = MeshBest{h.t, -1, 0.0f, 0.0f};
          cur = 0;
          leaf = kEmptyEntry;
          sp = 0;
          visits = 0;
          phase = RF_TRAVERSE;
          break;
        }
        ++inst;
      }
      if (phase == RF_INSTANCE) phase = RF_FINISH;
    }
    if (phase == RF_TRAVERSE) {
      const SceneView& sc = w.jobs[job].sc;
      const DevMesh& m = sc.meshes[sc.instances[inst].mesh];
      ww_round<COUNT, true>(m, r, k.isect, b, stack, cur, leaf, sp, visits, vc);
      if (cur == kEmptyEntry) {
        if (b.prim >= 0) { h.t = b.t; h.u = b.u; h.v = b.v; h.prim = b.prim; h.geom = inst; }
        ++inst;
        phase = RF_INSTANCE;
      }
    }
    const unsigned fin = __ballot_sync(FULL, phase == RF_FINISH);
    if (phase == RF_FINISH) {
      const JobDesc& J = w.jobs[job];
      const float4 qo = w.q_orig[parity][slot], qd = w.q_dir[parity][slot];
      const int packed = __float_as_int(qd.w);
      const int cls = event_class(w, J, J.sc, h, __float_as_int(qo.w), (packed & ((1 << kMediumBits) - 1)) - 1,
                                  ray_bounce(w, parity, slot, it));
      w.hit[slot] = make_float4(h.t, h.u, h.v, __int_as_float(h.prim));
      w.hit_geom[slot] = h.geom;
      const int pos = warp_append_keyed(fin, cls, counts);
      w.evq[(size_t)cls * w.qcap + pos] = slot;
      phase = RF_IDLE;
      slot = -1;
    }
  }
  if (vc.dropped) atomicOr(w.counters + kCounterStackDrops, 1);
  if (COUNT) {
    unsigned long long my_nodes = vc.nodes, my_tris = vc.tris;
    for (int off = 16; off > 0; off >>= 1) {
      my_nodes += __shfl_down_sync(FULL, my_nodes, off);
      my_tris += __shfl_down_sync(FULL, my_tris, off);
    }
    if (lane == 0) {
      atomicAdd(w.visits, my_nodes);
      atomicAdd(w.visits + 1, my_tris);
    }
  }
}

// Shadow rays of the next-event estimator: a contribution is added to its path's
// radiance when nothing lies within the ray's maximum distance. Occlusion needs no
// closest hit, so the traversal stops at the first hit (binary and 4-wide layouts);
// warps take 32 rays at a time from a counter (counters[48 + parity]).
template <int KIND>
__global__ void __launch_bounds__(128, 8) k_shadow(WaveBuffers w, RenderKnobs k, int bounce) {
  const int parity = pass_iteration(w, bounce) & 1;
  const int n = w.counters[46 + parity];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    w.counters[46 + (parity ^ 1)] = 0;
    w.counters[48 + (parity ^ 1)] = 0;
    atomicAdd(w.rays, (unsigned long long)n);
  }
  int* fetch = w.counters + 48 + parity;
  const int lane = threadIdx.x & 31;
  typename std::conditional<KIND == BVH_WIDE8, uint2, int>::type stack[kStack];
  for (;;) {
    int b0 = 0;
    if (lane == 0) b0 = atomicAdd(fetch, 32);
    const int base = __shfl_sync(0xffffffffu, b0, 0);
    if (base >= n) break;
    const int i = base + lane;
    const bool valid = i < n;
    const unsigned mask = __ballot_sync(0xffffffffu, valid);
    if (!valid) continue;
    const float4 so = w.s_orig[i], sd = w.s_dir[i], sv = w.s_val[i];
    const int job = __float_as_int(so.w);
    const SceneView& sc = w.jobs[job].sc;
    VisitCount vc;
    const HitRecord h =
        closest_hit<KIND, false, KIND == BVH_BINARY, KIND == BVH_BINARY, KIND != BVH_WIDE8, false, KIND == BVH_WIDE4>(
            sc, v3(so.x, so.y, so.z), v3(sd.x, sd.y, sd.z), k.isect, stack, &vc, sd.w);
    if (vc.dropped) atomicOr(w.counters + kCounterStackDrops, 1);
    if (h.geom == -1) {
      float4* c = w.contrib + __float_as_int(sv.w);
      const float4 v = *c;
      *c = make_float4(v.x + sv.x, v.y + sv.y, v.z + sv.z, v.w);
    }
    const unsigned peers = __match_any_sync(mask, job);
    if (lane == __ffs(peers) - 1) atomicAdd(&w.jobs[job].rays, (unsigned long long)__popc(peers));
  }
}

// Persistent trace kernel for the 8-wide BVH. Each lane owns one ray at a time and walks
// it through a small state machine (spheres at load, then per instance: box cull, object
// ray set-up, traversal steps); every loop iteration runs one traversal step per lane,
// with the kind of step (node fetch or triangle test) chosen per warp by a vote, and a
// lane whose ray is finished takes its next ray at once (rays are assigned statically:
// lane i handles rays i, i + stride, ...). HOOK = test-hook variant (rays and illume_hit
// records in caller buffers).
enum { PH_IDLE = 0, PH_INST = 1, PH_TRAV = 2, PH_DONE = 3 };

template <bool COUNT, bool HOOK>
__global__ void __launch_bounds__(128) k_trace_sm(WaveBuffers w, const SceneView* hook_view, RenderKnobs k, int bounce,
                                                  const float4* hook_rays, int hook_n, illume_hit* hook_out) {
  const unsigned FULL = 0xffffffffu;
  const int it = HOOK ? 0 : pass_iteration(w, bounce);
  const int parity = it & 1;
  const int n = HOOK ? hook_n : w.counters[parity];
  if (!HOOK && blockIdx.x == 0 && threadIdx.x == 0) w.counters[parity ^ 1] = 0;
  int* counts = HOOK ? nullptr : ev_counts(w, parity);
  const int stride = gridDim.x * blockDim.x;
  int next = blockIdx.x * blockDim.x + threadIdx.x;
  uint2 stack[kStack];
  int slot = -1, phase = PH_IDLE, inst = 0, g = 0, medium = -1, steps = 0;
  const SceneView* scp = hook_view;
  const JobDesc* jp = nullptr;
  V3 o = v3(0.0f, 0.0f, 0.0f), d = v3(0.0f, 0.0f, 1.0f);
  HitRecord h;
  h.t = FLT_MAX; h.u = h.v = 0.0f; h.prim = -1; h.geom = -1;
  TraceRay r;
  MeshBest b{FLT_MAX, -1, 0.0f, 0.0f};
  WideState s{kNoNode, 0u, 0u, 0};
  VisitCount vc;
  TraceRay wr;
  for (;;) {
    if (phase == PH_IDLE && next < n) {
      slot = next;
      next += stride;
      if (HOOK) {
        const float4 a = hook_rays[2 * slot], c = hook_rays[2 * slot + 1];
        o = v3(a.x, a.y, a.z);
        d = v3(c.x, c.y, c.z);
      } else {
        const float4 qo = w.q_orig[parity][slot], qd = w.q_dir[parity][slot];
        o = v3(qo.x, qo.y, qo.z);
        d = v3(qd.x, qd.y, qd.z);
        g = __float_as_int(qo.w);
        const int packed = __float_as_int(qd.w);
        jp = w.jobs + (packed >> kMediumBits);
        scp = &jp->sc;
        medium = (packed & ((1 << kMediumBits) - 1)) - 1;
      }
      h.t = FLT_MAX; h.u = h.v = 0.0f; h.prim = -1; h.geom = -1;
      for (int sidx = 0; sidx < scp->num_spheres; ++sidx) {
        const DevSphere sp = scp->spheres[sidx];
        const V3 l = sub(v3(sp.cx, sp.cy, sp.cz), o);
        const float sd = dot(l, d), ls = dot(l, l), rs = sp.r * sp.r;
        if (sd < 0.0f && ls > rs) continue;
        const float ms = ls - sd * sd;
        if (ms > rs) continue;
        const float q = sqrtf(rs - ms);
        const float t = ls > rs ? sd - q : sd + q;
        if (t < h.t) { h.t = t; h.geom = -2 - sidx; h.prim = -1; }
      }
      wr.o = o;
      wr.d = d;
      wr.idir = v3(safe_rcp(d.x), safe_rcp(d.y), safe_rcp(d.z));
      inst = 0;
      phase = PH_INST;
    }
    if (__all_sync(FULL, phase == PH_IDLE)) break;
    if (phase == PH_INST) {
      while (inst < scp->num_instances) {
        const DevInstance& in = scp->instances[inst];
        float te;
        if (box_hit(in.lo[0], in.lo[1], in.lo[2], in.hi[0], in.hi[1], in.hi[2], wr, h.t, te)) {
          setup_ray(r, xform(in.inv, o, 1.0f), xform(in.inv, d, 0.0f), k.isect);
          b = MeshBest{h.t, -1, 0.0f, 0.0f};
          s = WideState{0u, 0u, 0u, 0};
          steps = 0;
          phase = PH_TRAV;
          break;
        }
        ++inst;
      }
      if (phase == PH_INST) phase = PH_DONE;
    }
    const bool trav = phase == PH_TRAV;
    const bool has_tri = trav && s.tri_mask != 0;
    const bool has_node = trav && wide_has_node_work(s);
    const unsigned want_tri = __ballot_sync(FULL, has_tri);
    const unsigned want_node = __ballot_sync(FULL, has_node);
    if (want_tri | want_node) {
      const bool do_tri = __popc(want_tri) >= __popc(want_node);
      if (trav) {
        const DevMesh& m = scp->meshes[scp->instances[inst].mesh];
        if (do_tri) {
          if (has_tri) wide_tri_step<COUNT>(m, r, k.isect, b, s, vc);
        } else if (has_node) {
          wide_node_step<COUNT>(m, r, b, s, stack, vc);
        }
      }
    }
    if (trav) {
      if (++steps > kMaxNodeVisits) s = WideState{kNoNode, 0u, 0u, 0};
      if (wide_done(s)) {
        if (b.prim >= 0) { h.t = b.t; h.u = b.u; h.v = b.v; h.prim = b.prim; h.geom = inst; }
        ++inst;
        phase = PH_INST;
      }
    }
    const unsigned fin = __ballot_sync(FULL, phase == PH_DONE);
    if (phase == PH_DONE) {
      if (HOOK) {
        illume_hit out;
        out.t = h.t;
        out.u = h.geom >= 0 ? h.u : 0.0f;
        out.v = h.geom >= 0 ? h.v : 0.0f;
        out.inst = h.geom >= 0 ? h.geom : -1;
        out.prim = h.geom >= 0 ? h.prim : -1;
        out.sphere = h.geom <= -2 ? -2 - h.geom : -1;
        out.pad[0] = out.pad[1] = 0;
        hook_out[slot] = out;
      } else {
        const int cls = event_class(w, *jp, *scp, h, g, medium, ray_bounce(w, parity, slot, it));
        w.hit[slot] = make_float4(h.t, h.u, h.v, __int_as_float(h.prim));
        w.hit_geom[slot] = h.geom;
        const int pos = warp_append_keyed(fin, cls, counts);
        w.evq[(size_t)cls * w.qcap + pos] = slot;
      }
      phase = PH_IDLE;
      slot = -1;
    }
  }
  if (!HOOK && vc.dropped) atomicOr(w.counters + kCounterStackDrops, 1);
  if (COUNT) {
    unsigned long long my_nodes = vc.nodes, my_tris = vc.tris;
    for (int off = 16; off > 0; off >>= 1) {
      my_nodes += __shfl_down_sync(FULL, my_nodes, off);
      my_tris += __shfl_down_sync(FULL, my_tris, off);
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
    // the binary layout is tested with the box arithmetic and traversal order of the
    // default trace kernel
    const HitRecord h =
        closest_hit<KIND, false, KIND == BVH_BINARY, KIND == BVH_BINARY, false, false, KIND == BVH_WIDE4>(
            sc, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), isect, stack);
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

// Trace kernel variants (RenderKnobs::trace_variant):
//   binary BVH: 0 = at most 64 registers (8 blocks of 128 per SM), fused box tests, dynamic
//   ray fetch, while-while traversal (traverse_bvh2_ww; the default); 1 = compiler's
//   register choice, grid-stride rays, plain box tests, leaves tested where met; 2 =
//   variant 1 held to 64 registers; 3 = variant 0 with leaves tested where met; 4 =
//   variant 0 with lane refill (k_trace_refill);
//   8-wide BVH: 0 = one ray per lane to completion, 1 = persistent state machine;
//   4-wide BVH: 0 = at most 64 registers (8 blocks of 128 per SM), near and far planes
//   loaded by per-ray byte offsets, traversal stack in local memory (the default); 1 =
//   four compare-swaps instead of five in the child ordering; 2 = lo and hi planes
//   loaded and selected per child box; 3 = 6 blocks per SM (at most 80 registers).
const void* trace_kernel_ptr(int bvh_kind, int variant) {
  if (bvh_kind == BVH_WIDE4) {
    if (variant == 1) return (const void*)k_trace<BVH_WIDE4, false, 8, true, false, true, true>;
    if (variant == 2) return (const void*)k_trace<BVH_WIDE4, false, 8, true>;
    if (variant == 3) return (const void*)k_trace<BVH_WIDE4, false, 6, true, false, false, true>;
    if (variant == 4) return (const void*)k_trace<BVH_WIDE4, false, 8, true, false, false, true>;
    return (const void*)k_trace<BVH_WIDE4, false, 8, true, false, false, true, true, true>;
  }
  if (bvh_kind == BVH_WIDE8) {
    if (variant == 2) return (const void*)k_trace<BVH_WIDE8, false>;
    return variant == 1 ? (const void*)k_trace_sm<false, false> : (const void*)k_trace<BVH_WIDE8, false, 8>;
  }
  if (variant == 1) return (const void*)k_trace<BVH_BINARY, false>;
  if (variant == 2) return (const void*)k_trace<BVH_BINARY, false, 8>;
  if (variant == 3) return (const void*)k_trace<BVH_BINARY, false, 8, true>;
  if (variant == 4) return (const void*)k_trace_refill<false>;
  return (const void*)k_trace<BVH_BINARY, false, 8, true, true>;
}

void launch_trace(const WaveBuffers& w, const RenderKnobs& k, int bounce, int grid, cudaStream_t st,
                  bool count_visits) {
  if (k.bvh_kind == BVH_WIDE4) {
    if (k.trace_variant == 1) {
      if (count_visits) k_trace<BVH_WIDE4, true, 8, true, false, true, true><<<grid, 128, 0, st>>>(w, k, bounce);
      else k_trace<BVH_WIDE4, false, 8, true, false, true, true><<<grid, 128, 0, st>>>(w, k, bounce);
    } else if (k.trace_variant == 2) {
      if (count_visits) k_trace<BVH_WIDE4, true, 8, true><<<grid, 128, 0, st>>>(w, k, bounce);
      else k_trace<BVH_WIDE4, false, 8, true><<<grid, 128, 0, st>>>(w, k, bounce);
    } else if (k.trace_variant == 3) {
      if (count_visits) k_trace<BVH_WIDE4, true, 6, true, false, false, true><<<grid, 128, 0, st>>>(w, k, bounce);
      else k_trace<BVH_WIDE4, false, 6, true, false, false, true><<<grid, 128, 0, st>>>(w, k, bounce);
    } else if (k.trace_variant == 4) {
      if (count_visits) k_trace<BVH_WIDE4, true, 8, true, false, false, true><<<grid, 128, 0, st>>>(w, k, bounce);
      else k_trace<BVH_WIDE4, false, 8, true, false, false, true><<<grid, 128, 0, st>>>(w, k, bounce);
    } else {
      if (count_visits) k_trace<BVH_WIDE4, true, 8, true, false, false, true, true, true><<<grid, 128, 0, st>>>(w, k, bounce);
      else k_trace<BVH_WIDE4, false, 8, true, false, false, true, true, true><<<grid, 128, 0, st>>>(w, k, bounce);
    }
    return;
  }
  if (k.bvh_kind == BVH_WIDE8) {
    if (k.trace_variant == 1) {
      if (count_visits) k_trace_sm<true, false><<<grid, 128, 0, st>>>(w, nullptr, k, bounce, nullptr, 0, nullptr);
      else k_trace_sm<false, false><<<grid, 128, 0, st>>>(w, nullptr, k, bounce, nullptr, 0, nullptr);
    } else if (k.trace_variant == 2) {
      if (count_visits) k_trace<BVH_WIDE8, true><<<grid, 128, 0, st>>>(w, k, bounce);
      else k_trace<BVH_WIDE8, false><<<grid, 128, 0, st>>>(w, k, bounce);
    } else {
      if (count_visits) k_trace<BVH_WIDE8, true, 8><<<grid, 128, 0, st>>>(w, k, bounce);
      else k_trace<BVH_WIDE8, false, 8><<<grid, 128, 0, st>>>(w, k, bounce);
    }
    return;
  }
  if (k.trace_variant == 1) {
    if (count_visits) k_trace<BVH_BINARY, true><<<grid, 128, 0, st>>>(w, k, bounce);
    else k_trace<BVH_BINARY, false><<<grid, 128, 0, st>>>(w, k, bounce);
    return;
  }
  if (k.trace_variant == 2) {
    if (count_visits) k_trace<BVH_BINARY, true, 8><<<grid, 128, 0, st>>>(w, k, bounce);
    else k_trace<BVH_BINARY, false, 8><<<grid, 128, 0, st>>>(w, k, bounce);
    return;
  }
  if (k.trace_variant == 3) {
    if (count_visits) k_trace<BVH_BINARY, true, 8, true><<<grid, 128, 0, st>>>(w, k, bounce);
    else k_trace<BVH_BINARY, false, 8, true><<<grid, 128, 0, st>>>(w, k, bounce);
    return;
  }
  if (k.trace_variant == 4) {
    if (count_visits) k_trace_refill<true><<<grid, 128, 0, st>>>(w, k, bounce);
    else k_trace_refill<false><<<grid, 128, 0, st>>>(w, k, bounce);
    return;
  }
  if (count_visits) k_trace<BVH_BINARY, true, 8, true, true><<<grid, 128, 0, st>>>(w, k, bounce);
  else k_trace<BVH_BINARY, false, 8, true, true><<<grid, 128, 0, st>>>(w, k, bounce);
}

const void* shadow_kernel_ptr(int bvh_kind) {
  if (bvh_kind == BVH_WIDE4) return (const void*)k_shadow<BVH_WIDE4>;
  return bvh_kind == BVH_WIDE8 ? (const void*)k_shadow<BVH_WIDE8> : (const void*)k_shadow<BVH_BINARY>;
}

void launch_shadow(const WaveBuffers& w, const RenderKnobs& k, int bounce, int grid, cudaStream_t st) {
  if (k.bvh_kind == BVH_WIDE4) k_shadow<BVH_WIDE4><<<grid, 128, 0, st>>>(w, k, bounce);
  else if (k.bvh_kind == BVH_WIDE8) k_shadow<BVH_WIDE8><<<grid, 128, 0, st>>>(w, k, bounce);
  else k_shadow<BVH_BINARY><<<grid, 128, 0, st>>>(w, k, bounce);
}

void launch_trace_hook(const SceneView& sc, const SceneView* d_view, const float* rays8, int n, int isect,
                       int bvh_kind, void* hits, cudaStream_t st) {
  if (n <= 0) return;
  if (bvh_kind == 2) {  // 8-wide BVH through the persistent state machine
    int dev = 0;
    cudaGetDevice(&dev);
    const int cap = kernel_grid_blocks((const void*)k_trace_sm<false, true>, 128, dev);
    const int grid = std::max(1, std::min(cap, (n + 127) / 128));
    WaveBuffers w{};
    RenderKnobs k{};
    k.isect = isect;
    k.bvh_kind = BVH_WIDE8;
    k_trace_sm<false, true><<<grid, 128, 0, st>>>(w, d_view, k, 0, (const float4*)rays8, n, (illume_hit*)hits);
    return;
  }
  const int grid = (n + 127) / 128;
  if (bvh_kind == 3)   // 4-wide BVH (illume_bvh_kind ILLUME_BVH_WIDE4)
    k_trace_hook<BVH_WIDE4><<<grid, 128, 0, st>>>(sc, (const float4*)rays8, n, isect, (illume_hit*)hits);
  else if (bvh_kind == BVH_WIDE8)
    k_trace_hook<BVH_WIDE8><<<grid, 128, 0, st>>>(sc, (const float4*)rays8, n, isect, (illume_hit*)hits);
  else
    k_trace_hook<BVH_BINARY><<<grid, 128, 0, st>>>(sc, (const float4*)rays8, n, isect, (illume_hit*)hits);
}

// Read bandwidth of data that stays in L2: a grid-stride sweep of the buffer with
// 16-byte loads that skip L1, `reps` times, XOR-folded so the loads are kept.
__global__ void __launch_bounds__(256) k_l2_read(const uint4* buf, size_t n16, int reps, unsigned* sink) {
  unsigned acc = 0;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (int r = 0; r < reps; ++r)
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += stride) {
      const uint4 v = __ldcg(buf + i);
      acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
  if (acc == 0x9e3779b9u) atomicAdd(sink, 1u);
}

void launch_l2_read(const void* buf, size_t bytes, int reps, unsigned* sink, int grid, cudaStream_t st) {
  k_l2_read<<<grid, 256, 0, st>>>(reinterpret_cast<const uint4*>(buf), bytes / 16, reps, sink);
}

const void* l2_read_kernel_ptr() { return (const void*)k_l2_read; }

int kernel_grid_blocks(const void* fn, int block, int device) {
  int sms = 0, per_sm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, 0);
  if (per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

}  // namespace illume
