// Closest-hit queries on the device: spheres, then mesh instances, each instance's
// triangles through its binary or 8-wide BVH.
//
// Semantics follow get_min_hit (src/renderer.cu:112-137) with a deterministic tie rule:
// spheres in index order, then instances in index order, a later primitive replaces the
// best only when strictly closer; inside one mesh the closest t wins and equal t goes
// to the lower triangle index (the reference keeps the first one its traversal order
// meets). Triangle tests are Moller-Trumbore as src/primitives/mesh.cu:445-476, or the
// watertight test of Woop, Benthin and Wald (JCGT 2013), written operation by operation
// like the CPU oracle so that, in this -fmad=false build, hits match it bit for bit.
// Box tests are conservative: boxes are padded when built and the exit distance is
// widened by 8 ulp, so no box that contains a reported hit is culled.
#pragma once

#include "../common/dmath.cuh"
#include "../common/types.h"

namespace illume {

static constexpr float kExitSlack = 1.000001f;  // ~8 ulp widening of box exit distances
static constexpr int kStack = 64;
// Upper bound on node fetches of one ray in one mesh: a well-formed tree never comes
// close (each node is fetched at most once per ray); it only bounds the loop.
static constexpr int kMaxNodeVisits = 1 << 22;

struct TraceRay {
  V3 o, d;        // object-space origin / direction (direction as given, not normalised)
  V3 idir;        // clamped reciprocal direction for box tests
  V3 oi;          // o * idir (box tests in fused multiply-add form)
  int oct;        // bit 2: d.x < 0, bit 1: d.y < 0, bit 0: d.z < 0
  // watertight setup
  int kx, ky, kz;
  float Sx, Sy, Sz;
};

__device__ __forceinline__ float safe_rcp(float d) {
  return 1.0f / (fabsf(d) > 1e-20f ? d : copysignf(1e-20f, d));
}

// The same reciprocal from the hardware approximation (rcp.approx.ftz.f32, at most about
// one ulp off; the clamp keeps the input normal). Used only for box tests: a relative
// error e on a ray's reciprocal direction scales each axis's slab distances by (1 + e),
// so entry and exit distances of different axes move apart by at most twice that, far
// inside the ~8 ulp exit widening (kExitSlack), and no box that contains a hit is culled.
__device__ __forceinline__ float fast_rcp(float d) {
  const float c = fabsf(d) > 1e-20f ? d : copysignf(1e-20f, d);
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(c));
  return r;
}

template <bool FR = false>
__device__ __forceinline__ void setup_ray(TraceRay& r, V3 o, V3 d, int isect) {
  r.o = o;
  r.d = d;
  r.idir = FR ? v3(fast_rcp(d.x), fast_rcp(d.y), fast_rcp(d.z)) : v3(safe_rcp(d.x), safe_rcp(d.y), safe_rcp(d.z));
  r.oi = v3(o.x * r.idir.x, o.y * r.idir.y, o.z * r.idir.z);
  r.oct = (d.x < 0.0f ? 4 : 0) | (d.y < 0.0f ? 2 : 0) | (d.z < 0.0f ? 1 : 0);
  if (isect == ISECT_WATERTIGHT) {
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    const float dd[3] = {d.x, d.y, d.z};
    const float dz = dd[kz];
    if (dz < 0.0f) { const int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = dd[kx] / dz;
    r.Sy = dd[ky] / dz;
    r.Sz = 1.0f / dz;
  }
}

__device__ __forceinline__ float comp(V3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// Moller-Trumbore (returns -1 on a miss)
__device__ __forceinline__ float tri_mt(V3 v0, V3 v1, V3 v2, const TraceRay& r, float& u, float& v) {
  const V3 e1 = sub(v1, v0), e2 = sub(v2, v0);
  const V3 P = cross(r.d, e2);
  float det = dot(e1, P);
  if (fabsf(det) < FLT_EPSILON) return -1.0f;
  det = 1.0f / det;
  const V3 T = sub(r.o, v0);
  u = dot(T, P) * det;
  if (u < 0.0f || u > 1.0f) return -1.0f;
  const V3 Q = cross(T, e1);
  v = dot(r.d, Q) * det;
  if (v < 0.0f || u + v > 1.0f) return -1.0f;
  return dot(e2, Q) * det;
}

// Watertight test (returns -1 on a miss); u, v weight vertices 1 and 2.
__device__ __forceinline__ float tri_wt(V3 v0, V3 v1, V3 v2, const TraceRay& r, float& u, float& v) {
  const V3 A = sub(v0, r.o), B = sub(v1, r.o), C = sub(v2, r.o);
  const float Akz = comp(A, r.kz), Bkz = comp(B, r.kz), Ckz = comp(C, r.kz);
  const float Ax = comp(A, r.kx) - r.Sx * Akz, Ay = comp(A, r.ky) - r.Sy * Akz;
  const float Bx = comp(B, r.kx) - r.Sx * Bkz, By = comp(B, r.ky) - r.Sy * Bkz;
  const float Cx = comp(C, r.kx) - r.Sx * Ckz, Cy = comp(C, r.ky) - r.Sy * Ckz;
  float U = Cx * By - Cy * Bx;
  float V = Ax * Cy - Ay * Cx;
  float W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = (float)(__dmul_rn((double)Cx, (double)By) - __dmul_rn((double)Cy, (double)Bx));
    V = (float)(__dmul_rn((double)Ax, (double)Cy) - __dmul_rn((double)Ay, (double)Cx));
    W = (float)(__dmul_rn((double)Bx, (double)Ay) - __dmul_rn((double)By, (double)Ax));
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return -1.0f;
  const float det = U + V + W;
  if (det == 0.0f) return -1.0f;
  const float Az = r.Sz * Akz, Bz = r.Sz * Bkz, Cz = r.Sz * Ckz;
  const float T = U * Az + V * Bz + W * Cz;
  if ((det < 0.0f && T >= 0.0f) || (det > 0.0f && T <= 0.0f)) return -1.0f;
  const float rcp = 1.0f / det;
  u = V * rcp;
  v = W * rcp;
  return T * rcp;
}

struct MeshBest { float t; int prim; float u, v; };

// Visit counters of the instrumented trace kernel (node fetches, triangle tests), and
// whether a push found the traversal stack full (the entry is dropped, so the ray may
// miss a hit; scene upload rejects trees deep enough for that, so it is a defect flag).
struct VisitCount { unsigned nodes = 0, tris = 0; bool dropped = false; };

__device__ __forceinline__ void test_triangle(const float4* tv, int isect, const TraceRay& r, MeshBest& b) {
  const float4 a = __ldg(tv), bb = __ldg(tv + 1), c = __ldg(tv + 2);
  const V3 v0 = v3(a.x, a.y, a.z), v1 = v3(bb.x, bb.y, bb.z), v2 = v3(c.x, c.y, c.z);
  float u = 0.0f, v = 0.0f;
  const float t = isect == ISECT_MT ? tri_mt(v0, v1, v2, r, u, v) : tri_wt(v0, v1, v2, r, u, v);
  const int prim = __float_as_int(a.w);
  if (t > 0.0f && (t < b.t || (t == b.t && prim < b.prim))) {
    b.t = t; b.prim = prim; b.u = u; b.v = v;
  }
}

// Slab test against one box with sign-selected near/far planes.
__device__ __forceinline__ bool box_hit(float lox, float loy, float loz, float hix, float hiy, float hiz,
                                        const TraceRay& r, float tbest, float& tentry) {
  const float nx = r.idir.x >= 0.0f ? lox : hix, fx = r.idir.x >= 0.0f ? hix : lox;
  const float ny = r.idir.y >= 0.0f ? loy : hiy, fy = r.idir.y >= 0.0f ? hiy : loy;
  const float nz = r.idir.z >= 0.0f ? loz : hiz, fz = r.idir.z >= 0.0f ? hiz : loz;
  const float t0 = fmaxf(fmaxf((nx - r.o.x) * r.idir.x, (ny - r.o.y) * r.idir.y), fmaxf((nz - r.o.z) * r.idir.z, 0.0f));
  const float t1 = fminf(fminf((fx - r.o.x) * r.idir.x, (fy - r.o.y) * r.idir.y), (fz - r.o.z) * r.idir.z) * kExitSlack;
  tentry = t0;
  return t0 <= t1 && t0 <= tbest * kExitSlack;
}

// The same slab test with one fused multiply-add per plane, t = plane * idir - o * idir.
// It differs from box_hit by the rounding of o * idir, a relative 2^-24 of |o| / |d|,
// far inside the boxes' build padding (2^-16 of extent plus magnitude) for origins
// within ~100x the mesh extent, so it culls no box that contains a hit either.
// Three-input minimum / maximum (sm_100 and later), as fminf / fmaxf of the three.
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

__device__ __forceinline__ bool box_hit_fma(float lox, float loy, float loz, float hix, float hiy, float hiz,
                                            const TraceRay& r, float tbest, float& tentry) {
  const float nx = r.idir.x >= 0.0f ? lox : hix, fx = r.idir.x >= 0.0f ? hix : lox;
  const float ny = r.idir.y >= 0.0f ? loy : hiy, fy = r.idir.y >= 0.0f ? hiy : loy;
  const float nz = r.idir.z >= 0.0f ? loz : hiz, fz = r.idir.z >= 0.0f ? hiz : loz;
  const float t0 = max3f(__fmaf_rn(nx, r.idir.x, -r.oi.x), __fmaf_rn(ny, r.idir.y, -r.oi.y),
                         fmaxf(__fmaf_rn(nz, r.idir.z, -r.oi.z), 0.0f));
  const float t1 = min3f(__fmaf_rn(fx, r.idir.x, -r.oi.x), __fmaf_rn(fy, r.idir.y, -r.oi.y),
                         __fmaf_rn(fz, r.idir.z, -r.oi.z)) * kExitSlack;
  tentry = t0;
  return t0 <= t1 && t0 <= tbest * kExitSlack;
}

// ---- binary BVH ----
template <bool COUNT, bool FMA = false>
__device__ __forceinline__ void traverse_bvh2(const DevMesh& m, const TraceRay& r, int isect, MeshBest& best,
                                              int* stack, VisitCount& vc) {
  int sp = 0;
  int node = 0;
  for (int guard = 0; guard < kMaxNodeVisits; ++guard) {
    if (COUNT) vc.nodes++;
    const Bvh2Node* n = m.bvh2 + node;
    const float4 a = __ldg(&n->a), b = __ldg(&n->b), c = __ldg(&n->c);
    const int4 d = __ldg(&n->d);
    float te0, te1;
    const bool h0 = FMA ? box_hit_fma(a.x, a.y, a.z, a.w, b.x, b.y, r, best.t, te0)
                        : box_hit(a.x, a.y, a.z, a.w, b.x, b.y, r, best.t, te0);
    const bool h1 = FMA ? box_hit_fma(b.z, b.w, c.x, c.y, c.z, c.w, r, best.t, te1)
                        : box_hit(b.z, b.w, c.x, c.y, c.z, c.w, r, best.t, te1);
    // leaves are tested at once; inner children are visited near first
    int inner0 = -1, inner1 = -1;
    if (h0) {
      if (d.x < 0) {
        if (COUNT) vc.tris += d.z;
        for (int i = ~d.x >> 3; i < (~d.x >> 3) + d.z; ++i) test_triangle(m.bvh2_tris + 3 * i, isect, r, best);
      }
      else inner0 = d.x;
    }
    if (h1) {
      if (d.y < 0) {
        if (COUNT) vc.tris += d.w;
        for (int i = ~d.y >> 3; i < (~d.y >> 3) + d.w; ++i) test_triangle(m.bvh2_tris + 3 * i, isect, r, best);
      }
      else inner1 = d.y;
    }
    if (inner0 >= 0 && inner1 >= 0) {
      const bool swap = te1 < te0;
      node = swap ? inner1 : inner0;
      if (sp < kStack) stack[sp++] = swap ? inner0 : inner1;
      else vc.dropped = true;
      continue;
    }
    if (inner0 >= 0) { node = inner0; continue; }
    if (inner1 >= 0) { node = inner1; continue; }
    if (sp == 0) break;
    node = stack[--sp];
  }
}

// Binary BVH, "while-while" order (after Aila and Laine, "Understanding the efficiency
// of ray traversal on GPUs", HPG 2009): a lane keeps visiting inner nodes and sets aside
// the first leaf it meets; the warp leaves the node loop once every lane still in it
// holds a leaf, and then tests those leaves together. Stack entries are inner node
// indices (>= 0) or leaf codes ~(first << 3 | count) (<= -2); -1 is empty.
static constexpr int kEmptyEntry = -1;

// One while-while round: inner nodes until every lane still in the loop holds a leaf (or
// this lane has nothing left), then the set-aside leaves. cur / leaf / sp carry the
// traversal between rounds; visits bounds the node fetches of one ray.
// ANY: stop at the first triangle hit closer than best.t (occlusion queries).
template <bool COUNT, bool FMA, bool ANY = false>
__device__ __forceinline__ void ww_round(const DevMesh& m, const TraceRay& r, int isect, MeshBest& best, int* stack,
                                         int& cur, int& leaf, int& sp, int& visits, VisitCount& vc) {
  constexpr int kEmpty = kEmptyEntry;
  while (cur >= 0) {
    if (COUNT) vc.nodes++;
    if (++visits > kMaxNodeVisits) { cur = kEmpty; leaf = kEmpty; sp = 0; break; }
    const Bvh2Node* n = m.bvh2 + cur;
    const float4 a = __ldg(&n->a), b = __ldg(&n->b), c = __ldg(&n->c);
    const int4 d = __ldg(&n->d);
    float te0, te1;
    const bool h0 = FMA ? box_hit_fma(a.x, a.y, a.z, a.w, b.x, b.y, r, best.t, te0)
                        : box_hit(a.x, a.y, a.z, a.w, b.x, b.y, r, best.t, te0);
    const bool h1 = FMA ? box_hit_fma(b.z, b.w, c.x, c.y, c.z, c.w, r, best.t, te1)
                        : box_hit(b.z, b.w, c.x, c.y, c.z, c.w, r, best.t, te1);
    // children are stored as visited: inner index, leaf code, or -1 for an empty slot
    int c0 = h0 ? d.x : kEmpty;
    int c1 = h1 ? d.y : kEmpty;
    if (c0 != kEmpty && c1 != kEmpty && te1 < te0) { const int t = c0; c0 = c1; c1 = t; }
    if (c0 == kEmpty) { c0 = c1; c1 = kEmpty; }
    if (c0 != kEmpty) {
      cur = c0;
      if (c1 != kEmpty) {
        if (sp < kStack) stack[sp++] = c1;
        else vc.dropped = true;
      }
    } else {
      cur = sp > 0 ? stack[--sp] : kEmpty;
    }
    if (cur < kEmpty && leaf == kEmpty) {
      leaf = cur;
      cur = sp > 0 ? stack[--sp] : kEmpty;
    }
    if (__all_sync(__activemask(), leaf != kEmpty)) break;
  }
  while (leaf != kEmpty) {
    const int code = ~leaf;
    const int first = code >> 3, count = code & 7;
    if (COUNT) vc.tris += count;
    for (int i = first; i < first + count; ++i) test_triangle(m.bvh2_tris + 3 * i, isect, r, best);
    if (ANY && best.prim >= 0) { cur = kEmpty; leaf = kEmpty; sp = 0; break; }
    leaf = kEmpty;
    if (cur < kEmpty) {
      leaf = cur;
      cur = sp > 0 ? stack[--sp] : kEmpty;
    }
  }
}

template <bool COUNT, bool FMA, bool ANY = false>
__device__ __forceinline__ void traverse_bvh2_ww(const DevMesh& m, const TraceRay& r, int isect, MeshBest& best,
                                                 int* stack, VisitCount& vc) {
  int sp = 0, cur = 0, leaf = kEmptyEntry, visits = 0;
  do {
    ww_round<COUNT, FMA, ANY>(m, r, isect, best, stack, cur, leaf, sp, visits, vc);
  } while (cur != kEmptyEntry);
}

// ---- 4-wide BVH ----
__device__ __forceinline__ void bvh4_slot(float lox, float loy, float loz, float hix, float hiy, float hiz, int child,
                                          const TraceRay& r, float tbest, float& key, int& entry) {
  float te;
  const bool h = box_hit_fma(lox, loy, loz, hix, hiy, hiz, r, tbest, te);
  key = h ? te : FLT_MAX;
  entry = h ? child : kEmptyEntry;
}

// The same test with the near and far planes already chosen by the ray's direction signs.
__device__ __forceinline__ void bvh4_slot_nf(float nx, float ny, float nz, float fx, float fy, float fz, int child,
                                             const TraceRay& r, float tbest, float& key, int& entry) {
  const float t0 = max3f(__fmaf_rn(nx, r.idir.x, -r.oi.x), __fmaf_rn(ny, r.idir.y, -r.oi.y),
                         fmaxf(__fmaf_rn(nz, r.idir.z, -r.oi.z), 0.0f));
  const float t1 = min3f(__fmaf_rn(fx, r.idir.x, -r.oi.x), __fmaf_rn(fy, r.idir.y, -r.oi.y),
                         __fmaf_rn(fz, r.idir.z, -r.oi.z)) * kExitSlack;
  const bool h = t0 <= t1 && t0 <= tbest * kExitSlack;
  key = h ? t0 : FLT_MAX;
  entry = h ? child : kEmptyEntry;
}

__device__ __forceinline__ void sort_pair(float& ka, int& ea, float& kb, int& eb) {
  const bool s = kb < ka;
  const float k = s ? kb : ka;
  kb = s ? ka : kb;
  ka = k;
  const int e = s ? eb : ea;
  eb = s ? ea : eb;
  ea = e;
}

// 4-wide BVH in while-while order: per node the four child boxes are tested, the hit
// children (inner or leaf) ordered by entry distance with a 5-comparator network; the
// nearest becomes the next entry and the others are pushed farthest first. Leaves are
// set aside and tested warp-together as in ww_round; triangles are the binary layout's.
// NF: each ray loads its near and far planes straight from their byte offsets in the
// node (chosen once per ray by the direction's signs and OR-ed into the 128-byte-aligned
// node address) instead of loading lo and hi and selecting per child box; the box test
// arithmetic is the same, so are the results.
// PS: four compare-swaps instead of five: the nearest child is exact, the middle two of
// the pushed ones may come out of order (order changes the work, never the result).
template <bool COUNT, bool ANY = false, bool PS = false, bool NF = false>
__device__ __forceinline__ void traverse_bvh4_ww(const DevMesh& m, const TraceRay& r, int isect, MeshBest& best,
                                                 int* stack, VisitCount& vc) {
  constexpr int kEmpty = kEmptyEntry;
  int sp = 0, cur = 0, leaf = kEmpty, visits = 0;
  // near-plane offsets in a Bvh4Node: lox/loy/loz at 0/16/32, hix/hiy/hiz at 48/64/80
  const unsigned near_x = r.idir.x >= 0.0f ? 0u : 48u, near_y = r.idir.y >= 0.0f ? 16u : 64u,
                 near_z = r.idir.z >= 0.0f ? 32u : 80u;
  auto push = [&](int v) {
    if (sp < kStack) stack[sp++] = v;
    else vc.dropped = true;
  };
  auto pop = [&]() -> int { return stack[--sp]; };
  do {
    while (cur >= 0) {
      if (COUNT) vc.nodes++;
      if (++visits > kMaxNodeVisits) { cur = kEmpty; leaf = kEmpty; sp = 0; break; }
      const Bvh4Node* n = m.bvh4 + cur;
      const int4 ch = __ldg(&n->child);
      float k0, k1, k2, k3;
      int e0, e1, e2, e3;
      if (NF) {
        const uintptr_t a = reinterpret_cast<uintptr_t>(n);
        auto plane = [&](unsigned off) { return __ldg(reinterpret_cast<const float4*>(a | off)); };
        const float4 nx = plane(near_x), fx = plane(near_x ^ 48u), ny = plane(near_y), fy = plane(near_y ^ 80u);
        const float4 nz = plane(near_z), fz = plane(near_z ^ 112u);
        bvh4_slot_nf(nx.x, ny.x, nz.x, fx.x, fy.x, fz.x, ch.x, r, best.t, k0, e0);
        bvh4_slot_nf(nx.y, ny.y, nz.y, fx.y, fy.y, fz.y, ch.y, r, best.t, k1, e1);
        bvh4_slot_nf(nx.z, ny.z, nz.z, fx.z, fy.z, fz.z, ch.z, r, best.t, k2, e2);
        bvh4_slot_nf(nx.w, ny.w, nz.w, fx.w, fy.w, fz.w, ch.w, r, best.t, k3, e3);
      } else {
        const float4 lx = __ldg(&n->lox), ly = __ldg(&n->loy), lz = __ldg(&n->loz);
        const float4 hx = __ldg(&n->hix), hy = __ldg(&n->hiy), hz = __ldg(&n->hiz);
        bvh4_slot(lx.x, ly.x, lz.x, hx.x, hy.x, hz.x, ch.x, r, best.t, k0, e0);
        bvh4_slot(lx.y, ly.y, lz.y, hx.y, hy.y, hz.y, ch.y, r, best.t, k1, e1);
        bvh4_slot(lx.z, ly.z, lz.z, hx.z, hy.z, hz.z, ch.z, r, best.t, k2, e2);
        bvh4_slot(lx.w, ly.w, lz.w, hx.w, hy.w, hz.w, ch.w, r, best.t, k3, e3);
      }
      if (!ANY) {
        sort_pair(k0, e0, k1, e1);
        sort_pair(k2, e2, k3, e3);
        sort_pair(k0, e0, k2, e2);
        sort_pair(k1, e1, k3, e3);
        if (!PS) sort_pair(k1, e1, k2, e2);
      }
      // (occlusion: any hit ends the walk, so the children go unordered.) The room for
      // the three pushes is checked once per node; a full stack drops what does not fit.
      if (__builtin_expect(sp <= kStack - 3, 1)) {
        if (e3 != kEmpty) stack[sp++] = e3;
        if (e2 != kEmpty) stack[sp++] = e2;
        if (e1 != kEmpty) stack[sp++] = e1;
      } else {
        if (e3 != kEmpty) push(e3);
        if (e2 != kEmpty) push(e2);
        if (e1 != kEmpty) push(e1);
      }
      cur = e0 != kEmpty ? e0 : (sp > 0 ? pop() : kEmpty);
      if (cur < kEmpty && leaf == kEmpty) {
        leaf = cur;
        cur = sp > 0 ? pop() : kEmpty;
      }
      if (__all_sync(__activemask(), leaf != kEmpty)) break;
    }
    while (leaf != kEmpty) {
      const int code = ~leaf;
      const int first = code >> 3, count = code & 7;
      if (COUNT) vc.tris += count;
      for (int i = first; i < first + count; ++i) test_triangle(m.bvh2_tris + 3 * i, isect, r, best);
      if (ANY && best.prim >= 0) { cur = kEmpty; leaf = kEmpty; sp = 0; break; }
      leaf = kEmpty;
      if (cur < kEmpty) {
        leaf = cur;
        cur = sp > 0 ? pop() : kEmpty;
      }
    }
  } while (cur != kEmpty);
}

// ---- 8-wide quantised BVH ----
__device__ __forceinline__ float exp2i(uint8_t biased) { return __int_as_float((int)biased << 23); }

// Byte k (0-3) of `word` as a float, exact. PB: a byte permute builds 2^23 + q (the byte
// in the low mantissa bits under the exponent of 2^23) and one subtraction removes 2^23;
// otherwise a shift, a mask and an integer-to-float conversion.
template <bool PB>
__device__ __forceinline__ float byte_as_float(uint32_t word, int k) {
  if (PB) return __int_as_float((int)__byte_perm(word, 0x4B000000u, 0x7650u | (unsigned)k)) - 8388608.0f;
  return (float)((word >> (8 * k)) & 0xffu);
}
static constexpr bool kBytePermute = false;   // the conversion measured faster (see the design notes)

template <bool COUNT>
__device__ __forceinline__ void traverse_wide(const DevMesh& m, const TraceRay& r, int isect, MeshBest& best,
                                              uint2* stack, VisitCount& vc) {
  // group = (child_base, imask << 8 | pending visit-rank bits)
  int sp = 0;
  uint32_t node = 0;
  for (int guard = 0; guard < kMaxNodeVisits; ++guard) {
    if (COUNT) vc.nodes++;
    const float4* np = reinterpret_cast<const float4*>(m.wide + node);
    const float4 q0 = __ldg(np), q1 = __ldg(np + 1), q2 = __ldg(np + 2), q3 = __ldg(np + 3), q4 = __ldg(np + 4);
    const float px = q0.x, py = q0.y, pz = q0.z;
    const uint32_t ew = __float_as_uint(q0.w);
    const uint8_t ex = ew & 0xff, ey = (ew >> 8) & 0xff, ez = (ew >> 16) & 0xff;
    const uint32_t imask = ew >> 24;
    const uint32_t child_base = __float_as_uint(q1.x), tri_base = __float_as_uint(q1.y);
    const uint32_t meta[2] = {__float_as_uint(q1.z), __float_as_uint(q1.w)};
    const uint32_t qlx[2] = {__float_as_uint(q2.x), __float_as_uint(q2.y)};
    const uint32_t qly[2] = {__float_as_uint(q2.z), __float_as_uint(q2.w)};
    const uint32_t qlz[2] = {__float_as_uint(q3.x), __float_as_uint(q3.y)};
    const uint32_t qhx[2] = {__float_as_uint(q3.z), __float_as_uint(q3.w)};
    const uint32_t qhy[2] = {__float_as_uint(q4.x), __float_as_uint(q4.y)};
    const uint32_t qhz[2] = {__float_as_uint(q4.z), __float_as_uint(q4.w)};
    // per-axis affine map q -> t
    const float sx = exp2i(ex) * r.idir.x, sy = exp2i(ey) * r.idir.y, sz = exp2i(ez) * r.idir.z;
    const float bx = (px - r.o.x) * r.idir.x, by = (py - r.o.y) * r.idir.y, bz = (pz - r.o.z) * r.idir.z;
    uint32_t pending = 0;
    for (int s = 0; s < 8; ++s) {
      const int w = s >> 2, sh = (s & 3) * 8;
      const uint32_t me = (meta[w] >> sh) & 0xff;
      const bool inner = (imask >> s) & 1;
      if (!inner && me == 0) continue;
      const int kb = s & 3;
      const float lx = byte_as_float<kBytePermute>(qlx[w], kb), hx = byte_as_float<kBytePermute>(qhx[w], kb);
      const float ly = byte_as_float<kBytePermute>(qly[w], kb), hy = byte_as_float<kBytePermute>(qhy[w], kb);
      const float lz = byte_as_float<kBytePermute>(qlz[w], kb), hz = byte_as_float<kBytePermute>(qhz[w], kb);
      const float nx = r.idir.x >= 0.0f ? lx : hx, fx = r.idir.x >= 0.0f ? hx : lx;
      const float ny = r.idir.y >= 0.0f ? ly : hy, fy = r.idir.y >= 0.0f ? hy : ly;
      const float nz = r.idir.z >= 0.0f ? lz : hz, fz = r.idir.z >= 0.0f ? hz : lz;
      const float t0 = fmaxf(fmaxf(__fmaf_rn(nx, sx, bx), __fmaf_rn(ny, sy, by)), fmaxf(__fmaf_rn(nz, sz, bz), 0.0f));
      const float t1 = fminf(fminf(__fmaf_rn(fx, sx, bx), __fmaf_rn(fy, sy, by)), __fmaf_rn(fz, sz, bz)) * kExitSlack;
      if (!(t0 <= t1 && t0 <= best.t * kExitSlack)) continue;
      if (inner) {
        pending |= 1u << (s ^ r.oct);
      } else {
        const uint32_t cnt = me >> 5, off = me & 31;
        if (COUNT) vc.tris += cnt;
        for (uint32_t i = 0; i < cnt; ++i) test_triangle(m.wide_tris + 3 * (tri_base + off + i), isect, r, best);
      }
    }
    if (pending) {
      const int k = __ffs(pending) - 1;
      pending &= pending - 1;
      const int slot = k ^ r.oct;
      node = child_base + __popc(imask & ((1u << slot) - 1));
      if (pending) {
        if (sp < kStack) stack[sp++] = make_uint2(child_base, (imask << 8) | pending);
        else vc.dropped = true;
      }
      continue;
    }
    // pop the next pending child of a stacked group
    bool found = false;
    while (sp > 0) {
      uint2& g = stack[sp - 1];
      uint32_t pend = g.y & 0xff;
      if (!pend) { --sp; continue; }
      const int k = __ffs(pend) - 1;
      pend &= pend - 1;
      const uint32_t im = g.y >> 8;
      const int slot = k ^ r.oct;
      node = g.x + __popc(im & ((1u << slot) - 1));
      if (pend) g.y = (im << 8) | pend; else --sp;
      found = true;
      break;
    }
    if (!found) break;
  }
}

// ---- 8-wide BVH, one traversal step at a time (persistent state machine) ----
//
// A lane's traversal of one instance is a small state: the next node to fetch, one
// pending triangle group (base + bit mask) and a stack of postponed node groups
// (child base, inner mask, pending visit ranks) and triangle groups (flag bit 31). A
// step either fetches one node (testing its 8 quantised child boxes) or tests one
// triangle. The kernel chooses per warp which kind of step to run, so that the lanes of
// a warp execute the same code path, and refills lanes that finished their ray.
static constexpr uint32_t kNoNode = 0xffffffffu;
static constexpr uint32_t kTriGroup = 0x80000000u;

struct WideState {
  uint32_t fetch;       // node to fetch next, kNoNode if none
  uint32_t tri_base;    // pending triangle group
  uint32_t tri_mask;
  int sp;
};

__device__ __forceinline__ bool wide_has_node_work(const WideState& s) {
  return s.fetch != kNoNode || (s.sp > 0 && s.tri_mask == 0);
}
__device__ __forceinline__ bool wide_done(const WideState& s) {
  return s.fetch == kNoNode && s.tri_mask == 0 && s.sp == 0;
}

// One node step: pop if needed, then fetch and test a node.
template <bool COUNT>
__device__ __forceinline__ void wide_node_step(const DevMesh& m, const TraceRay& r, const MeshBest& best, WideState& s,
                                               uint2* stack, VisitCount& vc) {
  if (s.fetch == kNoNode) {
    uint2& g = stack[s.sp - 1];
    if (g.y & kTriGroup) {
      s.tri_base = g.x;
      s.tri_mask = g.y & ~kTriGroup;
      --s.sp;
      return;
    }
    uint32_t pend = g.y & 0xff;
    const uint32_t im = (g.y >> 8) & 0xff;
    const int k = __ffs(pend) - 1;
    pend &= pend - 1;
    s.fetch = g.x + __popc(im & ((1u << (k ^ r.oct)) - 1));
    if (pend) g.y = (im << 8) | pend;
    else --s.sp;
  }
  if (COUNT) vc.nodes++;
  const float4* np = reinterpret_cast<const float4*>(m.wide + s.fetch);
  const float4 q0 = __ldg(np), q1 = __ldg(np + 1), q2 = __ldg(np + 2), q3 = __ldg(np + 3), q4 = __ldg(np + 4);
  const uint32_t ew = __float_as_uint(q0.w);
  const uint32_t imask = ew >> 24;
  const uint32_t child_base = __float_as_uint(q1.x), tri_base = __float_as_uint(q1.y);
  const float sx = exp2i(ew & 0xff) * r.idir.x, sy = exp2i((ew >> 8) & 0xff) * r.idir.y,
              sz = exp2i((ew >> 16) & 0xff) * r.idir.z;
  const float bx = (q0.x - r.o.x) * r.idir.x, by = (q0.y - r.o.y) * r.idir.y, bz = (q0.z - r.o.z) * r.idir.z;
  const float tlim = best.t * kExitSlack;
  uint32_t pending = 0, tmask = 0;
#pragma unroll
  for (int s8 = 0; s8 < 8; ++s8) {
    const int w = s8 >> 2, sh = (s8 & 3) * 8;
    const uint32_t me = (__float_as_uint(w ? q1.w : q1.z) >> sh) & 0xff;
    const bool inner = (imask >> s8) & 1;
    const int kb = s8 & 3;
    const float lx = byte_as_float<kBytePermute>(__float_as_uint(w ? q2.y : q2.x), kb);
    const float ly = byte_as_float<kBytePermute>(__float_as_uint(w ? q2.w : q2.z), kb);
    const float lz = byte_as_float<kBytePermute>(__float_as_uint(w ? q3.y : q3.x), kb);
    const float hx = byte_as_float<kBytePermute>(__float_as_uint(w ? q3.w : q3.z), kb);
    const float hy = byte_as_float<kBytePermute>(__float_as_uint(w ? q4.y : q4.x), kb);
    const float hz = byte_as_float<kBytePermute>(__float_as_uint(w ? q4.w : q4.z), kb);
    const float nx = r.idir.x >= 0.0f ? lx : hx, fx = r.idir.x >= 0.0f ? hx : lx;
    const float ny = r.idir.y >= 0.0f ? ly : hy, fy = r.idir.y >= 0.0f ? hy : ly;
    const float nz = r.idir.z >= 0.0f ? lz : hz, fz = r.idir.z >= 0.0f ? hz : lz;
    const float t0 = fmaxf(fmaxf(__fmaf_rn(nx, sx, bx), __fmaf_rn(ny, sy, by)), fmaxf(__fmaf_rn(nz, sz, bz), 0.0f));
    const float t1 = fminf(fminf(__fmaf_rn(fx, sx, bx), __fmaf_rn(fy, sy, by)), __fmaf_rn(fz, sz, bz)) * kExitSlack;
    const bool hit = (inner || me != 0) && t0 <= t1 && t0 <= tlim;
    if (hit) {
      if (inner) pending |= 1u << (s8 ^ r.oct);
      else tmask |= ((1u << (me >> 5)) - 1u) << (me & 31);
    }
  }
  if (tmask) {
    if (s.tri_mask) {
      if (s.sp < kStack) stack[s.sp++] = make_uint2(s.tri_base, s.tri_mask | kTriGroup);
      else vc.dropped = true;
    }
    s.tri_base = tri_base;
    s.tri_mask = tmask;
  }
  if (pending) {
    const int k = __ffs(pending) - 1;
    pending &= pending - 1;
    s.fetch = child_base + __popc(imask & ((1u << (k ^ r.oct)) - 1));
    if (pending) {
      if (s.sp < kStack) stack[s.sp++] = make_uint2(child_base, (imask << 8) | pending);
      else vc.dropped = true;
    }
  } else {
    s.fetch = kNoNode;
  }
}

template <bool COUNT>
__device__ __forceinline__ void wide_tri_step(const DevMesh& m, const TraceRay& r, int isect, MeshBest& best,
                                              WideState& s, VisitCount& vc) {
  const int k = __ffs(s.tri_mask) - 1;
  s.tri_mask &= s.tri_mask - 1;
  if (COUNT) vc.tris++;
  test_triangle(m.wide_tris + 3 * (s.tri_base + k), isect, r, best);
}

// Full closest-hit query for a world-space ray (direction used as given).
// tmax: only hits closer than tmax count (shadow rays). ANY: return at the first hit
// found closer than tmax (occlusion; with the binary and 4-wide layouts).
// PS, NF: options of the 4-wide traversal (traverse_bvh4_ww).
// FR: box-test reciprocals from the hardware approximation (fast_rcp).
// SI: instances visited nearest box entry first (scenes of 3 to kSortedInstances
// instances; with two the index order costs less than sorting), stopping at the first
// box that starts beyond the best hit; see below.
static constexpr int kSortedInstances = 16;
template <int KIND, bool COUNT = false, bool FMA = false, bool WW = false, bool ANY = false, bool PS = false,
          bool NF = false, bool FR = false, bool SI = false>
__device__ __forceinline__ HitRecord closest_hit(const SceneView& sc, V3 o, V3 d, int isect, void* stack_mem,
                                                 VisitCount* vcp = nullptr, float tmax = FLT_MAX) {
  VisitCount vc;
  HitRecord h;
  h.t = tmax; h.u = 0.0f; h.v = 0.0f; h.prim = -1; h.geom = -1;
  // spheres (src/primitives/sphere.cu:43-77)
  for (int s = 0; s < sc.num_spheres; ++s) {
    const DevSphere sp = sc.spheres[s];
    const V3 l = sub(v3(sp.cx, sp.cy, sp.cz), o);
    const float sd = dot(l, d);
    const float ls = dot(l, l);
    const float rs = sp.r * sp.r;
    if (sd < 0.0f && ls > rs) continue;
    const float ms = ls - sd * sd;
    if (ms > rs) continue;
    const float q = sqrtf(rs - ms);
    const float t = ls > rs ? sd - q : sd + q;
    if (t < h.t) { h.t = t; h.geom = -2 - s; h.prim = -1; }
  }
  if (ANY && h.geom != -1) return h;
  // world-space probe for instance boxes
  TraceRay wr;
  wr.o = o; wr.d = d;
  wr.idir = FR ? v3(fast_rcp(d.x), fast_rcp(d.y), fast_rcp(d.z)) : v3(safe_rcp(d.x), safe_rcp(d.y), safe_rcp(d.z));
  // Instances in index order, or (SI) the boxes the ray enters sorted by entry distance
  // (equal entries by index), stopping at the first box that starts beyond the best hit.
  // The walk keeps the index-order result whatever the order of visits: a hit at the
  // best distance replaces the best when it comes from an instance of lower index (its
  // mesh best starts with prim INT_MAX, so an equal t wins), never when the best is a
  // sphere or an instance of lower index (prim -1).
  const bool sorted = SI && sc.num_instances > 2 && sc.num_instances <= kSortedInstances;
  float key[SI ? kSortedInstances : 1];
  int idx[SI ? kSortedInstances : 1];
  int count = sc.num_instances;
  if (sorted) {
    count = 0;
    for (int i = 0; i < sc.num_instances; ++i) {
      const DevInstance& in = sc.instances[i];
      float te;
      if (!box_hit(in.lo[0], in.lo[1], in.lo[2], in.hi[0], in.hi[1], in.hi[2], wr, h.t, te)) continue;
      key[count] = te;
      idx[count] = i;
      ++count;
    }
  }
  for (int k = 0; k < count; ++k) {
    int i = k;
    if (sorted) {
      int m = k;
      for (int j = k + 1; j < count; ++j)
        if (key[j] < key[m] || (key[j] == key[m] && idx[j] < idx[m])) m = j;
      const float km = key[m];
      i = idx[m];
      key[m] = key[k];
      idx[m] = idx[k];
      if (!(km <= h.t * kExitSlack)) break;   // this box and every later one start beyond the best hit
    } else {
      const DevInstance& in = sc.instances[i];
      float te;
      if (!box_hit(in.lo[0], in.lo[1], in.lo[2], in.hi[0], in.hi[1], in.hi[2], wr, h.t, te)) continue;
    }
    const DevInstance& in = sc.instances[i];
    TraceRay r;
    setup_ray<FR>(r, xform(in.inv, o, 1.0f), xform(in.inv, d, 0.0f), isect);
    const int seed = h.geom > i ? INT_MAX : -1;
    MeshBest b{h.t, seed, 0.0f, 0.0f};
    const DevMesh& m = sc.meshes[in.mesh];
    if (KIND == BVH_WIDE8) traverse_wide<COUNT>(m, r, isect, b, reinterpret_cast<uint2*>(stack_mem), vc);
    else if (KIND == BVH_WIDE4) traverse_bvh4_ww<COUNT, ANY, PS, NF>(m, r, isect, b, reinterpret_cast<int*>(stack_mem), vc);
    else if (WW) traverse_bvh2_ww<COUNT, FMA, ANY>(m, r, isect, b, reinterpret_cast<int*>(stack_mem), vc);
    else traverse_bvh2<COUNT, FMA>(m, r, isect, b, reinterpret_cast<int*>(stack_mem), vc);
    if (b.prim >= 0 && b.prim != INT_MAX) { h.t = b.t; h.u = b.u; h.v = b.v; h.prim = b.prim; h.geom = i; }
    if (ANY && h.geom != -1) break;
  }
  if (vcp) {
    if (COUNT) *vcp = vc;
    else vcp->dropped = vc.dropped;
  }
  return h;
}

}  // namespace illume
