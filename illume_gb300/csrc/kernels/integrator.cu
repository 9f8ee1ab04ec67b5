// Wavefront integrator stages over a job table: pass planning, camera-ray generation,
// material-sorted shading, radiance accumulation, pass advance and tonemapping, plus
// the BSDF test hook.
//
// One pass renders the current sample range of every job in the table: k_plan lays the
// jobs' paths out in slots, raygen fills the bounce-0 queue, then depth x (trace,
// shade), then accumulate and advance. The bounce loop of src/renderer.cu:538-557 (host
// compaction after every bounce) becomes device-side warp-aggregated appends; the
// per-path arithmetic is that of pathtrace_kernel (src/renderer.cu:139-388). A path
// depends only on its own job row (scene, camera, Philox key, sample index), never on
// which other jobs share the pass.
#include "launch.h"
#include "nee.cuh"
#include "shading.cuh"
#include "../common/philox.cuh"

namespace illume {

__device__ __forceinline__ int* ev_counts2(const WaveBuffers& w, int parity) { return w.counters + 2 + 16 * parity; }

// Row of the job table that owns index x of a pass-wide numbering (paths or pixels):
// the last row whose first index is <= x. Rows with nothing in the pass share their
// first index with the next row, so the search passes over them.
__device__ __forceinline__ int find_row(const int* base, int n, int x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(base + mid) <= x) lo = mid + 1;
    else hi = mid;
  }
  return lo - 1;
}

__device__ __forceinline__ float pack_job_medium(int job, int medium) {
  return __int_as_float((job << kMediumBits) | (medium + 1));
}

// Prefix sums of the pass's paths and pixels over the job table (one block). A table
// whose paths would exceed the slot capacity runs no pass and raises counters[42].
__global__ void __launch_bounds__(1024) k_plan(WaveBuffers w) {
  const unsigned FULL = 0xffffffffu;
  __shared__ int wsum[2][32];
  __shared__ long long carry[2];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, nw = blockDim.x >> 5;
  if (tid == 0) carry[0] = carry[1] = 0;
  __syncthreads();
  for (int base = 0; base < w.njobs; base += blockDim.x) {
    const int j = base + tid;
    int np = 0, nx = 0;
    if (j < w.njobs) {
      const int ns = w.jobs[j].nsamples;
      if (ns > 0) {
        np = ns * w.jobs[j].npix;
        nx = w.jobs[j].npix;
      }
    }
    int sp = np, sx = nx;
    for (int o = 1; o < 32; o <<= 1) {
      const int a = __shfl_up_sync(FULL, sp, o), b = __shfl_up_sync(FULL, sx, o);
      if (lane >= o) { sp += a; sx += b; }
    }
    if (lane == 31) { wsum[0][wid] = sp; wsum[1][wid] = sx; }
    __syncthreads();
    if (wid == 0) {
      int a = lane < nw ? wsum[0][lane] : 0, b = lane < nw ? wsum[1][lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int c = __shfl_up_sync(FULL, a, o), d = __shfl_up_sync(FULL, b, o);
        if (lane >= o) { a += c; b += d; }
      }
      wsum[0][lane] = a;
      wsum[1][lane] = b;
    }
    __syncthreads();
    if (j < w.njobs) {
      const long long pb = carry[0] + (wid > 0 ? wsum[0][wid - 1] : 0) + sp - np;
      const long long xb = carry[1] + (wid > 0 ? wsum[1][wid - 1] : 0) + sx - nx;
      const int pbi = pb > w.cap ? w.cap : (int)pb, xbi = xb > w.cap ? w.cap : (int)xb;
      w.jobs[j].path_base = pbi;
      w.jobs[j].pixel_base = xbi;
      w.job_path_base[j] = pbi;
      w.job_pixel_base[j] = xbi;
    }
    __syncthreads();
    if (tid == 0) {
      carry[0] += wsum[0][nw - 1];
      carry[1] += wsum[1][nw - 1];
    }
    __syncthreads();
  }
  if (tid == 0) {
    const bool over = carry[0] > (long long)w.cap;
    const int paths = over ? 0 : (int)carry[0], pixels = over ? 0 : (int)carry[1];
    w.job_path_base[w.njobs] = paths;
    w.job_pixel_base[w.njobs] = pixels;
    w.counters[kCounterPaths] = paths;
    w.counters[kCounterPixels] = pixels;
    w.counters[0] = paths;
    w.counters[1] = 0;
    w.counters[44] = 0;   // trace ray-fetch counters by bounce parity
    w.counters[45] = 0;
    w.counters[46] = 0;   // shadow-ray counts by bounce parity
    w.counters[47] = 0;
    w.counters[48] = 0;   // shadow-ray fetch counters by bounce parity
    w.counters[49] = 0;
    if (over) w.counters[42] = 1;
    for (int c = 0; c < EV_COUNT; ++c) ev_counts2(w, 0)[c] = 0;
  }
}

// init_rays, src/renderer.cu:81-110, for path slot g of job row j: pid = g - path_base
// = sample_in_pass * npix + pixel.
// Pixel of queue position q (0 <= q < w * h) when a sample's camera rays are queued in
// 8x4 tiles: the pixels of whole tiles first, tile after tile in row-major order (so a
// warp's 32 rays cover a compact patch of the image and traverse alike), then the pixels
// of the partial tiles at the right and bottom edges in row-major order.
__device__ __forceinline__ int tiled_pixel(int q, int w, int h) {
  const int tw = w >> 3, th = h >> 2;
  const int full = tw * th * 32;
  if (q < full) {
    const int t = q >> 5, k = q & 31;
    return ((t / tw) * 4 + (k >> 3)) * w + (t % tw) * 8 + (k & 7);
  }
  const int r = q - full, rw = w - tw * 8, right = th * 4 * rw;
  if (r < right) return (r / rw) * w + tw * 8 + r % rw;
  return th * 4 * w + (r - right);
}

// Starts path i of the pass (0 <= i < the pass's paths) at position q of queue `par`.
__device__ __forceinline__ void start_path(const WaveBuffers& w, int i, int q, int par) {
  const int j = find_row(w.job_path_base, w.njobs, i);
  const JobDesc& J = w.jobs[j];
  const int npix = J.npix;
  const CameraView& cam = J.cam;
  // path i (in tile order) is this pixel's; its slot g keys the radiance
  // the pass's samples come in groups of k; a group's paths are queued pixel by pixel
  // (pixels in tile order) with the group's k samples of a pixel next to each other
  const int rel = i - J.path_base;
  const int ns = J.nsamples > 0 ? J.nsamples : 1;
  const int k = w.ray_group > 1 ? (w.ray_group < ns ? w.ray_group : ns) : 1;
  const int grp = rel / (k * npix);
  const int kk = (grp + 1) * k <= ns ? k : ns - grp * k;   // the last group may be smaller
  const int within = rel - grp * k * npix;
  const int s = grp * k + within % kk;
  const int pixel = tiled_pixel(within / kk, cam.width, cam.height);
  const int g = J.path_base + s * npix + pixel;
  const int sample = J.sample_base + s;
  RngStream rng;
  rng.init((uint32_t)pixel, (uint32_t)sample, 0u, J.seed, J.job);
  const int x = pixel % cam.width, y = pixel / cam.width;
  const float left_edge = cam.left + cam.pixel_size * (float)x;
  const float top_edge = cam.top - cam.pixel_size * (float)y;
  const float r_x = left_edge + cam.pixel_size * rng.next();
  const float r_y = top_edge - cam.pixel_size * rng.next();
  V3 pos = v3(0.0f, 0.0f, 0.0f);
  if (cam.aperture > FLT_EPSILON) {
    const float u1 = rng.next(), u2 = rng.next();
    pos = mul(sample_circle(u1, u2), cam.aperture);
  }
  const V3 origin = xform(cam.m, pos, 1.0f);
  const V3 image_pos = xform(cam.m, v3(r_x, r_y, cam.dof), 1.0f);
  const V3 dir = normalize(sub(image_pos, origin));
  w.q_orig[par][q] = make_float4(origin.x, origin.y, origin.z, __int_as_float(g));
  w.q_dir[par][q] = make_float4(dir.x, dir.y, dir.z, pack_job_medium(j, -1));
  w.q_thr[par][q] = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
  if (w.q_bounce[par]) w.q_bounce[par][q] = 0;
  w.contrib[g] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__global__ void __launch_bounds__(256) k_raygen(WaveBuffers w) {
  const int total = w.counters[kCounterPaths];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) start_path(w, i, i, 0);
}

// ---- path regeneration (see launch.h) ----

// The first batch: min(qcap, paths) paths into queue 0, iteration 0.
__global__ void k_regen_start(WaveBuffers w) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const int total = w.counters[kCounterPaths];
  const int n = total < w.qcap ? total : w.qcap;
  w.counters[kCounterRegenN] = n;
  w.counters[kCounterRegenFirst] = 0;
  w.counters[kCounterRegenQ] = 0;
  w.counters[0] = n;
  w.counters[kCounterGen] = n;
  w.counters[kCounterIter] = 0;
  w.counters[kCounterMore] = 1;
}

// Camera rays of the batch the last plan chose, appended to the queue of the current
// iteration.
__global__ void __launch_bounds__(256) k_regen(WaveBuffers w) {
  const int n = w.counters[kCounterRegenN], first = w.counters[kCounterRegenFirst], q0 = w.counters[kCounterRegenQ];
  const int par = w.counters[kCounterIter] & 1;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x)
    start_path(w, first + k, q0 + k, par);
}

// After an iteration's shading: the next batch of new paths and the loop condition. A
// refill starts at least (1 - threshold) x qcap paths (or all that are left), and a queue
// of at most qcap rays empties within `depth` iterations, so the loop needs fewer than
// (paths / ((1 - threshold) qcap) + 2) (depth + 1) iterations; past twice that bound it
// stops and raises counters[kCounterLoopLimit].
__global__ void k_regen_plan(WaveBuffers w, cudaGraphConditionalHandle cond, int use_cond, int depth,
                             float threshold) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const int it = w.counters[kCounterIter];
  const int np = (it & 1) ^ 1;
  const int total = w.counters[kCounterPaths], gen = w.counters[kCounterGen];
  const int nq = w.counters[np];
  int n = 0;
  if (gen < total && (float)nq <= threshold * (float)w.qcap) {
    n = w.qcap - nq;
    if (n > total - gen) n = total - gen;
    if (n < 0) n = 0;
  }
  w.counters[kCounterRegenN] = n;
  w.counters[kCounterRegenFirst] = gen;
  w.counters[kCounterRegenQ] = nq;
  w.counters[np] = nq + n;
  w.counters[kCounterGen] = gen + n;
  w.counters[kCounterIter] = it + 1;
  w.counters[kCounterIterTotal] += 1;
  bool more = nq + n > 0 || gen + n < total;
  float fill = (1.0f - threshold) * (float)w.qcap;
  if (fill < 1.0f) fill = 1.0f;
  const long long bound = 2 * ((long long)((float)total / fill) + 2) * (long long)(depth + 1) + 16;
  if (more && (long long)it + 1 >= bound) {
    more = false;
    w.counters[kCounterLoopLimit] = 1;
  }
  w.counters[kCounterMore] = more ? 1 : 0;
  if (use_cond) cudaGraphSetConditional(cond, more ? 1u : 0u);
}

// A path's radiance: the reference estimator ends a path at its one contribution, so
// the slot is written once; with next-event estimation contributions add up.
template <bool NEE>
__device__ __forceinline__ void add_radiance(float4* c, V3 L) {
  if (NEE) {
    const float4 v = *c;
    *c = make_float4(v.x + L.x, v.y + L.y, v.z + L.z, 0.0f);
  } else {
    *c = make_float4(L.x, L.y, L.z, 0.0f);
  }
}

struct BounceRng {
  RngStream s;
  __device__ __forceinline__ float operator()() { return s.next(); }
};

// Shading of one bounce over the material-sorted event queues. MINB = blocks of 128
// threads per SM the register allocation must allow (1 = the compiler's choice).
// NEE: the instance with the next-event estimator compiled in (launched only when a job
// of the pass uses it; its extra registers stay out of the reference path).
template <int MINB, bool NEE>
__global__ void __launch_bounds__(128, MINB) k_shade(WaveBuffers w, int bounce_arg) {
  const int it = pass_iteration(w, bounce_arg);
  const int parity = it & 1;
  const int* counts = ev_counts2(w, parity);
  __shared__ int prefix[EV_COUNT + 1];
  // block-level aggregation of the counters every warp would otherwise hit with its own
  // atomic (one address each, so those atomics serialise in L2): the rays of the block's
  // first job, and the block's share of the next-bounce and shadow queues per iteration
  __shared__ int s_job;
  __shared__ unsigned long long s_rays;
  __shared__ int s_warp_cnt[2][4], s_warp_base[2][4], s_base[2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int c = 0; c < EV_COUNT; ++c) { prefix[c] = acc; acc += counts[c]; }
    prefix[EV_COUNT] = acc;
    s_job = -1;
    s_rays = 0;
  }
  __syncthreads();
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    int* next_counts = ev_counts2(w, parity ^ 1);
    for (int c = 0; c < EV_COUNT; ++c) next_counts[c] = 0;
    atomicAdd(w.rays, (unsigned long long)w.counters[parity]);
  }
  const int total = prefix[EV_COUNT];
  int* next_count = w.counters + (parity ^ 1);
  for (int base = blockIdx.x * blockDim.x; base < total; base += gridDim.x * blockDim.x) {
    const int gi = base + threadIdx.x;
    bool cont = false, shadow = false;
    int myjob = -1;
    float4 no = make_float4(0, 0, 0, 0), nd = no, nt = no;
    float4 so = no, sd = no, sv = no;
    int bounce = it;   // this ray's bounce (per ray under path regeneration)
    const unsigned live = __ballot_sync(0xffffffffu, gi < total);
    if (gi < total) {
      int cls = 0;
      while (cls + 1 < EV_COUNT && gi >= prefix[cls + 1]) ++cls;
      const int i = w.evq[(size_t)cls * w.qcap + (gi - prefix[cls])];
      bounce = ray_bounce(w, parity, i, it);
      const float4 qo = w.q_orig[parity][i];
      const float4 qd = w.q_dir[parity][i];
      const float4 qt = w.q_thr[parity][i];
      // The hit record is not gathered for escaped rays, whose record is what every trace
      // kernel writes for no hit (FLT_MAX, 0, 0, prim -1, instance -1), nor for scatter
      // events in a medium, which do not read it.
      const bool no_hit = cls == EV_MISS || cls == EV_MEDIUM;
      const float4 hv = no_hit ? make_float4(FLT_MAX, 0.0f, 0.0f, __int_as_float(-1)) : w.hit[i];
      const int geom = no_hit ? -1 : w.hit_geom[i];
      const int g = __float_as_int(qo.w);
      const int packed = __float_as_int(qd.w);
      const int job = packed >> kMediumBits;
      myjob = job;
      int medium = (packed & ((1 << kMediumBits) - 1)) - 1;
      const JobDesc& J = w.jobs[job];
      const SceneView sc = J.sc;
      const int pid = g - J.path_base;
      const int npix = J.npix;
      const V3 o = v3(qo.x, qo.y, qo.z), d = v3(qd.x, qd.y, qd.z);
      V3 thr = v3(qt.x, qt.y, qt.z);
      const float t = hv.x;
      BounceRng rng;
      rng.s.init((uint32_t)(pid % npix), (uint32_t)(J.sample_base + pid / npix), (uint32_t)(bounce + 1), J.seed,
                 J.job);
      float4* contrib = w.contrib + g;
      const bool last = bounce + 1 >= J.max_depth;
      const bool nee = NEE && (J.flags & JOB_NEE) != 0;
      const float pdf_prev = qt.w;   // density of the BSDF sample that led here (next-event paths)
      if (medium >= 0 && sc.mediums[medium].active) {
        const DevMedium md = sc.mediums[medium];
        const float u = rng();
        const float dist = -logf(u) / md.scattering;
        if (cls == EV_MEDIUM) {
          const float u1 = rng(), u2 = rng();
          const V3 dir = to_basis(sample_hg(md.g, u1, u2, (J.flags & JOB_EXACT_HG) != 0), d);
          const V3 no3 = add(o, mul(d, dist));
          const V3 nd3 = normalize(dir);
          thr = mulv(thr, v3(expf(-1.0f * dist * md.absorption[0]), expf(-1.0f * dist * md.absorption[1]),
                             expf(-1.0f * dist * md.absorption[2])));
          if (!((double)length2(thr) < 1e-4) && !last) {
            cont = true;
            no = make_float4(no3.x, no3.y, no3.z, qo.w);
            nd = make_float4(nd3.x, nd3.y, nd3.z, qd.w);
            nt = make_float4(thr.x, thr.y, thr.z, 0.0f);
          }
          goto done;
        }
        thr = mulv(thr, v3(expf(-1.0f * t * md.absorption[0]), expf(-1.0f * t * md.absorption[1]),
                           expf(-1.0f * t * md.absorption[2])));
      }
      if (cls == EV_MISS) {
        V3 L = mulv(thr, env_eval(sc, d));
        if (nee && pdf_prev > 0.0f) L = mul(L, power_heuristic(pdf_prev, env_light_pdf(*sc.lights, d)));
        add_radiance<NEE>(contrib, L);
        goto done;
      }
      {
        // shading frame of the hit
        V3 N;
        float uv0, uv1;
        int matid;
        if (geom >= 0) {
          const DevInstance& in = sc.instances[geom];
          const DevMesh& m = sc.meshes[in.mesh];
          const int prim = __float_as_int(hv.w);
          const int i0 = __ldg(m.tris + 3 * prim), i1 = __ldg(m.tris + 3 * prim + 1), i2 = __ldg(m.tris + 3 * prim + 2);
          const float bu = hv.y, bv = hv.z;
          V3 n;
          if (!m.normals) {
            const V3 v0 = v3(__ldg(m.positions + 3 * i0), __ldg(m.positions + 3 * i0 + 1), __ldg(m.positions + 3 * i0 + 2));
            const V3 v1 = v3(__ldg(m.positions + 3 * i1), __ldg(m.positions + 3 * i1 + 1), __ldg(m.positions + 3 * i1 + 2));
            const V3 v2 = v3(__ldg(m.positions + 3 * i2), __ldg(m.positions + 3 * i2 + 1), __ldg(m.positions + 3 * i2 + 2));
            n = normalize(cross(sub(v1, v0), sub(v2, v0)));
          } else {
            const V3 n0 = v3(__ldg(m.normals + 3 * i0), __ldg(m.normals + 3 * i0 + 1), __ldg(m.normals + 3 * i0 + 2));
            const V3 n1 = v3(__ldg(m.normals + 3 * i1), __ldg(m.normals + 3 * i1 + 1), __ldg(m.normals + 3 * i1 + 2));
            const V3 n2 = v3(__ldg(m.normals + 3 * i2), __ldg(m.normals + 3 * i2 + 1), __ldg(m.normals + 3 * i2 + 2));
            n = normalize(add(mul(n0, 1.0f - bu - bv), add(mul(n1, bu), mul(n2, bv))));
          }
          N = normalize(xform(in.trans_inv, n, 0.0f));
          if (m.texcoords) {
            const float w0 = 1.0f - bu - bv;
            uv0 = (__ldg(m.texcoords + 2 * i0) * w0 + __ldg(m.texcoords + 2 * i1) * bu) + __ldg(m.texcoords + 2 * i2) * bv;
            uv1 = (__ldg(m.texcoords + 2 * i0 + 1) * w0 + __ldg(m.texcoords + 2 * i1 + 1) * bu) +
                  __ldg(m.texcoords + 2 * i2 + 1) * bv;
          } else {
            uv0 = bu;
            uv1 = bv;
          }
          matid = in.material;
        } else {
          const DevSphere sp = sc.spheres[-2 - geom];
          const V3 pos = add(o, mul(d, t));
          N = normalize(sub(pos, v3(sp.cx, sp.cy, sp.cz)));
          uv0 = (float)((double)(atan2f(N.z, N.x) * 0.5f) * ILLUME_INV_PI_D + 0.5);
          uv1 = (float)(0.5 - (double)asinf(N.y) * ILLUME_INV_PI_D);
          matid = sp.material;
        }
        const DevMaterial mat = sc.materials[matid];
        const V3 albedo = tex_eval(sc, mat.albedo_tex, uv0, uv1);
        const float roughness = tex_eval(sc, mat.roughness_tex, uv0, uv1).x;
        if (mat.type == MAT_EMISSIVE) {
          V3 L = mulv(thr, albedo);
          if (nee && pdf_prev > 0.0f && geom >= 0) {
            const LightView& LV = *sc.lights;
            const int base = LV.num_tri > 0 ? __ldg(LV.inst_light_base + geom) : -1;
            if (base >= 0) {
              const int l = base + __float_as_int(hv.w);
              const float4 e1 = __ldg(&LV.tri[3 * l + 1]), e2 = __ldg(&LV.tri[3 * l + 2]);
              const V3 ln = cross(v3(e1.x, e1.y, e1.z), v3(e2.x, e2.y, e2.z));
              const float lnl = sqrtf(dot(ln, ln));
              const float cos_l = lnl > 0.0f ? dot(ln, d) / lnl : 0.0f;
              L = mul(L, power_heuristic(pdf_prev, tri_light_pdf(LV, l, t, cos_l)));
            }
          }
          add_radiance<NEE>(contrib, L);
          goto done;
        }
        if (last) goto done;   // the path has used all its closest-hit queries
        // next-event estimation: one light sample at a non-delta reflection vertex in air
        if (nee && (medium < 0 || !sc.mediums[medium].active) &&
            (mat.type == MAT_LAMBERT || mat.type == MAT_ROUGHCONDUCTOR || mat.type == MAT_ROUGHREFLECTIVE)) {
          RngStream nr;
          nr.init((uint32_t)(pid % npix), (uint32_t)(J.sample_base + pid / npix), 0x40000000u | (uint32_t)(bounce + 1),
                  J.seed, J.job);
          const float u0 = nr.next(), u1 = nr.next(), u2 = nr.next();
          const V3 ph = add(o, mul(d, t));
          const LightSample ls = sample_light(sc, *sc.lights, ph, u0, u1, u2);
          V3 fcos;
          float pdf_b = 0.0f;
          if (ls.ok && bsdf_eval_cos(mat, d, N, albedo, roughness, ls.dir, fcos, pdf_b)) {
            const V3 Cn = mul(mulv(mulv(thr, fcos), ls.Le), power_heuristic(ls.pdf, pdf_b) / ls.pdf);
            if (isfinite(Cn.x + Cn.y + Cn.z) && (Cn.x > 0.0f || Cn.y > 0.0f || Cn.z > 0.0f)) {
              const V3 norm_o = mul(N, dot(N, d) > 0.0f ? -1.0f : 1.0f);
              const V3 org = add(ph, mul(norm_o, J.ray_bias));
              const float tmax = ls.dist == FLT_MAX ? FLT_MAX : ls.dist * (1.0f - 1e-4f) - J.ray_bias;
              if (tmax > 0.0f) {
                shadow = true;
                so = make_float4(org.x, org.y, org.z, __int_as_float(job));
                sd = make_float4(ls.dir.x, ls.dir.y, ls.dir.z, tmax);
                sv = make_float4(Cn.x, Cn.y, Cn.z, __int_as_float(g));
              }
            }
          }
        }
        const ScatterResult s = scatter(mat, d, N, albedo, roughness, rng);
        if (s.status == SCATTER_KILLED) goto done;
        if (s.medium != kMediumUnchanged) medium = s.medium;
        thr = mulv(thr, s.weight);
        const V3 p = add(add(o, mul(d, t)), mul(s.offset_dir, s.offset_sign * J.ray_bias));
        const V3 dir = normalize(s.dir);
        cont = true;
        no = make_float4(p.x, p.y, p.z, qo.w);
        nd = make_float4(dir.x, dir.y, dir.z, pack_job_medium(job, medium));
        nt = make_float4(thr.x, thr.y, thr.z, nee ? bsdf_sampled_pdf(mat, s, d, N) : 0.0f);
      }
    done:;
      // closest-hit queries of this bounce, per job: the block's first job in shared
      // memory, any other job with a global atomic
      const unsigned peers = __match_any_sync(live, myjob);
      if (lane == __ffs(peers) - 1) {
        int bj = *(volatile int*)&s_job;
        if (bj < 0) {
          atomicCAS(&s_job, -1, myjob);
          bj = *(volatile int*)&s_job;
        }
        if (bj == myjob) atomicAdd(&s_rays, (unsigned long long)__popc(peers));
        else atomicAdd(&w.jobs[myjob].rays, (unsigned long long)__popc(peers));
      }
    }
    // compacted appends of the shadow rays and of the continuing paths: one atomic per
    // block and queue (the loop's trip count is uniform over the block)
    const unsigned ballot = __ballot_sync(0xffffffffu, cont);
    const unsigned sballot = NEE ? __ballot_sync(0xffffffffu, shadow) : 0u;
    if (lane == 0) {
      s_warp_cnt[0][warp] = __popc(ballot);
      if (NEE) s_warp_cnt[1][warp] = __popc(sballot);
    }
    __syncthreads();
    if (threadIdx.x < (NEE ? 2 : 1)) {
      const int q = threadIdx.x;
      int acc = 0;
      for (int v = 0; v < 4; ++v) { s_warp_base[q][v] = acc; acc += s_warp_cnt[q][v]; }
      s_base[q] = acc ? atomicAdd(q == 0 ? next_count : w.counters + 46 + parity, acc) : 0;
    }
    __syncthreads();
    const unsigned below = (1u << lane) - 1;
    if (NEE && shadow) {
      const int j = s_base[1] + s_warp_base[1][warp] + __popc(sballot & below);
      w.s_orig[j] = so;
      w.s_dir[j] = sd;
      w.s_val[j] = sv;
    }
    if (cont) {
      const int j = s_base[0] + s_warp_base[0][warp] + __popc(ballot & below);
      w.q_orig[parity ^ 1][j] = no;
      w.q_dir[parity ^ 1][j] = nd;
      w.q_thr[parity ^ 1][j] = nt;
      if (w.q_bounce[parity ^ 1]) w.q_bounce[parity ^ 1][j] = bounce + 1;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_job >= 0 && s_rays) atomicAdd(&w.jobs[s_job].rays, s_rays);
}

// Adds the pass's per-path radiance into each job's per-pixel accumulators, sample by
// sample in sample order (deterministic), in the job's precision.
__global__ void __launch_bounds__(256) k_accumulate(WaveBuffers w) {
  const int total = w.counters[kCounterPixels];
  for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < total; x += gridDim.x * blockDim.x) {
    const int j = find_row(w.job_pixel_base, w.njobs, x);
    const JobDesc& J = w.jobs[j];
    const int p = x - J.pixel_base;
    const int ns = J.nsamples, npix = J.npix, mode = J.accum_mode, path_base = J.path_base;
    const Accumulators acc = J.acc;
    const bool squares = acc.sumsq != nullptr;   // FP64 work only where it is kept
    float s32[3], c32[3];
    double s64[3], q64[3];
    for (int c = 0; c < 3; ++c) {
      s32[c] = mode != ACCUM_FP64 ? acc.sum32[3 * p + c] : 0.0f;
      c32[c] = mode == ACCUM_KAHAN ? acc.comp32[3 * p + c] : 0.0f;
      s64[c] = mode == ACCUM_FP64 ? acc.sum64[3 * p + c] : 0.0;
      q64[c] = acc.sumsq ? acc.sumsq[3 * p + c] : 0.0;
    }
    // squares of this pass's samples summed in FP32 (at most samples-per-pass terms),
    // then added to the FP64 total once per pass
    float qp[3] = {0.0f, 0.0f, 0.0f};
    for (int s = 0; s < ns; ++s) {
      const float4 L = w.contrib[path_base + (size_t)s * npix + p];
      const float l[3] = {L.x, L.y, L.z};
      for (int c = 0; c < 3; ++c) {
        if (mode == ACCUM_FP32) {
          s32[c] = s32[c] + l[c];
        } else if (mode == ACCUM_KAHAN) {
          // Kahan-Babuska-Neumaier compensated summation
          const float tsum = s32[c] + l[c];
          if (fabsf(s32[c]) >= fabsf(l[c])) c32[c] += (s32[c] - tsum) + l[c];
          else c32[c] += (l[c] - tsum) + s32[c];
          s32[c] = tsum;
        } else {
          s64[c] += (double)l[c];
        }
        if (squares) qp[c] = __fmaf_rn(l[c], l[c], qp[c]);
      }
    }
    if (squares)
      for (int c = 0; c < 3; ++c) q64[c] += (double)qp[c];
    for (int c = 0; c < 3; ++c) {
      if (mode != ACCUM_FP64) acc.sum32[3 * p + c] = s32[c];
      if (mode == ACCUM_KAHAN) acc.comp32[3 * p + c] = c32[c];
      if (mode == ACCUM_FP64) acc.sum64[3 * p + c] = s64[c];
      if (acc.sumsq) acc.sumsq[3 * p + c] = q64[c];
    }
  }
}

// Moves every job row to its next sample range.
__global__ void k_advance(JobDesc* jobs, int njobs) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= njobs) return;
  JobDesc& J = jobs[j];
  if (J.nsamples <= 0) return;
  advance_pass_state(J.sample_base, J.nsamples, J.sample_end, J.per_pass, J.flags);
}

// Tonemap of mean radiance: src/renderer.cu:426-441 and src/tonemapper.cu:32-76.
__device__ __forceinline__ V3 uncharted2(V3 x) {
  const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
  const V3 num = v3(C * B + x.x * A, C * B + x.y * A, C * B + x.z * A);
  const V3 nn = v3(D * E + x.x * num.x, D * E + x.y * num.y, D * E + x.z * num.z);
  const V3 den = v3(B + x.x * A, B + x.y * A, B + x.z * A);
  const V3 dd = v3(D * F + x.x * den.x, D * F + x.y * den.y, D * F + x.z * den.z);
  return v3(-E / F + nn.x / dd.x, -E / F + nn.y / dd.y, -E / F + nn.z / dd.z);
}
__device__ __forceinline__ V3 tonemap_op(int op, V3 in) {
  const float gamma = 1.0f / 2.2f;
  switch (op) {
    case 1:
      return v3(powf(in.x / (1.0f + in.x), gamma), powf(in.y / (1.0f + in.y), gamma), powf(in.z / (1.0f + in.z), gamma));
    case 2: {
      const V3 x = v3(fmaxf(-0.004f + in.x, 0.0f), fmaxf(-0.004f + in.y, 0.0f), fmaxf(-0.004f + in.z, 0.0f));
      return v3((x.x * (0.5f + x.x * 6.2f)) / (0.06f + x.x * (1.7f + x.x * 6.2f)),
                (x.y * (0.5f + x.y * 6.2f)) / (0.06f + x.y * (1.7f + x.y * 6.2f)),
                (x.z * (0.5f + x.z * 6.2f)) / (0.06f + x.z * (1.7f + x.z * 6.2f)));
    }
    case 3: {
      const float W = 11.2f;
      const V3 curr = uncharted2(mul(in, 2.0f));
      const V3 white = uncharted2(v3(W, W, W));
      const V3 ws = v3(1.0f / white.x, 1.0f / white.y, 1.0f / white.z);
      return v3(powf(curr.x * ws.x, gamma), powf(curr.y * ws.y, gamma), powf(curr.z * ws.z, gamma));
    }
    default:
      return v3(powf(in.x, gamma), powf(in.y, gamma), powf(in.z, gamma));
  }
}

__global__ void k_tonemap(Accumulators acc, int mode, int npix, float samples, int op, uint8_t* rgb8, float* mean) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
    V3 sum;
    if (mode == ACCUM_FP64) sum = v3((float)acc.sum64[3 * p], (float)acc.sum64[3 * p + 1], (float)acc.sum64[3 * p + 2]);
    else if (mode == ACCUM_KAHAN)
      sum = v3(acc.sum32[3 * p] + acc.comp32[3 * p], acc.sum32[3 * p + 1] + acc.comp32[3 * p + 1],
               acc.sum32[3 * p + 2] + acc.comp32[3 * p + 2]);
    else sum = v3(acc.sum32[3 * p], acc.sum32[3 * p + 1], acc.sum32[3 * p + 2]);
    V3 avg = mul(sum, 1.0f / samples);
    if (mean) {
      mean[3 * p] = avg.x; mean[3 * p + 1] = avg.y; mean[3 * p + 2] = avg.z;
    }
    if (rgb8) {
      avg = tonemap_op(op, avg);
      avg = v3(fmaxf(fminf(avg.x, 1.0f), 0.0f), fmaxf(fminf(avg.y, 1.0f), 0.0f), fmaxf(fminf(avg.z, 1.0f), 0.0f));
      rgb8[3 * p] = (uint8_t)(int)(255.0f * avg.x);
      rgb8[3 * p + 1] = (uint8_t)(int)(255.0f * avg.y);
      rgb8[3 * p + 2] = (uint8_t)(int)(255.0f * avg.z);
    }
  }
}

__global__ void k_clear(Accumulators acc, int npix) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 3 * npix; i += gridDim.x * blockDim.x) {
    if (acc.sum32) acc.sum32[i] = 0.0f;
    if (acc.comp32) acc.comp32[i] = 0.0f;
    if (acc.sum64) acc.sum64[i] = 0.0;
    if (acc.sumsq) acc.sumsq[i] = 0.0;
  }
}

// BSDF test hook: layout of illume_bsdf_batch (include/illume.h).
struct FixedRng {
  float u[3];
  int k;
  __device__ __forceinline__ float operator()() { return u[k < 3 ? k++ : 2]; }
};

__global__ void k_bsdf_batch(int type, int dist, const float* in, int n, float* out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float* x = in + 16 * (size_t)i;
    float* y = out + 16 * (size_t)i;
    DevMaterial m;
    m.type = type; m.albedo_tex = 0; m.roughness_tex = 0; m.medium = -1; m.distribution = dist;
    m.ior = x[10];
    for (int c = 0; c < 3; ++c) { m.eta[c] = x[11 + c]; m.k[c] = x[14]; }
    m.diffuse_fresnel = x[15];
    const V3 wi = v3(x[0], x[1], x[2]), N = v3(x[3], x[4], x[5]);
    const V3 d = mul(wi, -1.0f);
    FixedRng rng{{x[6], x[7], x[8]}, 0};
    const ScatterResult s = scatter(m, d, N, v3(1.0f, 1.0f, 1.0f), x[9], rng);
    const V3 nd = s.status == SCATTER_KILLED ? v3(0.0f, 0.0f, 0.0f) : normalize(s.dir);
    y[0] = nd.x; y[1] = nd.y; y[2] = nd.z;
    y[3] = s.weight.x; y[4] = s.weight.y; y[5] = s.weight.z;
    y[6] = s.D; y[7] = s.pdf_m; y[8] = s.G; y[9] = s.F;
    float ev = 0.0f, pd = 0.0f;
    if (s.status == SCATTER_REFLECT && (type == MAT_ROUGHREFLECTIVE || type == MAT_ROUGHCONDUCTOR || type == MAT_ROUGHREFRACTIVE)) {
      const float win = fabsf(dot(wi, N)), wom = fabsf(dot(nd, s.m));
      ev = s.F * s.D * s.G / (4.0f * win);
      pd = s.pdf_m / (4.0f * wom);
    } else if (type == MAT_LAMBERT) {
      const float won = fabsf(dot(nd, N));
      ev = (float)((double)won * ILLUME_INV_PI_D);
      pd = ev;
    }
    y[10] = ev; y[11] = pd; y[12] = (float)s.status; y[13] = y[14] = y[15] = 0.0f;
  }
}

// Shade kernel variants (RenderKnobs::shade_variant), by the blocks of 128 that must fit
// an SM (the kernel waits on chains of dependent gathers, so resident warps matter):
// 0 = the measured best (8 blocks, at most 64 registers, for both estimators, although
// the next-event instance spills), 1 = compiler's register choice, 2 = 6 blocks (at most
// 80 registers), 3 = 7 blocks (72), 4 = 8 blocks.
template <bool NEE>
static const void* shade_ptr(int variant) {
  switch (variant) {
    case 1: return (const void*)k_shade<1, NEE>;
    case 2: return (const void*)k_shade<6, NEE>;
    case 3: return (const void*)k_shade<7, NEE>;
    case 4: return (const void*)k_shade<8, NEE>;
    default: return (const void*)k_shade<8, NEE>;
  }
}
const void* shade_kernel_ptr(int variant, bool nee) { return nee ? shade_ptr<true>(variant) : shade_ptr<false>(variant); }

void launch_plan(const WaveBuffers& w, cudaStream_t st) {
  const int threads = w.njobs >= 1024 ? 1024 : ((w.njobs + 31) / 32) * 32;
  k_plan<<<1, threads > 32 ? threads : 32, 0, st>>>(w);
}
void launch_raygen(const WaveBuffers& w, int grid, cudaStream_t st) { k_raygen<<<grid, 256, 0, st>>>(w); }
void launch_regen_start(const WaveBuffers& w, cudaStream_t st) { k_regen_start<<<1, 32, 0, st>>>(w); }
void launch_regen(const WaveBuffers& w, int grid, cudaStream_t st) { k_regen<<<grid, 256, 0, st>>>(w); }
void launch_regen_plan(const WaveBuffers& w, cudaGraphConditionalHandle cond, bool use_cond, int depth, float threshold,
                       cudaStream_t st) {
  k_regen_plan<<<1, 32, 0, st>>>(w, cond, use_cond ? 1 : 0, depth, threshold);
}
void launch_shade(const WaveBuffers& w, const RenderKnobs& k, int bounce, int grid, cudaStream_t st, bool nee) {
  const void* fn = shade_kernel_ptr(k.shade_variant, nee);
  void* args[] = {const_cast<WaveBuffers*>(&w), &bounce};
  cudaLaunchKernel(fn, dim3(grid), dim3(128), args, 0, st);
}
void launch_accumulate(const WaveBuffers& w, int grid, cudaStream_t st) { k_accumulate<<<grid, 256, 0, st>>>(w); }
void launch_advance(const WaveBuffers& w, cudaStream_t st) {
  k_advance<<<(w.njobs + 255) / 256, 256, 0, st>>>(w.jobs, w.njobs);
}
void launch_tonemap(const Accumulators& acc, int mode, int npix, float samples, int op, uint8_t* rgb8, float* mean,
                    cudaStream_t st) {
  const int grid = (npix + 255) / 256;
  if (grid > 0) k_tonemap<<<grid, 256, 0, st>>>(acc, mode, npix, samples, op, rgb8, mean);
}
void launch_clear_accumulators(const Accumulators& acc, int npix, cudaStream_t st) {
  const int grid = (3 * npix + 255) / 256;
  if (grid > 0) k_clear<<<grid < 4096 ? grid : 4096, 256, 0, st>>>(acc, npix);
}
void launch_bsdf_batch(int type, int dist, const float* in, int n, float* out, cudaStream_t st) {
  if (n > 0) k_bsdf_batch<<<(n + 127) / 128, 128, 0, st>>>(type, dist, in, n, out);
}

}  // namespace illume
