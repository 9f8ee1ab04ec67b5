#include "renderer.h"

#include <math.h>
#include <string.h>

#include <stddef.h>

#include <algorithm>
#include <chrono>

namespace illume {

// allocate_render_info_gpu, src/renderer.cu:443-458
static CameraView camera_view(const float* m12, float fov, float dof, float aperture, int W, int H) {
  CameraView c{};
  memcpy(c.m, m12, sizeof(c.m));
  const float dim_ratio = (float)H / (float)W;
  const float tan_half_fov = tanf((float)(3.14159265358979323846 * (double)fov / 360));
  const float dofmfov = dof * tan_half_fov;
  c.pixel_size = dofmfov * 2 / (float)W;
  c.left = -1 * dofmfov;
  c.top = dim_ratio * dofmfov;
  c.dof = dof;
  c.aperture = aperture;
  c.width = W;
  c.height = H;
  return c;
}

CameraView make_camera(const SceneHost& h, int W, int H) {
  return camera_view(h.camera_transform, h.camera_fov, h.camera_dof, h.camera_aperture, W, H);
}

int check_render_params(const illume_render_params& p, Scene& scene, std::string* err) {
  if (p.width <= 0 || p.height <= 0 || p.spp < 0 || p.max_depth < 0) { *err = "invalid render size, spp or depth"; return ILLUME_ERR_INVALID; }
  if ((long long)p.width * p.height > (1LL << 28)) { *err = "image too large"; return ILLUME_ERR_INVALID; }
  if (p.intersector != ISECT_MT && p.intersector != ISECT_WATERTIGHT) { *err = "unknown intersector"; return ILLUME_ERR_INVALID; }
  if (p.bvh_kind < 0 || p.bvh_kind > 3) { *err = "unknown BVH kind"; return ILLUME_ERR_INVALID; }
  if (p.bvh_kind == BVH_BINARY && (p.trace_variant < 0 || p.trace_variant > 4)) { *err = "unknown trace kernel variant"; return ILLUME_ERR_INVALID; }
  if (p.bvh_kind == 3 && (p.trace_variant < 0 || p.trace_variant > 4)) { *err = "unknown trace kernel variant"; return ILLUME_ERR_INVALID; }
  if (p.accum_mode < ACCUM_FP32 || p.accum_mode > ACCUM_FP64) { *err = "unknown accumulation mode"; return ILLUME_ERR_INVALID; }
  if (p.samples_per_pass < 0) { *err = "negative samples per pass"; return ILLUME_ERR_INVALID; }
  if (p.shade_variant < 0 || p.shade_variant > 4) { *err = "unknown shade kernel variant"; return ILLUME_ERR_INVALID; }
  if (p.engines < 0 || p.engines > 16) { *err = "engines out of range (0-16)"; return ILLUME_ERR_INVALID; }
  if (p.estimator < ILLUME_ESTIMATOR_REFERENCE || p.estimator > ILLUME_ESTIMATOR_NEE) { *err = "unknown estimator"; return ILLUME_ERR_INVALID; }
  if (p.queue_slots < 0) { *err = "negative queue slots"; return ILLUME_ERR_INVALID; }
  if (p.ray_group < 0) { *err = "negative ray group"; return ILLUME_ERR_INVALID; }
  if (p.queue_slots > 0 && !(p.regen_threshold >= 0.0f && p.regen_threshold <= 1.0f)) {
    *err = "regeneration threshold outside [0, 1]";
    return ILLUME_ERR_INVALID;
  }
  if ((int)scene.t_mediums.size() > kMaxMediums) { *err = "too many mediums"; return ILLUME_ERR_UNSUPPORTED; }
  // the 8-wide kernels push up to two stack entries per level (a triangle group and a
  // node group); upload bounds the binary and 4-wide trees the same way
  if (!scene.ctx || !scene.view_dev) { *err = "scene has not been uploaded to a device"; return ILLUME_ERR_INVALID; }
  if (p.bvh_kind == ILLUME_BVH_WIDE8 || p.bvh_kind == ILLUME_BVH_WIDE8_PERSISTENT) {
    const int st = scene.ensure_wide(err);   // built and uploaded on first use
    if (st != ILLUME_OK) return st;
    for (const MeshBvh& b : scene.bvhs)
      if (2 * b.stats.wide_depth > 60) { *err = "8-wide BVH deeper than the traversal stack"; return ILLUME_ERR_UNSUPPORTED; }
  }
  return ILLUME_OK;
}

RenderKnobs render_knobs(const illume_render_params& p) {
  RenderKnobs k{};
  k.isect = p.intersector;
  k.bvh_kind = p.bvh_kind == 2 ? BVH_WIDE8 : (p.bvh_kind == 3 ? BVH_WIDE4 : p.bvh_kind);
  k.trace_variant = p.bvh_kind == 2 ? 1
                    : (p.bvh_kind == 1 ? (p.trace_variant == 2 ? 2 : 0)
                                       : (p.bvh_kind == BVH_BINARY || p.bvh_kind == 3 ? p.trace_variant : 0));
  k.shade_variant = p.shade_variant;
  return k;
}

JobDesc job_row(const Scene& scene, const illume_render_params& p, const Accumulators& acc) {
  JobDesc J{};
  J.sc = scene.view;
  J.cam = p.camera ? camera_view(p.camera, p.camera[12], p.camera[13], p.camera[14], p.width, p.height)
                   : make_camera(scene.host, p.width, p.height);
  J.acc = acc;
  J.seed = p.seed;
  J.job = p.job;
  J.max_depth = p.max_depth;
  J.ray_bias = p.ray_bias;
  J.flags = (p.exact_hg ? JOB_EXACT_HG : 0) | (p.estimator == ILLUME_ESTIMATOR_NEE ? JOB_NEE : 0);
  J.accum_mode = p.accum_mode;
  J.npix = p.width * p.height;
  J.width = p.width;
  return J;
}

Renderer::~Renderer() {
  for (cudaStream_t s : more_streams) cudaStreamSynchronize(s);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  for (cudaEvent_t e : acc_ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : join_ev)
    if (e) cudaEventDestroy(e);
  more.clear();   // the extra engines' buffers before their streams
  for (cudaStream_t s : more_streams) cudaStreamDestroy(s);
}

size_t Renderer::device_bytes() const {
  size_t b = eng.device_bytes();
  for (const auto& e : more) b += e->device_bytes();
  const DevBuffer* all[] = {&sum32, &comp32, &sum64, &sumsq, &out_mean, &out_rgb8};
  for (const DevBuffer* d : all) b += d->size();
  return b;
}

int Renderer::init(std::string* err) {
  int st = check_render_params(p, *scene, err);
  if (st != ILLUME_OK) return st;
  npix = p.width * p.height;
  const long long target = 1LL << 27;  // paths in flight per pass (128M: 22.5 GB of path state)
  per_pass = p.samples_per_pass > 0 ? p.samples_per_pass : (int)std::max(1LL, std::min<long long>(std::max(p.spp, 1), target / npix));
  if ((long long)per_pass * npix > (1LL << 30)) { *err = "too many paths per pass"; return ILLUME_ERR_INVALID; }
  // engines taking turns: by default, for a pass of 4M paths or more, one per 16M paths
  // of the pass, at least two and at most four; p.engines asks for a number (1 = never)
  const long long pass_paths = (long long)per_pass * npix;
  nengines = p.engines > 0 ? p.engines
                           : (per_pass >= 2 && pass_paths >= (1LL << 22)
                                  ? (int)std::max(2LL, std::min(4LL, pass_paths >> 24)) : 1);
  nengines = std::max(1, std::min(nengines, per_pass));
  per_pass = (per_pass + nengines - 1) / nengines;
#define ALLOC(buf, bytes) if ((st = (buf).alloc(ctx, (bytes))) != ILLUME_OK) { *err = last_error(); return st; }
  if (p.accum_mode == ACCUM_FP64) { ALLOC(sum64, sizeof(double) * 3 * (size_t)npix); }
  else { ALLOC(sum32, sizeof(float) * 3 * (size_t)npix); }
  if (p.accum_mode == ACCUM_KAHAN) { ALLOC(comp32, sizeof(float) * 3 * (size_t)npix); }
  ALLOC(sumsq, sizeof(double) * 3 * (size_t)npix);
#undef ALLOC
  acc.sum32 = sum32.as<float>();
  acc.comp32 = comp32.as<float>();
  acc.sum64 = sum64.as<double>();
  acc.sumsq = sumsq.as<double>();
  eng.ray_group = p.ray_group > 0 ? p.ray_group : kDefaultRayGroup;
  if ((st = eng.init(ctx, 1, per_pass * npix, render_knobs(p), err, p.queue_slots, p.regen_threshold)) != ILLUME_OK)
    return st;
  JobDesc row = job_row(*scene, p, acc);
  if (nengines > 1) row.flags |= nengines << kInterleaveShift;
  eng.mirror[0] = row;
  p.camera = nullptr;   // read once; the caller's array need not outlive this call
  if ((st = eng.write_row(0)) != ILLUME_OK) { *err = last_error(); return st; }
  if (nengines > 1) {
    acc_ev.assign(nengines, nullptr);
    for (cudaEvent_t& e : acc_ev) ILLUME_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    for (int e = 1; e < nengines; ++e) {
      cudaStream_t s = nullptr;
      ILLUME_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
      more_streams.push_back(s);
      cudaEvent_t j = nullptr;
      ILLUME_CUDA_TRY(cudaEventCreateWithFlags(&j, cudaEventDisableTiming));
      join_ev.push_back(j);
      more.emplace_back(new Engine);
      Engine& x = *more.back();
      x.stream = s;
      x.ray_group = eng.ray_group;
      if ((st = x.init(ctx, 1, per_pass * npix, render_knobs(p), err, p.queue_slots, p.regen_threshold)) != ILLUME_OK)
        return st;
      x.mirror[0] = row;
      if ((st = x.write_row(0)) != ILLUME_OK) { *err = last_error(); return st; }
      ILLUME_CUDA_TRY(cudaStreamSynchronize(s));
    }
  }
  iter_total.assign(nengines, 0);
  ILLUME_CUDA_TRY(cudaEventCreate(&ev0));
  ILLUME_CUDA_TRY(cudaEventCreate(&ev1));
  launch_clear_accumulators(acc, npix, ctx->stream);
  ILLUME_CUDA_TRY(cudaGetLastError());
  ILLUME_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return ILLUME_OK;
}

void Renderer::set_range(int first, int count) {
  JobDesc& J = eng.mirror[0];
  J.sample_base = first;
  J.sample_end = first + count;
  J.per_pass = per_pass;
  J.nsamples = std::min(per_pass, count);
  for (int e = 1; e < nengines; ++e) {   // engine e starts e passes later
    JobDesc& K = engine(e).mirror[0];
    K.sample_base = first + e * per_pass;
    K.sample_end = first + count;
    K.per_pass = per_pass;
    K.nsamples = std::max(0, std::min(per_pass, count - e * per_pass));
  }
}

int Renderer::render_device(bool accumulate, illume_render_stats* stats) {
  auto wall0 = std::chrono::steady_clock::now();
  cudaStream_t st = ctx->stream;
  if (!accumulate) {
    launch_clear_accumulators(acc, npix, st);
    samples_done = 0;
    next_sample = p.sample_begin;
  }
  const int spp = p.spp;
  set_range(next_sample, spp);
  int s;
  for (int e = 0; e < nengines; ++e)
    if ((s = engine(e).write_pass_state(0)) != ILLUME_OK) return s;
  // every engine's ray total before and after, read on the context's stream (the extra
  // engines' streams are idle here and joined into it before the second read)
  std::vector<unsigned long long> rays_before(nengines, 0), rays_after(nengines, 0);
  const size_t rays_off = offsetof(JobDesc, rays);
  for (int e = 0; e < nengines; ++e) {
    if (e > 0) ILLUME_CUDA_TRY(cudaStreamSynchronize(more_streams[e - 1]));   // its row write
    ILLUME_CUDA_TRY(cudaMemcpyAsync(&rays_before[e], reinterpret_cast<const char*>(engine(e).w.jobs) + rays_off, 8,
                                    cudaMemcpyDeviceToHost, st));
  }
  const int npasses = spp > 0 ? (spp + per_pass - 1) / per_pass : 0;
  ILLUME_CUDA_TRY(cudaEventRecord(ev0, st));
  if (nengines > 1) {
    // passes go round the engines; each accumulation waits for the previous one
    for (cudaStream_t x : more_streams) ILLUME_CUDA_TRY(cudaStreamWaitEvent(x, ev0, 0));
    for (int i = 0; i < npasses; ++i) {
      const int e = i % nengines;
      cudaEvent_t wait = i > 0 ? acc_ev[(i - 1) % nengines] : nullptr;
      if ((s = engine(e).run_interleaved(p.max_depth, wait, acc_ev[e])) != ILLUME_OK) return s;
    }
    for (int e = 1; e < nengines; ++e) {
      ILLUME_CUDA_TRY(cudaEventRecord(join_ev[e - 1], more_streams[e - 1]));
      ILLUME_CUDA_TRY(cudaStreamWaitEvent(st, join_ev[e - 1], 0));
    }
  } else {
    if ((s = eng.run(npasses, p.max_depth)) != ILLUME_OK) return s;
  }
  ILLUME_CUDA_TRY(cudaEventRecord(ev1, st));
  // per engine: the traversal-overflow flag, the regeneration loop's iteration total and
  // its bound flag (a word each, after the ray total)
  std::vector<int> flags(3 * (size_t)nengines, 0);
  for (int e = 0; e < nengines; ++e) {
    ILLUME_CUDA_TRY(cudaMemcpyAsync(&rays_after[e], reinterpret_cast<const char*>(engine(e).w.jobs) + rays_off, 8,
                                    cudaMemcpyDeviceToHost, st));
    ILLUME_CUDA_TRY(cudaMemcpyAsync(&flags[3 * e], engine(e).w.counters + kCounterStackDrops, sizeof(int),
                                    cudaMemcpyDeviceToHost, st));
    ILLUME_CUDA_TRY(cudaMemcpyAsync(&flags[3 * e + 1], engine(e).w.counters + kCounterIterTotal, sizeof(int),
                                    cudaMemcpyDeviceToHost, st));
    ILLUME_CUDA_TRY(cudaMemcpyAsync(&flags[3 * e + 2], engine(e).w.counters + kCounterLoopLimit, sizeof(int),
                                    cudaMemcpyDeviceToHost, st));
  }
  ILLUME_CUDA_TRY(cudaStreamSynchronize(st));
  ILLUME_CUDA_TRY(cudaGetLastError());
  stack_overflow = false;
  long long iters = 0;
  bool loop_limit = false;
  for (int e = 0; e < nengines; ++e) {
    stack_overflow = stack_overflow || flags[3 * e] != 0;
    iters += (long long)flags[3 * e + 1] - iter_total[e];
    iter_total[e] = flags[3 * e + 1];
    loop_limit = loop_limit || flags[3 * e + 2] != 0;
  }
  if (loop_limit) {
    set_error("a path-regeneration loop reached its iteration bound: the pass ended before all its paths");
    return ILLUME_ERR_TIMEOUT;
  }
  samples_done += spp;
  next_sample += spp;
  if (stats) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    int64_t rays = 0;
    for (int e = 0; e < nengines; ++e) rays += (int64_t)(rays_after[e] - rays_before[e]);
    stats->rays = rays;
    stats->paths = (int64_t)spp * npix;
    stats->render_ms = ms;
    const bool nee = p.estimator == ILLUME_ESTIMATOR_NEE;
    stats->kernel_launches = eng.regen ? Engine::launches_regen(npasses, iters, nee)
                                       : (int64_t)npasses * Engine::launches_per_pass(p.max_depth, nee);
    stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
    stats->h2d_bytes = 4 * sizeof(int);
    stats->d2h_bytes = 16 + 3 * sizeof(int) * (size_t)nengines;
  }
  return ILLUME_OK;
}

int Renderer::profile(bool count_visits, illume_profile* out) {
  cudaStream_t st = ctx->stream;
  memset(out, 0, sizeof(*out));
  set_range(next_sample, per_pass);
  int s;
  if ((s = eng.write_pass_state(0)) != ILLUME_OK) return s;
  ILLUME_CUDA_TRY(cudaMemsetAsync(eng.visits.get(), 0, eng.visits.size(), st));
  unsigned long long rays_before = 0, rays_after = 0;
  ILLUME_CUDA_TRY(cudaMemcpyAsync(&rays_before, reinterpret_cast<const char*>(eng.w.jobs) + offsetof(JobDesc, rays), 8,
                                  cudaMemcpyDeviceToHost, st));
  std::vector<cudaEvent_t> ev;
  int iters = 0;
  const int ps = eng.run_profiled(p.max_depth, count_visits, ev, &iters);
  if (ps != ILLUME_OK) {
    for (auto& e : ev) if (e) cudaEventDestroy(e);
    return ps;
  }
  unsigned long long vis[3] = {0, 0, 0};
  ILLUME_CUDA_TRY(cudaMemcpyAsync(&rays_after, reinterpret_cast<const char*>(eng.w.jobs) + offsetof(JobDesc, rays), 8,
                                  cudaMemcpyDeviceToHost, st));
  ILLUME_CUDA_TRY(cudaMemcpyAsync(vis, eng.visits.get(), sizeof(vis), cudaMemcpyDeviceToHost, st));
  ILLUME_CUDA_TRY(cudaStreamSynchronize(st));
  auto ms = [&](int a, int b) {
    float x = 0.0f;
    cudaEventElapsedTime(&x, ev[a], ev[b]);
    return (double)x;
  };
  out->raygen_ms = ms(0, 1);
  for (int b = 0; b < iters; ++b) {
    out->trace_ms += ms(1 + 2 * b, 2 + 2 * b);
    out->shade_ms += ms(2 + 2 * b, 3 + 2 * b);
  }
  out->accumulate_ms = ms(1 + 2 * iters, 2 + 2 * iters);
  out->trace_launches = iters;
  out->shade_launches = iters;
  out->rays = (int64_t)(rays_after - rays_before);
  out->node_fetches = (int64_t)vis[0];
  out->tri_tests = (int64_t)vis[1];
  out->lane_slots = (int64_t)vis[2];
  out->node_bytes = eng.knobs.bvh_kind == BVH_WIDE8 ? (int64_t)sizeof(WideNode)
                    : eng.knobs.bvh_kind == BVH_WIDE4 ? (int64_t)sizeof(Bvh4Node) : (int64_t)sizeof(Bvh2Node);
  out->tri_bytes = 3 * (int64_t)sizeof(float4);
  for (auto& e : ev) cudaEventDestroy(e);
  samples_done += per_pass;
  next_sample += per_pass;
  return ILLUME_OK;
}

int Renderer::read(float* mean, double* sum, double* sumsq_out, uint8_t* rgb8) {
  cudaStream_t st = ctx->stream;
  int s;
  if ((mean || rgb8) && !out_mean.get()) {
    if ((s = out_mean.alloc(ctx, sizeof(float) * 3 * (size_t)npix)) != ILLUME_OK) return s;
    if ((s = out_rgb8.alloc(ctx, 3 * (size_t)npix)) != ILLUME_OK) return s;
  }
  if (mean || rgb8) {
    launch_tonemap(acc, p.accum_mode, npix, (float)std::max<long long>(samples_done, 1), p.tonemapper,
                   out_rgb8.as<uint8_t>(), out_mean.as<float>(), st);
    ILLUME_CUDA_TRY(cudaGetLastError());
    if (mean) ILLUME_CUDA_TRY(cudaMemcpyAsync(mean, out_mean.get(), sizeof(float) * 3 * (size_t)npix, cudaMemcpyDeviceToHost, st));
    if (rgb8) ILLUME_CUDA_TRY(cudaMemcpyAsync(rgb8, out_rgb8.get(), 3 * (size_t)npix, cudaMemcpyDeviceToHost, st));
  }
  std::vector<float> s32, c32;
  if (sum) {
    if (p.accum_mode == ACCUM_FP64) {
      ILLUME_CUDA_TRY(cudaMemcpyAsync(sum, sum64.get(), sizeof(double) * 3 * (size_t)npix, cudaMemcpyDeviceToHost, st));
    } else {
      s32.resize(3 * (size_t)npix);
      ILLUME_CUDA_TRY(cudaMemcpyAsync(s32.data(), sum32.get(), sizeof(float) * s32.size(), cudaMemcpyDeviceToHost, st));
      if (p.accum_mode == ACCUM_KAHAN) {
        c32.resize(3 * (size_t)npix);
        ILLUME_CUDA_TRY(cudaMemcpyAsync(c32.data(), comp32.get(), sizeof(float) * c32.size(), cudaMemcpyDeviceToHost, st));
      }
    }
  }
  if (sumsq_out) ILLUME_CUDA_TRY(cudaMemcpyAsync(sumsq_out, sumsq.get(), sizeof(double) * 3 * (size_t)npix, cudaMemcpyDeviceToHost, st));
  ILLUME_CUDA_TRY(cudaStreamSynchronize(st));
  if (sum && p.accum_mode != ACCUM_FP64)
    for (size_t i = 0; i < s32.size(); ++i) sum[i] = (double)s32[i] + (c32.empty() ? 0.0 : (double)c32[i]);
  return ILLUME_OK;
}

}  // namespace illume
