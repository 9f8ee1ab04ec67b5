#include "renderer.h"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>

namespace illume {

// allocate_render_info_gpu, src/renderer.cu:443-458
CameraView make_camera(const SceneHost& h, int W, int H) {
  CameraView c{};
  memcpy(c.m, h.camera_transform, sizeof(c.m));
  const float dim_ratio = (float)H / (float)W;
  const float tan_half_fov = tanf((float)(3.14159265358979323846 * (double)h.camera_fov / 360));
  const float dofmfov = h.camera_dof * tan_half_fov;
  c.pixel_size = dofmfov * 2 / (float)W;
  c.left = -1 * dofmfov;
  c.top = dim_ratio * dofmfov;
  c.dof = h.camera_dof;
  c.aperture = h.camera_aperture;
  c.width = W;
  c.height = H;
  return c;
}

Renderer::~Renderer() {
  if (graph) cudaGraphExecDestroy(graph);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
}

size_t Renderer::device_bytes() const {
  size_t b = 0;
  const DevBuffer* all[] = {&q_orig[0], &q_orig[1], &q_dir[0], &q_dir[1], &q_thr[0], &q_thr[1], &hit, &hit_geom, &evq,
                            &counters, &contrib, &rays, &pass, &sum32, &comp32, &sum64, &sumsq, &out_mean, &out_rgb8};
  for (const DevBuffer* d : all) b += d->size();
  return b;
}

int Renderer::init(std::string* err) {
  if (p.width <= 0 || p.height <= 0 || p.spp < 0 || p.max_depth < 0) { *err = "invalid render size, spp or depth"; return ILLUME_ERR_INVALID; }
  if ((long long)p.width * p.height > (1LL << 28)) { *err = "image too large"; return ILLUME_ERR_INVALID; }
  if (p.intersector != ISECT_MT && p.intersector != ISECT_WATERTIGHT) { *err = "unknown intersector"; return ILLUME_ERR_INVALID; }
  if (p.bvh_kind < BVH_BINARY || p.bvh_kind > 2) { *err = "unknown BVH kind"; return ILLUME_ERR_INVALID; }
  if (p.accum_mode < ACCUM_FP32 || p.accum_mode > ACCUM_FP64) { *err = "unknown accumulation mode"; return ILLUME_ERR_INVALID; }
  npix = p.width * p.height;
  const long long target = 1LL << 22;  // paths in flight per pass
  per_pass = p.samples_per_pass > 0 ? p.samples_per_pass : (int)std::max(1LL, std::min<long long>(std::max(p.spp, 1), target / npix));
  cap = per_pass * npix;
  if ((long long)per_pass * npix > (1LL << 30)) { *err = "too many paths per pass"; return ILLUME_ERR_INVALID; }
  int st;
#define ALLOC(buf, bytes) if ((st = (buf).alloc(ctx, (bytes))) != ILLUME_OK) { *err = last_error(); return st; }
  for (int k = 0; k < 2; ++k) {
    ALLOC(q_orig[k], sizeof(float4) * (size_t)cap);
    ALLOC(q_dir[k], sizeof(float4) * (size_t)cap);
    ALLOC(q_thr[k], sizeof(float4) * (size_t)cap);
  }
  ALLOC(hit, sizeof(float4) * (size_t)cap);
  ALLOC(hit_geom, sizeof(int) * (size_t)cap);
  ALLOC(evq, sizeof(int) * (size_t)cap * EV_COUNT);
  ALLOC(counters, sizeof(int) * 64);
  ALLOC(contrib, sizeof(float4) * (size_t)cap);
  ALLOC(rays, sizeof(unsigned long long));
  ALLOC(visits, 2 * sizeof(unsigned long long));
  ALLOC(pass, sizeof(PassState));
  if (p.accum_mode == ACCUM_FP64) { ALLOC(sum64, sizeof(double) * 3 * (size_t)npix); }
  else { ALLOC(sum32, sizeof(float) * 3 * (size_t)npix); }
  if (p.accum_mode == ACCUM_KAHAN) { ALLOC(comp32, sizeof(float) * 3 * (size_t)npix); }
  ALLOC(sumsq, sizeof(double) * 3 * (size_t)npix);
#undef ALLOC
  ILLUME_CUDA_TRY(cudaMemsetAsync(counters.get(), 0, counters.size(), ctx->stream));
  ILLUME_CUDA_TRY(cudaMemsetAsync(rays.get(), 0, rays.size(), ctx->stream));
  for (int k = 0; k < 2; ++k) {
    w.q_orig[k] = q_orig[k].as<float4>();
    w.q_dir[k] = q_dir[k].as<float4>();
    w.q_thr[k] = q_thr[k].as<float4>();
  }
  w.hit = hit.as<float4>();
  w.hit_geom = hit_geom.as<int>();
  w.evq = evq.as<int>();
  w.counters = counters.as<int>();
  w.contrib = contrib.as<float4>();
  w.rays = rays.as<unsigned long long>();
  w.visits = visits.as<unsigned long long>();
  w.pass = pass.as<PassState>();
  w.cap = cap;
  w.npix = npix;
  w.width = p.width;
  w.height = p.height;
  acc.sum32 = sum32.as<float>();
  acc.comp32 = comp32.as<float>();
  acc.sum64 = sum64.as<double>();
  acc.sumsq = sumsq.as<double>();
  cam = make_camera(scene->host, p.width, p.height);
  knobs.seed = p.seed;
  knobs.job = p.job;
  knobs.max_depth = p.max_depth;
  knobs.ray_bias = p.ray_bias;
  knobs.isect = p.intersector;
  knobs.exact_hg = p.exact_hg;
  knobs.bvh_kind = p.bvh_kind == 2 ? BVH_WIDE8 : p.bvh_kind;
  knobs.accum_mode = p.accum_mode;
  knobs.trace_variant = p.bvh_kind == 2 ? 1 : (p.bvh_kind == BVH_BINARY ? p.reserved[0] : 0);
  grid_trace = kernel_grid_blocks(trace_kernel_ptr(knobs.bvh_kind, knobs.trace_variant), 128, ctx->device);
  grid_shade = kernel_grid_blocks(shade_kernel_ptr(), 128, ctx->device);
  grid_raygen = std::max(1, std::min((cap + 255) / 256, ctx->sm_count * 8));
  grid_acc = std::max(1, std::min((npix + 255) / 256, ctx->sm_count * 8));
  ILLUME_CUDA_TRY(cudaEventCreate(&ev0));
  ILLUME_CUDA_TRY(cudaEventCreate(&ev1));
  launch_clear_accumulators(acc, npix, ctx->stream);
  ILLUME_CUDA_TRY(cudaGetLastError());
  ILLUME_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return ILLUME_OK;
}

int Renderer::launch_pass(cudaStream_t st) {
  launch_raygen(w, cam, knobs, grid_raygen, st);
  for (int b = 0; b < p.max_depth; ++b) {
    launch_trace(w, scene->view, knobs, b, grid_trace, st);
    launch_shade(w, scene->view, knobs, b, grid_shade, st);
  }
  launch_accumulate(w, acc, p.accum_mode, grid_acc, st);
  launch_advance_pass(w, st);
  return 3 + 2 * p.max_depth;
}

int Renderer::render_device(bool accumulate, illume_render_stats* stats) {
  auto wall0 = std::chrono::steady_clock::now();
  cudaStream_t st = ctx->stream;
  if (!accumulate) {
    launch_clear_accumulators(acc, npix, st);
    ILLUME_CUDA_TRY(cudaMemsetAsync(rays.get(), 0, rays.size(), st));
    samples_done = 0;
    next_sample = p.sample_begin;
  }
  const int spp = p.spp;
  PassState ps;
  ps.sample_base = next_sample;
  ps.per_pass = per_pass;
  ps.sample_end = next_sample + spp;
  ps.nsamples = std::min(per_pass, spp);
  ILLUME_CUDA_TRY(cudaMemcpyAsync(pass.get(), &ps, sizeof(ps), cudaMemcpyHostToDevice, st));
  unsigned long long rays_before = 0;
  if (accumulate) ILLUME_CUDA_TRY(cudaMemcpyAsync(&rays_before, rays.get(), 8, cudaMemcpyDeviceToHost, st));
  const int npasses = spp > 0 ? (spp + per_pass - 1) / per_pass : 0;
  long long launches = 0;
  if (npasses > 0 && !graph) {
    cudaGraph_t g;
    ILLUME_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    launch_pass(st);
    ILLUME_CUDA_TRY(cudaStreamEndCapture(st, &g));
    const cudaError_t e = cudaGraphInstantiate(&graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { set_error(std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e)); graph = nullptr; return ILLUME_ERR_CUDA; }
  }
  ILLUME_CUDA_TRY(cudaEventRecord(ev0, st));
  for (int i = 0; i < npasses; ++i) {
    ILLUME_CUDA_TRY(cudaGraphLaunch(graph, st));
    launches += 3 + 2 * p.max_depth;
  }
  ILLUME_CUDA_TRY(cudaEventRecord(ev1, st));
  unsigned long long rays_after = 0;
  ILLUME_CUDA_TRY(cudaMemcpyAsync(&rays_after, rays.get(), 8, cudaMemcpyDeviceToHost, st));
  ILLUME_CUDA_TRY(cudaStreamSynchronize(st));
  ILLUME_CUDA_TRY(cudaGetLastError());
  samples_done += spp;
  next_sample += spp;
  ctx->launches += launches;
  if (stats) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    stats->rays = (int64_t)(rays_after - rays_before);
    stats->paths = (int64_t)spp * npix;
    stats->render_ms = ms;
    stats->kernel_launches = launches;
    stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
    stats->h2d_bytes = sizeof(PassState);
    stats->d2h_bytes = 8;
  }
  return ILLUME_OK;
}

int Renderer::profile(bool count_visits, illume_profile* out) {
  cudaStream_t st = ctx->stream;
  memset(out, 0, sizeof(*out));
  PassState ps;
  ps.sample_base = next_sample;
  ps.per_pass = per_pass;
  ps.sample_end = next_sample + per_pass;
  ps.nsamples = per_pass;
  ILLUME_CUDA_TRY(cudaMemcpyAsync(pass.get(), &ps, sizeof(ps), cudaMemcpyHostToDevice, st));
  ILLUME_CUDA_TRY(cudaMemsetAsync(visits.get(), 0, visits.size(), st));
  unsigned long long rays_before = 0, rays_after = 0;
  ILLUME_CUDA_TRY(cudaMemcpyAsync(&rays_before, rays.get(), 8, cudaMemcpyDeviceToHost, st));
  const int nev = 3 + 2 * p.max_depth;
  std::vector<cudaEvent_t> ev(nev + 1);
  for (auto& e : ev) ILLUME_CUDA_TRY(cudaEventCreate(&e));
  int k = 0;
  cudaEventRecord(ev[k++], st);
  launch_raygen(w, cam, knobs, grid_raygen, st);
  cudaEventRecord(ev[k++], st);
  for (int b = 0; b < p.max_depth; ++b) {
    launch_trace(w, scene->view, knobs, b, grid_trace, st, count_visits);
    cudaEventRecord(ev[k++], st);
    launch_shade(w, scene->view, knobs, b, grid_shade, st);
    cudaEventRecord(ev[k++], st);
  }
  launch_accumulate(w, acc, p.accum_mode, grid_acc, st);
  cudaEventRecord(ev[k++], st);
  launch_advance_pass(w, st);
  ILLUME_CUDA_TRY(cudaGetLastError());
  unsigned long long vis[2] = {0, 0};
  ILLUME_CUDA_TRY(cudaMemcpyAsync(&rays_after, rays.get(), 8, cudaMemcpyDeviceToHost, st));
  ILLUME_CUDA_TRY(cudaMemcpyAsync(vis, visits.get(), 16, cudaMemcpyDeviceToHost, st));
  ILLUME_CUDA_TRY(cudaStreamSynchronize(st));
  auto ms = [&](int a, int b) {
    float x = 0.0f;
    cudaEventElapsedTime(&x, ev[a], ev[b]);
    return (double)x;
  };
  out->raygen_ms = ms(0, 1);
  for (int b = 0; b < p.max_depth; ++b) {
    out->trace_ms += ms(1 + 2 * b, 2 + 2 * b);
    out->shade_ms += ms(2 + 2 * b, 3 + 2 * b);
  }
  out->accumulate_ms = ms(1 + 2 * p.max_depth, 2 + 2 * p.max_depth);
  out->trace_launches = p.max_depth;
  out->shade_launches = p.max_depth;
  out->rays = (int64_t)(rays_after - rays_before);
  out->node_fetches = (int64_t)vis[0];
  out->tri_tests = (int64_t)vis[1];
  out->node_bytes = knobs.bvh_kind == BVH_WIDE8 ? (int64_t)sizeof(WideNode) : (int64_t)sizeof(Bvh2Node);
  out->tri_bytes = 3 * (int64_t)sizeof(float4);
  for (auto& e : ev) cudaEventDestroy(e);
  samples_done += per_pass;
  next_sample += per_pass;
  ctx->launches += nev;
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
