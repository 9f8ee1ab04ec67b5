// extern "C" entry points of include/illume.h.
#include <stdio.h>
#include <string.h>

#include <chrono>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <vector>

#include "../../../include/illume.h"
#include "handles.h"
#include "image_io.h"

using namespace illume;

#define CHECK_ARG(cond, msg)            \
  do {                                  \
    if (!(cond)) {                      \
      set_error(msg);                   \
      return ILLUME_ERR_INVALID;        \
    }                                   \
  } while (0)

extern "C" {

const char* illume_last_error(void) { return last_error(); }
int illume_abi_version(void) { return ILLUME_ABI_VERSION; }

int illume_context_create(int device, size_t hbm_budget_bytes, illume_context** out) {
  CHECK_ARG(out, "null output handle");
  *out = nullptr;
  int n = 0;
  ILLUME_CUDA_TRY(cudaGetDeviceCount(&n));
  CHECK_ARG(device >= 0 && device < n, "device index out of range");
  ILLUME_CUDA_TRY(cudaSetDevice(device));
  std::unique_ptr<illume_context> ctx(new illume_context);
  ctx->c.device = device;
  ctx->c.budget = hbm_budget_bytes;
  ILLUME_CUDA_TRY(cudaDeviceGetAttribute(&ctx->c.sm_count, cudaDevAttrMultiProcessorCount, device));
  ILLUME_CUDA_TRY(cudaDeviceGetAttribute(&ctx->c.l2_bytes, cudaDevAttrL2CacheSize, device));
  ILLUME_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->c.stream, cudaStreamNonBlocking));
  *out = ctx.release();
  return ILLUME_OK;
}

int illume_context_destroy(illume_context* ctx) {
  if (!ctx) return ILLUME_OK;
  if (ctx->c.stream) {
    cudaStreamSynchronize(ctx->c.stream);
    cudaStreamDestroy(ctx->c.stream);
  }
  delete ctx;
  return ILLUME_OK;
}

void* illume_context_stream(illume_context* ctx) { return ctx ? (void*)ctx->c.stream : nullptr; }

int illume_context_set_bvh_builder(illume_context* ctx, int builder) {
  CHECK_ARG(ctx, "null context");
  CHECK_ARG(builder == ILLUME_BVH_BUILD_HOST || builder == ILLUME_BVH_BUILD_DEVICE, "unknown BVH builder");
  ctx->c.bvh_builder = builder;
  return ILLUME_OK;
}

static int finish_scene(illume_context* ctx, std::unique_ptr<illume_scene>& sc, illume_scene** out) {
  std::string err;
  if (!ctx) {
    const int st = sc->s.build_host(&err);
    if (st != ILLUME_OK) { set_error(err); return st; }
    *out = sc.release();
    return ILLUME_OK;
  }
  cudaSetDevice(ctx->c.device);
  sc->s.ctx = &ctx->c;
  const int st = sc->s.build_and_upload(&err);
  if (st != ILLUME_OK) {
    set_error(err.empty() ? std::string(last_error()) : err);
    return st;
  }
  *out = sc.release();
  return ILLUME_OK;
}

int illume_scene_load_json_string(illume_context* ctx, const char* json, const char* base_dir, illume_scene** out) {
  CHECK_ARG(json && out, "null argument");
  *out = nullptr;
  std::unique_ptr<illume_scene> sc(new illume_scene);
  std::string err;
  const int st = load_scene_json(json, base_dir ? base_dir : "", &sc->s.host, &err);
  if (st != ILLUME_OK) { set_error(err); return st; }
  return finish_scene(ctx, sc, out);
}

int illume_scene_load_json(illume_context* ctx, const char* path, const char* base_dir, illume_scene** out) {
  CHECK_ARG(path && out, "null argument");
  *out = nullptr;
  std::ifstream f(path);
  if (!f) { set_error(std::string("cannot read scene file ") + path); return ILLUME_ERR_IO; }
  std::stringstream ss;
  ss << f.rdbuf();
  return illume_scene_load_json_string(ctx, ss.str().c_str(), base_dir, out);
}

int illume_scene_create(illume_context* ctx, const illume_scene_desc* desc, illume_scene** out) {
  CHECK_ARG(desc && out, "null argument");
  *out = nullptr;
  std::unique_ptr<illume_scene> sc(new illume_scene);
  std::string err;
  const int st = sc->s.host.from_desc(*desc, &err);
  if (st != ILLUME_OK) { set_error(err); return st; }
  return finish_scene(ctx, sc, out);
}

int illume_scene_describe(const illume_scene* scene, illume_scene_desc* out) {
  CHECK_ARG(scene && out, "null argument");
  scene->s.host.to_desc(out);
  return ILLUME_OK;
}

int illume_scene_device_bytes(const illume_scene* scene, size_t* out) {
  CHECK_ARG(scene && out, "null argument");
  *out = scene->s.device_bytes;
  return ILLUME_OK;
}

int illume_scene_upload(illume_scene* scene, size_t* bytes) {
  CHECK_ARG(scene, "null scene");
  CHECK_ARG(scene->s.ctx, "host-only scene");
  cudaSetDevice(scene->s.ctx->device);
  return scene->s.upload_again(bytes);
}

int illume_renderer_profile(illume_renderer* r, int count_visits, illume_profile* out) {
  CHECK_ARG(r && out, "null argument");
  cudaSetDevice(r->r.ctx->device);
  return r->r.profile(count_visits != 0, out);
}

int illume_bvh_cache_stats(int64_t* entries, int64_t* bytes, int64_t* hits, int64_t* misses) {
  long long e = 0, b = 0, h = 0, m = 0;
  illume::bvh_cache_stats(&e, &b, &h, &m);
  if (entries) *entries = e;
  if (bytes) *bytes = b;
  if (hits) *hits = h;
  if (misses) *misses = m;
  return ILLUME_OK;
}

int illume_bvh_cache_clear(void) {
  illume::bvh_cache_clear();
  return ILLUME_OK;
}

int illume_scene_build_info(const illume_scene* scene, int* device_meshes, double* build_ms) {
  CHECK_ARG(scene, "null scene");
  int d = 0;
  for (const MeshBvh& b : scene->s.bvhs) d += b.stats.device_built;
  if (device_meshes) *device_meshes = d;
  if (build_ms) *build_ms = scene->s.build_ms;
  return ILLUME_OK;
}

int illume_scene_check_bvh(const illume_scene* scene, char* report, size_t report_len) {
  CHECK_ARG(scene, "null scene");
  {   // every layout is checked, so the 8-wide one is built if it is not yet
    std::string err;
    const int st = const_cast<illume_scene*>(scene)->s.ensure_wide(&err);
    if (st != ILLUME_OK) { set_error(err.empty() ? std::string(last_error()) : err); return st; }
  }
  const SceneHost& h = scene->s.host;
  std::string rep;
  for (int i = 0; i < h.num_meshes(); ++i) {
    const MeshBvh& b = scene->s.bvhs[i];
    std::string msg;
    const float* P = h.positions.data() + 3 * (size_t)h.mesh_vertex_offset[i];
    const int* T = h.tris.data() + 3 * (size_t)h.mesh_tri_offset[i];
    if (!check_mesh_bvh(P, T, h.mesh_num_tris[i], b, &msg)) {
      set_error("mesh " + std::to_string(i) + ": " + msg);
      return ILLUME_ERR_INVALID;
    }
    char line[256];
    snprintf(line, sizeof(line),
             "mesh %d: %d tris, binary %d nodes depth %d, 4-wide %d nodes depth %d, wide %d nodes %d leaves depth %d, %s",
             i, h.mesh_num_tris[i], b.stats.bvh2_nodes, b.stats.bvh2_depth, b.stats.bvh4_nodes, b.stats.bvh4_depth,
             b.stats.wide_nodes, b.stats.wide_leaves, b.stats.wide_depth,
             b.stats.device_built ? "device build" : "host build");
    rep += line;
    if (b.stats.device_built) {
      char d[96];
      snprintf(d, sizeof(d), " (%d clustering rounds, %.1f ms on the device)", b.stats.device_rounds, b.stats.device_ms);
      rep += d;
    }
    if (!b.stats.device_fallback.empty()) rep += " (device build replaced: " + b.stats.device_fallback + ")";
    rep += "\n";
  }
  if (report && report_len) {
    strncpy(report, rep.c_str(), report_len - 1);
    report[report_len - 1] = 0;
  }
  return ILLUME_OK;
}

static uint64_t fnv1a(uint64_t h, const void* data, size_t bytes) {
  const unsigned char* p = static_cast<const unsigned char*>(data);
  for (size_t i = 0; i < bytes; ++i) h = (h ^ p[i]) * 0x100000001b3ULL;
  return h;
}

int illume_scene_bvh_digest(const illume_scene* scene, int mesh, uint64_t out[4]) {
  CHECK_ARG(scene && out, "null argument");
  CHECK_ARG(mesh >= 0 && mesh < (int)scene->s.bvhs.size(), "mesh index out of range");
  {   // the digest covers every layout, so the 8-wide one is built if it is not yet
    std::string err;
    const int st = const_cast<illume_scene*>(scene)->s.ensure_wide(&err);
    if (st != ILLUME_OK) { set_error(err.empty() ? std::string(last_error()) : err); return st; }
  }
  const MeshBvh& b = scene->s.bvhs[mesh];
  const uint64_t h0 = 0xcbf29ce484222325ULL;
  out[0] = fnv1a(h0, b.bvh2.data(), b.bvh2.size() * sizeof(Bvh2Node));
  out[1] = fnv1a(h0, b.bvh4.data(), b.bvh4.size() * sizeof(Bvh4Node));
  out[2] = fnv1a(h0, b.bvh2_tris.data(), b.bvh2_tris.size() * sizeof(float4));
  out[3] = fnv1a(fnv1a(h0, b.wide.data(), b.wide.size() * sizeof(WideNode)), b.wide_tris.data(),
                 b.wide_tris.size() * sizeof(float4));
  return ILLUME_OK;
}

int illume_scene_destroy(illume_scene* scene) {
  if (!scene) return ILLUME_OK;
  if (scene->s.ctx) cudaStreamSynchronize(scene->s.ctx->stream);
  delete scene;
  return ILLUME_OK;
}

int illume_render_params_default(const illume_scene* scene, int spp, int max_depth, illume_render_params* out) {
  CHECK_ARG(scene && out, "null argument");
  memset(out, 0, sizeof(*out));
  const SceneHost& h = scene->s.host;
  out->width = h.width;
  out->height = h.height;
  out->spp = spp;
  out->max_depth = max_depth;
  out->sample_begin = 0;
  out->ray_bias = h.ray_bias;
  out->tonemapper = h.tonemapper;
  out->seed = 0;
  out->job = 0;
  out->accum_mode = ILLUME_ACCUM_FP32;
  out->intersector = ILLUME_ISECT_WATERTIGHT;
  out->bvh_kind = ILLUME_BVH_WIDE4;
  out->exact_hg = 0;
  out->samples_per_pass = 0;
  out->queue_slots = 0;
  out->regen_threshold = 1.0f;
  return ILLUME_OK;
}

int illume_renderer_create(illume_context* ctx, illume_scene* scene, const illume_render_params* params,
                           illume_renderer** out) {
  CHECK_ARG(ctx && scene && params && out, "null argument");
  CHECK_ARG(scene->s.ctx == &ctx->c, "scene was not uploaded with this context");
  *out = nullptr;
  cudaSetDevice(ctx->c.device);
  std::unique_ptr<illume_renderer> r(new illume_renderer);
  r->r.ctx = &ctx->c;
  r->r.scene = &scene->s;
  r->r.p = *params;
  std::string err;
  const int st = r->r.init(&err);
  if (st != ILLUME_OK) { set_error(err.empty() ? std::string(last_error()) : err); return st; }
  *out = r.release();
  return ILLUME_OK;
}

int illume_renderer_destroy(illume_renderer* r) {
  if (!r) return ILLUME_OK;
  cudaStreamSynchronize(r->r.ctx->stream);
  delete r;
  return ILLUME_OK;
}

int illume_renderer_get_width(const illume_renderer* r) { return r ? r->r.p.width : 0; }
int illume_renderer_get_height(const illume_renderer* r) { return r ? r->r.p.height : 0; }

// The status of a finished render: ILLUME_ERR_TRAVERSAL (outputs written) when a
// traversal of the call found its stack full.
static int traversal_status(illume_renderer* r) {
  if (!r->r.stack_overflow) return ILLUME_OK;
  set_error("a BVH traversal stack overflowed during the render: the outputs are written, but rays may have missed hits");
  return ILLUME_ERR_TRAVERSAL;
}

int illume_render_device(illume_renderer* r, int accumulate, illume_render_stats* stats) {
  CHECK_ARG(r, "null renderer");
  cudaSetDevice(r->r.ctx->device);
  const int st = r->r.render_device(accumulate != 0, stats);
  return st != ILLUME_OK ? st : traversal_status(r);
}

int illume_renderer_read(illume_renderer* r, float* out_mean, double* out_sum, double* out_sumsq, uint8_t* out_rgb8) {
  CHECK_ARG(r, "null renderer");
  cudaSetDevice(r->r.ctx->device);
  return r->r.read(out_mean, out_sum, out_sumsq, out_rgb8);
}

int illume_render(illume_renderer* r, float* out_mean, double* out_sum, double* out_sumsq, uint8_t* out_rgb8,
                  illume_render_stats* stats) {
  CHECK_ARG(r, "null renderer");
  auto t0 = std::chrono::steady_clock::now();
  int st = r->r.render_device(false, stats);
  if (st != ILLUME_OK) return st;
  st = r->r.read(out_mean, out_sum, out_sumsq, out_rgb8);
  if (st != ILLUME_OK) return st;
  if (stats) {
    stats->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    const size_t n = 3 * (size_t)r->r.npix;
    stats->d2h_bytes += (out_mean ? 4 * n : 0) + (out_sum ? 8 * n : 0) + (out_sumsq ? 8 * n : 0) + (out_rgb8 ? n : 0);
  }
  return traversal_status(r);
}

int illume_render_to_bitmap(illume_renderer* r, illume_bitmap* bitmap, illume_render_stats* stats) {
  CHECK_ARG(r && bitmap && bitmap->pixels, "null argument");
  CHECK_ARG(bitmap->width == (size_t)r->r.p.width && bitmap->height == (size_t)r->r.p.height,
            "bitmap size differs from the renderer's resolution");
  std::vector<uint8_t> rgb(3 * (size_t)r->r.npix);
  const int st = illume_render(r, nullptr, nullptr, nullptr, rgb.data(), stats);
  if (st != ILLUME_OK && st != ILLUME_ERR_TRAVERSAL) return st;
  for (size_t i = 0; i < (size_t)r->r.npix; ++i) {
    bitmap->pixels[i].red = rgb[3 * i];
    bitmap->pixels[i].green = rgb[3 * i + 1];
    bitmap->pixels[i].blue = rgb[3 * i + 2];
  }
  return st;
}

illume_bitmap* illume_bitmap_new(size_t width, size_t height) {
  illume_bitmap* b = (illume_bitmap*)calloc(1, sizeof(illume_bitmap));
  if (!b) return nullptr;
  const size_t n = width * height;
  b->pixels = (illume_pixel*)calloc(n > 0 ? n : 1, sizeof(illume_pixel));
  if (!b->pixels) { free(b); return nullptr; }
  b->width = width;
  b->height = height;
  return b;
}

void illume_bitmap_free(illume_bitmap* b) {
  if (!b) return;
  free(b->pixels);
  free(b);
}

static std::vector<uint8_t> bitmap_rgb8(const illume_bitmap* b) {
  std::vector<uint8_t> rgb(3 * b->width * b->height);
  for (size_t i = 0; i < b->width * b->height; ++i) {
    rgb[3 * i] = (uint8_t)b->pixels[i].red;
    rgb[3 * i + 1] = (uint8_t)b->pixels[i].green;
    rgb[3 * i + 2] = (uint8_t)b->pixels[i].blue;
  }
  return rgb;
}

int illume_bitmap_save_png(const illume_bitmap* bitmap, const char* path) {
  CHECK_ARG(bitmap && path, "null argument");
  std::string err;
  const auto rgb = bitmap_rgb8(bitmap);
  if (!save_png_rgb8(path, rgb.data(), (int)bitmap->width, (int)bitmap->height, &err)) { set_error(err); return ILLUME_ERR_IO; }
  return ILLUME_OK;
}

int illume_bitmap_save_ppm(const illume_bitmap* bitmap, const char* path) {
  CHECK_ARG(bitmap && path, "null argument");
  std::string err;
  const auto rgb = bitmap_rgb8(bitmap);
  if (!save_ppm_rgb8(path, rgb.data(), (int)bitmap->width, (int)bitmap->height, &err)) { set_error(err); return ILLUME_ERR_IO; }
  return ILLUME_OK;
}

int illume_save_pfm(const float* rgb, int width, int height, const char* path) {
  CHECK_ARG(rgb && path && width > 0 && height > 0, "bad argument");
  std::string err;
  if (!save_pfm_rgb(path, rgb, width, height, &err)) { set_error(err); return ILLUME_ERR_IO; }
  return ILLUME_OK;
}

int illume_trace_closest_device(illume_context* ctx, illume_scene* scene, const float* d_rays, int n, int intersector,
                                int bvh_kind, illume_hit* d_hits) {
  CHECK_ARG(ctx && scene && (n == 0 || (d_rays && d_hits)) && n >= 0, "bad argument");
  CHECK_ARG(intersector == ILLUME_ISECT_MT || intersector == ILLUME_ISECT_WATERTIGHT, "unknown intersector");
  CHECK_ARG(bvh_kind == ILLUME_BVH_BINARY || bvh_kind == ILLUME_BVH_WIDE8 || bvh_kind == ILLUME_BVH_WIDE8_PERSISTENT ||
                bvh_kind == ILLUME_BVH_WIDE4,
            "unknown BVH kind");
  CHECK_ARG(((uintptr_t)d_rays & 15) == 0, "rays must be 16-byte aligned");
  CHECK_ARG(scene->s.ctx == &ctx->c, "scene was not uploaded with this context");
  cudaSetDevice(ctx->c.device);
  if (bvh_kind == ILLUME_BVH_WIDE8 || bvh_kind == ILLUME_BVH_WIDE8_PERSISTENT) {
    std::string err;
    const int st = scene->s.ensure_wide(&err);
    if (st != ILLUME_OK) { set_error(err.empty() ? std::string(last_error()) : err); return st; }
  }
  launch_trace_hook(scene->s.view, scene->s.view_dev, d_rays, n, intersector, bvh_kind, d_hits, ctx->c.stream);
  ILLUME_CUDA_TRY(cudaGetLastError());
  ctx->c.launches += n > 0 ? 1 : 0;
  return ILLUME_OK;
}

int illume_trace_closest(illume_context* ctx, illume_scene* scene, const float* rays, int n, int intersector,
                         int bvh_kind, illume_hit* hits) {
  CHECK_ARG(ctx && scene && n >= 0 && (n == 0 || (rays && hits)), "bad argument");
  if (n == 0) return ILLUME_OK;
  cudaSetDevice(ctx->c.device);
  DevBuffer dr, dh;
  int st;
  if ((st = dr.upload(&ctx->c, rays, sizeof(float) * 8 * (size_t)n)) != ILLUME_OK) return st;
  if ((st = dh.alloc(&ctx->c, sizeof(illume_hit) * (size_t)n)) != ILLUME_OK) return st;
  if ((st = illume_trace_closest_device(ctx, scene, dr.as<float>(), n, intersector, bvh_kind, dh.as<illume_hit>())) != ILLUME_OK)
    return st;
  ILLUME_CUDA_TRY(cudaMemcpyAsync(hits, dh.get(), sizeof(illume_hit) * (size_t)n, cudaMemcpyDeviceToHost, ctx->c.stream));
  ILLUME_CUDA_TRY(cudaStreamSynchronize(ctx->c.stream));
  return ILLUME_OK;
}

int illume_measure_l2_read(illume_context* ctx, size_t bytes, int reps, double* gbs) {
  CHECK_ARG(ctx && gbs && bytes >= 16 && reps >= 1, "invalid argument");
  cudaSetDevice(ctx->c.device);
  bytes &= ~(size_t)15;
  DevBuffer buf, sink;
  int st;
  if ((st = buf.alloc(&ctx->c, bytes)) != ILLUME_OK) return st;
  if ((st = sink.alloc(&ctx->c, sizeof(unsigned))) != ILLUME_OK) return st;
  cudaStream_t s = ctx->c.stream;
  ILLUME_CUDA_TRY(cudaMemsetAsync(buf.get(), 1, bytes, s));
  const int grid = kernel_grid_blocks(l2_read_kernel_ptr(), 256, ctx->c.device);
  launch_l2_read(buf.get(), bytes, 2, sink.as<unsigned>(), grid, s);   // warm L2
  cudaEvent_t e0, e1;
  ILLUME_CUDA_TRY(cudaEventCreate(&e0));
  ILLUME_CUDA_TRY(cudaEventCreate(&e1));
  cudaEventRecord(e0, s);
  launch_l2_read(buf.get(), bytes, reps, sink.as<unsigned>(), grid, s);
  cudaEventRecord(e1, s);
  const cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ILLUME_CUDA_TRY(e);
  ILLUME_CUDA_TRY(cudaGetLastError());
  *gbs = ms > 0.0f ? (double)bytes * reps / (ms * 1e-3) / 1e9 : 0.0;
  return ILLUME_OK;
}

int illume_alias_table(int n, const double* weights, float* keep, int32_t* alias) {
  CHECK_ARG(n >= 0 && (n == 0 || (weights && keep && alias)), "null argument");
  std::vector<AliasEntry> t(n);
  if (!build_alias(weights, (size_t)n, t.data())) {
    set_error("weights sum to zero");
    return ILLUME_ERR_INVALID;
  }
  for (int i = 0; i < n; ++i) {
    keep[i] = t[i].keep;
    alias[i] = t[i].alias;
  }
  return ILLUME_OK;
}

int illume_bsdf_batch(illume_context* ctx, int material_type, int distribution, const float* inputs, int n,
                      float* outputs) {
  CHECK_ARG(ctx && n >= 0 && (n == 0 || (inputs && outputs)), "bad argument");
  CHECK_ARG(material_type > ILLUME_MAT_EMISSIVE && material_type <= ILLUME_MAT_PLASTIC, "unsupported material type");
  CHECK_ARG(distribution == ILLUME_DIST_BECKMANN || distribution == ILLUME_DIST_GGX, "unknown distribution");
  if (n == 0) return ILLUME_OK;
  cudaSetDevice(ctx->c.device);
  std::vector<float> in(inputs, inputs + 16 * (size_t)n);
  if (material_type == ILLUME_MAT_PLASTIC)
    for (int i = 0; i < n; ++i)
      if (in[16 * (size_t)i + 15] == 0.0f) in[16 * (size_t)i + 15] = plastic_diffuse_fresnel(in[16 * (size_t)i + 10]);
  DevBuffer di, dout;
  int st;
  if ((st = di.upload(&ctx->c, in.data(), sizeof(float) * in.size())) != ILLUME_OK) return st;
  if ((st = dout.alloc(&ctx->c, sizeof(float) * in.size())) != ILLUME_OK) return st;
  launch_bsdf_batch(material_type, distribution, di.as<float>(), n, dout.as<float>(), ctx->c.stream);
  ILLUME_CUDA_TRY(cudaGetLastError());
  ctx->c.launches += 1;
  ILLUME_CUDA_TRY(cudaMemcpyAsync(outputs, dout.get(), sizeof(float) * in.size(), cudaMemcpyDeviceToHost, ctx->c.stream));
  ILLUME_CUDA_TRY(cudaStreamSynchronize(ctx->c.stream));
  return ILLUME_OK;
}

}  // extern "C"
