// Host runtime of the C-ABI: context (device, stream, HBM budget), device buffers,
// scenes (host copy + device tables + BVHs) and the error channel.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../common/types.h"
#include "bvh_build.h"
#include "lights.h"
#include "../../../include/illume.h"

namespace illume {

// Thread-local message of the last failing call (illume_last_error).
void set_error(const std::string& msg);
const char* last_error();

#define ILLUME_CUDA_TRY(expr)                                                                 \
  do {                                                                                        \
    cudaError_t e_ = (expr);                                                                  \
    if (e_ != cudaSuccess) {                                                                  \
      set_error(std::string(#expr) + ": " + cudaGetErrorString(e_));                          \
      return e_ == cudaErrorMemoryAllocation ? ILLUME_ERR_OOM : ILLUME_ERR_CUDA;              \
    }                                                                                         \
  } while (0)

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  size_t budget = 0;                 // 0 = unlimited
  std::atomic<size_t> used{0};
  int sm_count = 0;
  int l2_bytes = 0;
  int bvh_builder = 0;               // illume_bvh_builder of the scenes made on this context
  std::atomic<long long> launches{0};
  // illume_render_noalloc's set-up on this context: the device address of its fixed
  // scratch array, the driver context it was looked up in, and grid sizes per kernel
  // (trace by BVH kind and variant, shade by variant; 0 = not yet computed)
  void* noalloc_scratch = nullptr;
  void* noalloc_cu_ctx = nullptr;
  int noalloc_grid_trace[4][8] = {};
  int noalloc_grid_shade[8] = {};
};

// Device allocation charged against the context's budget.
class DevBuffer {
 public:
  DevBuffer() = default;
  DevBuffer(const DevBuffer&) = delete;
  DevBuffer& operator=(const DevBuffer&) = delete;
  ~DevBuffer() { release(); }
  int alloc(Context* ctx, size_t bytes);
  int upload(Context* ctx, const void* src, size_t bytes);  // alloc + async copy on the context stream
  void release();
  void* get() const { return ptr_; }
  size_t size() const { return bytes_; }
  template <class T> T* as() const { return reinterpret_cast<T*>(ptr_); }

 private:
  Context* ctx_ = nullptr;
  void* ptr_ = nullptr;
  size_t bytes_ = 0;
};

// Owned copy of a scene in the layout of illume_scene_desc.
struct SceneHost {
  std::vector<int32_t> mesh_vertex_offset, mesh_num_vertices, mesh_tri_offset, mesh_num_tris, mesh_has_normals,
      mesh_has_texcoords, mesh_bvh_leaf_size;
  std::vector<float> positions, normals, texcoords;
  std::vector<int32_t> tris;
  std::vector<int32_t> inst_mesh, inst_material;
  std::vector<float> inst_mat, inst_inv, inst_trans_inv;
  std::vector<float> sphere_center_radius;
  std::vector<int32_t> sphere_material;
  std::vector<int32_t> mat_type, mat_albedo_tex, mat_roughness_tex, mat_medium, mat_distribution;
  std::vector<float> mat_ior, mat_diffuse_fresnel, mat_eta, mat_k;
  std::vector<float> med_absorption, med_scattering, med_g;
  std::vector<int32_t> med_active;
  std::vector<int32_t> tex_type, tex_width, tex_height, tex_hdr;
  std::vector<float> tex_color, tex_off, tex_scale;
  std::vector<int64_t> tex_texel_offset;
  std::vector<float> texels;
  int32_t env_tex = -1;
  float camera_transform[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  float camera_fov = 40.0f, camera_dof = 1.0f, camera_aperture = 0.0f;
  int32_t width = 512, height = 512;
  float ray_bias = 0.0f;
  int32_t tonemapper = 0;
  std::vector<std::string> warnings;

  int num_meshes() const { return (int)mesh_num_tris.size(); }
  int num_materials() const { return (int)mat_type.size(); }
  int num_textures() const { return (int)tex_type.size(); }
  // Copies and validates a caller description; returns ILLUME_OK or an error status.
  int from_desc(const illume_scene_desc& d, std::string* err);
  void to_desc(illume_scene_desc* d) const;
  int validate(std::string* err) const;
};

struct Scene {
  Context* ctx = nullptr;
  SceneHost host;
  std::vector<MeshBvh> bvhs;
  std::vector<std::unique_ptr<DevBuffer>> buffers;
  SceneView view{};
  SceneView* view_dev = nullptr;   // device copy of `view`
  HostLights lights_host;           // light sampling tables (host copies)
  LightView lights_view{};          // host source of the device light view
  size_t device_bytes = 0;
  size_t trace_bytes[3] = {0, 0, 0};   // node + triangle bytes a traversal reads: binary, 8-wide, 4-wide
  // device tables (kept for re-uploads) and the host source of every device buffer
  std::vector<DevMesh> t_meshes;
  std::vector<DevInstance> t_instances;
  std::vector<DevSphere> t_spheres;
  std::vector<DevMaterial> t_materials;
  std::vector<DevTexture> t_textures;
  std::vector<DevMedium> t_mediums;
  struct Upload { void* dst; const void* src; size_t bytes; bool resident; };
  std::vector<Upload> uploads;
  // Page-locked copy of the per-render (non-resident) sources, made once after the build
  // (the host tables never change afterwards), so that re-uploads are DMA copies from
  // pinned memory; the sources stay pageable if it cannot be allocated.
  struct PinnedCopy {
    void* p = nullptr;
    size_t bytes = 0;
    PinnedCopy() = default;
    PinnedCopy(const PinnedCopy&) = delete;
    PinnedCopy& operator=(const PinnedCopy&) = delete;
    ~PinnedCopy() { if (p) cudaFreeHost(p); }
  } pinned;
  void pin_upload_sources();
  int upload_again(size_t* bytes);
  double build_ms = 0.0, upload_ms = 0.0;
  int build_host(std::string* err);        // BVHs only (host-only scenes)
  int build_and_upload(std::string* err);  // BVHs + device tables
  // The 8-wide layout of every mesh, built on first need (an 8-wide render, trace, check
  // or digest) on the host cores and, for a scene on a device, uploaded (resident) with
  // the device mesh table pointed at it. Renders of other layouts never wait for it.
  int ensure_wide(std::string* err);
  std::mutex wide_mu;
};

// Process-wide cache of mesh BVH builds keyed by mesh content (runtime.cpp).
void bvh_cache_stats(long long* entries, long long* bytes, long long* hits, long long* misses);
void bvh_cache_clear();

// JSON scene ingest (src/scene/scene.cpp:11-99 and the *_from_json functions it calls).
int load_scene_json(const std::string& text, const std::string& base_dir, SceneHost* out, std::string* err);

// Plastic's diffuse Fresnel constant, Fresnel::diffuse_fresnel(1 / ior, 1000000)
// (src/fresnel.h:59-73, src/material.cu:172-177).
float plastic_diffuse_fresnel(float ior);

}  // namespace illume
