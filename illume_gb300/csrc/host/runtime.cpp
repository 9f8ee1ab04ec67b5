#include "runtime.h"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <map>
#include <mutex>
#include <thread>

namespace illume {

static thread_local std::string g_error;
void set_error(const std::string& msg) { g_error = msg; }
const char* last_error() { return g_error.c_str(); }

int DevBuffer::alloc(Context* ctx, size_t bytes) {
  release();
  ctx_ = ctx;
  if (bytes == 0) bytes = 16;
  if (ctx->budget && ctx->used.load() + bytes > ctx->budget) {
    set_error("device allocation of " + std::to_string(bytes) + " bytes exceeds the context budget");
    return ILLUME_ERR_BUDGET;
  }
  cudaError_t e = cudaMalloc(&ptr_, bytes);
  if (e != cudaSuccess) {
    ptr_ = nullptr;
    set_error(std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? ILLUME_ERR_OOM : ILLUME_ERR_CUDA;
  }
  bytes_ = bytes;
  ctx->used += bytes;
  return ILLUME_OK;
}

int DevBuffer::upload(Context* ctx, const void* src, size_t bytes) {
  int st = alloc(ctx, bytes);
  if (st != ILLUME_OK) return st;
  if (bytes && src) ILLUME_CUDA_TRY(cudaMemcpyAsync(ptr_, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  return ILLUME_OK;
}

void DevBuffer::release() {
  if (ptr_) {
    cudaFree(ptr_);
    if (ctx_) ctx_->used -= bytes_;
  }
  ptr_ = nullptr;
  bytes_ = 0;
}

// ---------------------------------------------------------------- SceneHost
template <class T>
static void assign_from(std::vector<T>& dst, const T* src, size_t n) {
  dst.assign(src, src + n);
}

int SceneHost::from_desc(const illume_scene_desc& d, std::string* err) {
  if (d.num_meshes < 0 || d.num_instances < 0 || d.num_spheres < 0 || d.num_materials < 0 || d.num_mediums < 0 ||
      d.num_textures < 0) {
    *err = "negative count in scene description";
    return ILLUME_ERR_INVALID;
  }
  const int nm = d.num_meshes;
  if (nm && (!d.mesh_vertex_offset || !d.mesh_num_vertices || !d.mesh_tri_offset || !d.mesh_num_tris ||
             !d.mesh_has_normals || !d.mesh_has_texcoords || !d.positions || !d.tris)) {
    *err = "mesh arrays missing in scene description";
    return ILLUME_ERR_INVALID;
  }
  assign_from(mesh_vertex_offset, d.mesh_vertex_offset, nm);
  assign_from(mesh_num_vertices, d.mesh_num_vertices, nm);
  assign_from(mesh_tri_offset, d.mesh_tri_offset, nm);
  assign_from(mesh_num_tris, d.mesh_num_tris, nm);
  assign_from(mesh_has_normals, d.mesh_has_normals, nm);
  assign_from(mesh_has_texcoords, d.mesh_has_texcoords, nm);
  if (d.mesh_bvh_leaf_size) assign_from(mesh_bvh_leaf_size, d.mesh_bvh_leaf_size, nm);
  else mesh_bvh_leaf_size.assign(nm, 4);
  size_t V = 0, T = 0;
  for (int i = 0; i < nm; ++i) {
    if (mesh_vertex_offset[i] < 0 || mesh_num_vertices[i] < 0 || mesh_tri_offset[i] < 0 || mesh_num_tris[i] < 0) {
      *err = "negative mesh offset or count";
      return ILLUME_ERR_INVALID;
    }
    V = std::max(V, (size_t)mesh_vertex_offset[i] + mesh_num_vertices[i]);
    T = std::max(T, (size_t)mesh_tri_offset[i] + mesh_num_tris[i]);
  }
  assign_from(positions, d.positions, 3 * V);
  bool any_n = false, any_t = false;
  for (int i = 0; i < nm; ++i) { any_n |= mesh_has_normals[i] != 0; any_t |= mesh_has_texcoords[i] != 0; }
  if (any_n && !d.normals) { *err = "normals missing"; return ILLUME_ERR_INVALID; }
  if (any_t && !d.texcoords) { *err = "texcoords missing"; return ILLUME_ERR_INVALID; }
  if (any_n) assign_from(normals, d.normals, 3 * V); else normals.assign(3 * V, 0.0f);
  if (any_t) assign_from(texcoords, d.texcoords, 2 * V); else texcoords.assign(2 * V, 0.0f);
  assign_from(tris, d.tris, 3 * T);
  const int ni = d.num_instances;
  if (ni && (!d.inst_mesh || !d.inst_material || !d.inst_mat || !d.inst_inv || !d.inst_trans_inv)) {
    *err = "instance arrays missing";
    return ILLUME_ERR_INVALID;
  }
  assign_from(inst_mesh, d.inst_mesh, ni);
  assign_from(inst_material, d.inst_material, ni);
  assign_from(inst_mat, d.inst_mat, 12 * (size_t)ni);
  assign_from(inst_inv, d.inst_inv, 12 * (size_t)ni);
  assign_from(inst_trans_inv, d.inst_trans_inv, 12 * (size_t)ni);
  const int ns = d.num_spheres;
  if (ns && (!d.sphere_center_radius || !d.sphere_material)) { *err = "sphere arrays missing"; return ILLUME_ERR_INVALID; }
  assign_from(sphere_center_radius, d.sphere_center_radius, 4 * (size_t)ns);
  assign_from(sphere_material, d.sphere_material, ns);
  const int nmat = d.num_materials;
  if (nmat && (!d.mat_type || !d.mat_albedo_tex || !d.mat_roughness_tex || !d.mat_medium || !d.mat_distribution ||
               !d.mat_ior || !d.mat_diffuse_fresnel || !d.mat_eta || !d.mat_k)) {
    *err = "material arrays missing";
    return ILLUME_ERR_INVALID;
  }
  assign_from(mat_type, d.mat_type, nmat);
  assign_from(mat_albedo_tex, d.mat_albedo_tex, nmat);
  assign_from(mat_roughness_tex, d.mat_roughness_tex, nmat);
  assign_from(mat_medium, d.mat_medium, nmat);
  assign_from(mat_distribution, d.mat_distribution, nmat);
  assign_from(mat_ior, d.mat_ior, nmat);
  assign_from(mat_diffuse_fresnel, d.mat_diffuse_fresnel, nmat);
  assign_from(mat_eta, d.mat_eta, 3 * (size_t)nmat);
  assign_from(mat_k, d.mat_k, 3 * (size_t)nmat);
  const int nmed = d.num_mediums;
  if (nmed && (!d.med_absorption || !d.med_scattering || !d.med_g || !d.med_active)) {
    *err = "medium arrays missing";
    return ILLUME_ERR_INVALID;
  }
  assign_from(med_absorption, d.med_absorption, 3 * (size_t)nmed);
  assign_from(med_scattering, d.med_scattering, nmed);
  assign_from(med_g, d.med_g, nmed);
  assign_from(med_active, d.med_active, nmed);
  const int nt = d.num_textures;
  if (nt && (!d.tex_type || !d.tex_color || !d.tex_off || !d.tex_scale || !d.tex_width || !d.tex_height || !d.tex_hdr ||
             !d.tex_texel_offset)) {
    *err = "texture arrays missing";
    return ILLUME_ERR_INVALID;
  }
  assign_from(tex_type, d.tex_type, nt);
  assign_from(tex_color, d.tex_color, 3 * (size_t)nt);
  assign_from(tex_off, d.tex_off, 3 * (size_t)nt);
  assign_from(tex_scale, d.tex_scale, 2 * (size_t)nt);
  assign_from(tex_width, d.tex_width, nt);
  assign_from(tex_height, d.tex_height, nt);
  assign_from(tex_hdr, d.tex_hdr, nt);
  assign_from(tex_texel_offset, d.tex_texel_offset, nt);
  size_t texel_floats = 0;
  for (int i = 0; i < nt; ++i)
    if (tex_type[i] == TEX_BITMAP) {
      if (tex_width[i] <= 0 || tex_height[i] <= 0 || tex_texel_offset[i] < 0) {
        *err = "bitmap texture with invalid size or offset";
        return ILLUME_ERR_INVALID;
      }
      texel_floats = std::max(texel_floats, (size_t)tex_texel_offset[i] + 4 * (size_t)tex_width[i] * tex_height[i]);
    }
  if (texel_floats && !d.texels) { *err = "texels missing"; return ILLUME_ERR_INVALID; }
  assign_from(texels, d.texels, texel_floats);
  env_tex = d.env_tex;
  memcpy(camera_transform, d.camera_transform, sizeof(camera_transform));
  camera_fov = d.camera_fov;
  camera_dof = d.camera_dof;
  camera_aperture = d.camera_aperture;
  width = d.width;
  height = d.height;
  ray_bias = d.ray_bias;
  tonemapper = d.tonemapper;
  return validate(err);
}

int SceneHost::validate(std::string* err) const {
  const int nm = num_meshes(), nmat = num_materials(), nt = num_textures(), nmed = (int)med_active.size();
  for (int i = 0; i < nm; ++i) {
    const int V = mesh_num_vertices[i];
    for (int t = 0; t < mesh_num_tris[i]; ++t)
      for (int k = 0; k < 3; ++k) {
        const int v = tris[3 * ((size_t)mesh_tri_offset[i] + t) + k];
        if (v < 0 || v >= V) { *err = "triangle vertex index out of range in mesh " + std::to_string(i); return ILLUME_ERR_INVALID; }
      }
  }
  for (size_t i = 0; i < inst_mesh.size(); ++i) {
    if (inst_mesh[i] < 0 || inst_mesh[i] >= nm) { *err = "instance mesh index out of range"; return ILLUME_ERR_INVALID; }
    if (inst_material[i] < 0 || inst_material[i] >= nmat) { *err = "instance material index out of range"; return ILLUME_ERR_INVALID; }
  }
  for (size_t i = 0; i < sphere_material.size(); ++i)
    if (sphere_material[i] < 0 || sphere_material[i] >= nmat) { *err = "sphere material index out of range"; return ILLUME_ERR_INVALID; }
  for (int i = 0; i < nmat; ++i) {
    if (mat_type[i] < 0 || mat_type[i] >= MAT_COUNT) { *err = "unknown material type"; return ILLUME_ERR_INVALID; }
    if (mat_albedo_tex[i] < 0 || mat_albedo_tex[i] >= nt || mat_roughness_tex[i] < 0 || mat_roughness_tex[i] >= nt) {
      *err = "material texture index out of range";
      return ILLUME_ERR_INVALID;
    }
    if (mat_medium[i] < -1 || mat_medium[i] >= nmed) { *err = "material medium index out of range"; return ILLUME_ERR_INVALID; }
  }
  for (int i = 0; i < nt; ++i)
    if (tex_type[i] < 0 || tex_type[i] > 2) { *err = "unknown texture type"; return ILLUME_ERR_INVALID; }
  if (env_tex < -1 || env_tex >= nt) { *err = "environment texture index out of range"; return ILLUME_ERR_INVALID; }
  if (width <= 0 || height <= 0) { *err = "invalid resolution"; return ILLUME_ERR_INVALID; }
  return ILLUME_OK;
}

void SceneHost::to_desc(illume_scene_desc* d) const {
  memset(d, 0, sizeof(*d));
  d->num_meshes = num_meshes();
  d->mesh_vertex_offset = mesh_vertex_offset.data();
  d->mesh_num_vertices = mesh_num_vertices.data();
  d->mesh_tri_offset = mesh_tri_offset.data();
  d->mesh_num_tris = mesh_num_tris.data();
  d->mesh_has_normals = mesh_has_normals.data();
  d->mesh_has_texcoords = mesh_has_texcoords.data();
  d->mesh_bvh_leaf_size = mesh_bvh_leaf_size.data();
  d->positions = positions.data();
  d->normals = normals.data();
  d->texcoords = texcoords.data();
  d->tris = tris.data();
  d->num_instances = (int)inst_mesh.size();
  d->inst_mesh = inst_mesh.data();
  d->inst_material = inst_material.data();
  d->inst_mat = inst_mat.data();
  d->inst_inv = inst_inv.data();
  d->inst_trans_inv = inst_trans_inv.data();
  d->num_spheres = (int)sphere_material.size();
  d->sphere_center_radius = sphere_center_radius.data();
  d->sphere_material = sphere_material.data();
  d->num_materials = num_materials();
  d->mat_type = mat_type.data();
  d->mat_albedo_tex = mat_albedo_tex.data();
  d->mat_roughness_tex = mat_roughness_tex.data();
  d->mat_medium = mat_medium.data();
  d->mat_distribution = mat_distribution.data();
  d->mat_ior = mat_ior.data();
  d->mat_diffuse_fresnel = mat_diffuse_fresnel.data();
  d->mat_eta = mat_eta.data();
  d->mat_k = mat_k.data();
  d->num_mediums = (int)med_active.size();
  d->med_absorption = med_absorption.data();
  d->med_scattering = med_scattering.data();
  d->med_g = med_g.data();
  d->med_active = med_active.data();
  d->num_textures = num_textures();
  d->tex_type = tex_type.data();
  d->tex_color = tex_color.data();
  d->tex_off = tex_off.data();
  d->tex_scale = tex_scale.data();
  d->tex_width = tex_width.data();
  d->tex_height = tex_height.data();
  d->tex_hdr = tex_hdr.data();
  d->tex_texel_offset = tex_texel_offset.data();
  d->texels = texels.empty() ? nullptr : texels.data();
  d->env_tex = env_tex;
  memcpy(d->camera_transform, camera_transform, sizeof(camera_transform));
  d->camera_fov = camera_fov;
  d->camera_dof = camera_dof;
  d->camera_aperture = camera_aperture;
  d->width = width;
  d->height = height;
  d->ray_bias = ray_bias;
  d->tonemapper = tonemapper;
}

// ---------------------------------------------------------------- device scene
static float pad_down(double v, double pad) {
  float f = (float)(v - pad);
  if ((double)f > v - pad) f = nextafterf(f, -INFINITY);
  return f;
}
static float pad_up(double v, double pad) {
  float f = (float)(v + pad);
  if ((double)f < v + pad) f = nextafterf(f, INFINITY);
  return f;
}

// ---- BVH cache keyed by mesh content ----
//
// Scenes that share meshes (instanced assets, a pool of meshes reused across jobs) build
// each distinct mesh once per process. The key is two independent 64-bit hashes of the
// vertex and index words plus the counts; a hit copies the cached build.
namespace {

struct BvhKey {
  uint64_t h1, h2;
  int nv, nt;
  int builder;   // illume_bvh_builder: the device and host builds make different trees
  bool operator<(const BvhKey& o) const {
    if (h1 != o.h1) return h1 < o.h1;
    if (h2 != o.h2) return h2 < o.h2;
    if (nv != o.nv) return nv < o.nv;
    if (nt != o.nt) return nt < o.nt;
    return builder < o.builder;
  }
};

inline uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }

BvhKey mesh_key(const float* P, int nv, const int* T, int nt) {
  uint64_t h1 = 0x243f6a8885a308d3ULL, h2 = 0x13198a2e03707344ULL;
  auto mix = [&](uint32_t w) {
    h1 = rotl64(h1 ^ (w * 0x9e3779b97f4a7c15ULL), 29) * 0xbf58476d1ce4e5b9ULL;
    h2 = rotl64(h2 + (uint64_t)w * 0xc2b2ae3d27d4eb4fULL, 31) ^ (h2 >> 17);
  };
  const uint32_t* pw = reinterpret_cast<const uint32_t*>(P);
  for (size_t i = 0; i < 3 * (size_t)nv; ++i) mix(pw[i]);
  for (size_t i = 0; i < 3 * (size_t)nt; ++i) mix((uint32_t)T[i]);
  return BvhKey{h1, h2, nv, nt, 0};
}

std::mutex g_bvh_mu;
std::map<BvhKey, MeshBvh> g_bvh_cache;
size_t g_bvh_bytes = 0;
long long g_bvh_hits = 0, g_bvh_misses = 0;
constexpr size_t kBvhCacheMaxBytes = size_t(4) << 30;

size_t bvh_bytes(const MeshBvh& b) {
  return b.bvh4.size() * sizeof(Bvh4Node) + b.bvh2.size() * sizeof(Bvh2Node) + b.bvh2_tris.size() * sizeof(float4) + b.wide.size() * sizeof(WideNode) +
         b.wide_tris.size() * sizeof(float4);
}

void build_cached(const float* P, int nv, const int* T, int nt, MeshBvh* out, Context* device) {
  BvhKey key = mesh_key(P, nv, T, nt);
  key.builder = device ? ILLUME_BVH_BUILD_DEVICE : ILLUME_BVH_BUILD_HOST;
  {
    std::lock_guard<std::mutex> lk(g_bvh_mu);
    auto it = g_bvh_cache.find(key);
    if (it != g_bvh_cache.end()) {
      ++g_bvh_hits;
      *out = it->second;
      return;
    }
    ++g_bvh_misses;
  }
  build_mesh_bvh(P, nv, T, nt, out, device, kLayoutBinary4);   // the 8-wide layout on first need
  // a device build that fell back to the host tree is not kept under the device key
  if (device && !out->stats.device_built) return;
  const size_t bytes = bvh_bytes(*out);
  std::lock_guard<std::mutex> lk(g_bvh_mu);
  if (bytes > kBvhCacheMaxBytes) return;
  if (g_bvh_bytes + bytes > kBvhCacheMaxBytes) {
    g_bvh_cache.clear();
    g_bvh_bytes = 0;
  }
  if (g_bvh_cache.emplace(key, *out).second) g_bvh_bytes += bytes;
}

}  // namespace

void bvh_cache_stats(long long* entries, long long* bytes, long long* hits, long long* misses) {
  std::lock_guard<std::mutex> lk(g_bvh_mu);
  *entries = (long long)g_bvh_cache.size();
  *bytes = (long long)g_bvh_bytes;
  *hits = g_bvh_hits;
  *misses = g_bvh_misses;
}

void bvh_cache_clear() {
  std::lock_guard<std::mutex> lk(g_bvh_mu);
  g_bvh_cache.clear();
  g_bvh_bytes = 0;
}

// Builds every mesh's BVHs, distinct meshes in parallel on the host cores.
int Scene::build_host(std::string* err) {
  auto t0 = std::chrono::steady_clock::now();
  const SceneHost& h = host;
  const int nm = h.num_meshes();
  for (int i = 0; i < nm; ++i)
    if (h.mesh_num_tris[i] >= (1 << 28)) {   // leaf codes hold the first triangle in 28 bits
      *err = "mesh " + std::to_string(i) + " has 2^28 or more triangles";
      return ILLUME_ERR_UNSUPPORTED;
    }
  bvhs.assign(nm, MeshBvh{});
  Context* device = ctx && ctx->bvh_builder == ILLUME_BVH_BUILD_DEVICE ? ctx : nullptr;
  const int nthreads = std::max(1, std::min<int>(nm, build_threads()));
  const int share = build_thread_share(h.mesh_num_tris.data(), nm, nthreads);
  std::vector<std::thread> pool;
  std::atomic<int> next{0};
  auto work = [&]() {
    const BuildThreadShare scope(share);
    for (int i = next++; i < nm; i = next++) {
      const float* P = h.positions.data() + 3 * (size_t)h.mesh_vertex_offset[i];
      const int* T = h.tris.data() + 3 * (size_t)h.mesh_tri_offset[i];
      build_cached(P, h.mesh_num_vertices[i], T, h.mesh_num_tris[i], &bvhs[i], device);
    }
  };
  for (int t = 1; t < nthreads; ++t) pool.emplace_back(work);
  work();
  for (auto& th : pool) th.join();
  for (int i = 0; i < nm; ++i) {
    if (bvhs[i].stats.bvh2_depth > 60) {
      *err = "binary BVH deeper than the traversal stack (mesh " + std::to_string(i) + ")";
      return ILLUME_ERR_UNSUPPORTED;
    }
    if (3 * bvhs[i].stats.bvh4_depth > 60) {   // up to 3 entries pushed per 4-wide level
      *err = "4-wide BVH deeper than the traversal stack (mesh " + std::to_string(i) + ")";
      return ILLUME_ERR_UNSUPPORTED;
    }
  }
  trace_bytes[0] = trace_bytes[1] = trace_bytes[2] = 0;
  for (const MeshBvh& b : bvhs) {
    trace_bytes[0] += b.bvh2.size() * sizeof(Bvh2Node) + b.bvh2_tris.size() * sizeof(float4);
    trace_bytes[2] += b.bvh4.size() * sizeof(Bvh4Node) + b.bvh2_tris.size() * sizeof(float4);
    trace_bytes[1] += b.wide.size() * sizeof(WideNode) + b.wide_tris.size() * sizeof(float4);
  }
  build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return ILLUME_OK;
}

int Scene::build_and_upload(std::string* err) {
  const SceneHost& h = host;
  const int nm = h.num_meshes();
  const int bst = build_host(err);
  if (bst != ILLUME_OK) return bst;
  auto t1 = std::chrono::steady_clock::now();

  // resident: uploaded once (textures, light tables), like the reference's texture
  // objects, which HostScene creates once; the rest is what SceneRef copies per render
  bool resident = false;
  auto up = [&](const void* src, size_t bytes, void** out) -> int {
    buffers.emplace_back(new DevBuffer);
    int st = buffers.back()->upload(ctx, src, bytes);
    if (st != ILLUME_OK) return st;
    *out = buffers.back()->get();
    uploads.push_back({*out, src, bytes, resident});
    device_bytes += buffers.back()->size();
    return ILLUME_OK;
  };
#define UP(src, bytes, dst)                                  \
  do {                                                       \
    void* p_ = nullptr;                                      \
    int st_ = up((src), (bytes), &p_);                       \
    if (st_ != ILLUME_OK) { *err = last_error(); return st_; } \
    dst = reinterpret_cast<decltype(dst)>(p_);               \
  } while (0)

  std::vector<DevMesh>& meshes = t_meshes;
  meshes.assign(nm, DevMesh{});
  for (int i = 0; i < nm; ++i) {
    const MeshBvh& b = bvhs[i];
    DevMesh& m = meshes[i];
    memset(&m, 0, sizeof(m));
    UP(b.bvh2.data(), b.bvh2.size() * sizeof(Bvh2Node), m.bvh2);
    UP(b.bvh4.data(), b.bvh4.size() * sizeof(Bvh4Node), m.bvh4);
    UP(b.wide.data(), b.wide.size() * sizeof(WideNode), m.wide);
    UP(b.bvh2_tris.data(), b.bvh2_tris.size() * sizeof(float4), m.bvh2_tris);
    UP(b.wide_tris.data(), b.wide_tris.size() * sizeof(float4), m.wide_tris);
    const size_t vo = h.mesh_vertex_offset[i], V = h.mesh_num_vertices[i];
    UP(h.tris.data() + 3 * (size_t)h.mesh_tri_offset[i], 3 * sizeof(int) * (size_t)h.mesh_num_tris[i], m.tris);
    UP(h.positions.data() + 3 * vo, 3 * sizeof(float) * V, m.positions);
    if (h.mesh_has_normals[i]) UP(h.normals.data() + 3 * vo, 3 * sizeof(float) * V, m.normals);
    if (h.mesh_has_texcoords[i]) UP(h.texcoords.data() + 2 * vo, 2 * sizeof(float) * V, m.texcoords);
    m.num_tris = h.mesh_num_tris[i];
    m.bvh2_root_leaf = b.root_leaf ? 1 : 0;
  }
  const int ni = (int)h.inst_mesh.size();
  std::vector<DevInstance>& inst = t_instances;
  inst.assign(ni, DevInstance{});
  for (int i = 0; i < ni; ++i) {
    DevInstance& d = inst[i];
    memcpy(d.inv, h.inst_inv.data() + 12 * (size_t)i, 48);
    memcpy(d.trans_inv, h.inst_trans_inv.data() + 12 * (size_t)i, 48);
    d.mesh = h.inst_mesh[i];
    d.material = h.inst_material[i];
    // world bounds: the 8 corners of the padded object bounds through mat, padded again
    const MeshBvh& b = bvhs[d.mesh];
    const float* M = h.inst_mat.data() + 12 * (size_t)i;
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < 8; ++c) {
      const double p[3] = {(c & 1) ? b.hi[0] : b.lo[0], (c & 2) ? b.hi[1] : b.lo[1], (c & 4) ? b.hi[2] : b.lo[2]};
      for (int r = 0; r < 3; ++r) {
        const double w = M[4 * r] * p[0] + M[4 * r + 1] * p[1] + M[4 * r + 2] * p[2] + M[4 * r + 3];
        lo[r] = std::min(lo[r], w);
        hi[r] = std::max(hi[r], w);
      }
    }
    double ext = 0, mag = 0;
    for (int r = 0; r < 3; ++r) { ext = std::max(ext, hi[r] - lo[r]); mag = std::max(mag, std::max(fabs(lo[r]), fabs(hi[r]))); }
    const double pad = 1e-4 * (ext + mag) + 1e-30;
    for (int r = 0; r < 3; ++r) { d.lo[r] = pad_down(lo[r], pad); d.hi[r] = pad_up(hi[r], pad); }
    if (b.stats.bvh2_nodes == 0 && h.mesh_num_tris[d.mesh] == 0)
      for (int r = 0; r < 3; ++r) { d.lo[r] = INFINITY; d.hi[r] = -INFINITY; }
  }
  const int ns = (int)h.sphere_material.size();
  std::vector<DevSphere>& spheres = t_spheres;
  spheres.assign(ns, DevSphere{});
  for (int i = 0; i < ns; ++i) {
    spheres[i].cx = h.sphere_center_radius[4 * i];
    spheres[i].cy = h.sphere_center_radius[4 * i + 1];
    spheres[i].cz = h.sphere_center_radius[4 * i + 2];
    spheres[i].r = h.sphere_center_radius[4 * i + 3];
    spheres[i].material = h.sphere_material[i];
  }
  const int nmat = h.num_materials();
  std::vector<DevMaterial>& mats = t_materials;
  mats.assign(nmat, DevMaterial{});
  for (int i = 0; i < nmat; ++i) {
    DevMaterial& m = mats[i];
    memset(&m, 0, sizeof(m));
    m.type = h.mat_type[i];
    m.albedo_tex = h.mat_albedo_tex[i];
    m.roughness_tex = h.mat_roughness_tex[i];
    m.medium = h.mat_medium[i];
    m.distribution = h.mat_distribution[i];
    m.ior = h.mat_ior[i];
    m.diffuse_fresnel = h.mat_diffuse_fresnel[i];
    for (int c = 0; c < 3; ++c) { m.eta[c] = h.mat_eta[3 * i + c]; m.k[c] = h.mat_k[3 * i + c]; }
  }
  const int nmed = (int)h.med_active.size();
  std::vector<DevMedium>& meds = t_mediums;
  meds.assign(nmed, DevMedium{});
  for (int i = 0; i < nmed; ++i) {
    memset(&meds[i], 0, sizeof(DevMedium));
    for (int c = 0; c < 3; ++c) meds[i].absorption[c] = h.med_absorption[3 * i + c];
    meds[i].scattering = h.med_scattering[i];
    meds[i].g = h.med_g[i];
    meds[i].active = h.med_active[i];
  }
  float4* texels = nullptr;
  resident = true;
  if (!h.texels.empty()) UP(h.texels.data(), h.texels.size() * sizeof(float), texels);
  resident = false;
  const int nt = h.num_textures();
  std::vector<DevTexture>& texs = t_textures;
  texs.assign(nt, DevTexture{});
  for (int i = 0; i < nt; ++i) {
    DevTexture& t = texs[i];
    memset(&t, 0, sizeof(t));
    t.type = h.tex_type[i];
    t.width = h.tex_width[i];
    t.height = h.tex_height[i];
    t.hdr = h.tex_hdr[i];
    for (int c = 0; c < 3; ++c) { t.c[c] = h.tex_color[3 * i + c]; t.off[c] = h.tex_off[3 * i + c]; }
    t.scale[0] = h.tex_scale[2 * i];
    t.scale[1] = h.tex_scale[2 * i + 1];
    if (t.type == TEX_BITMAP) {
      if (h.tex_texel_offset[i] % 4 != 0) { *err = "texel offset must be a multiple of 4 floats"; return ILLUME_ERR_INVALID; }
      t.texels = texels + h.tex_texel_offset[i] / 4;
    }
  }
  SceneView v{};
  UP(meshes.data(), meshes.size() * sizeof(DevMesh), v.meshes);
  UP(inst.data(), inst.size() * sizeof(DevInstance), v.instances);
  UP(spheres.data(), spheres.size() * sizeof(DevSphere), v.spheres);
  UP(mats.data(), mats.size() * sizeof(DevMaterial), v.materials);
  UP(texs.data(), texs.size() * sizeof(DevTexture), v.textures);
  UP(meds.data(), meds.size() * sizeof(DevMedium), v.mediums);
  v.num_meshes = nm;
  v.num_instances = ni;
  v.num_spheres = ns;
  v.num_materials = nmat;
  v.env_tex = h.env_tex;
  // light sampling tables of the next-event estimator
  build_lights(h, &lights_host);
  resident = true;
  {
    const HostLights& L = lights_host;
    LightView lv{};
    lv.env_w = L.env_w;
    lv.env_h = L.env_h;
    lv.env_integral = L.env_integral;
    lv.env_prob = L.env_prob;
    if (L.env_w > 0) {
      UP(L.env_func.data(), L.env_func.size() * sizeof(float), lv.env_func);
      UP(L.env_rows.data(), L.env_rows.size() * sizeof(AliasEntry), lv.env_rows);
      UP(L.env_cols.data(), L.env_cols.size() * sizeof(AliasEntry), lv.env_cols);
    }
    lv.num_tri = (int)L.tri_alias.size();
    if (lv.num_tri > 0) {
      UP(L.tri.data(), L.tri.size() * sizeof(float4), lv.tri);
      UP(L.tri_alias.data(), L.tri_alias.size() * sizeof(AliasEntry), lv.tri_alias);
    }
    if (!L.inst_light_base.empty()) UP(L.inst_light_base.data(), L.inst_light_base.size() * sizeof(int), lv.inst_light_base);
    lights_view = lv;
    UP(&lights_view, sizeof(LightView), v.lights);
  }
  resident = false;
#undef UP
  view = v;
  {
    void* p_ = nullptr;
    const int st_ = up(&view, sizeof(SceneView), &p_);
    if (st_ != ILLUME_OK) { *err = last_error(); return st_; }
    view_dev = reinterpret_cast<SceneView*>(p_);
  }
  ILLUME_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  upload_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t1).count();
  pin_upload_sources();
  return ILLUME_OK;
}

int Scene::ensure_wide(std::string* err) {
  std::lock_guard<std::mutex> lk(wide_mu);
  const SceneHost& h = host;
  const int nm = h.num_meshes();
  std::vector<int> todo;
  for (int i = 0; i < nm && i < (int)bvhs.size(); ++i)
    if (!bvhs[i].has_wide) todo.push_back(i);
  if (todo.empty()) return ILLUME_OK;
  std::atomic<int> next{0};
  std::vector<int> sizes;
  for (int i : todo) sizes.push_back(h.mesh_num_tris[i]);
  const int nthreads = std::max(1, std::min<int>((int)todo.size(), build_threads()));
  const int share = build_thread_share(sizes.data(), (int)sizes.size(), nthreads);
  auto work = [&]() {
    const BuildThreadShare scope(share);
    for (int k = next++; k < (int)todo.size(); k = next++) {
      const int i = todo[k];
      const float* P = h.positions.data() + 3 * (size_t)h.mesh_vertex_offset[i];
      const int* T = h.tris.data() + 3 * (size_t)h.mesh_tri_offset[i];
      build_mesh_bvh(P, h.mesh_num_vertices[i], T, h.mesh_num_tris[i], &bvhs[i], nullptr, kLayoutWide);
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nthreads; ++t) pool.emplace_back(work);
  work();
  for (auto& th : pool) th.join();
  trace_bytes[1] = 0;
  for (const MeshBvh& b : bvhs) trace_bytes[1] += b.wide.size() * sizeof(WideNode) + b.wide_tris.size() * sizeof(float4);
  if (!ctx) return ILLUME_OK;
  ILLUME_CUDA_TRY(cudaSetDevice(ctx->device));
  // resident uploads: a per-render re-upload (upload_again) leaves them alone
  auto up = [&](const void* src, size_t bytes, void** out) -> int {
    buffers.emplace_back(new DevBuffer);
    const int st = buffers.back()->upload(ctx, src, bytes);
    if (st != ILLUME_OK) return st;
    *out = buffers.back()->get();
    uploads.push_back({*out, src, bytes, true});
    device_bytes += buffers.back()->size();
    return ILLUME_OK;
  };
  for (int i : todo) {
    const MeshBvh& b = bvhs[i];
    void* pw = nullptr;
    void* pt = nullptr;
    int st = up(b.wide.data(), b.wide.size() * sizeof(WideNode), &pw);
    if (st == ILLUME_OK) st = up(b.wide_tris.data(), b.wide_tris.size() * sizeof(float4), &pt);
    if (st != ILLUME_OK) { *err = last_error(); return st; }
    t_meshes[i].wide = reinterpret_cast<const WideNode*>(pw);
    t_meshes[i].wide_tris = reinterpret_cast<const float4*>(pt);
  }
  // the mesh table: the source the per-render re-uploads copy from, then its device copy
  for (Upload& u : uploads)
    if (u.dst == (const void*)view.meshes) {
      if (u.src != t_meshes.data()) memcpy(const_cast<void*>(u.src), t_meshes.data(), u.bytes);
      break;
    }
  ILLUME_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  ILLUME_CUDA_TRY(cudaMemcpy(const_cast<DevMesh*>(view.meshes), t_meshes.data(), sizeof(DevMesh) * (size_t)nm,
                             cudaMemcpyHostToDevice));
  return ILLUME_OK;
}

void Scene::pin_upload_sources() {
  size_t total = 0;
  for (const Upload& u : uploads)
    if (!u.resident && u.src && u.bytes) total += (u.bytes + 255) & ~(size_t)255;
  if (total == 0) return;
  void* p = nullptr;
  if (cudaHostAlloc(&p, total, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();   // keep the pageable sources
    return;
  }
  pinned.p = p;
  pinned.bytes = total;
  char* at = static_cast<char*>(p);
  for (Upload& u : uploads) {
    if (u.resident || !u.src || !u.bytes) continue;
    memcpy(at, u.src, u.bytes);
    u.src = at;
    at += (u.bytes + 255) & ~(size_t)255;
  }
}

int Scene::upload_again(size_t* bytes) {
  size_t total = 0;
  for (const Upload& u : uploads) {
    if (u.resident) continue;
    if (u.bytes && u.src) ILLUME_CUDA_TRY(cudaMemcpyAsync(u.dst, u.src, u.bytes, cudaMemcpyHostToDevice, ctx->stream));
    total += u.bytes;
  }
  ILLUME_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (bytes) *bytes = total;
  return ILLUME_OK;
}

// Fresnel::dielectric (src/fresnel.h:10-26) and the hemispherical integral that calls
// it with its arguments in the order src/fresnel.h:68 passes them.
static float dielectric_f(float cosI, float ior, float& cosT) {
  const float eta = cosI < 0.0f ? ior : 1.0f / ior;
  const float sinTSq = eta * eta * (1.0f - cosI * cosI);
  if (sinTSq >= 1.0f) { cosT = 0.0f; return 1.0f; }
  cosI = fabsf(cosI);
  cosT = sqrtf(1.0f - sinTSq);
  const float rperp = (eta * cosI - cosT) / (eta * cosI + cosT);
  const float rpar = (cosI - eta * cosT) / (cosI + eta * cosT);
  return (rperp * rperp + rpar * rpar) * 0.5f;
}

float plastic_diffuse_fresnel(float ior_in) {
  static std::mutex mu;
  static std::map<float, float> cache;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(ior_in);
    if (it != cache.end()) return it->second;
  }
  const float ior = 1.0f / ior_in;
  const int samples = 1000000;
  float cosT;
  double ret = 0.0;
  float fb = dielectric_f(0.0f, ior, cosT);
  for (int i = 1; i <= samples; i++) {
    const float cosTSq = (float)i / samples;
    const float fa = dielectric_f(ior, sqrtf(cosTSq), cosT);
    ret += (double)(fa + fb) * (0.5 / samples);
    fb = fa;
  }
  std::lock_guard<std::mutex> lk(mu);
  cache[ior_in] = (float)ret;
  return (float)ret;
}

}  // namespace illume
