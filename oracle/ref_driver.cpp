// Host driver for the reference renderer's own sources, compiled unchanged from the
// reference checkout together with oracle/ref_shim/ (one translation unit).
//
// TEST INFRASTRUCTURE ONLY: built by oracle/build_ref.py into oracle/_ref/ in the build
// container, where the reference sources exist. It pins the oracle (oracle/oracle.h)
// and generates the golden fixtures under tests/golden/. The product never links it.
//
// Three source-level incompatibilities of the reference with g++ are handled here
// without editing the sources:
//  * jsonutils.h:36,46 names a parameter `default`: the header is included once with
//    `default` defined to another identifier, after every header it pulls in.
//  * math/transform.h:4 includes "rapidjson\document.h": build_ref.py writes a file of
//    that literal name into oracle/_ref/inc that forwards to rapidjson/document.h.
//  * math/vector2.h:12-28 and math/transform.cu:38 bind temporaries to non-const
//    references: const-reference / rvalue overloads declared below are picked instead,
//    with the same arithmetic.
// The per-index kernel loop below restates Renderer::render_to_bitmap
// (src/renderer.cu:498-597): spp passes, max_depth bounce launches, host compaction.

#include <string>
#include <vector>
#include <map>
#include <unordered_map>
#include <fstream>
#include <sstream>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <unistd.h>
#include <omp.h>

#include "illume_ref_shim.h"

thread_local uint3 blockIdx = {0, 0, 0};
thread_local uint3 threadIdx = {0, 0, 0};
thread_local uint3 blockDim = {1, 1, 1};
double illume_shim_now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

#include "rapidjson/document.h"
#include "rapidjson/error/en.h"
#include "math/vector3.h"
#include "math/vector2.h"

#define default default_value_
#include "jsonutils.h"
#undef default

inline Vec2f operator+(const Vec2f& a, const Vec2f& b) { return Vec2f(a.x + b.x, a.y + b.y); }

#include "math/transform.h"
Transform transform_from_matrix(Matrix4&& m);

// ---- the reference sources (unity build) ----
#include "math/vector3.cu"
#include "math/ray.cu"
#include "math/aabb.cu"
#include "math/matrix4.cu"
#include "math/sample.cu"
#include "math/transform.cu"
#include "jsonutils.cpp"
#include "medium.cu"
#include "texture.cu"
#include "material.cu"
#include "microfacet.cu"
#include "hit.cu"
#include "camera.cu"
#include "tonemapper.cu"
#include "accel/bvh.cpp"
#include "primitives/sphere.cu"
#include "primitives/mesh.cu"
#include "primitives/mesh_instance.cu"
#include "scene/scene.cpp"
#include "scene/sceneref.cpp"
#include "imageio.cpp"
#include "renderer.cu"

Transform transform_from_matrix(Matrix4&& m) { return transform_from_matrix(static_cast<Matrix4&>(m)); }

// Renderer keeps its settings private; these mirror the fields it reads from
// render_settings (src/renderer.cu:39-59) so the driver can restate render_to_bitmap.
struct RefHandle {
  rapidjson::Document doc;
  HostScene* scene = nullptr;
  SceneRef* ref = nullptr;
  Tonemapper tonemapper;
  int width = 512, height = 512;
  float ray_bias = 0.0f;
  Texture env_override;
  bool has_env_override = false;
};

// Flat copy of the loaded scene in the layout of illume_scene_desc (include/illume.h).
struct RefExport {
  std::vector<int32_t> mvo, mnv, mto, mnt, mhn, mht, mls, tris, inst_mesh, inst_mat, sph_mat;
  std::vector<int32_t> mat_type, mat_alb, mat_rough, mat_med, mat_dist, med_active;
  std::vector<int32_t> tex_type, tex_w, tex_h, tex_hdr;
  std::vector<int64_t> tex_off;
  std::vector<float> pos, nrm, tc, imat, iinv, itinv, sph, mat_ior, mat_df, mat_eta, mat_k;
  std::vector<float> med_abs, med_sc, med_g, tex_c, tex_o, tex_s, texels;
};
#include "../include/illume.h"

struct RefHandle;
static RefExport* export_scene(RefHandle* h, illume_scene_desc* d);

static void set_index(int index) {
  blockIdx.x = 0;
  blockDim.x = 1;
  threadIdx.x = (unsigned)index;
}

extern "C" {

void* ref_scene_load(const char* json_path, const char* work_dir) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof(cwd))) return nullptr;
  if (work_dir && chdir(work_dir) != 0) return nullptr;
  RefHandle* h = new RefHandle;
  JsonUtils::read_and_parse_json(json_path, h->doc);
  h->scene = new HostScene(h->doc);
  auto rs = h->doc.FindMember("render_settings");
  if (rs != h->doc.MemberEnd()) {
    JsonUtils::from_json(rs->value, "ray_bias", h->ray_bias);
    h->tonemapper = Tonemapper(rs->value);
    auto res = rs->value.FindMember("resolution");
    if (res != rs->value.MemberEnd()) {
      h->width = res->value.GetArray()[0].GetInt();
      h->height = res->value.GetArray()[1].GetInt();
    }
  }
  h->ref = new SceneRef(*h->scene);
  if (chdir(cwd) != 0) return h;
  return h;
}

// Replaces the scene's environment texture by an RGBA float image (HDR bitmap path,
// src/texture.cu:49-56 after the file decode).
int ref_scene_set_env(void* hp, const float* rgba, int w, int hgt) {
  RefHandle* h = (RefHandle*)hp;
  float* copy = (float*)malloc(sizeof(float) * 4 * (size_t)w * hgt);
  memcpy(copy, rgba, sizeof(float) * 4 * (size_t)w * hgt);
  h->env_override = texture_bitmap<float4>(copy, w, hgt, Vec2f(1, 1), true);
  h->ref->getScene()->envmap = h->env_override;
  h->has_env_override = true;
  return 0;
}

void ref_scene_info(void* hp, int* w, int* hgt, float* ray_bias) {
  RefHandle* h = (RefHandle*)hp;
  *w = h->width; *hgt = h->height; *ray_bias = h->ray_bias;
}

void ref_scene_free(void* hp) {
  RefHandle* h = (RefHandle*)hp;
  if (!h) return;
  if (h->has_env_override) h->env_override.destroy();
  delete h->ref;
  delete h->scene;
  delete h;
}

// Renders passes [sample_begin, sample_begin + spp) of an image of width x height
// (0 = the scene's resolution). out_sum (W*H*3) receives the sum over those passes of
// final_colors; out_sumsq the sum of squared per-pass contributions (nullable).
// Returns the number of rays traced, counted as src/renderer.cu:554 counts them.
long long ref_render(void* hp, int width, int height, int spp, int sample_begin, int max_depth,
                     uint32_t seed, uint32_t job, float ray_bias_override, int use_bias_override,
                     float* out_sum, float* out_sumsq, int nthreads) {
  RefHandle* h = (RefHandle*)hp;
  const int W = width > 0 ? width : h->width;
  const int H = height > 0 ? height : h->height;
  const float bias = use_bias_override ? ray_bias_override : h->ray_bias;
  const int N = W * H;
  if (nthreads > 0) omp_set_num_threads(nthreads);

  RenderInfo* info = allocate_render_info_gpu(W, H, h->scene->get_camera());
  DeviceScene* scene = h->ref->getScene();
  std::vector<curandState> states(N);
  std::vector<Ray> rays(N);
  std::vector<int> statuses(N), host_statuses(N);
  std::vector<Vector3> colors(N), finals(N);
  std::vector<Medium> mediums(N);
  std::vector<double> sum((size_t)N * 3, 0.0), sumsq((size_t)N * 3, 0.0);
  long long total_rays = 0;

  for (int s = sample_begin; s < sample_begin + spp; ++s) {
    for (int i = 0; i < N; ++i) {
      states[i] = curandState{(uint32_t)i, (uint32_t)s, 0u, seed, job, 0u, {0, 0, 0, 0}};
      finals[i] = vector3_create(0, 0, 0);
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < N; ++i) {
      set_index(i);
      init_rays(rays.data(), statuses.data(), colors.data(), mediums.data(), info, states.data(), N);
    }
    int active = N;
    for (int j = 0; j < max_depth; ++j) {
      for (int i = 0; i < N; ++i) { states[i].slot = (uint32_t)(j + 1); states[i].dim = 0; }
#pragma omp parallel for schedule(dynamic, 256)
      for (int i = 0; i < active; ++i) {
        set_index(i);
        pathtrace_kernel(finals.data(), rays.data(), statuses.data(), colors.data(), mediums.data(),
                         j, scene, states.data(), bias, active);
      }
      total_rays += active;
      compact_pixels(statuses.data(), host_statuses.data(), &active);
    }
    for (int i = 0; i < N; ++i) {
      const double c[3] = {finals[i].x, finals[i].y, finals[i].z};
      for (int k = 0; k < 3; ++k) {
        sum[(size_t)i * 3 + k] += c[k];
        sumsq[(size_t)i * 3 + k] += c[k] * c[k];
      }
    }
  }
  for (size_t k = 0; k < (size_t)N * 3; ++k) {
    out_sum[k] = (float)sum[k];
    if (out_sumsq) out_sumsq[k] = (float)sumsq[k];
  }
  cudaFree(info);
  return total_rays;
}

// Tonemaps mean radiance (sum / samples) like the tonemap kernel (src/renderer.cu:426-441).
void ref_tonemap_image(void* hp, const float* sum, int n, float samples, int op_override, unsigned char* out_rgb8) {
  RefHandle* h = (RefHandle*)hp;
  Tonemapper op = h ? h->tonemapper : Tonemapper();
  if (op_override >= 0) { memcpy((void*)&op, &op_override, sizeof(int)); }
  std::vector<Vector3> fc(n);
  std::vector<Pixel> px(n);
  for (int i = 0; i < n; ++i) fc[i] = vector3_create(sum[3 * i], sum[3 * i + 1], sum[3 * i + 2]);
  for (int i = 0; i < n; ++i) {
    set_index(i);
    tonemap(fc.data(), px.data(), samples, op, n);
  }
  for (int i = 0; i < n; ++i) {
    out_rgb8[3 * i] = (unsigned char)px[i].red;
    out_rgb8[3 * i + 1] = (unsigned char)px[i].green;
    out_rgb8[3 * i + 2] = (unsigned char)px[i].blue;
  }
}

// Closest hit of get_min_hit (src/renderer.cu:112-137) for n rays (o, d: 6 floats each,
// d is normalised as ray_create does). Writes t (FLT_MAX on a miss), the primitive
// (sphere index, or sphere_count + instance index, -1 on a miss) and the shading normal.
void ref_closest_hit(void* hp, const float* rays, int n, float* t, int* prim, float* normal) {
  RefHandle* h = (RefHandle*)hp;
  DeviceScene* scene = h->ref->getScene();
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < n; ++i) {
    Ray r = ray_create(vector3_create(rays[6 * i], rays[6 * i + 1], rays[6 * i + 2]),
                       vector3_create(rays[6 * i + 3], rays[6 * i + 4], rays[6 * i + 5]));
    Hit m;
    hit_set_no_intersect(&m);
    get_min_hit(scene, r, &m);
    int p = -1;
    if (m.is_intersect) {
      for (int s = 0; s < scene->sphere_amount; ++s)
        if (m.m == &scene->spheres[s].m) p = s;
      for (int k = 0; k < scene->instance_amount; ++k)
        if (m.m == &scene->instances[k].m) p = scene->sphere_amount + k;
    }
    t[i] = m.is_intersect ? m.d : FLT_MAX;
    prim[i] = p;
    normal[3 * i] = m.is_intersect ? m.normal.x : 0.f;
    normal[3 * i + 1] = m.is_intersect ? m.normal.y : 0.f;
    normal[3 * i + 2] = m.is_intersect ? m.normal.z : 0.f;
  }
}

// ---- component functions (device code of the reference, called on the host) ----
float ref_fresnel_dielectric(float cosI, float ior, float* cosT) { return Fresnel::dielectric(cosI, ior, *cosT); }
float ref_fresnel_conductor1(float eta, float k, float cosI) { return Fresnel::conductor(eta, k, cosI); }
float ref_diffuse_fresnel(float ior, int samples) { return Fresnel::diffuse_fresnel(ior, samples); }
float ref_D_beckmann(const float* m, const float* n, float a) {
  return Microfacet::D_Beckmann(vector3_create(m[0], m[1], m[2]), vector3_create(n[0], n[1], n[2]), a);
}
float ref_G_beckmann(const float* i, const float* o, const float* n, float a) {
  return Microfacet::G_Beckmann(vector3_create(i[0], i[1], i[2]), vector3_create(o[0], o[1], o[2]),
                                vector3_create(n[0], n[1], n[2]), a);
}
static void put3(float* o, Vector3 v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; }
void ref_sample_beckmann(float a, float u1, float u2, float* out) { put3(out, Microfacet::sample_Beckmann(a, u1, u2)); }
void ref_sample_hemisphere_cosine(float u1, float u2, float* out) { put3(out, sample_hemisphere_cosine(u1, u2)); }
void ref_sample_circle(float u1, float u2, float* out) { put3(out, sample_circle(u1, u2)); }
void ref_sample_sphere(float u1, float u2, float* out) { put3(out, sample_sphere(u1, u2)); }
void ref_sample_hg(float g, float u1, float u2, float* out) { put3(out, sample_henyey_greenstein(g, u1, u2)); }
void ref_to_basis(const float* v, const float* n, float* out) {
  put3(out, vector3_to_basis(vector3_create(v[0], v[1], v[2]), vector3_create(n[0], n[1], n[2])));
}
float ref_triangle_intersect(const float* v0, const float* v1, const float* v2, const float* o, const float* d,
                             float* u, float* v) {
  Ray r;
  r.o = vector3_create(o[0], o[1], o[2]);
  r.d = vector3_create(d[0], d[1], d[2]);
  *u = 0; *v = 0;
  return triangle_ray_intersect(vector3_create(v0[0], v0[1], v0[2]), vector3_create(v1[0], v1[1], v1[2]),
                                vector3_create(v2[0], v2[1], v2[2]), r, *u, *v);
}
float ref_aabb_intersect(const float* mn, const float* mx, const float* o, const float* d) {
  AABB b;
  b.min = vector3_create(mn[0], mn[1], mn[2]);
  b.max = vector3_create(mx[0], mx[1], mx[2]);
  Ray r;
  r.o = vector3_create(o[0], o[1], o[2]);
  r.d = vector3_create(d[0], d[1], d[2]);
  return aabb_ray_intersect(b, r);
}
int ref_sphere_intersect(const float* c, float rad, const float* o, const float* d, float* t, float* n, float* uv) {
  Sphere s;
  s.r = rad;
  s.center = vector3_create(c[0], c[1], c[2]);
  Ray r;
  r.o = vector3_create(o[0], o[1], o[2]);
  r.d = vector3_create(d[0], d[1], d[2]);
  Hit hit;
  hit_set_no_intersect(&hit);
  sphere_ray_intersect(&s, r, &hit);
  if (!hit.is_intersect) return 0;
  *t = hit.d;
  put3(n, hit.normal);
  uv[0] = hit.uv.x; uv[1] = hit.uv.y;
  return 1;
}
void ref_tonemap_eval(int op, const float* in, float* out) {
  Tonemapper t;
  memcpy((void*)&t, &op, sizeof(int));
  put3(out, t.eval(vector3_create(in[0], in[1], in[2])));
}
static void parse(rapidjson::Document& d, const char* json) { d.Parse(json); }
void ref_transform_from_json(const char* json, float* mat, float* inv, float* trans_inv) {
  rapidjson::Document d;
  parse(d, json);
  Transform t = transform_from_json(d);
  memcpy(mat, t.mat.m, 64);
  memcpy(inv, t.inv.m, 64);
  memcpy(trans_inv, t.trans_inv.m, 64);
}
int ref_texture_eval(const char* json, float u, float v, float* out) {
  rapidjson::Document d;
  parse(d, json);
  Texture t = texture_from_json(d);
  put3(out, t.eval(Vec2f(u, v)));
  return (int)t.type;
}
void ref_medium_from_json(const char* json, float* absorption, float* scattering, float* g, int* active) {
  rapidjson::Document d;
  parse(d, json);
  Medium m = medium_from_json(d);
  put3(absorption, m.absorption);
  *scattering = m.scattering;
  *g = m.g;
  *active = m.active ? 1 : 0;
}
int ref_material_from_json(const char* json, float* ior, float* diffuse_fresnel, float* eta, float* k,
                           float* albedo_c, float* roughness_c) {
  rapidjson::Document d;
  parse(d, json);
  std::vector<Texture> cache;
  Material m = material_from_json(d, medium_air(), cache);
  *ior = m.ior;
  *diffuse_fresnel = m.diffuse_fresnel;
  put3(eta, m.eta);
  put3(k, m.k);
  put3(albedo_c, m.albedo.eval(Vec2f(0, 0)));
  put3(roughness_c, m.roughness.eval(Vec2f(0, 0)));
  return m.type;
}
// Camera rays of init_rays (src/renderer.cu:81-110) for pass `sample` of a W x H image.
void ref_camera_rays(void* hp, int W, int H, uint32_t sample, uint32_t seed, uint32_t job, float* out) {
  RefHandle* h = (RefHandle*)hp;
  const int N = W * H;
  RenderInfo* info = allocate_render_info_gpu(W, H, h->scene->get_camera());
  std::vector<curandState> states(N);
  std::vector<Ray> rays(N);
  std::vector<int> statuses(N);
  std::vector<Vector3> colors(N);
  std::vector<Medium> mediums(N);
  for (int i = 0; i < N; ++i) {
    states[i] = curandState{(uint32_t)i, sample, 0u, seed, job, 0u, {0, 0, 0, 0}};
    set_index(i);
    init_rays(rays.data(), statuses.data(), colors.data(), mediums.data(), info, states.data(), N);
    out[6 * i] = rays[i].o.x; out[6 * i + 1] = rays[i].o.y; out[6 * i + 2] = rays[i].o.z;
    out[6 * i + 3] = rays[i].d.x; out[6 * i + 4] = rays[i].d.y; out[6 * i + 5] = rays[i].d.z;
  }
  cudaFree(info);
}

// Exports the loaded scene as an illume_scene_desc. Materials are embedded per primitive
// in the reference (Sphere::m, MeshInstance::m), so every sphere and instance gets its own
// material, and every material its own medium and textures. The export stays valid
// until ref_scene_free.
int ref_scene_export(void* hp, illume_scene_desc* d) {
  RefHandle* h = (RefHandle*)hp;
  export_scene(h, d);
  return 0;
}

}  // extern "C"

static int add_texture(RefExport* e, const Texture& t) {
  const int id = (int)e->tex_type.size();
  e->tex_type.push_back((int)t.type);
  float c[3] = {0, 0, 0}, o[3] = {0, 0, 0}, s[2] = {1, 1};
  int w = 0, hh = 0, hdr = 1;
  int64_t off = (int64_t)e->texels.size();
  if (t.type == TextureType::CONSTANT) {
    c[0] = t.constant.c.x; c[1] = t.constant.c.y; c[2] = t.constant.c.z;
  } else if (t.type == TextureType::CHECKERBOARD) {
    c[0] = t.checkerboard.on.x; c[1] = t.checkerboard.on.y; c[2] = t.checkerboard.on.z;
    o[0] = t.checkerboard.off.x; o[1] = t.checkerboard.off.y; o[2] = t.checkerboard.off.z;
    s[0] = t.checkerboard.scale.x; s[1] = t.checkerboard.scale.y;
  } else {
    const ShimTexture* st = (const ShimTexture*)(uintptr_t)t.bitmap.texObj;
    const cudaArray* a = st->a;
    w = a->width; hh = a->height; hdr = t.bitmap.is_hdr ? 1 : 0;
    s[0] = t.bitmap.scale.x; s[1] = t.bitmap.scale.y;
    for (size_t i = 0; i < (size_t)w * hh * 4; ++i)
      e->texels.push_back(a->is_float ? ((const float*)a->data)[i] : (float)a->data[i]);
  }
  e->tex_c.insert(e->tex_c.end(), c, c + 3);
  e->tex_o.insert(e->tex_o.end(), o, o + 3);
  e->tex_s.insert(e->tex_s.end(), s, s + 2);
  e->tex_w.push_back(w); e->tex_h.push_back(hh); e->tex_hdr.push_back(hdr); e->tex_off.push_back(off);
  return id;
}

static int add_material(RefExport* e, const Material& m) {
  const int id = (int)e->mat_type.size();
  e->mat_type.push_back(m.type);
  e->mat_alb.push_back(add_texture(e, m.albedo));
  e->mat_rough.push_back(add_texture(e, m.roughness));
  e->mat_dist.push_back(0);
  e->mat_ior.push_back(m.ior);
  e->mat_df.push_back(m.diffuse_fresnel);
  e->mat_eta.insert(e->mat_eta.end(), {m.eta.x, m.eta.y, m.eta.z});
  e->mat_k.insert(e->mat_k.end(), {m.k.x, m.k.y, m.k.z});
  if (m.medium.active) {
    e->mat_med.push_back((int)e->med_active.size());
    e->med_abs.insert(e->med_abs.end(), {m.medium.absorption.x, m.medium.absorption.y, m.medium.absorption.z});
    e->med_sc.push_back(m.medium.scattering);
    e->med_g.push_back(m.medium.g);
    e->med_active.push_back(1);
  } else {
    e->mat_med.push_back(-1);
  }
  return id;
}

static void put34(std::vector<float>& v, const Matrix4& m) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) v.push_back(m.m[r][c]);
}

struct RefHandleExport { RefExport* e = nullptr; };
static std::map<void*, RefExport*> g_exports;

static RefExport* export_scene(RefHandle* h, illume_scene_desc* d) {
  RefExport*& e = g_exports[h];
  delete e;
  e = new RefExport;
  DeviceScene* s = h->ref->getScene();
  int vo = 0, to = 0;
  for (int i = 0; i < s->mesh_amount; ++i) {
    const Mesh& m = s->meshes[i];
    e->mvo.push_back(vo); e->mto.push_back(to);
    e->mnv.push_back(m.vertex_amount); e->mnt.push_back(m.triangle_amount);
    e->mhn.push_back(m.face_normals ? 0 : 1); e->mht.push_back(m.has_texcoords ? 1 : 0);
    e->mls.push_back(4);
    for (int v = 0; v < m.vertex_amount; ++v) {
      e->pos.insert(e->pos.end(), {m.positions[v].x, m.positions[v].y, m.positions[v].z});
      if (!m.face_normals) e->nrm.insert(e->nrm.end(), {m.normals[v].x, m.normals[v].y, m.normals[v].z});
      else e->nrm.insert(e->nrm.end(), {0.f, 0.f, 0.f});
      if (m.has_texcoords) e->tc.insert(e->tc.end(), {m.texcoords[v].x, m.texcoords[v].y});
      else e->tc.insert(e->tc.end(), {0.f, 0.f});
    }
    for (int t = 0; t < m.triangle_amount; ++t)
      e->tris.insert(e->tris.end(), {m.triangles[t].indices[0], m.triangles[t].indices[1], m.triangles[t].indices[2]});
    vo += m.vertex_amount;
    to += m.triangle_amount;
  }
  for (int i = 0; i < s->sphere_amount; ++i) {
    const Sphere& sp = s->spheres[i];
    e->sph.insert(e->sph.end(), {sp.center.x, sp.center.y, sp.center.z, sp.r});
    e->sph_mat.push_back(add_material(e, sp.m));
  }
  for (int i = 0; i < s->instance_amount; ++i) {
    const MeshInstance& in = s->instances[i];
    e->inst_mesh.push_back(in.mesh_index);
    e->inst_mat.push_back(add_material(e, in.m));
    put34(e->imat, in.t.mat);
    put34(e->iinv, in.t.inv);
    put34(e->itinv, in.t.trans_inv);
  }
  int env = -1;
  if (s->envmap.type != TextureType::CONSTANT || s->envmap.constant.c.x != 0 || s->envmap.constant.c.y != 0 ||
      s->envmap.constant.c.z != 0)
    env = add_texture(e, s->envmap);
  memset(d, 0, sizeof(*d));
  d->num_meshes = s->mesh_amount;
  d->mesh_vertex_offset = e->mvo.data(); d->mesh_num_vertices = e->mnv.data();
  d->mesh_tri_offset = e->mto.data(); d->mesh_num_tris = e->mnt.data();
  d->mesh_has_normals = e->mhn.data(); d->mesh_has_texcoords = e->mht.data(); d->mesh_bvh_leaf_size = e->mls.data();
  d->positions = e->pos.data(); d->normals = e->nrm.data(); d->texcoords = e->tc.data(); d->tris = e->tris.data();
  d->num_instances = s->instance_amount;
  d->inst_mesh = e->inst_mesh.data(); d->inst_material = e->inst_mat.data();
  d->inst_mat = e->imat.data(); d->inst_inv = e->iinv.data(); d->inst_trans_inv = e->itinv.data();
  d->num_spheres = s->sphere_amount;
  d->sphere_center_radius = e->sph.data(); d->sphere_material = e->sph_mat.data();
  d->num_materials = (int)e->mat_type.size();
  d->mat_type = e->mat_type.data(); d->mat_albedo_tex = e->mat_alb.data(); d->mat_roughness_tex = e->mat_rough.data();
  d->mat_medium = e->mat_med.data(); d->mat_distribution = e->mat_dist.data();
  d->mat_ior = e->mat_ior.data(); d->mat_diffuse_fresnel = e->mat_df.data();
  d->mat_eta = e->mat_eta.data(); d->mat_k = e->mat_k.data();
  d->num_mediums = (int)e->med_active.size();
  d->med_absorption = e->med_abs.data(); d->med_scattering = e->med_sc.data(); d->med_g = e->med_g.data();
  d->med_active = e->med_active.data();
  d->num_textures = (int)e->tex_type.size();
  d->tex_type = e->tex_type.data(); d->tex_color = e->tex_c.data(); d->tex_off = e->tex_o.data();
  d->tex_scale = e->tex_s.data(); d->tex_width = e->tex_w.data(); d->tex_height = e->tex_h.data();
  d->tex_hdr = e->tex_hdr.data(); d->tex_texel_offset = e->tex_off.data();
  d->texels = e->texels.empty() ? nullptr : e->texels.data();
  d->env_tex = env;
  const Camera& cam = h->scene->get_camera();
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) d->camera_transform[4 * r + c] = cam.transform.m[r][c];
  d->camera_fov = cam.fov; d->camera_dof = cam.dof; d->camera_aperture = cam.aperture;
  d->width = h->width; d->height = h->height; d->ray_bias = h->ray_bias;
  int op;
  memcpy(&op, (const void*)&h->tonemapper, sizeof(int));
  d->tonemapper = op;
  return e;
}
