// C entry points of the oracle (CPU restatement in oracle.h).
//
// TEST INFRASTRUCTURE: loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline (through oracle/pyoracle.py). Built by __graft_entry__.build() into
// oracle/_build/liboracle.so with -O2 -ffp-contract=off -fopenmp.

#include <omp.h>
#include <string.h>
#include <atomic>

#include "oracle.h"
#include "../include/illume.h"

namespace oracle {

// Median-split binary BVH over triangle boxes (double precision bounds).
void build_obvh(const Mesh& m, OBvh& bvh) {
  const int T = m.num_tris;
  bvh.order.resize(T);
  std::vector<double> lo((size_t)T * 3), hi((size_t)T * 3), ctr((size_t)T * 3);
  for (int i = 0; i < T; ++i) {
    bvh.order[i] = i;
    for (int a = 0; a < 3; ++a) {
      double l = INFINITY, h = -INFINITY;
      for (int k = 0; k < 3; ++k) {
        const double p = m.positions[3 * m.tris[3 * i + k] + a];
        l = fmin(l, p);
        h = fmax(h, p);
      }
      lo[3 * i + a] = l; hi[3 * i + a] = h; ctr[3 * i + a] = 0.5 * (l + h);
    }
  }
  bvh.nodes.clear();
  bvh.nodes.reserve(2 * (size_t)T + 1);
  struct Item { int node, first, count; };
  std::vector<Item> work;
  bvh.nodes.push_back(OBvh::Node{});
  work.push_back(Item{0, 0, T});
  while (!work.empty()) {
    Item it = work.back();
    work.pop_back();
    OBvh::Node nd{};
    double clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int a = 0; a < 3; ++a) { nd.lo[a] = INFINITY; nd.hi[a] = -INFINITY; }
    for (int i = it.first; i < it.first + it.count; ++i) {
      const int p = bvh.order[i];
      for (int a = 0; a < 3; ++a) {
        nd.lo[a] = fmin(nd.lo[a], lo[3 * p + a]);
        nd.hi[a] = fmax(nd.hi[a], hi[3 * p + a]);
        clo[a] = fmin(clo[a], ctr[3 * p + a]);
        chi[a] = fmax(chi[a], ctr[3 * p + a]);
      }
    }
    if (it.count <= 4) {
      nd.first = it.first; nd.count = it.count; nd.left = nd.right = -1;
      bvh.nodes[it.node] = nd;
      continue;
    }
    int axis = 0;
    for (int a = 1; a < 3; ++a)
      if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
    const int mid = it.first + it.count / 2;
    std::nth_element(bvh.order.begin() + it.first, bvh.order.begin() + mid, bvh.order.begin() + it.first + it.count,
                     [&](int x, int y) {
                       const double cx = ctr[3 * x + axis], cy = ctr[3 * y + axis];
                       return cx < cy || (cx == cy && x < y);
                     });
    nd.count = 0;
    nd.left = (int)bvh.nodes.size();
    nd.right = nd.left + 1;
    bvh.nodes.push_back(OBvh::Node{});
    bvh.nodes.push_back(OBvh::Node{});
    bvh.nodes[it.node] = nd;
    work.push_back(Item{nd.left, it.first, mid - it.first});
    work.push_back(Item{nd.right, mid, it.first + it.count - mid});
  }
}

static Mat34 mat34(const float* p) {
  Mat34 m;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 4; ++c) m.m[r][c] = p[4 * r + c];
  return m;
}

static Scene* scene_from_desc(const illume_scene_desc* d) {
  Scene* s = new Scene;
  for (int i = 0; i < d->num_meshes; ++i) {
    Mesh m;
    const int vo = d->mesh_vertex_offset[i], to = d->mesh_tri_offset[i];
    m.positions = d->positions + 3 * (size_t)vo;
    m.tris = d->tris + 3 * (size_t)to;
    m.normals = d->mesh_has_normals[i] ? d->normals + 3 * (size_t)vo : nullptr;
    m.texcoords = d->mesh_has_texcoords[i] ? d->texcoords + 2 * (size_t)vo : nullptr;
    m.num_vertices = d->mesh_num_vertices[i];
    m.num_tris = d->mesh_num_tris[i];
    s->meshes.push_back(m);
  }
  s->bvhs.resize(s->meshes.size());
  for (size_t i = 0; i < s->meshes.size(); ++i) build_obvh(s->meshes[i], s->bvhs[i]);
  for (int i = 0; i < d->num_instances; ++i) {
    Instance in;
    in.mesh = d->inst_mesh[i];
    in.material = d->inst_material[i];
    in.mat = mat34(d->inst_mat + 12 * i);
    in.inv = mat34(d->inst_inv + 12 * i);
    in.trans_inv = mat34(d->inst_trans_inv + 12 * i);
    s->instances.push_back(in);
  }
  for (int i = 0; i < d->num_spheres; ++i) {
    Sphere sp;
    memcpy(sp.center, d->sphere_center_radius + 4 * i, 12);
    sp.radius = d->sphere_center_radius[4 * i + 3];
    sp.material = d->sphere_material[i];
    s->spheres.push_back(sp);
  }
  for (int i = 0; i < d->num_materials; ++i) {
    Material m;
    m.type = d->mat_type[i];
    m.albedo_tex = d->mat_albedo_tex[i];
    m.roughness_tex = d->mat_roughness_tex[i];
    m.medium = d->mat_medium[i];
    m.distribution = d->mat_distribution[i];
    m.ior = d->mat_ior[i];
    m.diffuse_fresnel = d->mat_diffuse_fresnel[i];
    memcpy(m.eta, d->mat_eta + 3 * i, 12);
    memcpy(m.k, d->mat_k + 3 * i, 12);
    s->materials.push_back(m);
  }
  for (int i = 0; i < d->num_mediums; ++i) {
    Medium m;
    memcpy(m.absorption, d->med_absorption + 3 * i, 12);
    m.scattering = d->med_scattering[i];
    m.g = d->med_g[i];
    m.active = d->med_active[i];
    s->mediums.push_back(m);
  }
  for (int i = 0; i < d->num_textures; ++i) {
    Texture t{};
    t.type = d->tex_type[i];
    memcpy(t.c, d->tex_color + 3 * i, 12);
    memcpy(t.off, d->tex_off + 3 * i, 12);
    memcpy(t.scale, d->tex_scale + 2 * i, 8);
    t.width = d->tex_width[i];
    t.height = d->tex_height[i];
    t.hdr = d->tex_hdr[i];
    t.texels = t.type == TEX_BITMAP ? d->texels + d->tex_texel_offset[i] : nullptr;
    s->textures.push_back(t);
  }
  s->env_tex = d->env_tex;
  s->camera.transform = mat34(d->camera_transform);
  s->camera.fov = d->camera_fov;
  s->camera.dof = d->camera_dof;
  s->camera.aperture = d->camera_aperture;
  return s;
}

}  // namespace oracle

using namespace oracle;

extern "C" {

typedef struct {
  int32_t width, height, max_depth;
  float ray_bias;
  uint32_t seed, job;
  int32_t isect, exact_hg;
  int32_t spp, sample_begin;
  int32_t precision;        // 32 or 64
  int32_t num_pixels;       // 0 = every pixel of the image
  const int32_t* pixels;    // pixel indices (y * width + x) when num_pixels > 0
  int32_t nthreads;         // 0 = OpenMP default
  int32_t nee;              // 1 = next-event estimation with MIS (EXTENSION)
} oracle_render_args;

void* oracle_scene_create(const illume_scene_desc* desc) { return scene_from_desc(desc); }
void oracle_scene_destroy(void* s) { delete (Scene*)s; }

void oracle_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) { philox::philox4x32_10(ctr, key, out); }

static void fill_hit(const Hit<float>& h, illume_hit* o) {
  o->t = h.hit ? h.t : FLT_MAX;
  o->u = h.hit && h.inst >= 0 ? h.bu : 0.f;
  o->v = h.hit && h.inst >= 0 ? h.bv : 0.f;
  o->inst = h.hit ? h.inst : -1;
  o->prim = h.hit ? h.prim : -1;
  o->sphere = h.hit ? h.sphere : -1;
  o->pad[0] = o->pad[1] = 0;
}

// Closest hit for rays of 8 floats (o, -, d, -), FP32, directions used as given.
void oracle_closest_hit(void* sp, const float* rays, int n, int isect, illume_hit* out, int nthreads) {
  const Scene& sc = *(const Scene*)sp;
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < n; ++i) {
    const float* r = rays + 8 * (size_t)i;
    Ray<float> ray{v3<float>(r[0], r[1], r[2]), v3<float>(r[4], r[5], r[6])};
    fill_hit(closest_hit<float>(sc, ray, isect), out + i);
  }
}

// Brute force over every triangle (FP32): checks that the oracle's BVH never culls.
void oracle_closest_hit_brute(void* sp, const float* rays, int n, int isect, illume_hit* out, int nthreads) {
  const Scene& sc = *(const Scene*)sp;
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16)
  for (int i = 0; i < n; ++i) {
    const float* r = rays + 8 * (size_t)i;
    const Ray<float> ray{v3<float>(r[0], r[1], r[2]), v3<float>(r[4], r[5], r[6])};
    Hit<float> best{};
    best.t = FLT_MAX;
    best.inst = best.prim = best.sphere = -1;
    for (int s = 0; s < (int)sc.spheres.size(); ++s) {
      const Sphere& spr = sc.spheres[s];
      float t, u, v;
      V3<float> nn;
      if (sphere_intersect(v3<float>(spr.center[0], spr.center[1], spr.center[2]), spr.radius, ray, t, nn, u, v) &&
          t < best.t) {
        best.hit = true; best.t = t; best.sphere = s; best.inst = -1; best.prim = -1;
      }
    }
    for (int k = 0; k < (int)sc.instances.size(); ++k) {
      const Instance& in = sc.instances[k];
      const V3<float> o = xform(in.inv, ray.o, 1.0f), d = xform(in.inv, ray.d, 0.0f);
      const Mesh& m = sc.meshes[in.mesh];
      const WtRay wt = watertight_setup(d);
      float bt = FLT_MAX, bu = 0, bv = 0;
      int bp = -1;
      for (int p = 0; p < m.num_tris; ++p) {
        const int* tri = m.tris + 3 * p;
        const float* P = m.positions;
        const V3<float> v0 = v3<float>(P[3 * tri[0]], P[3 * tri[0] + 1], P[3 * tri[0] + 2]);
        const V3<float> v1 = v3<float>(P[3 * tri[1]], P[3 * tri[1] + 1], P[3 * tri[1] + 2]);
        const V3<float> v2 = v3<float>(P[3 * tri[2]], P[3 * tri[2] + 1], P[3 * tri[2] + 2]);
        float u = 0, v = 0;
        const float t = isect == ISECT_MT ? triangle_mt(v0, v1, v2, Ray<float>{o, d}, u, v)
                                          : triangle_watertight(v0, v1, v2, o, wt, u, v);
        if (t > 0 && (t < bt || (t == bt && p < bp))) { bt = t; bp = p; bu = u; bv = v; }
      }
      if (bp >= 0 && bt < best.t) {
        best.hit = true; best.t = bt; best.sphere = -1; best.inst = k; best.prim = bp; best.bu = bu; best.bv = bv;
      }
    }
    fill_hit(best, out + i);
  }
}

// Camera rays of one sample pass (6 floats per pixel: origin, direction).
void oracle_camera_rays(void* sp, int W, int H, uint32_t sample, uint32_t seed, uint32_t job, float* out) {
  const Scene& sc = *(const Scene*)sp;
  const CameraSetup cs = camera_setup(sc.camera, W, H);
  for (int i = 0; i < W * H; ++i) {
    philox::Stream rng;
    rng.init((uint32_t)i, sample, 0, seed, job);
    const Ray<float> r = camera_ray<float>(sc, cs, W, i, rng);
    out[6 * i] = r.o.x; out[6 * i + 1] = r.o.y; out[6 * i + 2] = r.o.z;
    out[6 * i + 3] = r.d.x; out[6 * i + 4] = r.d.y; out[6 * i + 5] = r.d.z;
  }
}

// Renders samples [sample_begin, sample_begin + spp) of the listed pixels.
// out_sum / out_sumsq: 3 doubles per listed pixel. Returns the rays traced.
int64_t oracle_render(void* sp, const oracle_render_args* a, double* out_sum, double* out_sumsq) {
  const Scene& sc = *(const Scene*)sp;
  RenderParams p;
  p.width = a->width; p.height = a->height; p.max_depth = a->max_depth; p.ray_bias = a->ray_bias;
  p.seed = a->seed; p.job = a->job; p.isect = a->isect; p.exact_hg = a->exact_hg; p.nee = a->nee;
  const CameraSetup cs = camera_setup(sc.camera, a->width, a->height);
  LightTables lights;
  if (a->nee) lights = build_light_tables(sc);
  const int np = a->num_pixels > 0 ? a->num_pixels : a->width * a->height;
  if (a->nthreads > 0) omp_set_num_threads(a->nthreads);
  std::atomic<int64_t> rays{0};
#pragma omp parallel for schedule(dynamic, 16)
  for (int i = 0; i < np; ++i) {
    const int pixel = a->num_pixels > 0 ? a->pixels[i] : i;
    double s[3] = {0, 0, 0}, s2[3] = {0, 0, 0};
    int64_t local = 0;
    for (int k = 0; k < a->spp; ++k) {
      const uint32_t sample = (uint32_t)(a->sample_begin + k);
      const PathResult r = a->precision == 64 ? trace_path<double>(sc, p, cs, pixel, sample, &lights)
                                              : trace_path<float>(sc, p, cs, pixel, sample, &lights);
      local += r.rays;
      for (int c = 0; c < 3; ++c) { s[c] += r.L[c]; s2[c] += r.L[c] * r.L[c]; }
    }
    rays += local;
    for (int c = 0; c < 3; ++c) {
      out_sum[3 * (size_t)i + c] = s[c];
      if (out_sumsq) out_sumsq[3 * (size_t)i + c] = s2[c];
    }
  }
  return rays.load();
}

// Alias table of n weights (EXTENSION: the next-event estimator's light choice).
void oracle_alias_build(const double* w, int n, float* prob, int* alias) {
  std::vector<AliasSlot> t(n > 0 ? n : 0);
  alias_build(w, (size_t)(n > 0 ? n : 0), t.data());
  for (int i = 0; i < n; ++i) { prob[i] = t[i].prob; alias[i] = t[i].alias; }
}

// The scene's light tables (EXTENSION): sizes, then the environment's texel weights,
// row and column tables, and the triangle table with each triangle's choice probability.
void oracle_light_info(void* sp, int* env_wh, float* env_integral_prob, int* num_tri) {
  const LightTables L = build_light_tables(*(const Scene*)sp);
  env_wh[0] = L.env_w;
  env_wh[1] = L.env_h;
  env_integral_prob[0] = L.env_integral;
  env_integral_prob[1] = L.env_prob;
  *num_tri = (int)L.tris.size();
}

void oracle_tonemap_image(const float* sum, int n, float samples, int op, unsigned char* out) {
  for (int i = 0; i < n; ++i) tonemap_pixel(op, sum + 3 * i, samples, out + 3 * i);
}

// ---- component functions (FP32 unless suffixed _d) ----
float oracle_fresnel_dielectric(float cosI, float ior, float* cosT) { return fresnel_dielectric<float>(cosI, ior, *cosT); }
double oracle_fresnel_dielectric_d(double cosI, double ior, double* cosT) { return fresnel_dielectric<double>(cosI, ior, *cosT); }
float oracle_fresnel_conductor1(float eta, float k, float cosI) { return fresnel_conductor<float>(eta, k, cosI); }
float oracle_diffuse_fresnel(float ior, int samples) { return diffuse_fresnel(ior, samples); }
static V3<float> f3(const float* p) { return v3<float>(p[0], p[1], p[2]); }
static void put(float* o, V3<float> v) { o[0] = v.x; o[1] = v.y; o[2] = v.z; }
float oracle_D_beckmann(const float* m, const float* n, float a) { return D_beckmann<float>(f3(m), f3(n), a); }
float oracle_G_beckmann(const float* i, const float* o, const float* n, float a) { return G_beckmann<float>(f3(i), f3(o), f3(n), a); }
void oracle_sample_beckmann(float a, float u1, float u2, float* out) { put(out, sample_beckmann<float>(a, u1, u2)); }
void oracle_sample_hemisphere_cosine(float u1, float u2, float* out) { put(out, sample_hemisphere_cosine<float>(u1, u2)); }
void oracle_sample_circle(float u1, float u2, float* out) { put(out, sample_circle<float>(u1, u2)); }
void oracle_sample_sphere(float u1, float u2, float* out) { put(out, sample_sphere<float>(u1, u2)); }
void oracle_sample_hg(float g, float u1, float u2, int exact, float* out) { put(out, sample_hg<float>(g, u1, u2, exact != 0)); }
void oracle_to_basis(const float* v, const float* n, float* out) { put(out, to_basis<float>(f3(v), f3(n))); }
float oracle_triangle_mt(const float* v0, const float* v1, const float* v2, const float* o, const float* d, float* u, float* v) {
  *u = 0; *v = 0;
  return triangle_mt<float>(f3(v0), f3(v1), f3(v2), Ray<float>{f3(o), f3(d)}, *u, *v);
}
float oracle_triangle_watertight(const float* v0, const float* v1, const float* v2, const float* o, const float* d,
                                 float* u, float* v) {
  *u = 0; *v = 0;
  return triangle_watertight(f3(v0), f3(v1), f3(v2), f3(o), watertight_setup(f3(d)), *u, *v);
}
float oracle_aabb_intersect(const float* mn, const float* mx, const float* o, const float* d) {
  return aabb_intersect<float>(f3(mn), f3(mx), Ray<float>{f3(o), f3(d)});
}
int oracle_sphere_intersect(const float* c, float r, const float* o, const float* d, float* t, float* n, float* uv) {
  V3<float> nn;
  if (!sphere_intersect<float>(f3(c), r, Ray<float>{f3(o), f3(d)}, *t, nn, uv[0], uv[1])) return 0;
  put(n, nn);
  return 1;
}
void oracle_tonemap_eval(int op, const float* in, float* out) { put(out, tonemap_op(op, f3(in))); }
void oracle_texture_eval(void* sp, int tex, float u, float v, float* out) {
  put(out, tex_eval<float>(*(const Scene*)sp, tex, u, v));
}

// BSDF batch with the layout of illume_bsdf_batch (include/illume.h). precision 32/64.
void oracle_bsdf_batch(int material_type, int distribution, const float* in, int n, float* out, int precision) {
  for (int i = 0; i < n; ++i) {
    const float* x = in + 16 * (size_t)i;
    float* y = out + 16 * (size_t)i;
    Material m2{};
    m2.type = material_type;
    m2.distribution = distribution;
    m2.medium = -1;
    const float uu[3] = {x[6], x[7], x[8]};
    // Layout: wi(0..2) n(3..5) u1 u2 u3 (6..8) roughness (9) ior (10) eta (11..13) k (14)
    m2.ior = x[10];
    for (int c = 0; c < 3; ++c) { m2.eta[c] = x[11 + c]; m2.k[c] = x[14]; }
    m2.diffuse_fresnel = material_type != MAT_PLASTIC ? 0.0f : (x[15] != 0.0f ? x[15] : diffuse_fresnel(1.0f / x[10], 1000000));
    auto run2 = [&](auto zero) {
      using R = decltype(zero);
      int k = 0;
      const V3<R> wi = v3<R>(x[0], x[1], x[2]);
      const V3<R> N = v3<R>(x[3], x[4], x[5]);
      const V3<R> d = mul(wi, (R)-1.0f);
      ScatterOut<R> s = scatter<R>(m2, d, N, v3<R>(1, 1, 1), (R)x[9], [&]() { return (R)uu[k++]; });
      const V3<R> nd = s.status == SCATTER_KILLED ? v3<R>(0, 0, 0) : normalize(s.dir);
      y[0] = (float)nd.x; y[1] = (float)nd.y; y[2] = (float)nd.z;
      y[3] = (float)s.weight.x; y[4] = (float)s.weight.y; y[5] = (float)s.weight.z;
      y[6] = (float)s.D; y[7] = (float)s.pdf_m; y[8] = (float)s.G; y[9] = (float)s.F;
      // eval (f * |wo.n|) and solid-angle pdf of the sampled direction, reflection only
      R ev = 0, pd = 0;
      if (s.status == SCATTER_REFLECT && (material_type == MAT_ROUGHREFLECTIVE || material_type == MAT_ROUGHCONDUCTOR ||
                                          material_type == MAT_ROUGHREFRACTIVE)) {
        const R won = m_abs(dot(nd, N)), win = m_abs(dot(wi, N)), wom = m_abs(dot(nd, s.m));
        ev = s.F * s.D * s.G / ((R)4 * win);
        pd = s.pdf_m / ((R)4 * wom);
        (void)won;
      } else if (material_type == MAT_DIFFUSE) {
        const R won = m_abs(dot(nd, N));
        ev = won * (R)kInvPi;
        pd = won * (R)kInvPi;
      }
      y[10] = (float)ev; y[11] = (float)pd;
      y[12] = (float)s.status; y[13] = y[14] = y[15] = 0;
    };
    if (precision == 64) run2(0.0); else run2(0.0f);
  }
}

}  // extern "C"
