// Next-event estimation with multiple importance sampling (opt-in estimator; the
// reference finds light only by BSDF sampling, src/renderer.cu:183-386).
//
// At a surface vertex with a non-delta reflection lobe (lambert, rough conductor, rough
// dielectric reflection) that is not the path's last, one light sample is taken: the
// environment (piecewise-constant density over the map, luminance x cos(elevation)) or
// an emissive mesh triangle (chosen by area x luminance, uniform over its area), each
// choice an alias-table lookup. Its contribution, weighted by the power heuristic
// against the BSDF's density for the same direction, is added if a shadow ray finds
// nothing in between. A BSDF-sampled ray that
// then reaches an emitter or escapes is weighted by the power heuristic against the
// light density; after delta or transmissive interactions, in media, and for emissive
// spheres (not light-sampled) the weight is 1. Both estimators have the same
// expectation; tests compare them per pixel.
#pragma once

#include "../common/dmath.cuh"
#include "../common/types.h"
#include "shading.cuh"

namespace illume {

static constexpr float kTwoPiSq = 19.7392088021787172f;   // 2 pi^2

__device__ __forceinline__ float power_heuristic(float a, float b) {
  const float a2 = a * a, b2 = b * b;
  return a2 + b2 > 0.0f ? a2 / (a2 + b2) : 0.0f;
}

// Environment density (solid angle) of direction d, including the choice probability.
__device__ __forceinline__ float env_light_pdf(const LightView& L, V3 d) {
  if (L.env_w == 0) return 0.0f;
  const float u = atan2f(d.z, d.x) * (0.5f * (float)ILLUME_INV_PI_D) + 0.5f;
  const float v = 0.5f - asinf(fminf(fmaxf(d.y, -1.0f), 1.0f)) * (float)ILLUME_INV_PI_D;
  const int x = min(max((int)(u * (float)L.env_w), 0), L.env_w - 1);
  const int y = min(max((int)(v * (float)L.env_h), 0), L.env_h - 1);
  const float cos_e = sqrtf(fmaxf(1.0f - d.y * d.y, 0.0f));
  if (cos_e < 1e-6f) return 0.0f;
  const float puv = __ldg(L.env_func + (size_t)y * L.env_w + x) / L.env_integral;
  return L.env_prob * puv / (kTwoPiSq * cos_e);
}

// Density (solid angle, including the choice probabilities) of reaching light triangle l
// at distance t with cosine cos_l between the light's normal and the ray.
__device__ __forceinline__ float tri_light_pdf(const LightView& L, int l, float t, float cos_l) {
  if (l < 0 || fabsf(cos_l) < 1e-7f) return 0.0f;
  const float area = __ldg(&L.tri[3 * l].w), psel = __ldg(&L.tri[3 * l + 1].w);
  if (!(area > 0.0f)) return 0.0f;
  return (1.0f - L.env_prob) * psel * t * t / (area * fabsf(cos_l));
}

// Entry of an alias table of n slots chosen by u in [0, 1): one load instead of a binary
// search's chain of dependent loads. `frac` receives the rest of u's randomness, uniform
// in [0, 1) given the choice.
__device__ __forceinline__ int alias_pick(const AliasEntry* table, int n, float u, float& frac) {
  const float x = u * (float)n;
  const int i = min(max((int)x, 0), n - 1);
  const float f = fminf(fmaxf(x - (float)i, 0.0f), 0.99999994f);
  const float2 e = __ldg(reinterpret_cast<const float2*>(table + i));
  if (f < e.x) {
    frac = fminf(f / e.x, 0.99999994f);
    return i;
  }
  frac = fminf((f - e.x) / (1.0f - e.x), 0.99999994f);
  return __float_as_int(e.y);
}

struct LightSample {
  V3 dir;        // unit direction from the shading point
  float dist;    // distance to the light point (FLT_MAX for the environment)
  V3 Le;         // emitted radiance toward the shading point
  float pdf;     // solid-angle density including choice probabilities
  bool ok;
};

// u0 chooses the light kind and triangle; (u1, u2) place the point.
__device__ __forceinline__ LightSample sample_light(const SceneView& sc, const LightView& L, V3 p, float u0, float u1,
                                                    float u2) {
  LightSample s;
  s.ok = false;
  s.pdf = 0.0f;
  s.dist = FLT_MAX;
  s.Le = v3(0.0f, 0.0f, 0.0f);
  s.dir = v3(0.0f, 0.0f, 1.0f);
  if (u0 < L.env_prob) {
    // environment: a row by its weight, then a texel of the row, uniform within the texel
    float ry, rx;
    const int y = alias_pick(L.env_rows, L.env_h, u2, ry);
    const int x = alias_pick(L.env_cols + (size_t)y * L.env_w, L.env_w, u1, rx);
    const float u = ((float)x + rx) / (float)L.env_w, v = ((float)y + ry) / (float)L.env_h;
    const float phi = (u - 0.5f) * 6.28318530717958648f;
    const float elev = (0.5f - v) * 3.14159265358979324f;
    const float ce = cosf(elev);
    if (ce < 1e-6f) return s;
    s.dir = v3(ce * cosf(phi), sinf(elev), ce * sinf(phi));
    const float puv = __ldg(L.env_func + (size_t)y * L.env_w + x) / L.env_integral;
    s.pdf = L.env_prob * puv / (kTwoPiSq * ce);
    s.Le = env_eval(sc, s.dir);
    s.ok = s.pdf > 0.0f;
    return s;
  }
  if (L.num_tri == 0) return s;
  const float ut = (u0 - L.env_prob) / (1.0f - L.env_prob);
  float rest;
  const int l = alias_pick(L.tri_alias, L.num_tri, fminf(fmaxf(ut, 0.0f), 0.99999994f), rest);
  const float4 a = __ldg(&L.tri[3 * l]), b = __ldg(&L.tri[3 * l + 1]), c = __ldg(&L.tri[3 * l + 2]);
  // uniform point on the triangle
  const float su = sqrtf(u1);
  const float b1 = 1.0f - su, b2 = u2 * su;
  const V3 q = add(v3(a.x, a.y, a.z), add(mul(v3(b.x, b.y, b.z), b1), mul(v3(c.x, c.y, c.z), b2)));
  const V3 to = sub(q, p);
  const float d2 = dot(to, to);
  if (!(d2 > 0.0f)) return s;
  const float dist = sqrtf(d2);
  s.dir = mul(to, 1.0f / dist);
  s.dist = dist;
  const V3 n = cross(v3(b.x, b.y, b.z), v3(c.x, c.y, c.z));
  const float nl = sqrtf(dot(n, n));
  if (!(nl > 0.0f)) return s;
  const float cos_l = dot(n, s.dir) / nl;
  s.pdf = tri_light_pdf(L, l, dist, cos_l);
  // radiance: the emitter material's albedo at the point (texcoords as in shading)
  const int inst = __float_as_int(c.w);
  const DevInstance& in = sc.instances[inst];
  const DevMesh& m = sc.meshes[in.mesh];
  const int prim = l - __ldg(L.inst_light_base + inst);
  float uv0 = b1, uv1 = b2;
  if (m.texcoords) {
    const int i0 = __ldg(m.tris + 3 * prim), i1 = __ldg(m.tris + 3 * prim + 1), i2 = __ldg(m.tris + 3 * prim + 2);
    const float w0 = 1.0f - b1 - b2;
    uv0 = (__ldg(m.texcoords + 2 * i0) * w0 + __ldg(m.texcoords + 2 * i1) * b1) + __ldg(m.texcoords + 2 * i2) * b2;
    uv1 = (__ldg(m.texcoords + 2 * i0 + 1) * w0 + __ldg(m.texcoords + 2 * i1 + 1) * b1) + __ldg(m.texcoords + 2 * i2 + 1) * b2;
  }
  const DevMaterial& mat = sc.materials[in.material];
  s.Le = tex_eval(sc, mat.albedo_tex, uv0, uv1);
  s.ok = s.pdf > 0.0f;
  return s;
}

// BSDF value times the cosine for light direction wl and the density the material's own
// sampling gives wl, for the lobes the estimator samples lights for; false otherwise.
// d: incoming ray direction, N: geometric normal.
__device__ __forceinline__ bool bsdf_eval_cos(const DevMaterial& mat, V3 d, V3 N, V3 albedo, float roughness, V3 wl,
                                              V3& fcos, float& pdf) {
  const V3 norm_o = mul(N, dot(N, d) > 0.0f ? -1.0f : 1.0f);
  if (mat.type == MAT_LAMBERT) {
    const float c = dot(wl, norm_o);
    if (c <= 0.0f) return false;
    fcos = mul(albedo, c * (float)ILLUME_INV_PI_D);
    pdf = c * (float)ILLUME_INV_PI_D;
    return true;
  }
  if (mat.type != MAT_ROUGHCONDUCTOR && mat.type != MAT_ROUGHREFLECTIVE) return false;
  const V3 wi = mul(d, -1.0f);
  const float wiDotN = dot(wi, N);
  const float woDotN = dot(wl, N);
  if (mat.type == MAT_ROUGHCONDUCTOR && wiDotN <= 0.0f) return false;
  if (wiDotN * woDotN <= 0.0f) return false;
  V3 m = add(wi, wl);
  const float ml = sqrtf(dot(m, m));
  if (!(ml > 0.0f)) return false;
  m = mul(m, 1.0f / ml);
  if (dot(m, N) < 0.0f) m = mul(m, -1.0f);
  const bool ggx = mat.distribution == DIST_GGX;
  const float a = ggx ? roughness : roughness * (1.2f - 0.2f * sqrtf(fabsf(wiDotN)));
  const float D = ggx ? D_ggx(m, N, a) : D_beckmann(m, N, a);
  const float G = ggx ? G1_ggx(wi, m, N, a) * G1_ggx(wl, m, N, a) : G1_beckmann(wi, m, a) * G1_beckmann(wl, m, a);
  const float woDotM = fabsf(dot(wl, m));
  if (!(woDotM > 0.0f) || !(D > 0.0f)) return false;
  pdf = D * fabsf(dot(m, N)) / (4.0f * woDotM);
  const float base = D * G / (4.0f * fabsf(wiDotN));
  if (mat.type == MAT_ROUGHCONDUCTOR) {
    fcos = v3(fresnel_conductor(mat.eta[0], mat.k[0], wiDotN) * base, fresnel_conductor(mat.eta[1], mat.k[1], wiDotN) * base,
              fresnel_conductor(mat.eta[2], mat.k[2], wiDotN) * base);
  } else {
    float cosT = 0.0f;
    const float F = fresnel_dielectric(dot(wi, m), mat.ior, cosT);
    fcos = mul(albedo, F * base);
  }
  return isfinite(pdf) && pdf > 0.0f;
}

// Density of the material's own sampling for the direction it just sampled (0 for delta
// and transmissive lobes, which take no light samples).
__device__ __forceinline__ float bsdf_sampled_pdf(const DevMaterial& mat, const ScatterResult& s, V3 d, V3 N) {
  if (s.status != SCATTER_REFLECT) return 0.0f;
  if (mat.type == MAT_LAMBERT) {
    const V3 norm_o = mul(N, dot(N, d) > 0.0f ? -1.0f : 1.0f);
    return fmaxf(dot(normalize(s.dir), norm_o), 0.0f) * (float)ILLUME_INV_PI_D;
  }
  if (mat.type == MAT_ROUGHCONDUCTOR || mat.type == MAT_ROUGHREFLECTIVE) {
    const float woDotM = fabsf(dot(normalize(s.dir), s.m));
    return woDotM > 0.0f ? s.pdf_m / (4.0f * woDotM) : 0.0f;
  }
  return 0.0f;
}

}  // namespace illume
