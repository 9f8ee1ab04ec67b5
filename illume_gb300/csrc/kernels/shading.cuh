// Surface shading on the device: textures (src/texture.cu:129-162) and one BSDF
// interaction per material (the material switch of pathtrace_kernel,
// src/renderer.cu:183-376), plus the GGX variant of the rough materials.
#pragma once

#include "../common/dmath.cuh"
#include "../common/types.h"

namespace illume {

__device__ __forceinline__ int wrap_index(int i, int n) {
  const int r = i % n;
  return r < 0 ? r + n : r;
}

// Constant / checkerboard / bitmap. Bitmaps: wrap addressing, normalised coordinates;
// HDR texels filtered bilinearly with exact FP32 weights, LDR texels point sampled / 255.
__device__ __forceinline__ V3 tex_eval(const SceneView& sc, int id, float u, float v) {
  const DevTexture& t = sc.textures[id];
  if (t.type == TEX_CONSTANT) return v3(t.c[0], t.c[1], t.c[2]);
  if (t.type == TEX_CHECKER) {
    const int x = (int)((float)(int)t.scale[0] * (u + 0.25f));
    const int y = (int)((float)(int)t.scale[1] * v);
    const bool on = (x + y) % 2 == 0;
    return on ? v3(t.c[0], t.c[1], t.c[2]) : v3(t.off[0], t.off[1], t.off[2]);
  }
  const float fu = u * t.scale[0], fv = v * t.scale[1];
  const int w = t.width, h = t.height;
  if (!t.hdr) {
    const int ix = wrap_index((int)floorf(fu * (float)w), w), iy = wrap_index((int)floorf(fv * (float)h), h);
    const float4 p = __ldg(t.texels + (size_t)iy * w + ix);
    return v3(p.x / 255.0f, p.y / 255.0f, p.z / 255.0f);
  }
  const float x = fu * (float)w - 0.5f, y = fv * (float)h - 0.5f;
  const float x0f = floorf(x), y0f = floorf(y);
  const float ax = x - x0f, ay = y - y0f;
  const int x0 = wrap_index((int)x0f, w), x1 = wrap_index((int)x0f + 1, w);
  const int y0 = wrap_index((int)y0f, h), y1 = wrap_index((int)y0f + 1, h);
  const float4 t00 = __ldg(t.texels + (size_t)y0 * w + x0), t10 = __ldg(t.texels + (size_t)y0 * w + x1);
  const float4 t01 = __ldg(t.texels + (size_t)y1 * w + x0), t11 = __ldg(t.texels + (size_t)y1 * w + x1);
  const float bx = 1.0f - ax, by = 1.0f - ay;
  const float r = (t00.x * bx + t10.x * ax) * by + (t01.x * bx + t11.x * ax) * ay;
  const float g = (t00.y * bx + t10.y * ax) * by + (t01.y * bx + t11.y * ax) * ay;
  const float b = (t00.z * bx + t10.z * ax) * by + (t01.z * bx + t11.z * ax) * ay;
  return v3(r, g, b);
}

// Environment lookup on escape (src/renderer.cu:378-386).
__device__ __forceinline__ V3 env_eval(const SceneView& sc, V3 d) {
  if (sc.env_tex < 0) return v3(0.0f, 0.0f, 0.0f);
  const float u = (float)((double)(atan2f(d.z, d.x) * 0.5f) * ILLUME_INV_PI_D + 0.5);
  const float v = (float)(0.5 - (double)asinf(d.y) * ILLUME_INV_PI_D);
  return tex_eval(sc, sc.env_tex, u, v);
}

enum { SCATTER_KILLED = 0, SCATTER_REFLECT = 1, SCATTER_TRANSMIT = 2 };
static constexpr int kMediumUnchanged = -2;

struct ScatterResult {
  int status;
  V3 dir, weight, offset_dir;
  float offset_sign;
  int medium;
  float D, pdf_m, G, F;
  V3 m;
};

// One interaction with a non-emissive material. `rng()` returns the next uniform of the
// path's bounce stream, consumed in the reference's order. The throughput multiplier
// keeps the reference's grouping of products.
template <class Rng>
__device__ __forceinline__ ScatterResult scatter(const DevMaterial& mat, V3 d, V3 N, V3 albedo, float roughness,
                                                 Rng& rng) {
  ScatterResult s;
  s.status = SCATTER_REFLECT;
  s.medium = kMediumUnchanged;
  s.offset_sign = 1.0f;
  s.D = s.pdf_m = s.G = s.F = 0.0f;
  s.m = v3(0.0f, 0.0f, 0.0f);
  s.weight = v3(0.0f, 0.0f, 0.0f);
  s.dir = v3(0.0f, 0.0f, 0.0f);
  const V3 norm_o = mul(N, dot(N, d) > 0.0f ? -1.0f : 1.0f);
  s.offset_dir = norm_o;
  switch (mat.type) {
    case MAT_LAMBERT: {
      s.weight = albedo;
      const float u1 = rng(), u2 = rng();
      s.dir = to_basis(sample_hemisphere_cosine(u1, u2), norm_o);
      return s;
    }
    case MAT_REFLECTIVE:
      s.weight = v3(0.99f, 0.99f, 0.99f);
      s.dir = reflect(d, norm_o);
      return s;
    case MAT_REFRACTIVE: {
      const float cosI = -dot(d, N);
      float cosT = 0.0f;
      const float F = fresnel_dielectric(cosI, mat.ior, cosT);
      s.F = F;
      if (F == 1.0f || rng() < F) {
        s.dir = reflect(d, N);
      } else {
        const float eta = cosI < 0.0f ? mat.ior : 1.0f / mat.ior;
        s.medium = cosI > 0.0f ? mat.medium : -1;
        s.dir = add(mul(d, eta), mul(norm_o, eta * fabsf(cosI) - cosT));
        s.offset_sign = -1.0f;
        s.status = SCATTER_TRANSMIT;
      }
      s.weight = albedo;
      return s;
    }
    case MAT_ROUGHREFLECTIVE:
    case MAT_ROUGHREFRACTIVE:
    case MAT_ROUGHCONDUCTOR: {
      const V3 wi = mul(d, -1.0f);
      const float wiDotN = dot(wi, N);
      if (mat.type == MAT_ROUGHCONDUCTOR && wiDotN <= 0.0f) { s.status = SCATTER_KILLED; return s; }
      const bool ggx = mat.distribution == DIST_GGX;
      const float a = ggx ? roughness : roughness * (1.2f - 0.2f * sqrtf(fabsf(wiDotN)));
      const float u1 = rng(), u2 = rng();
      V3 m = ggx ? sample_ggx(a, u1, u2) : sample_beckmann(a, u1, u2);
      m = to_basis(m, N);
      s.m = m;
      s.D = ggx ? D_ggx(m, N, a) : D_beckmann(m, N, a);
      s.pdf_m = s.D * fabsf(dot(m, N));
      const float wiDotM = dot(wi, m);
      if (mat.type == MAT_ROUGHCONDUCTOR) {
        const V3 F = v3(fresnel_conductor(mat.eta[0], mat.k[0], wiDotN), fresnel_conductor(mat.eta[1], mat.k[1], wiDotN),
                        fresnel_conductor(mat.eta[2], mat.k[2], wiDotN));
        s.F = F.x;
        s.dir = reflect(d, m);
        if (wiDotN * dot(s.dir, N) <= 0.0f) { s.status = SCATTER_KILLED; return s; }
        s.G = ggx ? G1_ggx(wi, m, N, a) * G1_ggx(s.dir, m, N, a) : G1_beckmann(wi, m, a) * G1_beckmann(s.dir, m, a);
        const float weight = (s.G * fabsf(wiDotM)) / (fabsf(wiDotN) * fabsf(dot(m, N)));
        s.weight = mul(F, weight);
        s.offset_dir = m;
        return s;
      }
      float wiDotT = 0.0f;
      const float F = fresnel_dielectric(wiDotM, mat.ior, wiDotT);
      s.F = F;
      float weight;
      if (mat.type == MAT_ROUGHREFLECTIVE) {
        s.dir = reflect(d, m);
        if (wiDotN * dot(s.dir, N) <= 0.0f) { s.status = SCATTER_KILLED; return s; }
        s.G = ggx ? G1_ggx(wi, m, N, a) * G1_ggx(s.dir, m, N, a) : G1_beckmann(wi, m, a) * G1_beckmann(s.dir, m, a);
        weight = (F * s.G * fabsf(wiDotM)) / (fabsf(wiDotN) * fabsf(dot(m, N)));
      } else {
        if (F == 1.0f || rng() < F) {
          s.dir = reflect(d, m);
          if (wiDotN * dot(s.dir, N) <= 0.0f) { s.status = SCATTER_KILLED; return s; }
        } else {
          const float eta = wiDotM < 0.0f ? mat.ior : 1.0f / mat.ior;
          s.medium = wiDotM > 0.0f ? mat.medium : -1;
          s.dir = sub(mul(m, wiDotM * eta - (wiDotM > 0.0f ? 1.0f : -1.0f) * wiDotT), mul(wi, eta));
          if (wiDotN * dot(s.dir, N) >= 0.0f) { s.status = SCATTER_KILLED; return s; }
          s.offset_sign = -1.0f;
          s.status = SCATTER_TRANSMIT;
        }
        s.G = ggx ? G1_ggx(wi, m, N, a) * G1_ggx(s.dir, m, N, a) : G1_beckmann(wi, m, a) * G1_beckmann(s.dir, m, a);
        weight = (s.G * fabsf(wiDotM)) / (fabsf(wiDotN) * fabsf(dot(m, N)));
      }
      s.weight = mul(albedo, weight);
      return s;
    }
    case MAT_CONDUCTOR: {
      const float cosI = -dot(d, N);
      if (cosI <= 0.0f) { s.status = SCATTER_KILLED; return s; }
      s.dir = reflect(d, norm_o);
      s.weight = v3(fresnel_conductor(mat.eta[0], mat.k[0], cosI), fresnel_conductor(mat.eta[1], mat.k[1], cosI),
                    fresnel_conductor(mat.eta[2], mat.k[2], cosI));
      s.F = s.weight.x;
      return s;
    }
    case MAT_PLASTIC: {
      const float cosI = -dot(d, N);
      float cosT = 0.0f;
      const float F = fresnel_dielectric(cosI, mat.ior, cosT);
      s.F = F;
      const float u1 = rng();
      if (F == 1.0f || u1 < F) {
        s.dir = reflect(d, N);
        s.weight = v3(0.99f, 0.99f, 0.99f);
      } else {
        const float u2 = rng();
        const float uu = (float)((double)(u1 - F) / (1.0 - (double)F));
        s.dir = to_basis(sample_hemisphere_cosine(uu, u2), norm_o);
        const float cosO = dot(s.dir, N);
        const float Fo = fresnel_dielectric(cosO, mat.ior, cosT);
        const V3 diff = divs(albedo, 1.0f - mat.diffuse_fresnel);
        const float inv_eta = 1.0f / mat.ior;
        s.weight = mul(diff, inv_eta * inv_eta * (1.0f - Fo));
      }
      return s;
    }
    default:
      s.status = SCATTER_KILLED;
      return s;
  }
}

}  // namespace illume
