// Device vector math for the path tracer kernels.
//
// The operation order of every helper follows the reference's vector code
// (src/math/vector3.cu, src/math/matrix4.cu:203-209, src/math/sample.cu) so that, with
// this project's -fmad=false build, the FP32 results match a CPU evaluation of the same
// expressions operation by operation. Fused multiply-adds appear only where written
// explicitly (__fmaf_rn), in code whose result is not compared bit for bit (box tests).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <float.h>
#include <stdint.h>

namespace illume {

#define ILLUME_PI_D 3.14159265358979323846
#define ILLUME_INV_PI_D 0.318309886183790671538

struct V3 { float x, y, z; };

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 mul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 mulv(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ V3 divs(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return (a.x * b.x) + (a.y * b.y) + (a.z * b.z); }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float length2(V3 v) { return (v.x * v.x) + (v.y * v.y) + (v.z * v.z); }
// reciprocal of the length, then three multiplies (src/math/vector3.cu:43-51)
__device__ __forceinline__ V3 normalize(V3 v) {
  const float inv = 1.0f / sqrtf(length2(v));
  return v3(v.x * inv, v.y * inv, v.z * inv);
}
// src/math/vector3.cu:85-104
__device__ __forceinline__ V3 to_basis(V3 v, V3 n) {
  V3 t = fabsf(n.x) > fabsf(n.y) ? v3(n.z, 0.0f, -n.x) : v3(0.0f, n.z, -n.y);
  const V3 b = cross(n, t);
  t = cross(b, n);
  return normalize(add(add(mul(t, v.x), mul(n, v.y)), mul(b, v.z)));
}
// src/math/vector3.cu:129-133
__device__ __forceinline__ V3 reflect(V3 v, V3 n) { return sub(v, mul(mul(n, dot(v, n)), 2.0f)); }

// rows of a 3x4 affine matrix applied to (v, w): src/math/matrix4.cu:203-209
__device__ __forceinline__ V3 xform(const float* m, V3 v, float w) {
  return v3(m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * w,
            m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * w,
            m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * w);
}

// (float)(2 * ILLUME_PI * u) evaluated in double, as the reference's double constant
// makes it (src/math/sample.cu:11).
__device__ __forceinline__ float two_pi_times(float u) { return (float)(2.0 * ILLUME_PI_D * (double)u); }

// ---- samplers: src/math/sample.cu ----
__device__ __forceinline__ V3 sample_hemisphere_cosine(float u1, float u2) {
  const float r = sqrtf(u1);
  const float t = two_pi_times(u2);
  float s, c;
  sincosf(t, &s, &c);
  return v3(r * c, sqrtf(1.0f - u1), r * s);
}
__device__ __forceinline__ V3 sample_circle(float u1, float u2) {
  const float r = sqrtf(u1);
  const float d = two_pi_times(u2);
  float s, c;
  sincosf(d, &s, &c);
  return v3(r * c, r * s, 0.0f);
}
__device__ __forceinline__ V3 sample_sphere(float u1, float u2) {
  const float up = u1 * 2.0f - 1.0f;
  const float theta = two_pi_times(u2);
  const float o = sqrtf(1.0f - up * up);
  float s, c;
  sincosf(theta, &s, &c);
  return v3(c * o, up, s * o);
}
// src/math/sample.cu:36-52; exact = sin from 1 - cos^2 (the reference uses 1 - cos)
__device__ __forceinline__ V3 sample_hg(float g, float u1, float u2, bool exact) {
  if (g == 0.0f) return sample_sphere(u1, u2);
  const float phi = two_pi_times(u1);
  const float frac = (1.0f - g * g) / (1.0f + g * (2.0f * u2 - 1.0f));
  const float cosT = (1.0f + g * g - frac * frac) / (2.0f * g);
  const float sinT = sqrtf(exact ? fmaxf(1.0f - cosT * cosT, 0.0f) : fmaxf(1.0f - cosT, 0.0f));
  float s, c;
  sincosf(phi, &s, &c);
  return v3(c * sinT, cosT, s * sinT);
}

// ---- Fresnel: src/fresnel.h:10-57 ----
__device__ __forceinline__ float fresnel_dielectric(float cosI, float ior, float& cosT) {
  const float eta = cosI < 0.0f ? ior : 1.0f / ior;
  const float sinTSq = eta * eta * (1.0f - cosI * cosI);
  if (sinTSq >= 1.0f) { cosT = 0.0f; return 1.0f; }
  cosI = fabsf(cosI);
  cosT = sqrtf(1.0f - sinTSq);
  const float rperp = (eta * cosI - cosT) / (eta * cosI + cosT);
  const float rpar = (cosI - eta * cosT) / (cosI + eta * cosT);
  return (rperp * rperp + rpar * rpar) * 0.5f;
}
__device__ __forceinline__ float fresnel_conductor(float eta, float k, float cosI) {
  const float cosISq = cosI * cosI;
  const float sinISq = 1.0f - cosISq;
  const float etaSq = eta * eta;
  const float kSq = k * k;
  const float t0 = etaSq - kSq - sinISq;
  const float a2pb2 = sqrtf(t0 * t0 + 4.0f * etaSq * kSq);
  const float t1 = a2pb2 + cosISq;
  const float a = sqrtf(0.5f * (a2pb2 + t0));
  const float t2 = 2.0f * a * cosI;
  const float Rs = (t1 - t2) / (t1 + t2);
  const float t3 = cosISq * a2pb2 + sinISq * sinISq;
  const float t4 = t2 * sinISq;
  const float Rp = Rs * (t3 - t4) / (t3 + t4);
  return 0.5f * (Rp + Rs);
}

// ---- microfacet distributions ----
// Beckmann: src/microfacet.cu:7-52
__device__ __forceinline__ float D_beckmann(V3 m, V3 n, float alpha) {
  const float alphaSq = alpha * alpha;
  const float cosT = dot(m, n);
  const float cosTSq = cosT * cosT;
  const float tanTSq = (cosTSq - 1.0f) / cosTSq;
  return (float)(ILLUME_INV_PI_D * (double)expf(-tanTSq / alphaSq) / (double)(alphaSq * cosTSq * cosTSq));
}
__device__ __forceinline__ float G1_beckmann(V3 v, V3 n, float alpha) {
  const float cosV = dot(v, n);
  const float tanV = sqrtf(1.0f - cosV * cosV) / cosV;
  const float a = 1.0f / (alpha * fabsf(tanV));
  if ((double)a < 1.6) return (3.535f * a + 2.181f * a * a) / (1.0f + 2.276f * a + 2.577f * a * a);
  return 1.0f;
}
__device__ __forceinline__ V3 sample_beckmann(float a, float u1, float u2) {
  const float theta = atanf(sqrtf(-a * a * logf(1.0f - u1)));
  const float phi = two_pi_times(u2);
  float st, ct, sp, cp;
  sincosf(theta, &st, &ct);
  sincosf(phi, &sp, &cp);
  return v3(st * cp, ct, st * sp);
}
// GGX (Walter, Marschner, Li, Torrance 2007, eqs. 33-35)
__device__ __forceinline__ float D_ggx(V3 m, V3 n, float alpha) {
  const float c = dot(m, n);
  if (c <= 0.0f) return 0.0f;
  const float c2 = c * c;
  const float a2 = alpha * alpha;
  const float t = a2 + (1.0f - c2) / c2;
  return (float)((double)a2 * ILLUME_INV_PI_D / (double)(c2 * c2 * t * t));
}
__device__ __forceinline__ float G1_ggx(V3 v, V3 m, V3 n, float alpha) {
  const float vn = dot(v, n);
  const float vm = dot(v, m);
  if (vm * vn <= 0.0f) return 0.0f;
  const float c2 = vn * vn;
  const float tan2 = fmaxf(1.0f - c2, 0.0f) / c2;
  return 2.0f / (1.0f + sqrtf(1.0f + alpha * alpha * tan2));
}
__device__ __forceinline__ V3 sample_ggx(float a, float u1, float u2) {
  const float theta = atanf(a * sqrtf(u1) / sqrtf(1.0f - u1));
  const float phi = two_pi_times(u2);
  float st, ct, sp, cp;
  sincosf(theta, &st, &ct);
  sincosf(phi, &sp, &cp);
  return v3(st * cp, ct, st * sp);
}

}  // namespace illume
