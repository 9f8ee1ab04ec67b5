// CPU restatement of illume's unidirectional path tracer ("the oracle").
//
// TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline
// use it, as the checker and as the timed CPU baseline; the product never links it.
//
// Templated on the arithmetic type R: R = float follows the reference's FP32 arithmetic
// operation by operation (compile with -ffp-contract=off), including the places where
// the reference's double-precision constants ILLUME_PI / ILLUME_INV_PI promote an
// expression to double (src/math/mathutils.h:6-7). R = double evaluates the same
// estimator in double precision (the FP64 oracle).
//
// Each function cites the reference code it restates (paths relative to the reference
// project). Extensions beyond the reference are marked EXTENSION:
//   * watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013),
//   * GGX microfacet distribution (Walter, Marschner, Li, Torrance, EGSR 2007),
//   * exact Henyey-Greenstein sampling (the reference's sampler has a sin/cos slip,
//     src/math/sample.cu:49, kept as the default "reference" phase mode).
#pragma once

#include <stdint.h>
#include <float.h>
#include <math.h>
#include <vector>
#include <algorithm>

#include "philox.h"

namespace oracle {

static const double kPi = 3.14159265358979323846;       // src/math/mathutils.h:6
static const double kInvPi = 0.318309886183790671538;   // src/math/mathutils.h:7

// ---- type-dispatched math (float -> the f-suffixed libm call, double -> double) ----
static inline float m_sqrt(float x) { return sqrtf(x); }
static inline double m_sqrt(double x) { return sqrt(x); }
static inline float m_sin(float x) { return sinf(x); }
static inline double m_sin(double x) { return sin(x); }
static inline float m_cos(float x) { return cosf(x); }
static inline double m_cos(double x) { return cos(x); }
static inline float m_exp(float x) { return expf(x); }
static inline double m_exp(double x) { return exp(x); }
static inline float m_log(float x) { return logf(x); }
static inline double m_log(double x) { return log(x); }
static inline float m_atan(float x) { return atanf(x); }
static inline double m_atan(double x) { return atan(x); }
static inline float m_atan2(float y, float x) { return atan2f(y, x); }
static inline double m_atan2(double y, double x) { return atan2(y, x); }
static inline float m_asin(float x) { return asinf(x); }
static inline double m_asin(double x) { return asin(x); }
static inline float m_pow(float x, float y) { return powf(x, y); }
static inline double m_pow(double x, double y) { return pow(x, y); }
static inline float m_tan(float x) { return tanf(x); }
static inline double m_tan(double x) { return tan(x); }
static inline float m_abs(float x) { return fabsf(x); }
static inline double m_abs(double x) { return fabs(x); }
static inline float m_min(float a, float b) { return fminf(a, b); }
static inline double m_min(double a, double b) { return fmin(a, b); }
static inline float m_max(float a, float b) { return fmaxf(a, b); }
static inline double m_max(double a, double b) { return fmax(a, b); }

// (R)(2 * ILLUME_PI * u): the reference evaluates this product in double and stores
// it into a float (src/math/sample.cu:11, 23, 31, 46; src/microfacet.cu:50).
template <class R> static inline R two_pi_times(R u) { return (R)(2.0 * kPi * (double)u); }

template <class R> struct V3 { R x, y, z; };
template <class R> static inline V3<R> v3(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> static inline V3<R> add(V3<R> a, V3<R> b) { return v3<R>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> static inline V3<R> sub(V3<R> a, V3<R> b) { return v3<R>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> static inline V3<R> mul(V3<R> a, R s) { return v3<R>(a.x * s, a.y * s, a.z * s); }
template <class R> static inline V3<R> mulv(V3<R> a, V3<R> b) { return v3<R>(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class R> static inline V3<R> divv(V3<R> a, V3<R> b) { return v3<R>(a.x / b.x, a.y / b.y, a.z / b.z); }
template <class R> static inline V3<R> divs(V3<R> a, R s) { return v3<R>(a.x / s, a.y / s, a.z / s); }
template <class R> static inline V3<R> adds(V3<R> a, R s) { return v3<R>(s + a.x, s + a.y, s + a.z); }
// src/math/vector3.cu:79-83 (left to right)
template <class R> static inline R dot(V3<R> a, V3<R> b) { return (a.x * b.x) + (a.y * b.y) + (a.z * b.z); }
// src/math/vector3.cu:71-77
template <class R> static inline V3<R> cross(V3<R> a, V3<R> b) {
  return v3<R>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class R> static inline R length2(V3<R> v) { return (v.x * v.x) + (v.y * v.y) + (v.z * v.z); }
// src/math/vector3.cu:43-51: multiply by the reciprocal length
template <class R> static inline V3<R> normalize(V3<R> v) {
  const R inv = (R)1 / m_sqrt(length2(v));
  return v3<R>(v.x * inv, v.y * inv, v.z * inv);
}
// src/math/vector3.cu:85-104
template <class R> static inline V3<R> to_basis(V3<R> v, V3<R> n) {
  V3<R> t = m_abs(n.x) > m_abs(n.y) ? v3<R>(n.z, 0, -n.x) : v3<R>(0, n.z, -n.y);
  const V3<R> b = cross(n, t);
  t = cross(b, n);
  return normalize(add(add(mul(t, v.x), mul(n, v.y)), mul(b, v.z)));
}
// src/math/vector3.cu:129-133
template <class R> static inline V3<R> reflect(V3<R> v, V3<R> n) { return sub(v, mul(mul(n, dot(v, n)), (R)2)); }
template <class R, class S> static inline V3<R> cast3(V3<S> a) { return v3<R>((R)a.x, (R)a.y, (R)a.z); }

// 3x4 affine matrix (rows), applied as src/math/matrix4.cu:203-209.
struct Mat34 { float m[3][4]; };
template <class R> static inline V3<R> xform(const Mat34& M, V3<R> v, R w) {
  R r[3];
  for (int i = 0; i < 3; ++i)
    r[i] = (R)M.m[i][0] * v.x + (R)M.m[i][1] * v.y + (R)M.m[i][2] * v.z + (R)M.m[i][3] * w;
  return v3<R>(r[0], r[1], r[2]);
}

// ---- sampling: src/math/sample.cu ----
template <class R> static inline V3<R> sample_hemisphere_cosine(R u1, R u2) {   // :7-17
  const R r = m_sqrt(u1);
  const R t = two_pi_times(u2);
  return v3<R>(r * m_cos(t), m_sqrt((R)1 - u1), r * m_sin(t));
}
template <class R> static inline V3<R> sample_circle(R u1, R u2) {              // :19-25
  const R r = m_sqrt(u1);
  const R d = two_pi_times(u2);
  return v3<R>(r * m_cos(d), r * m_sin(d), 0);
}
template <class R> static inline V3<R> sample_sphere(R u1, R u2) {              // :27-34
  const R up = u1 * 2 - 1;
  const R theta = two_pi_times(u2);
  const R o = m_sqrt((R)1 - up * up);
  return v3<R>(m_cos(theta) * o, up, m_sin(theta) * o);
}
// :36-52. exact_hg selects sin = sqrt(1 - cos^2) (EXTENSION); the reference takes
// sqrt(max(1 - cos, 0)).
template <class R> static inline V3<R> sample_hg(R g, R u1, R u2, bool exact_hg) {
  if (g == (R)0) return sample_sphere(u1, u2);
  const R phi = two_pi_times(u1);
  const R frac = ((R)1 - g * g) / ((R)1 + g * ((R)2 * u2 - 1));
  const R cosT = ((R)1 + g * g - frac * frac) / ((R)2 * g);
  const R s = exact_hg ? m_max((R)1 - cosT * cosT, (R)0) : m_max((R)1 - cosT, (R)0);
  const R sinT = m_sqrt(s);
  return v3<R>(m_cos(phi) * sinT, cosT, m_sin(phi) * sinT);
}

// ---- Fresnel: src/fresnel.h ----
template <class R> static inline R fresnel_dielectric(R cosI, R ior, R& cosT) {   // :10-26
  const R eta = cosI < (R)0 ? ior : (R)1 / ior;
  const R sinTSq = eta * eta * ((R)1 - cosI * cosI);
  if (sinTSq >= (R)1) { cosT = 0; return 1; }
  cosI = m_abs(cosI);
  cosT = m_sqrt((R)1 - sinTSq);
  const R rperp = (eta * cosI - cosT) / (eta * cosI + cosT);
  const R rpar = (cosI - eta * cosT) / (cosI + eta * cosT);
  return (rperp * rperp + rpar * rpar) * (R)0.5f;
}
template <class R> static inline R fresnel_conductor(R eta, R k, R cosI) {         // :28-49
  const R cosISq = cosI * cosI;
  const R sinISq = 1 - cosISq;
  const R etaSq = eta * eta;
  const R kSq = k * k;
  const R t0 = etaSq - kSq - sinISq;
  const R a2pb2 = m_sqrt(t0 * t0 + (R)4 * etaSq * kSq);
  const R t1 = a2pb2 + cosISq;
  const R a = m_sqrt((R)0.5f * (a2pb2 + t0));
  const R t2 = (R)2 * a * cosI;
  const R Rs = (t1 - t2) / (t1 + t2);
  const R t3 = cosISq * a2pb2 + sinISq * sinISq;
  const R t4 = t2 * sinISq;
  const R Rp = Rs * (t3 - t4) / (t3 + t4);
  return (R)0.5f * (Rp + Rs);
}
template <class R> static inline V3<R> fresnel_conductor3(V3<R> eta, V3<R> k, R cosI) {
  return v3<R>(fresnel_conductor(eta.x, k.x, cosI), fresnel_conductor(eta.y, k.y, cosI),
               fresnel_conductor(eta.z, k.z, cosI));
}
// :59-73, with the reference's argument order (cosI := ior, ior := sqrt(i/N)).
static inline float diffuse_fresnel(float ior, int samples) {
  float cosT;
  double ret = 0.0;
  float fb = fresnel_dielectric<float>(0.0f, ior, cosT);
  for (int i = 1; i <= samples; i++) {
    const float cosTSq = (float)i / samples;
    const float fa = fresnel_dielectric<float>(ior, sqrtf(cosTSq), cosT);
    ret += (double)(fa + fb) * (0.5 / samples);
    fb = fa;
  }
  return (float)ret;
}

// ---- microfacet distributions ----
enum { DIST_BECKMANN = 0, DIST_GGX = 1 };
// Beckmann: src/microfacet.cu:7-52.
template <class R> static inline R D_beckmann(V3<R> m, V3<R> n, R alpha) {
  const R alphaSq = alpha * alpha;
  const R cosT = dot(m, n);
  const R cosTSq = cosT * cosT;
  const R tanTSq = (cosTSq - (R)1) / cosTSq;
  return (R)(kInvPi * (double)m_exp(-tanTSq / alphaSq) / (double)(alphaSq * cosTSq * cosTSq));
}
template <class R> static inline R G1_beckmann(V3<R> v, V3<R> n, R alpha) {
  const R cosV = dot(v, n);
  const R tanV = m_sqrt((R)1 - cosV * cosV) / cosV;
  const R a = (R)1 / (alpha * m_abs(tanV));
  if ((double)a < 1.6) return ((R)3.535f * a + (R)2.181f * a * a) / ((R)1 + (R)2.276f * a + (R)2.577f * a * a);
  return 1;
}
template <class R> static inline R G_beckmann(V3<R> i, V3<R> o, V3<R> n, R alpha) {
  return G1_beckmann(i, n, alpha) * G1_beckmann(o, n, alpha);
}
template <class R> static inline V3<R> sample_beckmann(R a, R u1, R u2) {
  const R theta = m_atan(m_sqrt(-a * a * m_log((R)1 - u1)));
  const R phi = (R)(2.0 * kPi * (double)u2);
  return v3<R>(m_sin(theta) * m_cos(phi), m_cos(theta), m_sin(theta) * m_sin(phi));
}
// EXTENSION: GGX (Walter et al. 2007, eqs. 33-35). G1 uses the macro normal n and the
// positive-characteristic test on (v.m)/(v.n).
template <class R> static inline R D_ggx(V3<R> m, V3<R> n, R alpha) {
  const R c = dot(m, n);
  if (c <= (R)0) return 0;
  const R c2 = c * c;
  const R a2 = alpha * alpha;
  const R t = a2 + ((R)1 - c2) / c2;
  return (R)((double)a2 * kInvPi / (double)(c2 * c2 * t * t));
}
template <class R> static inline R G1_ggx(V3<R> v, V3<R> m, V3<R> n, R alpha) {
  const R vn = dot(v, n);
  const R vm = dot(v, m);
  if (vm * vn <= (R)0) return 0;
  const R c2 = vn * vn;
  const R tan2 = m_max((R)1 - c2, (R)0) / c2;
  return (R)2 / ((R)1 + m_sqrt((R)1 + alpha * alpha * tan2));
}
template <class R> static inline R G_ggx(V3<R> i, V3<R> o, V3<R> m, V3<R> n, R alpha) {
  return G1_ggx(i, m, n, alpha) * G1_ggx(o, m, n, alpha);
}
template <class R> static inline V3<R> sample_ggx(R a, R u1, R u2) {
  const R theta = m_atan(a * m_sqrt(u1) / m_sqrt((R)1 - u1));
  const R phi = two_pi_times(u2);
  return v3<R>(m_sin(theta) * m_cos(phi), m_cos(theta), m_sin(theta) * m_sin(phi));
}

// ---- ray/primitive tests ----
template <class R> struct Ray { V3<R> o, d; };

// Moller-Trumbore, src/primitives/mesh.cu:445-476 (returns -1 on a miss).
template <class R> static inline R triangle_mt(V3<R> v0, V3<R> v1, V3<R> v2, const Ray<R>& ray, R& u, R& v) {
  const V3<R> e1 = sub(v1, v0), e2 = sub(v2, v0);
  const V3<R> P = cross(ray.d, e2);
  R det = dot(e1, P);
  if (m_abs(det) < (R)FLT_EPSILON) return -1;
  det = (R)1 / det;
  const V3<R> T = sub(ray.o, v0);
  u = dot(T, P) * det;
  if (u < (R)0 || u > (R)1) return -1;
  const V3<R> Q = cross(T, e1);
  v = dot(ray.d, Q) * det;
  if (v < (R)0 || u + v > (R)1) return -1;
  return dot(e2, Q) * det;
}

// EXTENSION: watertight test (Woop et al. 2013), no backface culling, double-precision
// recomputation of the edge functions when one is exactly zero. Returns -1 on a miss;
// u, v are the weights of v1 and v2 (the convention of the test above).
struct WtRay { int kx, ky, kz; float Sx, Sy, Sz; };
static inline WtRay watertight_setup(V3<float> d) {
  WtRay w;
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  w.kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  w.kx = w.kz + 1 == 3 ? 0 : w.kz + 1;
  w.ky = w.kx + 1 == 3 ? 0 : w.kx + 1;
  const float dz = (&d.x)[w.kz];
  if (dz < 0.0f) { int t = w.kx; w.kx = w.ky; w.ky = t; }
  w.Sx = (&d.x)[w.kx] / dz;
  w.Sy = (&d.x)[w.ky] / dz;
  w.Sz = 1.0f / dz;
  return w;
}
static inline float triangle_watertight(V3<float> v0, V3<float> v1, V3<float> v2, V3<float> o, const WtRay& w,
                                        float& u, float& v) {
  const V3<float> A = sub(v0, o), B = sub(v1, o), C = sub(v2, o);
  const float* a = &A.x; const float* b = &B.x; const float* c = &C.x;
  const float Ax = a[w.kx] - w.Sx * a[w.kz], Ay = a[w.ky] - w.Sy * a[w.kz];
  const float Bx = b[w.kx] - w.Sx * b[w.kz], By = b[w.ky] - w.Sy * b[w.kz];
  const float Cx = c[w.kx] - w.Sx * c[w.kz], Cy = c[w.ky] - w.Sy * c[w.kz];
  float U = Cx * By - Cy * Bx;
  float V = Ax * Cy - Ay * Cx;
  float W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
    V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
    W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return -1;
  const float det = U + V + W;
  if (det == 0.0f) return -1;
  const float Az = w.Sz * a[w.kz], Bz = w.Sz * b[w.kz], Cz = w.Sz * c[w.kz];
  const float T = U * Az + V * Bz + W * Cz;
  if ((det < 0.0f && T >= 0.0f) || (det > 0.0f && T <= 0.0f)) return -1;
  const float rcp = 1.0f / det;
  u = V * rcp;
  v = W * rcp;
  return T * rcp;
}
// Double-precision watertight test for the FP64 oracle: same decisions as above with
// every quantity in double.
static inline double triangle_watertight_d(V3<double> v0, V3<double> v1, V3<double> v2, V3<double> o, V3<double> d,
                                           double& u, double& v) {
  const double ax = fabs(d.x), ay = fabs(d.y), az = fabs(d.z);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz + 1 == 3 ? 0 : kz + 1;
  int ky = kx + 1 == 3 ? 0 : kx + 1;
  const double dz = (&d.x)[kz];
  if (dz < 0.0) std::swap(kx, ky);
  const double Sx = (&d.x)[kx] / dz, Sy = (&d.x)[ky] / dz, Sz = 1.0 / dz;
  const V3<double> A = sub(v0, o), B = sub(v1, o), C = sub(v2, o);
  const double* a = &A.x; const double* b = &B.x; const double* c = &C.x;
  const double Ax = a[kx] - Sx * a[kz], Ay = a[ky] - Sy * a[kz];
  const double Bx = b[kx] - Sx * b[kz], By = b[ky] - Sy * b[kz];
  const double Cx = c[kx] - Sx * c[kz], Cy = c[ky] - Sy * c[kz];
  const double U = Cx * By - Cy * Bx, V = Ax * Cy - Ay * Cx, W = Bx * Ay - By * Ax;
  if ((U < 0 || V < 0 || W < 0) && (U > 0 || V > 0 || W > 0)) return -1;
  const double det = U + V + W;
  if (det == 0) return -1;
  const double T = U * (Sz * a[kz]) + V * (Sz * b[kz]) + W * (Sz * c[kz]);
  if ((det < 0 && T >= 0) || (det > 0 && T <= 0)) return -1;
  u = V / det;
  v = W / det;
  return T / det;
}

// Slab test, src/math/aabb.cu:118-151 (returns -FLT_MAX on a miss).
template <class R> static inline R aabb_intersect(V3<R> mn, V3<R> mx, const Ray<R>& r) {
  R tmin = -FLT_MAX, tmax = FLT_MAX;
  const R* o = &r.o.x; const R* d = &r.d.x; const R* lo = &mn.x; const R* hi = &mx.x;
  for (int a = 0; a < 3; ++a) {
    if (d[a] != (R)0) {
      const R t1 = (lo[a] - o[a]) / d[a], t2 = (hi[a] - o[a]) / d[a];
      tmin = m_max(tmin, m_min(t1, t2));
      tmax = m_min(tmax, m_max(t1, t2));
    }
  }
  if (tmax > tmin && tmax >= (R)0) return tmin;
  return -FLT_MAX;
}

// Sphere, src/primitives/sphere.cu:43-77.
template <class R> static inline bool sphere_intersect(V3<R> center, R radius, const Ray<R>& ray, R& t, V3<R>& normal,
                                                     R& u, R& v) {
  const V3<R> l = sub(center, ray.o);
  const R s = dot(l, ray.d);
  const R ls = dot(l, l);
  const R rs = radius * radius;
  if (s < (R)0 && ls > rs) return false;
  const R ms = ls - s * s;
  if (ms > rs) return false;
  const R q = m_sqrt(rs - ms);
  t = s;
  if (ls > rs) t -= q; else t += q;
  const V3<R> pos = add(ray.o, mul(ray.d, t));
  normal = normalize(sub(pos, center));
  u = (R)((double)(m_atan2(normal.z, normal.x) * (R)0.5f) * kInvPi + 0.5);
  v = (R)(0.5 - (double)m_asin(normal.y) * kInvPi);
  return true;
}

// ---- scene ----
enum TexType { TEX_CONSTANT = 0, TEX_CHECKER = 1, TEX_BITMAP = 2 };
struct Texture {
  int type;
  float c[3];        // constant colour, or checkerboard "on"
  float off[3];      // checkerboard "off"
  float scale[2];
  int width, height, hdr;
  const float* texels;  // RGBA float, row-major (LDR texels hold byte values 0..255)
};
enum MatType {
  MAT_EMISSIVE = 0, MAT_DIFFUSE, MAT_SPECULAR, MAT_REFRACTIVE, MAT_ROUGHREFLECTIVE,
  MAT_ROUGHREFRACTIVE, MAT_CONDUCTOR, MAT_ROUGHCONDUCTOR, MAT_PLASTIC
};
struct Material {
  int type;
  int albedo_tex, roughness_tex;
  float ior, diffuse_fresnel;
  float eta[3], k[3];
  int medium;        // index into mediums, -1 = air
  int distribution;  // DIST_BECKMANN / DIST_GGX
};
struct Medium {
  float absorption[3];  // already 1 - json absorption (src/medium.cu:9)
  float scattering, g;
  int active;
};
struct Mesh {
  const float* positions;  // V x 3
  const int* tris;         // T x 3
  const float* normals;    // V x 3 or null (face normals)
  const float* texcoords;  // V x 2 or null
  int num_vertices, num_tris;
};
struct Instance { int mesh, material; Mat34 mat, inv, trans_inv; };
struct Sphere { float center[3]; float radius; int material; };
struct Camera { Mat34 transform; float fov, dof, aperture; };

// Binary BVH over one mesh, built by median split (independent of the product's
// builders); traversal tests boxes in double with a relative margin, so it never
// rejects a box that contains a triangle hit, and the closest hit equals brute force.
struct OBvh {
  struct Node { double lo[3], hi[3]; int left, right, first, count; };
  std::vector<Node> nodes;
  std::vector<int> order;
};
void build_obvh(const Mesh& m, OBvh& bvh);

struct Scene {
  std::vector<Mesh> meshes;
  std::vector<OBvh> bvhs;
  std::vector<Instance> instances;
  std::vector<Sphere> spheres;
  std::vector<Material> materials;
  std::vector<Medium> mediums;
  std::vector<Texture> textures;
  int env_tex = -1;
  Camera camera;
};

enum { ISECT_MT = 0, ISECT_WATERTIGHT = 1 };

// Closest hit, restating get_min_hit (src/renderer.cu:112-137): spheres first, then
// instances, a later candidate replaces the best only if strictly closer. Within one
// mesh the closest t wins and equal t goes to the lower triangle index.
template <class R> struct Hit {
  bool hit;
  R t;
  int sphere;   // index or -1
  int inst;     // index or -1
  int prim;     // triangle index within the mesh, -1 for spheres
  R bu, bv;     // barycentric weights of v1, v2 (mesh) or sphere uv
  V3<R> normal; // world-space shading normal
  int material;
  R uv[2];
};

template <class R> struct TraceCounters { uint64_t nodes = 0, tris = 0; };

// Closest triangle of a mesh along an object-space ray (o, d).
template <class R>
static inline void mesh_closest(const Scene& sc, int mesh_id, V3<R> o, V3<R> d, int isect, R& best_t, int& best_prim,
                                R& best_u, R& best_v) {
  const Mesh& m = sc.meshes[mesh_id];
  const OBvh& bvh = sc.bvhs[mesh_id];
  const Ray<R> ray{o, d};
  WtRay wt{};
  if (isect == ISECT_WATERTIGHT && sizeof(R) == 4) wt = watertight_setup(v3<float>((float)d.x, (float)d.y, (float)d.z));
  const double od[3] = {(double)o.x, (double)o.y, (double)o.z};
  const double dd[3] = {(double)d.x, (double)d.y, (double)d.z};
  int stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const OBvh::Node& nd = bvh.nodes[stack[--sp]];
    // conservative box test in double, boxes widened by a relative margin
    double t0 = 0.0, t1 = INFINITY;
    bool miss = false;
    for (int a = 0; a < 3 && !miss; ++a) {
      const double ext = nd.hi[a] - nd.lo[a];
      const double mag = fmax(fabs(nd.lo[a]), fabs(nd.hi[a]));
      const double pad = 1e-5 * (ext + mag) + 1e-30;
      const double lo = nd.lo[a] - pad, hi = nd.hi[a] + pad;
      if (dd[a] == 0.0) {
        if (od[a] < lo || od[a] > hi) miss = true;
      } else {
        double ta = (lo - od[a]) / dd[a], tb = (hi - od[a]) / dd[a];
        if (ta > tb) std::swap(ta, tb);
        t0 = fmax(t0, ta);
        t1 = fmin(t1, tb);
        if (t0 > t1 * (1.0 + 1e-9) + 1e-300) miss = true;
      }
    }
    if (miss || t0 > (double)best_t * (1.0 + 1e-4) + 1e-30) continue;
    if (nd.count > 0) {
      for (int i = nd.first; i < nd.first + nd.count; ++i) {
        const int p = bvh.order[i];
        const int* tri = m.tris + 3 * p;
        const float* P = m.positions;
        const V3<R> v0 = v3<R>(P[3 * tri[0]], P[3 * tri[0] + 1], P[3 * tri[0] + 2]);
        const V3<R> v1 = v3<R>(P[3 * tri[1]], P[3 * tri[1] + 1], P[3 * tri[1] + 2]);
        const V3<R> v2 = v3<R>(P[3 * tri[2]], P[3 * tri[2] + 1], P[3 * tri[2] + 2]);
        R u = 0, v = 0, t;
        if (isect == ISECT_MT) {
          t = triangle_mt(v0, v1, v2, ray, u, v);
        } else if (sizeof(R) == 4) {
          float fu = 0, fv = 0;
          t = (R)triangle_watertight(cast3<float>(v0), cast3<float>(v1), cast3<float>(v2), cast3<float>(o), wt, fu, fv);
          u = (R)fu; v = (R)fv;
        } else {
          double du = 0, dv = 0;
          t = (R)triangle_watertight_d(cast3<double>(v0), cast3<double>(v1), cast3<double>(v2), cast3<double>(o),
                                       cast3<double>(d), du, dv);
          u = (R)du; v = (R)dv;
        }
        if (t > (R)0 && (t < best_t || (t == best_t && p < best_prim))) {
          best_t = t; best_prim = p; best_u = u; best_v = v;
        }
      }
    } else {
      stack[sp++] = nd.left;
      stack[sp++] = nd.right;
    }
  }
}

// Texture::eval, src/texture.cu:129-162. Bitmaps: wrap addressing with normalised
// coordinates; HDR bilinear with exact weights, LDR point sampled and divided by 255.
template <class R> static inline V3<R> tex_eval(const Scene& sc, int id, R u, R v) {
  const Texture& t = sc.textures[id];
  if (t.type == TEX_CONSTANT) return v3<R>(t.c[0], t.c[1], t.c[2]);
  if (t.type == TEX_CHECKER) {
    const int x = (int)((R)(int)t.scale[0] * (u + (R)0.25f));
    const int y = (int)((R)(int)t.scale[1] * v);
    const bool on = (x + y) % 2 == 0;
    return on ? v3<R>(t.c[0], t.c[1], t.c[2]) : v3<R>(t.off[0], t.off[1], t.off[2]);
  }
  const float fu = (float)u * t.scale[0], fv = (float)v * t.scale[1];
  const int w = t.width, h = t.height;
  auto wrap = [](int i, int n) { int r = i % n; return r < 0 ? r + n : r; };
  if (!t.hdr) {
    const int ix = wrap((int)floorf(fu * (float)w), w), iy = wrap((int)floorf(fv * (float)h), h);
    const float* p = t.texels + 4 * ((size_t)iy * w + ix);
    return v3<R>((R)(p[0] / 255.0f), (R)(p[1] / 255.0f), (R)(p[2] / 255.0f));
  }
  const float x = fu * (float)w - 0.5f, y = fv * (float)h - 0.5f;
  const float x0f = floorf(x), y0f = floorf(y);
  const float ax = x - x0f, ay = y - y0f;
  const int x0 = wrap((int)x0f, w), x1 = wrap((int)x0f + 1, w);
  const int y0 = wrap((int)y0f, h), y1 = wrap((int)y0f + 1, h);
  float out[3];
  for (int c = 0; c < 3; ++c) {
    const float t00 = t.texels[4 * ((size_t)y0 * w + x0) + c], t10 = t.texels[4 * ((size_t)y0 * w + x1) + c];
    const float t01 = t.texels[4 * ((size_t)y1 * w + x0) + c], t11 = t.texels[4 * ((size_t)y1 * w + x1) + c];
    const float top = t00 * (1.0f - ax) + t10 * ax;
    const float bot = t01 * (1.0f - ax) + t11 * ax;
    out[c] = top * (1.0f - ay) + bot * ay;
  }
  return v3<R>(out[0], out[1], out[2]);
}

template <class R>
static inline Hit<R> closest_hit(const Scene& sc, const Ray<R>& ray, int isect, TraceCounters<R>* cnt = nullptr) {
  Hit<R> best{};
  best.hit = false;
  best.t = (R)FLT_MAX;
  best.sphere = best.inst = best.prim = -1;
  for (int s = 0; s < (int)sc.spheres.size(); ++s) {
    const Sphere& sp = sc.spheres[s];
    R t, u, v;
    V3<R> n;
    if (sphere_intersect(v3<R>(sp.center[0], sp.center[1], sp.center[2]), (R)sp.radius, ray, t, n, u, v) && t < best.t) {
      best.hit = true; best.t = t; best.sphere = s; best.inst = -1; best.prim = -1;
      best.normal = n; best.material = sp.material; best.uv[0] = u; best.uv[1] = v;
    }
  }
  for (int i = 0; i < (int)sc.instances.size(); ++i) {
    const Instance& in = sc.instances[i];
    const V3<R> o = xform(in.inv, ray.o, (R)1);
    const V3<R> d = xform(in.inv, ray.d, (R)0);
    R t = (R)FLT_MAX, u = 0, v = 0;
    int prim = -1;
    mesh_closest(sc, in.mesh, o, d, isect, t, prim, u, v);
    if (prim >= 0 && t < best.t) {
      best.hit = true; best.t = t; best.sphere = -1; best.inst = i; best.prim = prim;
      best.bu = u; best.bv = v; best.material = in.material;
    }
  }
  if (best.hit && best.inst >= 0) {
    // normal and uv of the winning triangle, src/primitives/mesh.cu:532-561 and
    // src/primitives/mesh_instance.cu:102-107
    const Instance& in = sc.instances[best.inst];
    const Mesh& m = sc.meshes[in.mesh];
    const int* tri = m.tris + 3 * best.prim;
    const R u = best.bu, v = best.bv;
    V3<R> n;
    if (!m.normals) {
      const float* P = m.positions;
      const V3<R> v0 = v3<R>(P[3 * tri[0]], P[3 * tri[0] + 1], P[3 * tri[0] + 2]);
      const V3<R> v1 = v3<R>(P[3 * tri[1]], P[3 * tri[1] + 1], P[3 * tri[1] + 2]);
      const V3<R> v2 = v3<R>(P[3 * tri[2]], P[3 * tri[2] + 1], P[3 * tri[2] + 2]);
      n = normalize(cross(sub(v1, v0), sub(v2, v0)));
    } else {
      const float* N = m.normals;
      const V3<R> n0 = v3<R>(N[3 * tri[0]], N[3 * tri[0] + 1], N[3 * tri[0] + 2]);
      const V3<R> n1 = v3<R>(N[3 * tri[1]], N[3 * tri[1] + 1], N[3 * tri[1] + 2]);
      const V3<R> n2 = v3<R>(N[3 * tri[2]], N[3 * tri[2] + 1], N[3 * tri[2] + 2]);
      n = normalize(add(mul(n0, (R)1 - u - v), add(mul(n1, u), mul(n2, v))));
    }
    best.normal = normalize(xform(in.trans_inv, n, (R)0));
    if (m.texcoords) {
      const float* T = m.texcoords;
      const R w0 = (R)1 - u - v;
      best.uv[0] = (T[2 * tri[0]] * w0 + T[2 * tri[1]] * u) + T[2 * tri[2]] * v;
      best.uv[1] = (T[2 * tri[0] + 1] * w0 + T[2 * tri[1] + 1] * u) + T[2 * tri[2] + 1] * v;
    } else {
      best.uv[0] = u;
      best.uv[1] = v;
    }
  }
  (void)cnt;
  return best;
}

// ---- one path, restating init_rays (src/renderer.cu:81-110) and the bounce loop of
// pathtrace_kernel (src/renderer.cu:139-388) for a single (pixel, sample) ----
struct RenderParams {
  int width, height;
  int max_depth;
  float ray_bias;
  uint32_t seed, job;
  int isect;      // ISECT_MT / ISECT_WATERTIGHT
  int exact_hg;   // 0 = reference HG sampler, 1 = exact
  int nee;        // EXTENSION: 1 = next-event estimation with MIS (needs the scene's light tables)
};

struct CameraSetup { float pixel_size, left, top; };
// allocate_render_info_gpu, src/renderer.cu:443-458
static inline CameraSetup camera_setup(const Camera& cam, int W, int H) {
  CameraSetup c;
  const float dim_ratio = (float)H / (float)W;
  const float tan_half_fov = tanf((float)(kPi * (double)cam.fov / 360));
  const float dofmfov = cam.dof * tan_half_fov;
  c.pixel_size = dofmfov * 2 / (float)W;
  c.left = -1 * dofmfov;
  c.top = dim_ratio * dofmfov;
  return c;
}

template <class R>
static inline Ray<R> camera_ray(const Scene& sc, const CameraSetup& cs, int W, int pixel, philox::Stream& rng) {
  const int x = pixel % W, y = pixel / W;
  const R ps = (R)cs.pixel_size;
  const R left_edge = (R)cs.left + ps * (R)x;
  const R top_edge = (R)cs.top - ps * (R)y;
  const R r_x = left_edge + ps * (R)rng.next();
  const R r_y = top_edge - ps * (R)rng.next();
  V3<R> pos = v3<R>(0, 0, 0);
  if (sc.camera.aperture > FLT_EPSILON) {
    const R u1 = (R)rng.next(), u2 = (R)rng.next();
    pos = mul(sample_circle(u1, u2), (R)sc.camera.aperture);
  }
  const V3<R> origin = xform(sc.camera.transform, pos, (R)1);
  const V3<R> image_pos = xform(sc.camera.transform, v3<R>(r_x, r_y, (R)sc.camera.dof), (R)1);
  return Ray<R>{origin, normalize(sub(image_pos, origin))};
}

// ---- one surface interaction: the material switch of pathtrace_kernel
// (src/renderer.cu:183-376) for every non-emissive material. `next()` supplies the
// uniform numbers in the reference's call order. The throughput multiplier `weight`
// keeps the reference's grouping (for example albedo * scalar is formed first and then
// multiplied into the throughput). The new ray starts at hit + offset_dir * offset_sign
// * ray_bias with direction normalize(dir). ----
enum { SCATTER_KILLED = 0, SCATTER_REFLECT = 1, SCATTER_TRANSMIT = 2 };
static const int MEDIUM_UNCHANGED = -2;
template <class R> struct ScatterOut {
  int status;
  V3<R> dir, weight, offset_dir;
  R offset_sign;
  int medium;                  // MEDIUM_UNCHANGED, -1 (air) or a medium index
  R D, pdf_m, G, F;            // microfacet terms of the sampled normal (rough materials)
  V3<R> m;                     // sampled microfacet normal (rough materials)
};

template <class R, class Next>
static inline ScatterOut<R> scatter(const Material& mat, V3<R> d, V3<R> N, V3<R> albedo, R roughness, Next next) {
  ScatterOut<R> s{};
  s.status = SCATTER_REFLECT;
  s.medium = MEDIUM_UNCHANGED;
  s.offset_sign = 1;
  const V3<R> norm_o = mul(N, dot(N, d) > (R)0 ? (R)-1.0f : (R)1.0f);
  s.offset_dir = norm_o;
  switch (mat.type) {
    case MAT_DIFFUSE: {  // :199-207
      s.weight = albedo;
      const R u1 = next(), u2 = next();
      s.dir = to_basis(sample_hemisphere_cosine(u1, u2), norm_o);
      return s;
    }
    case MAT_SPECULAR:  // :208-213 (albedo is not used)
      s.weight = v3<R>((R)0.99f, (R)0.99f, (R)0.99f);
      s.dir = reflect(d, norm_o);
      return s;
    case MAT_REFRACTIVE: {  // :214-235
      const R cosI = -dot(d, N);
      R cosT = 0;
      const R F = fresnel_dielectric(cosI, (R)mat.ior, cosT);
      s.F = F;
      if (F == (R)1 || next() < F) {
        s.dir = reflect(d, N);
      } else {
        const R eta = cosI < (R)0 ? (R)mat.ior : (R)1 / (R)mat.ior;
        s.medium = cosI > (R)0 ? mat.medium : -1;
        s.dir = add(mul(d, eta), mul(norm_o, eta * m_abs(cosI) - cosT));
        s.offset_sign = -1;
        s.status = SCATTER_TRANSMIT;
      }
      s.weight = albedo;
      return s;
    }
    case MAT_ROUGHREFLECTIVE:
    case MAT_ROUGHREFRACTIVE:
    case MAT_ROUGHCONDUCTOR: {  // :236-349
      const V3<R> wi = mul(d, (R)-1.0f);
      const R wiDotN = dot(wi, N);
      if (mat.type == MAT_ROUGHCONDUCTOR && wiDotN <= (R)0) { s.status = SCATTER_KILLED; return s; }
      const bool ggx = mat.distribution == DIST_GGX;
      const R a = ggx ? roughness : roughness * ((R)1.2f - (R)0.2f * m_sqrt(m_abs(wiDotN)));
      const R u1 = next(), u2 = next();
      V3<R> m = ggx ? sample_ggx(a, u1, u2) : sample_beckmann(a, u1, u2);
      m = to_basis(m, N);
      s.m = m;
      s.D = ggx ? D_ggx(m, N, a) : D_beckmann(m, N, a);
      s.pdf_m = s.D * m_abs(dot(m, N));
      const R wiDotM = dot(wi, m);
      if (mat.type == MAT_ROUGHCONDUCTOR) {
        const V3<R> F = fresnel_conductor3(v3<R>(mat.eta[0], mat.eta[1], mat.eta[2]),
                                           v3<R>(mat.k[0], mat.k[1], mat.k[2]), wiDotN);
        s.F = F.x;
        s.dir = reflect(d, m);
        if (wiDotN * dot(s.dir, N) <= (R)0) { s.status = SCATTER_KILLED; return s; }
        s.G = ggx ? G_ggx(wi, s.dir, m, N, a) : G_beckmann(wi, s.dir, m, a);
        const R weight = (s.G * m_abs(wiDotM)) / (m_abs(wiDotN) * m_abs(dot(m, N)));
        s.weight = mul(F, weight);
        s.offset_dir = m;
        return s;
      }
      R wiDotT = 0;
      const R F = fresnel_dielectric(wiDotM, (R)mat.ior, wiDotT);
      s.F = F;
      R weight;
      if (mat.type == MAT_ROUGHREFLECTIVE) {
        s.dir = reflect(d, m);
        if (wiDotN * dot(s.dir, N) <= (R)0) { s.status = SCATTER_KILLED; return s; }
        s.G = ggx ? G_ggx(wi, s.dir, m, N, a) : G_beckmann(wi, s.dir, m, a);
        weight = (F * s.G * m_abs(wiDotM)) / (m_abs(wiDotN) * m_abs(dot(m, N)));
      } else {
        if (F == (R)1 || next() < F) {
          s.dir = reflect(d, m);
          if (wiDotN * dot(s.dir, N) <= (R)0) { s.status = SCATTER_KILLED; return s; }
        } else {
          const R eta = wiDotM < (R)0 ? (R)mat.ior : (R)1 / (R)mat.ior;
          s.medium = wiDotM > (R)0 ? mat.medium : -1;
          s.dir = sub(mul(m, wiDotM * eta - (wiDotM > (R)0 ? (R)1.0f : (R)-1.0f) * wiDotT), mul(wi, eta));
          if (wiDotN * dot(s.dir, N) >= (R)0) { s.status = SCATTER_KILLED; return s; }
          s.offset_sign = -1;
          s.status = SCATTER_TRANSMIT;
        }
        s.G = ggx ? G_ggx(wi, s.dir, m, N, a) : G_beckmann(wi, s.dir, m, a);
        weight = (s.G * m_abs(wiDotM)) / (m_abs(wiDotN) * m_abs(dot(m, N)));
      }
      s.weight = mul(albedo, weight);
      return s;
    }
    case MAT_CONDUCTOR: {  // :307-318
      const R cosI = -dot(d, N);
      if (cosI <= (R)0) { s.status = SCATTER_KILLED; return s; }
      s.dir = reflect(d, norm_o);
      s.weight = fresnel_conductor3(v3<R>(mat.eta[0], mat.eta[1], mat.eta[2]), v3<R>(mat.k[0], mat.k[1], mat.k[2]), cosI);
      s.F = s.weight.x;
      return s;
    }
    case MAT_PLASTIC: {  // :350-374
      const R cosI = -dot(d, N);
      R cosT = 0;
      const R F = fresnel_dielectric(cosI, (R)mat.ior, cosT);
      s.F = F;
      const R u1 = next();
      if (F == (R)1 || u1 < F) {
        s.dir = reflect(d, N);
        s.weight = v3<R>((R)0.99f, (R)0.99f, (R)0.99f);
      } else {
        const R u2 = next();
        const R uu = (R)((double)(u1 - F) / (1.0 - (double)F));
        s.dir = to_basis(sample_hemisphere_cosine(uu, u2), norm_o);
        const R cosO = dot(s.dir, N);
        const R Fo = fresnel_dielectric(cosO, (R)mat.ior, cosT);
        const V3<R> diff = divs(albedo, (R)1 - (R)mat.diffuse_fresnel);
        const R inv_eta = (R)1 / (R)mat.ior;
        s.weight = mul(diff, inv_eta * inv_eta * ((R)1 - Fo));
      }
      return s;
    }
    default:
      s.status = SCATTER_KILLED;
      return s;
  }
}

// ---- EXTENSION: next-event estimation with multiple importance sampling ----
//
// The library's opt-in estimator (the reference finds light only by BSDF sampling,
// src/renderer.cu:183-386). At a lambert, rough conductor or rough dielectric reflection
// vertex in air that is not the path's last, one light is sampled from a separate
// Philox stream (counter slot 0x40000000 | bounce): the environment (probability 1/2
// when emissive mesh triangles exist too; a row by its weight, then a texel of the row,
// uniform within the texel; density luminance x cos(elevation), floored at 1e-4 of the
// largest texel weight) or an emissive mesh triangle (chosen by world-space area x the
// emitter's luminance, uniform point). Choices go through Walker alias tables built by
// Vose's method. The sample's contribution, weighted by the power heuristic against the
// BSDF's own density, is added when the shadow ray finds nothing closer than the light.
// A BSDF-sampled continuation that then escapes or reaches an emissive mesh triangle is
// weighted by the power heuristic against the light density; after delta or
// transmissive interactions, in media and for emissive spheres the weight is 1.

struct AliasSlot { float prob; int alias; };

// Vose's alias method (Vose, IEEE TSE 1991): slots whose scaled weight is below 1 take
// the rest of their probability from a slot above 1, both lists worked from the back.
// Slots left at the end keep themselves with probability 1. Zero total weight: every
// slot keeps itself.
static inline void alias_build(const double* w, size_t n, AliasSlot* out) {
  double total = 0.0;
  for (size_t i = 0; i < n; ++i) total += std::max(w[i], 0.0);
  for (size_t i = 0; i < n; ++i) out[i] = AliasSlot{1.0f, (int)i};
  if (!(total > 0.0) || n == 0) return;
  std::vector<double> q(n);
  std::vector<size_t> lo, hi;
  for (size_t i = 0; i < n; ++i) {
    q[i] = std::max(w[i], 0.0) * (double)n / total;
    if (q[i] < 1.0) lo.push_back(i); else hi.push_back(i);
  }
  while (!lo.empty() && !hi.empty()) {
    const size_t a = lo.back(), b = hi.back();
    lo.pop_back();
    out[a] = AliasSlot{(float)q[a], (int)b};
    q[b] = (q[b] + q[a]) - 1.0;
    if (q[b] < 1.0) { hi.pop_back(); lo.push_back(b); }
  }
  for (size_t i : hi) out[i] = AliasSlot{1.0f, (int)i};
  for (size_t i : lo) out[i] = AliasSlot{1.0f, (int)i};
}

// Slot chosen by u in [0, 1); frac = the rest of u's randomness, uniform given the slot.
static inline int alias_pick(const AliasSlot* t, int n, float u, float& frac) {
  const float x = u * (float)n;
  const int i = std::min(std::max((int)x, 0), n - 1);
  const float f = fminf(fmaxf(x - (float)i, 0.0f), 0.99999994f);
  if (f < t[i].prob) {
    frac = fminf(f / t[i].prob, 0.99999994f);
    return i;
  }
  frac = fminf((f - t[i].prob) / (1.0f - t[i].prob), 0.99999994f);
  return t[i].alias;
}

struct LightTables {
  int env_w = 0, env_h = 0;
  std::vector<float> env_func;            // texel weights, row-major
  std::vector<AliasSlot> env_rows, env_cols;
  float env_integral = 0.0f;              // mean texel weight
  float env_prob = 0.0f;                  // probability of choosing the environment
  struct Tri { float v0[3], area, e1[3], psel, e2[3]; int inst; };
  std::vector<Tri> tris;                  // world-space emissive triangles
  std::vector<AliasSlot> tri_alias;
  std::vector<int> inst_base;             // per instance: its first light triangle, -1 if none
};

static inline float luminance_f(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }

static inline LightTables build_light_tables(const Scene& sc) {
  LightTables L;
  // environment
  const int id = sc.env_tex;
  if (id >= 0 && id < (int)sc.textures.size()) {
    const Texture& t = sc.textures[id];
    int w = 0, h = 0;
    std::vector<float> lum;
    if (t.type == TEX_BITMAP && t.scale[0] == 1.0f && t.scale[1] == 1.0f && t.width > 0 && t.height > 0) {
      w = t.width;
      h = t.height;
      const float s = t.hdr ? 1.0f : 1.0f / 255.0f;
      lum.resize((size_t)w * h);
      for (size_t i = 0; i < lum.size(); ++i) lum[i] = s * luminance_f(t.texels[4 * i], t.texels[4 * i + 1], t.texels[4 * i + 2]);
    } else if (t.type == TEX_CONSTANT) {
      w = h = 1;
      lum.assign(1, luminance_f(t.c[0], t.c[1], t.c[2]));
    }
    if (w > 0) {
      std::vector<double> f((size_t)w * h);
      double fmax = 0.0;
      for (int y = 0; y < h; ++y) {
        const double c = cos((0.5 - (y + 0.5) / h) * kPi);
        for (int x = 0; x < w; ++x) {
          f[(size_t)y * w + x] = std::max(0.0, (double)lum[(size_t)y * w + x]) * c;
          fmax = std::max(fmax, f[(size_t)y * w + x]);
        }
      }
      if (fmax > 0.0) {
        for (int y = 0; y < h; ++y) {
          const double c = cos((0.5 - (y + 0.5) / h) * kPi);
          for (int x = 0; x < w; ++x) f[(size_t)y * w + x] = std::max(f[(size_t)y * w + x], 1e-4 * fmax * c);
        }
        L.env_w = w;
        L.env_h = h;
        L.env_cols.resize((size_t)w * h);
        L.env_rows.resize(h);
        L.env_func.resize((size_t)w * h);
        std::vector<double> rows(h);
        double total = 0.0;
        for (int y = 0; y < h; ++y) {
          alias_build(&f[(size_t)y * w], w, &L.env_cols[(size_t)y * w]);
          double r = 0.0;
          for (int x = 0; x < w; ++x) r += f[(size_t)y * w + x];
          rows[y] = r;
          total += r;
        }
        alias_build(rows.data(), h, L.env_rows.data());
        for (size_t i = 0; i < f.size(); ++i) L.env_func[i] = (float)f[i];
        L.env_integral = (float)(total / ((double)w * h));
      }
    }
  }
  // emissive mesh triangles, world space
  L.inst_base.assign(sc.instances.size(), -1);
  std::vector<double> weight;
  for (int i = 0; i < (int)sc.instances.size(); ++i) {
    const Instance& in = sc.instances[i];
    const Material& mat = sc.materials[in.material];
    if (mat.type != MAT_EMISSIVE) continue;
    float col[3] = {1.0f, 1.0f, 1.0f};
    if (mat.albedo_tex >= 0 && mat.albedo_tex < (int)sc.textures.size() && sc.textures[mat.albedo_tex].type == TEX_CONSTANT)
      for (int c = 0; c < 3; ++c) col[c] = sc.textures[mat.albedo_tex].c[c];
    const double lw = std::max(1e-6, (double)luminance_f(col[0], col[1], col[2]));
    const Mesh& m = sc.meshes[in.mesh];
    L.inst_base[i] = (int)L.tris.size();
    for (int t = 0; t < m.num_tris; ++t) {
      double v[3][3];
      for (int k = 0; k < 3; ++k) {
        const float* p = m.positions + 3 * (size_t)m.tris[3 * t + k];
        for (int r = 0; r < 3; ++r)
          v[k][r] = (double)in.mat.m[r][0] * p[0] + (double)in.mat.m[r][1] * p[1] + (double)in.mat.m[r][2] * p[2] +
                    in.mat.m[r][3];
      }
      const double e1[3] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]};
      const double e2[3] = {v[2][0] - v[0][0], v[2][1] - v[0][1], v[2][2] - v[0][2]};
      const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                   cz = e1[0] * e2[1] - e1[1] * e2[0];
      const double area = 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
      LightTables::Tri T;
      for (int r = 0; r < 3; ++r) { T.v0[r] = (float)v[0][r]; T.e1[r] = (float)e1[r]; T.e2[r] = (float)e2[r]; }
      T.area = (float)area;
      T.psel = 0.0f;
      T.inst = i;
      L.tris.push_back(T);
      weight.push_back(area * lw);
    }
  }
  double total = 0.0;
  for (double x : weight) total += x;
  if (!(total > 0.0)) {
    L.tris.clear();
    for (int& b : L.inst_base) b = -1;
  } else {
    L.tri_alias.resize(weight.size());
    alias_build(weight.data(), weight.size(), L.tri_alias.data());
    for (size_t k = 0; k < weight.size(); ++k) L.tris[k].psel = (float)(weight[k] / total);
  }
  const bool env = L.env_w > 0, tri = !L.tri_alias.empty();
  L.env_prob = env && tri ? 0.5f : (env ? 1.0f : 0.0f);
  return L;
}

static const float kTwoPiSqF = 19.7392088021787172f;   // 2 pi^2

template <class R> static inline R power_heuristic(R a, R b) {
  const R a2 = a * a, b2 = b * b;
  return a2 + b2 > (R)0 ? a2 / (a2 + b2) : (R)0;
}

// Environment radiance of direction d, the miss lookup of src/renderer.cu:378-386.
template <class R> static inline V3<R> env_radiance(const Scene& sc, V3<R> d) {
  if (sc.env_tex < 0) return v3<R>(0, 0, 0);
  const R u = (R)((double)(m_atan2(d.z, d.x) * (R)0.5f) * kInvPi + 0.5);
  const R v = (R)(0.5 - (double)m_asin(d.y) * kInvPi);
  return tex_eval<R>(sc, sc.env_tex, u, v);
}

// Solid-angle density (with the choice probability) of the environment toward d.
template <class R> static inline R env_light_pdf(const LightTables& L, V3<R> d) {
  if (L.env_w == 0) return (R)0;
  const R u = m_atan2(d.z, d.x) * ((R)0.5f * (R)(float)kInvPi) + (R)0.5f;
  const R v = (R)0.5f - m_asin(m_min(m_max(d.y, (R)-1.0f), (R)1.0f)) * (R)(float)kInvPi;
  const int x = std::min(std::max((int)(u * (R)L.env_w), 0), L.env_w - 1);
  const int y = std::min(std::max((int)(v * (R)L.env_h), 0), L.env_h - 1);
  const R ce = m_sqrt(m_max((R)1.0f - d.y * d.y, (R)0.0f));
  if (ce < (R)1e-6f) return (R)0;
  const R puv = (R)L.env_func[(size_t)y * L.env_w + x] / (R)L.env_integral;
  return (R)L.env_prob * puv / ((R)kTwoPiSqF * ce);
}

// Solid-angle density of reaching light triangle l at distance t with cosine cos_l.
template <class R> static inline R tri_light_pdf(const LightTables& L, int l, R t, R cos_l) {
  if (l < 0 || m_abs(cos_l) < (R)1e-7f) return (R)0;
  const R area = (R)L.tris[l].area, psel = (R)L.tris[l].psel;
  if (!(area > (R)0)) return (R)0;
  return ((R)1.0f - (R)L.env_prob) * psel * t * t / (area * m_abs(cos_l));
}

template <class R> struct LightSampleO { V3<R> dir; R dist; V3<R> Le; R pdf; bool ok; };

// u0 picks the kind and the triangle, (u1, u2) the point.
template <class R>
static inline LightSampleO<R> sample_light(const Scene& sc, const LightTables& L, V3<R> p, R u0, R u1, R u2) {
  LightSampleO<R> s;
  s.ok = false;
  s.pdf = 0;
  s.dist = (R)FLT_MAX;
  s.Le = v3<R>(0, 0, 0);
  s.dir = v3<R>(0, 0, 1);
  if (u0 < (R)L.env_prob) {
    float ry, rx;
    const int y = alias_pick(L.env_rows.data(), L.env_h, (float)u2, ry);
    const int x = alias_pick(L.env_cols.data() + (size_t)y * L.env_w, L.env_w, (float)u1, rx);
    const R u = ((R)x + (R)rx) / (R)L.env_w, v = ((R)y + (R)ry) / (R)L.env_h;
    const R phi = (u - (R)0.5f) * (R)6.28318530717958648f;
    const R elev = ((R)0.5f - v) * (R)3.14159265358979324f;
    const R ce = m_cos(elev);
    if (ce < (R)1e-6f) return s;
    s.dir = v3<R>(ce * m_cos(phi), m_sin(elev), ce * m_sin(phi));
    const R puv = (R)L.env_func[(size_t)y * L.env_w + x] / (R)L.env_integral;
    s.pdf = (R)L.env_prob * puv / ((R)kTwoPiSqF * ce);
    s.Le = env_radiance<R>(sc, s.dir);
    s.ok = s.pdf > (R)0;
    return s;
  }
  if (L.tris.empty()) return s;
  const R ut = (u0 - (R)L.env_prob) / ((R)1.0f - (R)L.env_prob);
  float rest;
  const int l = alias_pick(L.tri_alias.data(), (int)L.tris.size(), fminf(fmaxf((float)ut, 0.0f), 0.99999994f), rest);
  const LightTables::Tri& T = L.tris[l];
  const V3<R> a = v3<R>(T.v0[0], T.v0[1], T.v0[2]), e1 = v3<R>(T.e1[0], T.e1[1], T.e1[2]),
              e2 = v3<R>(T.e2[0], T.e2[1], T.e2[2]);
  const R su = m_sqrt(u1);
  const R b1 = (R)1.0f - su, b2 = u2 * su;
  const V3<R> q = add(a, add(mul(e1, b1), mul(e2, b2)));
  const V3<R> to = sub(q, p);
  const R d2 = dot(to, to);
  if (!(d2 > (R)0)) return s;
  const R dist = m_sqrt(d2);
  s.dir = mul(to, (R)1.0f / dist);
  s.dist = dist;
  const V3<R> n = cross(e1, e2);
  const R nl = m_sqrt(dot(n, n));
  if (!(nl > (R)0)) return s;
  const R cos_l = dot(n, s.dir) / nl;
  s.pdf = tri_light_pdf<R>(L, l, dist, cos_l);
  // emitted radiance: the emitter's albedo at the point, texcoords as in shading
  const Instance& in = sc.instances[T.inst];
  const Mesh& m = sc.meshes[in.mesh];
  const int prim = l - L.inst_base[T.inst];
  R uv0 = b1, uv1 = b2;
  if (m.texcoords) {
    const int* tri = m.tris + 3 * prim;
    const float* tc = m.texcoords;
    const R w0 = (R)1.0f - b1 - b2;
    uv0 = (tc[2 * tri[0]] * w0 + tc[2 * tri[1]] * b1) + tc[2 * tri[2]] * b2;
    uv1 = (tc[2 * tri[0] + 1] * w0 + tc[2 * tri[1] + 1] * b1) + tc[2 * tri[2] + 1] * b2;
  }
  s.Le = tex_eval<R>(sc, sc.materials[in.material].albedo_tex, uv0, uv1);
  s.ok = s.pdf > (R)0;
  return s;
}

// f x cos toward wl and the density the material's own sampling gives wl (lambert,
// rough conductor, rough dielectric reflection); false for other lobes or no value.
template <class R>
static inline bool bsdf_eval_cos(const Material& mat, V3<R> d, V3<R> N, V3<R> albedo, R roughness, V3<R> wl, V3<R>& fcos,
                                 R& pdf) {
  const V3<R> norm_o = mul(N, dot(N, d) > (R)0 ? (R)-1.0f : (R)1.0f);
  if (mat.type == MAT_DIFFUSE) {
    const R c = dot(wl, norm_o);
    if (c <= (R)0) return false;
    fcos = mul(albedo, c * (R)(float)kInvPi);
    pdf = c * (R)(float)kInvPi;
    return true;
  }
  if (mat.type != MAT_ROUGHCONDUCTOR && mat.type != MAT_ROUGHREFLECTIVE) return false;
  const V3<R> wi = mul(d, (R)-1.0f);
  const R wiDotN = dot(wi, N), woDotN = dot(wl, N);
  if (mat.type == MAT_ROUGHCONDUCTOR && wiDotN <= (R)0) return false;
  if (wiDotN * woDotN <= (R)0) return false;
  V3<R> m = add(wi, wl);
  const R ml = m_sqrt(dot(m, m));
  if (!(ml > (R)0)) return false;
  m = mul(m, (R)1.0f / ml);
  if (dot(m, N) < (R)0) m = mul(m, (R)-1.0f);
  const bool ggx = mat.distribution == DIST_GGX;
  const R a = ggx ? roughness : roughness * ((R)1.2f - (R)0.2f * m_sqrt(m_abs(wiDotN)));
  const R D = ggx ? D_ggx(m, N, a) : D_beckmann(m, N, a);
  const R G = ggx ? G_ggx(wi, wl, m, N, a) : G_beckmann(wi, wl, m, a);
  const R woDotM = m_abs(dot(wl, m));
  if (!(woDotM > (R)0) || !(D > (R)0)) return false;
  pdf = D * m_abs(dot(m, N)) / ((R)4.0f * woDotM);
  const R base = D * G / ((R)4.0f * m_abs(wiDotN));
  if (mat.type == MAT_ROUGHCONDUCTOR) {
    fcos = v3<R>(fresnel_conductor((R)mat.eta[0], (R)mat.k[0], wiDotN) * base,
                 fresnel_conductor((R)mat.eta[1], (R)mat.k[1], wiDotN) * base,
                 fresnel_conductor((R)mat.eta[2], (R)mat.k[2], wiDotN) * base);
  } else {
    R cosT = 0;
    const R F = fresnel_dielectric(dot(wi, m), (R)mat.ior, cosT);
    fcos = mul(albedo, F * base);
  }
  return std::isfinite((double)pdf) && pdf > (R)0;
}

// Density of the material's own sampling for the direction it just sampled.
template <class R> static inline R bsdf_sampled_pdf(const Material& mat, const ScatterOut<R>& s, V3<R> d, V3<R> N) {
  if (s.status != SCATTER_REFLECT) return (R)0;
  if (mat.type == MAT_DIFFUSE) {
    const V3<R> norm_o = mul(N, dot(N, d) > (R)0 ? (R)-1.0f : (R)1.0f);
    return m_max(dot(normalize(s.dir), norm_o), (R)0) * (R)(float)kInvPi;
  }
  if (mat.type == MAT_ROUGHCONDUCTOR || mat.type == MAT_ROUGHREFLECTIVE) {
    const R woDotM = m_abs(dot(normalize(s.dir), s.m));
    return woDotM > (R)0 ? s.pdf_m / ((R)4.0f * woDotM) : (R)0;
  }
  return (R)0;
}

struct PathResult { double L[3]; int rays; };

template <class R>
static inline PathResult trace_path(const Scene& sc, const RenderParams& p, const CameraSetup& cs, int pixel,
                                    uint32_t sample, const LightTables* lights = nullptr) {
  PathResult res{{0, 0, 0}, 0};
  philox::Stream rng;
  rng.init((uint32_t)pixel, sample, 0, p.seed, p.job);
  Ray<R> ray = camera_ray<R>(sc, cs, p.width, pixel, rng);
  V3<R> color = v3<R>(1, 1, 1);
  int medium = -1;
  const R bias = (R)p.ray_bias;
  const bool nee = p.nee != 0 && lights != nullptr;
  // radiance in the path's arithmetic: the reference estimator sets it once; with
  // next-event estimation the light samples and the final emission add up in order
  V3<R> Lsum = v3<R>(0, 0, 0);
  auto finish = [&]() { res.L[0] = (double)Lsum.x; res.L[1] = (double)Lsum.y; res.L[2] = (double)Lsum.z; return res; };
  auto accumulate = [&](V3<R> c) { Lsum = nee ? add(Lsum, c) : c; };
  R pdf_prev = 0;   // density of the BSDF sample that led to this vertex (0: weight 1)
  for (int j = 0; j < p.max_depth; ++j) {
    res.rays++;
    rng.init((uint32_t)pixel, sample, (uint32_t)(j + 1), p.seed, p.job);
    Hit<R> h = closest_hit<R>(sc, ray, p.isect);
    if (medium >= 0 && sc.mediums[medium].active) {
      const Medium& md = sc.mediums[medium];
      const R u = (R)rng.next();
      const R scatter_dist = -m_log(u) / (R)md.scattering;
      if (scatter_dist < h.t) {
        const R u1 = (R)rng.next(), u2 = (R)rng.next();
        const V3<R> dir = to_basis(sample_hg((R)md.g, u1, u2, p.exact_hg != 0), ray.d);
        ray = Ray<R>{add(ray.o, mul(ray.d, scatter_dist)), normalize(dir)};
        color = mulv(color, v3<R>(m_exp((R)-1.0f * scatter_dist * (R)md.absorption[0]),
                                  m_exp((R)-1.0f * scatter_dist * (R)md.absorption[1]),
                                  m_exp((R)-1.0f * scatter_dist * (R)md.absorption[2])));
        pdf_prev = 0;
        if ((double)length2(color) < 1e-4) return finish();
        continue;
      }
      color = mulv(color, v3<R>(m_exp((R)-1.0f * h.t * (R)md.absorption[0]),
                                m_exp((R)-1.0f * h.t * (R)md.absorption[1]),
                                m_exp((R)-1.0f * h.t * (R)md.absorption[2])));
    }
    if (!h.hit) {
      // miss: environment lookup, src/renderer.cu:378-386
      V3<R> Le = mulv(color, env_radiance<R>(sc, ray.d));
      if (nee && pdf_prev > (R)0) Le = mul(Le, power_heuristic<R>(pdf_prev, env_light_pdf<R>(*lights, ray.d)));
      accumulate(Le);
      return finish();
    }
    const Material& mat = sc.materials[h.material];
    const V3<R> albedo = tex_eval<R>(sc, mat.albedo_tex, h.uv[0], h.uv[1]);
    const R roughness = tex_eval<R>(sc, mat.roughness_tex, h.uv[0], h.uv[1]).x;
    if (mat.type == MAT_EMISSIVE) {  // :192-198
      V3<R> Le = mulv(color, albedo);
      if (nee && pdf_prev > (R)0 && h.inst >= 0 && !lights->tris.empty()) {
        const int base = lights->inst_base[h.inst];
        if (base >= 0) {
          const int l = base + h.prim;
          const LightTables::Tri& T = lights->tris[l];
          const V3<R> ln = cross(v3<R>(T.e1[0], T.e1[1], T.e1[2]), v3<R>(T.e2[0], T.e2[1], T.e2[2]));
          const R lnl = m_sqrt(dot(ln, ln));
          const R cos_l = lnl > (R)0 ? dot(ln, ray.d) / lnl : (R)0;
          Le = mul(Le, power_heuristic<R>(pdf_prev, tri_light_pdf<R>(*lights, l, h.t, cos_l)));
        }
      }
      accumulate(Le);
      return finish();
    }
    if (j + 1 >= p.max_depth) return finish();   // every closest-hit query is used
    if (nee && (medium < 0 || !sc.mediums[medium].active) &&
        (mat.type == MAT_DIFFUSE || mat.type == MAT_ROUGHCONDUCTOR || mat.type == MAT_ROUGHREFLECTIVE)) {
      philox::Stream lr;
      lr.init((uint32_t)pixel, sample, 0x40000000u | (uint32_t)(j + 1), p.seed, p.job);
      const R u0 = (R)lr.next(), u1 = (R)lr.next(), u2 = (R)lr.next();
      const V3<R> ph = add(ray.o, mul(ray.d, h.t));
      const LightSampleO<R> ls = sample_light<R>(sc, *lights, ph, u0, u1, u2);
      V3<R> fcos;
      R pdf_b = 0;
      if (ls.ok && bsdf_eval_cos<R>(mat, ray.d, h.normal, albedo, roughness, ls.dir, fcos, pdf_b)) {
        const V3<R> Cn = mul(mulv(mulv(color, fcos), ls.Le), power_heuristic<R>(ls.pdf, pdf_b) / ls.pdf);
        if (std::isfinite((double)(Cn.x + Cn.y + Cn.z)) && (Cn.x > (R)0 || Cn.y > (R)0 || Cn.z > (R)0)) {
          const V3<R> norm_o = mul(h.normal, dot(h.normal, ray.d) > (R)0 ? (R)-1.0f : (R)1.0f);
          const V3<R> org = add(ph, mul(norm_o, bias));
          const R tmax = ls.dist == (R)FLT_MAX ? (R)FLT_MAX : ls.dist * ((R)1.0f - (R)1e-4f) - bias;
          if (tmax > (R)0) {
            res.rays++;   // the shadow ray is a closest-hit query too
            const Hit<R> o = closest_hit<R>(sc, Ray<R>{org, ls.dir}, p.isect);
            if (!(o.hit && o.t < tmax)) accumulate(Cn);
          }
        }
      }
    }
    ScatterOut<R> s = scatter<R>(mat, ray.d, h.normal, albedo, roughness, [&]() { return (R)rng.next(); });
    if (s.status == SCATTER_KILLED) return finish();
    if (s.medium != MEDIUM_UNCHANGED) medium = s.medium;
    color = mulv(color, s.weight);
    pdf_prev = nee ? bsdf_sampled_pdf<R>(mat, s, ray.d, h.normal) : (R)0;
    const V3<R> new_origin = add(add(ray.o, mul(ray.d, h.t)), mul(s.offset_dir, s.offset_sign * bias));
    const V3<R> new_dir = s.dir;
    ray = Ray<R>{new_origin, normalize(new_dir)};
  }
  return finish();
}

// ---- tonemap: src/tonemapper.cu:32-76 and src/renderer.cu:426-441 ----
enum { TONE_LINEAR = 0, TONE_REINHARD = 1, TONE_FILMIC = 2, TONE_UNCHARTED = 3 };
static inline V3<float> uncharted2(V3<float> x) {
  const float A = 0.15f, B = 0.50f, C = 0.10f, D = 0.20f, E = 0.02f, F = 0.30f;
  const V3<float> num = adds(mulv(x, adds(mul(x, A), C * B)), D * E);
  const V3<float> den = adds(mulv(x, adds(mul(x, A), B)), D * F);
  return adds(divv(num, den), -E / F);
}
static inline V3<float> pow3(V3<float> v, float p) { return v3<float>(powf(v.x, p), powf(v.y, p), powf(v.z, p)); }
static inline V3<float> tonemap_op(int op, V3<float> in) {
  const float gamma = 1.0f / 2.2f;
  switch (op) {
    case TONE_REINHARD: return pow3(divv(in, adds(in, 1.0f)), gamma);
    case TONE_FILMIC: {
      const V3<float> x = v3<float>(fmaxf(in.x + -0.004f, 0.0f), fmaxf(in.y + -0.004f, 0.0f), fmaxf(in.z + -0.004f, 0.0f));
      return divv(mulv(x, adds(mul(x, 6.2f), 0.5f)), adds(mulv(x, adds(mul(x, 6.2f), 1.7f)), 0.06f));
    }
    case TONE_UNCHARTED: {
      const float W = 11.2f;
      const V3<float> curr = uncharted2(mul(in, 2.0f));
      const V3<float> white = divv(v3<float>(1, 1, 1), uncharted2(v3<float>(W, W, W)));
      return pow3(mulv(curr, white), gamma);
    }
    default: return pow3(in, gamma);
  }
}
static inline void tonemap_pixel(int op, const float sum[3], float samples, unsigned char out[3]) {
  V3<float> avg = mul(v3<float>(sum[0], sum[1], sum[2]), 1 / samples);
  avg = tonemap_op(op, avg);
  avg = v3<float>(fmaxf(fminf(avg.x, 1), 0), fmaxf(fminf(avg.y, 1), 0), fmaxf(fminf(avg.z, 1), 0));
  out[0] = (unsigned char)(int)(255 * avg.x);
  out[1] = (unsigned char)(int)(255 * avg.y);
  out[2] = (unsigned char)(int)(255 * avg.z);
}

}  // namespace oracle
