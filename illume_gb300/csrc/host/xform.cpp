#include "xform.h"

#include <math.h>

namespace illume {

static const double kPi = 3.14159265358979323846;

Vec3f v3f(float x, float y, float z) { return Vec3f{x, y, z}; }
Vec3f vsub(Vec3f a, Vec3f b) { return v3f(a.x - b.x, a.y - b.y, a.z - b.z); }
Vec3f vcross(Vec3f a, Vec3f b) { return v3f(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
float vlength2(Vec3f v) { return (v.x * v.x) + (v.y * v.y) + (v.z * v.z); }
Vec3f vnormalized(Vec3f v) {
  const float inv = 1.0f / sqrtf(vlength2(v));
  return v3f(v.x * inv, v.y * inv, v.z * inv);
}
void vnormalize(Vec3f* v) {
  const float inv = 1.0f / sqrtf(vlength2(*v));
  v->x *= inv;
  v->y *= inv;
  v->z *= inv;
}

float deg_to_rad(float deg) { return (float)((double)deg * kPi / 180.0); }

Mat4 mat4_identity() {
  Mat4 r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) r.m[i][j] = i == j ? 1.0f : 0.0f;
  return r;
}

Mat4 mat4_from_axis_angle(Vec3f axis, float angle) {
  vnormalize(&axis);
  const float s = sinf(angle / 2), w = cosf(angle / 2);
  const Vec3f v = v3f(axis.x * s, axis.y * s, axis.z * s);
  Mat4 m = mat4_identity();
  m.m[0][0] = 1 - 2 * (v.y * v.y + v.z * v.z);
  m.m[1][0] = 2 * (v.x * v.y + w * v.z);
  m.m[2][0] = 2 * (v.x * v.z - w * v.y);
  m.m[0][1] = 2 * (v.x * v.y - w * v.z);
  m.m[1][1] = 1 - 2 * (v.x * v.x + v.z * v.z);
  m.m[2][1] = 2 * (v.y * v.z + w * v.x);
  m.m[0][2] = 2 * (v.x * v.z + w * v.y);
  m.m[1][2] = 2 * (v.y * v.z - w * v.x);
  m.m[2][2] = 1 - 2 * (v.x * v.x + v.y * v.y);
  return m;
}

Mat4 mat4_from_scale(Vec3f s) {
  Mat4 m = mat4_identity();
  m.m[0][0] = s.x;
  m.m[1][1] = s.y;
  m.m[2][2] = s.z;
  return m;
}

void mat4_set_translate(Mat4* m, Vec3f t) {
  m->m[0][3] = t.x;
  m->m[1][3] = t.y;
  m->m[2][3] = t.z;
}

Mat4 mat4_lookat(Vec3f pos, Vec3f fwd, Vec3f up) {
  const Vec3f f = vnormalized(fwd);
  const Vec3f r = vnormalized(vcross(up, f));
  const Vec3f u = vnormalized(vcross(f, r));
  Mat4 m;
  m.m[0][0] = r.x; m.m[0][1] = u.x; m.m[0][2] = f.x; m.m[0][3] = pos.x;
  m.m[1][0] = r.y; m.m[1][1] = u.y; m.m[1][2] = f.y; m.m[1][3] = pos.y;
  m.m[2][0] = r.z; m.m[2][1] = u.z; m.m[2][2] = f.z; m.m[2][3] = pos.z;
  m.m[3][0] = 0; m.m[3][1] = 0; m.m[3][2] = 0; m.m[3][3] = 1;
  return m;
}

Mat4 mat4_mul(const Mat4& a, const Mat4& b) {
  Mat4 r;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j)
      r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j] + a.m[i][3] * b.m[3][j];
  return r;
}

Mat4 mat4_transpose(const Mat4& m) {
  Mat4 t;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) t.m[j][i] = m.m[i][j];
  return t;
}

// 3x3 minor of m without row `row` and column `col`, expanded by the rule of Sarrus
// with the six products in the order the reference sums them.
static float minor3(const Mat4& m, int row, int col) {
  int rs[3], cs[3];
  for (int k = 0, r = 0; k < 4; ++k) if (k != row) rs[r++] = k;
  for (int k = 0, c = 0; k < 4; ++k) if (k != col) cs[c++] = k;
  float d[3][3];
  for (int y = 0; y < 3; ++y)
    for (int x = 0; x < 3; ++x) d[y][x] = m.m[rs[y]][cs[x]];
  return (d[0][0] * d[1][1] * d[2][2]) + (d[0][1] * d[1][2] * d[2][0]) + (d[0][2] * d[1][0] * d[2][1]) -
         (d[0][2] * d[1][1] * d[2][0]) - (d[0][1] * d[1][0] * d[2][2]) - (d[0][0] * d[1][2] * d[2][1]);
}

// Leibniz expansion of the determinant, the 24 products summed in the reference's order
// (src/math/matrix4.cu:174-201). Its tenth product reads m[2][0] where m[1][0] belongs;
// that product carries the factor m[3][1], which is zero for the affine matrices scenes
// use, so the value is the determinant.
static float det4(const Mat4& M) {
  const float(*m)[4] = M.m;
  return (m[0][0] * m[1][1] * m[2][2] * m[3][3]) + (m[0][0] * m[1][2] * m[2][3] * m[3][1]) +
         (m[0][0] * m[1][3] * m[2][1] * m[3][2]) + (m[0][1] * m[1][0] * m[2][3] * m[3][2]) +
         (m[0][1] * m[1][2] * m[2][0] * m[3][3]) + (m[0][1] * m[1][3] * m[2][2] * m[3][0]) +
         (m[0][2] * m[1][0] * m[2][1] * m[3][3]) + (m[0][2] * m[1][1] * m[2][3] * m[3][0]) +
         (m[0][2] * m[1][3] * m[2][0] * m[3][1]) + (m[0][3] * m[2][0] * m[2][2] * m[3][1]) +
         (m[0][3] * m[1][1] * m[2][0] * m[3][2]) + (m[0][3] * m[1][2] * m[2][1] * m[3][0]) -
         (m[0][0] * m[1][1] * m[2][3] * m[3][2]) - (m[0][0] * m[1][2] * m[2][1] * m[3][3]) -
         (m[0][0] * m[1][3] * m[2][2] * m[3][1]) - (m[0][1] * m[1][0] * m[2][2] * m[3][3]) -
         (m[0][1] * m[1][2] * m[2][3] * m[3][0]) - (m[0][1] * m[1][3] * m[2][0] * m[3][2]) -
         (m[0][2] * m[1][0] * m[2][3] * m[3][1]) - (m[0][2] * m[1][1] * m[2][0] * m[3][3]) -
         (m[0][2] * m[1][3] * m[2][1] * m[3][0]) - (m[0][3] * m[1][0] * m[2][1] * m[3][2]) -
         (m[0][3] * m[1][1] * m[2][2] * m[3][0]) - (m[0][3] * m[1][2] * m[2][0] * m[3][1]);
}

Mat4 mat4_inverse(const Mat4& m) {
  Mat4 adj;
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      const float c = minor3(m, j, i);
      adj.m[i][j] = ((i + j) % 2 == 0) ? c : -1 * c;
    }
  const float inv_det = 1 / det4(m);
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) adj.m[i][j] *= inv_det;
  return adj;
}

Transform transform_from_matrix(const Mat4& m) {
  Transform t;
  t.mat = m;
  t.inv = mat4_inverse(t.mat);
  t.trans = mat4_transpose(t.mat);
  t.trans_inv = mat4_transpose(t.inv);
  return t;
}

Transform transform_create(Vec3f translation, Vec3f scale, const Mat4& rotation) {
  Mat4 tr = mat4_identity();
  mat4_set_translate(&tr, translation);
  return transform_from_matrix(mat4_mul(mat4_mul(tr, rotation), mat4_from_scale(scale)));
}

Transform transform_trs(Vec3f translation, Vec3f scale, Vec3f rot) {
  const Mat4 x = mat4_from_axis_angle(v3f(1, 0, 0), deg_to_rad(rot.x));
  const Mat4 y = mat4_from_axis_angle(v3f(0, 1, 0), deg_to_rad(rot.y));
  const Mat4 z = mat4_from_axis_angle(v3f(0, 0, 1), deg_to_rad(rot.z));
  return transform_create(translation, scale, mat4_mul(mat4_mul(x, y), z));
}

Transform transform_lookat(Vec3f translation, Vec3f lookat) {
  return transform_from_matrix(mat4_lookat(translation, vsub(lookat, translation), v3f(0, 1, 0)));
}

}  // namespace illume
