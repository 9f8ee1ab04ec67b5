// Host-side 4x4 matrix and transform construction for scene ingest.
//
// The arithmetic follows the reference's matrix code operation by operation
// (src/math/matrix4.cu, src/math/transform.cu, src/math/mathutils.h:9-12), so that
// matrices parsed from JSON match the reference's float results bit for bit; the host
// library is compiled with -ffp-contract=off for that reason.
#pragma once

namespace illume {

struct Vec3f { float x, y, z; };
struct Mat4 { float m[4][4]; };
struct Transform { Mat4 mat, inv, trans, trans_inv; };

Mat4 mat4_identity();
Mat4 mat4_from_axis_angle(Vec3f axis, float angle);   // src/math/matrix4.cu:16-34
Mat4 mat4_from_scale(Vec3f s);                        // :36-43
void mat4_set_translate(Mat4* m, Vec3f t);            // :45-53
Mat4 mat4_lookat(Vec3f pos, Vec3f fwd, Vec3f up);     // :55-67
Mat4 mat4_mul(const Mat4& a, const Mat4& b);          // :82-96
Mat4 mat4_transpose(const Mat4& m);                   // :98-109
Mat4 mat4_inverse(const Mat4& m);                     // :115-201 (adjugate / determinant)
float deg_to_rad(float deg);                          // src/math/mathutils.h:9-12

Transform transform_create(Vec3f translation, Vec3f scale, const Mat4& rotation);  // src/math/transform.cu:6-16
Transform transform_from_matrix(const Mat4& m);                                    // :18-26
// transform_from_json's construction (src/math/transform.cu:28-44)
Transform transform_trs(Vec3f translation, Vec3f scale, Vec3f rotation_deg);
Transform transform_lookat(Vec3f translation, Vec3f lookat);

Vec3f v3f(float x, float y, float z);
Vec3f vsub(Vec3f a, Vec3f b);
Vec3f vcross(Vec3f a, Vec3f b);
Vec3f vnormalized(Vec3f v);      // src/math/vector3.cu:53-57
void vnormalize(Vec3f* v);       // src/math/vector3.cu:43-51
float vlength2(Vec3f v);

}  // namespace illume
