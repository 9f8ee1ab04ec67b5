// Plain data shared by the host code and the sm_103a kernels: the device-resident scene
// (SoA tables in HBM) and the wavefront queues. No torch types, no pointers into host
// memory.
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define ILLUME_HD __host__ __device__ __forceinline__
#else
#define ILLUME_HD inline
#include <vector_types.h>
#endif

namespace illume {

enum MaterialType : int {
  MAT_EMISSIVE = 0, MAT_LAMBERT = 1, MAT_REFLECTIVE = 2, MAT_REFRACTIVE = 3, MAT_ROUGHREFLECTIVE = 4,
  MAT_ROUGHREFRACTIVE = 5, MAT_CONDUCTOR = 6, MAT_ROUGHCONDUCTOR = 7, MAT_PLASTIC = 8, MAT_COUNT = 9
};
enum TextureType : int { TEX_CONSTANT = 0, TEX_CHECKER = 1, TEX_BITMAP = 2 };
enum Distribution : int { DIST_BECKMANN = 0, DIST_GGX = 1 };
enum Intersector : int { ISECT_MT = 0, ISECT_WATERTIGHT = 1 };
enum BvhKind : int { BVH_BINARY = 0, BVH_WIDE8 = 1, BVH_WIDE4 = 2 };
enum AccumMode : int { ACCUM_FP32 = 0, ACCUM_KAHAN = 1, ACCUM_FP64 = 2 };

// Event classes of one bounce, the keys of the material-sorted shading queues.
enum EventClass : int {
  EV_MISS = 0,                  // escaped: environment lookup
  EV_MEDIUM = 1,                // scattered inside a medium before reaching the surface
  EV_SURFACE = 2,               // + material type (EV_SURFACE + MAT_*)
  EV_COUNT = EV_SURFACE + MAT_COUNT
};

// Binary BVH node (64 B): the boxes of both children are stored in the parent, so one
// node fetch decides both children. child >= 0: inner node index; child <= -2: leaf
// ~(first << 3 | count) with triangles [first, first + count); child == -1: empty slot.
struct Bvh2Node {
  float4 a;   // c0.lo.x c0.lo.y c0.lo.z c0.hi.x
  float4 b;   // c0.hi.y c0.hi.z c1.lo.x c1.lo.y
  float4 c;   // c1.lo.z c1.hi.x c1.hi.y c1.hi.z
  int4 d;     // child0, child1: inner node index (>= 0), leaf ~(first << 3 | count), empty
              // slot -1; count0, count1: triangles of leaf children (0 otherwise)
};

// 8-wide BVH node with child boxes quantised to 8 bits per axis (80 B), after Ylitie,
// Karras and Laine, "Efficient incoherent ray traversal on GPUs through compressed wide
// BVHs" (HPG 2017). Child box i spans p + 2^e * q (q in 0..255) per axis, rounded
// outward when built. meta[i]: 0 = empty slot; for inner children 0x20 | (24 + slot);
// for leaves the upper 3 bits hold the triangle count in unary and the lower 5 bits the
// triangle offset from tri_base.
struct WideNode {
  float px, py, pz;
  uint8_t ex, ey, ez, imask;    // exponents (biased by 127), inner-child mask
  uint32_t child_base;          // index of the first inner child node
  uint32_t tri_base;            // index of the first triangle of this node's leaves
  uint8_t meta[8];
  uint8_t qlox[8], qloy[8], qloz[8];
  uint8_t qhix[8], qhiy[8], qhiz[8];
};
static_assert(sizeof(WideNode) == 80, "wide node must be 80 bytes");

// 4-wide BVH node (128 B, one cache line): the four child boxes as rows of x / y / z
// bounds, then the four children encoded as the binary node's (inner node index, leaf
// ~(first << 3 | count) into the binary layout's triangle order, or -1 for an empty slot
// whose box is empty).
struct Bvh4Node {
  float4 lox, loy, loz, hix, hiy, hiz;
  int4 child;
  int4 pad;
};
static_assert(sizeof(Bvh4Node) == 128, "4-wide node must be 128 bytes");

struct DevMesh {
  const Bvh4Node* bvh4;         // 4-wide BVH over the binary layout's triangles
  const Bvh2Node* bvh2;         // binary BVH
  const WideNode* wide;         // 8-wide quantised BVH
  const float4* bvh2_tris;      // 3 float4 per triangle in BVH2 leaf order; .w of the first = prim id
  const float4* wide_tris;      // 3 float4 per triangle in wide-BVH leaf order
  const int* tris;              // original triangles (3 ints each)
  const float* positions;       // 3 floats per vertex
  const float* normals;         // 3 floats per vertex or null (face normals)
  const float* texcoords;       // 2 floats per vertex or null
  int num_tris;
  int bvh2_root_leaf;           // 1 if the whole mesh is one leaf (no inner node)
  int pad[2];
};

struct DevInstance {
  float inv[12];                // world -> object rows
  float trans_inv[12];          // normal matrix rows
  float lo[3], hi[3];           // world-space bounds (padded)
  int mesh, material;
};

struct DevSphere { float cx, cy, cz, r; int material; int pad[3]; };

struct DevMaterial {
  int type, albedo_tex, roughness_tex, medium;
  int distribution; float ior, diffuse_fresnel, pad0;
  float eta[3], pad1;
  float k[3], pad2;
};

struct DevTexture {
  int type, width, height, hdr;
  float c[3], pad0;
  float off[3], pad1;
  float scale[2], pad2[2];
  const float4* texels;         // RGBA, 8-bit textures hold 0..255
  long long pad3;
};

struct DevMedium { float absorption[3]; float scattering, g; int active; int pad[2]; };

// Light sampling data of a scene (the opt-in next-event estimator; the reference
// estimator never reads it).
// Alias table entry (Walker): slot i keeps itself with probability `keep`, else `alias`.
struct AliasEntry {
  float keep;
  int alias;
};

struct LightView {
  // environment: piecewise-constant density over the map's texels, proportional to
  // luminance x cos(elevation); env_w == 0 when the environment is not sampled
  int env_w, env_h;
  const float* env_func;          // env_h x env_w texel weights
  const AliasEntry* env_rows;     // env_h entries: a row by its total weight
  const AliasEntry* env_cols;     // env_h x env_w entries: a texel of a row by its weight
  float env_integral;             // mean texel weight (density normaliser)
  float env_prob;                 // probability of sampling the environment rather than a triangle
  // emissive triangles of mesh instances, world space, chosen by area x luminance
  int num_tri;
  const float4* tri;              // 3 float4 per light: (v0, area), (e1, select prob), (e2, instance / prim bits)
  const AliasEntry* tri_alias;    // num_tri entries: a triangle by its weight
  const int* inst_light_base;     // per instance: index of its first light (-1: not emissive)
  int pad[2];
};

// Everything a kernel needs about a scene, passed by value as a kernel parameter.
struct SceneView {
  const DevMesh* meshes;
  const DevInstance* instances;
  const DevSphere* spheres;
  const DevMaterial* materials;
  const DevTexture* textures;
  const DevMedium* mediums;
  int num_meshes, num_instances, num_spheres, num_materials;
  int env_tex;
  int pad;
  const LightView* lights;      // device copy, read only by the next-event estimator
};

struct CameraView {
  float m[12];                  // camera -> world rows
  float pixel_size, left, top, dof, aperture;
  int width, height;
  int pad;
};

// Hit record written by the trace kernels.
struct HitRecord {
  float t, u, v;
  int prim;                     // triangle (mesh hits), -1 otherwise
  int geom;                     // >= 0 instance, -2 - s sphere s, -1 miss
};

}  // namespace illume
