// OBJ ingest for mesh entries of the scene format (src/primitives/mesh.cu:159-443):
// triangles only, vertex dedup on (position, normal, texcoord) in first-use order,
// optional z-up swap, vertex normals normalised, normal flip.
#pragma once

#include <string>
#include <vector>

namespace illume {

struct MeshOptions {
  bool z_up = false;           // swap y and z of positions (mesh.cu:181-186)
  bool flip_normals = false;   // swap triangle winding (face normals) or negate normals
  bool has_texcoords = false;
  bool face_normals = true;    // JSON default true (mesh.cu:440)
  int leaf_size = 4;           // bvh_items_per_node, default 4 (mesh.cu:441)
};

struct MeshData {
  std::vector<float> positions;   // 3 per vertex
  std::vector<float> normals;     // 3 per vertex, empty with face normals
  std::vector<float> texcoords;   // 2 per vertex, empty without texcoords
  std::vector<int> tris;          // 3 per triangle
  int leaf_size = 4;
};

// Returns false with *err set when the file cannot be read or an index is out of range.
bool load_obj_mesh(const std::string& path, const MeshOptions& opt, MeshData* out, std::string* err);

}  // namespace illume
