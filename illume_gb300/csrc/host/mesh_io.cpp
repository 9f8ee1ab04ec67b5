#include "mesh_io.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <fstream>
#include <map>
#include <tuple>

#include "xform.h"

namespace illume {

namespace {

struct FaceCorner { int pos, tex, norm; };

// Split on one delimiter character, dropping empty fields (strtok semantics).
static std::vector<std::string> split(const std::string& s, char delim) {
  std::vector<std::string> out;
  std::string cur;
  for (char c : s) {
    if (c == delim) {
      if (!cur.empty()) out.push_back(cur);
      cur.clear();
    } else {
      cur += c;
    }
  }
  if (!cur.empty()) out.push_back(cur);
  return out;
}

// One corner token of an "f" line: p, p/t, p//n or p/t/n (1-based indices).
static FaceCorner parse_corner(const std::string& tok) {
  FaceCorner c{-1, -1, -1};
  const auto parts = split(tok, '/');
  int slashes = 0;
  for (char ch : tok) slashes += ch == '/';
  auto num = [&](size_t k) { return k < parts.size() ? (int)strtol(parts[k].c_str(), nullptr, 10) - 1 : -1; };
  if (slashes == 0) {
    c.pos = num(0);
  } else if (slashes == 1) {
    c.pos = num(0); c.tex = num(1);
  } else if (slashes == 2) {
    if (tok.find("//") != std::string::npos) { c.pos = num(0); c.norm = num(1); }
    else { c.pos = num(0); c.tex = num(1); c.norm = num(2); }
  }
  return c;
}

struct PackedKey {
  float p[3], n[3], uv[2];
  bool operator<(const PackedKey& o) const {
    const float* a = p;
    const float* b = o.p;
    for (int i = 0; i < 8; ++i) {
      if (a[i] < b[i]) return true;
      if (a[i] > b[i]) return false;
    }
    return false;
  }
};

}  // namespace

bool load_obj_mesh(const std::string& path, const MeshOptions& opt, MeshData* out, std::string* err) {
  std::ifstream f(path);
  if (!f) { *err = "cannot read OBJ file " + path; return false; }
  std::vector<Vec3f> v, vn;
  std::vector<float> vt;
  std::vector<FaceCorner> corners;
  std::string line;
  while (std::getline(f, line)) {
    if (!line.empty() && line.back() == '\r') line.pop_back();
    const auto tok = split(line, ' ');
    if (tok.empty()) continue;
    auto fl = [&](size_t k) { return k < tok.size() ? strtof(tok[k].c_str(), nullptr) : 0.0f; };
    if (tok[0] == "v") {
      v.push_back(opt.z_up ? v3f(fl(1), fl(3), fl(2)) : v3f(fl(1), fl(2), fl(3)));
    } else if (tok[0] == "vt") {
      vt.push_back(fl(1));
      vt.push_back(fl(2));
    } else if (tok[0] == "vn") {
      vn.push_back(v3f(fl(1), fl(2), fl(3)));
    } else if (tok[0] == "f") {
      if (tok.size() < 4) { *err = "OBJ face with fewer than 3 vertices in " + path; return false; }
      for (int k = 1; k <= 3; ++k) corners.push_back(parse_corner(tok[k]));
    }
  }
  // vertex dedup on (position, normal, texcoord), first use order (mesh.cu:264-340)
  std::map<PackedKey, int> index;
  out->positions.clear();
  out->normals.clear();
  out->texcoords.clear();
  out->tris.clear();
  out->leaf_size = opt.leaf_size;
  for (const FaceCorner& c : corners) {
    if (c.pos < 0 || c.pos >= (int)v.size()) { *err = "OBJ position index out of range in " + path; return false; }
    PackedKey key{};
    key.p[0] = v[c.pos].x; key.p[1] = v[c.pos].y; key.p[2] = v[c.pos].z;
    if (!opt.face_normals) {
      if (c.norm < 0 || c.norm >= (int)vn.size()) { *err = "OBJ normal index out of range in " + path; return false; }
      Vec3f n = vn[c.norm];
      vnormalize(&n);
      key.n[0] = n.x; key.n[1] = n.y; key.n[2] = n.z;
    }
    if (opt.has_texcoords) {
      if (c.tex < 0 || 2 * c.tex + 1 >= (int)vt.size()) { *err = "OBJ texcoord index out of range in " + path; return false; }
      key.uv[0] = vt[2 * c.tex];
      key.uv[1] = vt[2 * c.tex + 1];
    }
    auto it = index.find(key);
    int id;
    if (it == index.end()) {
      id = (int)(out->positions.size() / 3);
      index.emplace(key, id);
      out->positions.insert(out->positions.end(), key.p, key.p + 3);
      if (!opt.face_normals) out->normals.insert(out->normals.end(), key.n, key.n + 3);
      if (opt.has_texcoords) out->texcoords.insert(out->texcoords.end(), key.uv, key.uv + 2);
    } else {
      id = it->second;
    }
    out->tris.push_back(id);
  }
  // normal flip (mesh.cu:363-388)
  if (opt.flip_normals) {
    if (opt.face_normals) {
      for (size_t t = 0; t + 2 < out->tris.size(); t += 3) std::swap(out->tris[t + 1], out->tris[t + 2]);
    } else {
      for (float& x : out->normals) x = x * -1.0f;
    }
  }
  return true;
}

}  // namespace illume
