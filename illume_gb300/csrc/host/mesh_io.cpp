#include "mesh_io.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "xform.h"

namespace illume {

namespace {

struct FaceCorner { int pos, tex, norm; };

// A field of a line: [p, p + n) of the file buffer.
struct Field { const char* p; size_t n; };

// strtof / strtol on a field alone (as on a NUL-terminated copy of it), so that a number
// never runs on into the next field. A field that std::from_chars reads whole to a finite
// value in range takes that value (both round correctly, so it is strtof's); any other
// field (signs, spaces, hex, inf, nan, out of range, trailing text) goes to strtof itself.
float field_float(const Field& f) {
  float x;
  const std::from_chars_result r = std::from_chars(f.p, f.p + f.n, x);
  if (r.ec == std::errc() && r.ptr == f.p + f.n && std::isfinite(x)) return x;
  char buf[64];
  if (f.n < sizeof(buf)) {
    memcpy(buf, f.p, f.n);
    buf[f.n] = 0;
    return strtof(buf, nullptr);
  }
  return strtof(std::string(f.p, f.n).c_str(), nullptr);
}
int field_int(const char* p, size_t n) {
  int x;
  const std::from_chars_result r = std::from_chars(p, p + n, x);
  if (r.ec == std::errc() && r.ptr == p + n) return x;
  char buf[32];
  if (n < sizeof(buf)) {
    memcpy(buf, p, n);
    buf[n] = 0;
    return (int)strtol(buf, nullptr, 10);
  }
  return (int)strtol(std::string(p, n).c_str(), nullptr, 10);
}

// One corner field of an "f" line: p, p/t, p//n or p/t/n (1-based indices). The fields
// between slashes are taken with empty ones dropped, as strtok would.
FaceCorner parse_corner(const Field& tok) {
  FaceCorner c{-1, -1, -1};
  const char* part[3];
  size_t plen[3];
  int nparts = 0, slashes = 0;
  bool double_slash = false;
  size_t start = 0;
  for (size_t i = 0; i <= tok.n; ++i) {
    if (i == tok.n || tok.p[i] == '/') {
      if (i > start && nparts < 3) { part[nparts] = tok.p + start; plen[nparts] = i - start; ++nparts; }
      if (i < tok.n) {
        ++slashes;
        if (i + 1 < tok.n && tok.p[i + 1] == '/') double_slash = true;
      }
      start = i + 1;
    }
  }
  auto num = [&](int k) { return k < nparts ? field_int(part[k], plen[k]) - 1 : -1; };
  if (slashes == 0) {
    c.pos = num(0);
  } else if (slashes == 1) {
    c.pos = num(0); c.tex = num(1);
  } else if (slashes == 2) {
    if (double_slash) { c.pos = num(0); c.norm = num(1); }
    else { c.pos = num(0); c.tex = num(1); c.norm = num(2); }
  }
  return c;
}

// Canonical id of each of `count` values of N floats: the first index holding an equal
// value (every component equal as a number, +0 and -0 alike), through an open-addressing
// table keyed by the components.
template <int N>
std::vector<int> canonical_ids(const float* vals, size_t count) {
  std::vector<int> id(count);
  size_t cap = 16;
  while (cap < 2 * count) cap <<= 1;
  std::vector<int> table(cap, -1);
  for (size_t i = 0; i < count; ++i) {
    const float* x = vals + N * i;
    uint64_t h = 0x9e3779b97f4a7c15ULL;
    for (int k = 0; k < N; ++k) {
      float c = x[k];
      if (c == 0.0f) c = 0.0f;   // -0 hashes as +0, as it compares equal
      uint32_t u;
      memcpy(&u, &c, 4);
      h = (h ^ u) * 0xff51afd7ed558ccdULL;
      h ^= h >> 33;
    }
    size_t slot = (size_t)h & (cap - 1);
    int found = -1;
    while (table[slot] >= 0) {
      const float* y = vals + N * (size_t)table[slot];
      bool same = true;
      for (int k = 0; k < N; ++k) same = same && x[k] == y[k];
      if (same) { found = table[slot]; break; }
      slot = (slot + 1) & (cap - 1);
    }
    if (found < 0) { table[slot] = (int)i; found = (int)i; }
    id[i] = found;
  }
  return id;
}

}  // namespace

bool load_obj_mesh(const std::string& path, const MeshOptions& opt, MeshData* out, std::string* err) {
  FILE* fp = fopen(path.c_str(), "rb");
  if (!fp) { *err = "cannot read OBJ file " + path; return false; }
  std::vector<char> text;
  {
    char chunk[1 << 16];
    size_t got;
    while ((got = fread(chunk, 1, sizeof(chunk), fp)) > 0) text.insert(text.end(), chunk, chunk + got);
    fclose(fp);
  }
  std::vector<Vec3f> v, vn;
  std::vector<float> vt;
  std::vector<FaceCorner> corners;
  const char* at = text.data();
  const char* const end = text.data() + text.size();
  // lines end at '\n'; one '\r' before it is dropped; fields are split on ' ' only
  // (tabs stay inside fields), empty fields dropped
  constexpr int kKeep = 8;
  Field tok[kKeep];
  while (at < end) {
    const char* eol = static_cast<const char*>(memchr(at, '\n', (size_t)(end - at)));
    if (!eol) eol = end;
    const char* line_end = eol;
    if (line_end > at && line_end[-1] == '\r') --line_end;
    size_t ntok = 0;
    for (const char* q = at; q < line_end;) {
      while (q < line_end && *q == ' ') ++q;
      if (q >= line_end) break;
      const char* b = q;
      while (q < line_end && *q != ' ') ++q;
      if (ntok < (size_t)kKeep) tok[ntok] = Field{b, (size_t)(q - b)};
      ++ntok;
    }
    at = eol < end ? eol + 1 : end;
    if (ntok == 0) continue;
    auto is = [&](const char* word) { return tok[0].n == strlen(word) && memcmp(tok[0].p, word, tok[0].n) == 0; };
    auto fl = [&](size_t k) { return k < ntok && k < (size_t)kKeep ? field_float(tok[k]) : 0.0f; };
    if (is("v")) {
      v.push_back(opt.z_up ? v3f(fl(1), fl(3), fl(2)) : v3f(fl(1), fl(2), fl(3)));
    } else if (is("vt")) {
      vt.push_back(fl(1));
      vt.push_back(fl(2));
    } else if (is("vn")) {
      vn.push_back(v3f(fl(1), fl(2), fl(3)));
    } else if (is("f")) {
      if (ntok < 4) { *err = "OBJ face with fewer than 3 vertices in " + path; return false; }
      for (int k = 1; k <= 3; ++k) corners.push_back(parse_corner(tok[k]));
    }
  }
  // vertex dedup on (position, normal, texcoord) values, first use order
  // (mesh.cu:264-340): equal values get one canonical id per attribute, so two corners
  // are the same vertex exactly when their (position, normal, texcoord) ids are; a new
  // vertex takes its first corner's own values
  out->positions.clear();
  out->normals.clear();
  out->texcoords.clear();
  out->tris.clear();
  out->tris.reserve(corners.size());
  out->leaf_size = opt.leaf_size;
  static_assert(sizeof(Vec3f) == 3 * sizeof(float), "Vec3f packing");
  const std::vector<int> cpos = canonical_ids<3>(v.empty() ? nullptr : &v[0].x, v.size());
  std::vector<Vec3f> nn;
  std::vector<int> cnorm, ctex;
  if (!opt.face_normals) {
    nn = vn;
    for (Vec3f& n : nn) vnormalize(&n);
    cnorm = canonical_ids<3>(nn.empty() ? nullptr : &nn[0].x, nn.size());
  }
  if (opt.has_texcoords) ctex = canonical_ids<2>(vt.data(), vt.size() / 2);
  const bool by_position = opt.face_normals && !opt.has_texcoords;
  std::vector<int> first_of_pos(by_position ? v.size() : 0, -1);
  struct Triple { int p, n, t; };
  size_t cap = 16;
  if (!by_position)
    while (cap < 2 * std::max(v.size(), corners.size() / 4)) cap <<= 1;
  std::vector<int> table(by_position ? 0 : cap, -1);
  std::vector<Triple> triples;
  int next_id = 0;
  for (const FaceCorner& c : corners) {
    if (c.pos < 0 || c.pos >= (int)v.size()) { *err = "OBJ position index out of range in " + path; return false; }
    Triple k{cpos[c.pos], -1, -1};
    if (!opt.face_normals) {
      if (c.norm < 0 || c.norm >= (int)vn.size()) { *err = "OBJ normal index out of range in " + path; return false; }
      k.n = cnorm[c.norm];
    }
    if (opt.has_texcoords) {
      if (c.tex < 0 || 2 * c.tex + 1 >= (int)vt.size()) { *err = "OBJ texcoord index out of range in " + path; return false; }
      k.t = ctex[c.tex];
    }
    int id = -1;
    if (by_position) {
      id = first_of_pos[k.p];
      if (id < 0) first_of_pos[k.p] = id = next_id++;
      else { out->tris.push_back(id); continue; }
    } else {
      if (2 * (triples.size() + 1) > cap) {   // grow: rehash the triples
        cap <<= 1;
        table.assign(cap, -1);
        for (size_t q = 0; q < triples.size(); ++q) {
          const Triple& x = triples[q];
          size_t slot = ((uint64_t)(uint32_t)x.p * 0x9e3779b97f4a7c15ULL ^ (uint64_t)(uint32_t)x.n * 0xc2b2ae3d27d4eb4fULL ^
                         (uint64_t)(uint32_t)x.t * 0x165667b19e3779f9ULL) >> 17 & (cap - 1);
          while (table[slot] >= 0) slot = (slot + 1) & (cap - 1);
          table[slot] = (int)q;
        }
      }
      size_t slot = ((uint64_t)(uint32_t)k.p * 0x9e3779b97f4a7c15ULL ^ (uint64_t)(uint32_t)k.n * 0xc2b2ae3d27d4eb4fULL ^
                     (uint64_t)(uint32_t)k.t * 0x165667b19e3779f9ULL) >> 17 & (cap - 1);
      while (table[slot] >= 0) {
        const Triple& x = triples[table[slot]];
        if (x.p == k.p && x.n == k.n && x.t == k.t) { id = table[slot]; break; }
        slot = (slot + 1) & (cap - 1);
      }
      if (id >= 0) { out->tris.push_back(id); continue; }
      id = next_id++;
      table[slot] = id;
      triples.push_back(k);
    }
    // a new vertex: this corner's own values
    const Vec3f& p = v[c.pos];
    out->positions.push_back(p.x);
    out->positions.push_back(p.y);
    out->positions.push_back(p.z);
    if (!opt.face_normals) {
      const Vec3f& n = nn[c.norm];
      out->normals.push_back(n.x);
      out->normals.push_back(n.y);
      out->normals.push_back(n.z);
    }
    if (opt.has_texcoords) {
      out->texcoords.push_back(vt[2 * c.tex]);
      out->texcoords.push_back(vt[2 * c.tex + 1]);
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
