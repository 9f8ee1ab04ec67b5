#include "lights.h"

#include "runtime.h"

#include <math.h>
#include <string.h>

#include <algorithm>

namespace illume {

namespace {

float luminance(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }

// Colour of texture `id` when it is constant, else white (used only to weight choices).
void texture_weight_color(const SceneHost& h, int id, float* rgb) {
  rgb[0] = rgb[1] = rgb[2] = 1.0f;
  if (id < 0 || id >= h.num_textures()) return;
  if (h.tex_type[id] == TEX_CONSTANT)
    for (int c = 0; c < 3; ++c) rgb[c] = h.tex_color[3 * id + c];
}

void build_env(const SceneHost& h, HostLights* L) {
  const int id = h.env_tex;
  if (id < 0 || id >= h.num_textures()) return;
  int w = 0, hh = 0;
  std::vector<float> lum;
  if (h.tex_type[id] == TEX_BITMAP) {
    if (h.tex_scale[2 * id] != 1.0f || h.tex_scale[2 * id + 1] != 1.0f) return;   // not sampled
    w = h.tex_width[id];
    hh = h.tex_height[id];
    if (w <= 0 || hh <= 0) return;
    const float* t = h.texels.data() + h.tex_texel_offset[id];
    const float s = h.tex_hdr[id] ? 1.0f : 1.0f / 255.0f;
    lum.resize((size_t)w * hh);
    for (size_t i = 0; i < lum.size(); ++i) lum[i] = s * luminance(t[4 * i], t[4 * i + 1], t[4 * i + 2]);
  } else if (h.tex_type[id] == TEX_CONSTANT) {
    w = hh = 1;
    lum.assign(1, luminance(h.tex_color[3 * id], h.tex_color[3 * id + 1], h.tex_color[3 * id + 2]));
  } else {
    return;
  }
  // texel weight: luminance x cos(elevation) at the row centre, floored so that every
  // direction the environment can light keeps a positive density
  double maxw = 0.0;
  std::vector<double> f((size_t)w * hh);
  for (int y = 0; y < hh; ++y) {
    const double elev = (0.5 - (y + 0.5) / hh) * M_PI;
    const double c = cos(elev);
    for (int x = 0; x < w; ++x) {
      const double v = std::max(0.0, (double)lum[(size_t)y * w + x]) * c;
      f[(size_t)y * w + x] = v;
      maxw = std::max(maxw, v);
    }
  }
  if (!(maxw > 0.0)) return;
  const double floor_w = 1e-4 * maxw;
  for (int y = 0; y < hh; ++y) {
    const double c = cos((0.5 - (y + 0.5) / hh) * M_PI);
    for (int x = 0; x < w; ++x) f[(size_t)y * w + x] = std::max(f[(size_t)y * w + x], floor_w * c);
  }
  L->env_w = w;
  L->env_h = hh;
  L->env_func.resize((size_t)w * hh);
  L->env_cols.resize((size_t)w * hh);
  L->env_rows.resize(hh);
  std::vector<double> row(hh);
  double total = 0.0;
  for (int y = 0; y < hh; ++y) {
    build_alias(&f[(size_t)y * w], w, &L->env_cols[(size_t)y * w]);
    double acc = 0.0;
    for (int x = 0; x < w; ++x) acc += f[(size_t)y * w + x];
    row[y] = acc;
    total += acc;
  }
  build_alias(row.data(), hh, L->env_rows.data());
  const double mean = total / ((double)w * hh);
  for (size_t i = 0; i < f.size(); ++i) L->env_func[i] = (float)f[i];
  L->env_integral = (float)mean;
}

void build_triangles(const SceneHost& h, HostLights* L) {
  const int ni = (int)h.inst_mesh.size();
  L->inst_light_base.assign(ni, -1);
  std::vector<double> weight;
  for (int i = 0; i < ni; ++i) {
    const int mat = h.inst_material[i];
    if (mat < 0 || mat >= h.num_materials() || h.mat_type[mat] != MAT_EMISSIVE) continue;
    const int m = h.inst_mesh[i];
    const float* M = &h.inst_mat[12 * (size_t)i];
    const float* P = h.positions.data() + 3 * (size_t)h.mesh_vertex_offset[m];
    const int* T = h.tris.data() + 3 * (size_t)h.mesh_tri_offset[m];
    float col[3];
    texture_weight_color(h, h.mat_albedo_tex[mat], col);
    const double lw = std::max(1e-6, (double)luminance(col[0], col[1], col[2]));
    L->inst_light_base[i] = (int)(L->tri.size() / 3);
    for (int t = 0; t < h.mesh_num_tris[m]; ++t) {
      double v[3][3];
      for (int k = 0; k < 3; ++k) {
        const float* p = P + 3 * (size_t)T[3 * t + k];
        for (int r = 0; r < 3; ++r) v[k][r] = (double)M[4 * r] * p[0] + (double)M[4 * r + 1] * p[1] + (double)M[4 * r + 2] * p[2] + M[4 * r + 3];
      }
      const double e1[3] = {v[1][0] - v[0][0], v[1][1] - v[0][1], v[1][2] - v[0][2]};
      const double e2[3] = {v[2][0] - v[0][0], v[2][1] - v[0][1], v[2][2] - v[0][2]};
      const double cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2], cz = e1[0] * e2[1] - e1[1] * e2[0];
      const double area = 0.5 * sqrt(cx * cx + cy * cy + cz * cz);
      float4 a, b, c;
      a.x = (float)v[0][0]; a.y = (float)v[0][1]; a.z = (float)v[0][2]; a.w = (float)area;
      b.x = (float)e1[0]; b.y = (float)e1[1]; b.z = (float)e1[2]; b.w = 0.0f;
      int inst_bits = i;
      c.x = (float)e2[0]; c.y = (float)e2[1]; c.z = (float)e2[2];
      memcpy(&c.w, &inst_bits, sizeof(float));
      L->tri.push_back(a);
      L->tri.push_back(b);
      L->tri.push_back(c);
      weight.push_back(area * lw);
    }
  }
  const size_t n = weight.size();
  double total = 0.0;
  for (double w : weight) total += w;
  if (!(total > 0.0)) {
    L->tri.clear();
    L->tri_alias.clear();
    for (int& b : L->inst_light_base) b = -1;
    return;
  }
  L->tri_alias.resize(n);
  build_alias(weight.data(), n, L->tri_alias.data());
  for (size_t k = 0; k < n; ++k) L->tri[3 * k + 1].w = (float)(weight[k] / total);
}

}  // namespace

bool build_alias(const double* weights, size_t n, AliasEntry* out) {
  double total = 0.0;
  for (size_t i = 0; i < n; ++i) total += std::max(weights[i], 0.0);
  for (size_t i = 0; i < n; ++i) out[i] = AliasEntry{1.0f, (int)i};
  if (!(total > 0.0) || n == 0) return false;
  std::vector<double> scaled(n);
  std::vector<size_t> small, large;
  for (size_t i = 0; i < n; ++i) {
    scaled[i] = std::max(weights[i], 0.0) * (double)n / total;
    (scaled[i] < 1.0 ? small : large).push_back(i);
  }
  while (!small.empty() && !large.empty()) {
    const size_t s = small.back(), l = large.back();
    small.pop_back();
    out[s] = AliasEntry{(float)scaled[s], (int)l};
    scaled[l] = (scaled[l] + scaled[s]) - 1.0;
    if (scaled[l] < 1.0) {
      large.pop_back();
      small.push_back(l);
    }
  }
  // what is left has probability 1 up to rounding: keeps itself
  for (size_t i : large) out[i] = AliasEntry{1.0f, (int)i};
  for (size_t i : small) out[i] = AliasEntry{1.0f, (int)i};
  return true;
}

void build_lights(const SceneHost& h, HostLights* out) {
  *out = HostLights{};
  build_env(h, out);
  build_triangles(h, out);
  const bool env = out->env_w > 0, tri = !out->tri_alias.empty();
  out->env_prob = env && tri ? 0.5f : (env ? 1.0f : 0.0f);
}

}  // namespace illume
