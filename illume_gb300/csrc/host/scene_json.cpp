// Scene ingest from the reference's JSON format.
//
// Follows HostScene::HostScene (src/scene/scene.cpp:11-99) and the parsers it calls:
// texture_from_json (src/texture.cu:7-71), camera_from_json (src/camera.cu:20-30),
// transform_from_json (src/math/transform.cu:28-44), medium_from_json
// (src/medium.cu:5-14), material_from_json (src/material.cu:7-177), mesh_from_json
// (src/primitives/mesh.cu:430-443), sphere_from_json (src/primitives/sphere.cu:25-32),
// mesh_instance_from_json (src/primitives/mesh_instance.cu:35-49), and the
// render_settings read of Renderer::Renderer (src/renderer.cu:39-59).
//
// Where the reference leaves a value uninitialised (a missing "ior", a missing instance
// "transform", a missing "ray_bias") this loader uses a defined default and records a
// warning: ior 1.5, the identity transform, ray_bias 0. Numbers written as integers are
// accepted wherever the reference reads a float. Extensions: "eta"/"k" arrays on
// conductors, "distribution": "ggx" | "beckmann" on rough materials, and bitmap
// textures in the .pfm / .hdr / .ppm / .pgm / .png / .bmp / .tga formats.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <fstream>
#include <sstream>
#include <unordered_map>

#include "image_io.h"
#include "json.h"
#include "mesh_io.h"
#include "runtime.h"
#include "xform.h"

namespace illume {

namespace {

struct Loader {
  SceneHost* s;
  std::string base_dir;
  std::string err;

  void warn(const std::string& w) { s->warnings.push_back(w); }

  bool get_float(const JValue& o, const char* key, float* out) {
    const JValue* v = o.find(key);
    if (!v || !v->is_number()) return false;
    *out = v->as_float();
    return true;
  }
  // Vector3 from a number (replicated) or a 3-element array (src/jsonutils.cpp:33-37).
  bool vec3(const JValue& v, float out[3]) {
    if (v.is_number()) { out[0] = out[1] = out[2] = v.as_float(); return true; }
    if (v.is_array() && v.arr.size() >= 3 && v.arr[0].is_number() && v.arr[1].is_number() && v.arr[2].is_number()) {
      for (int i = 0; i < 3; ++i) out[i] = v.arr[i].as_float();
      return true;
    }
    return false;
  }
  bool get_vec3(const JValue& o, const char* key, float out[3]) {
    const JValue* v = o.find(key);
    return v && vec3(*v, out);
  }
  bool get_vec2(const JValue& o, const char* key, float out[2]) {
    const JValue* v = o.find(key);
    if (!v || !v->is_array() || v->arr.size() < 2 || !v->arr[0].is_number() || !v->arr[1].is_number()) return false;
    out[0] = v->arr[0].as_float();
    out[1] = v->arr[1].as_float();
    return true;
  }
  bool get_bool(const JValue& o, const char* key, bool def) {
    const JValue* v = o.find(key);
    if (!v) return def;
    if (v->type == JValue::Bool) return v->b;
    if (v->is_number()) return v->num != 0.0;
    return def;
  }
  std::string get_str(const JValue& o, const char* key, const std::string& def = "") {
    const JValue* v = o.find(key);
    return (v && v->is_string()) ? v->str : def;
  }

  int add_texture(int type, const float c[3], const float off[3], const float scale[2]) {
    const int id = (int)s->tex_type.size();
    s->tex_type.push_back(type);
    s->tex_color.insert(s->tex_color.end(), c, c + 3);
    s->tex_off.insert(s->tex_off.end(), off, off + 3);
    s->tex_scale.insert(s->tex_scale.end(), scale, scale + 2);
    s->tex_width.push_back(0);
    s->tex_height.push_back(0);
    s->tex_hdr.push_back(1);
    s->tex_texel_offset.push_back(0);
    return id;
  }
  int constant(float r, float g, float b) {
    const float c[3] = {r, g, b}, z[3] = {0, 0, 0}, one[2] = {1, 1};
    return add_texture(TEX_CONSTANT, c, z, one);
  }

  // src/texture.cu:7-71
  int texture(const JValue& j) {
    float c[3] = {0, 0, 0};
    if (j.is_number() || j.is_array()) {
      if (!vec3(j, c)) warn("texture: malformed constant");
      return constant(c[0], c[1], c[2]);
    }
    if (!j.is_object()) { warn("texture: not an object"); return constant(0, 0, 0); }
    const std::string type = get_str(j, "type");
    if (type == "constant") {
      get_vec3(j, "color", c);
      return constant(c[0], c[1], c[2]);
    }
    if (type == "checkerboard") {
      float on[3] = {0, 0, 0}, off[3] = {0, 0, 0}, sc[2] = {1, 1};
      get_vec3(j, "on_color", on);
      get_vec3(j, "off_color", off);
      get_vec2(j, "scale", sc);
      return add_texture(TEX_CHECKER, on, off, sc);
    }
    if (type == "bitmap") {
      std::string path = get_str(j, "file");
      float sc[2] = {1, 1};
      get_vec2(j, "scale", sc);
      if (path.empty()) { warn("texture: bitmap file not specified"); return constant(0, 0, 0); }
      Image img;
      std::string ierr;
      if (!load_image(resolve(path), &img, &ierr)) {
        warn("texture: " + ierr + " (bitmap replaced by black)");
        return constant(0, 0, 0);
      }
      const float z[3] = {0, 0, 0};
      const int id = add_texture(TEX_BITMAP, z, z, sc);
      s->tex_width[id] = img.width;
      s->tex_height[id] = img.height;
      s->tex_hdr[id] = img.hdr ? 1 : 0;
      s->tex_texel_offset[id] = (int64_t)s->texels.size();
      s->texels.insert(s->texels.end(), img.rgba.begin(), img.rgba.end());
      return id;
    }
    warn("texture: invalid texture type " + type);
    return constant(0, 0, 0);
  }

  std::string resolve(const std::string& p) const {
    if (p.empty() || p[0] == '/' || base_dir.empty()) return p;
    return base_dir + "/" + p;
  }

  // src/math/transform.cu:28-44
  Transform transform(const JValue& j) {
    float t[3] = {0, 0, 0}, sc[3] = {1, 1, 1}, r[3] = {0, 0, 0};
    get_vec3(j, "translation", t);
    get_vec3(j, "scale", sc);
    get_vec3(j, "rotation", r);
    if (j.find("lookat")) {
      float la[3] = {0, 0, 0};
      get_vec3(j, "lookat", la);
      return transform_lookat(v3f(t[0], t[1], t[2]), v3f(la[0], la[1], la[2]));
    }
    return transform_trs(v3f(t[0], t[1], t[2]), v3f(sc[0], sc[1], sc[2]), v3f(r[0], r[1], r[2]));
  }

  // src/medium.cu:5-14
  int medium(const JValue& j) {
    float a[3] = {0, 0, 0}, sc = 0, g = 0;
    if (!get_vec3(j, "absorption", a)) warn("medium: absorption missing");
    if (!get_float(j, "scattering", &sc)) warn("medium: scattering missing");
    get_float(j, "g", &g);
    const float ab[3] = {1 - a[0], 1 - a[1], 1 - a[2]};
    const float len2 = (ab[0] * ab[0]) + (ab[1] * ab[1]) + (ab[2] * ab[2]);
    const int id = (int)s->med_active.size();
    s->med_absorption.insert(s->med_absorption.end(), ab, ab + 3);
    s->med_scattering.push_back(sc);
    s->med_g.push_back(g);
    s->med_active.push_back(((double)len2 > 1e-5 || sc > 0) ? 1 : 0);
    return id;
  }

  static bool conductor_table(const std::string& name, float eta[3], float k[3]) {
    // measured complex index at 700, 510, 440 nm: the table of src/conductor.h:16-25
    struct E { const char* n; float eta[3], k[3]; };
    static const E tab[] = {
        {"Ag", {0.16761f, 0.14032f, 0.13529f}, {4.2868f, 2.8794f, 2.2916f}},
        {"Al", {1.66130f, 0.82373f, 0.58461f}, {8.0444f, 5.9742f, 5.1875f}},
        {"Au", {0.14311f, 0.37495f, 1.44247f}, {3.9831f, 2.3857f, 1.6032f}},
        {"Cu", {0.21249f, 0.97909f, 1.3343f}, {4.1005f, 2.3691f, 2.2965f}},
        {"Pb", {1.78000f, 1.74000f, 1.4400f}, {3.5700f, 3.3100f, 3.1800f}},
    };
    for (const E& e : tab)
      if (name == e.n) { memcpy(eta, e.eta, 12); memcpy(k, e.k, 12); return true; }
    return false;
  }

  int push_material(int type, int albedo, int rough, float ior, float dfres, const float eta[3], const float k[3],
                    int med, int dist) {
    const int id = (int)s->mat_type.size();
    s->mat_type.push_back(type);
    s->mat_albedo_tex.push_back(albedo);
    s->mat_roughness_tex.push_back(rough);
    s->mat_ior.push_back(ior);
    s->mat_diffuse_fresnel.push_back(dfres);
    s->mat_eta.insert(s->mat_eta.end(), eta, eta + 3);
    s->mat_k.insert(s->mat_k.end(), k, k + 3);
    s->mat_medium.push_back(med);
    s->mat_distribution.push_back(dist);
    return id;
  }

  // src/material.cu:7-177
  int material(const JValue& j, int med) {
    const std::string type = get_str(j, "type");
    const JValue* a = j.find("albedo");
    const JValue* r = j.find("roughness");
    const int albedo = a ? texture(*a) : constant(0, 0, 0);
    const int rough = r ? texture(*r) : constant(1e-4f, 1e-4f, 1e-4f);
    const float z[3] = {0, 0, 0};
    float ior = 0.0f;
    auto need_ior = [&]() {
      if (!get_float(j, "ior", &ior)) { warn("material: ior missing, using 1.5"); ior = 1.5f; }
    };
    std::string dname = get_str(j, "distribution", "beckmann");
    const int dist = dname == "ggx" ? DIST_GGX : DIST_BECKMANN;
    const int air = -1;
    if (type == "emissive") return push_material(MAT_EMISSIVE, albedo, constant(1e-4f, 1e-4f, 1e-4f), 0, 0, z, z, air, 0);
    if (type == "lambert") return push_material(MAT_LAMBERT, albedo, constant(1e-4f, 1e-4f, 1e-4f), 0, 0, z, z, air, 0);
    if (type == "reflective") return push_material(MAT_REFLECTIVE, albedo, constant(1e-4f, 1e-4f, 1e-4f), 0, 0, z, z, air, 0);
    if (type == "refractive") {
      need_ior();
      return push_material(MAT_REFRACTIVE, albedo, constant(1e-4f, 1e-4f, 1e-4f), ior, 0, z, z, med, 0);
    }
    if (type == "roughreflective") {
      need_ior();
      return push_material(MAT_ROUGHREFLECTIVE, albedo, rough, ior, 0, z, z, air, dist);
    }
    if (type == "roughrefractive") {
      need_ior();
      return push_material(MAT_ROUGHREFRACTIVE, albedo, rough, ior, 0, z, z, med, dist);
    }
    if (type == "conductor" || type == "roughconductor") {
      float eta[3], k[3];
      const std::string name = get_str(j, "material");
      if (!conductor_table(name, eta, k)) {
        if (!(j.find("eta") && j.find("k"))) warn("material: invalid conductor material " + name + ", defaulting to copper");
        conductor_table("Cu", eta, k);
      }
      get_vec3(j, "eta", eta);
      get_vec3(j, "k", k);
      const int black = constant(0, 0, 0);
      if (type == "conductor")
        return push_material(MAT_CONDUCTOR, black, constant(1e-4f, 1e-4f, 1e-4f), 0, 0, eta, k, air, 0);
      return push_material(MAT_ROUGHCONDUCTOR, black, rough, 0, 0, eta, k, air, dist);
    }
    if (type == "plastic") {
      need_ior();
      return push_material(MAT_PLASTIC, albedo, constant(1e-4f, 1e-4f, 1e-4f), ior, plastic_diffuse_fresnel(ior), z, z,
                           air, 0);
    }
    warn("material: invalid material type " + type);
    return push_material(MAT_LAMBERT, constant(0, 0, 0), constant(1e-4f, 1e-4f, 1e-4f), 0, 0, z, z, air, 0);
  }

  // a value-initialised Material (type 0 = emissive with zero radiance), which is what
  // an unknown material name yields in the reference (src/scene/scene.cpp:88, 95)
  int black_material() {
    const float z[3] = {0, 0, 0};
    return push_material(MAT_EMISSIVE, constant(0, 0, 0), constant(0, 0, 0), 0, 0, z, z, -1, 0);
  }

  int mesh(const JValue& j) {
    const std::string file = get_str(j, "file");
    MeshOptions opt;
    opt.z_up = get_bool(j, "z_up", false);
    opt.flip_normals = get_bool(j, "flip_normals", false);
    opt.has_texcoords = get_bool(j, "has_texcoords", false);
    opt.face_normals = get_bool(j, "face_normals", true);
    const JValue* lp = j.find("bvh_items_per_node");
    opt.leaf_size = lp && lp->is_number() ? lp->as_int() : 4;
    MeshData md;
    if (!load_obj_mesh(resolve(file), opt, &md, &err)) return -1;
    const int id = (int)s->mesh_num_tris.size();
    const int V = (int)(md.positions.size() / 3), T = (int)(md.tris.size() / 3);
    s->mesh_vertex_offset.push_back((int)(s->positions.size() / 3));
    s->mesh_tri_offset.push_back((int)(s->tris.size() / 3));
    s->mesh_num_vertices.push_back(V);
    s->mesh_num_tris.push_back(T);
    s->mesh_has_normals.push_back(opt.face_normals ? 0 : 1);
    s->mesh_has_texcoords.push_back(opt.has_texcoords ? 1 : 0);
    s->mesh_bvh_leaf_size.push_back(opt.leaf_size);
    s->positions.insert(s->positions.end(), md.positions.begin(), md.positions.end());
    if (opt.face_normals) s->normals.insert(s->normals.end(), (size_t)V * 3, 0.0f);
    else s->normals.insert(s->normals.end(), md.normals.begin(), md.normals.end());
    if (opt.has_texcoords) s->texcoords.insert(s->texcoords.end(), md.texcoords.begin(), md.texcoords.end());
    else s->texcoords.insert(s->texcoords.end(), (size_t)V * 2, 0.0f);
    s->tris.insert(s->tris.end(), md.tris.begin(), md.tris.end());
    return id;
  }

  static void put34(std::vector<float>& v, const Mat4& m) {
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 4; ++c) v.push_back(m.m[r][c]);
  }

  int run(const JValue& doc) {
    if (!doc.is_object()) { err = "scene root is not a JSON object"; return ILLUME_ERR_PARSE; }
    std::unordered_map<std::string, int> medium_map, mat_map, mesh_map;
    if (const JValue* env = doc.find("environment_map")) s->env_tex = texture(*env);
    if (const JValue* cam = doc.find("camera")) {
      get_float(*cam, "fov", &s->camera_fov);
      get_float(*cam, "depth_of_field", &s->camera_dof);
      get_float(*cam, "aperture_radius", &s->camera_aperture);
      const JValue* tr = cam->find("transform");
      if (!tr) { err = "camera: transform missing"; return ILLUME_ERR_PARSE; }
      const Transform t = transform(*tr);
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) s->camera_transform[4 * r + c] = t.mat.m[r][c];
    }
    if (const JValue* meds = doc.find("mediums")) {
      if (meds->is_array())
        for (const JValue& m : meds->arr) medium_map.emplace(get_str(m, "name"), medium(m));
    }
    if (const JValue* mats = doc.find("materials")) {
      if (mats->is_array())
        for (const JValue& m : mats->arr) {
          auto it = medium_map.find(get_str(m, "medium"));
          const int med = it == medium_map.end() ? -1 : it->second;
          mat_map.emplace(get_str(m, "name"), material(m, med));
        }
    }
    if (const JValue* meshes = doc.find("meshes")) {
      if (meshes->is_array())
        for (const JValue& m : meshes->arr) {
          const int id = mesh(m);
          if (id < 0) return ILLUME_ERR_IO;
          mesh_map.emplace(get_str(m, "name"), id);
        }
    }
    int black = -1;
    auto mat_of = [&](const std::string& name) {
      auto it = mat_map.find(name);
      if (it != mat_map.end()) return it->second;
      warn("primitive: unknown material " + name + " (black)");
      if (black < 0) black = black_material();
      return black;
    };
    if (const JValue* prims = doc.find("primitives")) {
      if (prims->is_array())
        for (const JValue& p : prims->arr) {
          const std::string type = get_str(p, "type");
          const std::string mname = get_str(p, "material");
          if (type == "sphere") {
            float c[3] = {0, 0, 0}, r = 0;
            get_float(p, "radius", &r);
            get_vec3(p, "center", c);
            s->sphere_center_radius.insert(s->sphere_center_radius.end(), {c[0], c[1], c[2], r});
            s->sphere_material.push_back(mat_of(mname));
          } else if (type == "mesh_instance") {
            const std::string mesh_name = get_str(p, "mesh");
            auto it = mesh_map.find(mesh_name);
            int mesh_index = 0;
            if (it == mesh_map.end()) {
              if (s->mesh_num_tris.empty()) { err = "mesh_instance refers to unknown mesh " + mesh_name; return ILLUME_ERR_PARSE; }
              warn("mesh_instance: unknown mesh " + mesh_name + ", using mesh 0");
            } else {
              mesh_index = it->second;
            }
            Transform t;
            if (const JValue* tr = p.find("transform")) t = transform(*tr);
            else { warn("mesh_instance: transform missing, using identity"); t = transform_from_matrix(mat4_identity()); }
            s->inst_mesh.push_back(mesh_index);
            s->inst_material.push_back(mat_of(mname));
            put34(s->inst_mat, t.mat);
            put34(s->inst_inv, t.inv);
            put34(s->inst_trans_inv, t.trans_inv);
          }
        }
    }
    if (const JValue* rs = doc.find("render_settings")) {
      if (!get_float(*rs, "ray_bias", &s->ray_bias)) { warn("render_settings: ray_bias missing, using 0"); s->ray_bias = 0.0f; }
      const std::string tm = get_str(*rs, "tonemapper", "linear");
      if (tm == "linear") s->tonemapper = 0;
      else if (tm == "Reinhard") s->tonemapper = 1;
      else if (tm == "Filmic") s->tonemapper = 2;
      else if (tm == "Uncharted") s->tonemapper = 3;
      else { warn("tonemapper: invalid operator " + tm); s->tonemapper = 0; }
      const JValue* res = rs->find("resolution");
      if (res && res->is_array() && res->arr.size() >= 2) {
        s->width = res->arr[0].as_int();
        s->height = res->arr[1].as_int();
      } else {
        s->width = s->height = 512;
      }
    }
    return ILLUME_OK;
  }
};

}  // namespace

int load_scene_json(const std::string& text, const std::string& base_dir, SceneHost* out, std::string* err) {
  JValue doc;
  std::string perr;
  if (!json_parse(text, &doc, &perr)) { *err = "JSON parse error: " + perr; return ILLUME_ERR_PARSE; }
  *out = SceneHost();
  Loader L{out, base_dir, ""};
  const int st = L.run(doc);
  if (st != ILLUME_OK) { *err = L.err; return st; }
  if (out->tex_type.empty()) L.constant(0, 0, 0);
  return out->validate(err);
}

}  // namespace illume
