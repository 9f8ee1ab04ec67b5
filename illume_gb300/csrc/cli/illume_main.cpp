// Command line front end with the reference's interface (src/main.cu:14-43):
//   illume <save> <scene.json> <spp> <maxdepth>  ->  <save>-<W>x<H>-<spp>spp-<maxdepth>md.png
// Relative mesh paths in the scene resolve against the current directory, as in the
// reference. Extra options (after the four positional arguments):
//   --seed N   --accum fp32|kahan|fp64   --bvh wide4|binary|wide   --isect mt|watertight
//   --estimator reference|nee
//   --pfm      also write the mean radiance as <name>.pfm
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "illume.h"

static int fail(const char* what) {
  fprintf(stderr, "illume: %s: %s\n", what, illume_last_error());
  return 1;
}

int main(int argc, char** argv) {
  if (argc < 5) {
    printf("illume: usage - <save> <scene> <spp> <maxdepth>\n");
    return 0;
  }
  const int spp = (int)strtol(argv[3], nullptr, 10);
  const int max_depth = (int)strtol(argv[4], nullptr, 10);
  uint32_t seed = 0;
  int accum = ILLUME_ACCUM_FP32, bvh = ILLUME_BVH_WIDE4, isect = ILLUME_ISECT_WATERTIGHT, estimator = ILLUME_ESTIMATOR_REFERENCE;
  bool pfm = false;
  for (int i = 5; i < argc; ++i) {
    const std::string a = argv[i];
    const char* v = i + 1 < argc ? argv[i + 1] : "";
    if (a == "--seed") { seed = (uint32_t)strtoul(v, nullptr, 10); ++i; }
    else if (a == "--accum") { accum = !strcmp(v, "fp64") ? ILLUME_ACCUM_FP64 : !strcmp(v, "kahan") ? ILLUME_ACCUM_KAHAN : ILLUME_ACCUM_FP32; ++i; }
    else if (a == "--bvh") { bvh = !strcmp(v, "wide") ? ILLUME_BVH_WIDE8 : !strcmp(v, "binary") ? ILLUME_BVH_BINARY : ILLUME_BVH_WIDE4; ++i; }
    else if (a == "--estimator") { estimator = !strcmp(v, "nee") ? ILLUME_ESTIMATOR_NEE : ILLUME_ESTIMATOR_REFERENCE; ++i; }
    else if (a == "--isect") { isect = !strcmp(v, "mt") ? ILLUME_ISECT_MT : ILLUME_ISECT_WATERTIGHT; ++i; }
    else if (a == "--pfm") { pfm = true; }
  }
  illume_context* ctx = nullptr;
  if (illume_context_create(0, 0, &ctx) != ILLUME_OK) return fail("context");
  illume_scene* scene = nullptr;
  if (illume_scene_load_json(ctx, argv[2], nullptr, &scene) != ILLUME_OK) return fail("scene");
  illume_render_params p;
  illume_render_params_default(scene, spp, max_depth, &p);
  p.seed = seed;
  p.accum_mode = accum;
  p.bvh_kind = bvh;
  p.intersector = isect;
  p.estimator = estimator;
  illume_renderer* r = nullptr;
  if (illume_renderer_create(ctx, scene, &p, &r) != ILLUME_OK) return fail("renderer");
  const int W = illume_renderer_get_width(r), H = illume_renderer_get_height(r);
  illume_bitmap* image = illume_bitmap_new((size_t)W, (size_t)H);
  illume_render_stats st;
  if (illume_render_to_bitmap(r, image, &st) != ILLUME_OK) return fail("render");
  printf("Rays per sec: %f rays/s\n", st.render_ms > 0 ? st.rays / (st.render_ms * 1e-3) : 0.0);
  printf("Render time: %f seconds\n", st.total_ms * 1e-3);
  char name[4096];
  snprintf(name, sizeof(name), "%s-%dx%d-%dspp-%dmd.png", argv[1], W, H, spp, max_depth);
  if (illume_bitmap_save_png(image, name) != ILLUME_OK) return fail("save");
  printf("Saved to: %s\n", name);
  if (pfm) {
    std::vector<float> mean((size_t)W * H * 3);
    illume_renderer_read(r, mean.data(), nullptr, nullptr, nullptr);
    std::string pname = std::string(name, strlen(name) - 4) + ".pfm";
    if (illume_save_pfm(mean.data(), W, H, pname.c_str()) != ILLUME_OK) return fail("save pfm");
  }
  illume_bitmap_free(image);
  illume_renderer_destroy(r);
  illume_scene_destroy(scene);
  illume_context_destroy(ctx);
  return 0;
}
