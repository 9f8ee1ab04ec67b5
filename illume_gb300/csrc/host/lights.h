// Light sampling tables of a scene for the opt-in next-event estimator (not in the
// reference, whose paths find light only by BSDF sampling, src/renderer.cu:183-386):
// a piecewise-constant density over the environment map and the list of emissive mesh
// triangles in world space. Built on the host when a scene is uploaded.
#pragma once

#include <vector>

#include "../common/types.h"

namespace illume {

struct SceneHost;

struct HostLights {
  int env_w = 0, env_h = 0;
  std::vector<float> env_func;
  std::vector<AliasEntry> env_rows, env_cols;
  float env_integral = 0.0f;
  float env_prob = 0.0f;
  std::vector<float4> tri;       // 3 per light (see LightView)
  std::vector<AliasEntry> tri_alias;
  std::vector<int> inst_light_base;
};

void build_lights(const SceneHost& h, HostLights* out);

// Walker's alias table of n non-negative weights (Vose's construction, in double):
// choosing slot floor(u n) and keeping it when the fraction of u n is below its `keep`,
// else taking its alias, picks i with probability weights[i] / sum. Returns false when
// the weights sum to zero.
bool build_alias(const double* weights, size_t n, AliasEntry* out);

}  // namespace illume
