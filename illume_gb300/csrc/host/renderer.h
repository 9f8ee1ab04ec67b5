// Renderer: the GB300 replacement of Renderer::render_to_bitmap (src/renderer.cu:498-597).
//
// A render is a sequence of wavefront passes over a one-row job table (engine.h). Each
// pass keeps `per_pass` samples of every pixel in flight: plan, raygen, max_depth x
// (trace, shade), accumulate, advance. The pass is captured once into a CUDA graph and
// replayed; the sample range lives in the device's job row, so the host issues one
// graph launch per pass and never waits inside the loop.
//
// Large renders split the path slots over several engines on their own streams that
// take turns on the sample ranges: while one pass is in its last bounces (few, long rays
// that leave most of the GPU idle), the next passes' first bounces fill the GPU.
// Accumulations stay in sample order (each waits for the previous pass's), so the image
// is the same as with one engine.
#pragma once

#include <memory>
#include <vector>

#include "engine.h"

namespace illume {

struct Renderer {
  Context* ctx = nullptr;
  Scene* scene = nullptr;
  illume_render_params p{};
  int npix = 0, per_pass = 1;
  Engine eng;                   // engine 0, on the context's stream
  // engines 1..nengines-1 of a split render, each on a stream of its own; engine e
  // renders samples [e p, (e + 1) p), [(e + n) p, (e + n + 1) p), ... of each call
  std::vector<std::unique_ptr<Engine>> more;
  std::vector<cudaStream_t> more_streams;
  int nengines = 1;
  std::vector<cudaEvent_t> acc_ev;   // per engine: its last pass's accumulation
  std::vector<cudaEvent_t> join_ev;  // per extra engine: the end of its work in a call
  DevBuffer sum32, comp32, sum64, sumsq, out_mean, out_rgb8;
  Accumulators acc{};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  long long samples_done = 0;   // samples accumulated since the last clear
  int next_sample = 0;          // first sample of the next progressive call
  // set by render_device when a traversal of the call found its stack full (the kernels'
  // defect flag, kCounterStackDrops): the image is complete but may lack hits
  bool stack_overflow = false;
  std::vector<int> iter_total;   // per engine: regeneration loop iterations read at the last call's end

  ~Renderer();
  int init(std::string* err);
  // Renders p.spp samples; restarts the accumulation unless `accumulate`.
  int render_device(bool accumulate, illume_render_stats* stats);
  int read(float* mean, double* sum, double* sumsq, uint8_t* rgb8);
  // One pass launched kernel by kernel with events (see illume_renderer_profile).
  int profile(bool count_visits, illume_profile* out);
  size_t device_bytes() const;

 private:
  void set_range(int first, int count);
  Engine& engine(int e) { return e == 0 ? eng : *more[e - 1]; }
};

CameraView make_camera(const SceneHost& h, int width, int height);

// Checks the parts of a render's parameters that every path of this library needs.
// Checks the parameters against the scene; an 8-wide BVH kind builds and uploads the
// scene's 8-wide layout first (Scene::ensure_wide).
int check_render_params(const illume_render_params& p, Scene& scene, std::string* err);

// Job row of a render: scene, camera, Philox key and depth of `p`, no sample range yet.
JobDesc job_row(const Scene& scene, const illume_render_params& p, const Accumulators& acc);

// Trace kernel settings of a render (intersector, BVH layout, kernel variant).
RenderKnobs render_knobs(const illume_render_params& p);

}  // namespace illume
