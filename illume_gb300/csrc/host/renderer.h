// Renderer: the GB300 replacement of Renderer::render_to_bitmap (src/renderer.cu:498-597).
//
// A render is a sequence of wavefront passes. Each pass keeps `per_pass` samples of every
// pixel in flight: raygen, max_depth x (trace, shade), accumulate, advance. The pass is
// captured once into a CUDA graph and replayed; everything that changes from pass to
// pass (first sample, samples in the pass) lives in device memory, so the host issues
// one graph launch per pass and never waits inside the loop.
#pragma once

#include <memory>

#include "../kernels/launch.h"
#include "runtime.h"

namespace illume {

struct Renderer {
  Context* ctx = nullptr;
  Scene* scene = nullptr;
  illume_render_params p{};
  int npix = 0, per_pass = 1, cap = 0;
  DevBuffer q_orig[2], q_dir[2], q_thr[2], hit, hit_geom, evq, counters, contrib, rays, visits, pass;
  DevBuffer sum32, comp32, sum64, sumsq, out_mean, out_rgb8;
  WaveBuffers w{};
  Accumulators acc{};
  CameraView cam{};
  RenderKnobs knobs{};
  int grid_trace = 0, grid_shade = 0, grid_raygen = 0, grid_acc = 0;
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  long long samples_done = 0;   // samples accumulated since the last clear
  int next_sample = 0;          // first sample of the next progressive call

  ~Renderer();
  int init(std::string* err);
  // Renders p.spp samples; restarts the accumulation unless `accumulate`.
  int render_device(bool accumulate, illume_render_stats* stats);
  int read(float* mean, double* sum, double* sumsq, uint8_t* rgb8);
  // One pass launched kernel by kernel with events (see illume_renderer_profile).
  int profile(bool count_visits, illume_profile* out);
  size_t device_bytes() const;

 private:
  int launch_pass(cudaStream_t st);
};

CameraView make_camera(const SceneHost& h, int width, int height);

}  // namespace illume
