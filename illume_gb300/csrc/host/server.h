// Render server: admits jobs by device-memory footprint, keeps scenes and accumulators
// resident, and interleaves progressive sample chunks across the running jobs. A job's
// image depends only on (scene, params): random numbers are keyed by (pixel, sample,
// bounce) and (seed, job), never by which jobs share the device.
#pragma once

#include <deque>
#include <map>
#include <memory>
#include <vector>

#include "renderer.h"

namespace illume {

struct ServerJob {
  int64_t id = 0;
  Scene* scene = nullptr;
  illume_render_params params{};
  std::unique_ptr<Renderer> r;
  int state = 0;            // 0 queued, 1 running, 2 done, 3 cancelled, 4 failed
  int spp_done = 0;
  size_t footprint = 0;
  std::vector<float> mean;
  std::vector<uint8_t> rgb8;
  illume_render_stats stats{};
  std::string error;
  double submit_ms = 0, start_ms = 0, finish_ms = 0;
};

struct Server {
  Context* ctx = nullptr;
  size_t budget = 0;
  int max_in_flight = 8;
  size_t reserved = 0;
  int64_t next_id = 1;
  std::map<int64_t, std::unique_ptr<ServerJob>> jobs;
  std::deque<int64_t> queue;

  static size_t footprint(const illume_render_params& p, int chunk);
  static int chunk_for(const illume_render_params& p);
  int submit(Scene* scene, const illume_render_params& p, int64_t* id);
  int step(int* running);
  int poll(int64_t id, float* mean, uint8_t* rgb8, illume_render_stats* stats);
  int cancel(int64_t id);
};

double now_ms();

}  // namespace illume
