// Render server with continuous batching.
//
// Jobs share one wavefront job table per trace-kernel setting (intersector, BVH layout).
// A queued job is admitted as soon as a table row and its device footprint fit. Before
// every step the server composes the next passes: jobs grouped by scene (one scene's
// BVH per pass stays in L2), groups taken smallest remaining job first while the slots
// and an L2 budget allow (or the pass is under half full), the chosen jobs sharing the
// path slots by water-filling, the others paused. Small jobs thus run together in one
// full pass instead of one under-filled pass each, and a finished job frees its row
// and slots for the next pass. Scenes, BVHs and accumulators stay resident on the
// device between passes.
//
// A job's image depends only on its own scene and parameters: random numbers are keyed
// by (pixel, sample, bounce) and (seed, job), and each pixel's samples are summed in
// sample order whatever the pass split, so the result is bit-identical alone and in
// any mix.
//
// Every trace-kernel setting has up to `lanes` job tables (4 by default, 16 for a
// batch), each on its own stream; an admitted job joins the table with the least work
// to go and stays there, and a new table is made only when every existing one has work. A step launches
// every table's passes at once, so one table's last bounces (few, long rays that leave
// most of the GPU idle) overlap the other tables' passes.
//
// The autotuner picks the tables' path slots and trace kernel variant from measured
// throughput on the live workload: each candidate runs a few steps of the real jobs
// (no work is thrown away, since the split of samples into passes and the kernel
// variant do not change any result), then the fastest is kept.
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
  float camera[15] = {};    // copy of params.camera when given
  int state = 0;            // 0 queued, 1 running, 2 done, 3 cancelled, 4 failed
  int key = -1, row = -1;   // engine and job-table row while running
  size_t footprint = 0;
  DevBuffer sum32, comp32, sum64, out_mean, out_rgb8;
  std::vector<float> mean;
  std::vector<uint8_t> rgb8;
  illume_render_stats stats{};
  std::string error;
  double submit_ms = 0, start_ms = 0, finish_ms = 0;
};

// A job table's stream and the event that marks the end of its work in a step.
struct LaneStream {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  LaneStream() = default;
  LaneStream(const LaneStream&) = delete;
  LaneStream& operator=(const LaneStream&) = delete;
  ~LaneStream();
};

struct ServerEngine {
  std::shared_ptr<LaneStream> lane;      // declared before eng: outlives the engine's buffers
  std::unique_ptr<Engine> eng;
  int base_key = 0;                      // trace-kernel setting (engine_key)
  std::vector<int64_t> row_job;          // job id per row, 0 = free
  unsigned long long rays_seen = 0;      // engine ray total at the last read
  int iters_seen = 0;                    // regeneration loop iterations at the last read
};

// Autotuner state of one trace-kernel setting (all its tables move together).
struct Tuner {
  int state = 0;                         // 0 not started, 1 measuring, 2 done
  int idx = 0, steps = 0;
  double rays = 0, ms = 0;
  struct Candidate { int cap, variant, queue_slots; float threshold; };
  std::vector<Candidate> candidates;             // path slots per table, trace variant, regeneration
  std::vector<double> rate;                      // rays per ms of each candidate
};

struct Server {
  Context* ctx = nullptr;
  size_t budget = 0;          // device bytes for engines and job buffers (0 = unlimited)
  int rows = 64;              // job-table rows per engine
  int path_capacity = 1 << 25;
  int passes_per_step = 1;
  int autotune = 0;
  int trace_variant = -1;     // -1 = per-layout default
  int lanes = 4;              // job tables per trace-kernel setting
  int queue_slots = 0;        // path regeneration: rays in flight per table (0 = off)
  float regen_threshold = 1.0f;
  size_t reserved = 0;        // job footprints
  int64_t next_id = 1;
  std::map<int64_t, std::unique_ptr<ServerJob>> jobs;
  std::deque<int64_t> queue;
  std::map<int, ServerEngine> engines;   // by engine_key * kMaxLanes + lane
  std::map<int, Tuner> tuners;           // by engine_key
  illume_server_stats totals{};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // the passes of the last step, still running on the device when step() returned
  struct Launched { ServerEngine* se; int k; unsigned long long total; int iter_total; };
  std::vector<Launched> in_flight;

  ~Server();
  static size_t footprint(const illume_render_params& p);
  int submit(Scene* scene, const illume_render_params& p, int64_t* id);
  int step(int* running);
  int poll(int64_t id, float* mean, uint8_t* rgb8, illume_render_stats* stats);
  int cancel(int64_t id);
  int set_option(int option, int64_t value);
  void get_stats(illume_server_stats* out) const;

 private:
  size_t engines_bytes() const;
  int admit();
  void compose(ServerEngine& se);
  int retire(ServerEngine& se, std::vector<ServerJob*>* done);
  int new_engine(const illume_render_params& p, int key, long long cap, ServerEngine** out);
  int finish_in_flight(std::vector<ServerJob*>* done);
  void tune(int base_key, double rays, double ms);
  int apply_candidate(int base_key, int idx);
};

double now_ms();

void plan_shares(const std::vector<long long>& npix, const std::vector<int>& left, long long cap,
                 std::vector<int>* per_pass);

}  // namespace illume
