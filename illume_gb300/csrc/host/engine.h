// Wavefront engine: the device buffers and captured passes of one job table.
//
// A pass renders the current sample range of every row of the table (see
// kernels/launch.h). The host keeps a mirror of the table that it advances exactly as
// k_advance advances the device copy, so it knows every row's sample range after any
// number of replayed passes without reading the device. Rows are written to the device
// only between passes (stream-ordered copies), whole when a job starts and as the
// pass-state words when its share of the slots changes.
#pragma once

#include <map>
#include <string>
#include <vector>

#include "../kernels/launch.h"
#include "runtime.h"

namespace illume {

struct Engine {
  Context* ctx = nullptr;
  int rows = 0;                  // job table rows
  int cap = 0;                   // path slots of one pass
  // Path regeneration: with queue_req > 0 and below the slots, the queues hold qcap rays
  // and new paths enter as earlier ones end (threshold: the next queue's fill, as a share
  // of qcap, at or below which new paths are started); otherwise qcap = cap.
  int queue_req = 0, qcap = 0;
  int ray_group = kDefaultRayGroup;   // samples of a pixel together in the camera-ray queue
  float regen_threshold = 1.0f;
  bool regen = false;
  RenderKnobs knobs{};
  DevBuffer q_orig[2], q_dir[2], q_thr[2], q_bounce[2], hit, hit_geom, evq, counters, contrib, rays, visits;
  DevBuffer jobs, path_base, pixel_base;
  DevBuffer s_orig, s_dir, s_val;   // shadow rays (allocated when a job uses next-event estimation)
  WaveBuffers w{};
  std::vector<JobDesc> mirror;   // the table as the device has it after the launched passes
  int grid_trace = 0, grid_shade = 0, grid_raygen = 0, grid_acc = 0, grid_shadow = 0, grid_shade_nee = 0;
  cudaStream_t stream = nullptr;            // the engine's stream (the context's unless set before init)
  cudaStream_t side = nullptr;              // captures the regeneration loop's body
  std::map<int, cudaGraphExec_t> graphs;   // captured pass by (depth, shadow stage)
  std::map<int, cudaGraphExec_t> head_graphs;   // the same without accumulate and advance
  cudaGraphExec_t acc_graph = nullptr;          // accumulate + advance
  long long passes = 0, launches = 0;

  Engine() = default;
  Engine(const Engine&) = delete;
  Engine& operator=(const Engine&) = delete;
  ~Engine();

  int init(Context* c, int rows, int cap, const RenderKnobs& k, std::string* err, int queue_slots = 0,
           float threshold = 1.0f);
  // Reallocates the per-path buffers for a new slot count (between passes only).
  int resize(int new_cap, std::string* err);
  // Selects another trace kernel instance (between passes only).
  int set_trace_variant(int variant);
  // Path regeneration with `queue_slots` rays in flight (0: off) and `threshold` (between
  // passes only; reallocates the queues when their size changes).
  int set_regen(int queue_slots, float threshold, std::string* err);
  int write_row(int r);          // whole row (a job starts: its ray total restarts at 0)
  int write_pass_state(int r);   // sample_base, nsamples, sample_end, per_pass of row r
  // Replays the captured pass `npasses` times with `depth` bounces and advances the mirror.
  int run(int npasses, int depth);
  // One pass launched kernel by kernel, with events after every stage:
  // ev[0] before plan, ev[1] after raygen, ev[2 + 2b] after trace b, ev[3 + 2b] after
  // shade b, ev[2 + 2 n] after accumulate, n = *iterations (depth, or under
  // regeneration the loop's iterations, driven from the host). count_visits selects the
  // instrumented trace.
  int run_profiled(int depth, bool count_visits, std::vector<cudaEvent_t>& ev, int* iterations = nullptr);
  // One pass whose accumulation waits for `wait_ev` (when not null) and is followed by a
  // record of `record_ev`: two engines on two streams alternate passes over one job's
  // samples, each pass's rendering overlapping the other's, their accumulations in
  // sample order.
  int run_interleaved(int depth, cudaEvent_t wait_ev, cudaEvent_t record_ev);
  int read_row_rays(int r, unsigned long long* out);   // synchronous
  int free_rows() const;
  long long paths_in_pass() const;                      // of the next pass, from the mirror
  static int launches_per_pass(int depth, bool nee = false) { return 5 + (nee ? 3 : 2) * depth; }
  // Launches of regenerating passes with `iterations` loop iterations in all.
  static long long launches_regen(long long passes, long long iterations, bool nee = false) {
    return 5 * passes + (nee ? 5 : 4) * iterations;
  }
  bool any_nee() const;   // a job of the next pass uses next-event estimation
  size_t device_bytes() const;

 private:
  int alloc_paths(std::string* err);
  void point();
  void advance_mirror();
  int launch_head(cudaStream_t st, int depth, bool nee);
  int launch_pass(cudaStream_t st, int depth, bool nee);
  void launch_iteration(cudaStream_t st, cudaGraphConditionalHandle cond, bool use_cond, int depth, bool nee);
  int ensure_shadow(std::string* err);
  void drop_graphs();
};

}  // namespace illume
