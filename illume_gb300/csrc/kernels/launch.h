// Host-side launchers of the sm_103a kernels (defined in the .cu files of this folder).
//
// Every wavefront pass runs over a table of jobs. A job is one render (scene, camera,
// Philox key, depth, accumulators, sample range); a plain render is a table of one job.
// The device advances each job's sample range after every pass, so a captured pass can
// be replayed any number of times without the host.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../common/types.h"

namespace illume {

struct Accumulators {
  float* sum32;          // FP32 / Kahan sum (3 per pixel)
  float* comp32;         // Kahan compensation (3 per pixel)
  double* sum64;         // FP64 sum (3 per pixel)
  double* sumsq;         // sum of squares of per-sample radiance (3 per pixel), nullable
};

// One row of the job table (256 bytes).
struct JobDesc {
  SceneView sc;
  CameraView cam;
  Accumulators acc;
  uint32_t seed, job;        // Philox key
  int max_depth;             // closest-hit queries per path
  float ray_bias;
  int flags, accum_mode;      // flags: JOB_EXACT_HG, JOB_NEE, interleave (job_interleave)
  int npix, width;
  // pass state: samples [sample_base, sample_base + nsamples) of every pixel are in the
  // current pass; advanced by k_advance after every pass; nsamples == 0 = idle row
  int sample_base, nsamples, sample_end, per_pass;
  int path_base;             // first path slot of this job in the current pass (k_plan)
  int pixel_base;            // first index of this job's pixels in the accumulation sweep (k_plan)
  unsigned long long rays;   // closest-hit queries traced for this job (running total)
};
static_assert(sizeof(JobDesc) == 256, "JobDesc layout");
enum JobFlags : int { JOB_EXACT_HG = 1, JOB_NEE = 2 };
// Bits 8..15 of the flags: how many job tables take turns on this job's sample ranges
// (0 or 1: this table alone). With n tables, a pass of one table is followed by one pass
// of each other table before its next range, so the row skips the others' samples.
static constexpr int kInterleaveShift = 8;
__host__ __device__ __forceinline__ int job_interleave(int flags) {
  const int n = (flags >> kInterleaveShift) & 0xff;
  return n > 1 ? n : 1;
}
// Pass state after a pass of `nsamples` (the same arithmetic on the host mirror and in
// k_advance).
__host__ __device__ __forceinline__ void advance_pass_state(int& sample_base, int& nsamples, int sample_end,
                                                            int per_pass, int flags) {
  sample_base += nsamples + (job_interleave(flags) - 1) * per_pass;
  const int left = sample_end - sample_base;
  nsamples = left < per_pass ? (left > 0 ? left : 0) : per_pass;
}

// A queued ray's fourth direction word packs its job row and medium:
// (job << kMediumBits) | (medium + 1), medium -1 = air.
static constexpr int kMediumBits = 12;
static constexpr int kMaxMediums = (1 << kMediumBits) - 2;
static constexpr int kMaxJobRows = 1 << 18;

// Wavefront buffers. Queues are double-buffered by bounce parity; a path's slot in the
// current pass indexes its radiance in `contrib`.
struct WaveBuffers {
  float4* q_orig[2];     // origin xyz, path slot (int bits)
  float4* q_dir[2];      // direction xyz, packed job / medium (int bits)
  float4* q_thr[2];      // throughput xyz
  float4* hit;           // t, u, v, prim (int bits), per slot of the current queue
  int* hit_geom;         // instance >= 0, sphere -2 - s, miss -1
  int* evq;              // EV_COUNT queues of `cap` slot indices each
  int* counters;         // see kCounter* below
  float4* contrib;       // per path radiance of the current pass
  float4* s_orig;        // shadow rays of the next-event estimator: origin, job row (int bits)
  float4* s_dir;         //   direction, maximum distance
  float4* s_val;         //   contribution if unoccluded, path slot (int bits)
  unsigned long long* rays;   // closest-hit queries traced (running total)
  unsigned long long* visits; // [node fetches, triangle tests, warp node-fetch slots] of the instrumented trace kernel
  JobDesc* jobs;
  int* job_path_base;    // njobs + 1 prefix sums of the pass's paths (k_plan)
  int* job_pixel_base;   // njobs + 1 prefix sums of the pass's pixels (k_plan)
  // Path regeneration: the bounce of each queued ray, by queue parity. Null: every ray of
  // a queue is at the pass's bounce (the queues hold all the pass's paths at once).
  int* q_bounce[2];
  int njobs;
  int ray_group;         // camera rays in the queue: up to ray_group samples of a pixel together (<= 1: one sample, pixels in tiles)

  int cap;               // path slots of one pass (per-path radiance)
  int qcap;              // queue slots (rays in flight); equal to cap without regeneration
};

// counters[]: [0..1] queue sizes by parity, [2 + 16 * parity + class] event counts,
// [kCounterPaths] paths of the pass, [kCounterPixels] pixels of the pass, [42] slot
// overflow flag, [44 + parity] trace ray-fetch counters, [46 + parity] shadow-ray counts,
// [48 + parity] shadow-ray fetch counters, [kCounterStackDrops] set when a traversal
// found its stack full (kept across passes; cleared when the engine is made and read by
// the renderer after each render).
static constexpr int kCounterPaths = 40;
static constexpr int kCounterStackDrops = 50;
// Path regeneration (a pass whose paths outnumber the queue slots): paths started so
// far, the loop's iteration, the next batch of new paths (count, first path, first queue
// position), whether the loop goes on, a flag set when its iteration bound ended a pass
// (kept across passes, like the stack-overflow flag) and the loop's iterations since the
// engine was made.
static constexpr int kCounterGen = 51;
static constexpr int kCounterIter = 52;
static constexpr int kCounterRegenN = 53;
static constexpr int kCounterRegenFirst = 54;
static constexpr int kCounterRegenQ = 55;
static constexpr int kCounterMore = 56;
static constexpr int kCounterLoopLimit = 57;
static constexpr int kCounterIterTotal = 58;
static constexpr int kCounterPixels = 41;
static constexpr int kCounterWords = 64;

// Iteration of a stage launched with `bounce` (-1 under path regeneration: read from the
// counters), and the bounce of queued ray i.
__device__ __forceinline__ int pass_iteration(const WaveBuffers& w, int bounce) {
  return bounce >= 0 ? bounce : w.counters[kCounterIter];
}
__device__ __forceinline__ int ray_bounce(const WaveBuffers& w, int parity, int i, int it) {
  return w.q_bounce[parity] ? w.q_bounce[parity][i] : it;
}

// Samples of a pixel kept together in a pass's camera-ray queue by default (traversal
// workload, Mrays/s: 1 -> 4168, 4 -> 4249, 8 -> 4311, 16 -> 4349, 32 -> 4266).
static constexpr int kDefaultRayGroup = 16;

// Settings shared by every job of a table (they select kernel instances).
struct RenderKnobs {
  int isect;           // illume_intersector
  int bvh_kind;        // BVH_BINARY or BVH_WIDE8
  int trace_variant;   // see trace_kernel_ptr
  int shade_variant;   // see shade_kernel_ptr
};

int kernel_grid_blocks(const void* fn, int block, int device);

void launch_plan(const WaveBuffers& w, cudaStream_t st);
void launch_raygen(const WaveBuffers& w, int grid, cudaStream_t st);
// Path regeneration. A pass runs as a loop of iterations (trace, shade, [shadow], plan of
// the next new paths, their camera rays) over queues of qcap rays, new paths entering
// the queue as earlier ones end, until every path of the pass has ended. The stages take
// bounce = -1 and read the iteration from the counters. regen_start: the first
// min(qcap, paths) paths; regen_plan: after an iteration's shading, starts new paths when
// the next queue holds at most threshold x qcap rays (filling it to qcap), and sets the
// loop's condition (through `cond` when launched inside a graph's while node, else only
// counters[kCounterMore]); the loop ends early, raising counters[kCounterLoopLimit], at
// an iteration bound derived from the paths, qcap, threshold and `depth`.
void launch_regen_start(const WaveBuffers& w, cudaStream_t st);
void launch_regen(const WaveBuffers& w, int grid, cudaStream_t st);
void launch_regen_plan(const WaveBuffers& w, cudaGraphConditionalHandle cond, bool use_cond, int depth, float threshold,
                       cudaStream_t st);
void launch_trace(const WaveBuffers& w, const RenderKnobs& k, int bounce, int grid, cudaStream_t st,
                  bool count_visits = false);
void launch_shade(const WaveBuffers& w, const RenderKnobs& k, int bounce, int grid, cudaStream_t st, bool nee = false);
void launch_shadow(const WaveBuffers& w, const RenderKnobs& k, int bounce, int grid, cudaStream_t st);
void launch_accumulate(const WaveBuffers& w, int grid, cudaStream_t st);
void launch_advance(const WaveBuffers& w, cudaStream_t st);
void launch_tonemap(const Accumulators& acc, int accum_mode, int npix, float samples, int op, uint8_t* rgb8,
                    float* mean, cudaStream_t st);
void launch_clear_accumulators(const Accumulators& acc, int npix, cudaStream_t st);

// test hooks
// d_view: a device copy of sc (read by the persistent 8-wide kernel, bvh_kind 2)
void launch_trace_hook(const SceneView& sc, const SceneView* d_view, const float* rays8, int n, int isect,
                       int bvh_kind, void* hits, cudaStream_t st);
void launch_bsdf_batch(int type, int distribution, const float* in, int n, float* out, cudaStream_t st);

const void* trace_kernel_ptr(int bvh_kind, int variant = 0);
// L2 read-bandwidth probe (measurement only).
void launch_l2_read(const void* buf, size_t bytes, int reps, unsigned* sink, int grid, cudaStream_t st);
const void* l2_read_kernel_ptr();
const void* shade_kernel_ptr(int variant = 0, bool nee = false);
const void* shadow_kernel_ptr(int bvh_kind);

}  // namespace illume
