// Host-side launchers of the sm_103a kernels (defined in the .cu files of this folder).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../common/types.h"

namespace illume {

// Device-side pass bookkeeping, advanced by the last kernel of every wavefront pass so
// that a captured pass can be replayed without host involvement.
struct PassState {
  int sample_base;   // first sample index of the current pass
  int nsamples;      // samples of every pixel in the current pass
  int sample_end;    // one past the last sample of the render
  int per_pass;      // samples per pass
};

// Wavefront buffers. Queues are double-buffered by bounce parity.
struct WaveBuffers {
  float4* q_orig[2];     // origin xyz, path id (int bits)
  float4* q_dir[2];      // direction xyz, medium index (int bits, -1 = air)
  float4* q_thr[2];      // throughput xyz
  float4* hit;           // t, u, v, prim (int bits), per slot of the current queue
  int* hit_geom;         // instance >= 0, sphere -2 - s, miss -1
  int* evq;              // EV_COUNT queues of `cap` slot indices each
  int* counters;         // [0..1] queue sizes, [2 + 16 * parity + class] event counts
  float4* contrib;       // per path radiance of the current pass (sample-major)
  unsigned long long* rays;   // closest-hit queries traced (running total)
  unsigned long long* visits; // [node fetches, triangle tests] of the instrumented trace kernel
  PassState* pass;
  int cap;               // path slots (pixels * samples per pass)
  int npix, width, height;
};

struct RenderKnobs {
  uint32_t seed, job;
  int max_depth;
  float ray_bias;
  int isect, exact_hg, bvh_kind, accum_mode;
  int trace_variant;   // 8-wide BVH: 0 = persistent state machine, 1 = one ray per lane to completion
};

struct Accumulators {
  float* sum32;          // FP32 / Kahan sum (3 per pixel)
  float* comp32;         // Kahan compensation (3 per pixel)
  double* sum64;         // FP64 sum (3 per pixel)
  double* sumsq;         // sum of squares of per-sample radiance (3 per pixel), nullable
};

int kernel_grid_blocks(const void* fn, int block, int device);

void launch_raygen(const WaveBuffers& w, const CameraView& cam, const RenderKnobs& k, int grid, cudaStream_t st);
void launch_trace(const WaveBuffers& w, const SceneView& sc, const RenderKnobs& k, int bounce, int grid,
                  cudaStream_t st, bool count_visits = false);
void launch_shade(const WaveBuffers& w, const SceneView& sc, const RenderKnobs& k, int bounce, int grid,
                  cudaStream_t st);
void launch_accumulate(const WaveBuffers& w, const Accumulators& acc, int accum_mode, int grid, cudaStream_t st);
void launch_advance_pass(const WaveBuffers& w, cudaStream_t st);
void launch_tonemap(const Accumulators& acc, int accum_mode, int npix, float samples, int op, uint8_t* rgb8,
                    float* mean, cudaStream_t st);
void launch_clear_accumulators(const Accumulators& acc, int npix, cudaStream_t st);

// test hooks
void launch_trace_hook(const SceneView& sc, const float* rays8, int n, int isect, int bvh_kind, void* hits,
                       cudaStream_t st);
void launch_bsdf_batch(int type, int distribution, const float* in, int n, float* out, cudaStream_t st);

const void* trace_kernel_ptr(int bvh_kind, int variant = 0);
const void* shade_kernel_ptr();

}  // namespace illume
