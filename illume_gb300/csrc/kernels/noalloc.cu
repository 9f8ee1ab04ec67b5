// illume_render_noalloc: the wavefront render for callers that cannot allocate device
// memory at render time.
//
// Who needs it: hosts that hand all device memory to their own pool at start-up (a
// later cudaMalloc then fails), and latency-bound frame loops in which a cudaMalloc or
// cudaFree would stall the frame (cudaFree synchronises the device). Such callers
// create the context and upload the scene once at set-up, then render every frame
// through this entry point, which allocates nothing.
//
// How: the queues and counters the wavefront kernels need live in one file-scope
// __device__ array of kNoAllocScratchBytes (about 12 MB). Every GPU that loads this
// library reserves that array until the process exits. Host code cannot use the
// array's name as a device address, so the first call on each device, with that device
// current, asks the runtime for the array's address (cudaGetSymbolAddress) and caches
// it in the illume_context, with the launch grid sizes; make that first call before any
// stream capture. A later call that finds another driver context current on the device
// (the caller reset the device, which also invalidates every handle made before it)
// looks the address up again. The kernels are the same ones
// illume_render_device launches, pointed at slices of the array, one sample of every
// pixel per pass, FP32 accumulation straight into the caller's output buffer.
//
// Every call shares the one array, which keeps the previous call's contents: each call
// clears the counters it needs and the caller's output before rendering. Calls whose
// work overlaps on the GPU (for example on two streams, or from two contexts on one
// device) race on the array: the caller must order them.
#include <algorithm>
#include <mutex>
#include <string>

#include "launch.h"
#include "../host/handles.h"
#include "../host/renderer.h"

namespace illume {

static constexpr size_t kNoAllocMaxPaths = ILLUME_NOALLOC_MAX_PIXELS;
static constexpr size_t kNoAllocPerPath = 6 * sizeof(float4) + sizeof(float4) + sizeof(int) + EV_COUNT * sizeof(int) +
                                          sizeof(float4);
static constexpr size_t kNoAllocScratchBytes = kNoAllocMaxPaths * kNoAllocPerPath + 8192;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mu;

// The driver context current on the calling thread (cuCtxGetCurrent, reached through the
// runtime so that the library does not link the driver library itself); null if the
// entry point is unavailable.
static void* current_driver_context() {
  typedef int (*CtxGetCurrent)(void**);
  static CtxGetCurrent fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return reinterpret_cast<CtxGetCurrent>(f);
  }();
  void* c = nullptr;
  if (!fn || fn(&c) != 0) return nullptr;
  return c;
}

// Clears what must start at zero (counters, ray and visit totals, the output sums) and
// writes the one-row job table.
__global__ void k_noalloc_begin(int* counters, unsigned long long* rays, unsigned long long* visits, JobDesc* job,
                                JobDesc row, float* sum, int npix) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kCounterWords) counters[i] = 0;
  if (i == 0) {
    *rays = 0;
    visits[0] = visits[1] = 0;
    *job = row;
  }
  for (int k = i; k < 3 * npix; k += gridDim.x * blockDim.x) sum[k] = 0.0f;
}

static unsigned char* carve(unsigned char*& p, size_t bytes) {
  unsigned char* r = p;
  p += (bytes + 255) & ~(size_t)255;
  return r;
}

}  // namespace illume

using namespace illume;

extern "C" int illume_render_noalloc(illume_context* ctx, illume_scene* scene, const illume_render_params* params,
                                     float* d_sum) {
  if (!ctx || !scene || !params || !d_sum) { set_error("null argument"); return ILLUME_ERR_INVALID; }
  if (scene->s.ctx != &ctx->c) { set_error("scene was not uploaded with this context"); return ILLUME_ERR_INVALID; }
  const illume_render_params& p = *params;
  // the checks every render takes (sizes, kinds, variants, the medium-field limit of the
  // queued rays), then the limits of this entry point
  std::string err;
  const int chk = check_render_params(p, scene->s, &err);
  if (chk != ILLUME_OK) { set_error("illume_render_noalloc: " + err); return chk; }
  const long long npix = (long long)p.width * p.height;
  if (npix > (long long)kNoAllocMaxPaths) {
    set_error("illume_render_noalloc: image of " + std::to_string(npix) + " pixels exceeds the fixed scratch limit of " +
              std::to_string(kNoAllocMaxPaths) + " pixels (use illume_render_device)");
    return ILLUME_ERR_INVALID;
  }
  if (p.accum_mode != ILLUME_ACCUM_FP32) { set_error("illume_render_noalloc accumulates in FP32 only"); return ILLUME_ERR_INVALID; }
  if (p.estimator != ILLUME_ESTIMATOR_REFERENCE) {
    set_error("illume_render_noalloc runs the reference estimator only (no shadow-ray scratch)");
    return ILLUME_ERR_UNSUPPORTED;
  }
  if (p.samples_per_pass > 1 || p.engines > 1 || p.queue_slots > 0) {
    set_error("illume_render_noalloc renders one sample per pass on one engine without path regeneration "
              "(samples_per_pass and engines must be 0 or 1, queue_slots 0)");
    return ILLUME_ERR_UNSUPPORTED;
  }
  const RenderKnobs k = render_knobs(p);
  const int dev = ctx->c.device;
  ILLUME_CUDA_TRY(cudaSetDevice(dev));
  void* base = nullptr;
  int grid_trace = 0, grid_shade = 0;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    void* cu_ctx = current_driver_context();
    if (!ctx->c.noalloc_scratch || cu_ctx != ctx->c.noalloc_cu_ctx) {
      void* ptr = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr) {
        set_error(std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        return ILLUME_ERR_CUDA;
      }
      ctx->c.noalloc_scratch = ptr;
      ctx->c.noalloc_cu_ctx = cu_ctx;
    }
    base = ctx->c.noalloc_scratch;
    int& gt = ctx->c.noalloc_grid_trace[k.bvh_kind & 3][k.trace_variant & 7];
    if (!gt) gt = kernel_grid_blocks(trace_kernel_ptr(k.bvh_kind, k.trace_variant), 128, dev);
    int& gs = ctx->c.noalloc_grid_shade[k.shade_variant & 7];
    if (!gs) gs = kernel_grid_blocks(shade_kernel_ptr(k.shade_variant), 128, dev);
    grid_trace = gt;
    grid_shade = gs;
  }
  const int cap = (int)npix;
  unsigned char* cur = static_cast<unsigned char*>(base);
  WaveBuffers w{};
  for (int q = 0; q < 2; ++q) {
    w.q_orig[q] = reinterpret_cast<float4*>(carve(cur, sizeof(float4) * cap));
    w.q_dir[q] = reinterpret_cast<float4*>(carve(cur, sizeof(float4) * cap));
    w.q_thr[q] = reinterpret_cast<float4*>(carve(cur, sizeof(float4) * cap));
  }
  w.hit = reinterpret_cast<float4*>(carve(cur, sizeof(float4) * cap));
  w.hit_geom = reinterpret_cast<int*>(carve(cur, sizeof(int) * cap));
  w.evq = reinterpret_cast<int*>(carve(cur, sizeof(int) * (size_t)cap * EV_COUNT));
  w.contrib = reinterpret_cast<float4*>(carve(cur, sizeof(float4) * cap));
  w.counters = reinterpret_cast<int*>(carve(cur, sizeof(int) * kCounterWords));
  w.rays = reinterpret_cast<unsigned long long*>(carve(cur, 8));
  w.visits = reinterpret_cast<unsigned long long*>(carve(cur, 16));
  w.jobs = reinterpret_cast<JobDesc*>(carve(cur, sizeof(JobDesc)));
  w.job_path_base = reinterpret_cast<int*>(carve(cur, 2 * sizeof(int)));
  w.job_pixel_base = reinterpret_cast<int*>(carve(cur, 2 * sizeof(int)));
  if ((size_t)(cur - static_cast<unsigned char*>(base)) > kNoAllocScratchBytes) {
    set_error("scratch layout exceeds the fixed array");
    return ILLUME_ERR_INVALID;
  }
  w.cap = cap;
  w.qcap = cap;
  w.njobs = 1;
  Accumulators acc{};
  acc.sum32 = d_sum;
  JobDesc row = job_row(scene->s, p, acc);
  row.sample_base = p.sample_begin;
  row.sample_end = p.sample_begin + p.spp;
  row.per_pass = 1;
  row.nsamples = p.spp > 0 ? 1 : 0;
  cudaStream_t st = ctx->c.stream;
  const int sms = ctx->c.sm_count > 0 ? ctx->c.sm_count : 1;
  const int grid_small = std::max(1, std::min((cap + 255) / 256, sms * 8));
  k_noalloc_begin<<<grid_small, 256, 0, st>>>(w.counters, w.rays, w.visits, w.jobs, row, d_sum, cap);
  for (int s = 0; s < p.spp; ++s) {
    launch_plan(w, st);
    launch_raygen(w, grid_small, st);
    for (int b = 0; b < p.max_depth; ++b) {
      launch_trace(w, k, b, grid_trace, st);
      launch_shade(w, k, b, grid_shade, st);
    }
    launch_accumulate(w, grid_small, st);
    launch_advance(w, st);
  }
  ILLUME_CUDA_TRY(cudaGetLastError());
  ctx->c.launches += 1 + (long long)p.spp * (4 + 2 * p.max_depth);
  return ILLUME_OK;
}
