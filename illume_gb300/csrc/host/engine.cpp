#include "engine.h"

#include <stddef.h>

#include <algorithm>
#include <functional>

namespace illume {

Engine::~Engine() {
  drop_graphs();
  if (side) cudaStreamDestroy(side);
}

void Engine::drop_graphs() {
  for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
  graphs.clear();
  for (auto& kv : head_graphs) cudaGraphExecDestroy(kv.second);
  head_graphs.clear();
  if (acc_graph) cudaGraphExecDestroy(acc_graph);
  acc_graph = nullptr;
}

static int capture(cudaStream_t st, cudaGraphExec_t* out, const std::function<int()>& body) {
  cudaGraph_t g = nullptr;
  ILLUME_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  const int bs = body();
  const cudaError_t ee = cudaStreamEndCapture(st, &g);   // ends the capture whatever the body did
  if (bs != ILLUME_OK) {
    if (g) cudaGraphDestroy(g);
    return bs;
  }
  if (ee != cudaSuccess) {
    set_error(std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ee));
    return ILLUME_ERR_CUDA;
  }
  const cudaError_t e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    set_error(std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
    return ILLUME_ERR_CUDA;
  }
  return ILLUME_OK;
}

// Inside a capture on `st`: appends a while node to the captured graph (its condition
// starts at 1 on every launch of the graph) and captures its body from body(cond) on the
// stream `side`; work captured on `st` afterwards follows the loop.
static int capture_while(cudaStream_t st, cudaStream_t side, const std::function<void(cudaGraphConditionalHandle)>& body) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  ILLUME_CUDA_TRY(cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd));
  if (cs != cudaStreamCaptureStatusActive) {
    set_error("capture_while: the stream is not capturing");
    return ILLUME_ERR_CUDA;
  }
  cudaGraphConditionalHandle cond;
  ILLUME_CUDA_TRY(cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams np = {};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = cond;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  ILLUME_CUDA_TRY(cudaGraphAddNode(&node, g, deps, nullptr, nd, &np));
  ILLUME_CUDA_TRY(cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  ILLUME_CUDA_TRY(cudaStreamBeginCaptureToGraph(side, np.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                                cudaStreamCaptureModeRelaxed));
  body(cond);
  cudaGraph_t bg = nullptr;
  ILLUME_CUDA_TRY(cudaStreamEndCapture(side, &bg));
  return ILLUME_OK;
}

int Engine::ensure_shadow(std::string* err) {
  if (s_orig.get() && s_orig.size() >= sizeof(float4) * (size_t)qcap) return ILLUME_OK;
  int st;
  if ((st = s_orig.alloc(ctx, sizeof(float4) * (size_t)qcap)) != ILLUME_OK) { *err = last_error(); return st; }
  if ((st = s_dir.alloc(ctx, sizeof(float4) * (size_t)qcap)) != ILLUME_OK) { *err = last_error(); return st; }
  if ((st = s_val.alloc(ctx, sizeof(float4) * (size_t)qcap)) != ILLUME_OK) { *err = last_error(); return st; }
  drop_graphs();
  point();
  return ILLUME_OK;
}

bool Engine::any_nee() const {
  for (const JobDesc& J : mirror)
    if (J.nsamples > 0 && (J.flags & JOB_NEE)) return true;
  return false;
}

int Engine::alloc_paths(std::string* err) {
  int st;
  regen = queue_req > 0 && queue_req < cap;
  qcap = regen ? queue_req : cap;
#define ALLOC(buf, bytes) if ((st = (buf).alloc(ctx, (bytes))) != ILLUME_OK) { *err = last_error(); return st; }
  for (int k = 0; k < 2; ++k) {
    ALLOC(q_orig[k], sizeof(float4) * (size_t)qcap);
    ALLOC(q_dir[k], sizeof(float4) * (size_t)qcap);
    ALLOC(q_thr[k], sizeof(float4) * (size_t)qcap);
    if (regen) { ALLOC(q_bounce[k], sizeof(int) * (size_t)qcap); }
    else q_bounce[k].release();
  }
  ALLOC(hit, sizeof(float4) * (size_t)qcap);
  ALLOC(hit_geom, sizeof(int) * (size_t)qcap);
  ALLOC(evq, sizeof(int) * (size_t)qcap * EV_COUNT);
  ALLOC(contrib, sizeof(float4) * (size_t)cap);
#undef ALLOC
  return ILLUME_OK;
}

void Engine::point() {
  for (int k = 0; k < 2; ++k) {
    w.q_orig[k] = q_orig[k].as<float4>();
    w.q_dir[k] = q_dir[k].as<float4>();
    w.q_thr[k] = q_thr[k].as<float4>();
  }
  w.hit = hit.as<float4>();
  w.hit_geom = hit_geom.as<int>();
  w.evq = evq.as<int>();
  w.counters = counters.as<int>();
  w.contrib = contrib.as<float4>();
  w.s_orig = s_orig.as<float4>();
  w.s_dir = s_dir.as<float4>();
  w.s_val = s_val.as<float4>();
  w.rays = rays.as<unsigned long long>();
  w.visits = visits.as<unsigned long long>();
  w.jobs = jobs.as<JobDesc>();
  w.job_path_base = path_base.as<int>();
  w.job_pixel_base = pixel_base.as<int>();
  w.njobs = rows;
  w.ray_group = ray_group;
  w.cap = cap;
  w.qcap = qcap;
  for (int k = 0; k < 2; ++k) w.q_bounce[k] = regen ? q_bounce[k].as<int>() : nullptr;
  const int sms = std::max(1, ctx->sm_count);
  grid_raygen = std::max(1, std::min((qcap + 255) / 256, sms * 8));
  grid_acc = grid_raygen;
}

int Engine::init(Context* c, int nrows, int ncap, const RenderKnobs& k, std::string* err, int queue_slots,
                 float threshold) {
  ctx = c;
  if (!stream) stream = ctx->stream;
  rows = nrows;
  cap = ncap;
  knobs = k;
  queue_req = queue_slots > 0 ? queue_slots : 0;
  regen_threshold = threshold;
  if (!(threshold >= 0.0f && threshold <= 1.0f)) { *err = "regeneration threshold outside [0, 1]"; return ILLUME_ERR_INVALID; }
  if (queue_req > 0 && !side) ILLUME_CUDA_TRY(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
  if (rows < 1 || rows > kMaxJobRows) { *err = "job table rows out of range"; return ILLUME_ERR_INVALID; }
  if (cap < 1 || cap > (1 << 30)) { *err = "path slots out of range"; return ILLUME_ERR_INVALID; }
  int st;
  if ((st = alloc_paths(err)) != ILLUME_OK) return st;
#define ALLOC(buf, bytes) if ((st = (buf).alloc(ctx, (bytes))) != ILLUME_OK) { *err = last_error(); return st; }
  ALLOC(counters, sizeof(int) * kCounterWords);
  ALLOC(rays, sizeof(unsigned long long));
  ALLOC(visits, 3 * sizeof(unsigned long long));
  ALLOC(jobs, sizeof(JobDesc) * (size_t)rows);
  ALLOC(path_base, sizeof(int) * (size_t)(rows + 1));
  ALLOC(pixel_base, sizeof(int) * (size_t)(rows + 1));
#undef ALLOC
  mirror.assign(rows, JobDesc{});
  ILLUME_CUDA_TRY(cudaMemsetAsync(counters.get(), 0, counters.size(), stream));
  ILLUME_CUDA_TRY(cudaMemsetAsync(rays.get(), 0, rays.size(), stream));
  ILLUME_CUDA_TRY(cudaMemsetAsync(visits.get(), 0, visits.size(), stream));
  ILLUME_CUDA_TRY(cudaMemsetAsync(jobs.get(), 0, jobs.size(), stream));
  point();
  grid_trace = kernel_grid_blocks(trace_kernel_ptr(knobs.bvh_kind, knobs.trace_variant), 128, ctx->device);
  grid_shade = kernel_grid_blocks(shade_kernel_ptr(knobs.shade_variant), 128, ctx->device);
  grid_shadow = kernel_grid_blocks(shadow_kernel_ptr(knobs.bvh_kind), 128, ctx->device);
  grid_shade_nee = kernel_grid_blocks(shade_kernel_ptr(knobs.shade_variant, true), 128, ctx->device);
  return ILLUME_OK;
}

int Engine::resize(int new_cap, std::string* err) {
  if (new_cap == cap) return ILLUME_OK;
  if (new_cap < 1 || new_cap > (1 << 30)) { *err = "path slots out of range"; return ILLUME_ERR_INVALID; }
  ILLUME_CUDA_TRY(cudaStreamSynchronize(stream));
  drop_graphs();
  const int old = cap;
  cap = new_cap;
  int st = alloc_paths(err);
  if (st != ILLUME_OK) {
    cap = old;
    std::string e2;
    alloc_paths(&e2);
    point();
    return st;
  }
  if (s_orig.get() && (st = ensure_shadow(err)) != ILLUME_OK) return st;
  point();
  return ILLUME_OK;
}

int Engine::set_regen(int queue_slots, float threshold, std::string* err) {
  if (!(threshold >= 0.0f && threshold <= 1.0f)) { *err = "regeneration threshold outside [0, 1]"; return ILLUME_ERR_INVALID; }
  queue_slots = std::max(queue_slots, 0);
  if (queue_slots == queue_req && threshold == regen_threshold) return ILLUME_OK;
  ILLUME_CUDA_TRY(cudaStreamSynchronize(stream));
  drop_graphs();
  if (queue_slots > 0 && !side) ILLUME_CUDA_TRY(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
  regen_threshold = threshold;
  if (queue_slots != queue_req) {
    queue_req = queue_slots;
    int st = alloc_paths(err);
    if (st != ILLUME_OK) return st;
    if (s_orig.get() && (st = ensure_shadow(err)) != ILLUME_OK) return st;
  }
  point();
  return ILLUME_OK;
}

int Engine::set_trace_variant(int variant) {
  if (variant == knobs.trace_variant) return ILLUME_OK;
  drop_graphs();
  knobs.trace_variant = variant;
  grid_trace = kernel_grid_blocks(trace_kernel_ptr(knobs.bvh_kind, knobs.trace_variant), 128, ctx->device);
  return ILLUME_OK;
}

int Engine::write_row(int r) {
  ILLUME_CUDA_TRY(cudaMemcpyAsync(jobs.as<JobDesc>() + r, &mirror[r], sizeof(JobDesc), cudaMemcpyHostToDevice,
                                  stream));
  return ILLUME_OK;
}

int Engine::write_pass_state(int r) {
  const size_t off = offsetof(JobDesc, sample_base);
  static_assert(offsetof(JobDesc, per_pass) == offsetof(JobDesc, sample_base) + 3 * sizeof(int), "pass state words");
  ILLUME_CUDA_TRY(cudaMemcpyAsync(reinterpret_cast<char*>(jobs.as<JobDesc>() + r) + off,
                                  reinterpret_cast<const char*>(&mirror[r]) + off, 4 * sizeof(int),
                                  cudaMemcpyHostToDevice, stream));
  return ILLUME_OK;
}

void Engine::advance_mirror() {
  for (JobDesc& J : mirror) {
    if (J.nsamples <= 0) continue;
    advance_pass_state(J.sample_base, J.nsamples, J.sample_end, J.per_pass, J.flags);
  }
}

long long Engine::paths_in_pass() const {
  long long n = 0;
  for (const JobDesc& J : mirror)
    if (J.nsamples > 0) n += (long long)J.nsamples * J.npix;
  return n;
}

int Engine::free_rows() const {
  int n = 0;
  for (const JobDesc& J : mirror) n += J.nsamples <= 0;
  return n;
}

// One iteration of the regeneration loop: the stages read the iteration from the
// counters (bounce -1), then the next batch of new paths.
void Engine::launch_iteration(cudaStream_t st, cudaGraphConditionalHandle cond, bool use_cond, int depth, bool nee) {
  launch_trace(w, knobs, -1, grid_trace, st);
  launch_shade(w, knobs, -1, nee ? grid_shade_nee : grid_shade, st, nee);
  if (nee) launch_shadow(w, knobs, -1, grid_shadow, st);
  launch_regen_plan(w, cond, use_cond, depth, regen_threshold, st);
  launch_regen(w, grid_raygen, st);
}

// Everything of a pass before the accumulation. Without regeneration: camera rays for
// every path, then depth x (trace, shade); with it: the first batch of paths, then a
// while node that iterates until every path has ended (called inside a capture).
int Engine::launch_head(cudaStream_t st, int depth, bool nee) {
  launch_plan(w, st);
  if (regen) {
    launch_regen_start(w, st);
    launch_regen(w, grid_raygen, st);
    return capture_while(st, side, [&](cudaGraphConditionalHandle cond) {
      launch_iteration(side, cond, true, depth, nee);
    });
  }
  launch_raygen(w, grid_raygen, st);
  for (int b = 0; b < depth; ++b) {
    launch_trace(w, knobs, b, grid_trace, st);
    launch_shade(w, knobs, b, nee ? grid_shade_nee : grid_shade, st, nee);
    if (nee) launch_shadow(w, knobs, b, grid_shadow, st);
  }
  return ILLUME_OK;
}

int Engine::launch_pass(cudaStream_t st, int depth, bool nee) {
  const int s = launch_head(st, depth, nee);
  if (s != ILLUME_OK) return s;
  launch_accumulate(w, grid_acc, st);
  launch_advance(w, st);
  return ILLUME_OK;
}

int Engine::run_interleaved(int depth, cudaEvent_t wait_ev, cudaEvent_t record_ev) {
  if (paths_in_pass() > cap) {
    set_error("job table needs more path slots than the engine has");
    return ILLUME_ERR_INVALID;
  }
  const bool nee = any_nee();
  if (nee) {
    std::string err;
    const int s = ensure_shadow(&err);
    if (s != ILLUME_OK) { set_error(err); return s; }
  }
  const int key = 2 * depth + (nee ? 1 : 0);
  auto it = head_graphs.find(key);
  if (it == head_graphs.end()) {
    cudaGraphExec_t exec = nullptr;
    const int s = capture(stream, &exec, [&] { return launch_head(stream, depth, nee); });
    if (s != ILLUME_OK) return s;
    it = head_graphs.emplace(key, exec).first;
  }
  if (!acc_graph) {
    const int s = capture(stream, &acc_graph, [&] {
      launch_accumulate(w, grid_acc, stream);
      launch_advance(w, stream);
      return ILLUME_OK;
    });
    if (s != ILLUME_OK) return s;
  }
  ILLUME_CUDA_TRY(cudaGraphLaunch(it->second, stream));
  if (wait_ev) ILLUME_CUDA_TRY(cudaStreamWaitEvent(stream, wait_ev, 0));
  ILLUME_CUDA_TRY(cudaGraphLaunch(acc_graph, stream));
  if (record_ev) ILLUME_CUDA_TRY(cudaEventRecord(record_ev, stream));
  advance_mirror();
  passes += 1;
  if (!regen) {
    launches += launches_per_pass(depth, nee);
    ctx->launches += launches_per_pass(depth, nee);
  }
  return ILLUME_OK;
}

int Engine::run(int npasses, int depth) {
  if (npasses <= 0) return ILLUME_OK;
  if (paths_in_pass() > cap) {
    set_error("job table needs more path slots than the engine has");
    return ILLUME_ERR_INVALID;
  }
  cudaStream_t st = stream;
  const bool nee = any_nee();
  if (nee) {
    std::string err;
    const int s = ensure_shadow(&err);
    if (s != ILLUME_OK) { set_error(err); return s; }
  }
  const int key = 2 * depth + (nee ? 1 : 0);
  auto it = graphs.find(key);
  if (it == graphs.end()) {
    cudaGraphExec_t exec = nullptr;
    const int s = capture(st, &exec, [&] { return launch_pass(st, depth, nee); });
    if (s != ILLUME_OK) return s;
    it = graphs.emplace(key, exec).first;
  }
  for (int i = 0; i < npasses; ++i) {
    ILLUME_CUDA_TRY(cudaGraphLaunch(it->second, st));
    advance_mirror();
  }
  passes += npasses;
  if (!regen) {
    launches += (long long)npasses * launches_per_pass(depth, nee);
    ctx->launches += (long long)npasses * launches_per_pass(depth, nee);
  }
  return ILLUME_OK;
}

int Engine::run_profiled(int depth, bool count_visits, std::vector<cudaEvent_t>& ev, int* iterations) {
  if (paths_in_pass() > cap) {
    set_error("job table needs more path slots than the engine has");
    return ILLUME_ERR_INVALID;
  }
  cudaStream_t st = stream;
  const bool nee = any_nee();
  if (nee) {
    std::string err;
    const int s = ensure_shadow(&err);
    if (s != ILLUME_OK) { set_error(err); return s; }
  }
  auto event = [&]() -> cudaError_t {
    ev.emplace_back();
    const cudaError_t e = cudaEventCreate(&ev.back());
    return e == cudaSuccess ? cudaEventRecord(ev.back(), st) : e;
  };
  ev.clear();
  int n = 0;
  long long nl = 0;
  ILLUME_CUDA_TRY(event());
  launch_plan(w, st);
  if (regen) {
    launch_regen_start(w, st);
    launch_regen(w, grid_raygen, st);
  } else {
    launch_raygen(w, grid_raygen, st);
  }
  ILLUME_CUDA_TRY(event());
  nl += regen ? 3 : 2;   // plan, then the first batch's slots and camera rays, or every camera ray
  for (int b = 0;; ++b) {
    if (!regen && b >= depth) break;
    launch_trace(w, knobs, regen ? -1 : b, grid_trace, st, count_visits);
    ILLUME_CUDA_TRY(event());
    launch_shade(w, knobs, regen ? -1 : b, nee ? grid_shade_nee : grid_shade, st, nee);
    if (nee) launch_shadow(w, knobs, regen ? -1 : b, grid_shadow, st);
    ILLUME_CUDA_TRY(event());
    nl += nee ? 3 : 2;
    ++n;
    if (regen) {
      // the loop's next batch and condition, read back on the host
      launch_regen_plan(w, 0, false, depth, regen_threshold, st);
      launch_regen(w, grid_raygen, st);
      nl += 2;
      int more = 0;
      ILLUME_CUDA_TRY(cudaMemcpyAsync(&more, w.counters + kCounterMore, sizeof(int), cudaMemcpyDeviceToHost, st));
      ILLUME_CUDA_TRY(cudaStreamSynchronize(st));
      if (!more) break;
    }
  }
  launch_accumulate(w, grid_acc, st);
  ILLUME_CUDA_TRY(event());
  launch_advance(w, st);
  nl += 3;
  ILLUME_CUDA_TRY(cudaGetLastError());
  advance_mirror();
  if (iterations) *iterations = n;
  passes += 1;
  launches += nl;
  ctx->launches += nl;
  return ILLUME_OK;
}

int Engine::read_row_rays(int r, unsigned long long* out) {
  ILLUME_CUDA_TRY(cudaMemcpyAsync(out, reinterpret_cast<const char*>(jobs.as<JobDesc>() + r) + offsetof(JobDesc, rays),
                                  sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream));
  ILLUME_CUDA_TRY(cudaStreamSynchronize(stream));
  return ILLUME_OK;
}

size_t Engine::device_bytes() const {
  size_t b = 0;
  const DevBuffer* all[] = {&q_orig[0], &q_orig[1], &q_dir[0], &q_dir[1], &q_thr[0], &q_thr[1], &q_bounce[0],
                            &q_bounce[1], &hit, &hit_geom, &evq, &counters, &contrib, &rays, &visits, &jobs,
                            &path_base, &pixel_base, &s_orig, &s_dir, &s_val};
  for (const DevBuffer* d : all) b += d->size();
  return b;
}

}  // namespace illume
