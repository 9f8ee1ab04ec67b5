#include "server.h"
#include "handles.h"

#include <string.h>

#include <algorithm>
#include <chrono>

#include "../../../include/illume.h"

namespace illume {

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int Server::chunk_for(const illume_render_params& p) {
  const long long npix = (long long)p.width * p.height;
  const long long target = 1LL << 21;
  return (int)std::max(1LL, std::min<long long>(std::max(p.spp, 1), target / std::max(npix, 1LL)));
}

// Device bytes a job holds while running: wavefront queues for one chunk of samples plus
// the per-pixel accumulators and output staging (the layout Renderer::init allocates).
size_t Server::footprint(const illume_render_params& p, int chunk) {
  const size_t npix = (size_t)p.width * p.height;
  const size_t paths = npix * (size_t)chunk;
  const size_t per_path = 6 * 16 + 16 + 4 + 4 * EV_COUNT + 16;
  const size_t per_pixel = (p.accum_mode == ACCUM_FP64 ? 24 : (p.accum_mode == ACCUM_KAHAN ? 24 : 12)) + 24 + 12 + 3;
  return paths * per_path + npix * per_pixel + 4096;
}

int Server::submit(Scene* scene, const illume_render_params& p, int64_t* id) {
  const int chunk = chunk_for(p);
  const size_t fp = footprint(p, chunk);
  if (budget && fp > budget) {
    set_error("job footprint " + std::to_string(fp) + " bytes exceeds the server budget");
    return ILLUME_ERR_BUDGET;
  }
  std::unique_ptr<ServerJob> j(new ServerJob);
  j->id = next_id++;
  j->scene = scene;
  j->params = p;
  j->params.samples_per_pass = chunk;
  j->footprint = fp;
  j->submit_ms = now_ms();
  *id = j->id;
  queue.push_back(j->id);
  jobs[j->id] = std::move(j);
  return ILLUME_OK;
}

int Server::step(int* running_out) {
  // admission: FIFO while the budget and the slot count allow
  int running = 0;
  for (auto& kv : jobs) running += kv.second->state == 1;
  while (!queue.empty()) {
    ServerJob* j = jobs[queue.front()].get();
    if (j->state == 3) { queue.pop_front(); continue; }
    if (running >= max_in_flight || (budget && reserved + j->footprint > budget)) break;
    queue.pop_front();
    j->r.reset(new Renderer);
    j->r->ctx = ctx;
    j->r->scene = j->scene;
    j->r->p = j->params;
    std::string err;
    const int st = j->r->init(&err);
    if (st != ILLUME_OK) {
      j->state = 4;
      j->error = err;
      j->r.reset();
      continue;
    }
    reserved += j->footprint;
    j->state = 1;
    j->start_ms = now_ms();
    ++running;
  }
  // one progressive chunk of every running job
  for (auto& kv : jobs) {
    ServerJob* j = kv.second.get();
    if (j->state != 1) continue;
    const int left = j->params.spp - j->spp_done;
    j->r->p.spp = std::min(left, j->params.samples_per_pass);
    illume_render_stats s{};
    const int st = j->r->render_device(j->spp_done > 0, &s);
    if (st != ILLUME_OK) {
      j->state = 4;
      j->error = last_error();
      reserved -= j->footprint;
      j->r.reset();
      continue;
    }
    j->spp_done += j->r->p.spp;
    j->stats.rays += s.rays;
    j->stats.paths += s.paths;
    j->stats.render_ms += s.render_ms;
    j->stats.kernel_launches += s.kernel_launches;
    if (j->spp_done >= j->params.spp) {
      const size_t n = 3 * (size_t)j->r->npix;
      j->mean.resize(n);
      j->rgb8.resize(n);
      j->r->p.spp = j->params.spp;
      const int rs = j->r->read(j->mean.data(), nullptr, nullptr, j->rgb8.data());
      j->state = rs == ILLUME_OK ? 2 : 4;
      j->finish_ms = now_ms();
      j->stats.total_ms = j->finish_ms - j->submit_ms;
      reserved -= j->footprint;
      j->r.reset();
    }
  }
  running = 0;
  for (auto& kv : jobs) running += kv.second->state == 1;
  if (running_out) *running_out = running + (int)queue.size();
  return ILLUME_OK;
}

int Server::poll(int64_t id, float* mean, uint8_t* rgb8, illume_render_stats* stats) {
  auto it = jobs.find(id);
  if (it == jobs.end()) { set_error("unknown job"); return ILLUME_ERR_INVALID; }
  ServerJob* j = it->second.get();
  if (j->state == 3) { set_error("job cancelled"); return ILLUME_ERR_CANCELLED; }
  if (j->state == 4) { set_error(j->error); return ILLUME_ERR_CUDA; }
  if (j->state != 2) return ILLUME_ERR_NOT_READY;
  if (mean) memcpy(mean, j->mean.data(), sizeof(float) * j->mean.size());
  if (rgb8) memcpy(rgb8, j->rgb8.data(), j->rgb8.size());
  if (stats) *stats = j->stats;
  return ILLUME_OK;
}

int Server::cancel(int64_t id) {
  auto it = jobs.find(id);
  if (it == jobs.end()) { set_error("unknown job"); return ILLUME_ERR_INVALID; }
  ServerJob* j = it->second.get();
  if (j->state == 1) {
    cudaStreamSynchronize(ctx->stream);
    reserved -= j->footprint;
    j->r.reset();
  }
  if (j->state <= 1) j->state = 3;
  return ILLUME_OK;
}

}  // namespace illume

// ---- C-ABI ----
extern "C" {

int illume_server_create(illume_context* ctx, size_t hbm_budget_bytes, int max_jobs_in_flight, illume_server** out) {
  if (!ctx || !out) { illume::set_error("null argument"); return ILLUME_ERR_INVALID; }
  illume_server* s = new illume_server;
  s->s.ctx = &ctx->c;
  s->s.budget = hbm_budget_bytes;
  s->s.max_in_flight = max_jobs_in_flight > 0 ? max_jobs_in_flight : 8;
  *out = s;
  return ILLUME_OK;
}

int illume_server_destroy(illume_server* s) {
  if (!s) return ILLUME_OK;
  if (s->s.ctx) cudaStreamSynchronize(s->s.ctx->stream);
  delete s;
  return ILLUME_OK;
}

int illume_job_submit(illume_server* s, illume_scene* scene, const illume_render_params* params, illume_job_id* out) {
  if (!s || !scene || !params || !out) { illume::set_error("null argument"); return ILLUME_ERR_INVALID; }
  return s->s.submit(&scene->s, *params, out);
}

int illume_server_step(illume_server* s, int* jobs_running) {
  if (!s) { illume::set_error("null server"); return ILLUME_ERR_INVALID; }
  return s->s.step(jobs_running);
}

int illume_job_poll(illume_server* s, illume_job_id id, float* out_mean, uint8_t* out_rgb8, illume_render_stats* stats) {
  if (!s) { illume::set_error("null server"); return ILLUME_ERR_INVALID; }
  return s->s.poll(id, out_mean, out_rgb8, stats);
}

int illume_job_cancel(illume_server* s, illume_job_id id) {
  if (!s) { illume::set_error("null server"); return ILLUME_ERR_INVALID; }
  return s->s.cancel(id);
}

}  // extern "C"
