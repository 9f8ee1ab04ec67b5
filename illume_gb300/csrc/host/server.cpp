#include "server.h"
#include "handles.h"

#include <stddef.h>
#include <string.h>

#include <algorithm>
#include <chrono>

#include "../../../include/illume.h"

namespace illume {

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

static constexpr size_t kBytesPerPath = 6 * sizeof(float4) + sizeof(float4) + sizeof(int) + EV_COUNT * sizeof(int) +
                                        sizeof(float4);

static int engine_key(const illume_render_params& p) { return p.intersector * 16 + p.bvh_kind; }
static constexpr int kMaxLanes = 16;

LaneStream::~LaneStream() {
  if (stream) {
    cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
  }
  if (done) cudaEventDestroy(done);
}

Server::~Server() {
  if (ctx) cudaStreamSynchronize(ctx->stream);
  engines.clear();
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
}

// A job table of `cap` path slots for the trace-kernel setting of `p`, on a new stream.
int Server::new_engine(const illume_render_params& p, int key, long long cap, ServerEngine** out) {
  ServerEngine se;
  se.lane = std::make_shared<LaneStream>();
  ILLUME_CUDA_TRY(cudaStreamCreateWithFlags(&se.lane->stream, cudaStreamNonBlocking));
  ILLUME_CUDA_TRY(cudaEventCreateWithFlags(&se.lane->done, cudaEventDisableTiming));
  se.eng.reset(new Engine);
  se.eng->stream = se.lane->stream;
  se.base_key = key / kMaxLanes;
  RenderKnobs k = render_knobs(p);
  k.trace_variant = trace_variant >= 0 ? trace_variant : (p.bvh_kind == 2 ? 1 : 0);
  k.shade_variant = 0;
  std::string err;
  const int st = se.eng->init(ctx, rows, (int)cap, k, &err, queue_slots, regen_threshold);
  if (st != ILLUME_OK) { set_error(err); return st; }
  // a table that joins a tuned setting takes the tuned candidate
  auto tit = tuners.find(se.base_key);
  if (tit != tuners.end() && tit->second.state == 2) {
    for (const auto& kv : engines)
      if (kv.second.base_key == se.base_key) {
        se.eng->set_trace_variant(kv.second.eng->knobs.trace_variant);
        if (se.eng->set_regen(kv.second.eng->queue_req, kv.second.eng->regen_threshold, &err) != ILLUME_OK) {
          set_error(err);
          return ILLUME_ERR_CUDA;
        }
        break;
      }
  }
  se.row_job.assign(rows, 0);
  *out = &engines.emplace(key, std::move(se)).first->second;
  return ILLUME_OK;
}

// Device bytes a running job holds: its accumulators and output staging.
size_t Server::footprint(const illume_render_params& p) {
  const size_t npix = (size_t)p.width * p.height;
  const size_t acc = p.accum_mode == ACCUM_FP32 ? 12 : 24;
  return npix * (acc + 12 + 3) + 4096;
}

size_t Server::engines_bytes() const {
  size_t b = 0;
  for (const auto& kv : engines) b += kv.second.eng->device_bytes();
  return b;
}

int Server::submit(Scene* scene, const illume_render_params& p, int64_t* id) {
  std::string err;
  int st = check_render_params(p, *scene, &err);
  if (st != ILLUME_OK) { set_error(err); return st; }
  const size_t fp = footprint(p);
  const size_t min_engine = (size_t)std::max<long long>((long long)p.width * p.height, 1) * kBytesPerPath;
  if (budget && fp + min_engine + (1 << 20) > budget) {
    set_error("job footprint " + std::to_string(fp + min_engine) + " bytes exceeds the server budget");
    return ILLUME_ERR_BUDGET;
  }
  std::unique_ptr<ServerJob> j(new ServerJob);
  j->id = next_id++;
  j->scene = scene;
  j->params = p;
  if (p.camera) {
    memcpy(j->camera, p.camera, sizeof(j->camera));
    j->params.camera = j->camera;
  }
  j->footprint = fp;
  j->submit_ms = now_ms();
  *id = j->id;
  queue.push_back(j->id);
  jobs[j->id] = std::move(j);
  return ILLUME_OK;
}

// Admits queued jobs in arrival order while a table row and the job's footprint fit
// (compose decides which admitted jobs run in each pass); a job that does not fit yet
// keeps its place and later jobs may pass it.
int Server::admit() {
  if (budget && !queue.empty()) {
    // under a budget, idle tables give their memory back to the queue
    for (auto eit = engines.begin(); eit != engines.end();) {
      bool idle = true;
      for (int64_t id : eit->second.row_job) idle &= id == 0;
      if (idle) eit = engines.erase(eit);
      else ++eit;
    }
  }
  for (auto it = queue.begin(); it != queue.end();) {
    ServerJob* j = jobs[*it].get();
    if (j->state == 3) { it = queue.erase(it); continue; }
    const illume_render_params& p = j->params;
    const int npix = p.width * p.height;
    const int base = engine_key(p);
    // the table of this setting with a free row and the least work to go; a table not
    // created yet when every existing one has work (or there is none)
    ServerEngine* pick = nullptr;
    int key = -1, missing = -1, existing = 0;
    double least = 0.0;
    for (int lane = 0; lane < lanes; ++lane) {
      auto eit = engines.find(base * kMaxLanes + lane);
      if (eit == engines.end()) {
        if (missing < 0) missing = lane;
        continue;
      }
      ServerEngine& c = eit->second;
      ++existing;
      bool free_row = false;
      double work = 0.0;
      for (int r = 0; r < c.eng->rows; ++r) {
        if (!c.row_job[r]) { free_row = true; continue; }
        const JobDesc& J = c.eng->mirror[r];
        work += (double)J.npix * std::max(J.sample_end - J.sample_base, 0);
      }
      if (free_row && (!pick || work < least)) {
        pick = &c;
        key = eit->first;
        least = work;
      }
    }
    if ((!pick || least > 0.0) && missing >= 0) {
      long long cap = std::max(path_capacity, npix);
      auto tit = tuners.find(base);
      if (tit != tuners.end() && tit->second.state == 2) {
        for (const auto& kv : engines)
          if (kv.second.base_key == base) cap = std::max<long long>(kv.second.eng->cap, npix);
      }
      if (budget) {
        const long long used = (long long)(reserved + engines_bytes() + j->footprint + (1 << 20));
        const long long affordable = ((long long)budget - used) / (long long)kBytesPerPath;
        cap = std::min(cap, affordable);
      }
      if (cap >= npix) {
        const int st = new_engine(p, base * kMaxLanes + missing, cap, &pick);
        if (st == ILLUME_OK) {
          key = base * kMaxLanes + missing;
        } else if ((st == ILLUME_ERR_OOM || st == ILLUME_ERR_BUDGET) && existing > 0) {
          // the device has no room for another table: the setting's existing tables
          // take the job (now, or when a row frees up)
          cudaGetLastError();
        } else {
          return st;
        }
      }
    }
    if (!pick) { ++it; continue; }
    ServerEngine& se = *pick;
    Engine& e = *se.eng;
    int running = 0;
    int free_row = -1;
    for (int r = 0; r < e.rows; ++r) {
      if (se.row_job[r]) ++running;
      else if (free_row < 0) free_row = r;
    }
    if (free_row < 0) { ++it; continue; }
    if (npix > e.cap) {
      if (running) { ++it; continue; }
      if (budget && reserved + engines_bytes() + ((size_t)npix - e.cap) * kBytesPerPath + j->footprint > budget) {
        ++it;
        continue;
      }
      std::string err;
      const int st = e.resize(npix, &err);
      if (st != ILLUME_OK) { set_error(err); return st; }
    }
    if (budget && reserved + engines_bytes() + j->footprint > budget) { ++it; continue; }
    // job buffers
    int st;
    const size_t n3 = 3 * (size_t)npix;
    Accumulators acc{};
    if (p.accum_mode == ACCUM_FP64) { if ((st = j->sum64.alloc(ctx, sizeof(double) * n3)) != ILLUME_OK) return st; }
    else if ((st = j->sum32.alloc(ctx, sizeof(float) * n3)) != ILLUME_OK) return st;
    if (p.accum_mode == ACCUM_KAHAN && (st = j->comp32.alloc(ctx, sizeof(float) * n3)) != ILLUME_OK) return st;
    if ((st = j->out_mean.alloc(ctx, sizeof(float) * n3)) != ILLUME_OK) return st;
    if ((st = j->out_rgb8.alloc(ctx, n3)) != ILLUME_OK) return st;
    acc.sum32 = j->sum32.as<float>();
    acc.comp32 = j->comp32.as<float>();
    acc.sum64 = j->sum64.as<double>();
    acc.sumsq = nullptr;
    launch_clear_accumulators(acc, npix, ctx->stream);
    JobDesc row = job_row(*j->scene, p, acc);
    row.sample_base = p.sample_begin;
    row.sample_end = p.sample_begin + p.spp;
    row.per_pass = 1;
    row.nsamples = p.spp > 0 ? 1 : 0;
    e.mirror[free_row] = row;
    if ((st = e.write_row(free_row)) != ILLUME_OK) return st;
    se.row_job[free_row] = j->id;
    j->key = key;
    j->row = free_row;
    j->state = 1;
    j->start_ms = now_ms();
    reserved += j->footprint;
    it = queue.erase(it);
  }
  return ILLUME_OK;
}

// Splits `cap` path slots between jobs of npix[i] pixels with left[i] samples to go:
// one sample of every pixel each (the caller guarantees that these fit), then the rest
// in equal shares, repeatedly, capped by each job's remaining samples.
void plan_shares(const std::vector<long long>& npix, const std::vector<int>& left, long long cap,
                 std::vector<int>* out) {
  const size_t n = npix.size();
  std::vector<int>& pp = *out;
  pp.assign(n, 1);
  long long R = cap;
  for (size_t i = 0; i < n; ++i) R -= npix[i];
  for (int iter = 0; iter < 64 && R > 0; ++iter) {
    int want = 0;
    for (size_t i = 0; i < n; ++i) want += pp[i] < left[i] && npix[i] <= R;
    if (!want) break;
    const long long share = R / want;
    bool progress = false;
    for (size_t i = 0; i < n; ++i) {
      if (pp[i] >= left[i] || npix[i] > R) continue;
      const long long add = std::min<long long>(std::max<long long>(share / npix[i], 1), left[i] - pp[i]);
      if (add * npix[i] > R) continue;
      pp[i] += (int)add;
      R -= add * npix[i];
      progress = true;
    }
    if (!progress) break;
  }
}

// Chooses the jobs of the next passes and splits the path slots between them.
//
// Running jobs are grouped by scene, because a pass whose rays traverse one scene's BVH
// keeps it in L2 while rays of many scenes evict each other. Groups enter the pass in
// order of their smallest remaining job (remaining paths = pixels x samples to go), so
// short requests finish first; a group enters while its jobs' one-sample minimum fits
// the slots and either the traversal data of the groups taken so far plus its own stays
// within three quarters of L2, or the pass is less than half full. Jobs left out are
// paused for these passes (no samples); the chosen ones share the slots by water-filling.
void Server::compose(ServerEngine& se) {
  Engine& e = *se.eng;
  struct Group {
    Scene* scene;
    double key;
    std::vector<int> rows;
  };
  std::vector<Group> groups;
  std::map<Scene*, size_t> index;
  for (int r = 0; r < e.rows; ++r) {
    if (!se.row_job[r]) continue;
    const JobDesc& J = e.mirror[r];
    if (J.sample_base >= J.sample_end) continue;
    ServerJob* j = jobs[se.row_job[r]].get();
    auto it = index.find(j->scene);
    if (it == index.end()) {
      it = index.emplace(j->scene, groups.size()).first;
      groups.push_back(Group{j->scene, 1e300, {}});
    }
    Group& g = groups[it->second];
    g.key = std::min(g.key, (double)J.npix * (double)(J.sample_end - J.sample_base));
    g.rows.push_back(r);
  }
  std::stable_sort(groups.begin(), groups.end(), [](const Group& a, const Group& b) { return a.key < b.key; });
  const size_t l2_target = ctx->l2_bytes > 0 ? (size_t)ctx->l2_bytes * 3 / 4 : ((size_t)96 << 20);
  const int kind = e.knobs.bvh_kind == BVH_WIDE8 ? 1 : (e.knobs.bvh_kind == BVH_WIDE4 ? 2 : 0);
  std::vector<char> chosen(e.rows, 0);
  long long paths = 0;
  size_t bytes = 0;
  bool any = false;
  for (Group& g : groups) {
    const size_t gb = g.scene->trace_bytes[kind];
    if (any && bytes + gb > l2_target && 2 * paths >= e.cap) continue;
    // the group's jobs, smallest remaining work first, while one sample of each fits
    std::stable_sort(g.rows.begin(), g.rows.end(), [&](int a, int b) {
      const JobDesc &A = e.mirror[a], &B = e.mirror[b];
      return (double)A.npix * (A.sample_end - A.sample_base) < (double)B.npix * (B.sample_end - B.sample_base);
    });
    bool took = false;
    for (int r : g.rows) {
      if (paths + e.mirror[r].npix > e.cap) continue;
      chosen[r] = 1;
      paths += e.mirror[r].npix;
      took = true;
    }
    if (took) {
      any = true;
      bytes += gb;
    }
  }
  std::vector<int> live, left, pp;
  std::vector<long long> npix;
  for (int r = 0; r < e.rows; ++r) {
    if (!chosen[r]) continue;
    const JobDesc& J = e.mirror[r];
    live.push_back(r);
    npix.push_back(J.npix);
    left.push_back(J.sample_end - J.sample_base);
  }
  plan_shares(npix, left, e.cap, &pp);
  std::vector<int> want_pp(e.rows, -1);
  for (size_t i = 0; i < live.size(); ++i) want_pp[live[i]] = pp[i];
  for (int r = 0; r < e.rows; ++r) {
    if (!se.row_job[r]) continue;
    JobDesc& J = e.mirror[r];
    const int per = want_pp[r] > 0 ? want_pp[r] : J.per_pass;
    const int ns = want_pp[r] > 0 ? std::min(want_pp[r], J.sample_end - J.sample_base) : 0;
    if (J.per_pass != per || J.nsamples != ns) {
      J.per_pass = per;
      J.nsamples = ns;
      e.write_pass_state(r);
    }
  }
}

// Jobs that have all their samples: tonemap, copy out, free the row and the buffers.
int Server::retire(ServerEngine& se, std::vector<ServerJob*>* done) {
  Engine& e = *se.eng;
  cudaStream_t st = ctx->stream;
  // every finished job's tonemap and copies first, one wait for all of them
  std::vector<int> rows_done;
  std::vector<unsigned long long> rays;
  for (int r = 0; r < e.rows; ++r)
    if (se.row_job[r] && e.mirror[r].sample_base >= e.mirror[r].sample_end) rows_done.push_back(r);
  if (rows_done.empty()) return ILLUME_OK;
  rays.assign(rows_done.size(), 0);
  for (size_t k = 0; k < rows_done.size(); ++k) {
    const int r = rows_done[k];
    ServerJob* j = jobs[se.row_job[r]].get();
    const illume_render_params& p = j->params;
    const int npix = p.width * p.height;
    Accumulators acc{};
    acc.sum32 = j->sum32.as<float>();
    acc.comp32 = j->comp32.as<float>();
    acc.sum64 = j->sum64.as<double>();
    launch_tonemap(acc, p.accum_mode, npix, (float)std::max(p.spp, 1), p.tonemapper, j->out_rgb8.as<uint8_t>(),
                   j->out_mean.as<float>(), st);
    ILLUME_CUDA_TRY(cudaGetLastError());
    j->mean.resize(3 * (size_t)npix);
    j->rgb8.resize(3 * (size_t)npix);
    ILLUME_CUDA_TRY(cudaMemcpyAsync(j->mean.data(), j->out_mean.get(), sizeof(float) * j->mean.size(),
                                    cudaMemcpyDeviceToHost, st));
    ILLUME_CUDA_TRY(cudaMemcpyAsync(j->rgb8.data(), j->out_rgb8.get(), j->rgb8.size(), cudaMemcpyDeviceToHost, st));
    ILLUME_CUDA_TRY(cudaMemcpyAsync(&rays[k], reinterpret_cast<const char*>(e.w.jobs + r) + offsetof(JobDesc, rays), 8,
                                    cudaMemcpyDeviceToHost, st));
  }
  // the table's traversal-overflow flag (kept across passes): every job it retires from
  // then on reports it
  int drops = 0;
  ILLUME_CUDA_TRY(cudaMemcpyAsync(&drops, e.w.counters + kCounterStackDrops, sizeof(int), cudaMemcpyDeviceToHost, st));
  ILLUME_CUDA_TRY(cudaStreamSynchronize(st));
  for (size_t k = 0; k < rows_done.size(); ++k) {
    const int r = rows_done[k];
    ServerJob* j = jobs[se.row_job[r]].get();
    const illume_render_params& p = j->params;
    j->stats.rays = (int64_t)rays[k];
    j->stats.paths = (int64_t)p.spp * p.width * p.height;
    j->stats.d2h_bytes = (int64_t)(j->mean.size() * sizeof(float) + j->rgb8.size());
    if (drops)
      j->error = "a BVH traversal stack of the job's table overflowed: the image is written, but rays may have "
                 "missed hits";
    j->sum32.release();
    j->comp32.release();
    j->sum64.release();
    j->out_mean.release();
    j->out_rgb8.release();
    reserved -= j->footprint;
    se.row_job[r] = 0;
    e.mirror[r] = JobDesc{};
    j->row = -1;
    j->state = 2;
    done->push_back(j);
  }
  return ILLUME_OK;
}

// Applies candidate `idx` (path slots per table, trace kernel variant, path
// regeneration) to every table of a trace-kernel setting; fails without change if a
// running job does not fit the slots.
int Server::apply_candidate(int base_key, int idx) {
  const Tuner& t = tuners[base_key];
  const Tuner::Candidate& c = t.candidates[idx];
  const int cap = c.cap;
  for (const auto& kv : engines) {
    if (kv.second.base_key != base_key) continue;
    for (int r = 0; r < kv.second.eng->rows; ++r)
      if (kv.second.row_job[r] && kv.second.eng->mirror[r].npix > cap) return ILLUME_ERR_INVALID;
  }
  for (auto& kv : engines) {
    if (kv.second.base_key != base_key) continue;
    Engine& e = *kv.second.eng;
    std::string err;
    int st = e.resize(cap, &err);
    if (st != ILLUME_OK) { set_error(err); return st; }
    if ((st = e.set_regen(c.queue_slots, c.threshold, &err)) != ILLUME_OK) { set_error(err); return st; }
    if ((st = e.set_trace_variant(c.variant)) != ILLUME_OK) return st;
  }
  return ILLUME_OK;
}

// Online autotuner of one trace-kernel setting: every candidate runs a window of steps
// on the live jobs; the rate of the window's steps after the first (rays of the
// setting's tables per device ms of the step) decides.
void Server::tune(int base_key, double rays, double ms) {
  static constexpr int kWindow = 3;
  Tuner& t = tuners[base_key];
  if (t.state == 0) {
    int kind = BVH_BINARY, ntables = 0, current = 0;
    size_t held = 0;
    for (const auto& kv : engines)
      if (kv.second.base_key == base_key) {
        kind = kv.second.eng->knobs.bvh_kind;
        held += kv.second.eng->device_bytes();
        current = std::max(current, kv.second.eng->cap);
        ++ntables;
      }
    // binary BVH: the default kernel and its while-while form; 8-wide: both kernels;
    // 4-wide: the traversal stack in local memory or partly in shared memory
    const std::vector<int> variants = kind == BVH_BINARY ? std::vector<int>{0, 3} : std::vector<int>{0, 1};
    // the tables' present size first: its windows need no reallocation
    const int other = current == (1 << 24) ? 1 << 25 : 1 << 24;
    const int first = current == (1 << 24) ? 1 << 24 : 1 << 25;
    for (int cap : {first, other}) {
      if (budget && reserved + engines_bytes() - held + (size_t)ntables * cap * kBytesPerPath > budget) continue;
      for (int v : variants) t.candidates.push_back({cap, v, queue_slots, regen_threshold});
    }
    // path regeneration at the first size: a quarter of the slots in flight, refilled
    // every iteration or once the queue is down to a quarter (fewer bytes than the
    // candidates above, so no budget check)
    if (queue_slots == 0)
      for (float thr : {1.0f, 0.25f}) t.candidates.push_back({first, variants[0], first / 4, thr});
    t.rate.assign(t.candidates.size(), 0.0);
    t.state = 1;
    t.idx = -1;
  } else {
    ++t.steps;
    if (t.steps > 1) { t.rays += rays; t.ms += ms; }
    if (t.steps < kWindow) return;
    t.rate[t.idx] = t.ms > 0 ? t.rays / t.ms : 0.0;
  }
  // next candidate that fits the running jobs
  for (++t.idx; t.idx < (int)t.candidates.size(); ++t.idx)
    if (apply_candidate(base_key, t.idx) == ILLUME_OK) break;
  if (t.idx < (int)t.candidates.size()) {
    t.rays = t.ms = 0;
    t.steps = 0;
    return;
  }
  int best = -1;
  for (size_t i = 0; i < t.rate.size(); ++i)
    if (t.rate[i] > 0 && (best < 0 || t.rate[i] > t.rate[best])) best = (int)i;
  if (best >= 0) apply_candidate(base_key, best);
  t.state = 2;
}

// Waits for the passes the last step launched, then retires the jobs they finished and
// feeds the autotuner.
int Server::finish_in_flight(std::vector<ServerJob*>* done) {
  if (in_flight.empty()) return ILLUME_OK;
  for (Launched& l : in_flight) {
    ILLUME_CUDA_TRY(cudaMemcpyAsync(&l.total, l.se->eng->w.rays, 8, cudaMemcpyDeviceToHost, ctx->stream));
    ILLUME_CUDA_TRY(cudaMemcpyAsync(&l.iter_total, l.se->eng->w.counters + kCounterIterTotal, sizeof(int),
                                    cudaMemcpyDeviceToHost, ctx->stream));
  }
  ILLUME_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, ev0, ev1);
  totals.device_ms += ms;
  std::map<int, double> rays_by_key;
  int st;
  for (Launched& l : in_flight) {
    const double rays = (double)(l.total - l.se->rays_seen);
    l.se->rays_seen = l.total;
    if (l.se->eng->regen) {
      // launches of the regeneration loops, known once the passes are done
      const long long iters = (long long)l.iter_total - l.se->iters_seen;
      const long long nl = Engine::launches_regen(l.k, iters, false);
      totals.kernel_launches += nl;
      for (int r = 0; r < l.se->eng->rows; ++r)
        if (l.se->row_job[r]) jobs[l.se->row_job[r]]->stats.kernel_launches += nl;
    }
    l.se->iters_seen = l.iter_total;
    totals.rays += (int64_t)rays;
    rays_by_key[l.se->base_key] += rays;
    if ((st = retire(*l.se, done)) != ILLUME_OK) return st;
  }
  in_flight.clear();
  if (autotune)
    for (const auto& kr : rays_by_key)
      if (tuners[kr.first].state != 2) tune(kr.first, kr.second, ms);
  return ILLUME_OK;
}

// One scheduling round. The passes it launches run on while the caller does its own
// work; the next call waits for them before it admits, composes and launches again, so
// the device does not sit idle between rounds. A job whose last samples were in those
// passes is retired (its results readable by poll) by that next call.
int Server::step(int* running_out) {
  if (!ev0) {
    ILLUME_CUDA_TRY(cudaEventCreate(&ev0));
    ILLUME_CUDA_TRY(cudaEventCreate(&ev1));
  }
  std::vector<ServerJob*> done;
  int st = finish_in_flight(&done);
  if (st != ILLUME_OK) return st;
  if ((st = admit()) != ILLUME_OK) return st;
  // every table's passes are launched on its own stream, and none is waited for here
  ILLUME_CUDA_TRY(cudaEventRecord(ev0, ctx->stream));
  for (auto& kv : engines) {
    ServerEngine& se = kv.second;
    Engine& e = *se.eng;
    if ((st = retire(se, &done)) != ILLUME_OK) return st;   // jobs with no samples
    compose(se);
    int depth = 0, k = passes_per_step;
    std::vector<int> active;
    for (int r = 0; r < e.rows; ++r) {
      const JobDesc& J = e.mirror[r];
      if (!se.row_job[r] || J.nsamples <= 0) continue;
      active.push_back(r);
      depth = std::max(depth, J.max_depth);
      k = std::min(k, (J.sample_end - J.sample_base + J.per_pass - 1) / J.per_pass);
    }
    if (depth == 0 && e.paths_in_pass() == 0) continue;
    k = std::max(k, 1);
    // (under regeneration the launches are counted when the passes are done)
    const int per_pass_launches = e.regen ? 0 : Engine::launches_per_pass(depth, e.any_nee());
    ILLUME_CUDA_TRY(cudaStreamWaitEvent(e.stream, ev0, 0));   // after admission's clears
    if ((st = e.run(k, depth)) != ILLUME_OK) return st;
    ILLUME_CUDA_TRY(cudaEventRecord(se.lane->done, e.stream));
    ILLUME_CUDA_TRY(cudaStreamWaitEvent(ctx->stream, se.lane->done, 0));
    for (int r : active) jobs[se.row_job[r]]->stats.kernel_launches += (int64_t)k * per_pass_launches;
    totals.passes += k;
    totals.kernel_launches += (int64_t)k * per_pass_launches;
    in_flight.push_back({&se, k, 0, 0});
  }
  ILLUME_CUDA_TRY(cudaEventRecord(ev1, ctx->stream));
  const double t = now_ms();
  for (ServerJob* j : done) {
    j->finish_ms = t;
    j->stats.total_ms = t - j->submit_ms;
    j->stats.render_ms = t - j->start_ms;
    totals.jobs_done++;
  }
  int running = 0;
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
  if (!j->error.empty()) { set_error(j->error); return ILLUME_ERR_TRAVERSAL; }
  return ILLUME_OK;
}

int Server::cancel(int64_t id) {
  auto it = jobs.find(id);
  if (it == jobs.end()) { set_error("unknown job"); return ILLUME_ERR_INVALID; }
  ServerJob* j = it->second.get();
  if (j->state == 1) {
    ServerEngine& se = engines[j->key];
    se.eng->mirror[j->row].nsamples = 0;
    se.eng->write_pass_state(j->row);
    ILLUME_CUDA_TRY(cudaStreamSynchronize(se.eng->stream));
    ILLUME_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    se.row_job[j->row] = 0;
    se.eng->mirror[j->row] = JobDesc{};
    j->row = -1;
    j->sum32.release();
    j->comp32.release();
    j->sum64.release();
    j->out_mean.release();
    j->out_rgb8.release();
    reserved -= j->footprint;
  }
  if (j->state <= 1) j->state = 3;
  return ILLUME_OK;
}

int Server::set_option(int option, int64_t value) {
  switch (option) {
    case ILLUME_SERVER_PATH_CAPACITY:
      if (value < 1 || value > (1 << 30)) { set_error("path capacity out of range"); return ILLUME_ERR_INVALID; }
      path_capacity = (int)value;
      return ILLUME_OK;
    case ILLUME_SERVER_PASSES_PER_STEP:
      if (value < 1 || value > 1000000) { set_error("passes per step out of range"); return ILLUME_ERR_INVALID; }
      passes_per_step = (int)value;
      return ILLUME_OK;
    case ILLUME_SERVER_AUTOTUNE:
      autotune = value != 0;
      return ILLUME_OK;
    case ILLUME_SERVER_TRACE_VARIANT:
      if (value < -1 || value > 4) { set_error("unknown trace kernel variant"); return ILLUME_ERR_INVALID; }
      trace_variant = (int)value;
      return ILLUME_OK;
    case ILLUME_SERVER_LANES:
      if (value < 1 || value > kMaxLanes) { set_error("lanes out of range"); return ILLUME_ERR_INVALID; }
      lanes = (int)value;
      return ILLUME_OK;
    case ILLUME_SERVER_QUEUE_SLOTS:
      if (value < 0 || value > (1 << 30)) { set_error("queue slots out of range"); return ILLUME_ERR_INVALID; }
      queue_slots = (int)value;
      return ILLUME_OK;
    case ILLUME_SERVER_REGEN_THRESHOLD:
      if (value < 0 || value > 1000) { set_error("regeneration threshold out of range (0-1000)"); return ILLUME_ERR_INVALID; }
      regen_threshold = (float)value / 1000.0f;
      return ILLUME_OK;
    default:
      set_error("unknown server option");
      return ILLUME_ERR_INVALID;
  }
}

void Server::get_stats(illume_server_stats* out) const {
  *out = totals;
  out->path_capacity = 0;
  out->trace_variant = -1;
  out->tuned = 0;
  out->queue_slots = 0;
  out->regen_threshold = 0.0f;
  for (const auto& kv : engines) {
    out->path_capacity = std::max<int64_t>(out->path_capacity, kv.second.eng->cap);
    out->trace_variant = kv.second.eng->knobs.trace_variant;
    if (kv.second.eng->regen) {
      out->queue_slots = kv.second.eng->qcap;
      out->regen_threshold = kv.second.eng->regen_threshold;
    }
  }
  for (const auto& kv : tuners) out->tuned |= kv.second.state == 2;
  out->device_bytes = (int64_t)(engines_bytes() + reserved);
}

}  // namespace illume

// ---- C-ABI ----
extern "C" {

int illume_server_create(illume_context* ctx, size_t hbm_budget_bytes, int max_jobs_in_flight, illume_server** out) {
  if (!ctx || !out) { illume::set_error("null argument"); return ILLUME_ERR_INVALID; }
  if (max_jobs_in_flight < 0 || max_jobs_in_flight > illume::kMaxJobRows) {
    illume::set_error("max_jobs_in_flight out of range");
    return ILLUME_ERR_INVALID;
  }
  illume_server* s = new illume_server;
  s->s.ctx = &ctx->c;
  s->s.budget = hbm_budget_bytes;
  s->s.rows = max_jobs_in_flight > 0 ? max_jobs_in_flight : 64;
  *out = s;
  return ILLUME_OK;
}

int illume_server_destroy(illume_server* s) {
  if (!s) return ILLUME_OK;
  delete s;
  return ILLUME_OK;
}

int illume_job_submit(illume_server* s, illume_scene* scene, const illume_render_params* params, illume_job_id* out) {
  if (!s || !scene || !params || !out) { illume::set_error("null argument"); return ILLUME_ERR_INVALID; }
  if (scene->s.ctx != s->s.ctx) { illume::set_error("scene was not uploaded with the server's context"); return ILLUME_ERR_INVALID; }
  return s->s.submit(&scene->s, *params, out);
}

int illume_server_step(illume_server* s, int* jobs_running) {
  if (!s) { illume::set_error("null server"); return ILLUME_ERR_INVALID; }
  cudaSetDevice(s->s.ctx->device);
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

int illume_server_set_option(illume_server* s, int option, int64_t value) {
  if (!s) { illume::set_error("null server"); return ILLUME_ERR_INVALID; }
  return s->s.set_option(option, value);
}

int illume_server_get_stats(const illume_server* s, illume_server_stats* out) {
  if (!s || !out) { illume::set_error("null argument"); return ILLUME_ERR_INVALID; }
  s->s.get_stats(out);
  return ILLUME_OK;
}

int illume_plan_pass_shares(int n, const int32_t* npix, const int32_t* left, int64_t cap, int32_t* per_pass) {
  if (n < 0 || (n > 0 && (!npix || !left || !per_pass))) { illume::set_error("null argument"); return ILLUME_ERR_INVALID; }
  std::vector<long long> px(n);
  std::vector<int> lf(n), pp;
  long long need = 0;
  for (int i = 0; i < n; ++i) {
    if (npix[i] < 1 || left[i] < 1) { illume::set_error("pixels and samples must be positive"); return ILLUME_ERR_INVALID; }
    px[i] = npix[i];
    lf[i] = left[i];
    need += npix[i];
  }
  if (need > cap) { illume::set_error("one sample of every job does not fit the path slots"); return ILLUME_ERR_BUDGET; }
  illume::plan_shares(px, lf, cap, &pp);
  for (int i = 0; i < n; ++i) per_pass[i] = pp[i];
  return ILLUME_OK;
}

int illume_render_batch(illume_context* ctx, int n, illume_scene* const* scenes, const illume_render_params* params,
                        float* const* out_mean, uint8_t* const* out_rgb8, illume_render_stats* job_stats,
                        int autotune, illume_server_stats* batch_stats) {
  if (!ctx || n < 0 || (n > 0 && (!scenes || !params))) { illume::set_error("null argument"); return ILLUME_ERR_INVALID; }
  illume_server* s = nullptr;
  int st = illume_server_create(ctx, 0, std::max(1, std::min(n, 1024)), &s);
  if (st != ILLUME_OK) return st;
  s->s.autotune = autotune != 0;
  // throughput over latency: more tables overlap more passes' tails (64-job batch: 4773,
  // 4851, 4911 Mrays/s with 8, 12, 16 tables). One pass per step (the default): a
  // finished job's row is refilled at the next step, not up to seven passes later (4739
  // against 4606 Mrays/s with 8 passes per step)
  s->s.lanes = illume::kMaxLanes;
  std::vector<illume_job_id> ids(n);
  for (int i = 0; i < n && st == ILLUME_OK; ++i) {
    if (!scenes[i]) { illume::set_error("null scene"); st = ILLUME_ERR_INVALID; break; }
    st = illume_job_submit(s, scenes[i], &params[i], &ids[i]);
  }
  int running = n;
  while (st == ILLUME_OK && running > 0) st = illume_server_step(s, &running);
  for (int i = 0; i < n && st == ILLUME_OK; ++i)
    st = s->s.poll(ids[i], out_mean ? out_mean[i] : nullptr, out_rgb8 ? out_rgb8[i] : nullptr,
                   job_stats ? &job_stats[i] : nullptr);
  if (st == ILLUME_OK && batch_stats) s->s.get_stats(batch_stats);
  illume_server_destroy(s);
  return st;
}

}  // extern "C"
