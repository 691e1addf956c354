// vt_server.cu — continuous-batching render server.
//
// A request loop thread owns a private launch lane (stream, work queue, job
// table).  Each round it admits queued requests while slots and the HBM
// budget allow (the job's accumulation buffers), traces every admitted job
// together in one wavefront launch (a path budget shared out by
// compose_round), and retires jobs that reached their sample target: their
// average image is copied to host memory and their device buffers are freed.
// Requests that arrive while a round is on the GPU join the next round.
// Because the random streams are counter based and every pixel accumulates
// its samples in order, a job's result does not depend on which other jobs
// shared its rounds.
//
// Residency: scenes submitted as host data (vt_server_submit_dense) are
// uploaded once per key onto the server's own upload context, counted
// against the budget, kept resident while requests use them and after (for
// reuse by later requests with the same key), and evicted least recently
// used first when a new scene or job needs the room.  Scenes the caller
// created itself (vt_server_submit) stay the caller's and are not counted.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/vt.h"
#include "vt_runtime.h"

using namespace vt;

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// A scene the server uploaded and keeps resident, by the caller's key.
struct Resident {
  uint64_t key = 0;
  vt_scene* scene = nullptr;
  int refs = 0;             // queued and running requests that use it
  uint64_t last_use = 0;    // submission counter of the last request that used it
  uint64_t bytes = 0;
};

struct Request {
  uint64_t ticket = 0;
  Resident* resident = nullptr;   // set when the scene is the server's
  const vt_scene* scene = nullptr;
  const vt_env* env = nullptr;
  vt_camera cam;
  vt_render_settings set;
  int32_t w = 0, h = 0, spp = 0;
  int32_t state = VT_REQ_QUEUED;
  vt_job* job = nullptr;
  int32_t samples = 0;
  bool cancel = false;
  std::vector<float> result;
  double t_submit = 0.0, t_done = 0.0;
  int error = VT_OK;
  uint64_t job_bytes() const { return (uint64_t)w * h * sizeof(float4) * 3; }
  uint64_t paths() const { return (uint64_t)w * h * (uint64_t)spp; }
};

}  // namespace

struct vt_server {
  vt_context* user = nullptr;
  vt_context lane;
  vt_server_opts opts;
  std::mutex mu;
  std::condition_variable wake;
  std::condition_variable changed;
  std::deque<Request*> queue;
  std::unordered_map<uint64_t, Request*> reqs;
  std::vector<Request*> active;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::thread loop;
  vt_server_stats stats;
  uint64_t resident = 0;   // bytes charged against the budget: job buffers and resident scenes
  // residency cache: the upload context (own stream and allocator) and its scenes
  vt_context uploads;
  std::mutex upload_mu;    // one upload at a time
  std::unordered_map<uint64_t, Resident*> cache;
  uint64_t use_clock = 0;

  void run();
  bool admit_locked(Request* r);
  void retire_locked(Request* r, int state);
  bool make_room_locked(uint64_t need);
  void release_ref_locked(Request* r);
  void compose_round(const std::vector<Request*>& round, std::vector<int32_t>& passes) const;
};

// Passes of each request in the next round.  Every request first gets
// passes_per_round (or what it has left; all of it when that is at most
// quick_paths paths); the rest of the round's path budget then goes to the
// requests with the fewest paths left first, as many whole passes as fit.
// round_paths_cap bounds any one request's share (at least one pass).
void vt_server::compose_round(const std::vector<Request*>& round, std::vector<int32_t>& passes) const {
  const size_t n = round.size();
  passes.assign(n, 0);
  const uint64_t budget = opts.round_paths ? opts.round_paths : ((uint64_t)1 << 26);
  uint64_t used = 0;
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; ++i) {
    const Request* r = round[i];
    const int32_t left = r->spp - r->samples;
    const uint64_t px = (uint64_t)r->w * r->h;
    int32_t p = (opts.quick_paths && px * (uint64_t)left <= opts.quick_paths) ? left
                                                                              : std::min(opts.passes_per_round, left);
    if (opts.round_paths_cap) p = (int32_t)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)p, opts.round_paths_cap / px));
    passes[i] = p;
    used += px * (uint64_t)p;
    order[i] = i;
  }
  auto left_paths = [&](size_t i) {
    return (uint64_t)round[i]->w * round[i]->h * (uint64_t)(round[i]->spp - round[i]->samples - passes[i]);
  };
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return left_paths(a) < left_paths(b); });
  for (size_t k = 0; k < n && used < budget; ++k) {
    const size_t i = order[k];
    const Request* r = round[i];
    const uint64_t px = (uint64_t)r->w * r->h;
    uint64_t more = std::min<uint64_t>((uint64_t)(r->spp - r->samples - passes[i]), (budget - used) / px);
    if (opts.round_paths_cap) {
      const uint64_t cap = std::max<uint64_t>(1, opts.round_paths_cap / px);
      more = std::min<uint64_t>(more, cap > (uint64_t)passes[i] ? cap - (uint64_t)passes[i] : 0);
    }
    passes[i] += (int32_t)more;
    used += px * more;
  }
}

// Evicts unused resident scenes, least recently used first, until `need`
// more bytes fit the budget; false if they cannot.
bool vt_server::make_room_locked(uint64_t need) {
  if (!opts.hbm_budget_bytes) return true;
  while (resident + need > opts.hbm_budget_bytes) {
    Resident* victim = nullptr;
    for (auto& kv : cache)
      if (kv.second->refs == 0 && (!victim || kv.second->last_use < victim->last_use)) victim = kv.second;
    if (!victim) return false;
    cache.erase(victim->key);
    resident -= victim->bytes;
    vt_scene_destroy(victim->scene);
    delete victim;
    stats.scene_evictions++;
    stats.scenes_resident = (int32_t)cache.size();
  }
  return true;
}

void vt_server::release_ref_locked(Request* r) {
  if (r->resident) {
    r->resident->refs--;
    r->resident = nullptr;
  }
}

bool vt_server::admit_locked(Request* r) {
  const uint64_t need = r->job_bytes();
  if (!make_room_locked(need)) return false;
  vt_job* j = nullptr;
  const int rc = vt_job_create(&lane, r->scene, r->env, &r->cam, &r->set, r->w, r->h, &j);
  if (rc != VT_OK) {
    r->error = rc;
    r->state = VT_REQ_FAILED;
    release_ref_locked(r);
    stats.failed++;
    return true;
  }
  r->job = j;
  r->state = VT_REQ_RUNNING;
  resident += need;
  active.push_back(r);
  return true;
}

void vt_server::retire_locked(Request* r, int state) {
  resident -= r->job_bytes();
  vt_job_destroy(r->job);
  r->job = nullptr;
  release_ref_locked(r);
  r->state = state;
  r->t_done = now_s();
}

void vt_server::run() {
  cudaSetDevice(lane.device);
  std::vector<vt_job*> jobs;
  std::vector<int32_t> passes;
  std::vector<Request*> round;
  double last_end = 0.0;   // end of the previous round, 0 after waiting for work
  for (;;) {
    {
      std::unique_lock<std::mutex> g(mu);
      // cancelled active requests leave before the round
      for (size_t i = 0; i < active.size();) {
        if (active[i]->cancel) {
          retire_locked(active[i], VT_REQ_CANCELLED);
          stats.cancelled++;
          active.erase(active.begin() + i);
        } else {
          ++i;
        }
      }
      // admission: in arrival order, or the request with the fewest paths first
      while (!queue.empty() && (int)active.size() < opts.max_active_jobs) {
        size_t at = 0;
        if (opts.order == VT_SERVE_LEAST_WORK)
          for (size_t i = 1; i < queue.size(); ++i)
            if (queue[i]->paths() < queue[at]->paths()) at = i;
        Request* r = queue[at];
        if (r->cancel) {
          queue.erase(queue.begin() + at);
          r->state = VT_REQ_CANCELLED;
          release_ref_locked(r);
          stats.cancelled++;
          continue;
        }
        const uint64_t alone = r->job_bytes() + (r->resident ? r->resident->bytes : 0);
        if (opts.hbm_budget_bytes && alone > opts.hbm_budget_bytes) {
          queue.erase(queue.begin() + at);
          r->state = VT_REQ_FAILED;
          r->error = VT_EBUDGET;
          release_ref_locked(r);
          stats.failed++;
          continue;
        }
        if (!admit_locked(r)) break;   // wait for memory to free up
        queue.erase(queue.begin() + at);
      }
      stats.active = (int32_t)active.size();
      stats.queued = (int32_t)queue.size();
      stats.bytes_in_use = resident;
      stats.scenes_resident = (int32_t)cache.size();
      changed.notify_all();
      if (active.empty()) {
        if (stop) return;
        last_end = 0.0;
        wake.wait_for(g, std::chrono::milliseconds(20));
        continue;
      }
      round = active;
    }
    jobs.clear();
    passes.clear();
    compose_round(round, passes);
    uint64_t paths = 0;
    for (size_t i = 0; i < round.size(); ++i) {
      jobs.push_back(round[i]->job);
      paths += (uint64_t)round[i]->w * round[i]->h * (uint64_t)passes[i];
    }
    vt::Range round_range("vt.server_round");
    const double t0 = now_s();
    int rc = render_jobs(&lane, jobs.data(), (int32_t)jobs.size(), passes.data(), 2, opts.path_slots, 0, false);
    if (rc == VT_OK && cudaStreamSynchronize(lane.stream) != cudaSuccess) rc = VT_EDEVICE;
    const double t1 = now_s();
    std::unique_lock<std::mutex> g(mu);
    stats.rounds++;
    stats.round_us += (uint64_t)(1e6 * (t1 - t0));
    if (last_end > 0.0) stats.between_us += (uint64_t)(1e6 * (t0 - last_end));
    for (size_t i = 0; i < round.size(); ++i) {
      Request* r = round[i];
      if (rc != VT_OK) {
        r->error = rc;
        retire_locked(r, VT_REQ_FAILED);
        stats.failed++;
        continue;
      }
      r->job->samples += passes[i];
      r->samples = r->job->samples;
      if (r->samples >= r->spp) {
        r->result.resize((size_t)r->w * r->h * 4);
        const int rr = vt_job_readback(r->job, r->result.data(), r->result.size() * sizeof(float), 0);
        if (rr != VT_OK) { r->error = rr; retire_locked(r, VT_REQ_FAILED); stats.failed++; continue; }
        retire_locked(r, VT_REQ_DONE);
        stats.completed++;
      }
    }
    if (rc == VT_OK) stats.paths_traced += paths;
    active.erase(std::remove_if(active.begin(), active.end(), [](Request* r) { return r->state != VT_REQ_RUNNING; }),
                 active.end());
    changed.notify_all();
    last_end = t1;
  }
}

extern "C" int vt_server_create(vt_context* ctx, const vt_server_opts* opts, vt_server** out) {
  if (!ctx || !out) return fail(VT_EINVAL, "null argument");
  *out = nullptr;
  vt_server* s = new vt_server();
  s->user = ctx;
  memset(&s->opts, 0, sizeof(s->opts));
  if (opts) s->opts = *opts;
  if (s->opts.max_active_jobs <= 0) s->opts.max_active_jobs = 64;
  if (s->opts.passes_per_round <= 0) s->opts.passes_per_round = 4;
  if (s->opts.order != VT_SERVE_LEAST_WORK) s->opts.order = VT_SERVE_ARRIVAL;
  memset(&s->stats, 0, sizeof(s->stats));
  vt_context& L = s->lane;
  L.device = ctx->device;
  L.sm_count = ctx->sm_count;
  L.kernel = 2;
  L.log_fn = ctx->log_fn;
  L.log_user = ctx->log_user;
  // the rounds take the creating context's launch shape (lanes, DDA kernel
  // form and grid, refill interval, queue chunk), tuned or not
  L.lanes = ctx->lanes;
  L.trace_blocks_per_sm = ctx->trace_blocks_per_sm;
  L.trace_steps = ctx->trace_steps;
  L.trace_chunk = ctx->trace_chunk;
  L.refill_min = ctx->refill_min;
  L.trace_form = ctx->trace_form;
  L.use_graphs = ctx->use_graphs;
  cudaSetDevice(L.device);
  cudaError_t e = cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete s; return cuda_fail(e, "server stream"); }
  int rc = L.alloc((void**)&L.d_counters, sizeof(unsigned long long) * C_NUM);
  if (rc == VT_OK) rc = L.alloc((void**)&L.d_queue, sizeof(unsigned long long) * 4);
  if (rc == VT_OK) rc = L.alloc((void**)&L.d_error, sizeof(int32_t) * 4);
  if (rc != VT_OK) { release_context(&L); delete s; return rc; }
  // the upload context of resident scenes: its own stream, so that an upload
  // does not queue behind the round on the lane's stream
  vt_context& U = s->uploads;
  U.device = ctx->device;
  U.sm_count = ctx->sm_count;
  U.log_fn = ctx->log_fn;
  U.log_user = ctx->log_user;
  e = cudaStreamCreateWithFlags(&U.stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { release_context(&L); delete s; return cuda_fail(e, "server upload stream"); }
  rc = U.alloc((void**)&U.d_counters, sizeof(unsigned long long) * C_NUM);
  if (rc == VT_OK) rc = U.alloc((void**)&U.d_queue, sizeof(unsigned long long) * 4);
  if (rc == VT_OK) rc = U.alloc((void**)&U.d_error, sizeof(int32_t) * 4);
  if (rc != VT_OK) { release_context(&U); release_context(&L); delete s; return rc; }
  s->loop = std::thread([s]() { s->run(); });
  *out = s;
  return VT_OK;
}

extern "C" int vt_server_submit(vt_server* s, const vt_scene* scene, const vt_env* env, const vt_camera* cam,
                                const vt_render_settings* set, int32_t w, int32_t h, int32_t spp, uint64_t* ticket) {
  if (!s || !scene || !cam || !set || !ticket) return fail(VT_EINVAL, "null argument");
  if (w <= 0 || h <= 0 || spp <= 0) return fail(VT_EINVAL, "bad size or sample target");
  Request* r = new Request();
  r->scene = scene;
  r->env = env;
  r->cam = *cam;
  r->set = *set;
  r->set.max_samples = spp;
  r->w = w;
  r->h = h;
  r->spp = spp;
  r->t_submit = now_s();
  {
    std::lock_guard<std::mutex> g(s->mu);
    r->ticket = s->next_ticket++;
    s->reqs[r->ticket] = r;
    s->queue.push_back(r);
    s->stats.submitted++;
    *ticket = r->ticket;
  }
  s->wake.notify_all();
  return VT_OK;
}

// Device bytes of a dense scene before its emissive list (vt_scene::bytes).
static uint64_t dense_scene_bytes(int32_t rx, int32_t ry, int32_t rz, int32_t n_palette) {
  const uint64_t nb = (uint64_t)((rx + 3) / 4 + 2) * ((ry + 3) / 4 + 2) * ((rz + 3) / 4 + 2);
  return (uint64_t)rx * ry * rz + 8 * nb + 16 * (uint64_t)std::max(n_palette, 1) + 4;
}

extern "C" int vt_server_submit_dense(vt_server* s, uint64_t scene_key, int32_t rx, int32_t ry, int32_t rz,
                                      const uint8_t* voxels, const vt_material* palette, int32_t n_palette,
                                      uint32_t scene_flags, const vt_env* env, const vt_camera* cam,
                                      const vt_render_settings* set, int32_t w, int32_t h, int32_t spp,
                                      uint64_t* ticket) {
  if (!s || !cam || !set || !ticket) return fail(VT_EINVAL, "null argument");
  if (w <= 0 || h <= 0 || spp <= 0) return fail(VT_EINVAL, "bad size or sample target");
  std::lock_guard<std::mutex> up(s->upload_mu);
  Resident* res = nullptr;
  {
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->cache.find(scene_key);
    if (it != s->cache.end()) {
      res = it->second;
      res->refs++;
      res->last_use = ++s->use_clock;
      s->stats.scene_hits++;
    }
  }
  if (!res) {
    if (!voxels || !palette)
      return fail(VT_EINVAL, "scene key %llu is not resident and no volume was given", (unsigned long long)scene_key);
    if (rx <= 0 || ry <= 0 || rz <= 0) return fail(VT_EINVAL, "resolution must be positive");
    const uint64_t estimate = dense_scene_bytes(rx, ry, rz, n_palette);
    {
      std::lock_guard<std::mutex> g(s->mu);
      if (!s->make_room_locked(estimate))
        return fail(VT_EBUDGET, "scene of %llu bytes does not fit the server's budget beside the scenes and jobs in use",
                    (unsigned long long)estimate);
      s->resident += estimate;   // held while the upload runs
    }
    vt_scene* sc = nullptr;
    cudaSetDevice(s->uploads.device);
    const int rc = vt_scene_create(&s->uploads, rx, ry, rz, voxels, palette, n_palette, nullptr, 0, scene_flags, &sc);
    std::lock_guard<std::mutex> g(s->mu);
    s->resident -= estimate;
    if (rc != VT_OK) return rc;
    res = new Resident();
    res->key = scene_key;
    res->scene = sc;
    res->refs = 1;
    res->last_use = ++s->use_clock;
    res->bytes = sc->bytes;
    s->resident += res->bytes;
    s->cache[scene_key] = res;
    s->stats.scene_uploads++;
    s->stats.scenes_resident = (int32_t)s->cache.size();
  }
  Request* r = new Request();
  r->resident = res;
  r->scene = res->scene;
  r->env = env;
  r->cam = *cam;
  r->set = *set;
  r->set.max_samples = spp;
  r->w = w;
  r->h = h;
  r->spp = spp;
  r->t_submit = now_s();
  {
    std::lock_guard<std::mutex> g(s->mu);
    r->ticket = s->next_ticket++;
    s->reqs[r->ticket] = r;
    s->queue.push_back(r);
    s->stats.submitted++;
    *ticket = r->ticket;
  }
  s->wake.notify_all();
  return VT_OK;
}

extern "C" int vt_server_poll(vt_server* s, uint64_t ticket, int32_t* state, int32_t* samples) {
  if (!s) return fail(VT_EINVAL, "server is null");
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return fail(VT_EINVAL, "unknown ticket %llu", (unsigned long long)ticket);
  if (state) *state = it->second->state;
  if (samples) *samples = it->second->samples;
  return VT_OK;
}

extern "C" int vt_server_wait(vt_server* s, uint64_t ticket, double timeout_s) {
  if (!s) return fail(VT_EINVAL, "server is null");
  std::unique_lock<std::mutex> g(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return fail(VT_EINVAL, "unknown ticket %llu", (unsigned long long)ticket);
  Request* r = it->second;
  auto finished = [r]() { return r->state == VT_REQ_DONE || r->state == VT_REQ_FAILED || r->state == VT_REQ_CANCELLED; };
  if (timeout_s < 0) s->changed.wait(g, finished);
  else if (!s->changed.wait_for(g, std::chrono::duration<double>(timeout_s), finished))
    return fail(VT_ETIMEOUT, "request %llu not finished after %.3f s", (unsigned long long)ticket, timeout_s);
  if (r->state == VT_REQ_FAILED) return fail(r->error ? r->error : VT_EDEVICE, "request %llu failed", (unsigned long long)ticket);
  if (r->state == VT_REQ_CANCELLED) return fail(VT_ECANCELLED, "request %llu cancelled", (unsigned long long)ticket);
  return VT_OK;
}

extern "C" int vt_server_result(vt_server* s, uint64_t ticket, float* rgba, size_t bytes, double* seconds) {
  if (!s) return fail(VT_EINVAL, "server is null");
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return fail(VT_EINVAL, "unknown ticket %llu", (unsigned long long)ticket);
  Request* r = it->second;
  if (r->state == VT_REQ_FAILED) return fail(r->error ? r->error : VT_EDEVICE, "request failed");
  if (r->state == VT_REQ_CANCELLED) return fail(VT_ECANCELLED, "request cancelled");
  if (r->state != VT_REQ_DONE) return fail(VT_ENOTREADY, "request %llu not finished", (unsigned long long)ticket);
  if (rgba) {
    if (bytes < r->result.size() * sizeof(float)) return fail(VT_EINVAL, "output buffer too small");
    memcpy(rgba, r->result.data(), r->result.size() * sizeof(float));
  }
  if (seconds) *seconds = r->t_done - r->t_submit;
  s->reqs.erase(it);
  delete r;
  return VT_OK;
}

extern "C" int vt_server_cancel(vt_server* s, uint64_t ticket) {
  if (!s) return fail(VT_EINVAL, "server is null");
  {
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return fail(VT_EINVAL, "unknown ticket %llu", (unsigned long long)ticket);
    it->second->cancel = true;
  }
  s->wake.notify_all();
  return VT_OK;
}

extern "C" int vt_server_get_stats(vt_server* s, vt_server_stats* st) {
  if (!s || !st) return fail(VT_EINVAL, "null argument");
  std::lock_guard<std::mutex> g(s->mu);
  *st = s->stats;
  return VT_OK;
}

extern "C" int vt_server_destroy(vt_server* s) {
  if (!s) return VT_OK;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
    for (Request* r : s->queue) { r->state = VT_REQ_CANCELLED; }
    s->queue.clear();
    for (Request* r : s->active) r->cancel = true;
  }
  s->wake.notify_all();
  if (s->loop.joinable()) s->loop.join();
  for (auto& kv : s->reqs) {
    if (kv.second->job) vt_job_destroy(kv.second->job);
    delete kv.second;
  }
  for (auto& kv : s->cache) {
    vt_scene_destroy(kv.second->scene);
    delete kv.second;
  }
  s->cache.clear();
  release_context(&s->lane);   // wavefront buffers, graphs and lane streams included
  release_context(&s->uploads);
  delete s;
  return VT_OK;
}
