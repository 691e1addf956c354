// vt_server.cu — continuous-batching render server.
//
// A request loop thread owns a private launch lane (stream, work queue, job
// table).  Each round it admits queued requests while slots and the HBM
// budget allow (accumulation buffers of the job plus, once per distinct
// scene, the scene's resident bytes), traces every admitted job together in
// one wavefront launch (passes_per_round samples per pixel each), and
// retires jobs that reached their sample target: their average image is
// copied to host memory and their device buffers are freed.  Requests that
// arrive while a round is on the GPU join the next round.  Because the random
// streams are counter based and every pixel accumulates its samples in order,
// a job's result does not depend on which other jobs shared its rounds.
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

struct Request {
  uint64_t ticket = 0;
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
  std::unordered_map<const vt_scene*, int> scene_refs;
  uint64_t next_ticket = 1;
  bool stop = false;
  std::thread loop;
  vt_server_stats stats;
  uint64_t resident = 0;   // bytes charged against the budget

  void run();
  bool admit_locked(Request* r);
  void retire_locked(Request* r, int state);
};

bool vt_server::admit_locked(Request* r) {
  uint64_t need = r->job_bytes();
  const bool new_scene = scene_refs.find(r->scene) == scene_refs.end();
  if (new_scene) need += r->scene->bytes;
  if (opts.hbm_budget_bytes && resident + need > opts.hbm_budget_bytes) return false;
  vt_job* j = nullptr;
  const int rc = vt_job_create(&lane, r->scene, r->env, &r->cam, &r->set, r->w, r->h, &j);
  if (rc != VT_OK) {
    r->error = rc;
    r->state = VT_REQ_FAILED;
    stats.failed++;
    return true;
  }
  r->job = j;
  r->state = VT_REQ_RUNNING;
  resident += need;
  scene_refs[r->scene]++;
  active.push_back(r);
  return true;
}

void vt_server::retire_locked(Request* r, int state) {
  uint64_t freed = r->job_bytes();
  auto it = scene_refs.find(r->scene);
  if (it != scene_refs.end() && --it->second == 0) {
    freed += r->scene->bytes;
    scene_refs.erase(it);
  }
  resident -= freed;
  vt_job_destroy(r->job);
  r->job = nullptr;
  r->state = state;
  r->t_done = now_s();
}

void vt_server::run() {
  cudaSetDevice(lane.device);
  std::vector<vt_job*> jobs;
  std::vector<int32_t> passes;
  std::vector<Request*> round;
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
          stats.cancelled++;
          continue;
        }
        const uint64_t alone = r->job_bytes() + r->scene->bytes;
        if (opts.hbm_budget_bytes && alone > opts.hbm_budget_bytes) {
          queue.erase(queue.begin() + at);
          r->state = VT_REQ_FAILED;
          r->error = VT_EBUDGET;
          stats.failed++;
          continue;
        }
        if (!admit_locked(r)) break;   // wait for memory to free up
        queue.erase(queue.begin() + at);
      }
      stats.active = (int32_t)active.size();
      stats.queued = (int32_t)queue.size();
      stats.bytes_in_use = resident;
      changed.notify_all();
      if (active.empty()) {
        if (stop) return;
        wake.wait_for(g, std::chrono::milliseconds(20));
        continue;
      }
      round = active;
    }
    jobs.clear();
    passes.clear();
    uint64_t paths = 0;
    for (Request* r : round) {
      jobs.push_back(r->job);
      const int32_t left = r->spp - r->samples;
      const uint64_t left_paths = (uint64_t)r->w * r->h * (uint64_t)left;
      int32_t p = (opts.quick_paths && left_paths <= opts.quick_paths) ? left : std::min(opts.passes_per_round, left);
      if (opts.round_paths_cap) {
        const uint64_t px = (uint64_t)r->w * r->h;
        p = (int32_t)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)p, opts.round_paths_cap / px));
      }
      passes.push_back(p);
      paths += (uint64_t)r->w * r->h * (uint64_t)p;
    }
    int rc = render_jobs(&lane, jobs.data(), (int32_t)jobs.size(), passes.data(), 2, opts.path_slots, 0, false);
    if (rc == VT_OK && cudaStreamSynchronize(lane.stream) != cudaSuccess) rc = VT_EDEVICE;
    std::unique_lock<std::mutex> g(mu);
    stats.rounds++;
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
  cudaSetDevice(L.device);
  cudaError_t e = cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete s; return cuda_fail(e, "server stream"); }
  int rc = L.alloc((void**)&L.d_counters, sizeof(unsigned long long) * C_NUM);
  if (rc == VT_OK) rc = L.alloc((void**)&L.d_queue, sizeof(unsigned long long) * 4);
  if (rc == VT_OK) rc = L.alloc((void**)&L.d_error, sizeof(int32_t) * 4);
  if (rc != VT_OK) { cudaStreamDestroy(L.stream); delete s; return rc; }
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
  release_context(&s->lane);   // wavefront buffers, graphs and lane streams included
  delete s;
  return VT_OK;
}
