// vt_fixed.cu — vt_render_batch_fixed: the wavefront renderer with all of its
// working memory in one file-scope device array instead of context buffers.
//
// Layout of the array (every part starts on a 256-byte boundary):
//   control     the wavefront control words (kCtlBytes, one 128-byte line
//               per counter; must start at zero)
//   job table   VT_FIXED_MAX_JOBS JobEntry records
//   grid table  VT_FIXED_MAX_JOBS Grid records
//   path slots  VT_FIXED_MAX_PATH_SLOTS x kWfSlotBytes (two path streams,
//               segment ends, hit records, two segment queues; wf_carve)
//   samples     VT_FIXED_MAX_SAMPLES float4 per-sample outputs
// The kernels are the ones vt_render_batch runs; only where their buffers
// live differs, so results are bit-identical.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "vt_runtime.h"

using namespace vt;

namespace {

constexpr size_t round256(size_t x) { return (x + 255) & ~(size_t)255; }

constexpr size_t kSlotBytes = kWfSlotBytes;
constexpr size_t kCtlOff = 0;
constexpr size_t kJobsOff = kCtlOff + round256(kCtlBytes);
constexpr size_t kGridsOff = kJobsOff + round256(sizeof(JobEntry) * VT_FIXED_MAX_JOBS);
constexpr size_t kSlotsOff = kGridsOff + round256(sizeof(Grid) * VT_FIXED_MAX_JOBS);
constexpr size_t kSamplesOff = kSlotsOff + round256(kSlotBytes * (size_t)VT_FIXED_MAX_PATH_SLOTS);
constexpr size_t kTotal = kSamplesOff + sizeof(float4) * (size_t)VT_FIXED_MAX_SAMPLES;
static_assert(kTotal == (size_t)VT_FIXED_SCRATCH_BYTES, "VT_FIXED_SCRATCH_BYTES does not match the layout");

constexpr int kMaxDevices = 64;

}  // namespace

static __device__ __align__(256) unsigned char g_fixed_scratch[kTotal];

static std::mutex g_fixed_mu;
static void* g_fixed_base[kMaxDevices];

// Looks up the device address of g_fixed_scratch with `device` current and
// keeps it for that device.  The CUDA runtime loads this file's device code
// (and so reserves the array) lazily, at the first use of one of its
// symbols; vt_create calls this for its device so that the reservation, and
// any failure to make it, happens there rather than in a frame loop.  Each
// vt_create looks the address up again, so a context created after a
// cudaDeviceReset never sees an address from before the reset.
int vt::fixed_scratch_setup(int device) {
  if (device < 0 || device >= kMaxDevices)
    return fail(VT_EINVAL, "device %d is beyond the %d devices vt_render_batch_fixed supports", device, kMaxDevices);
  std::lock_guard<std::mutex> lock(g_fixed_mu);
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_fixed_scratch);
  if (e != cudaSuccess) {
    g_fixed_base[device] = nullptr;
    return cuda_fail(e, "cudaGetSymbolAddress of the fixed scratch array");
  }
  g_fixed_base[device] = p;
  return VT_OK;
}

// Device address of g_fixed_scratch on the current device (set up by
// vt_create, or here if that set-up failed).
static int fixed_base(int device, char** out) {
  if (device < 0 || device >= kMaxDevices)
    return fail(VT_EINVAL, "device %d is beyond the %d devices vt_render_batch_fixed supports", device, kMaxDevices);
  {
    std::lock_guard<std::mutex> lock(g_fixed_mu);
    if (g_fixed_base[device]) { *out = (char*)g_fixed_base[device]; return VT_OK; }
  }
  const int rc = vt::fixed_scratch_setup(device);
  if (rc != VT_OK) return rc;
  std::lock_guard<std::mutex> lock(g_fixed_mu);
  *out = (char*)g_fixed_base[device];
  return VT_OK;
}

// A failure after work was queued: wait for that work (it may still use the
// shared array) before the error goes back to the caller.
static int drain(vt_context* ctx, int rc) {
  cudaStreamSynchronize(ctx->stream);
  return rc;
}

static Grid fixed_grid(const vt_job* j) { return make_grid(j->frame, j->dev.bricks); }

// One wavefront launch over entries[0..n) with `items` samples in total.
static int fixed_launch(vt_context* ctx, char* base, const JobEntry* entries, const Grid* grids, int n,
                        int64_t items, int64_t slots_cap) {
  cudaStream_t st = ctx->stream;
  const int64_t slots = std::max<int64_t>(32, std::min<int64_t>(items, slots_cap));
  const size_t S = (size_t)VT_FIXED_MAX_PATH_SLOTS;
  uint32_t* ctl = (uint32_t*)(base + kCtlOff);
  JobEntry* d_jobs = (JobEntry*)(base + kJobsOff);
  Grid* d_grids = (Grid*)(base + kGridsOff);
  WfParams P;
  memset(&P, 0, sizeof(P));
  P.jobs = d_jobs;
  P.n_jobs = n;
  P.grids = d_grids;
  wf_carve(base + kSlotsOff, S, P);
  P.n_slots = (int32_t)slots;
  P.ctl = ctl;
  P.next_item = (unsigned long long*)(ctl + kCtlNextItem);
  P.n_items = (unsigned long long)items;
  P.sbuf = (float4*)(base + kSamplesOff);
  P.counters = nullptr;
  P.trace_chunk = (uint32_t)ctx->trace_chunk;
  P.refill_min = ctx->refill_min;
  P.trace_form = ctx->trace_form;
  P.bricks_444 = 1;
  for (int i = 0; i < n; ++i)
    if (grids[i].shx != 2 || grids[i].shy != 2 || grids[i].shz != 2) P.bricks_444 = 0;
  // pageable sources: both copies have read the host tables when they return
  cudaError_t e = cudaMemcpyAsync(d_jobs, entries, sizeof(JobEntry) * n, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return drain(ctx, cuda_fail(e, "fixed job table"));
  e = cudaMemcpyAsync(d_grids, grids, sizeof(Grid) * n, cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return drain(ctx, cuda_fail(e, "fixed grid table"));
  e = cudaMemsetAsync(ctl, 0, kCtlBytes, st);
  if (e != cudaSuccess) return drain(ctx, cuda_fail(e, "fixed control words"));
  if (ctx->trace_occupancy <= 0) ctx->trace_occupancy = std::max(1, wf_trace_blocks_per_sm());
  const int bps = ctx->trace_blocks_per_sm > 0 ? ctx->trace_blocks_per_sm : ctx->trace_occupancy;
  const int trace_blocks = ctx->sm_count * bps;
  // the bound of the wavefront launch's loop: a path ends within
  // max_bounces + 2 rounds of its start
  int32_t max_b = 0;
  for (int i = 0; i < n; ++i) max_b = std::max(max_b, entries[i].F.max_bounces);
  const int64_t max_rounds = 4 * (items / slots + 2) * ((int64_t)max_b + 2) + 16;
  for (int64_t iter = 0;; ++iter) {
    if (iter >= max_rounds) return drain(ctx, fail(VT_EDEVICE, "wavefront did not drain within %lld rounds",
                                                   (long long)max_rounds));
    const int par = (int)(iter & 1);
    e = cudaMemsetAsync(ctl + ctl_index(par, 0), 0, CTL_PER_PARITY * kCtlStride * sizeof(uint32_t), st);
    if (e != cudaSuccess) return drain(ctx, cuda_fail(e, "fixed round counters"));
    e = launch_wf_shade(P, par, ctx->sm_count * 8, false, st);
    if (e != cudaSuccess) return drain(ctx, cuda_fail(e, "fixed wavefront shade"));
    e = launch_wf_trace(P, par, trace_blocks, ctx->trace_steps, false, st);
    if (e != cudaSuccess) return drain(ctx, cuda_fail(e, "fixed wavefront trace"));
    ctx->launches += 4;
    if ((iter & 7) == 7) {
      uint32_t live = 0;   // pageable: the copy has completed when it returns
      e = cudaMemcpyAsync(&live, ctl + ctl_index(par, CTL_NEXT_N), sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) return drain(ctx, cuda_fail(e, "fixed live count"));
      if (live == 0) break;
    }
  }
  long long max_pixels = 0;
  for (int i = 0; i < n; ++i) max_pixels = std::max<long long>(max_pixels, entries[i].n_pixels);
  e = launch_wf_accumulate(d_jobs, n, max_pixels, P.sbuf, st);
  if (e != cudaSuccess) return drain(ctx, cuda_fail(e, "fixed accumulate"));
  ctx->launches += 1;
  return VT_OK;
}

extern "C" int vt_render_batch_fixed(vt_context* ctx, vt_job* const* jobs, int32_t n_jobs, int32_t passes,
                                     int32_t path_slots, int32_t* results) {
  if (!ctx || n_jobs < 0 || (n_jobs > 0 && !jobs) || passes < 0 || path_slots < 0)
    return fail(VT_EINVAL, "bad argument");
  if (n_jobs > VT_FIXED_MAX_JOBS)
    return fail(VT_EINVAL, "%d jobs exceed VT_FIXED_MAX_JOBS (%d) of vt_render_batch_fixed", n_jobs,
                VT_FIXED_MAX_JOBS);
  if (path_slots > VT_FIXED_MAX_PATH_SLOTS)
    return fail(VT_EINVAL, "path_slots %d exceeds VT_FIXED_MAX_PATH_SLOTS (%d) of vt_render_batch_fixed", path_slots,
                VT_FIXED_MAX_PATH_SLOTS);
  int32_t np[VT_FIXED_MAX_JOBS];
  int32_t done[VT_FIXED_MAX_JOBS];
  for (int i = 0; i < n_jobs; ++i) {
    const vt_job* j = jobs[i];
    if (!j || j->ctx != ctx) return fail(VT_EINVAL, "job %d is null or belongs to another context", i);
    const int64_t px = (int64_t)j->w * j->h;
    if (px > VT_FIXED_MAX_SAMPLES)
      return fail(VT_EINVAL, "job %d has %lld pixels, more than VT_FIXED_MAX_SAMPLES (%d) of vt_render_batch_fixed",
                  i, (long long)px, VT_FIXED_MAX_SAMPLES);
    np[i] = std::max(0, std::min(passes, j->set.max_samples - j->samples));
    done[i] = 0;
  }
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
  char* base = nullptr;
  int rc = fixed_base(ctx->device, &base);
  if (rc != VT_OK) return rc;
  for (int i = 0; i < n_jobs; ++i) {   // frames of jobs whose scene was edited (no allocation)
    rc = refresh_job(jobs[i]);
    if (rc != VT_OK) return rc;
  }
  // edit-mode jobs take the per-pixel kernel, which needs no working memory
  for (int i = 0; i < n_jobs; ++i) {
    if (jobs[i]->integrator == VT_INTEGRATOR_PATH_TRACER) continue;
    for (int32_t k = 0; k < np[i]; ++k) {
      e = launch_plain(jobs[i]->frame, jobs[i]->dev, jobs[i]->samples + k, 1, nullptr, ctx->stream);
      if (e != cudaSuccess) return drain(ctx, cuda_fail(e, "fixed edit-mode pass"));
    }
    ctx->launches += (uint64_t)np[i];
    done[i] = np[i];
  }
  const int64_t slots_cap = path_slots > 0 ? path_slots : VT_FIXED_MAX_PATH_SLOTS;
  JobEntry entries[VT_FIXED_MAX_JOBS];
  Grid grids[VT_FIXED_MAX_JOBS];
  for (;;) {
    int64_t pix_left = 0;
    for (int i = 0; i < n_jobs; ++i)
      if (done[i] < np[i]) pix_left += (int64_t)jobs[i]->w * jobs[i]->h;
    if (pix_left == 0) break;
    const int64_t q = std::max<int64_t>(1, (int64_t)VT_FIXED_MAX_SAMPLES / pix_left);
    int n = 0;
    int64_t items = 0;
    for (int i = 0; i < n_jobs; ++i) {
      const int64_t px = (int64_t)jobs[i]->w * jobs[i]->h;
      const int64_t p = std::min<int64_t>(q, np[i] - done[i]);
      if (p <= 0 || items + px > VT_FIXED_MAX_SAMPLES) continue;   // no room for one pass: a later launch
      const int64_t fit = std::min<int64_t>(p, (VT_FIXED_MAX_SAMPLES - items) / px);
      JobEntry& en = entries[n];
      memset(&en, 0, sizeof(en));
      en.F = jobs[i]->frame;
      en.J = jobs[i]->dev;
      en.sample_base = jobs[i]->samples + done[i];
      en.passes = (int32_t)fit;
      en.tile_begin = items;
      en.n_pixels = px;
      grids[n] = fixed_grid(jobs[i]);
      items += px * fit;
      done[i] += (int32_t)fit;
      ++n;
    }
    rc = fixed_launch(ctx, base, entries, grids, n, items, slots_cap);
    if (rc != VT_OK) return rc;   // fixed_launch has drained the stream
  }
  e = cudaStreamSynchronize(ctx->stream);   // the array is free for the next call
  if (e != cudaSuccess) return cuda_fail(e, "fixed render");
  for (int i = 0; i < n_jobs; ++i) {
    jobs[i]->samples += np[i];
    if (results)
      results[i] = jobs[i]->samples >= jobs[i]->set.max_samples ? VT_FINISHED_RENDERING : VT_SAMPLES_PENDING;
  }
  return VT_OK;
}
