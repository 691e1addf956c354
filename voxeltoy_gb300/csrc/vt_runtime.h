// vt_runtime.h — host-side objects behind the opaque C handles.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <map>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "../../include/vt.h"
#include "vt_internal.h"
#include "vt_kernels.h"

struct vt_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  uint64_t budget = 0;          // 0 = unlimited
  uint64_t in_use = 0;          // bytes held through alloc()
  int sm_count = 0;
  int kernel = 2;               // 1 plain, 2 wavefront
  vt_log_fn log_fn = nullptr;
  void* log_user = nullptr;
  std::mutex mu;
  std::unordered_map<void*, size_t> sizes;
  float4* noise = nullptr;
  void* scratch = nullptr;      // reusable device scratch for diagnostics and picks
  size_t scratch_bytes = 0;
  vt::JobEntry* d_jobs = nullptr;
  size_t d_jobs_bytes = 0;
  // wavefront buffers (grown on demand)
  vt::Grid* d_grids = nullptr;
  size_t d_grids_bytes = 0;
  void* wf_mem = nullptr;        // slot state, flags, hits, queues
  int64_t wf_slots = 0;
  float4* sbuf = nullptr;        // per-sample outputs of one launch
  int64_t sbuf_items = 0;
  uint32_t* wf_ctl = nullptr;    // control words, one kCtlBytes block per lane (layout of ctl_index)
  uint32_t* h_live = nullptr;    // pinned host copy of a live counter
  int64_t max_slots = 1 << 23;   // path slots per launch
  int64_t max_items = 1 << 28;   // samples per launch (sample buffer entries)
  int trace_blocks_per_sm = 0;   // 0 = occupancy limit
  int trace_occupancy = 0;       // occupancy limit of the DDA kernel (cached)
  int trace_steps = 16;          // DDA steps between refills of the trace kernel
  int trace_chunk = 128;         // queue records per warp atomic of the trace kernel
  int refill_min = 0;            // early refill of a trace warp below this many stepping lanes (0 = off)
  int trace_form = 0;            // DDA kernel form: 0 per-lane segment set-up, 1 pooled set-up
  uint64_t launches = 0;         // render kernels launched by this context
  cudaGraphExec_t rounds_exec = nullptr;   // eight rounds of every lane, replayed
  bool use_graphs = true;
  // the second and later lanes of a wavefront launch: streams, and the
  // events that fork them from `stream` and join them back
  static constexpr int kMaxLanes = 4;
  cudaStream_t lane_stream[kMaxLanes - 1] = {nullptr, nullptr, nullptr};
  cudaEvent_t lane_ready = nullptr;
  cudaEvent_t lane_done[kMaxLanes - 1] = {nullptr, nullptr, nullptr};
  int lanes = 2;                 // wavefront lanes run side by side (1 to kMaxLanes)
  unsigned long long* d_counters = nullptr;
  unsigned long long* d_queue = nullptr;
  int32_t* d_error = nullptr;

  // Device memory: budget-checked, with released blocks kept for reuse.  A
  // released block waits for the context's stream to go idle and joins the
  // cache (up to cache_limit bytes); alloc takes the smallest cached block of
  // the rounded size up to a quarter larger before it calls cudaMalloc, and
  // live plus cached bytes stay within the budget.
  int alloc(void** ptr, size_t bytes);
  void release(void* ptr);
  uint64_t trim(uint64_t keep);           // free cached blocks down to `keep` bytes; returns bytes freed
  bool caching = true;
  std::multimap<size_t, void*> cache;     // size -> block
  uint64_t cached = 0;
  uint64_t cache_limit = 2ull << 30;
  int ensure_scratch(size_t bytes);
  int ensure_noise();
  void log(const char* fmt, ...);
};

struct vt_scene {
  vt_context* ctx = nullptr;
  int32_t res[3] = {0, 0, 0};
  int32_t bdim[3] = {0, 0, 0};
  int32_t bsh[3] = {2, 2, 2};    // brick shape: log2 extents (4x4x4)
  float bmin[3], bmax[3], vsize[3];
  uint8_t* grid = nullptr;
  unsigned long long* bricks = nullptr;
  uint4* palette = nullptr;
  int32_t n_palette = 0;
  int32_t* emissive = nullptr;
  int64_t n_emissive = 0;
  uint64_t bytes = 0;
  uint32_t flags = 0;            // creation flags (emissive list policy for edits)
  uint64_t generation = 0;       // bumped by edits that move device buffers
  std::vector<vt_material> host_palette;
  // the reference's flat material table and the record offset of each
  // palette entry in it (-1: the entry has no record there)
  std::vector<float> mat_table;
  std::vector<int64_t> mat_offset;
  ~vt_scene();
};

struct vt_env {
  vt_context* ctx = nullptr;
  int32_t w = 0, h = 0;
  int32_t cdf_w = 0, cdf_h = 0;  // image the CDFs were built from (w, h, or the shrunk size)
  uint2* texels = nullptr;
  float* cdf_u = nullptr;
  float* cdf_v = nullptr;
  float integral = 0.0f;
  ~vt_env();
};

struct vt_job {
  vt_context* ctx = nullptr;
  const vt_scene* scene = nullptr;
  const vt_env* env = nullptr;
  vt_camera cam;
  vt_render_settings set;
  int32_t w = 0, h = 0;
  float4* sum = nullptr;
  float4* comp = nullptr;
  float4* staging = nullptr;
  int32_t samples = 0;
  int32_t integrator = 0;        // VT_INTEGRATOR_* (Renderer::m_currentIntegrator)
  uint64_t scene_generation = 0; // scene->generation when frame/dev were built
  vt::Frame frame;
  vt::JobDev dev;
  ~vt_job();
};

namespace vt {
// A named host-side range for profilers (NVTX; a no-op unless a tool such as
// ncu --nvtx is attached): the phases of a render show up as ranges named
// "vt.<phase>" around the kernels they launch.
struct Range {
  explicit Range(const char* name) { nvtxRangePushA(name); }
  ~Range() { nvtxRangePop(); }
  Range(const Range&) = delete;
  Range& operator=(const Range&) = delete;
};
int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);
int build_frame(vt_job* j);
// Frees everything a context owns (vt_destroy, and the server's own lane).
void release_context(vt_context* ctx);
// Locates vt_render_batch_fixed's device array on `device` (current) and
// loads the code that holds it (vt_fixed.cu); called by vt_create.
int fixed_scratch_setup(int device);
// Rebuilds a job's frame when its scene was edited since (scene->generation).
int refresh_job(vt_job* j);
// passes[i] samples per pixel for jobs[i]; kernel 1 = plain, 2 = wavefront.
int render_jobs(vt_context* ctx, vt_job* const* jobs, int32_t n, const int32_t* passes, int kernel,
                int tile_pixels, int blocks_per_sm, bool count);
// Wavefront form; `slots` path slots per launch (0 = context default).
int render_wavefront(vt_context* ctx, vt_job* const* jobs, int32_t n, const int32_t* passes, int slots,
                     int blocks_per_sm, bool count);
}  // namespace vt
