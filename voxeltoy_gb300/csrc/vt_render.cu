// vt_render.cu — path-tracing kernels.
//
//   k_plain       one thread per pixel, `passes` samples per launch; the
//                 reference's one-pass-per-draw structure (renderer.cpp:584-611)
//   k_persistent  one launch for many jobs and passes: warps pull
//                 (job, 32-pixel tile) work items from a device counter, and
//                 every lane regenerates paths for its pixel until the tile's
//                 samples are done.  Lanes whose segment ended wait until at
//                 least half the warp needs an event, so shading runs with
//                 most of the warp active while the DDA loop keeps running
//                 for the rest.
//   k_diag        per-sample output and first-hit record (parity tests)
//   k_trace_rays  DDA of caller-supplied rays (parity tests)
//   k_pick        focal-distance pick of one pixel (focalDistance.vs:45-81)
//   k_resolve     average = sum / n (+ tonemap / flip) for readback
#include "vt_kernels.h"
#include "vt_shade.cuh"

namespace vt {

template <bool kCount>
__device__ __forceinline__ void flush_counters(Cnt<kCount>& cnt, unsigned long long* out) {
  if (!kCount || out == nullptr) return;
#pragma unroll
  for (int i = 0; i < C_NUM; ++i) {
    unsigned long long v = cnt.c[i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&out[i], v);
  }
}

// ------------------------------------------------------------------ plain
template <bool kCount>
__global__ void __launch_bounds__(128) k_plain(const Frame F, const JobDev J, int sample_base, int passes,
                                               unsigned long long* counters) {
  Cnt<kCount> cnt;
#pragma unroll
  for (int i = 0; i < C_NUM; ++i) cnt.c[i] = 0;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = F.width * F.height;
  if (idx < n) {
    const int px = idx % F.width, py = idx / F.width;
    float4 sum = J.sum[idx], comp = J.comp[idx];
    for (int k = 0; k < passes; ++k) {
      const float4 v = trace_sample(F, J, px, py, sample_base + k, cnt, (HitRecord*)nullptr);
      kahan_add(sum, comp, v);
    }
    J.sum[idx] = sum;
    J.comp[idx] = comp;
  }
  flush_counters(cnt, counters);
}

cudaError_t launch_plain(const Frame& F, const JobDev& J, int sample_base, int passes,
                         unsigned long long* counters, cudaStream_t st) {
  const int n = F.width * F.height;
  const int threads = 128;
  const int blocks = (n + threads - 1) / threads;
  if (counters) k_plain<true><<<blocks, threads, 0, st>>>(F, J, sample_base, passes, counters);
  else k_plain<false><<<blocks, threads, 0, st>>>(F, J, sample_base, passes, nullptr);
  return cudaGetLastError();
}

// ------------------------------------------------------------------- diag
__global__ void k_diag(const Frame F, const JobDev J, int sample, float4* out, HitRecord* hits,
                       unsigned long long* counters) {
  Cnt<true> cnt;
#pragma unroll
  for (int i = 0; i < C_NUM; ++i) cnt.c[i] = 0;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = F.width * F.height;
  if (idx < n) {
    const int px = idx % F.width, py = idx / F.width;
    HitRecord h;
    const float4 v = trace_sample(F, J, px, py, sample, cnt, &h);
    out[idx] = v;
    if (hits) hits[idx] = h;
  }
  flush_counters(cnt, counters);
}

cudaError_t launch_diag(const Frame& F, const JobDev& J, int sample, float4* out, HitRecord* hits,
                        unsigned long long* counters, cudaStream_t st) {
  const int n = F.width * F.height;
  k_diag<<<(n + 127) / 128, 128, 0, st>>>(F, J, sample, out, hits, counters);
  return cudaGetLastError();
}

// ------------------------------------------------------------- persistent
constexpr int kPersistThreads = 128;
constexpr int kWarpsPerBlock = kPersistThreads / 32;

template <bool kCount>
__global__ void __launch_bounds__(kPersistThreads) k_persistent(const PersistentParams P) {
  __shared__ JobEntry s_job[kWarpsPerBlock];
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  JobEntry& E = s_job[wid];
  const Frame& F = E.F;
  const JobDev& J = E.J;
  Cnt<kCount> cnt;
#pragma unroll
  for (int i = 0; i < C_NUM; ++i) cnt.c[i] = 0;
  int cur_job = -1;
  const int tiles_per_item = P.tile_pixels >> 5;   // lane owns tiles_per_item pixels, one after another

  for (;;) {
    unsigned long long item = 0;
    if (lane == 0) item = atomicAdd(P.queue, 1ull);
    item = __shfl_sync(0xffffffffu, item, 0);
    if ((long long)item >= P.n_tiles) break;
    // locate the job of this tile: binary search over tile_begin
    int lo = 0, hi = P.n_jobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if ((long long)__ldg(&P.jobs[mid].tile_begin) <= (long long)item) lo = mid; else hi = mid - 1;
    }
    if (lo != cur_job) {
      __syncwarp();
      const int words = (int)(sizeof(JobEntry) / 4);
      const uint32_t* src = reinterpret_cast<const uint32_t*>(&P.jobs[lo]);
      uint32_t* dst = reinterpret_cast<uint32_t*>(&E);
      for (int w = lane; w < words; w += 32) dst[w] = __ldg(&src[w]);
      __syncwarp();
      cur_job = lo;
    }
    const long long tile = (long long)item - E.tile_begin;
    const int passes = E.passes;
    const int base = E.sample_base;
    // lane-local work: pixels tile*tile_pixels + lane + 32*k, k < tiles_per_item
    int k_pix = 0;
    long long pix = tile * P.tile_pixels + lane;
    bool active = pix < E.n_pixels;
    int sample = 0;
    Path p;
    Dda s;
    float4 sum = make_float4(0.f, 0.f, 0.f, 0.f), comp = sum;
    if (active) {
      sum = J.sum[pix]; comp = J.comp[pix];
      path_start(F, J, p, s, (int)(pix % F.width), (int)(pix / F.width), base, cnt);
    }
    for (;;) {
      // traversal: keep stepping while more than half of the live lanes are mid-segment
      for (;;) {
        const bool run = active && p.phase != PH_DONE && s.state == DDA_RUNNING;
        const unsigned live = __ballot_sync(0xffffffffu, active);
        const unsigned running = __ballot_sync(0xffffffffu, run);
        if (live == 0u || running == 0u || 2 * __popc(running) < __popc(live)) break;
        if (run) dda_advance(F, J, s, 8, cnt);
      }
      if (active) {
        if (p.phase != PH_DONE && s.state != DDA_RUNNING) path_event(F, J, p, s, cnt);
        if (p.phase == PH_DONE) {
          kahan_add(sum, comp, path_output(F, p));
          ++sample;
          if (sample < passes) {
            path_start(F, J, p, s, (int)(pix % F.width), (int)(pix / F.width), base + sample, cnt);
          } else {
            J.sum[pix] = sum; J.comp[pix] = comp;
            ++k_pix;
            pix += 32;
            active = (k_pix < tiles_per_item) && pix < E.n_pixels;
            sample = 0;
            if (active) {
              sum = J.sum[pix]; comp = J.comp[pix];
              path_start(F, J, p, s, (int)(pix % F.width), (int)(pix / F.width), base, cnt);
            }
          }
        }
      }
      if (__ballot_sync(0xffffffffu, active) == 0u) break;
    }
  }
  flush_counters(cnt, P.counters);
}

int persistent_max_blocks_per_sm(int threads) {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent<false>, threads, 0);
  return n;
}

cudaError_t launch_persistent(const PersistentParams& P, int blocks, int threads, bool count,
                              cudaStream_t st) {
  (void)threads;
  if (count) k_persistent<true><<<blocks, kPersistThreads, 0, st>>>(P);
  else k_persistent<false><<<blocks, kPersistThreads, 0, st>>>(P);
  return cudaGetLastError();
}

// ------------------------------------------------------------- trace rays
// out[4*i] = voxel x, y, z, flags (hit << 8 | ground << 9 | normal code).
__global__ void k_trace_rays(const Frame F, const JobDev J, const float* origins, const float* dirs,
                             int64_t n, int32_t* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Cnt<false> cnt;
  const v3 o = mk3(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]);
  const v3 d = mk3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
  Dda s;
  dda_begin(F, s, o, d);
  if (s.state == DDA_RUNNING) dda_advance(F, J, s, 0x7fffffff, cnt);
  const bool h = dda_hit(F, s);
  int flags = (h ? 1 : 0) << 8 | ((h && s.state != DDA_HIT) ? 1 : 0) << 9 | (s.steps << 10);
  if (h) {
    const Basis b = voxel_basis(F, s.x, s.y, s.z, o, d);
    flags |= ((int)b.normal.x + 1) | (((int)b.normal.y + 1) << 2) | (((int)b.normal.z + 1) << 4);
  }
  out[4 * i] = s.x; out[4 * i + 1] = s.y; out[4 * i + 2] = s.z; out[4 * i + 3] = flags;
}

cudaError_t launch_trace_rays(const Frame& F, const JobDev& J, const float* origins, const float* dirs,
                              int64_t n, int32_t* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_trace_rays<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(F, J, origins, dirs, n, out);
  return cudaGetLastError();
}

// ------------------------------------------------------------------- pick
// focalDistance.vs:45-81: generateRay with rngOffset (0,0) and no pixel
// jitter consumption difference (the pinhole draws its jitter from the
// sequence start), AABB clip, traverse, exact voxel distance.
__global__ void k_pick(const Frame F, const JobDev J, float x, float y, float* out_dist, int32_t* out_voxel) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Cnt<false> cnt;
  Rng rng;
  rng.pixel = 0; rng.sample = 0; rng.call = 0; rng.ox = 0; rng.oy = 0;
  v3 o, d;
  generate_ray(F, J, mk3(x, y, 0.0f), rng, o, d);
  *out_dist = kInfinity;
  out_voxel[0] = out_voxel[1] = out_voxel[2] = -1;
  const float t = ray_aabb(o, d, ld3(F.bmin), ld3(F.bmax));
  if (t < 0.0f) return;
  Dda s;
  dda_begin(F, s, o + t * d, d);
  if (s.state == DDA_RUNNING) dda_advance(F, J, s, 0x7fffffff, cnt);
  if (!dda_hit(F, s)) return;
  const v3 vs = ld3(F.vsize);
  const v3 vmin = mk3((float)s.x, (float)s.y, (float)s.z) * vs + ld3(F.bmin);
  *out_dist = ray_aabb(o, d, vmin, vmin + vs);
  out_voxel[0] = s.x; out_voxel[1] = s.y; out_voxel[2] = s.z;
}

cudaError_t launch_pick(const Frame& F, const JobDev& J, float x, float y, float* out_dist,
                        int32_t* out_voxel, cudaStream_t st) {
  k_pick<<<1, 32, 0, st>>>(F, J, x, y, out_dist, out_voxel);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- resolve
__global__ void k_resolve(const float4* sum, int32_t w, int32_t h, int32_t samples, float exposure,
                          float inv_gamma, uint32_t flags, float4* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)w * h) return;
  const int x = (int)(i % w), y = (int)(i / w);
  float4 v = sum[i];
  const float n = samples > 0 ? (float)samples : 1.0f;
  v.x = v.x / n; v.y = v.y / n; v.z = v.z / n; v.w = v.w / n;
  if (flags & 2u) {
    v.x = vtb::vpow(v.x * exposure, inv_gamma);
    v.y = vtb::vpow(v.y * exposure, inv_gamma);
    v.z = vtb::vpow(v.z * exposure, inv_gamma);
  }
  const int oy = (flags & 1u) ? (h - 1 - y) : y;
  out[(int64_t)oy * w + x] = v;
}

cudaError_t launch_resolve(const float4* sum, int32_t w, int32_t h, int32_t samples, float exposure,
                           float inv_gamma, uint32_t flags, float4* out, cudaStream_t st) {
  const int64_t n = (int64_t)w * h;
  if (n <= 0) return cudaSuccess;
  k_resolve<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(sum, w, h, samples, exposure, inv_gamma, flags, out);
  return cudaGetLastError();
}

// --------------------------------------------------------------- builtins
__global__ void k_builtins(int32_t fn, const float* a, const float* b, float* out, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float x = a[i];
  float r;
  switch (fn) {
    case 0: r = vtb::vsin(x); break;
    case 1: r = vtb::vcos(x); break;
    case 2: r = vtb::vpow(x, b[i]); break;
    case 3: r = vtb::vacos(x); break;
    case 4: r = vtb::vatan2(x, b[i]); break;
    case 5: r = vtb::vlog2(x); break;
    case 6: r = vtb::vexp2(x); break;
    case 7: r = vtb::h2f(vtb::f2h(x)); break;
    default: r = 0.0f; break;
  }
  out[i] = r;
}

cudaError_t launch_builtins(int32_t fn, const float* a, const float* b, float* out, int64_t n,
                            cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_builtins<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(fn, a, b, out, n);
  return cudaGetLastError();
}

}  // namespace vt
