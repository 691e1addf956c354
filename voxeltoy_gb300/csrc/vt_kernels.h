// vt_kernels.h — host-side launchers of the CUDA kernels (internal API
// between the C-ABI runtime in vt_api.cu and the kernel translation units).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include "vt_internal.h"

namespace vt {

// One job as seen by the persistent kernel: its uniforms, device pointers and
// the work it contributes to the launch.
struct JobEntry {
  Frame F;
  JobDev J;
  int32_t sample_base;    // first sample index of this launch
  int32_t passes;         // samples per pixel in this launch
  int64_t tile_begin;     // first global tile index of this job
  int64_t n_pixels;
};

// ---- render (vt_render.cu)
cudaError_t launch_plain(const Frame& F, const JobDev& J, int sample_base, int passes,
                         unsigned long long* counters, cudaStream_t st);
cudaError_t launch_diag(const Frame& F, const JobDev& J, int sample, float4* out, HitRecord* hits,
                        unsigned long long* counters, cudaStream_t st);
struct PersistentParams {
  const JobEntry* jobs;          // device array
  int32_t n_jobs;
  int64_t n_tiles;               // total tiles over all jobs
  int32_t tile_pixels;           // multiple of 32
  unsigned long long* queue;     // device work counter, zeroed before launch
  unsigned long long* counters;  // nullable
  int32_t* error;                // device error word
};
cudaError_t launch_persistent(const PersistentParams& P, int blocks, int threads, bool count,
                              cudaStream_t st);
int persistent_max_blocks_per_sm(int threads);
cudaError_t launch_trace_rays(const Frame& F, const JobDev& J, const float* origins, const float* dirs,
                              int64_t n, int32_t* out, cudaStream_t st);
cudaError_t launch_pick(const Frame& F, const JobDev& J, float x, float y, float* out_dist,
                        int32_t* out_voxel, cudaStream_t st);
cudaError_t launch_resolve(const float4* sum, int32_t w, int32_t h, int32_t samples, float exposure,
                           float inv_gamma, uint32_t flags, float4* out, cudaStream_t st);
cudaError_t launch_builtins(int32_t fn, const float* a, const float* b, float* out, int64_t n,
                            cudaStream_t st);

// ---- scene (vt_scene.cu)
cudaError_t launch_build_bricks(const uint8_t* grid, int32_t rx, int32_t ry, int32_t rz,
                                unsigned long long* bricks, int32_t bx, int32_t by, int32_t bz,
                                cudaStream_t st);
cudaError_t launch_emissive_flags(const uint8_t* grid, int32_t rx, int32_t ry, int32_t rz,
                                  const int32_t* emissive, int64_t n, uint8_t* keep, cudaStream_t st);
cudaError_t launch_find_emissive(const uint8_t* grid, int64_t n_voxels, const uint8_t* emissive_entry,
                                 int32_t* out, unsigned long long* count, int64_t capacity,
                                 cudaStream_t st);
// Scratch buffers of the environment build (device memory, caller-owned).
struct EnvScratch {
  float* lum;        // w*h luminance of the FP16 texels
  float* tmp;        // w*h horizontal blur
  float* func;       // w*h sampled function: blurred luminance * sin(theta)
  float* sin_theta;  // h row weights sin(pi (y + 0.5) / h), computed on the host
  double* row_pre;   // h*(w+1) row prefix sums
  double* row_int;   // h row integrals
  double* marg_pre;  // h+1 marginal prefix sums
};
cudaError_t launch_env_build(const float* rgb, int32_t w, int32_t h, const EnvScratch& S, uint2* texels,
                             float* cdf_u, float* cdf_v, float* integral, cudaStream_t st);
// CDFs of a caller-supplied function (w*h floats) without blur or weighting.
cudaError_t launch_cdf(const float* func, int32_t w, int32_t h, const EnvScratch& S, float* cdf_u,
                       float* cdf_v, float* integral, cudaStream_t st);
cudaError_t launch_voxelize(const float* verts_voxel_space, const uint32_t* indices, int64_t n_tris,
                            int32_t rx, int32_t ry, int32_t rz, int32_t mode, uint8_t* grid,
                            uint8_t value, cudaStream_t st);
cudaError_t launch_transform_vertices(const float* in, int64_t n, const float* m44_row_major,
                                      int32_t rx, int32_t ry, int32_t rz, float* out, cudaStream_t st);

}  // namespace vt
