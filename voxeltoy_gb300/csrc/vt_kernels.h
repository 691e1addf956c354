// vt_kernels.h — host-side launchers of the CUDA kernels (internal API
// between the C-ABI runtime in vt_api.cu and the kernel translation units).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include "vt_internal.h"

namespace vt {

// One job as seen by the wavefront kernels: its uniforms, device pointers and
// the work it contributes to the launch.
struct JobEntry {
  Frame F;
  JobDev J;
  int32_t sample_base;    // first sample index of this launch
  int32_t passes;         // samples per pixel in this launch
  int64_t tile_begin;     // first global work item (sample) of this job
  int64_t n_pixels;
};

// ---- render (vt_render.cu)
cudaError_t launch_plain(const Frame& F, const JobDev& J, int sample_base, int passes,
                         unsigned long long* counters, cudaStream_t st);
cudaError_t launch_diag(const Frame& F, const JobDev& J, int sample, float4* out, HitRecord* hits,
                        unsigned long long* counters, cudaStream_t st);
// Wavefront path state: a stream of paths, structure of arrays over the
// stream positions.  Each round reads one stream and writes the next one
// compacted: the paths that continue first, then the new paths.
struct WfState {
  float4* a0;      // ro.xyz, -
  float4* a1;      // rd.xyz, item (uint bits)
  float4* a3;      // L.xyz, rng word
  float4* a4;      // T.xyz, bsdf_pdf
  float4* a5;      // nee_P.xyz (throughput * light sample), light (int bits); written and
                   // read only for paths with a shadow segment
  uint32_t* flags; // bounces | primary | has_cont | ext | shadow | active | NEE mask | job
};
// The hits k_wf_shade keeps for k_wf_hit, in hit-list order: Lambert hits
// from the front, the others from the back.
struct WfHitRecs {
  float4* h0;      // ro.xyz, item
  float4* h1;      // rd.xyz, flags
  float4* h2;      // L.xyz, rng word
  float4* h3;      // T.xyz, bsdf_pdf
  unsigned long long* h4;   // hit voxel x, y, z and DDA state, packed (pack_end)
};
// Control words of a wavefront launch, per round parity: records appended to
// the queue, records taken by the tracer, length of the stream the round
// writes, the item counter when the round started (64-bit), Lambert and other
// entries of the hit list.  Each word has its own 128-byte line, so atomics
// on different counters never queue behind each other in one L2 sector.
enum { CTL_QCOUNT = 0, CTL_QHEAD = 1, CTL_NEXT_N = 2, CTL_ITEM_SNAP = 3, CTL_HITS_LAMBERT = 4,
       CTL_HITS_OTHER = 5, CTL_REGEN_N = 6, CTL_PER_PARITY = 8 };
// Segment record tag of a queue entry that holds no segment (a new-path
// position that found no item).
constexpr uint32_t kNoSegment = 0xffffffffu;
constexpr int kCtlStride = 32;                                   // words per counter line
constexpr int kCtlNextItem = 2 * CTL_PER_PARITY * kCtlStride;    // word index of the item counter
constexpr size_t kCtlBytes = (size_t)(2 * CTL_PER_PARITY + 1) * kCtlStride * sizeof(uint32_t);
__host__ __device__ constexpr int ctl_index(int par, int k) { return (CTL_PER_PARITY * par + k) * kCtlStride; }

struct WfParams {
  const JobEntry* jobs;            // device array, tile_begin = first item of the job
  int32_t n_jobs;
  const Grid* grids;               // device array, DDA view of each job's volume
  WfState x[2];                    // round parity par reads x[par] and writes x[par ^ 1]
  unsigned long long* hits;        // [2][n_slots] segment ends (extension, shadow) by position, packed
                                   // (pack_end: voxel x, y, z and DDA state in 64 bits)
  WfHitRecs hr;
  int32_t n_slots;                 // stream capacity (paths in flight)
  float4* queue[2];                // segment records, two float4 each:
                                   // {origin.xyz, dir.x} {dir.yz, position << 1 | kind, job}
  uint32_t* ctl;                   // control words, see ctl_index
  unsigned long long* next_item;
  unsigned long long n_items;
  float4* sbuf;                    // per-item sample outputs
  unsigned long long* counters;    // nullable
  int32_t bricks_444;              // every job's bricks are 4x4x4 (the DDA kernel's fixed-shape form)
  int32_t trace_form;              // DDA kernel: 0 per-lane set-up, 1 pooled set-up (k_wf_trace_pool)
  uint32_t trace_chunk;            // queue records a trace warp takes per atomic (32-256)
  int32_t refill_min;              // trace warps refill early once fewer lanes step (0 = every
                                   // kTraceSteps steps only)
};
// Device bytes per stream position, and the carving of one allocation of
// slots * kWfSlotBytes bytes (256-byte aligned) into the buffers of P.
constexpr size_t kWfSlotBytes = 2 * (5 * sizeof(float4) + sizeof(uint32_t)) + 2 * sizeof(uint64_t) +
                                (4 * sizeof(float4) + sizeof(uint64_t)) + 8 * sizeof(float4);
void wf_carve(void* mem, size_t slots, WfParams& P);
// Launches of at most kWfParamJobs jobs pass their job and grid records as a
// kernel parameter as well, so the kernels read them through the constant
// cache instead of global memory.
constexpr int kWfParamJobs = 8;
constexpr int kWfMaxJobs = 1 << 15;   // jobs per wavefront launch (bits of the slot flags)
struct WfJobTable {
  JobEntry e[kWfParamJobs];
  Grid g[kWfParamJobs];
};
// A launch of one job: its records at fixed offsets of the parameter block,
// which the kernels read as constant operands.
struct WfOneJob {
  JobEntry e;
  Grid g;
};
// One round's shading: k_wf_shade over the stream, then k_wf_hit over the
// hits it keeps and k_wf_regen filling the rest of the next stream with new
// paths (persist_blocks blocks of 128 each for k_wf_hit, a multiple of 8;
// k_wf_regen scales it to its own residency).
// T (nullable): the launch's job and grid records; a one-job launch uses
// the WfOneJob form.
cudaError_t launch_wf_shade(const WfParams& P, int par, int persist_blocks, bool count, cudaStream_t st,
                            const WfJobTable* T = nullptr);
cudaError_t launch_wf_trace(const WfParams& P, int par, int blocks, int steps, bool count, cudaStream_t st,
                            const WfJobTable* T = nullptr);
cudaError_t launch_wf_accumulate(const JobEntry* jobs, int n_jobs, long long max_pixels, const float4* sbuf,
                                 cudaStream_t st);
int wf_trace_blocks_per_sm();
cudaError_t launch_trace_rays(const Frame& F, const JobDev& J, const float* origins, const float* dirs,
                              int64_t n, int32_t* out, cudaStream_t st);
cudaError_t launch_pick(const Frame& F, const JobDev& J, float x, float y, float* out_dist,
                        int32_t* out_voxel, cudaStream_t st);
// out: voxel x, y, z, hit (1) as int32 then the face normal as 3 floats.
cudaError_t launch_select(const Frame& F, const JobDev& J, float x, float y, float frag_z, int32_t* out,
                          cudaStream_t st);
cudaError_t launch_resolve(const float4* sum, int32_t w, int32_t h, int32_t samples, float exposure,
                           float inv_gamma, uint32_t flags, float4* out, cudaStream_t st);
cudaError_t launch_builtins(int32_t fn, const float* a, const float* b, float* out, int64_t n,
                            cudaStream_t st);
// `reps` L1-bypassing read sweeps of buf (n 16-byte words, n < 2^31) by
// `blocks` blocks of 512 threads; out holds blocks*512 words.
cudaError_t launch_l2_read(const uint4* buf, uint32_t n, int32_t reps, uint4* out, int blocks, cudaStream_t st);
// Check word of the bounds-checked build (VT_CHECKED); release builds give
// 0 and enabled = false.
cudaError_t read_check_word(uint32_t* word, bool* enabled, bool reset);

// ---- scene (vt_scene.cu)
cudaError_t launch_set_voxel(uint8_t* grid, unsigned long long* bricks, int32_t rx, int32_t ry, int32_t bx, int32_t by,
                             const BrickShape& sh, int32_t x, int32_t y, int32_t z, uint8_t entry, cudaStream_t st);
// max_entry (nullable): receives the largest palette entry of the volume.
cudaError_t launch_build_bricks(const uint8_t* grid, int32_t rx, int32_t ry, int32_t rz,
                                unsigned long long* bricks, int32_t bx, int32_t by, int32_t bz, const BrickShape& sh,
                                unsigned long long* max_entry, cudaStream_t st);
cudaError_t launch_emissive_flags(const uint8_t* grid, int32_t rx, int32_t ry, int32_t rz,
                                  const int32_t* emissive, int64_t n, uint8_t* keep, cudaStream_t st);
// Emissive voxels in increasing index order, in two launches:
// launch_emissive_count leaves in counts[0..chunks) each chunk's first output
// position and in counts[chunks] the total (counts holds chunks + 1 words,
// chunks = emissive_chunks(n_voxels)); launch_emissive_write then writes the
// total indices into out.
int64_t emissive_chunks(int64_t n_voxels);
cudaError_t launch_emissive_count(const uint8_t* grid, int64_t n_voxels, const uint8_t* emissive_entry,
                                  uint32_t* counts, cudaStream_t st);
cudaError_t launch_emissive_write(const uint8_t* grid, int64_t n_voxels, const uint8_t* emissive_entry,
                                  const uint32_t* offsets, int32_t* out, cudaStream_t st);
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
// FP16 texels of the w x h image, and the CDFs and integral of the cw x ch
// image (the same image, or it shrunk by k_env_shrink_lum; sin_theta holds
// ch row weights).  bad: set to the smallest index of a non-finite texel
// (the caller sets it to ~0 first).
cudaError_t launch_env_build(const float* rgb, int32_t w, int32_t h, int32_t cw, int32_t ch, const EnvScratch& S,
                             uint2* texels, float* cdf_u, float* cdf_v, float* integral, uint32_t* bad,
                             cudaStream_t st);
// CDFs of a caller-supplied function (w*h floats) without blur or weighting.
cudaError_t launch_cdf(const float* func, int32_t w, int32_t h, const EnvScratch& S, float* cdf_u,
                       float* cdf_v, float* integral, cudaStream_t st);
// Mesh input checks and placement on the device.  bad: (1 << 32 | index) of
// the largest triangle index at or past the vertex count, 0 if none.
struct MeshPrep {
  uint32_t kmin[3], kmax[3];   // order-preserving keys of the vertex bounds
  unsigned long long bad;
};
// The MeshPrep record inside a voxelization's scratch.
MeshPrep* voxelize_prep_record(void* scratch, int64_t n_tris);
// Checks the indices against nv and, with fit, applies computeMeshTransform
// and the scaling to voxel space to the nv vertices at V in place.
cudaError_t launch_mesh_prep(float* V, int64_t nv, const uint32_t* I, int64_t n_tris, bool fit, int32_t rx,
                             int32_t ry, int32_t rz, MeshPrep* P, int sm_count, cudaStream_t st);
// mode 0 = THIN, 1 = FAT; reference_bounds clamps each triangle's swizzled
// voxel range against the unswizzled resolution as the reference does;
// triangles with an index at or past n_vertices are skipped.
// bricks (nullable): the padded brick grid (bx, by bricks per row / slice
// inside the border), prepared by launch_bricks_init; every voxel written
// also sets its occupancy bit.  scratch: voxelize_scratch_bytes(n_tris)
// bytes of device memory for the list of large triangles; large_blocks:
// blocks of the block-per-triangle kernel.
size_t voxelize_scratch_bytes(int64_t n_tris);
cudaError_t launch_voxelize(const float* verts_voxel_space, int64_t n_vertices, const uint32_t* indices,
                            int64_t n_tris, int32_t rx, int32_t ry, int32_t rz, int32_t mode, bool reference_bounds,
                            uint8_t* grid, uint8_t value, unsigned long long* bricks, int32_t bx, int32_t by,
                            const BrickShape& sh, void* scratch, int large_blocks, cudaStream_t st);
// Bricks of an empty volume: border bricks all set, interior bricks set only
// for the voxels beyond the volume's extent.
cudaError_t launch_bricks_init(unsigned long long* bricks, int32_t rx, int32_t ry, int32_t rz, int32_t bx,
                               int32_t by, int32_t bz, const BrickShape& sh, cudaStream_t st);

}  // namespace vt
