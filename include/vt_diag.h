/*
 * vt_diag.h — diagnostic entry points of the GB300 voxel renderer.
 *
 * These have no counterpart in the reference's Renderer interface: they
 * expose intermediate results of the same kernels that vt.h drives (per-sample
 * radiance, first hits, DDA results of arbitrary rays, event counters, the
 * environment CDFs of a raw function) so that they can be compared with a CPU
 * restatement of the reference shaders, and select the kernel form used by
 * vt_job_render for measurement.
 */
#ifndef VT_DIAG_H
#define VT_DIAG_H

#include "vt.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Event counters (per launch, summed over paths):
 * [0] paths, [1] DDA cells tested, [2] palette records read,
 * [3] environment texel evaluations, [4] CDF entries probed,
 * [5] emissive-list reads, [6] DDA segments started, [7] DDA cells tested
 * inside bricks that hold no occupied voxel, [8] wavefront stream positions
 * shaded (one per path and round; 0 in the plain form). */
#define VT_DIAG_NUM_COUNTERS 9

/* Trace caller-supplied rays through the job's scene with the DDA of
 * src/shaders/shared/dda.h:7-100 (traverse with the default step cap).
 * origins/dirs: n*3 floats in world space.  out: n*4 int32 =
 * voxel x, y, z, flags (normal code | hit << 8 | ground << 9 | steps << 10),
 * normal code = (nx+1) | (ny+1) << 2 | (nz+1) << 4 of the hit face. */
VT_API int vt_diag_trace_rays(vt_job* job, const float* origins, const float* dirs,
                              int64_t n, int32_t* out);

/* Trace one sample per pixel with sample index `sample` without touching the
 * accumulation: rgba receives the per-sample output (width*height*4 floats),
 * hits (nullable) the first-hit record of each pixel (width*height*4 int32,
 * same layout as vt_diag_trace_rays), counters (nullable) the event counts. */
VT_API int vt_diag_samples(vt_job* job, int32_t sample, float* rgba, int32_t* hits,
                           uint64_t* counters);

/* Render like vt_job_render and also return the event counters of the
 * launch (counters: VT_DIAG_NUM_COUNTERS entries). */
VT_API int vt_diag_render_counted(vt_job* job, int32_t passes, uint64_t* counters,
                                  int32_t* result);

/* Kernel form used by vt_job_render and vt_render_batch when their options
 * do not say: 1 = plain (one thread per pixel, one launch per pass),
 * 2 = wavefront (path slots over all jobs' work items). */
VT_API int vt_diag_set_kernel(vt_context* ctx, int32_t kernel);

/* Wavefront rounds replayed as a captured CUDA graph (enabled = 1, the
 * default) or launched one by one (0).  Results are identical. */
VT_API int vt_diag_set_graphs(vt_context* ctx, int32_t enabled);

/* Wavefront lanes: 2 (the default) runs two independent wavefronts over the
 * two halves of a launch's samples on two streams, so that one's shading
 * overlaps the other's DDA; 1 runs one, 3 and 4 as many.  Results are
 * identical. */
VT_API int vt_diag_set_lanes(vt_context* ctx, int32_t lanes);

/* Evaluate a builtin of the renderer on the GPU: fn 0 sin, 1 cos, 2 pow(a, b),
 * 3 acos, 4 atan2(a, b), 5 log2, 6 exp2, 7 float -> half -> float. */
VT_API int vt_diag_builtins(vt_context* ctx, int32_t fn, const float* a, const float* b,
                            float* out, int64_t n);

/* Build the importance-sampling CDFs of a raw non-negative function
 * (width*height floats) on the GPU, without blur or sin(theta) weight:
 * the known-answer examples of src/renderer/image.cpp:107-154. */
VT_API int vt_diag_cdf_from_function(vt_context* ctx, const float* func, int32_t width,
                                     int32_t height, float* cdf_u, float* cdf_v,
                                     float* integral);

/* Tuning of the wavefront form (path_slots, trace_steps and max_items <= 0
 * and trace_blocks_per_sm < 0 keep their value):
 * path_slots paths in flight per launch (default 2M), trace_blocks_per_sm
 * resident blocks of the DDA kernel (0: occupancy limit, the default),
 * trace_steps DDA steps between ray-pool refills (4, 8, 16 or 32; default 16),
 * max_items samples per launch (sample-buffer entries, default 2^28). */
VT_API int vt_diag_set_tuning(vt_context* ctx, int64_t path_slots, int32_t trace_blocks_per_sm,
                              int32_t trace_steps, int64_t max_items);

/* The scene's occupancy bit-bricks: one 64-bit word per brick of
 * 2^sx x 2^sy x 2^sz voxels (vt_scene_get_brick_shape; bit
 * (x & (2^sx-1)) | (y & (2^sy-1)) << sx | (z & (2^sz-1)) << (sx+sy), set =
 * occupied or outside the volume), on the brick grid padded by one brick on
 * every side, x fastest: (bx+2)*(by+2)*(bz+2) words, bx = ceil(rx/2^sx) ...
 * *n_words receives that count; out (nullable) receives the words. */
VT_API int vt_diag_scene_bricks(const vt_scene* scene, uint64_t* out, size_t bytes, int64_t* n_words);

/* Bounds-checked build (libvoxeltoy_checked.so, compiled with VT_CHECKED):
 * every data-dependent gather of the path tracer checks its index, and a
 * failed check ORs a bit into a device word and reads a neutral value
 * instead, without trapping: 1 brick word, 2 voxel, 4 palette entry,
 * 8 emissive-list entry, 16 environment texel, 32 CDF entry, 64 sample-
 * buffer item, 128 noise texel.  *word receives the bits set since the
 * last call (the word is then cleared; the context's stream is synchronised
 * first); *enabled is 1 in the checked build and 0 (word 0) otherwise. */
VT_API int vt_diag_check_word(vt_context* ctx, uint32_t* word, int32_t* enabled);

/* L2 read bandwidth of this GPU in GB/s: one launch of `reps` sweeps over a
 * device buffer of `bytes` bytes (multiple of 16, 1 MiB to 1 GiB; choose it
 * well below the L2 size) with loads that bypass L1, after one warm sweep;
 * timed with CUDA events on the context's stream.  The buffer is allocated
 * and freed by the call. */
VT_API int vt_diag_l2_read_bandwidth(vt_context* ctx, int64_t bytes, int32_t reps, double* gbs);

/* Form of the wavefront's DDA kernel: 0 (the default) sets each segment up
 * in the lane that steps it, refilling lanes every trace_steps steps; 1
 * keeps a per-warp pool of set-up segments in shared memory, sets up a
 * warp's worth of segments at once and refills lanes from the pool after
 * each batch of trace_steps steps (4, 8 or 16).  Results are identical. */
VT_API int vt_diag_set_trace_form(vt_context* ctx, int32_t form);

/* Tuning of the wavefront form's DDA kernel (values <= 0, and refill_min
 * < 0, keep their setting): queue_chunk queue records a warp takes with one
 * atomic (a multiple of 32 in [32, 1024], default 128); refill_min: a warp
 * stops stepping and starts its lanes' next segments as soon as fewer than
 * refill_min of its lanes still step (checked every fourth step; 0, the
 * default, refills only every trace_steps steps).  Results are identical
 * for every setting. */
VT_API int vt_diag_set_trace_tuning(vt_context* ctx, int32_t queue_chunk, int32_t refill_min);

/* Number of rendering kernels (plain, wavefront shade/trace/accumulate) the
 * context has launched so far. */
VT_API int vt_diag_launch_count(const vt_context* ctx, uint64_t* launches);

/* The cudaStream_t on which the context issues its work (for timing with
 * CUDA events recorded on that stream). */
VT_API int vt_diag_stream(vt_context* ctx, void** stream);

/* Copy the environment's FP16 RGBA texels (width*height*4 uint16). */
VT_API int vt_diag_env_texels(const vt_env* env, uint16_t* out, size_t bytes);

/* Replace / read the 1024x1024 RGBA noise table used by VT_RNG_NOISE_TABLE
 * (src/renderer/renderer.cpp:739-760).  By default the table holds
 * (splitmix64(seed + i) >> 40) * 2^-24 for i in [0, 4M), seed 0. */
VT_API int vt_diag_set_noise_table(vt_context* ctx, const float* rgba, size_t bytes);
VT_API int vt_diag_get_noise_table(vt_context* ctx, float* rgba, size_t bytes);

#ifdef __cplusplus
}
#endif
#endif /* VT_DIAG_H */
