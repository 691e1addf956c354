/*
 * vt_oracle.h — CPU restatement of voxelToy's path-tracing pass and mesh
 * voxelizer, used ONLY as test infrastructure: the parity tests, the smoke
 * check and the CPU-baseline leg of the benchmark call it as the checker.
 * Nothing in the product links or calls it.
 *
 * It transcribes the reference's GLSL (src/shaders/...) and host code
 * (src/renderer/..., src/voxelize/..., src/camera/...) line by line; each
 * function in vt_oracle.cpp cites the lines it follows.  It is templated on
 * the arithmetic type: the float build evaluates the GLSL builtins with the
 * definitions shared with the GPU kernels (so the two can be compared bit for
 * bit); the double build uses libm in double precision and is the reference
 * for converged-image error.
 *
 * Parity status: the reference cannot be built here (its path is OpenGL 4.3
 * GLSL and its host side needs Qt, OpenImageIO, OpenEXR/Imath and boost), so
 * this restatement is pinned only by the known-answer examples the reference
 * documents (the CDF example of src/renderer/image.cpp:107-154 and the
 * binary-search example of src/shaders/envLight/envMapSample.h:10-21) and by
 * analytic known answers; the rest of its parity with the reference is
 * unpinned.
 */
#ifndef VT_ORACLE_H
#define VT_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* CameraParameters (src/camera/cameraParameters.h:117-129), world units. */
typedef struct orc_camera {
  float eye[3];
  float target[3];
  float fov_y;
  float near_distance;
  float far_distance;
  float focal_distance;
  float lens_radius;
  int32_t lens_model;   /* 0 pinhole, 1 thin lens, 2 orthographic */
} orc_camera;

/* RenderSettings + integrator uniforms (renderSettings.h:6-29, pathTracer.fs:25-44). */
typedef struct orc_settings {
  int32_t max_bounces;
  int32_t max_samples;
  int32_t rr_start_bounce;
  float gamma;
  float exposure;
  float nee_emission_scale;
  float wireframe_opacity;
  float wireframe_thickness;
  float background_top[3];
  float background_bottom[3];
  float background_rotation;
  int32_t selected_voxel[3];
  int32_t select_enabled;
  int32_t ground_material;
  uint32_t quirks;
  int32_t rng_mode;     /* 0 philox, 1 noise table */
  uint32_t seed;
  int32_t integrator;   /* 0 pathTracer.fs, 1 editMode.fs */
} orc_settings;

/* One material record: type, emission[3], albedo[3], roughness. */
typedef struct orc_material {
  int32_t type;
  float emission[3];
  float albedo[3];
  float roughness;
} orc_material;

typedef struct orc_scene {
  int32_t res[3];
  const uint8_t* grid;          /* palette entry + 1, 0 = empty */
  const orc_material* palette;  /* quantised to IEEE half by the oracle */
  int32_t n_palette;
  const int32_t* emissive;
  int64_t n_emissive;
} orc_scene;

/* Environment image: texels == NULL selects the gradient background. */
typedef struct orc_env {
  int32_t w, h;
  const uint16_t* texels;   /* w*h*4 IEEE halves (RGBA) */
  const float* cdf_u;       /* (cdf_w+1)*cdf_h */
  const float* cdf_v;       /* cdf_h+1 */
  float integral;
  int32_t cdf_w, cdf_h;     /* size of the image the CDFs were built from; 0 = w, h */
} orc_env;

/* Camera uniforms of Renderer::updateCamera (renderer.cpp:343-397):
 * out[0:16] proj, [16:32] inverse proj, [32:48] inverse model-view (row-major),
 * [48:52] viewport. */
int orc_camera_uniforms(const orc_camera* cam, int32_t width, int32_t height, float* out);

/* Environment build with options: flags bit 0 builds the CDFs and the
 * integral from the image shrunk to at most 512 texels on its long axis
 * (calculateCDF, image.cpp:14, 308-320; the size from the reference's float
 * arithmetic, an area-weighted box filter over the FP16 texels standing in
 * for OpenImageIO's resize), while the texels stay full size.  cdf_size
 * receives the CDF image's width and height. */
int orc_build_env_ex(const float* rgb, int32_t w, int32_t h, int32_t chunk, uint32_t flags, uint16_t* texels,
                     float* cdf_u, float* cdf_v, float* integral, int32_t* cdf_size);
/* The reference's CDF image size for a w x h environment (image.cpp:314-317). */
void orc_cdf_size(int32_t w, int32_t h, int32_t* cw, int32_t* ch);

/* CameraParameters defaults (cameraParameters.cpp:7-17): target 0, eye at
 * distance 100 on -Z, near 0.1, far 10000, 50 mm on a 36 mm film, pinhole,
 * focus at the pick buffer's initial value. */
void orc_camera_default(orc_camera* cam);
/* CameraParameters::orbitAroundTarget (cameraParameters.cpp:84-94):
 * eye = target - |target - eye| * (sin t cos p, cos t, sin t sin p). */
void orc_camera_orbit(orc_camera* cam, float theta, float phi);
/* RenderSettings defaults with every reference quirk on
 * (renderSettings.h, pathTracer.fs:25-26 background colours). */
void orc_settings_default(orc_settings* s);

/* One sample per pixel (sample index `sample`): per-sample output rgba
 * (w*h*4) and first-hit records hits (w*h*4 int32, nullable).
 * precision: 32 or 64.  counters (nullable): 8 event counts. */
int orc_render_samples(const orc_camera* cam, const orc_settings* s, const orc_scene* scene,
                       const orc_env* env, const float* noise, int32_t width, int32_t height,
                       int32_t sample, int32_t precision, int32_t threads, float* rgba,
                       int32_t* hits, uint64_t* counters);

/* spp samples per pixel starting at sample 0, accumulated with the running
 * average of accumulation.fs:10-17 in the working precision; out = average
 * (w*h*4).  rows [row0, row1) only (row1 <= 0 means all rows). */
int orc_render_average(const orc_camera* cam, const orc_settings* s, const orc_scene* scene,
                       const orc_env* env, const float* noise, int32_t width, int32_t height,
                       int32_t spp, int32_t precision, int32_t threads, int32_t row0,
                       int32_t row1, float* rgba, uint64_t* counters);

/* DDA of arbitrary rays (dda.h:7-100); out n*4 int32 as the GPU diagnostic. */
int orc_trace_rays(const orc_scene* scene, const float* origins, const float* dirs, int64_t n,
                   uint32_t quirks, int32_t* out);

/* Focal-distance pick (focalDistance.vs:45-81). */
int orc_pick(const orc_camera* cam, const orc_settings* s, const orc_scene* scene,
             const float* noise, int32_t width, int32_t height, float x, float y,
             float* distance, int32_t* voxel);

/* Environment: FP16 texels, luminance, 3x3 blur, sin weight, FP64 prefix
 * CDFs.  chunk = 32 reproduces the GPU's association order; chunk = 0 sums
 * strictly left to right. */
int orc_build_env(const float* rgb, int32_t w, int32_t h, int32_t chunk, uint16_t* texels,
                  float* cdf_u, float* cdf_v, float* integral);
int orc_cdf_from_function(const float* func, int32_t w, int32_t h, int32_t chunk, float* cdf_u,
                          float* cdf_v, float* integral);
/* The reference's own single-precision CDF of calculateCDF (image.cpp:176-280)
 * for a function given directly (no resize/blur): known-answer checks. */
int orc_cdf_reference_float(const float* func, int32_t w, int32_t h, float* cdf_u, float* cdf_v);
/* binarySearchCDFV (envMapSample.h:70-94) over cdf[0..n). */
int32_t orc_binary_search(const float* cdf, int32_t n, float u);

/* Voxelizer (cpuVoxelizer.cpp / voxelize.gs), mode 0 THIN, 1 FAT, OR'd with
 * 0x100 to clamp each triangle's swizzled voxel range against the unswizzled
 * resolution as the reference does (voxelize.gs:247-248); placement 1
 * applies computeMeshTransform; grid receives 1 for covered voxels. */
int orc_voxelize(const float* vertices, int64_t nv, const uint32_t* indices, int64_t nt,
                 int32_t rx, int32_t ry, int32_t rz, int32_t mode, int32_t placement,
                 int32_t threads, uint8_t* grid);
/* Independent check: triangle/box overlap by the separating axis theorem
 * (Akenine-Moller 2001) in double precision, for the box of half-size `half`
 * around each voxel centre (0.5 = the voxel; contact counts as overlap). */
int orc_voxelize_sat(const float* vertices_voxel_space, int64_t nv, const uint32_t* indices,
                     int64_t nt, int32_t rx, int32_t ry, int32_t rz, double half, uint8_t* grid);

/* pruneInteriorEmissiveVoxels (import.cpp:180-203) in place; returns new n. */
int64_t orc_prune_emissive(const uint8_t* grid, const int32_t* res, int32_t* list, int64_t n);

/* Default noise table: (splitmix64(i) >> 40) * 2^-24, 1024*1024*4 floats. */
int orc_noise_table(float* out);
/* Philox-4x32-10 block for known-answer tests. */
void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* BSDF of one material record (materials.h:7-43; type 0 Lambert, 1 metal,
 * 2 plastic), with the palette's FP16 rounding: sample n directions from
 * local wo (n*3, +Y = normal) and uniforms u (n*2) -> out n*8 {wi[3], f[3],
 * pdf, 0}; evaluate at (wo, wi) -> out n*4 {f[3], pdf}. */
int orc_bsdf_sample(int32_t type, const float* albedo, float roughness, uint32_t quirks,
                    const float* wo, const float* u, int64_t n, float* out);
int orc_bsdf_eval(int32_t type, const float* albedo, float roughness, uint32_t quirks,
                  const float* wo, const float* wi, int64_t n, float* out);
/* Environment light (lights.h:20-55, envMapSample.h:23-123): sample from
 * uniforms u (n*2) -> out n*8 {dir[3], L[3], pdf, 0}; evaluate along dirs
 * (n*3) -> out n*4 {L[3], pdf}.  The environment must hold an image. */
int orc_env_sample(const orc_env* env, float rotation, const float* u, int64_t n, float* out);
int orc_env_eval(const orc_env* env, float rotation, const float* dirs, int64_t n, float* out);
/* The first n draws (n*4 floats) of the noise-table stream of pixel (px, py)
 * and sample (randomNumberGeneratorOffset + rand, random.h:13-27). */
int orc_noise_walk(const float* noise, int32_t px, int32_t py, int32_t sample, int32_t n, float* out);
/* generateRay (generateRay.h:1-123) for fragments at window positions frag
 * (n*2) with the random block u (n*4) -> out n*6 {origin[3], direction[3]}. */
int orc_generate_rays(const orc_camera* cam, const orc_settings* s, int32_t width, int32_t height,
                      const float* frag, const float* u, int64_t n, float* out);
/* Builtins of the float build for accuracy tests (fn as vt_diag_builtins). */
int orc_builtins(int32_t fn, const float* a, const float* b, float* out, int64_t n);

#ifdef __cplusplus
}
#endif
#endif
