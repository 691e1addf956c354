/*
 * vt.h — C ABI of the GB300 voxel path tracer and mesh voxelizer.
 *
 * This is the drop-in boundary for the progressive path-tracing pass and the
 * mesh voxelizer of voxelToy.  The reference exposes that path as the C++
 * class `Renderer` (src/renderer/renderer.h:23-221) driving OpenGL shaders;
 * here the same verbs are plain C functions over opaque handles, with host
 * pointers and sizes only.  Every entry point cites the reference interface
 * it replaces.
 *
 * Conventions
 *   - Every function returns a vt_status (VT_OK == 0, errors < 0).  The text
 *     of the last error on the calling thread is available from
 *     vt_last_error().  No C++ exception crosses this boundary.
 *   - Host pointers are borrowed for the duration of the call and copied; the
 *     library keeps no reference to caller memory.  The library owns all
 *     device memory; handles are released with the matching *_destroy.
 *   - A context and the handles created from it are used by one host thread
 *     at a time.  vt_server_* calls are thread safe.
 *   - World space, voxel space and the material layout follow the reference:
 *     the volume is centred at the origin and scaled so that its largest axis
 *     spans 1000 world units (src/renderer/renderer.cpp:845-850); voxel
 *     (x, y, z) has linear index x + y*rx + z*rx*ry
 *     (src/shaders/shared/coordinates.h:118-127).
 */
#ifndef VT_H
#define VT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define VT_API __attribute__((visibility("default")))
#else
#define VT_API
#endif

/* ---------------------------------------------------------------- status -- */
typedef enum vt_status {
  VT_OK = 0,
  VT_EINVAL = -1,       /* bad argument (null handle, size, unknown material) */
  VT_ENOMEM = -2,       /* host or device allocation failed                    */
  VT_EBUDGET = -3,      /* request exceeds the context's device-memory budget  */
  VT_EDEVICE = -4,      /* CUDA error or device-side error word set             */
  VT_ETIMEOUT = -5,     /* a bounded wait ran out                               */
  VT_ECANCELLED = -6,   /* job cancelled                                        */
  VT_ENOTREADY = -7,    /* result not available yet                             */
  VT_EUNSUPPORTED = -8  /* feature not available in this build                  */
} vt_status;

/* Renderer::RenderResult (src/renderer/renderer.h:45-49). */
enum { VT_SAMPLES_PENDING = 0, VT_FINISHED_RENDERING = 1 };

/* --------------------------------------------------------------- handles -- */
typedef struct vt_context vt_context; /* Renderer + its GL context            */
typedef struct vt_scene vt_scene;     /* voxel volume, palette, emissive list  */
typedef struct vt_env vt_env;         /* HDR environment image + its CDFs      */
typedef struct vt_job vt_job;         /* camera, settings, accumulation buffer */
typedef struct vt_server vt_server;   /* continuous-batching render server     */

/* -------------------------------------------------------------- context -- */
typedef struct vt_device_opts {
  int32_t device;            /* CUDA ordinal                                  */
  uint64_t hbm_budget_bytes; /* 0 = no budget; allocations beyond it fail     */
  uint32_t flags;            /* VT_DEVICE_* flags, 0 by default               */
} vt_device_opts;
/* Device memory a context releases (scenes, environments, jobs destroyed)
 * is kept for its next allocations, up to 2 GiB, instead of returned at
 * once; live plus kept bytes stay within the budget.  This flag returns
 * every release at once; vt_context_trim returns the kept blocks. */
#define VT_DEVICE_NO_ALLOC_CACHE 1u

/* Renderer::initialize (src/renderer/renderer.h:31, renderer.cpp:76-140).
 * opts may be NULL (device 0, no budget). */
VT_API int vt_create(const vt_device_opts* opts, vt_context** out);
/* Renderer::~Renderer (src/renderer/renderer.h:28). */
VT_API int vt_destroy(vt_context* ctx);
/* Text of the last error raised on the calling thread ("" if none). */
VT_API const char* vt_last_error(void);
/* Renderer::setLogger (src/renderer/renderer.h:99; src/log/logger.h:7-11). */
typedef void (*vt_log_fn)(const char* message, void* user);
VT_API int vt_set_log_callback(vt_context* ctx, vt_log_fn fn, void* user);
/* Bytes of device memory the context currently holds for live objects
 * (blocks kept for reuse are not counted). */
VT_API int vt_context_memory(const vt_context* ctx, uint64_t* bytes_in_use);
/* Returns the device memory kept for reuse; released: bytes freed
 * (nullable). */
VT_API int vt_context_trim(vt_context* ctx, uint64_t* released);

/* ------------------------------------------------------------- materials -- */
/* Material::MaterialType (src/renderer/material/material.h:8-13). */
enum { VT_MATERIAL_LAMBERT = 0, VT_MATERIAL_METAL = 1, VT_MATERIAL_PLASTIC = 2 };

/* One palette record: LambertMaterialData / MetalMaterialData /
 * PlasticMaterialData (src/renderer/material/material.h:15-33) behind their
 * type tag (src/renderer/loaders/voxLoader.cpp:54-66).  albedo is the Lambert
 * albedo, the metal reflectance (Fresnel F0 when VT_QUIRK_FIXED_IOR is off)
 * or the plastic diffuse albedo (unused by the reference's plastic BSDF,
 * src/shaders/materials/plastic.h:15).  The device stores each record as
 * eight IEEE half floats. */
typedef struct vt_material {
  int32_t type;
  float emission[3];
  float albedo[3];
  float roughness;
} vt_material;

/* ---------------------------------------------------------------- images -- */
/* Float images for environment maps and saved frames (the reference reads
 * and writes them with OpenImageIO: image.cpp:28-59, renderer.cpp:1108-1140).
 * vt_image_decode reads PFM ("PF" colour, "Pf" grey) and Radiance RGBE
 * (.hdr, flat or run-length scanlines) into RGB floats, rows top first as
 * vt_env_create_image takes them; with rgb NULL it returns only the size.
 * vt_image_encode_pfm writes a colour PFM from RGB or RGBA floats whose rows
 * are bottom first (vt_job_readback's order, which PFM also uses);
 * vt_image_encode_hdr writes the same pixels as a flat Radiance RGBE file
 * (rows top first, as "-Y h +X w" orders them; negative and NaN channels
 * become 0).  With out NULL they return only the size.  None needs a GPU. */
VT_API int vt_image_decode(const uint8_t* data, size_t size, float* rgb,
                           size_t rgb_bytes, int32_t* width, int32_t* height);
VT_API int vt_image_encode_pfm(const float* pixels, int32_t width, int32_t height,
                               int32_t channels, uint8_t* out, size_t out_bytes,
                               size_t* written);
VT_API int vt_image_encode_hdr(const float* pixels, int32_t width, int32_t height,
                               int32_t channels, uint8_t* out, size_t out_bytes,
                               size_t* written);

/* ---------------------------------------------------------------- scenes -- */
enum {
  VT_SCENE_PRUNE_EMISSIVE = 1u << 0, /* drop emissive voxels with no empty 6-neighbour
                                        (Renderer::pruneInteriorEmissiveVoxels,
                                        src/renderer/import.cpp:180-203)          */
  VT_SCENE_AUTO_EMISSIVE = 1u << 1   /* build the emissive list from the palette:
                                        every voxel whose material emits          */
};

/* Upload a dense volume.  voxels[i] == 0 is empty, voxels[i] == k (1..255)
 * uses palette[k-1].  emissive_indices are linear voxel indices sampled by
 * next-event estimation (may be NULL when n_emissive == 0).
 * Replaces Renderer::createVoxelDataTexture (src/renderer/renderer.h:129-134,
 * renderer.cpp:833-940) for the byte-per-voxel palette layout. */
VT_API int vt_scene_create(vt_context* ctx, int32_t rx, int32_t ry, int32_t rz,
                           const uint8_t* voxels, const vt_material* palette,
                           int32_t n_palette, const int32_t* emissive_indices,
                           int64_t n_emissive, uint32_t flags, vt_scene** out);

/* Shape of the scene's occupancy bricks, the 64-bit words the DDA tests
 * (one word per block of 2^sx x 2^sy x 2^sz voxels, each of sx, sy, sz in
 * [1, 4] and sx + sy + sz = 6; scenes are created with 4x4x4, i.e. 2, 2, 2).  Changing it rebuilds the
 * bricks from the volume on the device; jobs on the scene pick the new
 * shape up before their next pass.  Images are identical for every shape:
 * the shape only changes how often the DDA loads a new word and how the
 * words share cache lines, which the autotuner measures.  No counterpart in
 * the reference, which tests a 3D integer texture per step (dda.h:41-45). */
VT_API int vt_scene_set_brick_shape(vt_scene* scene, int32_t sx, int32_t sy, int32_t sz);
VT_API int vt_scene_get_brick_shape(const vt_scene* scene, int32_t* shape);

/* Upload a volume in the reference's own layout: one int32 material-table
 * offset per voxel (-1 = empty) and a flat float material table of
 * [type, emission[3], albedo[3] (, roughness)] records
 * (Renderer::createVoxelDataTexture, src/renderer/renderer.cpp:833-940;
 * record layout src/renderer/loaders/voxLoader.cpp:54-66).  At most 255
 * distinct records may be referenced. */
VT_API int vt_scene_create_from_offsets(vt_context* ctx, int32_t rx, int32_t ry,
                                        int32_t rz, const int32_t* material_offsets,
                                        const float* material_data,
                                        int64_t material_data_size,
                                        const int32_t* emissive_indices,
                                        int64_t n_emissive, uint32_t flags,
                                        vt_scene** out);

/* Voxelizer coverage rule (src/shaders/shared/voxelize.gs:14-19), optionally
 * OR'd with VT_VOXELIZE_REFERENCE_BOUNDS.  Each triangle is scanned in its
 * swizzled frame (dominant normal axis as Z); its voxel range there is
 * clamped to the grid's extent along the same swizzled axes, so FAT marks
 * exactly the voxels a separating-axis overlap test marks on any grid.  The
 * reference clamps the swizzled range against the unswizzled resolution
 * (voxelize.gs:247-248, cpuVoxelizer.cpp:265-270), which is the same on
 * cubic grids and drops voxels on others; VT_VOXELIZE_REFERENCE_BOUNDS
 * reproduces that. */
enum { VT_VOXELIZE_THIN = 0, VT_VOXELIZE_FAT = 1, VT_VOXELIZE_REFERENCE_BOUNDS = 0x100 };
enum { VT_MESH_VOXEL_SPACE = 0, VT_MESH_FIT_UNIT_CUBE = 1 };

/* Voxelize a triangle mesh on the GPU into a new scene whose occupied voxels
 * use palette[0].  vertices: n_vertices * 3 floats; indices: n_triangles * 3.
 * With VT_MESH_FIT_UNIT_CUBE the mesh is first fitted into the unit cube with
 * a one-voxel margin (computeMeshTransform, src/renderer/import.cpp:46-64)
 * and scaled to voxel space (src/shaders/shared/voxelize.vs:20-27); with
 * VT_MESH_VOXEL_SPACE the vertices are already in voxel units.
 * Replaces Renderer::loadMesh + GPUVoxelizer::voxelizeMesh
 * (src/renderer/import.cpp:66-131, src/voxelize/gpuVoxelizer.cpp:46-72). */
VT_API int vt_scene_voxelize_mesh(vt_context* ctx, const float* vertices,
                                  int64_t n_vertices, const uint32_t* indices,
                                  int64_t n_triangles, int32_t rx, int32_t ry,
                                  int32_t rz, int32_t mode, int32_t placement,
                                  const vt_material* palette, int32_t n_palette,
                                  vt_scene** out);

/* ---------------------------------------------------------- file ingest -- */
/* MagicaVoxel .vox bytes (Renderer::loadVoxFile, src/renderer/renderer.h:62;
 * MagicaVoxelLoader::load, src/renderer/loaders/magicaVoxel.cpp:122-321).
 * As the reference: file versions 150 (and 200, which only adds chunks that
 * are skipped), axes converted so that the file's z is up (res = {x, z, y}),
 * colour index 254 left empty, one Lambert material per colour used, albedo
 * = palette RGB / 255, in order of first use, from the file's RGBA chunk or
 * MagicaVoxel's default palette.  Voxels outside the model are an error (the
 * reference writes past its grid).
 * vt_vox_decode needs no GPU: with voxels and palette NULL it returns the
 * resolution and palette size; then voxels (res[0]*res[1]*res[2] bytes,
 * 0 empty, k = palette[k-1]) and palette (n_palette entries) are filled. */
VT_API int vt_vox_decode(const uint8_t* data, size_t size, int32_t res[3],
                         uint8_t* voxels, size_t voxels_bytes,
                         vt_material* palette, int32_t* n_palette);
VT_API int vt_scene_create_from_vox(vt_context* ctx, const uint8_t* data,
                                    size_t size, uint32_t flags, vt_scene** out);

/* Wavefront OBJ text (MeshLoader::loadFromOBJ, src/mesh/meshLoader.cpp:11-74,
 * which merges every shape into one vertex and index list): `v` positions
 * and `f` faces (v, v/vt, v//vn, v/vt/vn references, negative = relative),
 * polygons fan-triangulated; other records are ignored.  vt_obj_decode needs
 * no GPU and follows the same two-call pattern as vt_vox_decode;
 * vt_scene_voxelize_obj decodes and calls vt_scene_voxelize_mesh
 * (Renderer::loadMesh, src/renderer/import.cpp:66-131). */
VT_API int vt_obj_decode(const char* text, size_t size, float* vertices,
                         int64_t vertex_capacity, uint32_t* indices,
                         int64_t triangle_capacity, int64_t* n_vertices,
                         int64_t* n_triangles);
VT_API int vt_scene_voxelize_obj(vt_context* ctx, const char* text, size_t size,
                                 int32_t rx, int32_t ry, int32_t rz, int32_t mode,
                                 int32_t placement, const vt_material* palette,
                                 int32_t n_palette, vt_scene** out);

typedef struct vt_scene_info {
  int32_t resolution[3];
  float bounds_min[3];
  float bounds_max[3];
  float voxel_size[3];
  int64_t n_emissive;     /* after pruning */
  int32_t n_palette;
  uint64_t device_bytes;
} vt_scene_info;
VT_API int vt_scene_get_info(const vt_scene* scene, vt_scene_info* info);
/* Copy the byte-per-voxel grid back to the host (rx*ry*rz bytes). */
VT_API int vt_scene_read_voxels(const vt_scene* scene, uint8_t* out, size_t bytes);
/* Copy the (pruned) emissive list back; *n receives its length. */
VT_API int vt_scene_read_emissive(const vt_scene* scene, int32_t* out,
                                  int64_t capacity, int64_t* n);
/* Renderer::getMaterials (src/renderer/renderer.h:120, renderer.cpp:1142-1203):
 * the scene's materials as the reference's flat float table, each record its
 * type followed by LambertMaterialData (6 floats) or MetalMaterialData /
 * PlasticMaterialData (7 floats) (src/renderer/material/material.h:15-33).
 * A scene made by vt_scene_create_from_offsets returns the caller's table as
 * given, so its offsets stay valid; any other scene lays its palette out
 * entry after entry.  *size receives the table's length in floats; with out
 * NULL nothing else is written. */
VT_API int vt_scene_read_material_table(const vt_scene* scene, float* out,
                                        int64_t capacity, int64_t* size);
/* Renderer::updateMaterialColor / updateMaterialValue (renderer.h:121-122,
 * renderer.cpp:1205-1235): overwrite n floats of that table from data_offset
 * on (3 for a colour, 1 for a value).  The range must lie inside the data of
 * one record, after its type.  Materials of the volume change in place for
 * later passes; with VT_SCENE_AUTO_EMISSIVE the emissive list follows the
 * new emissions.  Accumulated samples are kept: vt_job_reset restarts them,
 * as the reference's material editor does after each change. */
VT_API int vt_scene_write_material_table(vt_scene* scene, int64_t data_offset,
                                         const float* values, int32_t n);
VT_API int vt_scene_destroy(vt_scene* scene);

/* ------------------------------------------------------------ environment -- */
/* Upload a linear RGB float image (width*height*3, row 0 = zenith) as the
 * background, stored as FP16 RGBA, and build its importance-sampling CDFs on
 * the GPU with FP64 prefix sums at full resolution.
 * Replaces Renderer::loadBackgroundImage + calculateCDF
 * (src/renderer/renderer.cpp:947-1055, src/renderer/image.cpp:68-389). */
VT_API int vt_env_create_image(vt_context* ctx, const float* rgb, int32_t width,
                               int32_t height, vt_env** out);
/* vt_env_create_image with options.  VT_ENV_CDF_REFERENCE_SIZE builds the
 * CDFs and the integral from the image shrunk to at most 512 texels on its
 * long axis, as calculateCDF does (image.cpp:14, 308-320: the size from its
 * float arithmetic), while radiance is still looked up in the full-size
 * texels; samples then follow the shrunk image's distribution and their pdf
 * is the full-size luminance over the shrunk image's integral, as in the
 * reference.  The shrink is an area-weighted box average: the reference's
 * OpenImageIO resize filter is not restated (its weights are unpinned). */
enum { VT_ENV_CDF_REFERENCE_SIZE = 1u << 0 };
VT_API int vt_env_create_image_ex(vt_context* ctx, const float* rgb, int32_t width,
                                  int32_t height, uint32_t flags, vt_env** out);
/* size[0..3] = image width, height, and the width and height of the image
 * the CDFs describe (the same, or the shrunk size). */
VT_API int vt_env_get_info(const vt_env* env, int32_t* size);
/* Copy back the CDFs: cdf_u (cdf_width+1)*cdf_height floats, cdf_v
 * cdf_height+1 floats and the radiance integral (image.cpp:349-389).  Any
 * output may be NULL. */
VT_API int vt_env_read_cdf(const vt_env* env, float* cdf_u, size_t cdf_u_bytes,
                           float* cdf_v, size_t cdf_v_bytes, float* integral);
VT_API int vt_env_destroy(vt_env* env);

/* ---------------------------------------------------------------- camera -- */
/* CameraParameters::CameraLensModel (src/camera/cameraParameters.h:23-28). */
enum { VT_LENS_PINHOLE = 0, VT_LENS_THIN_LENS = 1, VT_LENS_ORTHOGRAPHIC = 2 };

/* CameraParameters (src/camera/cameraParameters.h:117-129) with the focus
 * distance and lens radius in world units. */
typedef struct vt_camera {
  float eye[3];
  float target[3];
  float fov_y;          /* vertical field of view, radians                     */
  float near_distance;  /* reference default 0.1                               */
  float far_distance;   /* reference default 10000                             */
  float focal_distance; /* thin-lens focus distance, world units               */
  float lens_radius;    /* thin-lens aperture radius, world units              */
  int32_t lens_model;
} vt_camera;

/* CameraParameters::CameraParameters + Renderer::Renderer defaults
 * (src/camera/cameraParameters.cpp:7-17, src/renderer/renderer.cpp:43-45). */
VT_API int vt_camera_default(vt_camera* cam);
/* CameraParameters::orbitAroundTarget: eye = target - r * sph(theta, phi)
 * (src/camera/cameraParameters.cpp:90-94). */
VT_API int vt_camera_orbit(vt_camera* cam, float theta, float phi);
/* CameraParameters::orbitAroundEye (cameraParameters.cpp:96-100). */
VT_API int vt_camera_orbit_eye(vt_camera* cam, float theta, float phi);
/* CameraParameters::setDistanceFromTarget (cameraParameters.cpp:38-41). */
VT_API int vt_camera_set_distance(vt_camera* cam, float distance);
/* CameraParameters::setFocalLength with the 35 mm film rule of
 * Renderer::render (cameraParameters.cpp:139-142, renderer.cpp:573-580). */
VT_API int vt_camera_set_focal_length(vt_camera* cam, float focal_length_mm,
                                      int32_t width, int32_t height);
/* CameraParameters::setFStop: lens radius = focal length / f-stop / 2
 * (cameraParameters.cpp:172-175), focal length from fov and film. */
VT_API int vt_camera_set_fstop(vt_camera* cam, float fstop, int32_t width,
                               int32_t height);
/* CameraController::focusOnBounds (src/camera/cameraController.cpp:16-23). */
VT_API int vt_camera_focus_on_bounds(vt_camera* cam, const float bounds_min[3],
                                     const float bounds_max[3]);
/* Orbit / fly controllers: mouse deltas normalised by the image size
 * (src/camera/orbitCameraController.cpp:15-41,
 * src/camera/flyCameraController.cpp:15-73).  buttons: 1 = rotate (right
 * button), 2 = dolly/pan (middle button). */
enum { VT_BUTTON_ROTATE = 1, VT_BUTTON_PAN = 2 };
enum { VT_KEY_FORWARD = 0, VT_KEY_BACK = 1, VT_KEY_RIGHT = 2, VT_KEY_LEFT = 3 };
VT_API int vt_camera_orbit_mouse(vt_camera* cam, float ndx, float ndy, int32_t buttons);
VT_API int vt_camera_fly_mouse(vt_camera* cam, float ndx, float ndy, int32_t buttons);
VT_API int vt_camera_fly_key(vt_camera* cam, int32_t key);

/* Shader uniforms derived from a camera (Renderer::updateCamera,
 * src/renderer/renderer.cpp:343-446): row-major 4x4 matrices as uploaded
 * with transpose = GL_TRUE. */
typedef struct vt_camera_uniforms {
  float proj[16];
  float inv_proj[16];
  float inv_model_view[16];
  float viewport[4];
} vt_camera_uniforms;
VT_API int vt_camera_compute_uniforms(const vt_camera* cam, int32_t width,
                                      int32_t height, vt_camera_uniforms* out);

/* -------------------------------------------------------------- settings -- */
/* Behaviours of the reference kept behind flags.  VT_QUIRKS_REFERENCE
 * reproduces the reference pass; the physically based configurations clear
 * them. */
#define VT_QUIRK_GAMMA_BEFORE_AVERAGE  (1u << 0) /* pathTracer.fs:294-295 + accumulation.fs:17 */
#define VT_QUIRK_GROUND                (1u << 1) /* exit through y<0 hits ground, dda.h:74-78   */
#define VT_QUIRK_GRADIENT_PDF_MISMATCH (1u << 2) /* lights.h:30 (1/4pi) vs sampling.h:34 (1/2pi) */
#define VT_QUIRK_DOUBLE_REFLECTANCE    (1u << 3) /* microfacet.h:57 + :116                      */
#define VT_QUIRK_FIXED_IOR             (1u << 4) /* Schlick with IOR 7.3, microfacet.h:2,64-69   */
#define VT_QUIRK_EXPONENT_IS_ROUGHNESS (1u << 5) /* Blinn exponent = roughness, metal.h:13-14    */
#define VT_QUIRK_THINLENS_NO_JITTER    (1u << 6) /* no pixel jitter, generateRay.h:83            */
#define VT_QUIRK_UNGUARDED_SAMPLES     (1u << 7) /* zero-pdf / below-surface samples propagate,  */
                                                 /* pathTracer.fs:164,276 divide by the pdf;    */
                                                 /* a hit on a voxel corner keeps the three-axis */
                                                 /* normal whose frame is NaN, coordinates.h:79 */
#define VT_QUIRKS_REFERENCE 0xffu

/* Random-number source.  VT_RNG_NOISE_TABLE walks a 1024x1024 RGBA table
 * from a per-pixel hashed offset (src/shaders/shared/random.h:3-27,
 * renderer.cpp:739-760); VT_RNG_PHILOX draws Philox-4x32-10 blocks keyed by
 * (seed, pixel) with counter (sample, call). */
enum { VT_RNG_PHILOX = 0, VT_RNG_NOISE_TABLE = 1 };

/* RenderSettings (src/renderer/renderSettings.h:6-29) plus the uniforms of
 * src/shaders/integrator/pathTracer.fs:25-44. */
typedef struct vt_render_settings {
  int32_t max_bounces;          /* m_pathtracerMaxNumBounces                    */
  int32_t max_samples;          /* m_pathtracerMaxSamples                       */
  int32_t rr_start_bounce;      /* Russian roulette from this bounce; -1 = off  */
  float gamma;                  /* tonemappingGamma (2.2)                       */
  float exposure;               /* tonemappingExposure (1)                      */
  float nee_emission_scale;     /* emissive light-sample scale (reference 10)   */
  float wireframe_opacity;      /* m_wireframeOpacity                           */
  float wireframe_thickness;    /* m_wireframeThickness                         */
  float background_top[3];      /* m_backgroundColor[0]                         */
  float background_bottom[3];   /* m_backgroundColor[1]                         */
  float background_rotation;    /* radians (m_backgroundRotationDegrees)         */
  int32_t selected_voxel[3];    /* SelectVoxelData.index (drawn red)            */
  int32_t select_enabled;
  int32_t ground_material;      /* palette entry used by VT_QUIRK_GROUND hits   */
  uint32_t quirks;              /* VT_QUIRK_* bits                              */
  int32_t rng_mode;             /* VT_RNG_*                                     */
  uint32_t seed;
} vt_render_settings;

/* RenderSettings defaults of Renderer::Renderer (renderer.cpp:49-53) and the
 * uniform initialisers of pathTracer.fs:25-44, all quirks on. */
VT_API int vt_settings_default(vt_render_settings* s);

/* ------------------------------------------------------------------- jobs -- */
/* A job is one progressive render: camera, settings, a scene, an optional
 * environment image (NULL = gradient background from the settings) and its
 * accumulation buffer.  Replaces Renderer::resizeFrame + updateCamera +
 * updateRenderSettings (src/renderer/renderer.cpp:343-554, 1057-1106). */
VT_API int vt_job_create(vt_context* ctx, const vt_scene* scene, const vt_env* env,
                         const vt_camera* cam, const vt_render_settings* settings,
                         int32_t width, int32_t height, vt_job** out);
/* Renderer::updateCamera + resetRender (renderer.cpp:343-446, 941-945). */
VT_API int vt_job_set_camera(vt_job* job, const vt_camera* cam);
/* Renderer::updateRenderSettings (renderer.cpp:1057-1106). */
VT_API int vt_job_set_settings(vt_job* job, const vt_render_settings* settings);
VT_API int vt_job_set_scene(vt_job* job, const vt_scene* scene, const vt_env* env);
/* Renderer::resizeFrame (renderer.cpp:448-554): resets accumulation. */
VT_API int vt_job_resize(vt_job* job, int32_t width, int32_t height);
/* Renderer::resetRender (renderer.cpp:941-945). */
VT_API int vt_job_reset(vt_job* job);
/* Renderer::Integrator (src/renderer/renderer.h:112-117), switched with the
 * space key in the reference (renderer.cpp:678-683): VT_INTEGRATOR_PATH_TRACER
 * (pathTracer.fs, the default) or VT_INTEGRATOR_EDIT_MODE (editMode.fs: white
 * voxels, a fixed light with one shadow ray, the selected voxel red, the
 * wireframe overlay; one launch per pass).  A switch restarts the
 * accumulation. */
enum { VT_INTEGRATOR_PATH_TRACER = 0, VT_INTEGRATOR_EDIT_MODE = 1 };
VT_API int vt_job_set_integrator(vt_job* job, int32_t integrator);
/* Renderer::render (renderer.cpp:556-645) called `passes` times: each pass
 * adds one sample per pixel until max_samples are accumulated.  *result
 * receives VT_SAMPLES_PENDING or VT_FINISHED_RENDERING.  The call queues GPU
 * work and returns; vt_job_synchronize or a readback waits for it. */
VT_API int vt_job_render(vt_job* job, int32_t passes, int32_t* result);
VT_API int vt_job_synchronize(vt_job* job);
VT_API int vt_job_sample_count(const vt_job* job, int32_t* samples);

enum {
  VT_READBACK_FLIP_Y = 1u << 0,  /* bottom row first, as saveImage writes (renderer.cpp:1133-1136) */
  VT_READBACK_TONEMAP = 1u << 1  /* apply pow(x*exposure, 1/gamma) to a linear accumulation  */
};
/* Copy the accumulated average image (width*height*4 floats, RGBA) to host
 * memory.  Replaces the glGetTexImage of Renderer::saveImage
 * (renderer.cpp:1108-1140). */
VT_API int vt_job_readback(vt_job* job, float* rgba, size_t bytes, uint32_t flags);

/* Accumulation state of a job: the Kahan-compensated running sums of its
 * samples (sum) and their compensation terms (comp), width*height*4 floats
 * each, and the number of samples they hold.  No counterpart in the
 * reference, whose resetRender (renderer.cpp:941-945) discards the
 * accumulation: a job restored from a snapshot into a job of the same
 * scene, camera, settings and size continues with the samples that come
 * next (the random streams are keyed by pixel and sample index), so its
 * image equals that of a job that was never interrupted, bit for bit.
 * Used to evict a long-running frame from device memory and resume it. */
VT_API int vt_job_snapshot(const vt_job* job, float* sum, float* comp, size_t bytes_each,
                           int32_t* samples);
VT_API int vt_job_restore(vt_job* job, const float* sum, const float* comp, size_t bytes_each,
                          int32_t samples);
/* Device pointer of the float4 accumulation sums and the sample count, for
 * zero-copy consumers (valid until the next render/reset/destroy). */
VT_API int vt_job_device_buffer(vt_job* job, void** sums, int32_t* samples);
/* Focal-distance pick: trace the ray through window pixel (x, y) and return
 * the hit distance (99999999 when nothing is hit) and voxel (-1 if none).
 * Replaces focalDistance.vs (src/shaders/focalDistance/focalDistance.vs:45-81)
 * and RendererServiceSetFocalDistance. */
VT_API int vt_job_pick(vt_job* job, float x, float y, float* distance,
                       int32_t voxel[3]);
VT_API int vt_job_destroy(vt_job* job);

/* ---------------------------------------------------------- voxel edits -- */
/* Set one voxel of a scene: entry 0 empties it, k (1..n_palette) gives it
 * palette[k-1].  The grid, its occupancy bricks and the emissive list follow:
 * scenes made with VT_SCENE_AUTO_EMISSIVE rediscover (and, with
 * VT_SCENE_PRUNE_EMISSIVE, prune) their list; otherwise an emptied voxel
 * leaves the caller's list.  Jobs on the scene see the edit at their next
 * render or pick; reset them to drop samples of the old volume.  Do not edit
 * a scene that a vt_server is rendering.  No counterpart as a function in
 * the reference, whose edits run as the shaders below. */
VT_API int vt_scene_set_voxel(vt_scene* scene, int32_t x, int32_t y, int32_t z,
                              int32_t entry);
/* RendererServiceSelectActiveVoxel (src/shaders/editVoxels/selectVoxel.vs:
 * 35-69): the voxel under window point (x, y) (pixels, origin bottom-left)
 * and the normal of its voxelSpaceToWorldSpace basis; voxel (-1,-1,-1) and
 * normal 0 when the ray hits nothing (the reference leaves index 0 there). */
VT_API int vt_job_select_voxel(vt_job* job, float x, float y, int32_t voxel[3],
                               float normal[3]);
/* RendererServiceAddVoxel (addVoxel.vs:16-41): select at (x, y); the new
 * voxel is the selected one plus the hit normal or, when the screen-space
 * motion (dx, dy) (pixels, y up) is not zero, plus the camera right / up
 * axis of its dominant component; it copies the selected voxel's material
 * (the ground's when the ground was hit).  voxel receives the new voxel, or
 * -1s when nothing was hit or the new voxel lies outside the volume (no
 * edit).  restart != 0 resets the job's accumulation (requestAction's
 * restartAccumulation, src/renderer/actions.cpp:5-52). */
VT_API int vt_job_add_voxel(vt_job* job, float x, float y, float dx, float dy,
                            int32_t restart, int32_t voxel[3]);
/* RendererServiceRemoveVoxel (removeVoxel.vs:8-11): select at (x, y) and
 * empty that voxel; voxel receives it, or -1s when nothing (or only the
 * implicit ground) was hit. */
VT_API int vt_job_remove_voxel(vt_job* job, float x, float y, int32_t restart,
                               int32_t voxel[3]);

/* ------------------------------------------------------------- batching -- */
/* Trace `passes` samples per pixel for every job in one wavefront launch:
 * path slots pull (job, pass, pixel) work items from a device counter and
 * rounds of shading and DDA kernels run over all jobs' paths at once,
 * instead of one launch per job and pass.  Results are identical to rendering
 * each job alone (counter-based random streams, per-pixel sample order).
 * opts may be NULL (context defaults). */
typedef struct vt_batch_opts {
  int32_t path_slots;      /* paths in flight per launch, 0 = context default (8M) */
  int32_t blocks_per_sm;   /* resident blocks per SM, 0 = auto                  */
  int32_t threads_per_block; /* 0 = auto                                        */
  int32_t kernel;          /* 0 = auto, 1 = plain per-pixel, 2 = wavefront      */
} vt_batch_opts;
VT_API int vt_render_batch(vt_context* ctx, vt_job* const* jobs, int32_t n_jobs,
                           int32_t passes, const vt_batch_opts* opts,
                           int32_t* results);

/* ------------------------------------------------ fixed-memory batching -- */
/* No counterpart in the reference: its renderer draws one GL pass per frame
 * and has no working memory of its own to speak of.
 *
 * vt_render_batch_fixed renders like vt_render_batch with the wavefront
 * kernels, with bit-identical results, but allocates nothing.  The normal
 * path grows per-context working buffers (path state, segment queues, the
 * sample buffer, job tables) with cudaMalloc the first time a batch needs
 * more.  That fails for a caller whose HBM budget (vt_create) is already
 * spent on scenes and images, and it stalls a caller that must keep steady
 * frame times, such as an interactive viewer, because cudaMalloc and
 * cudaFree can synchronise the whole device.  Instead, this call takes all
 * of its working memory from one array compiled into the library
 * (VT_FIXED_SCRATCH_BYTES, about 42 MB, not counted against any budget).
 * The CUDA runtime reserves it on a device when it loads the code that
 * holds it, which vt_create triggers for its device, so the reservation
 * (and a failure to make it) happens when the context is created, not in
 * the caller's frame loop; the array stays reserved until the process
 * exits.
 *
 * Limits, each rejected with VT_EINVAL and a message naming the limit:
 *   n_jobs        <= VT_FIXED_MAX_JOBS
 *   path_slots    <= VT_FIXED_MAX_PATH_SLOTS (0 = that maximum)
 *   width*height  <= VT_FIXED_MAX_SAMPLES for every job; a call traces at
 *                    most that many samples per launch and splits the rest
 *                    into further launches.
 *
 * vt_create looks up the array's device address (cudaGetSymbolAddress)
 * with its device current; if that failed, the first call on the device
 * tries again, so make that first call before any stream capture begins on
 * the device.  A call that fails after queuing work waits for that work
 * before it returns; the jobs of a failed call may hold part of their
 * passes, so reset them (vt_job_reset) before rendering them again.  Each
 * launch clears
 * the words that must start at zero (queue and hit-list counters, the path
 * stream's length, the item counter); everything else in the array is
 * written before it is read.  There is one array per device, shared by
 * every call on every context of that device: two calls whose device work
 * overlaps (two host threads, or two contexts driven at the same time) race
 * on it and both results are wrong.  A call returns only after its device
 * work has finished, so calls made one after another are safe. */
#define VT_FIXED_MAX_JOBS 16
#define VT_FIXED_MAX_PATH_SLOTS 65536
#define VT_FIXED_MAX_SAMPLES (1 << 20)
#define VT_FIXED_SCRATCH_BYTES 41956608
VT_API int vt_render_batch_fixed(vt_context* ctx, vt_job* const* jobs,
                                 int32_t n_jobs, int32_t passes,
                                 int32_t path_slots, int32_t* results);

/* -------------------------------------------------------------- serving -- */
typedef struct vt_server_opts {
  uint64_t hbm_budget_bytes;   /* admission budget for job buffers + scenes    */
  int32_t max_active_jobs;     /* slots traced concurrently                     */
  int32_t passes_per_round;    /* samples per pixel each active job gets per round */
  int32_t path_slots;          /* paths in flight per round, 0 = auto            */
  int32_t order;               /* which queued request is admitted next:
                                  VT_SERVE_ARRIVAL (0, first come first served) or
                                  VT_SERVE_LEAST_WORK (fewest paths w*h*spp first,
                                  arrival order among equals; under sustained
                                  overload large requests can wait indefinitely) */
  uint64_t quick_paths;        /* a running request whose remaining paths
                                  (w*h*(spp - samples)) are at most this many gets
                                  them all in the next round instead of
                                  passes_per_round; 0 = off                       */
  uint64_t round_paths_cap;    /* at most this many paths of one request per round
                                  (at least one pass), so that a large request
                                  does not lengthen every round; 0 = off          */
  uint64_t round_paths;        /* paths traced per round: every active request
                                  first gets passes_per_round passes (or what it
                                  has left), then the rest of this budget goes to
                                  the requests with the fewest paths left first,
                                  as many passes as fit; 0 = 2^26.  Rounds of
                                  many paths keep the GPU's path slots full;
                                  a request that arrives waits at most one round */
} vt_server_opts;

enum { VT_SERVE_ARRIVAL = 0, VT_SERVE_LEAST_WORK = 1 };

enum {
  VT_REQ_QUEUED = 0, VT_REQ_RUNNING = 1, VT_REQ_DONE = 2,
  VT_REQ_CANCELLED = 3, VT_REQ_FAILED = 4
};

typedef struct vt_server_stats {
  uint64_t submitted, completed, cancelled, failed;
  uint64_t paths_traced;
  uint64_t rounds;
  uint64_t bytes_in_use;       /* job buffers and resident scenes, against the budget */
  int32_t active, queued;
  uint64_t scene_uploads;      /* scenes uploaded by vt_server_submit_dense           */
  uint64_t scene_hits;         /* submissions that found their scene resident         */
  uint64_t scene_evictions;    /* resident scenes evicted to make room                */
  int32_t scenes_resident;
  int32_t pad;
  uint64_t round_us;           /* loop time in rounds: launch to completion            */
  uint64_t between_us;         /* loop time between consecutive rounds (retiring,
                                  admission, composing the next round)                 */
} vt_server_stats;

/* Start a request loop thread that admits jobs as slots and budget free up
 * and traces all admitted jobs together each round.  The rounds take ctx's
 * wavefront launch settings at this call (lanes, DDA kernel form, blocks,
 * refill interval, queue chunk). */
VT_API int vt_server_create(vt_context* ctx, const vt_server_opts* opts,
                            vt_server** out);
/* Submit a render request on a scene the caller created and owns; the
 * scene and env must outlive the request (destroying either while the
 * request is queued or running is undefined).  Its memory is the caller's
 * and is not counted against the server's budget. */
VT_API int vt_server_submit(vt_server* srv, const vt_scene* scene, const vt_env* env,
                            const vt_camera* cam, const vt_render_settings* settings,
                            int32_t width, int32_t height, int32_t spp_target,
                            uint64_t* ticket);
/* Submit a render request on a volume the server keeps resident, named by
 * the caller's scene_key (for example a content hash).  If the key is not
 * resident, the volume (voxels: rx*ry*rz palette entries + 1, 0 empty, x
 * fastest; palette; flags as vt_scene_create) is uploaded during this call,
 * after evicting unused resident scenes, least recently used first, until
 * it fits the budget (VT_EBUDGET if it cannot); if the key is resident the
 * volume arguments may be NULL / 0 and are not read.  Host pointers are
 * borrowed for the duration of the call.  A resident scene stays on the
 * device while requests use it and afterwards, until evicted (also to make
 * room for a request's job buffers) or the server is destroyed.  The env
 * stays the caller's and must outlive the request.  No counterpart in the
 * reference, which keeps exactly one volume (createVoxelDataTexture,
 * renderer.cpp:833-940). */
VT_API int vt_server_submit_dense(vt_server* srv, uint64_t scene_key, int32_t rx, int32_t ry,
                                  int32_t rz, const uint8_t* voxels, const vt_material* palette,
                                  int32_t n_palette, uint32_t scene_flags, const vt_env* env,
                                  const vt_camera* cam, const vt_render_settings* settings,
                                  int32_t width, int32_t height, int32_t spp_target,
                                  uint64_t* ticket);
VT_API int vt_server_poll(vt_server* srv, uint64_t ticket, int32_t* state,
                          int32_t* samples_done);
/* Wait until the request is done, failed or cancelled (timeout in seconds,
 * < 0 waits forever); VT_ETIMEOUT if it ran out. */
VT_API int vt_server_wait(vt_server* srv, uint64_t ticket, double timeout_s);
/* Copy the finished image (width*height*4 floats) and release the request. */
VT_API int vt_server_result(vt_server* srv, uint64_t ticket, float* rgba,
                            size_t bytes, double* seconds_to_target);
VT_API int vt_server_cancel(vt_server* srv, uint64_t ticket);
VT_API int vt_server_get_stats(vt_server* srv, vt_server_stats* stats);
VT_API int vt_server_destroy(vt_server* srv);

#ifdef __cplusplus
}
#endif
#endif /* VT_H */
