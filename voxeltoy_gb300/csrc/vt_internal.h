// vt_internal.h — data layout shared by the host runtime and the kernels.
//
// Device-memory layout of one scene (all resident in HBM):
//   grid     uint8[rx*ry*rz]        palette entry + 1 per voxel, 0 = empty,
//                                   linear index x + y*rx + z*rx*ry
//   bricks   uint64[(bx+2)*(by+2)*(bz+2)]  occupancy bit-bricks: one 64-bit word
//                                   per 4x4x4 voxel block, bit (x&3)|(y&3)<<2|(z&3)<<4,
//                                   bx = ceil(rx/4) ...; a border of one brick on
//                                   every side has all bits set, as do voxels of
//                                   the last bricks beyond the volume, so that a
//                                   ray leaving the volume stops on a set bit
//   palette  uint4[n_palette]       one 16-byte record per material: eight IEEE
//                                   halves {type, emission rgb, albedo rgb, roughness}
//   emissive int32[n_emissive]      linear voxel indices sampled by NEE
// One environment image:
//   texels   uint2[w*h]             four halves RGBA (A = 1)
//   cdf_u    float[(w+1)*h]         per-row conditional CDFs
//   cdf_v    float[h+1]             marginal CDF
// One job:
//   sum/comp float4[w*h] each       Kahan-compensated running sums of samples
#pragma once

#include <stdint.h>
#include <vector_types.h>

namespace vt {

constexpr int kNoiseW = 1024;   // reference noise texture size (renderer.cpp:749-758)
constexpr int kNoiseH = 1024;
constexpr float kInfinity = 99999999.0f;  // focalDistance.vs:43

// Per-job uniforms: the uniform block of pathTracer.fs:6-44 plus the volume
// description uploaded by createVoxelDataTexture (renderer.cpp:919-932).
struct Frame {
  int32_t res[3];
  int32_t max_steps;         // int(2*ceil(length(vec3(res)))), dda.h:98
  float bmin[3];
  float bmax[3];
  float vsize[3];            // (bmax-bmin)/res
  float vext[3];             // 1/(bmax-bmin), dda.h:16
  int32_t bdim[3];           // brick grid dimensions
  float viewport[4];
  float frag_z;              // gl_FragCoord.z of the full-screen quad drawn at z = near
  float proj[16];            // row-major, as uploaded with transpose = GL_TRUE
  float inv_proj[16];
  float inv_mv[16];
  float lens_radius;
  float focal_distance;
  int32_t lens_model;
  float bg_top[3];
  float bg_bottom[3];
  float bg_rot;
  int32_t use_image;
  float env_integral;
  int32_t env_w;
  int32_t env_h;
  int32_t n_emissive;
  int32_t max_bounces;
  int32_t rr_start;
  float inv_gamma;           // 1.0/tonemappingGamma
  float exposure;
  float nee_scale;
  float wire_opacity;
  float wire_thickness;
  int32_t sel[3];
  int32_t sel_enabled;
  int32_t ground_mat;
  uint32_t quirks;
  int32_t rng_mode;
  uint32_t seed;
  int32_t width;
  int32_t height;
  int32_t integrator;        // 0 path tracer (pathTracer.fs), 1 edit mode (editMode.fs)
};

// What the DDA needs of a volume: extents, bounds, brick layout, step cap.
struct Grid {
  int32_t rx, ry, rz;
  int32_t bx, bxy;           // padded brick-grid row and slice strides
  int32_t max_steps;         // int(2*ceil(length(vec3(res)))), dda.h:98
  float bminx, bminy, bminz;
  float vextx, vexty, vextz; // 1/(bmax-bmin), dda.h:16
  float bmaxx, bmaxy, bmaxz;
  int32_t pad;
  const unsigned long long* bricks;   // brick (0,0,0) of the padded array
};

// Device pointers of everything one job reads and writes.
struct JobDev {
  const uint8_t* grid;
  const unsigned long long* bricks;
  const uint4* palette;
  const int32_t* emissive;
  const uint2* env_texels;
  const float* cdf_u;
  const float* cdf_v;
  const float4* noise;       // VT_RNG_NOISE_TABLE only
  float4* sum;
  float4* comp;
};

// Quirk bits (mirror of the public VT_QUIRK_* values).
enum : uint32_t {
  Q_GAMMA_BEFORE_AVERAGE = 1u << 0,
  Q_GROUND = 1u << 1,
  Q_GRADIENT_PDF_MISMATCH = 1u << 2,
  Q_DOUBLE_REFLECTANCE = 1u << 3,
  Q_FIXED_IOR = 1u << 4,
  Q_EXPONENT_IS_ROUGHNESS = 1u << 5,
  Q_THINLENS_NO_JITTER = 1u << 6,
  Q_UNGUARDED = 1u << 7,
};

// Event counters of the algorithmic byte model (per path: 1 B per DDA cell
// tested, 16 B per palette record, 8 B per environment texel evaluation,
// 4 B per CDF entry probed, 4 B per emissive-list read, 64 B framebuffer).
enum Counter {
  C_PATHS = 0,
  C_DDA_CELLS = 1,
  C_PALETTE = 2,
  C_ENV_EVALS = 3,
  C_CDF_PROBES = 4,
  C_EMISSIVE_READS = 5,
  C_SEGMENTS = 6,
  C_EMPTY_CELLS = 7,   // DDA cells tested inside bricks with no occupied voxel
  C_NUM = 8
};

// Per-pixel first-hit record written by the diagnostic pass: voxel x, y, z
// and flags = normal code | hit << 8 | ground << 9, normal code =
// (nx+1) | (ny+1) << 2 | (nz+1) << 4.
struct HitRecord { int32_t x, y, z, flags; };

}  // namespace vt
