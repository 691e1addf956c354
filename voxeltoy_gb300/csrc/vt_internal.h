// vt_internal.h — data layout shared by the host runtime and the kernels.
//
// Device-memory layout of one scene (all resident in HBM):
//   grid     uint8[rx*ry*rz]        palette entry + 1 per voxel, 0 = empty,
//                                   linear index x + y*rx + z*rx*ry
//   bricks   uint64[(bx+2)*(by+2)*(bz+2)]  occupancy bit-bricks: one 64-bit word
//                                   per block of 2^sx x 2^sy x 2^sz voxels (the
//                                   scene's brick shape, sx+sy+sz = 6; 4x4x4 by
//                                   default), bit (x&mx)|(y&my)<<sx|(z&mz)<<(sx+sy),
//                                   bx = ceil(rx/2^sx) ...; a border of one brick on
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
  int32_t bsh[3];            // log2 of a brick's extent along x, y, z (sum 6)
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
  int32_t env_cdf_w;         // size of the image the CDFs describe (env_w x env_h, or
  int32_t env_cdf_h;         // the reference's shrunk size)
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
  int32_t n_palette;         // palette entries (bounds of the checked build)
  // screenToEyeSpacePerspective's depth terms for fragments at frag_z (the
  // camera rays): ndc z and the clip w, computed once per frame
  float persp_ndc_z, persp_cw;
  // multipliers for dividing by the frame's invariant integers (udiv_magic):
  // res[0], res[0] * res[1], width, width * height
  uint64_t m_res0, m_res01, m_width, m_pixels;
};

// Division by an integer d fixed for a frame, as one high multiply:
// floor(n / d) = floor(n * M / 2^64) with M = ceil(2^64 / d) for every
// n < 2^32 and 2 <= d < 2^32, since n * (M - 2^64 / d) / 2^64 < n / 2^64 < 1 / d
// keeps n * M / 2^64 below the next integer (Granlund and Montgomery,
// "Division by invariant integers using multiplication", 1994).  M = 0
// stands for d = 1.
__host__ __device__ __forceinline__ uint64_t udiv_magic(uint32_t d) {
  return d <= 1u ? 0ull : (~0ull / d) + 1ull;
}
#if defined(__CUDACC__)
__device__ __forceinline__ uint32_t udiv(uint32_t n, uint64_t m) {
  return m ? (uint32_t)__umul64hi((unsigned long long)n, m) : n;
}
#endif

// What the DDA needs of a volume: extents, bounds, brick layout, step cap.
struct Grid;
// Shape of a scene's bricks: log2 extents, sx + sy + sz = 6.
struct BrickShape {
  int32_t sx, sy, sz;
};
__host__ __device__ __forceinline__ int brick_bit_of(const BrickShape& b, int x, int y, int z) {
  return (x & ((1 << b.sx) - 1)) | ((y & ((1 << b.sy) - 1)) << b.sx) | ((z & ((1 << b.sz) - 1)) << (b.sx + b.sy));
}
// Index in the padded brick array (bx, by bricks inside the border) of the
// brick holding voxel (x, y, z), for voxels from -1 up to the volume's extent.
__host__ __device__ __forceinline__ int64_t brick_index_of(const BrickShape& b, int32_t bx, int32_t by, int x, int y,
                                                          int z) {
  return (int64_t)((x >> b.sx) + 1) + (int64_t)(bx + 2) * ((int64_t)((y >> b.sy) + 1) +
                                                           (int64_t)(by + 2) * (int64_t)((z >> b.sz) + 1));
}

struct Grid {
  int32_t rx, ry, rz;
  int32_t bx, bxy;           // padded brick-grid row and slice strides
  int32_t max_steps;         // int(2*ceil(length(vec3(res)))), dda.h:98
  float bminx, bminy, bminz;
  float vextx, vexty, vextz; // 1/(bmax-bmin), dda.h:16
  float bmaxx, bmaxy, bmaxz;
  int32_t shx, shy, shz;     // log2 of the brick extents
  int32_t shxy;              // shx + shy: bit of a brick's first z layer
  int32_t mx, my, mz;        // brick extents - 1
  int32_t n_words;           // words of the padded brick array (bounds of the checked build)
  const unsigned long long* bricks;   // brick (0,0,0) of the padded array
};

// Bit of voxel (x, y, z) in its brick word (brick shape shifts and masks).
__host__ __device__ __forceinline__ int brick_bit(int x, int y, int z, int shx, int shxy, int mx, int my, int mz) {
  return (x & mx) | ((y & my) << shx) | ((z & mz) << shxy);
}

// The DDA's view of a volume (frame uniforms + the job's brick array).
__host__ __device__ __forceinline__ Grid make_grid(const Frame& F, const unsigned long long* bricks) {
  Grid g;
  g.rx = F.res[0]; g.ry = F.res[1]; g.rz = F.res[2];
  g.bx = F.bdim[0] + 2; g.bxy = (F.bdim[0] + 2) * (F.bdim[1] + 2);
  g.max_steps = F.max_steps;
  g.bminx = F.bmin[0]; g.bminy = F.bmin[1]; g.bminz = F.bmin[2];
  g.vextx = F.vext[0]; g.vexty = F.vext[1]; g.vextz = F.vext[2];
  g.bmaxx = F.bmax[0]; g.bmaxy = F.bmax[1]; g.bmaxz = F.bmax[2];
  g.shx = F.bsh[0]; g.shy = F.bsh[1]; g.shz = F.bsh[2];
  g.shxy = F.bsh[0] + F.bsh[1];
  g.mx = (1 << F.bsh[0]) - 1; g.my = (1 << F.bsh[1]) - 1; g.mz = (1 << F.bsh[2]) - 1;
  const long long nw = (long long)g.bxy * (F.bdim[2] + 2);
  g.n_words = nw < 0x7fffffffLL ? (int32_t)nw : 0x7fffffff;
  g.bricks = bricks + 1 + g.bx + g.bxy;   // brick (0,0,0) inside the border
  return g;
}

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
  C_POSITIONS = 8,     // wavefront stream positions shaded (path-rounds; 0 in the plain form)
  C_NUM = 9
};

// Per-pixel first-hit record written by the diagnostic pass: voxel x, y, z
// and flags = normal code | hit << 8 | ground << 9, normal code =
// (nx+1) | (ny+1) << 2 | (nz+1) << 4.
struct HitRecord { int32_t x, y, z, flags; };

}  // namespace vt
