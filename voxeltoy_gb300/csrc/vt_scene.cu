// vt_scene.cu — kernels that build the device-resident scene and environment:
//   occupancy bit-bricks, emissive-voxel pruning flags and discovery, the
//   environment map's FP16 texels and importance-sampling CDFs (FP64 prefix
//   sums), and the triangle/voxel-overlap voxelizer.
#include <cuda_fp16.h>
#include <algorithm>
#include "vt_kernels.h"
#include "vt_builtins.h"

namespace vt {

// ------------------------------------------------------------- bit-bricks
// One thread per brick of the padded brick grid (one border brick on every
// side).  Voxels outside the volume read as occupied, so the DDA stops on
// the first voxel beyond the volume without a separate bounds test.
//
// With `max_entry`, the largest palette entry of the volume is atomically
// max-ed into *max_entry (the host checks it against the palette size).
__global__ void k_build_bricks(const uint8_t* __restrict__ grid, int32_t rx, int32_t ry, int32_t rz,
                               unsigned long long* __restrict__ bricks, int32_t bx, int32_t by, int32_t bz,
                               const BrickShape sh, unsigned long long* max_entry) {
  const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t px = bx + 2, py = by + 2, pz = bz + 2;
  unsigned top = 0;
  if (b < px * py * pz) {
    const int ex = 1 << sh.sx, ey = 1 << sh.sy, ez = 1 << sh.sz;
    const int x0 = ((int)(b % px) - 1) * ex;
    const int y0 = ((int)((b / px) % py) - 1) * ey;
    const int z0 = ((int)(b / (px * py)) - 1) * ez;
    unsigned long long w = 0ull;
    unsigned tops = 0u;   // byte-wise maximum of the word rows
    // 4x4x4 bricks: rows of four voxels as one aligned 32-bit word where the
    // brick's x range lies inside the volume and rows start on 4-byte
    // boundaries; the sixteen row loads are independent
    const bool words = sh.sx == 2 && sh.sy == 2 && (rx & 3) == 0 && x0 >= 0 && x0 + 4 <= rx;
    if (words) {
#pragma unroll
      for (int r = 0; r < 16; ++r) {
        const int y = y0 + (r & 3), z = z0 + (r >> 2);
        const bool in = y >= 0 && z >= 0 && y < ry && z < rz;
        const uint32_t v4 =
            in ? *reinterpret_cast<const uint32_t*>(grid + (size_t)x0 + (size_t)rx * ((size_t)y + (size_t)ry * (size_t)z))
               : 0u;
        tops = __vmaxu4(tops, v4);
        uint32_t m = __vcmpne4(v4, 0u) & 0x01010101u;   // bit 0 of each non-zero byte
        m = (m | (m >> 7) | (m >> 14) | (m >> 21)) & 0xfu;
        w |= (unsigned long long)(in ? m : 0xfu) << (4 * r);   // rows outside the volume read as set
      }
    } else {
      for (int k = 0; k < 64; ++k) {
        const int x = x0 + (k & (ex - 1)), y = y0 + ((k >> sh.sx) & (ey - 1)), z = z0 + (k >> (sh.sx + sh.sy));
        const bool outside = x < 0 || y < 0 || z < 0 || x >= rx || y >= ry || z >= rz;
        const unsigned v = outside ? 0u : grid[(size_t)x + (size_t)rx * ((size_t)y + (size_t)ry * (size_t)z)];
        top = v > top ? v : top;
        if (outside || v != 0) w |= 1ull << k;
      }
    }
    for (int k = 0; k < 32; k += 8) top = max(top, (tops >> k) & 0xffu);
    bricks[b] = w;
  }
  top = __reduce_max_sync(0xffffffffu, top);
  if (max_entry && (threadIdx.x & 31) == 0 && top) atomicMax(max_entry, (unsigned long long)top);
}

// One voxel edit: its grid entry and its bit in the padded brick grid.
__global__ void k_set_voxel(uint8_t* grid, unsigned long long* bricks, int32_t rx, int32_t ry, int32_t bx, int32_t by,
                            const BrickShape sh, int32_t x, int32_t y, int32_t z, uint8_t entry) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  grid[(size_t)x + (size_t)rx * ((size_t)y + (size_t)ry * (size_t)z)] = entry;
  const int64_t b = brick_index_of(sh, bx, by, x, y, z);
  const unsigned long long bit = 1ull << brick_bit_of(sh, x, y, z);
  if (entry) atomicOr(&bricks[b], bit);
  else atomicAnd(&bricks[b], ~bit);
}

cudaError_t launch_set_voxel(uint8_t* grid, unsigned long long* bricks, int32_t rx, int32_t ry, int32_t bx, int32_t by,
                             const BrickShape& sh, int32_t x, int32_t y, int32_t z, uint8_t entry, cudaStream_t st) {
  k_set_voxel<<<1, 32, 0, st>>>(grid, bricks, rx, ry, bx, by, sh, x, y, z, entry);
  return cudaGetLastError();
}

cudaError_t launch_build_bricks(const uint8_t* grid, int32_t rx, int32_t ry, int32_t rz,
                                unsigned long long* bricks, int32_t bx, int32_t by, int32_t bz, const BrickShape& sh,
                                unsigned long long* max_entry, cudaStream_t st) {
  const int64_t nb = (int64_t)(bx + 2) * (by + 2) * (bz + 2);
  k_build_bricks<<<(unsigned)((nb + 255) / 256), 256, 0, st>>>(grid, rx, ry, rz, bricks, bx, by, bz, sh, max_entry);
  return cudaGetLastError();
}

// --------------------------------------------------------- emissive voxels
// keep[i] = 1 if emissive voxel i has an empty or out-of-range 6-neighbour
// (anyVisibleFace, src/renderer/import.cpp:133-178).
__global__ void k_emissive_flags(const uint8_t* __restrict__ grid, int32_t rx, int32_t ry, int32_t rz,
                                 const int32_t* __restrict__ emissive, int64_t n, uint8_t* __restrict__ keep) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t v = emissive[i];
  const int64_t sxy = (int64_t)rx * ry;
  const int z = (int)(v / sxy);
  const int64_t r = v - (int64_t)z * sxy;
  const int y = (int)(r / rx);
  const int x = (int)(r - (int64_t)y * rx);
  const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  bool visible = false;
  for (int k = 0; k < 6 && !visible; ++k) {
    const int nx = x + off[k][0], ny = y + off[k][1], nz = z + off[k][2];
    if (nx < 0 || nx >= rx || ny < 0 || ny >= ry || nz < 0 || nz >= rz) { visible = true; break; }
    if (grid[(size_t)nx + (size_t)rx * ((size_t)ny + (size_t)ry * (size_t)nz)] == 0) visible = true;
  }
  keep[i] = visible ? 1 : 0;
}

cudaError_t launch_emissive_flags(const uint8_t* grid, int32_t rx, int32_t ry, int32_t rz,
                                  const int32_t* emissive, int64_t n, uint8_t* keep, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_emissive_flags<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(grid, rx, ry, rz, emissive, n, keep);
  return cudaGetLastError();
}

// Linear indices of voxels whose palette entry emits (emissive_entry[g] != 0),
// in increasing order: the volume is cut into chunks of kEmChunk voxels; one
// kernel counts each chunk's emissive voxels, one block turns the counts into
// chunk offsets, and a second pass over the chunks writes each chunk's
// indices from its offset, rows of 256 voxels at a time in voxel order.
constexpr int kEmThreads = 256;
constexpr int kEmRows = 16;
constexpr int64_t kEmChunk = (int64_t)kEmThreads * kEmRows;

// Exclusive prefix of `v` over the block (kThreads threads); *total gets the sum.
template <int kThreads = kEmThreads>
__device__ __forceinline__ uint32_t block_prefix(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  uint32_t before = 0, all = 0;
  for (int w = 0; w < kThreads / 32; ++w) {
    before += w < warp ? warp_sums[w] : 0u;
    all += warp_sums[w];
  }
  __syncthreads();   // warp_sums is reused by the next call
  *total = all;
  return before + x - v;
}

__global__ void k_emissive_count(const uint8_t* __restrict__ grid, int64_t n_voxels,
                                 const uint8_t* __restrict__ emissive_entry, uint32_t* __restrict__ counts) {
  __shared__ uint8_t s_em[256];
  __shared__ uint32_t s_warp[kEmThreads / 32];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) s_em[i] = emissive_entry[i];
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kEmChunk;
  uint32_t c = 0;
  for (int r = 0; r < kEmRows; ++r) {
    const int64_t i = base + (int64_t)r * kEmThreads + threadIdx.x;
    if (i < n_voxels && s_em[grid[i]]) ++c;
  }
  uint32_t total;
  block_prefix(c, s_warp, &total);
  if (threadIdx.x == 0) counts[blockIdx.x] = total;
}

// In place: counts[0..n) -> exclusive offsets, counts[n] = total.  One block
// of kScanThreads threads, each over a contiguous run of counts.
constexpr int kScanThreads = 1024;
__global__ void __launch_bounds__(kScanThreads) k_emissive_offsets(uint32_t* counts, int64_t n) {
  __shared__ uint32_t s_warp[kScanThreads / 32];
  const int64_t per = (n + kScanThreads - 1) / kScanThreads;
  const int64_t b = (int64_t)threadIdx.x * per, e = b + per < n ? b + per : n;
  uint32_t sum = 0;
  for (int64_t i = b; i < e; ++i) sum += counts[i];
  uint32_t total;
  uint32_t run = block_prefix<kScanThreads>(sum, s_warp, &total);
  for (int64_t i = b; i < e; ++i) {
    const uint32_t c = counts[i];
    counts[i] = run;
    run += c;
  }
  if (threadIdx.x == 0) counts[n] = total;
}

__global__ void k_emissive_write(const uint8_t* __restrict__ grid, int64_t n_voxels,
                                 const uint8_t* __restrict__ emissive_entry, const uint32_t* __restrict__ offsets,
                                 int32_t* __restrict__ out) {
  __shared__ uint8_t s_em[256];
  __shared__ uint32_t s_warp[kEmThreads / 32];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) s_em[i] = emissive_entry[i];
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kEmChunk;
  uint32_t at = offsets[blockIdx.x];
  for (int r = 0; r < kEmRows; ++r) {
    const int64_t i = base + (int64_t)r * kEmThreads + threadIdx.x;
    const bool e = i < n_voxels && s_em[grid[i]];
    uint32_t total;
    const uint32_t pre = block_prefix(e ? 1u : 0u, s_warp, &total);
    if (e) out[at + pre] = (int32_t)i;
    at += total;
  }
}

int64_t emissive_chunks(int64_t n_voxels) { return (n_voxels + kEmChunk - 1) / kEmChunk; }

cudaError_t launch_emissive_count(const uint8_t* grid, int64_t n_voxels, const uint8_t* emissive_entry,
                                  uint32_t* counts, cudaStream_t st) {
  const int64_t chunks = emissive_chunks(n_voxels);
  if (chunks <= 0) return cudaSuccess;
  k_emissive_count<<<(unsigned)chunks, kEmThreads, 0, st>>>(grid, n_voxels, emissive_entry, counts);
  k_emissive_offsets<<<1, kScanThreads, 0, st>>>(counts, chunks);
  return cudaGetLastError();
}

cudaError_t launch_emissive_write(const uint8_t* grid, int64_t n_voxels, const uint8_t* emissive_entry,
                                  const uint32_t* offsets, int32_t* out, cudaStream_t st) {
  const int64_t chunks = emissive_chunks(n_voxels);
  if (chunks <= 0) return cudaSuccess;
  k_emissive_write<<<(unsigned)chunks, kEmThreads, 0, st>>>(grid, n_voxels, emissive_entry, offsets, out);
  return cudaGetLastError();
}

// ------------------------------------------------------------ environment
// Three-tap Gaussian (sigma = 0.75 px) normalised to sum 1:
//   w_side = e / (1 + 2e), w_mid = 1 / (1 + 2e), e = exp(-1 / (2 * 0.75^2)).
#define VT_BLUR_SIDE 0.225610111284051620f
#define VT_BLUR_MID 0.548779777431896800f

// FP16 texels (A = 1) and the luminance of the quantised RGB
// (generateImageFunction's channel_sum, src/renderer/image.cpp:326-335).
// `bad` receives the smallest index of a texel with a non-finite channel.
__global__ void k_env_texels(const float* __restrict__ rgb, int64_t n, uint2* __restrict__ texels,
                             float* __restrict__ lum, uint32_t* bad) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (!(isfinite(rgb[3 * i]) && isfinite(rgb[3 * i + 1]) && isfinite(rgb[3 * i + 2]))) atomicMin(bad, (uint32_t)i);
  const uint16_t r = vtb::f2h(vtb::clamp_half(rgb[3 * i])), g = vtb::f2h(vtb::clamp_half(rgb[3 * i + 1])),
                 b = vtb::f2h(vtb::clamp_half(rgb[3 * i + 2]));
  texels[i] = make_uint2((uint32_t)r | ((uint32_t)g << 16), (uint32_t)b | (0x3c00u << 16));
  const float fr = vtb::h2f(r), fg = vtb::h2f(g), fb = vtb::h2f(b);
  lum[i] = (fr * 0.2126f + fg * 0.7152f) + fb * 0.0722f;
}

// 3x3 separable blur, clamp to edge (image.cpp:337-342), then the sin(theta)
// weight and the max(0, .) of calculateImageIntegral (image.cpp:361-374).
// Pass 0: horizontal into tmp; pass 1: vertical, * sin_theta[y] into func.
__global__ void k_env_blur(const float* __restrict__ src, float* __restrict__ dst, int32_t w, int32_t h,
                           int pass, const float* __restrict__ sin_theta) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)w * h) return;
  const int x = (int)(i % w), y = (int)(i / w);
  float a, b, c;
  if (pass == 0) {
    const int xm = x > 0 ? x - 1 : 0, xp = x < w - 1 ? x + 1 : w - 1;
    a = src[(int64_t)y * w + xm]; b = src[i]; c = src[(int64_t)y * w + xp];
  } else {
    const int ym = y > 0 ? y - 1 : 0, yp = y < h - 1 ? y + 1 : h - 1;
    a = src[(int64_t)ym * w + x]; b = src[i]; c = src[(int64_t)yp * w + x];
  }
  float v = (VT_BLUR_SIDE * a + VT_BLUR_MID * b) + VT_BLUR_SIDE * c;
  if (pass == 1) v = vtb::gmax(0.0f, v) * sin_theta[y];
  dst[i] = v;
}

// Exclusive prefix sums in FP64 with a fixed association order, so that the
// CPU restatement reproduces them exactly: consecutive chunks of 32 inputs
// are summed left to right, chunk offsets are accumulated left to right, and
// element prefix = chunk offset + in-chunk prefix.  out[0] = 0, out[n] = total.
// One warp; offs holds ceil(n/32) doubles.
template <typename T>
__device__ void warp_chunked_prefix(const T* in, int n, double* out, double* offs) {
  const int lane = threadIdx.x & 31;
  const int chunks = (n + 31) / 32;
  for (int c = lane; c < chunks; c += 32) {
    double acc = 0.0;
    const int end = min(n, (c + 1) * 32);
    for (int j = c * 32; j < end; ++j) { acc = acc + (double)in[j]; out[j + 1] = acc; }
  }
  __syncwarp();
  if (lane == 0) {
    out[0] = 0.0;
    double o = 0.0;
    offs[0] = 0.0;
    for (int c = 1; c < chunks; ++c) { o = o + out[c * 32]; offs[c] = o; }
  }
  __syncwarp();
  for (int c = lane; c < chunks; c += 32) {
    if (c == 0) continue;
    const double o = offs[c];
    const int end = min(n, (c + 1) * 32);
    for (int j = c * 32; j < end; ++j) out[j + 1] = o + out[j + 1];
  }
  __syncwarp();
}

// One warp per row (image.cpp:212-247): FP64 prefixes of the row function,
// normalised conditional CDF (uniform if the row is black), row integral =
// row sum / width.
__global__ void k_cdf_rows(const float* __restrict__ func, int32_t w, int32_t h, double* __restrict__ pre_all,
                           float* __restrict__ cdf_u, double* __restrict__ row_int) {
  extern __shared__ double s_offs[];
  const int row = blockIdx.x;
  const int lane = threadIdx.x & 31;
  if (row >= h) return;
  double* pre = pre_all + (int64_t)row * (w + 1);
  warp_chunked_prefix(func + (int64_t)row * w, w, pre, s_offs);
  const double total = pre[w];
  float* out = cdf_u + (int64_t)row * (w + 1);
  for (int x = lane; x <= w; x += 32) {
    if (total > 0.0) out[x] = (float)(pre[x] / total);
    else out[x] = (float)x / (float)w;
  }
  if (lane == 0) row_int[row] = total / (double)w;
}

// Marginal CDF over the row integrals (image.cpp:251-280) and the radiance
// integral 2 pi^2 * mean(f) (image.cpp:381-386).  One warp.
__global__ void k_cdf_marginal(const double* __restrict__ row_int, int32_t h, double* __restrict__ pre,
                               float* __restrict__ cdf_v, float* integral) {
  extern __shared__ double s_offs[];
  const int lane = threadIdx.x & 31;
  warp_chunked_prefix(row_int, h, pre, s_offs);
  const double total = pre[h];
  for (int y = lane; y <= h; y += 32) {
    if (total > 0.0) cdf_v[y] = (float)(pre[y] / total);
    else cdf_v[y] = (float)y / (float)h;
  }
  if (lane == 0 && integral) {
    *integral = (float)((total / (double)h) * (2.0 * 3.14159265358979323846 * 3.14159265358979323846));
  }
}

cudaError_t launch_cdf(const float* func, int32_t w, int32_t h, const EnvScratch& S, float* cdf_u,
                       float* cdf_v, float* integral, cudaStream_t st) {
  const size_t sm_rows = sizeof(double) * (size_t)((w + 31) / 32);
  const size_t sm_marg = sizeof(double) * (size_t)((h + 31) / 32);
  k_cdf_rows<<<h, 32, sm_rows, st>>>(func, w, h, S.row_pre, cdf_u, S.row_int);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_cdf_marginal<<<1, 32, sm_marg, st>>>(S.row_int, h, S.marg_pre, cdf_v, integral);
  return cudaGetLastError();
}

// The CDF image of a shrunk environment (image.cpp:308-320): each output
// texel is the area-weighted average of the FP16 texels its footprint
// covers (double sums, rows then columns in index order), then its Rec.709
// luminance.  A box filter standing in for OpenImageIO's resize.
__global__ void k_env_shrink_lum(const uint2* __restrict__ texels, int32_t w, int32_t h, int32_t ow, int32_t oh,
                                 float* __restrict__ lum) {
  const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= (int64_t)ow * oh) return;
  const int ox = (int)(o % ow), oy = (int)(o / ow);
  const double sx = (double)w / (double)ow, sy = (double)h / (double)oh;
  const double y0 = (double)oy * sy, y1 = (double)(oy + 1) * sy;
  const double x0 = (double)ox * sx, x1 = (double)(ox + 1) * sx;
  double acc0 = 0.0, acc1 = 0.0, acc2 = 0.0;
  for (int j = (int)floor(y0); j < (int)ceil(y1) && j < h; ++j) {
    const double wy = fmin(y1, (double)(j + 1)) - fmax(y0, (double)j);
    for (int i = (int)floor(x0); i < (int)ceil(x1) && i < w; ++i) {
      const double wx = fmin(x1, (double)(i + 1)) - fmax(x0, (double)i);
      const double wgt = wx * wy;
      const uint2 q = texels[(int64_t)j * w + i];
      acc0 = acc0 + wgt * (double)vtb::h2f((uint16_t)(q.x & 0xffffu));
      acc1 = acc1 + wgt * (double)vtb::h2f((uint16_t)(q.x >> 16));
      acc2 = acc2 + wgt * (double)vtb::h2f((uint16_t)(q.y & 0xffffu));
    }
  }
  const double area = sx * sy;
  const float fr = (float)(acc0 / area), fg = (float)(acc1 / area), fb = (float)(acc2 / area);
  lum[o] = (fr * 0.2126f + fg * 0.7152f) + fb * 0.0722f;
}

cudaError_t launch_env_build(const float* rgb, int32_t w, int32_t h, int32_t cw, int32_t ch, const EnvScratch& S,
                             uint2* texels, float* cdf_u, float* cdf_v, float* integral, uint32_t* bad,
                             cudaStream_t st) {
  const int64_t n = (int64_t)w * h;
  k_env_texels<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(rgb, n, texels, S.lum, bad);
  const int64_t m = (int64_t)cw * ch;
  const unsigned blocks = (unsigned)((m + 255) / 256);
  if (cw != w || ch != h) k_env_shrink_lum<<<blocks, 256, 0, st>>>(texels, w, h, cw, ch, S.lum);
  k_env_blur<<<blocks, 256, 0, st>>>(S.lum, S.tmp, cw, ch, 0, S.sin_theta);
  k_env_blur<<<blocks, 256, 0, st>>>(S.tmp, S.func, cw, ch, 1, S.sin_theta);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_cdf(S.func, cw, ch, S, cdf_u, cdf_v, integral, st);
}

// --------------------------------------------------------------- voxelizer
// Rauwendaal & Bailey, "Hybrid Computational Voxelization Using the Graphics
// Pipeline" (JCGT 2013) as implemented by src/shaders/shared/voxelize.gs:55-251
// and src/voxelize/cpuVoxelizer.cpp:42-235: project on the dominant axis,
// test the XY edge functions per column, derive the Z range from the plane,
// test the YZ and ZX edge functions per voxel.  mode 0 = THIN (6-separating,
// figure 18), 1 = FAT (conservative, figure 17).  The scan range of a
// triangle is its bounding box in the swizzled frame, clamped to the grid's
// extent along the swizzled axes; with ref_bounds, against the unswizzled
// resolution as voxelize.gs:247-248 does (the same on cubic grids; on others
// voxels near the far faces of the shorter axes are lost).  FAT without
// ref_bounds marks exactly the voxels that a separating-axis test marks,
// up to float rounding where a voxel only touches the triangle.
struct TriSetup {
  float d_xy[3], d_yz[3], d_zx[3];
  float n_xy[3][2], n_yz[3][2], n_zx[3][2];
  float nproj[3];
  float dmin, dmax, nz_inv;
  int perm;           // 0: swizzled yzx, 1: zxy, 2: identity
  int lo[3], hi[3];   // voxel index range in swizzled space
  bool valid;
};

__device__ __forceinline__ int sat_int(float f) {
  // float -> int with NaN and out-of-range values mapped into +-1e9
  if (f >= -1.0e9f && f <= 1.0e9f) return (int)f;
  return f > 0.0f ? 1000000000 : -1000000000;
}

__device__ __forceinline__ void edge_normal(float ea, float eb, bool pos, float* nrm) {
  // pos ? vec2(-eb, ea) : vec2(eb, -ea) for an edge (ea, eb)
  if (pos) { nrm[0] = -eb; nrm[1] = ea; } else { nrm[0] = eb; nrm[1] = -ea; }
}

__device__ __forceinline__ float edge_d(const float* nrm, float pa, float pb, int mode) {
  if (mode == 0) {
    // dot(n, .5 - v) + 0.5 * max(|n.x|, |n.y|)   (voxelize.gs:140-150)
    return (nrm[0] * (0.5f - pa) + nrm[1] * (0.5f - pb)) + 0.5f * vtb::gmax(fabsf(nrm[0]), fabsf(nrm[1]));
  }
  // -dot(n, v) + max(0, n.x) + max(0, n.y)      (voxelize.gs:152-162)
  return (-(nrm[0] * pa + nrm[1] * pb) + vtb::gmax(0.0f, nrm[0])) + vtb::gmax(0.0f, nrm[1]);
}

__device__ bool tri_setup(const float* V, int64_t nv, const uint32_t* I, int64_t t, int32_t rx, int32_t ry,
                          int32_t rz, int mode, bool ref_bounds, TriSetup& S) {
  float v[3][3];
  for (int k = 0; k < 3; ++k) {
    const uint32_t vi = I[3 * t + k];
    if ((int64_t)vi >= nv) return false;   // recorded by k_mesh_scan; the call fails
    v[k][0] = V[3 * (int64_t)vi]; v[k][1] = V[3 * (int64_t)vi + 1]; v[k][2] = V[3 * (int64_t)vi + 2];
  }
  // n = cross(v1 - v0, v2 - v1)   (voxelize.gs:62)
  const float a0 = v[1][0] - v[0][0], a1 = v[1][1] - v[0][1], a2 = v[1][2] - v[0][2];
  const float b0 = v[2][0] - v[1][0], b1 = v[2][1] - v[1][1], b2 = v[2][2] - v[1][2];
  float n[3] = {a1 * b2 - b1 * a2, a2 * b0 - b2 * a0, a0 * b1 - b0 * a1};
  const float ax = fabsf(n[0]), ay = fabsf(n[1]), az = fabsf(n[2]);
  int perm;
  if (ax >= ay && ax >= az) perm = 0;        // look down X: xyz <- yzx
  else if (ay >= ax && ay >= az) perm = 1;   // look down Y: xyz <- zxy
  else perm = 2;
  if (perm != 2) {
    const int i0 = perm == 0 ? 1 : 2, i1 = perm == 0 ? 2 : 0, i2 = perm == 0 ? 0 : 1;
    for (int k = 0; k < 3; ++k) {
      const float p0 = v[k][i0], p1 = v[k][i1], p2 = v[k][i2];
      v[k][0] = p0; v[k][1] = p1; v[k][2] = p2;
    }
    const float m0 = n[i0], m1 = n[i1], m2 = n[i2];
    n[0] = m0; n[1] = m1; n[2] = m2;
  }
  S.perm = perm;
  // grid extent along the swizzled axes: yzx -> (ry, rz, rx), zxy -> (rz, rx, ry)
  int res[3] = {rx, ry, rz};
  if (!ref_bounds && perm == 0) { res[0] = ry; res[1] = rz; res[2] = rx; }
  if (!ref_bounds && perm == 1) { res[0] = rz; res[1] = rx; res[2] = ry; }
  // ivec3(clamp(floor(min), 0, res)), ivec3(clamp(ceil(max), 0, res))
  // (voxelize.gs:247-248); a FAT scan also takes the voxels that only touch
  // the triangle at an integer bound, ceil(min) - 1 and floor(max) + 1, which
  // that range skips (a triangle lying in an integer plane would mark nothing).
  const bool touch = !ref_bounds && mode == 1;
  for (int c = 0; c < 3; ++c) {
    const float mn = vtb::gmin(vtb::gmin(v[0][c], v[1][c]), v[2][c]);
    const float mx = vtb::gmax(vtb::gmax(v[0][c], v[1][c]), v[2][c]);
    const int l = touch ? sat_int(ceilf(mn)) - 1 : sat_int(floorf(mn));
    const int u = touch ? sat_int(floorf(mx)) + 1 : sat_int(ceilf(mx));
    S.lo[c] = min(max(l, 0), res[c]);
    S.hi[c] = min(max(u, 0), res[c]);
  }
  float e[3][3];
  for (int c = 0; c < 3; ++c) {
    e[0][c] = v[1][c] - v[0][c];
    e[1][c] = v[2][c] - v[1][c];
    e[2][c] = v[0][c] - v[2][c];
  }
  for (int k = 0; k < 3; ++k) {
    edge_normal(e[k][0], e[k][1], n[2] >= 0.0f, S.n_xy[k]);   // (x, y)
    edge_normal(e[k][1], e[k][2], n[0] >= 0.0f, S.n_yz[k]);   // (y, z)
    edge_normal(e[k][2], e[k][0], n[1] >= 0.0f, S.n_zx[k]);   // (z, x)
    S.d_xy[k] = edge_d(S.n_xy[k], v[k][0], v[k][1], mode);
    S.d_yz[k] = edge_d(S.n_yz[k], v[k][1], v[k][2], mode);
    S.d_zx[k] = edge_d(S.n_zx[k], v[k][2], v[k][0], mode);
  }
  const bool neg = n[2] < 0.0f;
  S.nproj[0] = neg ? -n[0] : n[0]; S.nproj[1] = neg ? -n[1] : n[1]; S.nproj[2] = neg ? -n[2] : n[2];
  const float dtri = (S.nproj[0] * v[0][0] + S.nproj[1] * v[0][1]) + S.nproj[2] * v[0][2];
  if (mode == 0) {
    S.dmin = dtri - (S.nproj[0] * 0.5f + S.nproj[1] * 0.5f);  // voxelize.gs:169
    S.dmax = S.dmin;
  } else {
    S.dmin = (dtri - vtb::gmax(S.nproj[0], 0.0f)) - vtb::gmax(S.nproj[1], 0.0f);   // :171
    S.dmax = (dtri - vtb::gmin(S.nproj[0], 0.0f)) - vtb::gmin(S.nproj[1], 0.0f);   // :172
  }
  S.valid = S.nproj[2] != 0.0f;   // zero-area triangles cover nothing
  S.nz_inv = 1.0f / S.nproj[2];
  return S.valid;
}

// Where a voxelized voxel is recorded: its grid byte and, when the scene's
// bricks are being built alongside, its bit of the padded brick grid.
struct VoxOut {
  uint8_t* grid;
  uint8_t value;
  unsigned long long* bricks;   // nullable
  int32_t bx, by;               // bricks per row / column inside the border
  BrickShape sh;
};

// Brick bits a thread has set, gathered while they fall in one brick and
// OR'ed into the brick grid with one atomic when the brick changes.
struct BrickAcc {
  int64_t b = -1;
  unsigned long long bits = 0ull;
  __device__ __forceinline__ void add(const VoxOut& O, int64_t nb, unsigned long long bit) {
    if (nb != b) {
      flush(O);
      b = nb;
    }
    bits |= bit;
  }
  __device__ __forceinline__ void flush(const VoxOut& O) {
    if (bits) atomicOr(&O.bricks[b], bits);
    bits = 0ull;
  }
};

__device__ __forceinline__ void tri_column(const TriSetup& S, int px, int py, int mode, int32_t rx, int32_t ry,
                                           int32_t rz, const VoxOut& O, BrickAcc& acc) {
  bool xy = true;
  for (int k = 0; k < 3; ++k) {
    const float dd = S.d_xy[k] + (S.n_xy[k][0] * (float)px + S.n_xy[k][1] * (float)py);
    xy = xy && (dd >= 0.0f);
  }
  if (!xy) return;
  const float dnp = S.nproj[0] * (float)px + S.nproj[1] * (float)py;
  const float zmin_i = (-dnp + S.dmin) * S.nz_inv;
  const float zmax_i = (-dnp + S.dmax) * S.nz_inv;
  const float zmin_f = floorf(zmin_i), zmax_c = ceilf(zmax_i);
  int zmin = sat_int(zmin_f) - (zmin_f == zmin_i ? 1 : 0);
  int zmax = sat_int(zmax_c) + (zmax_c == zmax_i ? 1 : 0);
  zmin = max(S.lo[2], zmin);
  zmax = min(S.hi[2], zmax);
  for (int pz = zmin; pz < zmax; ++pz) {
    bool ok = true;
    for (int k = 0; k < 3; ++k) {
      const float dyz = S.d_yz[k] + (S.n_yz[k][0] * (float)py + S.n_yz[k][1] * (float)pz);
      const float dzx = S.d_zx[k] + (S.n_zx[k][0] * (float)pz + S.n_zx[k][1] * (float)px);
      ok = ok && (dyz >= 0.0f) && (dzx >= 0.0f);
    }
    if (!ok) continue;
    // unswizzle (voxelize.gs:40-48): yzx -> (z, x, y), zxy -> (y, z, x)
    int ox, oy, oz;
    if (S.perm == 0) { ox = pz; oy = px; oz = py; }
    else if (S.perm == 1) { ox = py; oy = pz; oz = px; }
    else { ox = px; oy = py; oz = pz; }
    // imageStore outside the image has no effect
    if (ox < 0 || oy < 0 || oz < 0 || ox >= rx || oy >= ry || oz >= rz) continue;
    O.grid[(size_t)ox + (size_t)rx * ((size_t)oy + (size_t)ry * (size_t)oz)] = O.value;
    if (O.bricks) acc.add(O, brick_index_of(O.sh, O.bx, O.by, ox, oy, oz), 1ull << brick_bit_of(O.sh, ox, oy, oz));
  }
  (void)mode;
}

constexpr int kLargeColumns = 64;

// One thread per triangle for triangles whose XY footprint is small; larger
// ones are appended to a list for the block-per-triangle kernel.
__global__ void k_vox_small(const float* __restrict__ V, int64_t nv, const uint32_t* __restrict__ I,
                            int64_t n_tris, int32_t rx, int32_t ry, int32_t rz, int mode, bool ref_bounds,
                            const VoxOut O, int64_t* large, unsigned long long* n_large) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tris) return;
  TriSetup S;
  if (!tri_setup(V, nv, I, t, rx, ry, rz, mode, ref_bounds, S)) return;
  const int64_t cols = (int64_t)(S.hi[0] - S.lo[0]) * (int64_t)(S.hi[1] - S.lo[1]);
  if (cols > kLargeColumns) {
    const unsigned long long slot = atomicAdd(n_large, 1ull);
    large[slot] = t;
    return;
  }
  BrickAcc acc;
  for (int px = S.lo[0]; px < S.hi[0]; ++px)
    for (int py = S.lo[1]; py < S.hi[1]; ++py) tri_column(S, px, py, mode, rx, ry, rz, O, acc);
  if (O.bricks) acc.flush(O);
}

__global__ void k_vox_large(const float* __restrict__ V, int64_t nv, const uint32_t* __restrict__ I,
                            const int64_t* large, const unsigned long long* n_large, int32_t rx, int32_t ry,
                            int32_t rz, int mode, bool ref_bounds, const VoxOut O) {
  __shared__ TriSetup S;
  const unsigned long long n = *n_large;
  for (unsigned long long k = blockIdx.x; k < n; k += gridDim.x) {
    __syncthreads();
    if (threadIdx.x == 0) tri_setup(V, nv, I, large[k], rx, ry, rz, mode, ref_bounds, S);   // listed: valid
    __syncthreads();
    const int wx = S.hi[0] - S.lo[0], wy = S.hi[1] - S.lo[1];
    const int64_t cols = (int64_t)wx * wy;
    BrickAcc acc;
    for (int64_t c = threadIdx.x; c < cols; c += blockDim.x) {
      const int px = S.lo[0] + (int)(c / wy), py = S.lo[1] + (int)(c % wy);
      tri_column(S, px, py, mode, rx, ry, rz, O, acc);
    }
    if (O.bricks) acc.flush(O);
  }
}

// Scratch of a voxelization: the large-triangle list, then 256 bytes for its
// length, then 256 bytes for the MeshPrep record.
static size_t large_list_bytes(int64_t n_tris) {
  return (sizeof(int64_t) * (size_t)std::max<int64_t>(n_tris, 1) + 255) / 256 * 256;
}
size_t voxelize_scratch_bytes(int64_t n_tris) { return large_list_bytes(n_tris) + 512; }
MeshPrep* voxelize_prep_record(void* scratch, int64_t n_tris) {
  return (MeshPrep*)((char*)scratch + large_list_bytes(n_tris) + 256);
}

// Order-preserving 32-bit keys of floats (not NaN): unsigned comparison of
// keys is float comparison, with -0 below +0.
__device__ __forceinline__ uint32_t fkey(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fkey_value(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// Triangle indices at or past the vertex count (the largest one is kept),
// and with `bounds` the vertices' bounding box (NaN coordinates ignored, as
// the left-to-right min / max of import.cpp:49-52 ignores them).
__global__ void __launch_bounds__(256) k_mesh_scan(const float* __restrict__ V, int64_t nv,
                                                   const uint32_t* __restrict__ I, int64_t n_idx, bool bounds,
                                                   MeshPrep* P) {
  uint32_t lo[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, hi[3] = {0u, 0u, 0u};
  unsigned long long bad = 0ull;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_idx; i += stride) {
    const uint32_t vi = I[i];
    if ((int64_t)vi >= nv) bad = max(bad, (1ull << 32) | vi);
  }
  if (bounds)
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += stride)
      for (int c = 0; c < 3; ++c) {
        const float f = V[3 * i + c];
        if (f == f) {
          lo[c] = min(lo[c], fkey(f));
          hi[c] = max(hi[c], fkey(f));
        }
      }
  // warp, then block (256 threads), then one atomic per value and block
  for (int o = 16; o > 0; o >>= 1) {
    bad = max(bad, __shfl_xor_sync(0xffffffffu, bad, o));
    for (int c = 0; c < 3; ++c) {
      lo[c] = min(lo[c], __shfl_xor_sync(0xffffffffu, lo[c], o));
      hi[c] = max(hi[c], __shfl_xor_sync(0xffffffffu, hi[c], o));
    }
  }
  __shared__ unsigned long long s_bad[8];
  __shared__ uint32_t s_lo[3][8], s_hi[3][8];
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_bad[warp] = bad;
    for (int c = 0; c < 3; ++c) { s_lo[c][warp] = lo[c]; s_hi[c][warp] = hi[c]; }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      bad = max(bad, s_bad[w]);
      for (int c = 0; c < 3; ++c) { lo[c] = min(lo[c], s_lo[c][w]); hi[c] = max(hi[c], s_hi[c][w]); }
    }
    if (bad) atomicMax(&P->bad, bad);
    if (bounds)
      for (int c = 0; c < 3; ++c) {
        if (lo[c] != 0xffffffffu) atomicMin(&P->kmin[c], lo[c]);
        if (hi[c] != 0u) atomicMax(&P->kmax[c], hi[c]);
      }
  }
}

// computeMeshTransform (import.cpp:46-64) from the scanned bounds, in the
// host's float and double arithmetic, then the vertex shader's
// modelTransform * v * voxelResolution (voxelize.vs:20-27) on every vertex in
// place.  One block; every thread computes the same matrix.
__global__ void k_mesh_fit(float* __restrict__ V, int64_t nv, int32_t rx, int32_t ry, int32_t rz,
                           const MeshPrep* P) {
  float bmin[3], bmax[3];
  for (int c = 0; c < 3; ++c) {   // an axis whose coordinates are all NaN keeps +inf / -inf, as on the host
    bmin[c] = P->kmin[c] == 0xffffffffu ? INFINITY : fkey_value(P->kmin[c]);
    bmax[c] = P->kmax[c] == 0u ? -INFINITY : fkey_value(P->kmax[c]);
  }
  const float res[3] = {(float)rx, (float)ry, (float)rz};
  float size[3], margin[3];
  for (int c = 0; c < 3; ++c) { size[c] = bmax[c] - bmin[c]; margin[c] = 1.0f / res[c]; }
  int major = 0;
  if (size[1] > size[major]) major = 1;
  if (size[2] > size[major]) major = 2;
  const float sc = (float)((1.0f - 2.0 * (double)margin[major]) / (double)size[major]);
  float M[12];
  for (int r = 0; r < 3; ++r) {
    const float t = -bmin[r] + margin[r] / sc;
    M[4 * r] = r == 0 ? sc : 0.0f;
    M[4 * r + 1] = r == 1 ? sc : 0.0f;
    M[4 * r + 2] = r == 2 ? sc : 0.0f;
    M[4 * r + 3] = t * sc;
  }
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += stride) {
    const float x = V[3 * i], y = V[3 * i + 1], z = V[3 * i + 2];
    for (int r = 0; r < 3; ++r) {
      const float p = ((M[4 * r] * x + M[4 * r + 1] * y) + M[4 * r + 2] * z) + M[4 * r + 3] * 1.0f;
      V[3 * i + r] = p * res[r];
    }
  }
}

cudaError_t launch_mesh_prep(float* V, int64_t nv, const uint32_t* I, int64_t n_tris, bool fit, int32_t rx,
                             int32_t ry, int32_t rz, MeshPrep* P, int sm_count, cudaStream_t st) {
  MeshPrep init;
  for (int c = 0; c < 3; ++c) { init.kmin[c] = 0xffffffffu; init.kmax[c] = 0u; }
  init.bad = 0ull;
  // pageable source: read when the copy returns
  cudaError_t e = cudaMemcpyAsync(P, &init, sizeof(init), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  const int64_t work = std::max<int64_t>(3 * n_tris, fit ? nv : 0);
  if (work <= 0) return cudaSuccess;
  const int blocks = (int)std::min<int64_t>((work + 255) / 256, (int64_t)sm_count * 8);
  k_mesh_scan<<<blocks, 256, 0, st>>>(V, nv, I, 3 * n_tris, fit, P);   // 256 threads: eight warps
  if (fit && nv > 0) {
    // the matrix needs the whole scan: a second launch, each block rebuilds it
    const int fb = (int)std::min<int64_t>((nv + 255) / 256, (int64_t)sm_count * 8);
    k_mesh_fit<<<fb, 256, 0, st>>>(V, nv, rx, ry, rz, P);
  }
  return cudaGetLastError();
}

cudaError_t launch_voxelize(const float* verts_voxel_space, int64_t n_vertices, const uint32_t* indices,
                            int64_t n_tris, int32_t rx, int32_t ry, int32_t rz, int32_t mode, bool reference_bounds,
                            uint8_t* grid, uint8_t value, unsigned long long* bricks, int32_t bx, int32_t by,
                            const BrickShape& sh, void* scratch, int large_blocks, cudaStream_t st) {
  if (n_tris <= 0) return cudaSuccess;
  int64_t* large = (int64_t*)scratch;
  unsigned long long* n_large = (unsigned long long*)((char*)scratch + large_list_bytes(n_tris));
  cudaError_t e = cudaMemsetAsync(n_large, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  VoxOut O;
  O.grid = grid;
  O.value = value;
  O.bricks = bricks ? bricks : nullptr;
  O.bx = bx;
  O.by = by;
  O.sh = sh;
  k_vox_small<<<(unsigned)((n_tris + 127) / 128), 128, 0, st>>>(verts_voxel_space, n_vertices, indices, n_tris, rx,
                                                                ry, rz, mode, reference_bounds, O, large, n_large);
  k_vox_large<<<std::max(1, large_blocks), 256, 0, st>>>(verts_voxel_space, n_vertices, indices, large, n_large, rx,
                                                         ry, rz, mode, reference_bounds, O);
  return cudaGetLastError();
}

// Word of brick (ix, iy, iz) of the padded grid of an empty volume: all bits
// of a border brick, and of an interior brick the bits of voxels at or
// beyond (rx, ry, rz); zero for every other brick.
__device__ __forceinline__ unsigned long long empty_brick_word(int ix, int iy, int iz, int32_t px, int32_t py,
                                                               int32_t pz, int32_t rx, int32_t ry, int32_t rz,
                                                               const BrickShape& sh) {
  if (ix == 0 || iy == 0 || iz == 0 || ix == px - 1 || iy == py - 1 || iz == pz - 1) return ~0ull;   // border
  const int ex = 1 << sh.sx, ey = 1 << sh.sy, ez = 1 << sh.sz;
  const int x0 = (ix - 1) * ex, y0 = (iy - 1) * ey, z0 = (iz - 1) * ez;
  unsigned long long w = 0ull;
  if (x0 < 0 || y0 < 0 || z0 < 0 || x0 + ex > rx || y0 + ey > ry || z0 + ez > rz) {
    for (int k = 0; k < 64; ++k) {
      const int x = x0 + (k & (ex - 1)), y = y0 + ((k >> sh.sx) & (ey - 1)), z = z0 + (k >> (sh.sx + sh.sy));
      if (x < 0 || y < 0 || z < 0 || x >= rx || y >= ry || z >= rz) w |= 1ull << k;
    }
  }
  return w;
}

// The bricks of an empty volume that are not zero, over a zeroed array: the
// border and the last interior brick along each axis (the only interior
// bricks that can reach past the volume).  One warp per row of the padded
// grid: rows in the y or z shell are written whole, the others at their
// three x-shell bricks (0, px - 2, px - 1).
__global__ void k_bricks_shell(unsigned long long* __restrict__ bricks, int32_t rx, int32_t ry, int32_t rz,
                               int32_t bx, int32_t by, int32_t bz, const BrickShape sh) {
  const int px = bx + 2, py = by + 2, pz = bz + 2;
  const int lane = threadIdx.x & 31;
  const int64_t rows = (int64_t)py * pz;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t r = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += warps) {
    const int iz = (int)(r / py), iy = (int)(r - (int64_t)iz * py);
    unsigned long long* row = bricks + r * px;
    if (iy == 0 || iy >= py - 2 || iz == 0 || iz >= pz - 2) {
      for (int ix = lane; ix < px; ix += 32) row[ix] = empty_brick_word(ix, iy, iz, px, py, pz, rx, ry, rz, sh);
    } else if (lane < 3) {
      const int ix = lane == 0 ? 0 : px - 3 + lane;
      row[ix] = empty_brick_word(ix, iy, iz, px, py, pz, rx, ry, rz, sh);
    }
  }
}

cudaError_t launch_bricks_init(unsigned long long* bricks, int32_t rx, int32_t ry, int32_t rz, int32_t bx,
                               int32_t by, int32_t bz, const BrickShape& sh, cudaStream_t st) {
  // a linear zero fill runs at copy bandwidth; the shell is a few rows' worth
  const int64_t px = bx + 2, py = by + 2, pz = bz + 2;
  cudaError_t e = cudaMemsetAsync(bricks, 0, sizeof(unsigned long long) * (size_t)(px * py * pz), st);
  if (e != cudaSuccess) return e;
  const int64_t blocks = std::min<int64_t>((py * pz + 7) / 8, 8192);
  k_bricks_shell<<<(unsigned)blocks, 256, 0, st>>>(bricks, rx, ry, rz, bx, by, bz, sh);
  return cudaGetLastError();
}

}  // namespace vt
