// vt_shade.cuh — device code of one progressive path sample, written as a
// per-lane state machine: a path alternates between DDA segments (the hot
// loop) and segment-end events (shading, light sampling, BSDF sampling).
// Both the plain kernel (one launch per pass) and the persistent kernel
// (many jobs and passes per launch) drive this same state machine, so every
// form produces the same bits for the same (job, pixel, sample).
//
// Semantics follow the reference integrator pass
// (src/shaders/integrator/pathTracer.fs:64-296 and the headers it includes);
// each function cites the lines it implements.  Arithmetic is written in the
// reference's expression order with multiply-add contraction disabled
// (-fmad=false) so that the results equal the CPU restatement bit for bit.
#pragma once

#include <cuda_fp16.h>
#include "vt_internal.h"
#include "vt_builtins.h"

namespace vt {

#define VT_D __device__ __forceinline__

// constants.h:1-3 (float literals)
constexpr float kPI = 3.14159265359f;
constexpr float kTWO_PI = 6.28318530718f;
constexpr float kINV_TWOPI = 0.15915494309f;

// ------------------------------------------------------------------ vectors
struct v3 { float x, y, z; };
VT_D v3 mk3(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
VT_D v3 operator+(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
VT_D v3 operator-(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
VT_D v3 operator*(v3 a, v3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
VT_D v3 operator/(v3 a, v3 b) { return mk3(a.x / b.x, a.y / b.y, a.z / b.z); }
VT_D v3 operator*(v3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
VT_D v3 operator*(float s, v3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
VT_D v3 operator/(v3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
VT_D v3 operator-(v3 a) { return mk3(-a.x, -a.y, -a.z); }
VT_D float dot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
VT_D v3 cross(v3 a, v3 b) {
  return mk3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
VT_D float length(v3 a) { return sqrtf(dot(a, a)); }
VT_D v3 normalize(v3 a) { return a / length(a); }
VT_D v3 vabs3(v3 a) { return mk3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
VT_D v3 ld3(const float* p) { return mk3(p[0], p[1], p[2]); }
VT_D bool finite3(v3 a) {
  const float inf = __int_as_float(0x7f800000);
  return fabsf(a.x) < inf && fabsf(a.y) < inf && fabsf(a.z) < inf;
}

// GLSL mat4 * vec4 with the matrix stored row-major (uploaded transposed).
VT_D float4 mul4(const float* m, float4 v) {
  float4 r;
  r.x = ((m[0] * v.x + m[1] * v.y) + m[2] * v.z) + m[3] * v.w;
  r.y = ((m[4] * v.x + m[5] * v.y) + m[6] * v.z) + m[7] * v.w;
  r.z = ((m[8] * v.x + m[9] * v.y) + m[10] * v.z) + m[11] * v.w;
  r.w = ((m[12] * v.x + m[13] * v.y) + m[14] * v.z) + m[15] * v.w;
  return r;
}

// ------------------------------------------------------------ checked build
// With VT_CHECKED every data-dependent gather of the path checks its index;
// a failed check ORs its bit into this module's check word (read by
// vt_diag_check_word) and the gather reads a neutral value instead: no
// trap, the launch runs to its end.  Without VT_CHECKED the checks compile
// away.
enum : uint32_t {
  CHK_BRICK = 1u << 0,     // brick word outside the padded brick array
  CHK_GRID = 1u << 1,      // voxel outside the volume
  CHK_PALETTE = 1u << 2,   // palette entry beyond the palette
  CHK_EMISSIVE = 1u << 3,  // emissive-list entry outside the volume
  CHK_TEXEL = 1u << 4,     // environment texel outside the image
  CHK_CDF = 1u << 5,       // CDF entry outside its table
  CHK_SAMPLE = 1u << 6,    // sample-buffer item beyond the launch's items
  CHK_NOISE = 1u << 7,     // noise-table texel outside the table
};
#ifdef VT_CHECKED
static __device__ unsigned int g_check_word;
VT_D bool chk(bool ok, uint32_t code) {
  if (!ok) atomicOr(&g_check_word, code);
  return ok;
}
#else
VT_D bool chk(bool, uint32_t) { return true; }
#endif

// ---------------------------------------------------------------- counters
template <bool kCount>
struct Cnt {
  unsigned long long c[C_NUM];
  VT_D void add(int i, unsigned long long v) { if (kCount) c[i] += v; }
};

// ---------------------------------------------------------------------- rng
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
// easy as 1, 2, 3", SC 2011): 10 rounds of two 32x32->64 multiplies with a
// Weyl-sequence key schedule.
VT_D uint4 philox(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    const uint32_t lo0 = 0xD2511F53u * c0, hi0 = __umulhi(0xD2511F53u, c0);
    const uint32_t lo1 = 0xCD9E8D57u * c2, hi1 = __umulhi(0xCD9E8D57u, c2);
    const uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  return make_uint4(c0, c1, c2, c3);
}
constexpr uint32_t kPhiloxKey1 = 0x6A09E667u;

VT_D float u01(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-8f; }

// Wang hash on a signed int (random.h:3-11): arithmetic shifts, wrapping products.
VT_D int32_t wang_hash(int32_t s) {
  s = (s ^ 61) ^ (s >> 16);
  s = (int32_t)((uint32_t)s * 9u);
  s = s ^ (s >> 4);
  s = (int32_t)((uint32_t)s * 0x27d4eb2du);
  s = s ^ (s >> 15);
  return s;
}

struct Rng {
  uint32_t pixel;   // philox counter word 0
  uint32_t sample;  // philox counter word 1
  uint32_t call;    // philox counter word 2 (rand() calls so far)
  int32_t ox, oy;   // noise-table walk position
};

// randomNumberGeneratorOffset (random.h:13-18).  The reference takes % of a
// possibly negative int; the offset is read as unsigned here.
VT_D void rng_init(const Frame& F, Rng& r, int px, int py, int sample) {
  r.pixel = (uint32_t)(py * F.width + px);
  r.sample = (uint32_t)sample;
  r.call = 0;
  r.ox = r.oy = 0;
  if (F.rng_mode != 1) return;   // the walk position matters only to the noise table
  const uint32_t off = (uint32_t)(wang_hash(px + py * kNoiseW) ^ wang_hash(sample));
  r.ox = (int32_t)(off % (uint32_t)kNoiseW);
  r.oy = (int32_t)((off / (uint32_t)kNoiseW) % (uint32_t)kNoiseH);
}

// rand (random.h:20-27) or one Philox block.
VT_D float4 rng_next(const Frame& F, const JobDev& J, Rng& r) {
  if (F.rng_mode == 1) {
    const float4 v = chk((unsigned)r.ox < (unsigned)kNoiseW && (unsigned)r.oy < (unsigned)kNoiseH, CHK_NOISE)
                         ? __ldg(&J.noise[r.oy * kNoiseW + r.ox]) : make_float4(0.f, 0.f, 0.f, 0.f);
    r.ox = (r.ox + 1) % kNoiseW;
    if (r.ox == 0) r.oy = (r.oy + 1) % kNoiseH;
    return v;
  }
  const uint4 b = philox(r.pixel, r.sample, r.call, 0u, F.seed, kPhiloxKey1);
  r.call += 1;
  return make_float4(u01(b.x), u01(b.y), u01(b.z), u01(b.w));
}

// ----------------------------------------------------------------- palette
struct Mat {
  int type;
  v3 emission;
  v3 albedo;
  float roughness;
};
VT_D float hf(unsigned short h) { return __half2float(__ushort_as_half(h)); }
VT_D Mat empty_mat();
VT_D Mat load_mat(const Frame& F, const JobDev& J, int entry) {
  if (!chk((unsigned)entry < (unsigned)F.n_palette, CHK_PALETTE)) return empty_mat();
  const uint4 q = __ldg(&J.palette[entry]);
  Mat m;
  m.type = (int)hf((unsigned short)(q.x & 0xffffu));
  m.emission = mk3(hf((unsigned short)(q.x >> 16)), hf((unsigned short)(q.y & 0xffffu)),
                   hf((unsigned short)(q.y >> 16)));
  m.albedo = mk3(hf((unsigned short)(q.z & 0xffffu)), hf((unsigned short)(q.z >> 16)),
                 hf((unsigned short)(q.w & 0xffffu)));
  m.roughness = hf((unsigned short)(q.w >> 16));
  return m;
}
VT_D Mat empty_mat() {
  Mat m; m.type = -1; m.emission = mk3(0.f, 0.f, 0.f); m.albedo = mk3(0.f, 0.f, 0.f);
  m.roughness = 0.f; return m;
}
// Material of voxel (x, y, z); the implicit ground below the volume uses the
// configured ground entry (texelFetch outside the texture is undefined in GL).
template <bool kCount>
VT_D Mat voxel_mat(const Frame& F, const JobDev& J, int x, int y, int z, Cnt<kCount>& cnt) {
  cnt.add(C_PALETTE, 1);
  if (y < 0) return load_mat(F, J, F.ground_mat);
  if (!chk((unsigned)x < (unsigned)F.res[0] && (unsigned)y < (unsigned)F.res[1] && (unsigned)z < (unsigned)F.res[2],
           CHK_GRID))
    return empty_mat();
  const uint8_t g = __ldg(&J.grid[(size_t)x + (size_t)F.res[0] * ((size_t)y + (size_t)F.res[1] * (size_t)z)]);
  if (g == 0) return empty_mat();
  return load_mat(F, J, (int)g - 1);
}

// -------------------------------------------------------------------- aabb
// rayAABBIntersection (aabb.h:1-32).
VT_D float ray_aabb(v3 o, v3 d, v3 bmin, v3 bmax) {
  const v3 inv = mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
  const v3 t0 = (bmin - o) * inv;
  const v3 t1 = (bmax - o) * inv;
  const v3 tmin = mk3(vtb::gmin(t0.x, t1.x), vtb::gmin(t0.y, t1.y), vtb::gmin(t0.z, t1.z));
  const float tminf = vtb::gmax(tmin.x, vtb::gmax(tmin.y, tmin.z));
  const v3 tmax = mk3(vtb::gmax(t0.x, t1.x), vtb::gmax(t0.y, t1.y), vtb::gmax(t0.z, t1.z));
  const float tmaxf = vtb::gmin(tmax.x, vtb::gmin(tmax.y, tmax.z));
  if (tmaxf < 0.0f) return -1.0f;
  if (tminf > tmaxf) return -1.0f;
  return vtb::gmax(0.0f, tminf);
}

// ------------------------------------------------------------------ basis
struct Basis { v3 position, tangent, normal, binormal; };

// voxelSpaceToWorldSpace (coordinates.h:59-82).  A hit exactly on a voxel
// corner ties all three axes; the reference's frame is then normalize(0),
// NaN.  With `one_axis` such a tie keeps only the axis along which the ray
// moves fastest (x before y before z on equal speeds).
VT_D Basis voxel_basis(const Frame& F, int x, int y, int z, v3 ro, v3 rd, bool one_axis = false) {
  const v3 vs = ld3(F.vsize);
  const v3 vmin = mk3((float)x, (float)y, (float)z) * vs + ld3(F.bmin);
  const v3 vmax = vmin + vs;
  const float t = ray_aabb(ro, rd, vmin, vmax);
  Basis b;
  b.position = ro + rd * t;
  const v3 center = vmin + vs * 0.5f;
  const v3 c2h = b.position - center;
  const v3 a = vabs3(c2h);
  float mx = (vtb::gstep(a.y, a.x) && vtb::gstep(a.z, a.x)) ? 1.0f : 0.0f;
  float my = (vtb::gstep(a.x, a.y) && vtb::gstep(a.z, a.y)) ? 1.0f : 0.0f;
  float mz = (vtb::gstep(a.x, a.z) && vtb::gstep(a.y, a.z)) ? 1.0f : 0.0f;
  if (one_axis && mx != 0.0f && my != 0.0f && mz != 0.0f) {
    const v3 ad = vabs3(rd);
    const bool kx = ad.x >= ad.y && ad.x >= ad.z;
    const bool ky = !kx && ad.y >= ad.z;
    mx = kx ? 1.0f : 0.0f;
    my = ky ? 1.0f : 0.0f;
    mz = (!kx && !ky) ? 1.0f : 0.0f;
  }
  b.normal = mk3(mx * vtb::gsign(c2h.x), my * vtb::gsign(c2h.y), mz * vtb::gsign(c2h.z));
  const float d3 = 0.57735026919f;
  const v3 tangent = cross(b.normal, mk3(d3, d3, d3));
  b.binormal = normalize(cross(tangent, b.normal));
  b.tangent = normalize(cross(b.binormal, b.normal));
  return b;
}
// localToWorld / worldToLocal (coordinates.h:43-57).
VT_D v3 local_to_world(v3 l, const Basis& b) {
  return (b.tangent * l.x + b.normal * l.y) + b.binormal * l.z;
}
VT_D v3 world_to_local(v3 w, const Basis& b) {
  return mk3(dot(w, b.tangent), dot(w, b.normal), dot(w, b.binormal));
}

// -------------------------------------------------------------------- dda
VT_D Grid grid_of(const Frame& F, const JobDev& J) { return make_grid(F, J.bricks); }

struct Dda {
  int32_t x, y, z;
  float dx, dy, dz;    // distances to the next face crossing (dda.h:34)
  float ax, ay, az;    // sign(d)/d = |1/d| (dda.h:31-32, 52)
  int32_t sx, sy, sz;  // sign(d)
  int32_t steps;
  int32_t state;       // 0 running, 1 hit voxel, 2 left grid / step cap
  int32_t cb;          // brick cached in `bits`
  unsigned long long bits;
};
enum { DDA_RUNNING = 0, DDA_HIT = 1, DDA_MISS = 2 };

// raymarch set-up (dda.h:15-34).  An origin outside the grid ends the
// segment at once with the out-of-grid voxel as position (the reference
// leaves the out parameter unwritten there).
VT_D void dda_begin(const Grid& g, Dda& s, v3 o, v3 d) {
  const v3 bmin = mk3(g.bminx, g.bminy, g.bminz);
  o = o + mk3(vtb::gsign(d.x), vtb::gsign(d.y), vtb::gsign(d.z)) * 0.001f;
  const v3 vo = ((o - bmin) * mk3(g.vextx, g.vexty, g.vextz)) * mk3((float)g.rx, (float)g.ry, (float)g.rz);
  const v3 vp = mk3(floorf(vo.x), floorf(vo.y), floorf(vo.z));
  s.x = (int32_t)vp.x; s.y = (int32_t)vp.y; s.z = (int32_t)vp.z;
  s.steps = 0;
  s.cb = -1;
  s.bits = 0ull;
  if (vp.x < 0.0f || vp.y < 0.0f || vp.z < 0.0f || vp.x >= (float)g.rx || vp.y >= (float)g.ry ||
      vp.z >= (float)g.rz) {
    s.state = DDA_MISS;
    return;
  }
  s.state = DDA_RUNNING;
  d.x = vtb::gstep(fabsf(d.x), 1e-5f) ? 1e-5f : d.x;
  d.y = vtb::gstep(fabsf(d.y), 1e-5f) ? 1e-5f : d.y;
  d.z = vtb::gstep(fabsf(d.z), 1e-5f) ? 1e-5f : d.z;
  const v3 inc = mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
  const v3 sg = mk3(vtb::gsign(d.x), vtb::gsign(d.y), vtb::gsign(d.z));
  const v3 dis = (((vp - vo) + mk3(0.5f, 0.5f, 0.5f)) + sg * 0.5f) * inc;
  s.dx = dis.x; s.dy = dis.y; s.dz = dis.z;
  s.ax = sg.x * inc.x; s.ay = sg.y * inc.y; s.az = sg.z * inc.z;
  s.sx = (int32_t)sg.x; s.sy = (int32_t)sg.y; s.sz = (int32_t)sg.z;
}

// A segment record in the form the DDA set-up uses (dda.h:15-31): the
// origin nudged by 0.001 along the direction's signs and taken to voxel
// space, and the reciprocals of the direction with components of magnitude
// at most 1e-5 raised to +1e-5.  The same operations as dda_begin's.
struct SegRec { v3 vo, inc; };
VT_D SegRec seg_rec(const Frame& F, v3 o, v3 d) {
  SegRec r;
  o = o + mk3(vtb::gsign(d.x), vtb::gsign(d.y), vtb::gsign(d.z)) * 0.001f;
  r.vo = ((o - ld3(F.bmin)) * ld3(F.vext)) * mk3((float)F.res[0], (float)F.res[1], (float)F.res[2]);
  d.x = vtb::gstep(fabsf(d.x), 1e-5f) ? 1e-5f : d.x;
  d.y = vtb::gstep(fabsf(d.y), 1e-5f) ? 1e-5f : d.y;
  d.z = vtb::gstep(fabsf(d.z), 1e-5f) ? 1e-5f : d.z;
  r.inc = mk3(1.0f / d.x, 1.0f / d.y, 1.0f / d.z);
  return r;
}
// dda_begin from a SegRec: the rest of its operations on the same values.
VT_D void dda_begin_rec(const Grid& g, Dda& s, v3 vo, v3 inc) {
  const v3 vp = mk3(floorf(vo.x), floorf(vo.y), floorf(vo.z));
  s.x = (int32_t)vp.x; s.y = (int32_t)vp.y; s.z = (int32_t)vp.z;
  s.steps = 0;
  s.cb = -1;
  s.bits = 0ull;
  if (vp.x < 0.0f || vp.y < 0.0f || vp.z < 0.0f || vp.x >= (float)g.rx || vp.y >= (float)g.ry ||
      vp.z >= (float)g.rz) {
    s.state = DDA_MISS;
    return;
  }
  s.state = DDA_RUNNING;
  const v3 sg = mk3(inc.x > 0.0f ? 1.0f : -1.0f, inc.y > 0.0f ? 1.0f : -1.0f, inc.z > 0.0f ? 1.0f : -1.0f);
  const v3 dis = (((vp - vo) + mk3(0.5f, 0.5f, 0.5f)) + sg * 0.5f) * inc;
  s.dx = dis.x; s.dy = dis.y; s.dz = dis.z;
  s.ax = sg.x * inc.x; s.ay = sg.y * inc.y; s.az = sg.z * inc.z;
  s.sx = (int32_t)sg.x; s.sy = (int32_t)sg.y; s.sz = (int32_t)sg.z;
}

// DDA loop (dda.h:38-57): at most `budget` iterations of
// bounds test -> occupancy test -> advance every minimal axis.
// The brick grid carries a one-brick border whose voxels are all set, so the
// bounds test folds into the occupancy test: a set bit outside [0, res) is
// the exit the reference detects at the top of its loop, with the same
// voxel position.  `bricks` points at brick (0, 0, 0) of the padded array.
// With kVote, the lanes of a warp also stop (still running, resumable) once
// fewer than `vote_min` of them are stepping, checked every fourth step, so
// that the caller can restart the lanes whose segments ended; the state is
// the same as if the segment had been stepped in one call.
// k444: the bricks are known to be 4x4x4 (shifts and masks are immediates);
// otherwise the grid's brick shape is read at run time.
template <bool kCount, bool kVote, bool k444>
VT_D void dda_steps(const Grid& g, Dda& s, int budget, Cnt<kCount>& cnt, int vote_min) {
  const int shx = k444 ? 2 : g.shx, shy = k444 ? 2 : g.shy, shz = k444 ? 2 : g.shz;
  const int shxy = k444 ? 4 : g.shxy, mx_ = k444 ? 3 : g.mx, my_ = k444 ? 3 : g.my, mz_ = k444 ? 3 : g.mz;
  int x = s.x, y = s.y, z = s.z, steps = s.steps, cb = s.cb;
  float dx = s.dx, dy = s.dy, dz = s.dz;
  unsigned long long bits = s.bits;
  int state = DDA_RUNNING;
  const int left = g.max_steps - steps;
  if (budget > left) budget = left;
  int k = 0;
  for (; k < budget; ++k) {
    if (kVote && (k & 3) == 3 && __popc(__activemask()) < vote_min) break;
    const int b = (x >> shx) + g.bx * (y >> shy) + g.bxy * (z >> shz);
    if (b != cb) {
      const long long w = (long long)b + 1 + g.bx + g.bxy;   // index in the padded array
      bits = chk(w >= 0 && w < g.n_words, CHK_BRICK) ? __ldg(&g.bricks[b]) : ~0ull;
      cb = b;
    }
    if ((bits >> brick_bit(x, y, z, shx, shxy, mx_, my_, mz_)) & 1ull) {
      const bool inside = (unsigned)x < (unsigned)g.rx && (unsigned)y < (unsigned)g.ry && (unsigned)z < (unsigned)g.rz;
      if (inside) cnt.add(C_DDA_CELLS, 1);
      state = inside ? DDA_HIT : DDA_MISS;
      break;
    }
    cnt.add(C_DDA_CELLS, 1);
    if (kCount && bits == 0ull) cnt.add(C_EMPTY_CELLS, 1);
    // step(dis.xyz, dis.yxy) * step(dis.xyz, dis.zzx): every axis whose
    // distance equals the minimum (distances are never NaN)
    const float m = fminf(dx, fminf(dy, dz));
    const bool mx = dx == m, my = dy == m, mz = dz == m;
    if (mx) { dx = dx + s.ax; x += s.sx; }
    if (my) { dy = dy + s.ay; y += s.sy; }
    if (mz) { dz = dz + s.az; z += s.sz; }
  }
  steps += k;
  if (state == DDA_RUNNING && steps >= g.max_steps) state = DDA_MISS;   // step cap
  s.x = x; s.y = y; s.z = z; s.steps = steps; s.cb = cb; s.bits = bits;
  s.dx = dx; s.dy = dy; s.dz = dz;
  s.state = state;
}

// The 4x4x4 DDA loop without event counts: the same visits, ends and
// resumable state as dda_steps<false, kVote, true>, in fewer instructions
// per step.  y and z are kept scaled (y * 4, z * 16), so the voxel's bit in
// its brick is two masks of the coordinates; the bit is read from the 32-bit
// half of the brick word that holds it; the budget and the vote are tested
// once every four steps.  It keeps no step count: a segment that starts
// inside the grid leaves it after at most rx + ry + rz steps (each step moves
// at least one axis one voxel in that axis's fixed direction), and
// rx + ry + rz <= sqrt(3) * length(res) < 2 * ceil(length(res)), the cap of
// dda.h:98, so the cap never ends a segment.  budget: a positive multiple of 4.
template <bool kVote>
VT_D void dda_steps_444(const Grid& g, Dda& s, int budget, int vote_min) {
  int x = s.x, y4 = s.y * 4, z16 = s.z * 16, cb = s.cb;
  float dx = s.dx, dy = s.dy, dz = s.dz;
  const float ax = s.ax, ay = s.ay, az = s.az;
  const int sx = s.sx, sy4 = s.sy * 4, sz16 = s.sz * 16;
  uint32_t lo = (uint32_t)s.bits, hi = (uint32_t)(s.bits >> 32);
  int state = DDA_RUNNING;
  for (int k = 0; k < budget; k += 4) {
    if (kVote && k > 0 && __popc(__activemask()) < vote_min) break;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int b = (x >> 2) + g.bx * (y4 >> 4) + g.bxy * (z16 >> 6);
      if (b != cb) {
        const long long w = (long long)b + 1 + g.bx + g.bxy;   // index in the padded array
        const unsigned long long v = chk(w >= 0 && w < g.n_words, CHK_BRICK) ? __ldg(&g.bricks[b]) : ~0ull;
        lo = (uint32_t)v;
        hi = (uint32_t)(v >> 32);
        cb = b;
      }
      // bit x%4 + 4 (y%4) + 16 (z%4); bits 6 and up of n are z / 4, unused
      const uint32_t n = ((uint32_t)x & 3u) | ((uint32_t)y4 & 12u) | ((uint32_t)z16 & ~15u);
      const uint32_t half = (n & 32u) ? hi : lo;
      if (__funnelshift_r(half, half, n) & 1u) {
        const int y = y4 >> 2, z = z16 >> 4;
        const bool inside = (unsigned)x < (unsigned)g.rx && (unsigned)y < (unsigned)g.ry && (unsigned)z < (unsigned)g.rz;
        state = inside ? DDA_HIT : DDA_MISS;
        goto done;
      }
      const float m = fminf(dx, fminf(dy, dz));
      const bool mx = dx == m, my = dy == m, mz = dz == m;
      if (mx) { dx = dx + ax; x += sx; }
      if (my) { dy = dy + ay; y4 += sy4; }
      if (mz) { dz = dz + az; z16 += sz16; }
    }
  }
done:
  s.x = x; s.y = y4 >> 2; s.z = z16 >> 4; s.cb = cb;
  s.bits = ((unsigned long long)hi << 32) | lo;
  s.dx = dx; s.dy = dy; s.dz = dz;
  s.state = state;
}

VT_D bool bricks_444(const Grid& g) { return g.shx == 2 && g.shy == 2 && g.shz == 2; }

// The DDA loop for the grid's brick shape (the 4x4x4 loop when it applies).
template <bool kCount, bool kVote = false>
VT_D void dda_advance(const Grid& g, Dda& s, int budget, Cnt<kCount>& cnt, int vote_min = 0) {
  if (bricks_444(g)) dda_steps<kCount, kVote, true>(g, s, budget, cnt, vote_min);
  else dda_steps<kCount, kVote, false>(g, s, budget, cnt, vote_min);
}

// traverse (dda.h:63-79): voxel hit, or with the ground quirk an exit below y = 0.
VT_D bool seg_hit(uint32_t quirks, int state, int y) {
  if (state == DDA_HIT) return true;
  return (quirks & Q_GROUND) && y < 0;
}
VT_D bool dda_hit(const Frame& F, const Dda& s) { return seg_hit(F.quirks, s.state, s.y); }

// End of one DDA segment as the shading code sees it.
struct SegEnd { int32_t x, y, z, state; };
VT_D SegEnd seg_end(const Dda& s) { SegEnd e; e.x = s.x; e.y = s.y; e.z = s.z; e.state = s.state; return e; }

// A segment end in one 64-bit word for the wavefront's buffers: x and y as
// 21-bit and z as a 20-bit two's-complement field, the DDA state in the top
// two bits.  Volumes are limited so that every position a segment can end
// on (-1 to the extent) fits; a value beyond a field saturates.
VT_D unsigned long long pack_end(int x, int y, int z, int state) {
  x = min(max(x, -(1 << 20)), (1 << 20) - 1);
  y = min(max(y, -(1 << 20)), (1 << 20) - 1);
  z = min(max(z, -(1 << 19)), (1 << 19) - 1);
  return ((unsigned long long)((uint32_t)x & 0x1fffffu)) | ((unsigned long long)((uint32_t)y & 0x1fffffu) << 21) |
         ((unsigned long long)((uint32_t)z & 0xfffffu) << 42) | ((unsigned long long)(uint32_t)state << 62);
}
VT_D SegEnd unpack_end(unsigned long long w) {
  SegEnd e;
  e.x = (int)((long long)(w << 43) >> 43);
  e.y = (int)((long long)(w << 22) >> 43);
  e.z = (int)((long long)(w << 2) >> 44);
  e.state = (int)(w >> 62);
  return e;
}

// --------------------------------------------------------------- sampling
// sampling.h:2-43
VT_D float2 sample_disk(float u0, float u1) {
  const float r = sqrtf(u0);
  const float theta = (2.0f * kPI) * u1;
  return make_float2(r * vtb::vcos(theta), r * vtb::vsin(theta));
}
VT_D float4 cosine_hemisphere(float u0, float u1) {
  const float2 p = sample_disk(u0, u1);
  const float y = sqrtf(vtb::gmax(0.0f, (1.0f - p.x * p.x) - p.y * p.y));
  return make_float4(p.x, y, p.y, y / kPI);
}
VT_D float4 uniform_hemisphere(float u0, float u1) {
  const float y = u0;
  const float r = sqrtf(vtb::gmax(0.0f, 1.0f - y * y));
  const float phi = (u1 * 2.0f) * kPI;
  return make_float4(r * vtb::vcos(phi), y, r * vtb::vsin(phi), 1.0f / (2.0f * kPI));
}
VT_D float power_heuristic(float f, float g) { return (f * f) / ((f * f) + (g * g)); }
VT_D float luminance(v3 c) { return (c.x * 0.2126f + c.y * 0.7152f) + c.z * 0.0722f; }

// ------------------------------------------------------------------- bsdfs
struct FPdf { v3 f; float pdf; };

// microfacet.h:5-15
VT_D float g_term(v3 wo, v3 wi, v3 wh) {
  const float nh = wh.y, no = wo.y, ni = wi.y;
  const float woh = fabsf(dot(wo, wh));
  return vtb::gmin(1.0f, vtb::gmin(((2.0f * nh) * no) / woh, ((2.0f * nh) * ni) / woh));
}
// Fresnel: Schlick with IOR 7.3 (microfacet.h:64-69) or with F0 = reflectance.
VT_D v3 fresnel(const Frame& F, v3 f0, float cos_h) {
  const float p = vtb::vpow(1.0f - cos_h, 5.0f);
  if (F.quirks & Q_FIXED_IOR) {
    const float ior = 7.3f;
    const float sr0 = (1.0f - ior) / (1.0f + ior);
    const float r0 = sr0 * sr0;
    const float fr = r0 + (1.0f - r0) * p;
    return mk3(fr, fr, fr);
  }
  return mk3(f0.x + (1.0f - f0.x) * p, f0.y + (1.0f - f0.y) * p, f0.z + (1.0f - f0.z) * p);
}
// Blinn distribution D and its pdf (microfacet.h:19-37); `color` multiplies f.
VT_D FPdf d_term(v3 color, float e, v3 wo, v3 wh) {
  const float pc = vtb::vpow(wh.y, e);
  const float f = ((e + 2.0f) * kINV_TWOPI) * pc;
  const float wodh = dot(wo, wh);
  FPdf r;
  r.pdf = (wodh <= 0.0f) ? 0.0f : ((e + 1.0f) * pc) / ((kTWO_PI * 4.0f) * wodh);
  r.f = color * f;
  return r;
}
VT_D float blinn_exponent(const Frame& F, float roughness) {
  if (F.quirks & Q_EXPONENT_IS_ROUGHNESS) return roughness;          // metal.h:13-14
  const float r2 = vtb::gmax(roughness * roughness, 1e-6f);
  return vtb::gmax(2.0f / r2 - 2.0f, 0.0f);
}
// evaluateMaterialBSDF (materials.h:7-19 + matte/metal/plastic).
VT_D FPdf eval_bsdf(const Frame& F, const Mat& m, v3 wo, v3 wi) {
  FPdf r;
  if (m.type == 0) {                                                 // lambertian.h:23-29
    r.pdf = wi.y / kPI;
    r.f = m.albedo / kPI;
    return r;
  }
  if (m.type == 1 || m.type == 2) {                                  // microfacet.h:73-91
    const v3 refl = (m.type == 1) ? m.albedo : mk3(1.0f, 1.0f, 1.0f);
    const float e = blinn_exponent(F, m.roughness);
    const float cwi = wi.y, cwo = wo.y;
    const v3 wh = normalize(wi + wo);
    const float ch = dot(wi, wh);
    const bool fixed = (F.quirks & Q_FIXED_IOR) != 0;
    r = d_term(fixed ? refl : mk3(1.0f, 1.0f, 1.0f), e, wo, wh);
    const float g = g_term(wo, wi, wh);
    const v3 fr = fresnel(F, refl, ch);
    const float den = (4.0f * cwo) * cwi;
    r.f = mk3(r.f.x * ((g * fr.x) / den), r.f.y * ((g * fr.y) / den), r.f.z * ((g * fr.z) / den));
    return r;
  }
  r.f = mk3(0.f, 0.f, 0.f); r.pdf = 0.0f;
  return r;
}
// sampleMaterialBSDF (materials.h:30-43): consumes one rand() block; returns
// the local direction, f and pdf, and the block's z for Russian roulette.
template <bool kCount>
VT_D v3 sample_bsdf(const Frame& F, const JobDev& J, const Mat& m, v3 wo, Rng& rng, FPdf& out, float& u_rr) {
  const float4 u = rng_next(F, J, rng);
  u_rr = u.z;
  if (m.type == 0) {                                                 // lambertian.h:10-19
    const float4 s = cosine_hemisphere(u.x, u.y);
    out.f = m.albedo / kPI;
    out.pdf = s.w;
    return mk3(s.x, s.y, s.z);
  }
  // microfacet.h:41-61 and 102-123
  const v3 refl = (m.type == 1) ? m.albedo : mk3(1.0f, 1.0f, 1.0f);
  const float e = blinn_exponent(F, m.roughness);
  const float ct = vtb::vpow(u.x, 1.0f / (e + 1.0f));
  const float st = sqrtf(vtb::gmax(0.0f, 1.0f - ct * ct));
  const float phi = (u.y * 2.0f) * kPI;
  const v3 wh = mk3(st * vtb::vcos(phi), ct, st * vtb::vsin(phi));
  const v3 wi = (-wo) + (2.0f * dot(wo, wh)) * wh;
  const bool fixed = (F.quirks & Q_FIXED_IOR) != 0;
  FPdf d = d_term(fixed ? refl : mk3(1.0f, 1.0f, 1.0f), e, wo, wh);
  const float cwi = wi.y, cwo = wo.y;
  const v3 wh2 = normalize(wi + wo);
  const float ch = dot(wi, wh2);
  const float g = g_term(wo, wi, wh2);
  const v3 fr = fresnel(F, refl, ch);
  const float den = (4.0f * cwo) * cwi;
  v3 f = d.f;
  if (F.quirks & Q_DOUBLE_REFLECTANCE) f = refl * f;
  out.f = mk3(((f.x * g) * fr.x) / den, ((f.y * g) * fr.y) / den, ((f.z * g) * fr.z) / den);
  out.pdf = d.pdf;
  return wi;
}

// --------------------------------------------------------------- env light
// uvCoordFromVector / directionFromUVCoord (coordinates.h:97-116).
VT_D float2 uv_from_dir(v3 v, float rot) {
  const float theta = vtb::vacos(v.y);
  const float phi = (vtb::vatan2(v.z, v.x) + kPI) + rot;
  const float x = phi / kTWO_PI;
  const float u = x - 1.0f * floorf(x / 1.0f);
  return make_float2(u, theta / kPI);
}
VT_D v3 dir_from_uv(float u, float v, float rot) {
  const float phi = ((u * kTWO_PI) - kPI) - rot;
  const float theta = v * kPI;
  const float st = vtb::vsin(theta);
  return mk3(st * vtb::vcos(phi), vtb::vcos(theta), st * vtb::vsin(phi));
}
VT_D v3 texel(const JobDev& J, int w, int h, int i, int j) {
  if (!chk((unsigned)i < (unsigned)w && (unsigned)j < (unsigned)h, CHK_TEXEL)) return mk3(0.f, 0.f, 0.f);
  const uint2 q = __ldg(&J.env_texels[(size_t)j * w + i]);
  return mk3(hf((unsigned short)(q.x & 0xffffu)), hf((unsigned short)(q.x >> 16)),
             hf((unsigned short)(q.y & 0xffffu)));
}
// texture(backgroundTexture, uv) with GL_LINEAR filtering and clamp to edge.
template <bool kCount>
VT_D v3 env_lookup(const Frame& F, const JobDev& J, float u, float v, Cnt<kCount>& cnt) {
  cnt.add(C_ENV_EVALS, 1);
  const int w = F.env_w, h = F.env_h;
  const float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
  const float x0 = floorf(x), y0 = floorf(y);
  const float fx = x - x0, fy = y - y0;
  int i0 = (int)x0, j0 = (int)y0;
  int i1 = i0 + 1, j1 = j0 + 1;
  i0 = min(max(i0, 0), w - 1); i1 = min(max(i1, 0), w - 1);
  j0 = min(max(j0, 0), h - 1); j1 = min(max(j1, 0), h - 1);
  const v3 t00 = texel(J, w, h, i0, j0), t10 = texel(J, w, h, i1, j0);
  const v3 t01 = texel(J, w, h, i0, j1), t11 = texel(J, w, h, i1, j1);
  const float gx = 1.0f - fx, gy = 1.0f - fy;
  const v3 a = t00 * gx + t10 * fx;
  const v3 b = t01 * gx + t11 * fx;
  return a * gy + b * fy;
}
// getBackgroundColor (lights.h:4-17).
template <bool kCount>
VT_D v3 background(const Frame& F, const JobDev& J, v3 d, Cnt<kCount>& cnt) {
  if (F.use_image) {
    const float2 uv = uv_from_dir(d, F.bg_rot);
    return env_lookup(F, J, uv.x, uv.y, cnt);
  }
  const float bias = vtb::gmax(0.0f, d.y);
  return ld3(F.bg_bottom) * (1.0f - bias) + ld3(F.bg_top) * bias;
}
// evaluateEnvironmentRadiance (lights.h:20-33).
template <bool kCount>
VT_D v3 eval_env(const Frame& F, const JobDev& J, v3 d, float& pdf, Cnt<kCount>& cnt) {
  const v3 L = background(F, J, d, cnt);
  if (F.use_image) pdf = luminance(L) / F.env_integral;
  else pdf = (F.quirks & Q_GRADIENT_PDF_MISMATCH) ? 1.0f / (4.0f * kPI) : 1.0f / (2.0f * kPI);
  return L;
}
// binarySearchCDFV / binarySearchCDFU (envMapSample.h:70-123).
template <bool kCount>
VT_D int search_cdf(const float* cdf, int high, float u, Cnt<kCount>& cnt) {
  int low = 0;
  while (low != high - 1) {
    const int mid = (low + high) / 2;
    cnt.add(C_CDF_PROBES, 1);
    if (u < __ldg(&cdf[mid])) high = mid; else low = mid;
  }
  return low;
}
// sampleEnvironmentRadiance (lights.h:36-55, envMapSample.h:23-65).
template <bool kCount>
VT_D v3 sample_env(const Frame& F, const JobDev& J, const Basis& b, float u0, float u1,
                   v3& dir, float& pdf, Cnt<kCount>& cnt) {
  if (F.use_image) {
    const int su = F.env_cdf_w + 1, sv = F.env_cdf_h + 1;
    const int row = search_cdf(J.cdf_v, sv - 1, u1, cnt);
    const float* cu = J.cdf_u + (size_t)row * su;
    const int col = search_cdf(cu, su - 1, u0, cnt);
    if (!chk(row >= 0 && row + 1 < sv && col >= 0 && col + 1 < su, CHK_CDF)) {
      dir = mk3(0.f, 1.f, 0.f);
      pdf = 0.0f;
      return mk3(0.f, 0.f, 0.f);
    }
    cnt.add(C_CDF_PROBES, 4);
    const float lu = __ldg(&cu[col]), hu = __ldg(&cu[col + 1]);
    const float du = (u0 - lu) / (hu - lu);
    const float lv = __ldg(&J.cdf_v[row]), hv = __ldg(&J.cdf_v[row + 1]);
    const float dv = (u1 - lv) / (hv - lv);
    const float u = ((float)col + du) / (float)(su - 1);
    const float v = ((float)row + dv) / (float)(sv - 1);
    dir = dir_from_uv(u, v, F.bg_rot);
    const v3 L = env_lookup(F, J, u, v, cnt);
    pdf = luminance(L) / F.env_integral;
    return L;
  }
  const float4 s = uniform_hemisphere(u0, u1);
  dir = local_to_world(mk3(s.x, s.y, s.z), b);
  pdf = s.w;
  return background(F, J, dir, cnt);
}

// ------------------------------------------------------------------ camera
// screenToEyeSpacePerspective / Orthographic (coordinates.h:1-27) with
// gl_DepthRange = [0, 1].
// kAtFragZ: w.z is the frame's frag_z, whose depth terms the frame holds.
template <bool kAtFragZ = false>
VT_D float4 screen_to_eye_persp(const Frame& F, v3 w) {
  v3 ndc;
  ndc.x = ((2.0f * w.x) - (2.0f * F.viewport[0])) / F.viewport[2] - 1.0f;
  ndc.y = ((2.0f * w.y) - (2.0f * F.viewport[1])) / F.viewport[3] - 1.0f;
  float cw;
  if (kAtFragZ) {
    ndc.z = F.persp_ndc_z;
    cw = F.persp_cw;
  } else {
    ndc.z = ((2.0f * w.z - 0.0f) - 1.0f) / (1.0f - 0.0f);
    cw = F.proj[11] / (ndc.z - (F.proj[10] / F.proj[14]));
  }
  return mul4(F.inv_proj, make_float4(ndc.x * cw, ndc.y * cw, ndc.z * cw, cw));
}
VT_D float4 screen_to_eye_ortho(const Frame& F, v3 w) {
  v3 ndc;
  ndc.x = (w.x / F.viewport[2]) * 2.0f - 1.0f;
  ndc.y = (w.y / F.viewport[3]) * 2.0f - 1.0f;
  ndc.z = ((2.0f * w.z - 0.0f) - 1.0f) / (1.0f - 0.0f);
  return mul4(F.inv_proj, make_float4(ndc.x, ndc.y, ndc.z, 1.0f));
}
VT_D v3 xyz(float4 v) { return mk3(v.x, v.y, v.z); }

// generateRay (generateRay.h:1-123).  frag = gl_FragCoord.xyz; kAtFragZ:
// frag.z is the frame's frag_z (the camera rays of a pass).
template <bool kAtFragZ = false>
VT_D void generate_ray(const Frame& F, const JobDev& J, v3 frag, Rng& rng, v3& o, v3& d) {
  const float* M = F.inv_mv;
  if (F.lens_model == 0) {                                         // pinhole :10-26
    const float4 u = rng_next(F, J, rng);
    const v3 jit = mk3(u.x - 0.5f, u.y - 0.5f, 0.0f);
    const float4 es = screen_to_eye_persp<kAtFragZ>(F, frag + jit);
    o = xyz(mul4(M, make_float4(0.0f, 0.0f, 0.0f, 1.0f)));
    const v3 n = normalize(mk3(es.x, es.y, es.z));
    const float4 w = mul4(M, make_float4(n.x, n.y, n.z, 0.0f));
    const float l = sqrtf(((w.x * w.x + w.y * w.y) + w.z * w.z) + w.w * w.w);
    d = mk3(w.x / l, w.y / l, w.z / l);
  } else if (F.lens_model == 1) {                                  // thin lens :30-101
    const float4 u = rng_next(F, J, rng);
    const float2 disk = sample_disk(u.x, u.y);
    const v3 lens = mk3(disk.x * F.lens_radius, disk.y * F.lens_radius, 0.0f);
    v3 fp = frag;
    if (!(F.quirks & Q_THINLENS_NO_JITTER)) fp = frag + mk3(u.z - 0.5f, u.w - 0.5f, 0.0f);
    const v3 eo = xyz(screen_to_eye_persp<kAtFragZ>(F, fp));
    const v3 ed = normalize(eo);
    const float t = F.focal_distance / -(ed.z);
    const v3 ef = eo + ed * t;
    const v3 wf = xyz(mul4(M, make_float4(ef.x, ef.y, ef.z, 1.0f)));
    o = xyz(mul4(M, make_float4(lens.x, lens.y, lens.z, 1.0f)));
    d = normalize(wf - o);
  } else {                                                         // orthographic :1-7
    o = xyz(mul4(M, screen_to_eye_ortho(F, frag)));
    d = xyz(mul4(M, make_float4(0.0f, 0.0f, -1.0f, 0.0f)));
  }
}

// ------------------------------------------------------------ path state
// A path alternates between DDA segments and shading events:
//   path_start   raygen and volume clip; leaves an extension segment (the
//                primary ray, traced from the volume entry point) or ends
//   ext_end      end of an extension segment: miss -> environment, hit ->
//                shade the vertex, which leaves a shadow segment (ro, sd)
//                and, unless the path ends there, a continuation (ro, rd)
//   shadow_end   end of a shadow segment: add the light sample if visible
// The megakernel runs these one segment at a time; the wavefront traces the
// shadow and continuation segments of a vertex in the same round and runs
// shadow_end before ext_end, which performs the same operations in the same
// order as the reference loop.
struct Path {
  Rng rng;
  v3 L;          // radiance
  v3 T;          // throughput
  v3 ro;         // origin of the current extension ray (camera or last vertex)
  v3 rd;         // direction of the current extension ray
  v3 sd;         // direction of the pending shadow ray (origin ro)
  v3 nee_P;      // throughput * directLighting value, added if the light is visible
  int32_t nee_nf;// bit c set: throughput component c was not finite (then an
                 // occluded light sample still turns L.c into NaN, as T * 0 does)
  int32_t light; // emissive voxel index of the light sample, -1 = environment
  float bsdf_pdf;
  int32_t bounces;
  int32_t primary;
  int32_t has_cont;
};

// Per-sample output: pow(L*exposure, 1/gamma) when the gamma quirk is on
// (pathTracer.fs:294-295), linear radiance otherwise; alpha = 1.
VT_D float4 path_output(const Frame& F, const Path& p) {
  if (F.quirks & Q_GAMMA_BEFORE_AVERAGE) {
    return make_float4(vtb::vpow(p.L.x * F.exposure, F.inv_gamma), vtb::vpow(p.L.y * F.exposure, F.inv_gamma),
                       vtb::vpow(p.L.z * F.exposure, F.inv_gamma), 1.0f);
  }
  return make_float4(p.L.x, p.L.y, p.L.z, 1.0f);
}

// main() up to the primary traversal (pathTracer.fs:172-196).  Returns true
// if the primary ray enters the volume; its segment then starts at
// ro + t_enter*rd with t_enter = ray_aabb(ro, rd, bounds).
template <bool kCount>
VT_D bool path_start(const Frame& F, const JobDev& J, Path& p, int px, int py, int sample, Cnt<kCount>& cnt,
                     float& t_enter) {
  rng_init(F, p.rng, px, py, sample);
  cnt.add(C_PATHS, 1);
  p.L = mk3(0.0f, 0.0f, 0.0f);
  p.T = mk3(1.0f, 1.0f, 1.0f);
  p.bounces = 0;
  p.primary = 1;
  p.has_cont = 0;
  p.light = -1;
  p.bsdf_pdf = 0.0f;
  p.nee_P = mk3(0.0f, 0.0f, 0.0f);
  p.nee_nf = 0;
  v3 o, d;
  generate_ray<true>(F, J, mk3((float)px + 0.5f, (float)py + 0.5f, F.frag_z), p.rng, o, d);
  p.ro = o;
  p.rd = d;
  p.sd = d;
  const float t = ray_aabb(o, d, ld3(F.bmin), ld3(F.bmax));
  t_enter = t;
  if (t < 0.0f) {
    p.L = background(F, J, d, cnt);
    return false;
  }
  cnt.add(C_SEGMENTS, 1);
  return true;
}

// directLighting (pathTracer.fs:64-170) up to the shadow ray: picks a light,
// evaluates the BSDF and MIS weight for it and leaves the shadow direction in
// p.sd.  The BSDF evaluation does not depend on visibility, so it is done
// before the shadow ray; the contribution is added only if the segment
// confirms visibility (shadow_end).
template <bool kCount>
VT_D void light_sample(const Frame& F, const JobDev& J, Path& p, const Basis& b, const Mat& m, v3 wo,
                       Cnt<kCount>& cnt) {
  const float4 u = rng_next(F, J, p.rng);
  const int num_lights = F.n_emissive + 1;
  const int li = (int)(u.x * (float)num_lights);
  v3 dir, Ll;
  float pdf;
  if (li < num_lights - 1) {
    cnt.add(C_EMISSIVE_READS, 1);
    const int idx0 = __ldg(&J.emissive[li]);
    const bool idx_ok = chk(idx0 >= 0 && (long long)idx0 < (long long)F.res[0] * F.res[1] * F.res[2], CHK_EMISSIVE);
    const int idx = idx_ok ? idx0 : 0;
    const int dz = F.res[0] * F.res[1], dy = F.res[0];
    const int ez = (int)udiv((uint32_t)idx, F.m_res01);
    const int r1 = idx - ez * dz;
    const int ey = (int)udiv((uint32_t)r1, F.m_res0);
    const int ex = r1 - ey * dy;
    const Mat lm = voxel_mat(F, J, ex, ey, ez, cnt);
    Ll = mk3(F.nee_scale, F.nee_scale, F.nee_scale) * lm.emission;
    const v3 res = mk3((float)F.res[0], (float)F.res[1], (float)F.res[2]);
    v3 wp = (mk3((float)ex, (float)ey, (float)ez) / res) * (ld3(F.bmax) - ld3(F.bmin)) + ld3(F.bmin);
    wp = wp + mk3(u.y, u.z, u.w) * ld3(F.vsize);
    const v3 to_light = wp - b.position;
    const float r = length(to_light);
    dir = to_light / r;
    const Basis lb = voxel_basis(F, ex, ey, ez, b.position, dir);
    const float area = (6.0f * F.vsize[0]) * F.vsize[1];
    const float jac = (r * r) / fabsf(dot(-dir, lb.normal));
    pdf = jac / area;
    p.light = idx;
  } else {
    Ll = sample_env(F, J, b, u.y, u.z, dir, pdf, cnt);
    p.light = -1;
  }
  pdf = pdf / (float)num_lights;
  const v3 lwo = world_to_local(wo, b);
  const v3 lwi = world_to_local(dir, b);
  const FPdf bf = eval_bsdf(F, m, lwo, lwi);
  const float mis = power_heuristic(pdf, bf.pdf);
  v3 C = (((bf.f * Ll) * fabsf(dot(dir, b.normal))) * mis) / pdf;
  // Without the unguarded-samples quirk a light sample with a zero, negative
  // or infinite pdf contributes nothing instead of dividing by it.
  if (!(F.quirks & Q_UNGUARDED) && !(pdf > 0.0f && pdf < __int_as_float(0x7f800000)))
    C = mk3(0.0f, 0.0f, 0.0f);
  p.nee_P = p.T * C;
  const float inf = __int_as_float(0x7f800000);
  p.nee_nf = (fabsf(p.T.x) < inf ? 0 : 1) | (fabsf(p.T.y) < inf ? 0 : 2) | (fabsf(p.T.z) < inf ? 0 : 4);
  p.sd = dir;
  cnt.add(C_SEGMENTS, 1);
}

// End of a shadow segment (pathTracer.fs:133-153, 248-251).
VT_D void shadow_end(const Frame& F, Path& p, SegEnd e) {
  const bool hit = seg_hit(F.quirks, e.state, e.y);
  bool visible;
  if (p.light >= 0) {
    const int dz = F.res[0] * F.res[1], dy = F.res[0];
    const int ez = (int)udiv((uint32_t)p.light, F.m_res01);
    const int r1 = p.light - ez * dz;
    const int ey = (int)udiv((uint32_t)r1, F.m_res0);
    const int ex = r1 - ey * dy;
    visible = hit && e.x == ex && e.y == ey && e.z == ez;
  } else {
    visible = !hit;
  }
  // radiance += throughput * directLighting: the product was formed at the
  // vertex; an occluded sample adds T * 0, which changes L only where T is
  // not finite (L is never -0, so adding +-0 is exact otherwise)
  if (visible) {
    p.L = p.L + p.nee_P;
  } else if (p.nee_nf) {
    const float nan = __int_as_float(0x7fffffff);
    if (p.nee_nf & 1) p.L.x = p.L.x + nan;
    if (p.nee_nf & 2) p.L.y = p.L.y + nan;
    if (p.nee_nf & 4) p.L.z = p.L.z + nan;
  }
}

// End of an extension segment, first part of the body of the bounce loop
// (pathTracer.fs:202-233): a miss adds the environment, and the bounce
// limit and the selected voxel end the path.  Returns true when the hit is
// shaded (ext_hit).
template <bool kCount>
VT_D bool ext_resolve(const Frame& F, const JobDev& J, Path& p, SegEnd e, Cnt<kCount>& cnt) {
  const bool hit = seg_hit(F.quirks, e.state, e.y);
  if (!hit) {
    if (p.primary) {
      p.L = background(F, J, p.rd, cnt);                          // :202-208
    } else {
      float lpdf;
      const v3 Le = eval_env(F, J, p.rd, lpdf, cnt);              // :282-289
      const float mis = power_heuristic(p.bsdf_pdf, lpdf);
      p.L = p.L + (p.T * Le) * mis;
    }
    return false;
  }
  if (!p.primary) p.bounces += 1;                                 // :291
  if (p.bounces >= F.max_bounces) return false;                   // :214
  if (F.sel_enabled && e.x == F.sel[0] && e.y == F.sel[1] && e.z == F.sel[2]) {
    cnt.add(C_PALETTE, 1);                                        // the material fetch of :225-226
    p.L = p.L + mk3(1.0f, 0.0f, 0.0f);                            // :228-233
    return false;
  }
  return true;
}

// Wireframe factor of a hit (pathTracer.fs:260-270, editMode.fs:113-124):
// 1 inside the face, 1 - opacity within `thickness` of a voxel edge.
VT_D float wire_factor(const Frame& F, const Basis& b, int x, int y, int z) {
  const v3 res = mk3((float)F.res[0], (float)F.res[1], (float)F.res[2]);
  const v3 vc = ((b.position - ld3(F.bmin)) / (ld3(F.bmax) - ld3(F.bmin))) * res;
  const v3 uvw = mk3((float)x, (float)y, (float)z) - vc;
  const v3 nyzx = mk3(b.normal.y, b.normal.z, b.normal.x);
  const v3 nzxy = mk3(b.normal.z, b.normal.x, b.normal.y);
  const float ux = fabsf(dot(nyzx, uvw)), uy = fabsf(dot(nzxy, uvw));
  const float th = F.wire_thickness;
  float wire = (vtb::gstep(th, ux) ? 1.0f : 0.0f) * (vtb::gstep(ux, 1.0f - th) ? 1.0f : 0.0f);
  wire = wire * (vtb::gstep(th, uy) ? 1.0f : 0.0f);
  wire = wire * (vtb::gstep(uy, 1.0f - th) ? 1.0f : 0.0f);
  return (1.0f - F.wire_opacity) + F.wire_opacity * wire;
}

// Second part (pathTracer.fs:220-279): shade a hit that ext_resolve kept.
// Leaves a shadow segment (ro, sd) and, if p.has_cont, a continuation
// segment (ro, rd).
template <bool kCount>
VT_D void ext_hit(const Frame& F, const JobDev& J, Path& p, SegEnd e, Cnt<kCount>& cnt) {
  const Basis b = voxel_basis(F, e.x, e.y, e.z, p.ro, p.rd, !(F.quirks & Q_UNGUARDED));   // :220-223
  const Mat m = voxel_mat(F, J, e.x, e.y, e.z, cnt);              // :225-226
  const v3 wo = -p.rd;
  const v3 lwo = world_to_local(wo, b);
  if (p.bounces == 0) p.L = p.L + p.T * m.emission;               // :241-245
  light_sample(F, J, p, b, m, wo, cnt);                           // :248-251
  FPdf bs;
  float u_rr;
  v3 lwi = sample_bsdf<kCount>(F, J, m, lwo, p.rng, bs, u_rr);    // :254-258
  if (F.wire_opacity > 0.0f) {                                    // :260-270
    const float wire = wire_factor(F, b, e.x, e.y, e.z);
    bs.f = bs.f * mk3(wire, wire, wire);
  }
  const v3 wwi = local_to_world(lwi, b);                          // :273
  const bool guard = !(F.quirks & Q_UNGUARDED);
  p.has_cont = 1;
  // Without the unguarded-samples quirk a BSDF sample with zero pdf or below
  // the surface ends the path (the reference divides by the pdf regardless).
  if (guard && (!(bs.pdf > 0.0f) || !(lwi.y > 0.0f))) p.has_cont = 0;
  if (p.has_cont) {
    p.T = p.T * ((bs.f * fabsf(dot(wwi, b.normal))) / bs.pdf);    // :276
    if (guard && !(finite3(p.T))) p.has_cont = 0;
  }
  if (p.has_cont && F.rr_start >= 0 && p.bounces >= F.rr_start) {  // Russian roulette
    const float q = vtb::gmin(1.0f, vtb::gmax(p.T.x, vtb::gmax(p.T.y, p.T.z)));
    if (!(u_rr < q)) p.has_cont = 0;
    else p.T = p.T / q;
  }
  if (p.has_cont) cnt.add(C_SEGMENTS, 1);
  p.ro = b.position;                                              // :278-279
  p.rd = wwi;
  p.bsdf_pdf = bs.pdf;
  p.primary = 0;
}

// The whole bounce-loop body: false when the path ends here.
template <bool kCount>
VT_D bool ext_end(const Frame& F, const JobDev& J, Path& p, SegEnd e, Cnt<kCount>& cnt) {
  if (!ext_resolve(F, J, p, e, cnt)) return false;
  ext_hit(F, J, p, e, cnt);
  return true;
}

// Material class of a hit for grouping hits before ext_hit: 0 Lambert,
// 1 anything else (the microfacet path).  No counter: ext_hit counts the
// material fetch.
VT_D int hit_class(const Frame& F, const JobDev& J, SegEnd e) {
  if (e.y < 0) return load_mat(F, J, F.ground_mat).type == 0 ? 0 : 1;
  if (!chk((unsigned)e.x < (unsigned)F.res[0] && (unsigned)e.y < (unsigned)F.res[1] &&
               (unsigned)e.z < (unsigned)F.res[2], CHK_GRID))
    return 1;
  const uint8_t g = __ldg(&J.grid[(size_t)e.x + (size_t)F.res[0] * ((size_t)e.y + (size_t)F.res[1] * (size_t)e.z)]);
  if (g == 0) return 1;
  return load_mat(F, J, (int)g - 1).type == 0 ? 0 : 1;
}

// One complete sample, run to the end by a single lane (megakernel form).
// The edit-mode integrator (editMode.fs:58-144): white voxels lit by
// sqrt(max(0, -d.n)), halved (ambientLight 0.5) when a shadow ray towards
// the fixed light direction (1, -1, -1) is blocked, the selected voxel red,
// the wireframe overlay; the background where the ray misses.  The reference
// uploads its light direction to a uniform the shader does not declare
// (renderer.cpp:279-280 sets "wsLightDir"), so the shader's initialiser is
// the direction in effect.  No gamma: the shader writes linear values.
template <bool kCount>
VT_D float4 edit_sample(const Frame& F, const JobDev& J, int px, int py, int sample, Cnt<kCount>& cnt,
                        HitRecord* first_hit) {
  const Grid g = grid_of(F, J);
  Path p;
  Dda s;
  if (first_hit) { first_hit->x = -1; first_hit->y = -1; first_hit->z = -1; first_hit->flags = 0; }
  float t_enter;
  if (!path_start(F, J, p, px, py, sample, cnt, t_enter)) return make_float4(p.L.x, p.L.y, p.L.z, 1.0f);
  dda_begin(g, s, p.ro + t_enter * p.rd, p.rd);
  if (s.state == DDA_RUNNING) dda_advance(g, s, 0x7fffffff, cnt);
  const bool hit = dda_hit(F, s);
  Basis b;
  if (hit) b = voxel_basis(F, s.x, s.y, s.z, p.ro, p.rd, !(F.quirks & Q_UNGUARDED));
  if (first_hit) {
    first_hit->x = s.x; first_hit->y = s.y; first_hit->z = s.z;
    int flags = (hit ? 1 : 0) << 8 | ((hit && s.state != DDA_HIT) ? 1 : 0) << 9;
    if (hit) {
      const Basis fb = voxel_basis(F, s.x, s.y, s.z, p.ro, p.rd);
      flags |= ((int)fb.normal.x + 1) | (((int)fb.normal.y + 1) << 2) | (((int)fb.normal.z + 1) << 4);
    }
    first_hit->flags = flags;
  }
  if (!hit) {                                                     // :88-92
    const v3 bg = background(F, J, p.rd, cnt);
    return make_float4(bg.x, bg.y, bg.z, 1.0f);
  }
  if (F.sel_enabled && s.x == F.sel[0] && s.y == F.sel[1] && s.z == F.sel[2])
    return make_float4(1.0f, 0.0f, 0.0f, 1.0f);                   // :107-112
  v3 albedo = mk3(1.0f, 1.0f, 1.0f);
  if (F.wire_opacity > 0.0f) {                                    // :114-125
    const float wire = wire_factor(F, b, s.x, s.y, s.z);
    albedo = albedo * mk3(wire, wire, wire);
  }
  float lighting = vtb::gmax(0.0f, dot(-p.rd, b.normal));         // :129-130
  lighting = sqrtf(lighting);
  cnt.add(C_SEGMENTS, 1);
  dda_begin(g, s, b.position, mk3(-1.0f, 1.0f, 1.0f));            // :133: -lightDirection
  if (s.state == DDA_RUNNING) dda_advance(g, s, 0x7fffffff, cnt);
  if (dda_hit(F, s)) lighting = lighting * 0.5f;
  const v3 radiance = albedo * lighting;
  return make_float4(radiance.x, radiance.y, radiance.z, 1.0f);
}

template <bool kCount>
VT_D float4 trace_sample(const Frame& F, const JobDev& J, int px, int py, int sample, Cnt<kCount>& cnt,
                         HitRecord* first_hit) {
  if (F.integrator == 1) return edit_sample(F, J, px, py, sample, cnt, first_hit);
  const Grid g = grid_of(F, J);
  Path p;
  Dda s;
  if (first_hit) { first_hit->x = -1; first_hit->y = -1; first_hit->z = -1; first_hit->flags = 0; }
  float t_enter;
  if (!path_start(F, J, p, px, py, sample, cnt, t_enter)) return path_output(F, p);
  dda_begin(g, s, p.ro + t_enter * p.rd, p.rd);
  if (s.state == DDA_RUNNING) dda_advance(g, s, 0x7fffffff, cnt);
  if (first_hit) {
    const bool h = dda_hit(F, s);
    first_hit->x = s.x; first_hit->y = s.y; first_hit->z = s.z;
    int flags = (h ? 1 : 0) << 8 | ((h && s.state != DDA_HIT) ? 1 : 0) << 9;
    if (h) {
      const Basis b = voxel_basis(F, s.x, s.y, s.z, p.ro, p.rd);
      flags |= ((int)b.normal.x + 1) | (((int)b.normal.y + 1) << 2) | (((int)b.normal.z + 1) << 4);
    }
    first_hit->flags = flags;
  }
  while (ext_end(F, J, p, seg_end(s), cnt)) {
    dda_begin(g, s, p.ro, p.sd);
    if (s.state == DDA_RUNNING) dda_advance(g, s, 0x7fffffff, cnt);
    shadow_end(F, p, seg_end(s));
    if (!p.has_cont) break;
    dda_begin(g, s, p.ro, p.rd);
    if (s.state == DDA_RUNNING) dda_advance(g, s, 0x7fffffff, cnt);
  }
  return path_output(F, p);
}

// Kahan-compensated accumulation of one sample into a pixel.
VT_D void kahan_add(float4& sum, float4& comp, float4 v) {
  float y, t;
  y = v.x - comp.x; t = sum.x + y; comp.x = (t - sum.x) - y; sum.x = t;
  y = v.y - comp.y; t = sum.y + y; comp.y = (t - sum.y) - y; sum.y = t;
  y = v.z - comp.z; t = sum.z + y; comp.z = (t - sum.z) - y; sum.z = t;
  y = v.w - comp.w; t = sum.w + y; comp.w = (t - sum.w) - y; sum.w = t;
}

}  // namespace vt
