// vt_oracle.cpp — CPU restatement of the reference's path-tracing pass,
// environment CDF build, mesh voxelizer, emissive pruning and camera math.
//
// TEST INFRASTRUCTURE ONLY: used by tests/, the smoke check and the CPU
// baseline of the benchmark as the checker; never linked into the product.
// Parity status: see vt_oracle.h (pinned only by the reference's documented
// known-answer examples and analytic known answers).
//
// The integrators below are written as straight-line code following
// src/shaders/integrator/pathTracer.fs:172-296 and editMode.fs:58-144 (not
// as the GPU's state machine), so that a mismatch in the GPU's
// restructuring shows up.
#include "vt_oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "../voxeltoy_gb300/csrc/vt_builtins.h"

namespace {

// ------------------------------------------------------------------ types
template <class R> struct V3 { R x, y, z; };
template <class R> V3<R> v3(R x, R y, R z) { V3<R> r; r.x = x; r.y = y; r.z = z; return r; }
template <class R> V3<R> operator+(V3<R> a, V3<R> b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> V3<R> operator-(V3<R> a, V3<R> b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> V3<R> operator*(V3<R> a, V3<R> b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
template <class R> V3<R> operator/(V3<R> a, V3<R> b) { return v3(a.x / b.x, a.y / b.y, a.z / b.z); }
template <class R> V3<R> operator*(V3<R> a, R s) { return v3(a.x * s, a.y * s, a.z * s); }
template <class R> V3<R> operator*(R s, V3<R> a) { return v3(s * a.x, s * a.y, s * a.z); }
template <class R> V3<R> operator/(V3<R> a, R s) { return v3(a.x / s, a.y / s, a.z / s); }
template <class R> V3<R> operator-(V3<R> a) { return v3(-a.x, -a.y, -a.z); }
// GLSL dot/cross/length/normalize (GLSL 4.30 section 8.5)
template <class R> R dot(V3<R> a, V3<R> b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
template <class R> V3<R> cross(V3<R> a, V3<R> b) {
  return v3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}

template <class R> struct M;
template <> struct M<float> {
  static float sin(float x) { return vtb::vsin(x); }
  static float cos(float x) { return vtb::vcos(x); }
  static float pow(float x, float y) { return vtb::vpow(x, y); }
  static float acos(float x) { return vtb::vacos(x); }
  static float atan2(float y, float x) { return vtb::vatan2(y, x); }
  static float sqrt(float x) { return std::sqrt(x); }
  static float floor(float x) { return std::floor(x); }
  static float abs(float x) { return std::fabs(x); }
  static constexpr float PI = 3.14159265359f, TWO_PI = 6.28318530718f, INV_TWOPI = 0.15915494309f;
};
template <> struct M<double> {
  static double sin(double x) { return std::sin(x); }
  static double cos(double x) { return std::cos(x); }
  static double pow(double x, double y) {
    if (y == 0.0) return 1.0;
    if (!(x > 0.0)) return 0.0;
    return std::pow(x, y);
  }
  static double acos(double x) { return std::acos(x < -1.0 ? -1.0 : (x > 1.0 ? 1.0 : x)); }
  static double atan2(double y, double x) { return (x == 0.0 && y == 0.0) ? 0.0 : std::atan2(y, x); }
  static double sqrt(double x) { return std::sqrt(x); }
  static double floor(double x) { return std::floor(x); }
  static double abs(double x) { return std::fabs(x); }
  static constexpr double PI = 3.14159265359, TWO_PI = 6.28318530718, INV_TWOPI = 0.15915494309;
};

template <class R> R glmin(R x, R y) { return y < x ? y : x; }    // GLSL min
template <class R> R glmax(R x, R y) { return x < y ? y : x; }    // GLSL max
template <class R> R glsign(R x) { return x > R(0) ? R(1) : (x < R(0) ? R(-1) : R(0)); }
template <class R> bool glstep(R edge, R x) { return !(x < edge); }  // step(edge, x) == 1
template <class R> R length(V3<R> a) { return M<R>::sqrt(dot(a, a)); }
template <class R> V3<R> normalize(V3<R> a) { return a / length(a); }
template <class R> V3<R> vabs(V3<R> a) { return v3(M<R>::abs(a.x), M<R>::abs(a.y), M<R>::abs(a.z)); }

enum : uint32_t {
  Q_GAMMA = 1u << 0, Q_GROUND = 1u << 1, Q_PDF_MISMATCH = 1u << 2, Q_DOUBLE_REFL = 1u << 3,
  Q_FIXED_IOR = 1u << 4, Q_EXP_ROUGH = 1u << 5, Q_THINLENS_NO_JITTER = 1u << 6, Q_UNGUARDED = 1u << 7,
};

struct Counters { uint64_t c[8] = {0, 0, 0, 0, 0, 0, 0, 0}; };

// ------------------------------------------------------------------ rng
uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// Philox-4x32-10, Salmon et al. SC'11 (Random123's philox4x32 with R = 10).
void philox4x32(const uint32_t in[4], const uint32_t key[2], uint32_t out[4]) {
  uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// Thomas Wang integer hash on a GLSL int (random.h:3-11).
int32_t hash(int32_t seed) {
  seed = (seed ^ 61) ^ (seed >> 16);
  seed = (int32_t)((uint32_t)seed * 9u);
  seed = seed ^ (seed >> 4);
  seed = (int32_t)((uint32_t)seed * 0x27d4eb2du);
  seed = seed ^ (seed >> 15);
  return seed;
}

struct Rng {
  int mode;
  uint32_t seed, pixel, sample, call;
  int32_t ox, oy;
  const float* noise;
  // randomNumberGeneratorOffset (random.h:13-18), offset read as unsigned
  void init(int m, uint32_t sd, const float* nz, int width, int px, int py, int smp) {
    mode = m; seed = sd; noise = nz;
    pixel = (uint32_t)(py * width + px); sample = (uint32_t)smp; call = 0;
    const uint32_t off = (uint32_t)(hash(px + py * 1024) ^ hash(smp));
    ox = (int32_t)(off % 1024u);
    oy = (int32_t)((off / 1024u) % 1024u);
  }
  // rand (random.h:20-27)
  void next(float u[4]) {
    if (mode == 1) {
      const float* t = noise + 4 * ((size_t)oy * 1024 + ox);
      u[0] = t[0]; u[1] = t[1]; u[2] = t[2]; u[3] = t[3];
      ox = (ox + 1) % 1024;
      if (ox == 0) oy = (oy + 1) % 1024;
      return;
    }
    const uint32_t ctr[4] = {pixel, sample, call, 0u};
    const uint32_t key[2] = {seed, 0x6A09E667u};
    uint32_t o[4];
    philox4x32(ctr, key, o);
    call += 1;
    for (int i = 0; i < 4; ++i) u[i] = (float)(o[i] >> 8) * 5.9604644775390625e-8f;
  }
};

// ------------------------------------------------------------- materials
struct Mat { int type; float e[3], a[3], rough; };
float q16(float x) { return vtb::h2f(vtb::f2h(x)); }

// ------------------------------------------------------------ camera math
template <class R>
void basis_of(const orc_camera* c, R* fwd, R* right, R* up) {
  // CameraParameters::getBasis (cameraParameters.cpp:43-50) with Imath's
  // normalized(): v / sqrt(x*x + y*y + z*z), zero vector stays zero.
  R d[3] = {R(c->target[0]) - R(c->eye[0]), R(c->target[1]) - R(c->eye[1]), R(c->target[2]) - R(c->eye[2])};
  auto norm = [](const R* v, R* o) {
    const R l = M<R>::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
    if (l == R(0)) { o[0] = o[1] = o[2] = R(0); return; }
    for (int i = 0; i < 3; ++i) o[i] = v[i] / l;
  };
  auto crs = [](const R* a, const R* b, R* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
  };
  norm(d, fwd);
  const R yaxis[3] = {R(0), R(1), R(0)};
  R r[3];
  crs(yaxis, fwd, r);
  norm(r, right);
  crs(fwd, right, up);
}

// Gauss-Jordan with partial pivoting (Imath::Matrix44::gjInverse).
template <class R>
bool gj_inverse(const R* m, R* out) {
  R t[4][4], s[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) { t[i][j] = m[4 * i + j]; s[i][j] = i == j ? R(1) : R(0); }
  for (int i = 0; i < 3; ++i) {
    int pivot = i;
    R pivotsize = M<R>::abs(t[i][i]);
    for (int j = i + 1; j < 4; ++j) {
      const R tmp = M<R>::abs(t[j][i]);
      if (tmp > pivotsize) { pivot = j; pivotsize = tmp; }
    }
    if (pivotsize == R(0)) return false;
    if (pivot != i)
      for (int j = 0; j < 4; ++j) { std::swap(t[i][j], t[pivot][j]); std::swap(s[i][j], s[pivot][j]); }
    for (int j = i + 1; j < 4; ++j) {
      const R f = t[j][i] / t[i][i];
      for (int k = 0; k < 4; ++k) { t[j][k] = t[j][k] - f * t[i][k]; s[j][k] = s[j][k] - f * s[i][k]; }
    }
  }
  for (int i = 3; i >= 0; --i) {
    const R f = t[i][i];
    if (f == R(0)) return false;
    for (int j = 0; j < 4; ++j) { t[i][j] = t[i][j] / f; s[i][j] = s[i][j] / f; }
    for (int j = 0; j < i; ++j) {
      const R g = t[j][i];
      for (int k = 0; k < 4; ++k) { t[j][k] = t[j][k] - g * t[i][k]; s[j][k] = s[j][k] - g * s[i][k]; }
    }
  }
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) out[4 * i + j] = s[i][j];
  return true;
}

template <class R> R rtan(R x) { return std::tan(x); }

// Renderer::updateCamera (renderer.cpp:343-397).
template <class R>
bool camera_uniforms(const orc_camera* c, int w, int h, R* proj, R* iproj, R* imv, R* vp) {
  R f[3], r[3], u[3];
  basis_of<R>(c, f, r, u);
  const R eye[3] = {R(c->eye[0]), R(c->eye[1]), R(c->eye[2])};
  auto d3 = [](const R* a, const R* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; };
  const R mv[16] = {r[0], r[1], r[2], -d3(eye, r), u[0], u[1], u[2], -d3(eye, u),
                    -f[0], -f[1], -f[2], d3(eye, f), R(0), R(0), R(0), R(1)};
  const R a = R(w) / R(h);
  const R fov = R(c->fov_y);
  R pm[16];
  if (c->lens_model == 2) {
    R dv[3] = {R(c->target[0]) - eye[0], R(c->target[1]) - eye[1], R(c->target[2]) - eye[2]};
    const R dist = M<R>::sqrt((dv[0] * dv[0] + dv[1] * dv[1]) + dv[2] * dv[2]);
    const R left = -rtan<R>(fov / R(2)) * dist;
    const R right = -left;
    const R bottom = -rtan<R>(fov / R(2)) * dist / a;
    const R top = -bottom;
    const R n = -R(c->near_distance), fr = -R(c->far_distance);
    const R tx = -(right + left) / (right - left);
    const R ty = -(top + bottom) / (top - bottom);
    const R tz = -(fr + n) / (fr - n);
    const R p[16] = {R(2) / (right - left), R(0), R(0), tx, R(0), R(2) / (top - bottom), R(0), ty,
                     R(0), R(0), R(-2) / (fr - n), tz, R(0), R(0), R(0), R(1)};
    std::memcpy(pm, p, sizeof(pm));
  } else {
    const R n = R(c->near_distance), fr = R(c->far_distance);
    const R e = R(1) / rtan<R>(fov / R(2));
    const R p[16] = {e / a, R(0), R(0), R(0), R(0), e, R(0), R(0),
                     R(0), R(0), (fr + n) / (n - fr), R(2) * fr * n / (n - fr), R(0), R(0), R(-1), R(0)};
    std::memcpy(pm, p, sizeof(pm));
  }
  std::memcpy(proj, pm, sizeof(pm));
  if (!gj_inverse<R>(mv, imv)) return false;
  if (!gj_inverse<R>(pm, iproj)) return false;
  vp[0] = R(0); vp[1] = R(0); vp[2] = R(w); vp[3] = R(h);
  return true;
}

// ---------------------------------------------------------------- tracer
template <class R>
struct Tracer {
  typedef V3<R> vec3;
  struct vec4 { R x, y, z, w; };
  struct Basis { vec3 position, tangent, normal, binormal; };

  // uniforms
  int res[3];
  int max_steps;
  vec3 bmin, bmax, vsize;
  R viewport[4], proj[16], iproj[16], imv[16];
  R frag_z;
  R lens_radius, focal_distance;
  int lens_model;
  vec3 bg_top, bg_bottom;
  R bg_rot;
  const orc_settings* S;
  const orc_scene* scene;
  const orc_env* env;
  std::vector<Mat> pal;
  R inv_gamma;
  int width;
  const float* noise;

  static R P() { return M<R>::PI; }

  bool setup(const orc_camera* c, const orc_settings* s, const orc_scene* sc, const orc_env* e, const float* nz,
             int w, int h) {
    S = s; scene = sc; env = e; noise = nz; width = w;
    for (int i = 0; i < 3; ++i) res[i] = sc->res[i];
    // createVoxelDataTexture bounds (renderer.cpp:845-850), voxel size uniform (:928-931)
    const float voxel = 1000.0f / (float)std::max(res[0], std::max(res[1], res[2]));
    float fmin[3], fmax[3], fvs[3];
    for (int i = 0; i < 3; ++i) {
      const float size = voxel * (float)res[i];
      fmin[i] = -size * 0.5f;
      fmax[i] = size * 0.5f;
      fvs[i] = (fmax[i] - fmin[i]) / (float)res[i];
    }
    bmin = v3<R>(fmin[0], fmin[1], fmin[2]);
    bmax = v3<R>(fmax[0], fmax[1], fmax[2]);
    vsize = v3<R>(fvs[0], fvs[1], fvs[2]);
    // int(2 * ceil(length(vec3(voxelResolution)))) (dda.h:98), in float as the shader
    const float len = std::sqrt(((float)res[0] * (float)res[0] + (float)res[1] * (float)res[1]) + (float)res[2] * (float)res[2]);
    max_steps = (int)(2.0f * std::ceil(len));
    if (!camera_uniforms<R>(c, w, h, proj, iproj, imv, viewport)) return false;
    frag_z = R(0.5f * c->near_distance + 0.5f);
    lens_radius = R(c->lens_radius);
    focal_distance = R(c->focal_distance);
    lens_model = c->lens_model;
    bg_top = v3<R>(s->background_top[0], s->background_top[1], s->background_top[2]);
    bg_bottom = v3<R>(s->background_bottom[0], s->background_bottom[1], s->background_bottom[2]);
    bg_rot = R(s->background_rotation);
    inv_gamma = R(1) / R(s->gamma);
    pal.resize(sc->n_palette);
    for (int i = 0; i < sc->n_palette; ++i) {
      const orc_material& m = sc->palette[i];
      pal[i].type = (int)q16((float)m.type);
      for (int k = 0; k < 3; ++k) { pal[i].e[k] = q16(m.emission[k]); pal[i].a[k] = q16(m.albedo[k]); }
      pal[i].rough = q16(m.roughness);
    }
    return true;
  }

  // GLSL mat4 * vec4 (row-major storage, transpose = GL_TRUE upload)
  vec4 mul(const R* m, vec4 v) const {
    vec4 r;
    r.x = ((m[0] * v.x + m[1] * v.y) + m[2] * v.z) + m[3] * v.w;
    r.y = ((m[4] * v.x + m[5] * v.y) + m[6] * v.z) + m[7] * v.w;
    r.z = ((m[8] * v.x + m[9] * v.y) + m[10] * v.z) + m[11] * v.w;
    r.w = ((m[12] * v.x + m[13] * v.y) + m[14] * v.z) + m[15] * v.w;
    return r;
  }
  static vec4 v4(R x, R y, R z, R w) { vec4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }

  // voxel occupancy (texelFetch(materialOffsetTexture).r >= 0)
  bool occupied(int x, int y, int z) const {
    return scene->grid[(size_t)x + (size_t)res[0] * ((size_t)y + (size_t)res[1] * (size_t)z)] != 0;
  }
  // material of a hit voxel; the ground below the volume uses the configured entry
  Mat material(int x, int y, int z, Counters& C) const {
    C.c[2] += 1;
    if (y < 0) return pal[S->ground_material];
    const uint8_t g = scene->grid[(size_t)x + (size_t)res[0] * ((size_t)y + (size_t)res[1] * (size_t)z)];
    if (g == 0) { Mat m; m.type = -1; for (int k = 0; k < 3; ++k) m.e[k] = m.a[k] = 0.0f; m.rough = 0.0f; return m; }
    return pal[g - 1];
  }

  // rayAABBIntersection (aabb.h:1-32)
  static R aabb(vec3 o, vec3 d, vec3 bmn, vec3 bmx) {
    const vec3 inv = v3<R>(R(1) / d.x, R(1) / d.y, R(1) / d.z);
    const vec3 tMin3 = (bmn - o) * inv;
    const vec3 tMax3 = (bmx - o) * inv;
    const vec3 tmin = v3<R>(glmin(tMin3.x, tMax3.x), glmin(tMin3.y, tMax3.y), glmin(tMin3.z, tMax3.z));
    const R tminf = glmax(tmin.x, glmax(tmin.y, tmin.z));
    const vec3 tmax = v3<R>(glmax(tMin3.x, tMax3.x), glmax(tMin3.y, tMax3.y), glmax(tMin3.z, tMax3.z));
    const R tmaxf = glmin(tmax.x, glmin(tmax.y, tmax.z));
    if (tmaxf < R(0)) return R(-1);
    if (tminf > tmaxf) return R(-1);
    return glmax(R(0), tminf);
  }

  // raymarch (dda.h:7-61); the early return on an origin outside the grid
  // reports that voxel position (the shader leaves it unwritten).
  bool raymarch(vec3 o, vec3 d, int maxSteps, int* hit, int* steps_out, Counters& C) const {
    bool isect = false;
    const vec3 voxelExtent = v3<R>(R(1), R(1), R(1)) / (bmax - bmin);
    o = o + v3<R>(glsign(d.x), glsign(d.y), glsign(d.z)) * R(0.001f);
    const vec3 resv = v3<R>(R(res[0]), R(res[1]), R(res[2]));
    const vec3 vo = ((o - bmin) * voxelExtent) * resv;
    vec3 vp = v3<R>(M<R>::floor(vo.x), M<R>::floor(vo.y), M<R>::floor(vo.z));
    *steps_out = 0;
    if (vp.x < R(0) || vp.y < R(0) || vp.z < R(0) || vp.x >= resv.x || vp.y >= resv.y || vp.z >= resv.z) {
      hit[0] = (int)vp.x; hit[1] = (int)vp.y; hit[2] = (int)vp.z;
      return false;
    }
    // mix(d, vec3(1e-5), step(abs(d), vec3(1e-5)))
    const R eps = R(1e-5f);
    d.x = glstep(M<R>::abs(d.x), eps) ? eps : d.x;
    d.y = glstep(M<R>::abs(d.y), eps) ? eps : d.y;
    d.z = glstep(M<R>::abs(d.z), eps) ? eps : d.z;
    const vec3 inc = v3<R>(R(1) / d.x, R(1) / d.y, R(1) / d.z);
    const vec3 sg = v3<R>(glsign(d.x), glsign(d.y), glsign(d.z));
    vec3 dis = (((vp - vo) + v3<R>(R(0.5f), R(0.5f), R(0.5f))) + sg * R(0.5f)) * inc;
    int steps = 0;
    while (steps < maxSteps) {
      if (vp.x < R(0) || vp.y < R(0) || vp.z < R(0) || vp.x >= resv.x || vp.y >= resv.y || vp.z >= resv.z) break;
      C.c[1] += 1;
      if (occupied((int)vp.x, (int)vp.y, (int)vp.z)) { isect = true; break; }
      // mask = step(dis.xyz, dis.yxy) * step(dis.xyz, dis.zzx)
      const R mx = (glstep(dis.x, dis.y) && glstep(dis.x, dis.z)) ? R(1) : R(0);
      const R my = (glstep(dis.y, dis.x) && glstep(dis.y, dis.z)) ? R(1) : R(0);
      const R mz = (glstep(dis.z, dis.y) && glstep(dis.z, dis.x)) ? R(1) : R(0);
      const vec3 mask = v3<R>(mx, my, mz);
      // dis += mask * sign * inc; voxelPos += mask * sign
      dis = dis + (mask * sg) * inc;
      vp = vp + mask * sg;
      ++steps;
    }
    hit[0] = (int)vp.x; hit[1] = (int)vp.y; hit[2] = (int)vp.z;
    *steps_out = steps;
    return isect;
  }

  // traverse (dda.h:63-100)
  bool traverse(vec3 o, vec3 d, int* vs, bool* ground, int* steps, Counters& C) const {
    C.c[6] += 1;
    if (raymarch(o, d, max_steps, vs, steps, C)) { *ground = false; return true; }
    *ground = (S->quirks & Q_GROUND) && vs[1] < 0;
    return *ground;
  }

  // voxelSpaceToWorldSpace (coordinates.h:59-82).  one_axis: a three-way
  // tie (a hit exactly on a voxel corner, whose reference frame is
  // normalize(0) = NaN) keeps only the axis of the largest |rd| component,
  // x before y before z.
  Basis voxel_basis(const int* p, vec3 ro, vec3 rd, bool one_axis = false) const {
    const vec3 vsP = v3<R>(R(p[0]), R(p[1]), R(p[2]));
    const vec3 wsVoxelMin = vsP * vsize + bmin;
    const vec3 wsVoxelMax = wsVoxelMin + vsize;
    const R t = aabb(ro, rd, wsVoxelMin, wsVoxelMax);
    Basis b;
    b.position = ro + rd * t;
    const vec3 center = wsVoxelMin + vsize * R(0.5f);
    const vec3 c2h = b.position - center;
    const vec3 a = vabs(c2h);
    // step(a.yxx, a.xyz) * step(a.zzy, a.xyz)
    R mx = (glstep(a.y, a.x) ? R(1) : R(0)) * (glstep(a.z, a.x) ? R(1) : R(0));
    R my = (glstep(a.x, a.y) ? R(1) : R(0)) * (glstep(a.z, a.y) ? R(1) : R(0));
    R mz = (glstep(a.x, a.z) ? R(1) : R(0)) * (glstep(a.y, a.z) ? R(1) : R(0));
    if (one_axis && mx != R(0) && my != R(0) && mz != R(0)) {
      const vec3 ad = vabs(rd);
      const bool kx = ad.x >= ad.y && ad.x >= ad.z;
      const bool ky = !kx && ad.y >= ad.z;
      mx = kx ? R(1) : R(0);
      my = ky ? R(1) : R(0);
      mz = (!kx && !ky) ? R(1) : R(0);
    }
    b.normal = v3<R>(mx, my, mz) * v3<R>(glsign(c2h.x), glsign(c2h.y), glsign(c2h.z));
    const R k = R(0.57735026919f);
    const vec3 tangent = cross(b.normal, v3<R>(k, k, k));
    b.binormal = normalize(cross(tangent, b.normal));
    b.tangent = normalize(cross(b.binormal, b.normal));
    return b;
  }
  static vec3 local_to_world(vec3 l, const Basis& b) { return (l.x * b.tangent + l.y * b.normal) + l.z * b.binormal; }
  static vec3 world_to_local(vec3 w, const Basis& b) {
    return v3<R>(dot(w, b.tangent), dot(w, b.normal), dot(w, b.binormal));
  }

  // sampling.h:2-43
  static void disk(R u0, R u1, R* x, R* y) {
    const R r = M<R>::sqrt(u0);
    const R theta = (R(2) * P()) * u1;
    *x = r * M<R>::cos(theta); *y = r * M<R>::sin(theta);
  }
  static vec4 cosine_hemisphere(R u0, R u1) {
    R px, py;
    disk(u0, u1, &px, &py);
    const R y = M<R>::sqrt(glmax(R(0), (R(1) - px * px) - py * py));
    return v4(px, y, py, y / P());
  }
  static vec4 uniform_hemisphere(R u0, R u1) {
    const R y = u0;
    const R r = M<R>::sqrt(glmax(R(0), R(1) - y * y));
    const R phi = (u1 * R(2)) * P();
    return v4(r * M<R>::cos(phi), y, r * M<R>::sin(phi), R(1) / (R(2) * P()));
  }
  static R power_heuristic(R f, R g) { return (f * f) / ((f * f) + (g * g)); }
  static R luminance(vec3 c) { return (c.x * R(0.2126f) + c.y * R(0.7152f)) + c.z * R(0.0722f); }

  // ---------------------------------------------------------------- bsdfs
  struct FP { vec3 f; R pdf; };
  static R G(vec3 wo, vec3 wi, vec3 wh) {                           // microfacet.h:5-15
    const R nh = wh.y, no = wo.y, ni = wi.y;
    const R woh = M<R>::abs(dot(wo, wh));
    return glmin(R(1), glmin(((R(2) * nh) * no) / woh, ((R(2) * nh) * ni) / woh));
  }
  vec3 F(vec3 f0, R ch) const {                                      // microfacet.h:64-69
    const R p = M<R>::pow(R(1) - ch, R(5));
    if (S->quirks & Q_FIXED_IOR) {
      const R ior = R(7.3f);
      const R sr0 = (R(1) - ior) / (R(1) + ior);
      const R r0 = sr0 * sr0;
      const R fr = r0 + (R(1) - r0) * p;
      return v3<R>(fr, fr, fr);
    }
    return v3<R>(f0.x + (R(1) - f0.x) * p, f0.y + (R(1) - f0.y) * p, f0.z + (R(1) - f0.z) * p);
  }
  static FP D(vec3 refl, R e, vec3 wo, vec3 wh) {                   // microfacet.h:19-37
    const R pc = M<R>::pow(wh.y, e);
    const R f = ((e + R(2)) * M<R>::INV_TWOPI) * pc;
    const R wodh = dot(wo, wh);
    FP r;
    r.pdf = (wodh <= R(0)) ? R(0) : ((e + R(1)) * pc) / ((M<R>::TWO_PI * R(4)) * wodh);
    r.f = refl * f;
    return r;
  }
  R exponent(R rough) const {                                        // metal.h:13-14
    if (S->quirks & Q_EXP_ROUGH) return rough;
    const R r2 = glmax(rough * rough, R(1e-6f));
    return glmax(R(2) / r2 - R(2), R(0));
  }
  FP eval_bsdf(const Mat& m, vec3 wo, vec3 wi) const {              // materials.h:7-19
    FP r;
    const vec3 albedo = v3<R>(m.a[0], m.a[1], m.a[2]);
    if (m.type == 0) { r.pdf = wi.y / P(); r.f = albedo / P(); return r; }   // lambertian.h:23-29
    if (m.type == 1 || m.type == 2) {                                // microfacet.h:73-91
      const vec3 refl = m.type == 1 ? albedo : v3<R>(R(1), R(1), R(1));
      const R e = exponent(R(m.rough));
      const R cwi = wi.y, cwo = wo.y;
      const vec3 wh = normalize(wi + wo);
      const R ch = dot(wi, wh);
      const bool fixed = (S->quirks & Q_FIXED_IOR) != 0;
      r = D(fixed ? refl : v3<R>(R(1), R(1), R(1)), e, wo, wh);
      const R g = G(wo, wi, wh);
      const vec3 fr = F(refl, ch);
      const R den = (R(4) * cwo) * cwi;
      r.f = v3<R>(r.f.x * ((g * fr.x) / den), r.f.y * ((g * fr.y) / den), r.f.z * ((g * fr.z) / den));
      return r;
    }
    r.f = v3<R>(R(0), R(0), R(0)); r.pdf = R(0);
    return r;
  }
  // sampleMaterialBSDF (materials.h:30-43); u_rr = the block's third value
  vec3 sample_bsdf(const Mat& m, vec3 wo, Rng& rng, FP& out, R& u_rr) const {
    float u[4];
    rng.next(u);
    u_rr = R(u[2]);
    const vec3 albedo = v3<R>(m.a[0], m.a[1], m.a[2]);
    if (m.type == 0) {                                               // lambertian.h:10-19
      const vec4 s = cosine_hemisphere(R(u[0]), R(u[1]));
      out.f = albedo / P();
      out.pdf = s.w;
      return v3<R>(s.x, s.y, s.z);
    }
    const vec3 refl = m.type == 1 ? albedo : v3<R>(R(1), R(1), R(1));
    const R e = exponent(R(m.rough));
    // sampleD (microfacet.h:41-61)
    const R cosTheta = M<R>::pow(R(u[0]), R(1) / (e + R(1)));
    const R sinTheta = M<R>::sqrt(glmax(R(0), R(1) - cosTheta * cosTheta));
    const R phi = (R(u[1]) * R(2)) * P();
    const vec3 wh = v3<R>(sinTheta * M<R>::cos(phi), cosTheta, sinTheta * M<R>::sin(phi));
    const vec3 wi = (-wo) + (R(2) * dot(wo, wh)) * wh;
    const bool fixed = (S->quirks & Q_FIXED_IOR) != 0;
    FP d = D(fixed ? refl : v3<R>(R(1), R(1), R(1)), e, wo, wh);
    // sampleBSDF_Microfacet (microfacet.h:102-123)
    const R cwi = wi.y, cwo = wo.y;
    const vec3 wh2 = normalize(wi + wo);
    const R ch = dot(wi, wh2);
    const R g = G(wo, wi, wh2);
    const vec3 fr = F(refl, ch);
    const R den = (R(4) * cwo) * cwi;
    vec3 f = d.f;
    if (S->quirks & Q_DOUBLE_REFL) f = refl * f;
    out.f = v3<R>(((f.x * g) * fr.x) / den, ((f.y * g) * fr.y) / den, ((f.z * g) * fr.z) / den);
    out.pdf = d.pdf;
    return wi;
  }

  // ----------------------------------------------------------------- env
  vec3 texel(int i, int j) const {
    const uint16_t* t = env->texels + 4 * ((size_t)j * env->w + i);
    return v3<R>(vtb::h2f(t[0]), vtb::h2f(t[1]), vtb::h2f(t[2]));
  }
  // texture() with GL_LINEAR and clamp to edge
  vec3 lookup(R u, R v, Counters& C) const {
    C.c[3] += 1;
    const int w = env->w, h = env->h;
    const R x = u * R(w) - R(0.5f), y = v * R(h) - R(0.5f);
    const R x0 = M<R>::floor(x), y0 = M<R>::floor(y);
    const R fx = x - x0, fy = y - y0;
    int i0 = (int)x0, j0 = (int)y0, i1 = i0 + 1, j1 = j0 + 1;
    i0 = std::min(std::max(i0, 0), w - 1); i1 = std::min(std::max(i1, 0), w - 1);
    j0 = std::min(std::max(j0, 0), h - 1); j1 = std::min(std::max(j1, 0), h - 1);
    const R gx = R(1) - fx, gy = R(1) - fy;
    const vec3 a = texel(i0, j0) * gx + texel(i1, j0) * fx;
    const vec3 b = texel(i0, j1) * gx + texel(i1, j1) * fx;
    return a * gy + b * fy;
  }
  // uvCoordFromVector / directionFromUVCoord (coordinates.h:97-116)
  void uv_of(vec3 v, R* u, R* vv) const {
    const R theta = M<R>::acos(v.y);
    const R phi = (M<R>::atan2(v.z, v.x) + P()) + bg_rot;
    const R x = phi / M<R>::TWO_PI;
    *u = x - R(1) * M<R>::floor(x / R(1));
    *vv = theta / P();
  }
  vec3 dir_of(R u, R v) const {
    const R phi = ((u * M<R>::TWO_PI) - P()) - bg_rot;
    const R theta = v * P();
    const R st = M<R>::sin(theta);
    return v3<R>(st * M<R>::cos(phi), M<R>::cos(theta), st * M<R>::sin(phi));
  }
  // getBackgroundColor (lights.h:4-17)
  vec3 background(vec3 d, Counters& C) const {
    if (env && env->texels) {
      R u, v;
      uv_of(d, &u, &v);
      return lookup(u, v, C);
    }
    const R bias = glmax(R(0), d.y);
    return bg_bottom * (R(1) - bias) + bg_top * bias;
  }
  // evaluateEnvironmentRadiance (lights.h:20-33)
  vec3 eval_env(vec3 d, R* pdf, Counters& C) const {
    const vec3 L = background(d, C);
    if (env && env->texels) *pdf = luminance(L) / R(env->integral);
    else *pdf = (S->quirks & Q_PDF_MISMATCH) ? R(1) / (R(4) * P()) : R(1) / (R(2) * P());
    return L;
  }
  // binarySearchCDFV/U (envMapSample.h:70-123)
  static int search(const float* cdf, int high, R u, Counters& C) {
    int low = 0;
    while (low != high - 1) {
      const int mid = (low + high) / 2;
      C.c[4] += 1;
      if (u < R(cdf[mid])) high = mid; else low = mid;
    }
    return low;
  }
  // sampleEnvironmentRadiance (lights.h:36-55) / sampleEnvironmentTexture (envMapSample.h:23-65)
  vec3 sample_env(const Basis& b, R u0, R u1, vec3* dir, R* pdf, Counters& C) const {
    if (env && env->texels) {
      const int su = (env->cdf_w ? env->cdf_w : env->w) + 1, sv = (env->cdf_h ? env->cdf_h : env->h) + 1;
      const int row = search(env->cdf_v, sv - 1, u1, C);
      const float* cu = env->cdf_u + (size_t)row * su;
      const int col = search(cu, su - 1, u0, C);
      C.c[4] += 4;
      const R du = (u0 - R(cu[col])) / (R(cu[col + 1]) - R(cu[col]));
      const R dv = (u1 - R(env->cdf_v[row])) / (R(env->cdf_v[row + 1]) - R(env->cdf_v[row]));
      const R u = (R(col) + du) / R(su - 1);
      const R v = (R(row) + dv) / R(sv - 1);
      *dir = dir_of(u, v);
      const vec3 L = lookup(u, v, C);
      *pdf = luminance(L) / R(env->integral);
      return L;
    }
    const vec4 s = uniform_hemisphere(u0, u1);
    *dir = local_to_world(v3<R>(s.x, s.y, s.z), b);
    *pdf = s.w;
    return background(*dir, C);
  }

  // ---------------------------------------------------------------- camera
  vec4 screen_to_eye_persp(vec3 w) const {                         // coordinates.h:12-27
    vec3 ndc;
    ndc.x = ((R(2) * w.x) - (R(2) * viewport[0])) / viewport[2] - R(1);
    ndc.y = ((R(2) * w.y) - (R(2) * viewport[1])) / viewport[3] - R(1);
    ndc.z = ((R(2) * w.z - R(0)) - R(1)) / (R(1) - R(0));
    const R cw = proj[11] / (ndc.z - (proj[10] / proj[14]));
    return mul(iproj, v4(ndc.x * cw, ndc.y * cw, ndc.z * cw, cw));
  }
  vec4 screen_to_eye_ortho(vec3 w) const {                         // coordinates.h:1-10
    vec3 ndc;
    ndc.x = (w.x / viewport[2]) * R(2) - R(1);
    ndc.y = (w.y / viewport[3]) * R(2) - R(1);
    ndc.z = ((R(2) * w.z - R(0)) - R(1)) / (R(1) - R(0));
    return mul(iproj, v4(ndc.x, ndc.y, ndc.z, R(1)));
  }
  // generateRay (generateRay.h:1-123)
  void generate_ray(vec3 frag, Rng& rng, vec3* o, vec3* d) const {
    if (lens_model == 0) {
      float u[4];
      rng.next(u);
      const vec3 jitter = v3<R>(R(u[0]) - R(0.5f), R(u[1]) - R(0.5f), R(0));
      const vec4 es = screen_to_eye_persp(frag + jitter);
      const vec4 oo = mul(imv, v4(R(0), R(0), R(0), R(1)));
      *o = v3<R>(oo.x, oo.y, oo.z);
      const vec3 n = normalize(v3<R>(es.x, es.y, es.z));
      const vec4 w = mul(imv, v4(n.x, n.y, n.z, R(0)));
      const R l = M<R>::sqrt(((w.x * w.x + w.y * w.y) + w.z * w.z) + w.w * w.w);
      *d = v3<R>(w.x / l, w.y / l, w.z / l);
    } else if (lens_model == 1) {
      float u[4];
      rng.next(u);
      R dx, dy;
      disk(R(u[0]), R(u[1]), &dx, &dy);
      const vec3 lens = v3<R>(dx * lens_radius, dy * lens_radius, R(0));
      vec3 fp = frag;
      if (!(S->quirks & Q_THINLENS_NO_JITTER)) fp = frag + v3<R>(R(u[2]) - R(0.5f), R(u[3]) - R(0.5f), R(0));
      const vec4 e4 = screen_to_eye_persp(fp);
      const vec3 eo = v3<R>(e4.x, e4.y, e4.z);
      const vec3 ed = normalize(eo);
      const R t = focal_distance / -(ed.z);
      const vec3 ef = eo + t * ed;
      const vec4 wf = mul(imv, v4(ef.x, ef.y, ef.z, R(1)));
      const vec4 wo = mul(imv, v4(lens.x, lens.y, lens.z, R(1)));
      *o = v3<R>(wo.x, wo.y, wo.z);
      *d = normalize(v3<R>(wf.x, wf.y, wf.z) - *o);
    } else {
      const vec4 e = mul(imv, screen_to_eye_ortho(frag));
      *o = v3<R>(e.x, e.y, e.z);
      const vec4 dd = mul(imv, v4(R(0), R(0), R(-1), R(0)));
      *d = v3<R>(dd.x, dd.y, dd.z);
    }
  }

  // directLighting (pathTracer.fs:64-170)
  vec3 direct_lighting(const Mat& m, const Basis& b, vec3 wo, Rng& rng, Counters& C) const {
    float u[4];
    rng.next(u);
    const int numLights = (int)scene->n_emissive + 1;
    const int lightIndex = (int)(R(u[0]) * R(numLights));
    const bool samplingEmissive = lightIndex < numLights - 1;
    vec3 dir, L;
    R pdf;
    int ev[3] = {0, 0, 0};
    if (samplingEmissive) {
      C.c[5] += 1;
      int idx = scene->emissive[lightIndex];
      // voxelIndexToVoxelPos (coordinates.h:118-127)
      const int dz = res[0] * res[1], dy = res[0];
      ev[2] = idx / dz; idx -= ev[2] * dz;
      ev[1] = idx / dy; idx -= ev[1] * dy;
      ev[0] = idx;
      const Mat lm = material(ev[0], ev[1], ev[2], C);
      const R sc = R(S->nee_emission_scale);
      L = v3<R>(sc, sc, sc) * v3<R>(lm.e[0], lm.e[1], lm.e[2]);
      const vec3 resv = v3<R>(R(res[0]), R(res[1]), R(res[2]));
      vec3 wp = (v3<R>(R(ev[0]), R(ev[1]), R(ev[2])) / resv) * (bmax - bmin) + bmin;
      wp = wp + v3<R>(R(u[1]), R(u[2]), R(u[3])) * vsize;
      const vec3 toLight = wp - b.position;
      const R r = length(toLight);
      dir = toLight / r;
      const Basis lb = voxel_basis(ev, b.position, dir);
      const R voxelArea = (R(6) * vsize.x) * vsize.y;
      const R jacobian = (r * r) / M<R>::abs(dot(-dir, lb.normal));
      pdf = jacobian / voxelArea;
    } else {
      L = sample_env(b, R(u[1]), R(u[2]), &dir, &pdf, C);
    }
    pdf = pdf / R(numLights);
    int sh[3], steps;
    bool ground;
    const bool missed = !traverse(b.position, dir, sh, &ground, &steps, C);
    const vec3 zero = v3<R>(R(0), R(0), R(0));
    if (samplingEmissive) {
      if (missed || sh[0] != ev[0] || sh[1] != ev[1] || sh[2] != ev[2]) return zero;
    } else {
      if (!missed) return zero;
    }
    // light samples with a degenerate pdf contribute nothing (unless the
    // unguarded-samples quirk asks for the reference's division)
    if (!(S->quirks & Q_UNGUARDED) && !(pdf > R(0) && pdf < R(INFINITY))) return zero;
    const vec3 lwo = world_to_local(wo, b);
    const vec3 lwi = world_to_local(dir, b);
    const FP bf = eval_bsdf(m, lwo, lwi);
    const R mis = power_heuristic(pdf, bf.pdf);
    return (((bf.f * L) * M<R>::abs(dot(dir, b.normal))) * mis) / pdf;
  }

  // main() of editMode.fs:58-144: white voxels lit by sqrt(max(0, -d.n)),
  // halved when the shadow ray towards -lightDirection = (-1, 1, 1) is
  // blocked (the uniform keeps its initialiser: renderer.cpp:279-280 sets a
  // name the shader does not declare), the selected voxel red, the
  // wireframe overlay; the background on a miss; no gamma.
  void trace_edit(int px, int py, int sample, R out[4], int32_t* hitrec, Counters& C) const {
    Rng rng;
    rng.init(S->rng_mode, S->seed, noise, width, px, py, sample);
    C.c[0] += 1;
    vec3 o, d;
    generate_ray(v3<R>(R((float)px + 0.5f), R((float)py + 0.5f), frag_z), rng, &o, &d);
    if (hitrec) { hitrec[0] = hitrec[1] = hitrec[2] = -1; hitrec[3] = 0; }
    out[3] = R(1);
    vec3 col;
    const R t = aabb(o, d, bmin, bmax);
    int vs[3], steps;
    bool ground = false;
    bool hit = false;
    if (t >= R(0)) {
      hit = traverse(o + t * d, d, vs, &ground, &steps, C);
      if (hitrec) {
        hitrec[0] = vs[0]; hitrec[1] = vs[1]; hitrec[2] = vs[2];
        int flags = (hit ? 1 : 0) << 8 | (ground ? 1 : 0) << 9;
        if (hit) {
          const Basis b = voxel_basis(vs, o, d);
          flags |= ((int)b.normal.x + 1) | (((int)b.normal.y + 1) << 2) | (((int)b.normal.z + 1) << 4);
        }
        hitrec[3] = flags;
      }
    }
    if (!hit) {                                                          // :79-92
      col = background(d, C);
    } else if (S->select_enabled && vs[0] == S->selected_voxel[0] && vs[1] == S->selected_voxel[1] &&
               vs[2] == S->selected_voxel[2]) {
      col = v3<R>(R(1), R(0), R(0));                                     // :107-112
    } else {
      const Basis b = voxel_basis(vs, o, d, !(S->quirks & Q_UNGUARDED));
      vec3 albedo = v3<R>(R(1), R(1), R(1));
      if (S->wireframe_opacity > 0.0f) {                                 // :114-125
        const vec3 resv = v3<R>(R(res[0]), R(res[1]), R(res[2]));
        const vec3 vc = ((b.position - bmin) / (bmax - bmin)) * resv;
        const vec3 uvw = v3<R>(R(vs[0]), R(vs[1]), R(vs[2])) - vc;
        const R ux = M<R>::abs(dot(v3<R>(b.normal.y, b.normal.z, b.normal.x), uvw));
        const R uy = M<R>::abs(dot(v3<R>(b.normal.z, b.normal.x, b.normal.y), uvw));
        const R th = R(S->wireframe_thickness);
        R wire = (glstep(th, ux) ? R(1) : R(0)) * (glstep(ux, R(1) - th) ? R(1) : R(0));
        wire = wire * (glstep(th, uy) ? R(1) : R(0));
        wire = wire * (glstep(uy, R(1) - th) ? R(1) : R(0));
        wire = (R(1) - R(S->wireframe_opacity)) + R(S->wireframe_opacity) * wire;
        albedo = albedo * v3<R>(wire, wire, wire);
      }
      R lighting = glmax(R(0), dot(-d, b.normal));                      // :129-130
      lighting = M<R>::sqrt(lighting);
      int sh[3], st2;
      bool g2;
      if (traverse(b.position, v3<R>(R(-1), R(1), R(1)), sh, &g2, &st2, C)) lighting = lighting * R(0.5);
      col = albedo * lighting;
    }
    out[0] = col.x; out[1] = col.y; out[2] = col.z;
  }

  // main() (pathTracer.fs:172-296); returns the per-sample output.
  void trace(int px, int py, int sample, R out[4], int32_t* hitrec, Counters& C) const {
    if (S->integrator == 1) {
      trace_edit(px, py, sample, out, hitrec, C);
      return;
    }
    Rng rng;
    rng.init(S->rng_mode, S->seed, noise, width, px, py, sample);
    C.c[0] += 1;
    vec3 radiance = v3<R>(R(0), R(0), R(0));
    vec3 o, d;
    generate_ray(v3<R>(R((float)px + 0.5f), R((float)py + 0.5f), frag_z), rng, &o, &d);
    if (hitrec) { hitrec[0] = hitrec[1] = hitrec[2] = -1; hitrec[3] = 0; }
    const R t = aabb(o, d, bmin, bmax);
    int vs[3], steps;
    bool ground = false;
    bool done = false;
    if (t < R(0)) {
      radiance = background(d, C);
      done = true;
    } else {
      const vec3 entry = o + t * d;
      const bool hit = traverse(entry, d, vs, &ground, &steps, C);
      if (hitrec) {
        hitrec[0] = vs[0]; hitrec[1] = vs[1]; hitrec[2] = vs[2];
        int flags = (hit ? 1 : 0) << 8 | (ground ? 1 : 0) << 9;
        if (hit) {
          const Basis b = voxel_basis(vs, o, d);
          flags |= ((int)b.normal.x + 1) | (((int)b.normal.y + 1) << 2) | (((int)b.normal.z + 1) << 4);
        }
        hitrec[3] = flags;
      }
      if (!hit) { radiance = background(d, C); done = true; }
    }
    if (!done) {
      vec3 throughput = v3<R>(R(1), R(1), R(1));
      int bounces = 0;
      while (bounces < S->max_bounces) {
        const Basis b = voxel_basis(vs, o, d, !(S->quirks & Q_UNGUARDED));
        const Mat m = material(vs[0], vs[1], vs[2], C);
        if (S->select_enabled && vs[0] == S->selected_voxel[0] && vs[1] == S->selected_voxel[1] &&
            vs[2] == S->selected_voxel[2]) {
          radiance = radiance + v3<R>(R(1), R(0), R(0));
          break;
        }
        const vec3 wo = -d;
        const vec3 lwo = world_to_local(wo, b);
        if (bounces == 0) radiance = radiance + throughput * v3<R>(m.e[0], m.e[1], m.e[2]);
        radiance = radiance + throughput * direct_lighting(m, b, wo, rng, C);
        FP bs;
        R u_rr;
        const vec3 lwi = sample_bsdf(m, lwo, rng, bs, u_rr);
        if (S->wireframe_opacity > 0.0f) {                              // :260-270
          const vec3 resv = v3<R>(R(res[0]), R(res[1]), R(res[2]));
          const vec3 vc = ((b.position - bmin) / (bmax - bmin)) * resv;
          const vec3 uvw = v3<R>(R(vs[0]), R(vs[1]), R(vs[2])) - vc;
          const R ux = M<R>::abs(dot(v3<R>(b.normal.y, b.normal.z, b.normal.x), uvw));
          const R uy = M<R>::abs(dot(v3<R>(b.normal.z, b.normal.x, b.normal.y), uvw));
          const R th = R(S->wireframe_thickness);
          R wire = (glstep(th, ux) ? R(1) : R(0)) * (glstep(ux, R(1) - th) ? R(1) : R(0));
          wire = wire * (glstep(th, uy) ? R(1) : R(0));
          wire = wire * (glstep(uy, R(1) - th) ? R(1) : R(0));
          wire = (R(1) - R(S->wireframe_opacity)) + R(S->wireframe_opacity) * wire;
          bs.f = bs.f * v3<R>(wire, wire, wire);
        }
        const vec3 wwi = local_to_world(lwi, b);
        const bool guard = !(S->quirks & Q_UNGUARDED);
        // zero-pdf or below-surface BSDF samples end the path unless unguarded
        if (guard && (!(bs.pdf > R(0)) || !(lwi.y > R(0)))) break;
        throughput = throughput * ((bs.f * M<R>::abs(dot(wwi, b.normal))) / bs.pdf);
        if (guard && !(std::isfinite(throughput.x) && std::isfinite(throughput.y) && std::isfinite(throughput.z))) break;
        if (S->rr_start_bounce >= 0 && bounces >= S->rr_start_bounce) {   // Russian roulette
          const R q = glmin(R(1), glmax(throughput.x, glmax(throughput.y, throughput.z)));
          if (!(u_rr < q)) break;
          throughput = throughput / q;
        }
        o = b.position;
        d = wwi;
        if (!traverse(o, d, vs, &ground, &steps, C)) {
          R lpdf;
          const vec3 Le = eval_env(d, &lpdf, C);
          const R mis = power_heuristic(bs.pdf, lpdf);
          radiance = radiance + (throughput * Le) * mis;
          break;
        }
        bounces++;
      }
    }
    if (S->quirks & Q_GAMMA) {                                         // :294-295
      const R ex = R(S->exposure);
      out[0] = M<R>::pow(radiance.x * ex, inv_gamma);
      out[1] = M<R>::pow(radiance.y * ex, inv_gamma);
      out[2] = M<R>::pow(radiance.z * ex, inv_gamma);
    } else {
      out[0] = radiance.x; out[1] = radiance.y; out[2] = radiance.z;
    }
    out[3] = R(1);
  }
};

template <class F>
void parallel_rows(int h, int threads, F fn) {
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  threads = std::min(threads, std::max(h, 1));
  std::atomic<int> next(0);
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t)
    pool.emplace_back([&, t]() {
      (void)t;
      for (;;) {
        const int y = next.fetch_add(1);
        if (y >= h) break;
        fn(y);
      }
    });
  for (auto& th : pool) th.join();
}

template <class R>
int render_samples(const orc_camera* c, const orc_settings* s, const orc_scene* sc, const orc_env* e,
                   const float* nz, int w, int h, int sample, int threads, float* rgba, int32_t* hits,
                   uint64_t* counters) {
  Tracer<R> T;
  if (!T.setup(c, s, sc, e, nz, w, h)) return -1;
  std::vector<Counters> per_row(h);
  parallel_rows(h, threads, [&](int y) {
    for (int x = 0; x < w; ++x) {
      R out[4];
      const size_t i = (size_t)y * w + x;
      T.trace(x, y, sample, out, hits ? hits + 4 * i : nullptr, per_row[y]);
      for (int k = 0; k < 4; ++k) rgba[4 * i + k] = (float)out[k];
    }
  });
  if (counters) {
    for (int k = 0; k < 8; ++k) counters[k] = 0;
    for (auto& pc : per_row) for (int k = 0; k < 8; ++k) counters[k] += pc.c[k];
  }
  return 0;
}

// Running average of accumulation.fs:10-17: avg = (s + avg * n) / (n + 1).
template <class R>
int render_average(const orc_camera* c, const orc_settings* s, const orc_scene* sc, const orc_env* e,
                   const float* nz, int w, int h, int spp, int threads, int row0, int row1, float* rgba,
                   uint64_t* counters) {
  Tracer<R> T;
  if (!T.setup(c, s, sc, e, nz, w, h)) return -1;
  if (row1 <= 0 || row1 > h) row1 = h;
  if (row0 < 0) row0 = 0;
  const int nrows = std::max(0, row1 - row0);
  std::vector<Counters> per_row(std::max(nrows, 1));
  parallel_rows(nrows, threads, [&](int r) {
    const int y = row0 + r;
    for (int x = 0; x < w; ++x) {
      R avg[4] = {R(0), R(0), R(0), R(0)};
      for (int n = 0; n < spp; ++n) {
        R smp[4];
        T.trace(x, y, n, smp, nullptr, per_row[r]);
        for (int k = 0; k < 4; ++k) avg[k] = (smp[k] + avg[k] * R(n)) / R(n + 1);
      }
      const size_t i = (size_t)y * w + x;
      for (int k = 0; k < 4; ++k) rgba[4 * i + k] = (float)avg[k];
    }
  });
  if (counters) {
    for (int k = 0; k < 8; ++k) counters[k] = 0;
    for (auto& pc : per_row) for (int k = 0; k < 8; ++k) counters[k] += pc.c[k];
  }
  return 0;
}

// ------------------------------------------------------------- env build
// Prefix sums in double: chunk == 0 sums strictly left to right; chunk == 32
// reproduces the GPU's fixed association (in-chunk prefix + chunk offset).
template <class T>
void prefix(const T* in, int n, int chunk, double* out) {
  out[0] = 0.0;
  if (chunk <= 0) {
    double acc = 0.0;
    for (int j = 0; j < n; ++j) { acc = acc + (double)in[j]; out[j + 1] = acc; }
    return;
  }
  const int chunks = (n + chunk - 1) / chunk;
  std::vector<double> offs(chunks, 0.0);
  for (int c = 0; c < chunks; ++c) {
    double acc = 0.0;
    for (int j = c * chunk; j < std::min(n, (c + 1) * chunk); ++j) { acc = acc + (double)in[j]; out[j + 1] = acc; }
  }
  double o = 0.0;
  for (int c = 1; c < chunks; ++c) { o = o + out[c * chunk]; offs[c] = o; }
  for (int c = 1; c < chunks; ++c)
    for (int j = c * chunk; j < std::min(n, (c + 1) * chunk); ++j) out[j + 1] = offs[c] + out[j + 1];
}

// calculateCDF (image.cpp:176-280) with FP64 prefix sums.
void cdf_fp64(const float* func, int w, int h, int chunk, float* cdf_u, float* cdf_v, float* integral) {
  std::vector<double> pre(w + 1), row_int(h), mpre(h + 1);
  for (int y = 0; y < h; ++y) {
    prefix(func + (size_t)y * w, w, chunk, pre.data());
    const double total = pre[w];
    for (int x = 0; x <= w; ++x)
      cdf_u[(size_t)y * (w + 1) + x] = total > 0.0 ? (float)(pre[x] / total) : (float)x / (float)w;
    row_int[y] = total / (double)w;
  }
  prefix(row_int.data(), h, chunk, mpre.data());
  const double total = mpre[h];
  for (int y = 0; y <= h; ++y) cdf_v[y] = total > 0.0 ? (float)(mpre[y] / total) : (float)y / (float)h;
  if (integral) *integral = (float)((total / (double)h) * (2.0 * 3.14159265358979323846 * 3.14159265358979323846));
}

// ------------------------------------------------------------- voxelizer
int sat_int(float f) {
  if (f >= -1.0e9f && f <= 1.0e9f) return (int)f;
  return f > 0.0f ? 1000000000 : -1000000000;
}

// voxelizeTriPostSwizzle after swizzleTri (cpuVoxelizer.cpp:42-235,
// voxelize.gs:55-251), THIN (mode 0) or FAT (mode 1).  The swizzled bounding
// box is clamped to the grid's extent along the swizzled axes, or with
// ref_bounds to the unswizzled resolution as voxelize.gs:247-248 and
// cpuVoxelizer.cpp:265-270 do.
void voxelize_triangle(const float* vv0, const float* vv1, const float* vv2, const int* res_xyz, int mode,
                       bool ref_bounds, uint8_t* grid) {
  const int* res = res_xyz;
  float v0[3] = {vv0[0], vv0[1], vv0[2]}, v1[3] = {vv1[0], vv1[1], vv1[2]}, v2[3] = {vv2[0], vv2[1], vv2[2]};
  // n = cross(v1 - v0, v2 - v1)
  const float a[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
  const float b[3] = {v2[0] - v1[0], v2[1] - v1[1], v2[2] - v1[2]};
  float n[3] = {a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1]};
  const float ax = std::fabs(n[0]), ay = std::fabs(n[1]), az = std::fabs(n[2]);
  int perm;
  auto swz = [](float* p, int i0, int i1, int i2) { const float q0 = p[i0], q1 = p[i1], q2 = p[i2]; p[0] = q0; p[1] = q1; p[2] = q2; };
  if (ax >= ay && ax >= az) { perm = 0; swz(v0, 1, 2, 0); swz(v1, 1, 2, 0); swz(v2, 1, 2, 0); swz(n, 1, 2, 0); }
  else if (ay >= ax && ay >= az) { perm = 1; swz(v0, 2, 0, 1); swz(v1, 2, 0, 1); swz(v2, 2, 0, 1); swz(n, 2, 0, 1); }
  else perm = 2;
  const float* V[3] = {v0, v1, v2};
  int ext[3] = {res[0], res[1], res[2]};
  if (!ref_bounds && perm == 0) { ext[0] = res[1]; ext[1] = res[2]; ext[2] = res[0]; }
  if (!ref_bounds && perm == 1) { ext[0] = res[2]; ext[1] = res[0]; ext[2] = res[1]; }
  // A FAT scan also takes the voxels that only touch the box at an integer
  // bound (ceil(min) - 1 and floor(max) + 1); the reference's floor/ceil
  // range skips them, so a triangle lying in an integer plane marks nothing.
  const bool touch = !ref_bounds && mode == 1;
  int lo[3], hi[3];
  for (int c = 0; c < 3; ++c) {
    const float mn = glmin(glmin(v0[c], v1[c]), v2[c]);
    const float mx = glmax(glmax(v0[c], v1[c]), v2[c]);
    const int l = touch ? sat_int(std::ceil(mn)) - 1 : sat_int(std::floor(mn));
    const int u = touch ? sat_int(std::floor(mx)) + 1 : sat_int(std::ceil(mx));
    lo[c] = std::min(std::max(l, 0), ext[c]);
    hi[c] = std::min(std::max(u, 0), ext[c]);
  }
  float e[3][3];
  for (int c = 0; c < 3; ++c) { e[0][c] = v1[c] - v0[c]; e[1][c] = v2[c] - v1[c]; e[2][c] = v0[c] - v2[c]; }
  float nxy[3][2], nyz[3][2], nzx[3][2], dxy[3], dyz[3], dzx[3];
  auto en = [](float ea, float eb, bool pos, float* o) { if (pos) { o[0] = -eb; o[1] = ea; } else { o[0] = eb; o[1] = -ea; } };
  auto ed = [mode](const float* nn, float pa, float pb) {
    if (mode == 0) return (nn[0] * (0.5f - pa) + nn[1] * (0.5f - pb)) + 0.5f * glmax(std::fabs(nn[0]), std::fabs(nn[1]));
    return (-(nn[0] * pa + nn[1] * pb) + glmax(0.0f, nn[0])) + glmax(0.0f, nn[1]);
  };
  for (int k = 0; k < 3; ++k) {
    en(e[k][0], e[k][1], n[2] >= 0.0f, nxy[k]);
    en(e[k][1], e[k][2], n[0] >= 0.0f, nyz[k]);
    en(e[k][2], e[k][0], n[1] >= 0.0f, nzx[k]);
    dxy[k] = ed(nxy[k], V[k][0], V[k][1]);
    dyz[k] = ed(nyz[k], V[k][1], V[k][2]);
    dzx[k] = ed(nzx[k], V[k][2], V[k][0]);
  }
  float np[3];
  const bool neg = n[2] < 0.0f;
  for (int c = 0; c < 3; ++c) np[c] = neg ? -n[c] : n[c];
  const float dtri = (np[0] * v0[0] + np[1] * v0[1]) + np[2] * v0[2];
  float dmin, dmax;
  if (mode == 0) { dmin = dtri - (np[0] * 0.5f + np[1] * 0.5f); dmax = dmin; }
  else {
    dmin = (dtri - glmax(np[0], 0.0f)) - glmax(np[1], 0.0f);
    dmax = (dtri - glmin(np[0], 0.0f)) - glmin(np[1], 0.0f);
  }
  if (np[2] == 0.0f) return;   // zero-area triangle
  const float nzinv = 1.0f / np[2];
  for (int px = lo[0]; px < hi[0]; ++px) {
    for (int py = lo[1]; py < hi[1]; ++py) {
      bool xy = true;
      for (int k = 0; k < 3; ++k) xy = xy && ((dxy[k] + (nxy[k][0] * (float)px + nxy[k][1] * (float)py)) >= 0.0f);
      if (!xy) continue;
      const float dnp = np[0] * (float)px + np[1] * (float)py;
      const float zmi = (-dnp + dmin) * nzinv, zma = (-dnp + dmax) * nzinv;
      const float zf = std::floor(zmi), zc = std::ceil(zma);
      int zmin = sat_int(zf) - (zf == zmi ? 1 : 0);
      int zmax = sat_int(zc) + (zc == zma ? 1 : 0);
      zmin = std::max(lo[2], zmin);
      zmax = std::min(hi[2], zmax);
      for (int pz = zmin; pz < zmax; ++pz) {
        bool ok = true;
        for (int k = 0; k < 3; ++k) {
          ok = ok && ((dyz[k] + (nyz[k][0] * (float)py + nyz[k][1] * (float)pz)) >= 0.0f);
          ok = ok && ((dzx[k] + (nzx[k][0] * (float)pz + nzx[k][1] * (float)px)) >= 0.0f);
        }
        if (!ok) continue;
        int o[3];
        if (perm == 0) { o[0] = pz; o[1] = px; o[2] = py; }
        else if (perm == 1) { o[0] = py; o[1] = pz; o[2] = px; }
        else { o[0] = px; o[1] = py; o[2] = pz; }
        if (o[0] < 0 || o[1] < 0 || o[2] < 0 || o[0] >= res[0] || o[1] >= res[1] || o[2] >= res[2]) continue;
        grid[(size_t)o[0] + (size_t)res[0] * ((size_t)o[1] + (size_t)res[1] * (size_t)o[2])] = 1;
      }
    }
  }
}

// Separating-axis triangle/box overlap (Akenine-Moller, "Fast 3D
// Triangle-Box Overlap Testing", JGT 2001) for a unit box, in double.
bool tri_box_overlap(const double* c, double h, const double* t0, const double* t1, const double* t2) {
  double v[3][3];
  for (int k = 0; k < 3; ++k) { v[0][k] = t0[k] - c[k]; v[1][k] = t1[k] - c[k]; v[2][k] = t2[k] - c[k]; }
  for (int ax = 0; ax < 3; ++ax) {   // box face normals
    const double mn = std::min(v[0][ax], std::min(v[1][ax], v[2][ax]));
    const double mx = std::max(v[0][ax], std::max(v[1][ax], v[2][ax]));
    if (mn > h || mx < -h) return false;
  }
  double e[3][3];
  for (int k = 0; k < 3; ++k) { e[0][k] = v[1][k] - v[0][k]; e[1][k] = v[2][k] - v[1][k]; e[2][k] = v[0][k] - v[2][k]; }
  double nrm[3] = {e[0][1] * e[1][2] - e[0][2] * e[1][1], e[0][2] * e[1][0] - e[0][0] * e[1][2],
                   e[0][0] * e[1][1] - e[0][1] * e[1][0]};
  {  // triangle plane
    const double d = nrm[0] * v[0][0] + nrm[1] * v[0][1] + nrm[2] * v[0][2];
    const double r = h * (std::fabs(nrm[0]) + std::fabs(nrm[1]) + std::fabs(nrm[2]));
    if (d > r || d < -r) return false;
  }
  for (int i = 0; i < 3; ++i)        // 9 edge cross products
    for (int j = 0; j < 3; ++j) {
      double ax[3] = {0, 0, 0};
      const double u[3] = {j == 0 ? 1.0 : 0.0, j == 1 ? 1.0 : 0.0, j == 2 ? 1.0 : 0.0};
      ax[0] = u[1] * e[i][2] - u[2] * e[i][1];
      ax[1] = u[2] * e[i][0] - u[0] * e[i][2];
      ax[2] = u[0] * e[i][1] - u[1] * e[i][0];
      double p[3];
      for (int k = 0; k < 3; ++k) p[k] = ax[0] * v[k][0] + ax[1] * v[k][1] + ax[2] * v[k][2];
      const double mn = std::min(p[0], std::min(p[1], p[2])), mx = std::max(p[0], std::max(p[1], p[2]));
      const double r = h * (std::fabs(ax[0]) + std::fabs(ax[1]) + std::fabs(ax[2]));
      if (mn > r || mx < -r) return false;
    }
  return true;
}

}  // namespace

// ================================================================ C ABI
extern "C" {

int orc_camera_uniforms(const orc_camera* cam, int32_t w, int32_t h, float* out) {
  float proj[16], ip[16], imv[16], vp[4];
  if (!camera_uniforms<float>(cam, w, h, proj, ip, imv, vp)) return -1;
  std::memcpy(out, proj, 64);
  std::memcpy(out + 16, ip, 64);
  std::memcpy(out + 32, imv, 64);
  std::memcpy(out + 48, vp, 16);
  return 0;
}

void orc_camera_default(orc_camera* cam) {
  std::memset(cam, 0, sizeof(*cam));
  cam->eye[2] = -100.0f;
  cam->near_distance = 0.1f;
  cam->far_distance = 10000.0f;
  cam->focal_distance = 99999999.0f;   // initial value of the focal-distance buffer (renderer.cpp:711-720)
  cam->lens_model = 0;
  cam->fov_y = std::atan2(36.0f * 0.5f, 50.0f) * 2.0f;   // setFocalLength(50) (cameraParameters.cpp:139-150)
}

void orc_camera_orbit(orc_camera* cam, float theta, float phi) {
  const float d[3] = {cam->target[0] - cam->eye[0], cam->target[1] - cam->eye[1], cam->target[2] - cam->eye[2]};
  const float r = std::sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
  const float st = std::sin(theta);
  const float s[3] = {st * std::cos(phi), std::cos(theta), st * std::sin(phi)};
  for (int i = 0; i < 3; ++i) cam->eye[i] = cam->target[i] - r * s[i];
}

void orc_settings_default(orc_settings* s) {
  std::memset(s, 0, sizeof(*s));
  s->max_bounces = 1;
  s->max_samples = 2048 * 2048;
  s->rr_start_bounce = -1;
  s->gamma = 2.2f;
  s->exposure = 1.0f;
  s->nee_emission_scale = 10.0f;
  s->wireframe_thickness = 0.01f;
  s->background_top[0] = 153.0f / 255 * 2; s->background_top[1] = 187.0f / 255 * 2; s->background_top[2] = 201.0f / 255 * 2;
  s->background_bottom[0] = 77.0f / 255; s->background_bottom[1] = 64.0f / 255; s->background_bottom[2] = 50.0f / 255;
  s->quirks = 0xFFu;
}

int orc_render_samples(const orc_camera* cam, const orc_settings* s, const orc_scene* scene, const orc_env* env,
                       const float* noise, int32_t w, int32_t h, int32_t sample, int32_t precision,
                       int32_t threads, float* rgba, int32_t* hits, uint64_t* counters) {
  if (precision == 64) return render_samples<double>(cam, s, scene, env, noise, w, h, sample, threads, rgba, hits, counters);
  return render_samples<float>(cam, s, scene, env, noise, w, h, sample, threads, rgba, hits, counters);
}

int orc_render_average(const orc_camera* cam, const orc_settings* s, const orc_scene* scene, const orc_env* env,
                       const float* noise, int32_t w, int32_t h, int32_t spp, int32_t precision, int32_t threads,
                       int32_t row0, int32_t row1, float* rgba, uint64_t* counters) {
  if (precision == 64)
    return render_average<double>(cam, s, scene, env, noise, w, h, spp, threads, row0, row1, rgba, counters);
  return render_average<float>(cam, s, scene, env, noise, w, h, spp, threads, row0, row1, rgba, counters);
}

int orc_trace_rays(const orc_scene* scene, const float* origins, const float* dirs, int64_t n, uint32_t quirks,
                   int32_t* out) {
  orc_settings s;
  std::memset(&s, 0, sizeof(s));
  s.quirks = quirks;
  s.gamma = 2.2f;
  orc_camera c;
  std::memset(&c, 0, sizeof(c));
  c.eye[2] = -1.0f; c.fov_y = 0.5f; c.near_distance = 0.1f; c.far_distance = 10000.0f;
  Tracer<float> T;
  if (!T.setup(&c, &s, scene, nullptr, nullptr, 1, 1)) return -1;
  Counters C;
  for (int64_t i = 0; i < n; ++i) {
    const V3<float> o = v3<float>(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]);
    const V3<float> d = v3<float>(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
    int vs[3], steps;
    bool ground;
    const bool hit = T.traverse(o, d, vs, &ground, &steps, C);
    int flags = (hit ? 1 : 0) << 8 | (ground ? 1 : 0) << 9 | (steps << 10);
    if (hit) {
      const auto b = T.voxel_basis(vs, o, d);
      flags |= ((int)b.normal.x + 1) | (((int)b.normal.y + 1) << 2) | (((int)b.normal.z + 1) << 4);
    }
    out[4 * i] = vs[0]; out[4 * i + 1] = vs[1]; out[4 * i + 2] = vs[2]; out[4 * i + 3] = flags;
  }
  return 0;
}

int orc_pick(const orc_camera* cam, const orc_settings* s, const orc_scene* scene, const float* noise, int32_t w,
             int32_t h, float x, float y, float* distance, int32_t* voxel) {
  Tracer<float> T;
  if (!T.setup(cam, s, scene, nullptr, noise, w, h)) return -1;
  Counters C;
  Rng rng;
  rng.mode = s->rng_mode; rng.seed = s->seed; rng.noise = noise;
  rng.pixel = 0; rng.sample = 0; rng.call = 0; rng.ox = 0; rng.oy = 0;
  V3<float> o, d;
  T.generate_ray(v3<float>(x, y, 0.0f), rng, &o, &d);
  *distance = 99999999.0f;
  voxel[0] = voxel[1] = voxel[2] = -1;
  const float t = T.aabb(o, d, T.bmin, T.bmax);
  if (t < 0.0f) return 0;
  int vs[3], steps;
  bool ground;
  if (!T.traverse(o + t * d, d, vs, &ground, &steps, C)) return 0;
  const V3<float> vmin = v3<float>((float)vs[0], (float)vs[1], (float)vs[2]) * T.vsize + T.bmin;
  *distance = T.aabb(o, d, vmin, vmin + T.vsize);
  voxel[0] = vs[0]; voxel[1] = vs[1]; voxel[2] = vs[2];
  return 0;
}

void orc_cdf_size(int32_t w, int32_t h, int32_t* cw, int32_t* ch) {
  const unsigned m = (unsigned)std::max(w, h);
  if (m <= 512u) { *cw = w; *ch = h; return; }
  // (unsigned)((float)imageWidth / std::max(imageWidth, imageHeight) * MAX_CDF_SIZE)
  *cw = (int32_t)(unsigned)((float)(unsigned)w / (float)m * 512.0f);
  *ch = (int32_t)(unsigned)((float)(unsigned)h / (float)m * 512.0f);
}

int orc_build_env_ex(const float* rgb, int32_t w, int32_t h, int32_t chunk, uint32_t flags, uint16_t* texels,
                     float* cdf_u, float* cdf_v, float* integral, int32_t* cdf_size) {
  const size_t n = (size_t)w * h;
  std::vector<float> lum(n), tmp(n), func(n);
  std::vector<uint16_t> half(3 * n);
  for (size_t i = 0; i < n; ++i) {
    // texels are stored as IEEE halves, clamped to the finite half range
    const uint16_t r = vtb::f2h(vtb::clamp_half(rgb[3 * i])), g = vtb::f2h(vtb::clamp_half(rgb[3 * i + 1])),
                   b = vtb::f2h(vtb::clamp_half(rgb[3 * i + 2]));
    if (texels) { texels[4 * i] = r; texels[4 * i + 1] = g; texels[4 * i + 2] = b; texels[4 * i + 3] = 0x3c00; }
    half[3 * i] = r; half[3 * i + 1] = g; half[3 * i + 2] = b;
    // channel_sum with Rec.709 weights (image.cpp:326-335)
    lum[i] = (vtb::h2f(r) * 0.2126f + vtb::h2f(g) * 0.7152f) + vtb::h2f(b) * 0.0722f;
  }
  int32_t ow = w, oh = h;
  if (flags & 1u) orc_cdf_size(w, h, &ow, &oh);
  if (ow != w || oh != h) {
    // shrink (image.cpp:308-320): area-weighted average of the texels each
    // output texel covers, in double, rows then columns in index order;
    // then the luminance of the average
    const double sx = (double)w / (double)ow, sy = (double)h / (double)oh;
    for (int oy = 0; oy < oh; ++oy) {
      const double y0 = (double)oy * sy, y1 = (double)(oy + 1) * sy;
      for (int ox = 0; ox < ow; ++ox) {
        const double x0 = (double)ox * sx, x1 = (double)(ox + 1) * sx;
        double acc[3] = {0.0, 0.0, 0.0};
        for (int j = (int)std::floor(y0); j < (int)std::ceil(y1) && j < h; ++j) {
          const double wy = std::min(y1, (double)(j + 1)) - std::max(y0, (double)j);
          for (int i = (int)std::floor(x0); i < (int)std::ceil(x1) && i < w; ++i) {
            const double wx = std::min(x1, (double)(i + 1)) - std::max(x0, (double)i);
            const double wgt = wx * wy;
            for (int c = 0; c < 3; ++c) acc[c] = acc[c] + wgt * (double)vtb::h2f(half[3 * ((size_t)j * w + i) + c]);
          }
        }
        const double area = sx * sy;
        const float fr = (float)(acc[0] / area), fg = (float)(acc[1] / area), fb = (float)(acc[2] / area);
        lum[(size_t)oy * ow + ox] = (fr * 0.2126f + fg * 0.7152f) + fb * 0.0722f;
      }
    }
    w = ow;
    h = oh;
  }
  if (cdf_size) { cdf_size[0] = w; cdf_size[1] = h; }
  // 3x3 Gaussian, sigma 0.75, clamp to edge (image.cpp:337-342)
  const float ws = 0.225610111284051620f, wm = 0.548779777431896800f;
  for (int y = 0; y < h; ++y)
    for (int x = 0; x < w; ++x) {
      const int xm = x > 0 ? x - 1 : 0, xp = x < w - 1 ? x + 1 : w - 1;
      tmp[(size_t)y * w + x] = (ws * lum[(size_t)y * w + xm] + wm * lum[(size_t)y * w + x]) + ws * lum[(size_t)y * w + xp];
    }
  for (int y = 0; y < h; ++y) {
    // sinTheta of calculateImageIntegral (image.cpp:366)
    const float st = (float)std::sin(M_PI * (double)((float)y + 0.5f) / (double)(float)h);
    const int ym = y > 0 ? y - 1 : 0, yp = y < h - 1 ? y + 1 : h - 1;
    for (int x = 0; x < w; ++x) {
      const float v = (ws * tmp[(size_t)ym * w + x] + wm * tmp[(size_t)y * w + x]) + ws * tmp[(size_t)yp * w + x];
      func[(size_t)y * w + x] = glmax(0.0f, v) * st;
    }
  }
  cdf_fp64(func.data(), w, h, chunk, cdf_u, cdf_v, integral);
  return 0;
}

int orc_build_env(const float* rgb, int32_t w, int32_t h, int32_t chunk, uint16_t* texels, float* cdf_u,
                  float* cdf_v, float* integral) {
  return orc_build_env_ex(rgb, w, h, chunk, 0u, texels, cdf_u, cdf_v, integral, nullptr);
}

int orc_cdf_from_function(const float* func, int32_t w, int32_t h, int32_t chunk, float* cdf_u, float* cdf_v,
                          float* integral) {
  cdf_fp64(func, w, h, chunk, cdf_u, cdf_v, integral);
  return 0;
}

// calculateCDF's single-precision recurrences (image.cpp:210-280).
int orc_cdf_reference_float(const float* func, int32_t w, int32_t h, float* cdfU, float* cdfV) {
  const unsigned W = (unsigned)w, H = (unsigned)h;
  std::vector<float> funcV(H + 1);
  const unsigned numStepsW = W;
  for (unsigned y = 0; y < H; ++y) {
    const unsigned row = y * (W + 1);
    cdfU[row] = 0.0f;
    for (unsigned x = 1; x <= W; ++x) cdfU[row + x] = cdfU[row + x - 1] + func[y * W + x - 1] / (float)numStepsW;
    const float rowIntegral = cdfU[row + W];
    funcV[y] = rowIntegral;
    if (rowIntegral > 0.0f) for (unsigned x = 1; x <= W; ++x) cdfU[row + x] /= rowIntegral;
    else for (unsigned x = 1; x <= W; ++x) cdfU[row + x] = (float)x / (float)numStepsW;
  }
  cdfV[0] = 0.0f;
  for (unsigned y = 1; y <= H; ++y) cdfV[y] = cdfV[y - 1] + funcV[y - 1] / (float)H;
  const float integral = cdfV[H];
  if (integral > 0.0f) for (unsigned y = 1; y <= H; ++y) cdfV[y] /= integral;
  else for (unsigned y = 1; y <= H; ++y) cdfV[y] = (float)y / (float)H;
  return 0;
}

int32_t orc_binary_search(const float* cdf, int32_t n, float u) {
  Counters C;
  return Tracer<float>::search(cdf, n - 1, u, C);
}

int orc_voxelize(const float* vertices, int64_t nv, const uint32_t* indices, int64_t nt, int32_t rx, int32_t ry,
                 int32_t rz, int32_t mode, int32_t placement, int32_t threads, uint8_t* grid) {
  const int res[3] = {rx, ry, rz};
  std::vector<float> vs(vertices, vertices + 3 * nv);
  if (placement == 1 && nv > 0) {
    // computeMeshTransform (import.cpp:46-64) + modelTransform * v * res (voxelize.vs:20-27)
    float bmin[3] = {INFINITY, INFINITY, INFINITY}, bmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int64_t i = 0; i < nv; ++i)
      for (int c = 0; c < 3; ++c) { bmin[c] = std::min(bmin[c], vertices[3 * i + c]); bmax[c] = std::max(bmax[c], vertices[3 * i + c]); }
    float size[3], margin[3];
    for (int c = 0; c < 3; ++c) { size[c] = bmax[c] - bmin[c]; margin[c] = 1.0f / (float)res[c]; }
    int major = 0;
    if (size[1] > size[major]) major = 1;
    if (size[2] > size[major]) major = 2;
    const float s = (float)((1.0f - 2.0 * (double)margin[major]) / (double)size[major]);
    float t[3];
    for (int c = 0; c < 3; ++c) t[c] = -bmin[c] + margin[c] / s;
    const float Mx[16] = {s, 0, 0, t[0] * s, 0, s, 0, t[1] * s, 0, 0, s, t[2] * s, 0, 0, 0, 1.0f};
    for (int64_t i = 0; i < nv; ++i) {
      const float x = vertices[3 * i], y = vertices[3 * i + 1], z = vertices[3 * i + 2];
      for (int r = 0; r < 3; ++r)
        vs[3 * i + r] = (((Mx[4 * r] * x + Mx[4 * r + 1] * y) + Mx[4 * r + 2] * z) + Mx[4 * r + 3] * 1.0f) * (float)res[r];
    }
  }
  std::memset(grid, 0, (size_t)rx * ry * rz);
  // Triangles are independent and only ever write 1, so any partition of the
  // triangle list gives the same grid (the reference's CPU twin splits it in
  // overlapping ranges, cpuVoxelizer.cpp:281-303).
  const int T = threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency());
  std::atomic<int64_t> next(0);
  std::vector<std::thread> pool;
  for (int t = 0; t < T; ++t)
    pool.emplace_back([&]() {
      for (;;) {
        const int64_t b = next.fetch_add(4096);
        if (b >= nt) break;
        for (int64_t k = b; k < std::min(nt, b + 4096); ++k)
          voxelize_triangle(&vs[3 * (size_t)indices[3 * k]], &vs[3 * (size_t)indices[3 * k + 1]],
                            &vs[3 * (size_t)indices[3 * k + 2]], res, mode & 1, (mode & 0x100) != 0, grid);
      }
    });
  for (auto& th : pool) th.join();
  return 0;
}

int orc_voxelize_sat(const float* v, int64_t nv, const uint32_t* idx, int64_t nt, int32_t rx, int32_t ry, int32_t rz,
                     double half, uint8_t* grid) {
  (void)nv;
  std::memset(grid, 0, (size_t)rx * ry * rz);
  for (int64_t t = 0; t < nt; ++t) {
    double p[3][3];
    for (int k = 0; k < 3; ++k)
      for (int c = 0; c < 3; ++c) p[k][c] = v[3 * (size_t)idx[3 * t + k] + c];
    int lo[3], hi[3];
    const int res[3] = {rx, ry, rz};
    for (int c = 0; c < 3; ++c) {
      const double mn = std::min(p[0][c], std::min(p[1][c], p[2][c]));
      const double mx = std::max(p[0][c], std::max(p[1][c], p[2][c]));
      lo[c] = std::max(0, (int)std::floor(mn) - 1);
      hi[c] = std::min(res[c], (int)std::ceil(mx) + 1);
    }
    for (int z = lo[2]; z < hi[2]; ++z)
      for (int y = lo[1]; y < hi[1]; ++y)
        for (int x = lo[0]; x < hi[0]; ++x) {
          const double c[3] = {x + 0.5, y + 0.5, z + 0.5};
          if (tri_box_overlap(c, half, p[0], p[1], p[2])) grid[(size_t)x + (size_t)rx * ((size_t)y + (size_t)ry * z)] = 1;
        }
  }
  return 0;
}

int64_t orc_prune_emissive(const uint8_t* grid, const int32_t* res, int32_t* list, int64_t n) {
  // anyVisibleFace / occupiedNeightbour (import.cpp:133-178), swap-with-last removal (:180-203)
  auto occupied = [&](int x, int y, int z) {
    if (x < 0 || x >= res[0] || y < 0 || y >= res[1] || z < 0 || z >= res[2]) return false;
    return grid[(size_t)x + (size_t)res[0] * ((size_t)y + (size_t)res[1] * z)] != 0;
  };
  const int off[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
  for (int64_t i = 0; i < n; ++i) {
    int v = list[i];
    const int z = v / (res[0] * res[1]);
    v -= z * res[0] * res[1];
    const int y = v / res[0];
    const int x = v - y * res[0];
    bool visible = false;
    for (int k = 0; k < 6; ++k) visible = visible || !occupied(x + off[k][0], y + off[k][1], z + off[k][2]);
    if (!visible) { list[i] = list[n - 1]; --n; --i; }
  }
  return n;
}

int orc_noise_table(float* out) {
  for (size_t i = 0; i < (size_t)1024 * 1024 * 4; ++i) out[i] = (float)(splitmix64((uint64_t)i) >> 40) * 5.9604644775390625e-8f;
  return 0;
}

void orc_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { philox4x32(ctr, key, out); }

namespace {
Tracer<float> unit_tracer(const orc_settings* s, const orc_env* env, float rotation) {
  Tracer<float> T;
  T.S = s; T.env = env; T.scene = nullptr; T.noise = nullptr;
  T.bg_rot = rotation;
  T.bg_top = v3<float>(0.0f, 0.0f, 0.0f); T.bg_bottom = T.bg_top;
  return T;
}
Mat unit_material(int32_t type, const float* albedo, float rough) {
  Mat m;
  m.type = type;
  for (int k = 0; k < 3; ++k) { m.e[k] = 0.0f; m.a[k] = q16(albedo[k]); }
  m.rough = q16(rough);
  return m;
}
}  // namespace

int orc_bsdf_sample(int32_t type, const float* albedo, float rough, uint32_t quirks, const float* wo,
                    const float* u, int64_t n, float* out) {
  orc_settings s;
  std::memset(&s, 0, sizeof(s));
  s.quirks = quirks;
  const Tracer<float> T = unit_tracer(&s, nullptr, 0.0f);
  const Mat m = unit_material(type, albedo, rough);
  for (int64_t i = 0; i < n; ++i) {
    // the noise-table stream reads its block from u: one rand() call
    const float block[4] = {u[2 * i], u[2 * i + 1], 0.0f, 0.0f};
    Rng rng;
    rng.mode = 1; rng.noise = block; rng.ox = 0; rng.oy = 0;
    Tracer<float>::FP fp;
    float u_rr;
    const V3<float> w = T.sample_bsdf(m, v3<float>(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), rng, fp, u_rr);
    float* o = out + 8 * i;
    o[0] = w.x; o[1] = w.y; o[2] = w.z; o[3] = fp.f.x; o[4] = fp.f.y; o[5] = fp.f.z; o[6] = fp.pdf; o[7] = 0.0f;
  }
  return 0;
}

int orc_bsdf_eval(int32_t type, const float* albedo, float rough, uint32_t quirks, const float* wo,
                  const float* wi, int64_t n, float* out) {
  orc_settings s;
  std::memset(&s, 0, sizeof(s));
  s.quirks = quirks;
  const Tracer<float> T = unit_tracer(&s, nullptr, 0.0f);
  const Mat m = unit_material(type, albedo, rough);
  for (int64_t i = 0; i < n; ++i) {
    const Tracer<float>::FP fp = T.eval_bsdf(m, v3<float>(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]),
                                             v3<float>(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]));
    float* o = out + 4 * i;
    o[0] = fp.f.x; o[1] = fp.f.y; o[2] = fp.f.z; o[3] = fp.pdf;
  }
  return 0;
}

int orc_env_sample(const orc_env* env, float rotation, const float* u, int64_t n, float* out) {
  if (!env || !env->texels) return -1;
  orc_settings s;
  std::memset(&s, 0, sizeof(s));
  const Tracer<float> T = unit_tracer(&s, env, rotation);
  Tracer<float>::Basis b;
  b.position = v3<float>(0.0f, 0.0f, 0.0f); b.normal = v3<float>(0.0f, 1.0f, 0.0f);
  b.tangent = v3<float>(1.0f, 0.0f, 0.0f); b.binormal = v3<float>(0.0f, 0.0f, 1.0f);
  Counters C;
  for (int64_t i = 0; i < n; ++i) {
    V3<float> d;
    float pdf;
    const V3<float> L = T.sample_env(b, u[2 * i], u[2 * i + 1], &d, &pdf, C);
    float* o = out + 8 * i;
    o[0] = d.x; o[1] = d.y; o[2] = d.z; o[3] = L.x; o[4] = L.y; o[5] = L.z; o[6] = pdf; o[7] = 0.0f;
  }
  return 0;
}

int orc_env_eval(const orc_env* env, float rotation, const float* dirs, int64_t n, float* out) {
  if (!env || !env->texels) return -1;
  orc_settings s;
  std::memset(&s, 0, sizeof(s));
  const Tracer<float> T = unit_tracer(&s, env, rotation);
  Counters C;
  for (int64_t i = 0; i < n; ++i) {
    float pdf = 0.0f;
    const V3<float> L = T.eval_env(v3<float>(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]), &pdf, C);
    float* o = out + 4 * i;
    o[0] = L.x; o[1] = L.y; o[2] = L.z; o[3] = pdf;
  }
  return 0;
}

int orc_noise_walk(const float* noise, int32_t px, int32_t py, int32_t sample, int32_t n, float* out) {
  Rng rng;
  rng.init(1, 0u, noise, 1, px, py, sample);
  for (int32_t i = 0; i < n; ++i) rng.next(out + 4 * (size_t)i);
  return 0;
}

int orc_generate_rays(const orc_camera* cam, const orc_settings* s, int32_t w, int32_t h, const float* frag,
                      const float* u, int64_t n, float* out) {
  const uint8_t cell = 0;
  orc_material m;
  std::memset(&m, 0, sizeof(m));
  orc_scene sc;
  sc.res[0] = sc.res[1] = sc.res[2] = 1;
  sc.grid = &cell; sc.palette = &m; sc.n_palette = 1; sc.emissive = nullptr; sc.n_emissive = 0;
  Tracer<float> T;
  if (!T.setup(cam, s, &sc, nullptr, nullptr, w, h)) return -1;
  for (int64_t i = 0; i < n; ++i) {
    Rng rng;
    rng.mode = 1; rng.noise = u + 4 * i; rng.ox = 0; rng.oy = 0;
    V3<float> o, d;
    T.generate_ray(v3<float>(frag[2 * i], frag[2 * i + 1], T.frag_z), rng, &o, &d);
    float* r = out + 6 * i;
    r[0] = o.x; r[1] = o.y; r[2] = o.z; r[3] = d.x; r[4] = d.y; r[5] = d.z;
  }
  return 0;
}

int orc_builtins(int32_t fn, const float* a, const float* b, float* out, int64_t n) {
  for (int64_t i = 0; i < n; ++i) {
    const float x = a[i];
    switch (fn) {
      case 0: out[i] = vtb::vsin(x); break;
      case 1: out[i] = vtb::vcos(x); break;
      case 2: out[i] = vtb::vpow(x, b[i]); break;
      case 3: out[i] = vtb::vacos(x); break;
      case 4: out[i] = vtb::vatan2(x, b[i]); break;
      case 5: out[i] = vtb::vlog2(x); break;
      case 6: out[i] = vtb::vexp2(x); break;
      case 7: out[i] = vtb::h2f(vtb::f2h(x)); break;
      default: return -1;
    }
  }
  return 0;
}

}  // extern "C"
