// vt_io.cu — file formats on the path's edges, host code only:
//   MagicaVoxel .vox   -> dense palette grid + Lambert palette
//                         (MagicaVoxelLoader::load, magicaVoxel.cpp:122-321)
//   Wavefront OBJ      -> triangle soup for the voxelizer
//                         (MeshLoader::loadFromOBJ, meshLoader.cpp:11-74)
//   PFM / Radiance HDR -> float RGB images (environment maps, readback)
// Decoders take bytes already in memory, so they run without a GPU; the
// scene entry points hand their output to vt_scene_create /
// vt_scene_voxelize_mesh.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "vt_runtime.h"

using namespace vt;

namespace {

// ------------------------------------------------------------------- .vox
uint32_t rd32(const uint8_t* p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
constexpr uint32_t fourcc(char a, char b, char c, char d) {
  return (uint32_t)(uint8_t)a | ((uint32_t)(uint8_t)b << 8) | ((uint32_t)(uint8_t)c << 16) |
         ((uint32_t)(uint8_t)d << 24);
}

// MagicaVoxel's default palette, entry k as RGB: entry 0 unused; 1..215 the
// 6x6x6 cube of channel values 255, 204, ..., 0 (red slowest, blue fastest)
// without black; 216..255 ramps of red, green, blue and grey through
// 238, 221, 187, 170, 136, 119, 85, 68, 34, 17.
void default_palette(uint8_t rgb[256][3]) {
  memset(rgb, 0, 256 * 3);
  int k = 1;
  for (int r = 0; r < 6; ++r)
    for (int g = 0; g < 6; ++g)
      for (int b = 0; b < 6; ++b) {
        if (r == 5 && g == 5 && b == 5) continue;
        rgb[k][0] = (uint8_t)(255 - 51 * r);
        rgb[k][1] = (uint8_t)(255 - 51 * g);
        rgb[k][2] = (uint8_t)(255 - 51 * b);
        ++k;
      }
  const uint8_t ramp[10] = {238, 221, 187, 170, 136, 119, 85, 68, 34, 17};
  for (int c = 0; c < 4; ++c)
    for (int i = 0; i < 10; ++i, ++k) {
      if (c == 3) rgb[k][0] = rgb[k][1] = rgb[k][2] = ramp[i];
      else rgb[k][c] = ramp[i];
    }
}

struct VoxModel {
  int32_t sx = 0, sy = 0, sz = 0;
  std::vector<uint8_t> xyzi;   // 4 bytes per voxel
  bool custom = false;
  uint8_t pal[256][3];
};

int vox_parse(const uint8_t* d, size_t n, VoxModel& m) {
  if (!d || n < 20) return fail(VT_EINVAL, ".vox: too short");
  if (rd32(d) != fourcc('V', 'O', 'X', ' ')) return fail(VT_EINVAL, ".vox: magic number does not match");
  const uint32_t version = rd32(d + 4);
  if (version != 150 && version != 200) return fail(VT_EINVAL, ".vox: version %u is not 150 or 200", version);
  if (rd32(d + 8) != fourcc('M', 'A', 'I', 'N')) return fail(VT_EINVAL, ".vox: main chunk is not found");
  const uint64_t main_content = rd32(d + 12), main_children = rd32(d + 16);
  size_t pos = 20 + main_content;
  const uint64_t end64 = 20 + main_content + main_children;
  const size_t end = (size_t)std::min<uint64_t>(end64, n);
  default_palette(m.pal);
  while (pos + 12 <= end) {
    const uint32_t id = rd32(d + pos);
    const uint64_t content = rd32(d + pos + 4), children = rd32(d + pos + 8);
    const size_t body = pos + 12;
    if (body + content > n) return fail(VT_EINVAL, ".vox: chunk runs past the end of the data");
    if (id == fourcc('S', 'I', 'Z', 'E')) {
      if (content < 12) return fail(VT_EINVAL, ".vox: short SIZE chunk");
      m.sx = (int32_t)rd32(d + body); m.sy = (int32_t)rd32(d + body + 4); m.sz = (int32_t)rd32(d + body + 8);
    } else if (id == fourcc('X', 'Y', 'Z', 'I')) {
      if (content < 4) return fail(VT_EINVAL, ".vox: short XYZI chunk");
      const int64_t nv = (int32_t)rd32(d + body);
      if (nv < 0) return fail(VT_EINVAL, ".vox: negative number of voxels");
      if ((uint64_t)nv * 4 + 4 > content) return fail(VT_EINVAL, ".vox: XYZI chunk shorter than its voxel count");
      m.xyzi.assign(d + body + 4, d + body + 4 + 4 * (size_t)nv);
    } else if (id == fourcc('R', 'G', 'B', 'A')) {
      if (content < 1024) return fail(VT_EINVAL, ".vox: short RGBA chunk");
      // file entries 0..254 are colour indices 1..255; the 256th is reserved
      m.custom = true;
      for (int i = 0; i < 255; ++i)
        for (int c = 0; c < 3; ++c) m.pal[i + 1][c] = d[body + 4 * i + c];
    }
    pos = body + content + children;   // skip the rest of the chunk and its children
  }
  if (m.sx <= 0 || m.sy <= 0 || m.sz <= 0) return fail(VT_EINVAL, ".vox: no SIZE chunk");
  return VT_OK;
}

// ------------------------------------------------------------------- OBJ
const char* skip_ws(const char* p, const char* e) {
  while (p < e && (*p == ' ' || *p == '\t' || *p == '\r')) ++p;
  return p;
}

// One "v/vt/vn" reference of a face; returns the position index (1-based or
// negative) and advances p, or 0 on a malformed token.
long face_ref(const char*& p, const char* e) {
  char* q = nullptr;
  const long v = strtol(p, &q, 10);
  if (q == p) return 0;
  p = q;
  while (p < e && *p != ' ' && *p != '\t' && *p != '\r' && *p != '\n') ++p;   // skip /vt/vn
  return v;
}

int obj_parse(const char* text, size_t n, std::vector<float>& v, std::vector<uint32_t>& idx) {
  const char* p = text;
  const char* e = text + n;
  int64_t line = 0;
  while (p < e) {
    const char* eol = (const char*)memchr(p, '\n', (size_t)(e - p));
    if (!eol) eol = e;
    ++line;
    const char* s = skip_ws(p, eol);
    if (s + 1 < eol && s[0] == 'v' && (s[1] == ' ' || s[1] == '\t')) {
      std::string tok(s + 1, eol);
      float x, y, z;
      if (sscanf(tok.c_str(), "%f %f %f", &x, &y, &z) != 3)
        return fail(VT_EINVAL, "OBJ line %lld: vertex needs three coordinates", (long long)line);
      v.push_back(x); v.push_back(y); v.push_back(z);
    } else if (s + 1 < eol && s[0] == 'f' && (s[1] == ' ' || s[1] == '\t')) {
      const char* q = s + 1;
      std::vector<long> refs;
      for (;;) {
        q = skip_ws(q, eol);
        if (q >= eol) break;
        const long r = face_ref(q, eol);
        if (r == 0) return fail(VT_EINVAL, "OBJ line %lld: bad face index", (long long)line);
        const long nvert = (long)(v.size() / 3);
        const long i0 = r > 0 ? r - 1 : nvert + r;   // negative: relative to the vertices so far
        if (i0 < 0 || i0 >= nvert)
          return fail(VT_EINVAL, "OBJ line %lld: face index %ld out of range", (long long)line, r);
        refs.push_back(i0);
      }
      if (refs.size() < 3) return fail(VT_EINVAL, "OBJ line %lld: face with fewer than 3 vertices", (long long)line);
      for (size_t k = 1; k + 1 < refs.size(); ++k) {   // fan triangulation
        idx.push_back((uint32_t)refs[0]);
        idx.push_back((uint32_t)refs[k]);
        idx.push_back((uint32_t)refs[k + 1]);
      }
    }
    p = eol + 1;
  }
  return VT_OK;
}

// ------------------------------------------------------------------ images
bool read_token(const uint8_t*& p, const uint8_t* e, std::string& out) {
  while (p < e && isspace(*p)) ++p;
  out.clear();
  while (p < e && !isspace(*p)) out.push_back((char)*p++);
  return !out.empty();
}

int decode_pfm(const uint8_t* d, size_t n, std::vector<float>& rgb, int32_t& w, int32_t& h) {
  const uint8_t* p = d;
  const uint8_t* e = d + n;
  std::string t, sw, sh, ss;
  if (!read_token(p, e, t) || (t != "PF" && t != "Pf")) return fail(VT_EINVAL, "PFM: bad header");
  if (!read_token(p, e, sw) || !read_token(p, e, sh) || !read_token(p, e, ss)) return fail(VT_EINVAL, "PFM: bad header");
  if (p >= e) return fail(VT_EINVAL, "PFM: no pixel data");
  ++p;   // the single whitespace byte after the scale
  w = atoi(sw.c_str());
  h = atoi(sh.c_str());
  const double scale = atof(ss.c_str());
  const int ch = t == "PF" ? 3 : 1;
  if (w <= 0 || h <= 0 || scale == 0.0) return fail(VT_EINVAL, "PFM: bad size or scale");
  const size_t need = (size_t)w * h * ch * 4;
  if ((size_t)(e - p) < need) return fail(VT_EINVAL, "PFM: %zu pixel bytes, %zu needed", (size_t)(e - p), need);
  const bool little = scale < 0.0;
  rgb.resize((size_t)w * h * 3);
  for (int32_t y = 0; y < h; ++y)          // PFM rows run bottom to top
    for (int32_t x = 0; x < w; ++x)
      for (int c = 0; c < 3; ++c) {
        const uint8_t* b = p + (((size_t)y * w + x) * ch + (ch == 3 ? c : 0)) * 4;
        const uint32_t u = little ? rd32(b)
                                  : ((uint32_t)b[3] | ((uint32_t)b[2] << 8) | ((uint32_t)b[1] << 16) |
                                     ((uint32_t)b[0] << 24));
        float f;
        memcpy(&f, &u, 4);
        rgb[(((size_t)(h - 1 - y)) * w + x) * 3 + c] = f;
      }
  return VT_OK;
}

// Radiance RGBE (Greg Ward's .hdr): header lines, a blank line, the
// resolution line "-Y h +X w", then scanlines flat or new-style run-length
// encoded (four channel planes of runs).
float rgbe_channel(uint8_t m, uint8_t ex) {
  if (ex == 0) return 0.0f;
  return (float)ldexp((double)m + 0.5, (int)ex - (128 + 8));
}

int decode_hdr(const uint8_t* d, size_t n, std::vector<float>& rgb, int32_t& w, int32_t& h) {
  const uint8_t* p = d;
  const uint8_t* e = d + n;
  auto line = [&](std::string& s) {
    s.clear();
    while (p < e && *p != '\n') s.push_back((char)*p++);
    if (p < e) ++p;
    return true;
  };
  std::string s;
  line(s);
  if (s.rfind("#?", 0) != 0) return fail(VT_EINVAL, "HDR: missing #? signature");
  for (;;) {
    if (p >= e) return fail(VT_EINVAL, "HDR: header does not end");
    line(s);
    if (s.empty()) break;
    if (s.rfind("FORMAT=", 0) == 0 && s != "FORMAT=32-bit_rle_rgbe") return fail(VT_EINVAL, "HDR: format %s", s.c_str());
  }
  line(s);
  char ya[3] = {0}, xa[3] = {0};
  if (sscanf(s.c_str(), "%2s %d %2s %d", ya, &h, xa, &w) != 4 || std::string(ya) != "-Y" || std::string(xa) != "+X")
    return fail(VT_EINVAL, "HDR: only -Y h +X w images are read");
  if (w <= 0 || h <= 0) return fail(VT_EINVAL, "HDR: bad size");
  rgb.resize((size_t)w * h * 3);
  std::vector<uint8_t> scan((size_t)w * 4);
  for (int32_t y = 0; y < h; ++y) {
    if (e - p >= 4 && p[0] == 2 && p[1] == 2 && ((p[2] << 8) | p[3]) == w && w >= 8 && w < 32768) {
      p += 4;
      for (int c = 0; c < 4; ++c) {
        int32_t x = 0;
        while (x < w) {
          if (p >= e) return fail(VT_EINVAL, "HDR: scanline %d truncated", y);
          int count = *p++;
          if (count > 128) {
            count -= 128;
            if (p >= e || x + count > w) return fail(VT_EINVAL, "HDR: bad run in scanline %d", y);
            const uint8_t v = *p++;
            for (int k = 0; k < count; ++k) scan[(size_t)(x++) * 4 + c] = v;
          } else {
            if (count == 0 || x + count > w || e - p < count) return fail(VT_EINVAL, "HDR: bad run in scanline %d", y);
            for (int k = 0; k < count; ++k) scan[(size_t)(x++) * 4 + c] = *p++;
          }
        }
      }
    } else {
      if ((size_t)(e - p) < (size_t)w * 4) return fail(VT_EINVAL, "HDR: scanline %d truncated", y);
      memcpy(scan.data(), p, (size_t)w * 4);
      p += (size_t)w * 4;
    }
    for (int32_t x = 0; x < w; ++x)
      for (int c = 0; c < 3; ++c)
        rgb[((size_t)y * w + x) * 3 + c] = rgbe_channel(scan[(size_t)x * 4 + c], scan[(size_t)x * 4 + 3]);
  }
  return VT_OK;
}

}  // namespace

// ---------------------------------------------------------------- C ABI
extern "C" int vt_vox_decode(const uint8_t* data, size_t size, int32_t res[3], uint8_t* voxels, size_t voxels_bytes,
                             vt_material* palette, int32_t* n_palette) {
  if (!res || !n_palette) return fail(VT_EINVAL, "null argument");
  VoxModel m;
  int rc = vox_parse(data, size, m);
  if (rc != VT_OK) return rc;
  // reference axes: x, y = file z, z = file y (magicaVoxel.cpp:267-269)
  res[0] = m.sx; res[1] = m.sz; res[2] = m.sy;
  const size_t nvox = (size_t)m.sx * m.sy * m.sz;
  // palette entries in order of first use, as the reference appends materials
  int entry_of[256];
  for (int i = 0; i < 256; ++i) entry_of[i] = -1;
  int n_used = 0;
  const size_t count = m.xyzi.size() / 4;
  for (size_t i = 0; i < count; ++i) {
    const uint8_t* v = &m.xyzi[4 * i];
    if (v[3] == 254) continue;   // the reference treats colour index 254 as empty
    if (v[0] >= m.sx || v[1] >= m.sy || v[2] >= m.sz)
      return fail(VT_EINVAL, ".vox: voxel %zu at (%d, %d, %d) lies outside the %dx%dx%d model", i, v[0], v[1], v[2],
                  m.sx, m.sy, m.sz);
    if (entry_of[v[3]] < 0) entry_of[v[3]] = n_used++;
  }
  *n_palette = n_used;
  if (!voxels && !palette) return VT_OK;   // size query
  if (!voxels || voxels_bytes < nvox) return fail(VT_EINVAL, "voxel buffer smaller than %zu bytes", nvox);
  memset(voxels, 0, nvox);
  for (size_t i = 0; i < count; ++i) {
    const uint8_t* v = &m.xyzi[4 * i];
    if (v[3] == 254) continue;
    const size_t at = (size_t)v[0] + (size_t)v[2] * m.sx + (size_t)v[1] * m.sx * m.sz;
    voxels[at] = (uint8_t)(entry_of[v[3]] + 1);
  }
  if (palette) {
    for (int c = 0; c < 256; ++c) {
      if (entry_of[c] < 0) continue;
      vt_material& mt = palette[entry_of[c]];
      mt.type = VT_MATERIAL_LAMBERT;
      mt.emission[0] = mt.emission[1] = mt.emission[2] = 0.0f;
      for (int k = 0; k < 3; ++k) mt.albedo[k] = (float)m.pal[c][k] / 255.0f;
      mt.roughness = 0.0f;
    }
  }
  return VT_OK;
}

extern "C" int vt_scene_create_from_vox(vt_context* ctx, const uint8_t* data, size_t size, uint32_t flags,
                                        vt_scene** out) {
  if (!ctx || !out) return fail(VT_EINVAL, "null argument");
  int32_t res[3], n_pal = 0;
  int rc = vt_vox_decode(data, size, res, nullptr, 0, nullptr, &n_pal);
  if (rc != VT_OK) return rc;
  if (n_pal == 0) return fail(VT_EINVAL, ".vox: the model has no voxels");
  std::vector<uint8_t> vox((size_t)res[0] * res[1] * res[2]);
  std::vector<vt_material> pal((size_t)n_pal);
  rc = vt_vox_decode(data, size, res, vox.data(), vox.size(), pal.data(), &n_pal);
  if (rc != VT_OK) return rc;
  return vt_scene_create(ctx, res[0], res[1], res[2], vox.data(), pal.data(), n_pal, nullptr, 0, flags, out);
}

extern "C" int vt_obj_decode(const char* text, size_t size, float* vertices, int64_t vertex_capacity,
                             uint32_t* indices, int64_t triangle_capacity, int64_t* n_vertices, int64_t* n_triangles) {
  if (!text || !n_vertices || !n_triangles) return fail(VT_EINVAL, "null argument");
  std::vector<float> v;
  std::vector<uint32_t> idx;
  int rc = obj_parse(text, size, v, idx);
  if (rc != VT_OK) return rc;
  *n_vertices = (int64_t)(v.size() / 3);
  *n_triangles = (int64_t)(idx.size() / 3);
  if (!vertices && !indices) return VT_OK;   // size query
  if (!vertices || !indices || vertex_capacity < *n_vertices || triangle_capacity < *n_triangles)
    return fail(VT_EINVAL, "output buffers too small (%lld vertices, %lld triangles)", (long long)*n_vertices,
                (long long)*n_triangles);
  memcpy(vertices, v.data(), v.size() * sizeof(float));
  memcpy(indices, idx.data(), idx.size() * sizeof(uint32_t));
  return VT_OK;
}

extern "C" int vt_scene_voxelize_obj(vt_context* ctx, const char* text, size_t size, int32_t rx, int32_t ry,
                                     int32_t rz, int32_t mode, int32_t placement, const vt_material* palette,
                                     int32_t n_palette, vt_scene** out) {
  if (!ctx || !text || !out) return fail(VT_EINVAL, "null argument");
  std::vector<float> v;
  std::vector<uint32_t> idx;
  int rc = obj_parse(text, size, v, idx);
  if (rc != VT_OK) return rc;
  if (idx.empty()) return fail(VT_EINVAL, "OBJ: no faces");
  return vt_scene_voxelize_mesh(ctx, v.data(), (int64_t)(v.size() / 3), idx.data(), (int64_t)(idx.size() / 3), rx, ry,
                                rz, mode, placement, palette, n_palette, out);
}

extern "C" int vt_image_decode(const uint8_t* data, size_t size, float* rgb, size_t rgb_bytes, int32_t* width,
                               int32_t* height) {
  if (!data || !width || !height) return fail(VT_EINVAL, "null argument");
  std::vector<float> img;
  int32_t w = 0, h = 0;
  int rc;
  if (size >= 2 && data[0] == 'P' && (data[1] == 'F' || data[1] == 'f')) rc = decode_pfm(data, size, img, w, h);
  else if (size >= 2 && data[0] == '#' && data[1] == '?') rc = decode_hdr(data, size, img, w, h);
  else return fail(VT_EINVAL, "image: neither PFM nor Radiance HDR");
  if (rc != VT_OK) return rc;
  *width = w;
  *height = h;
  if (!rgb) return VT_OK;   // size query
  if (rgb_bytes < img.size() * sizeof(float)) return fail(VT_EINVAL, "output buffer smaller than %zu bytes",
                                                          img.size() * sizeof(float));
  memcpy(rgb, img.data(), img.size() * sizeof(float));
  return VT_OK;
}

extern "C" int vt_image_encode_pfm(const float* pixels, int32_t width, int32_t height, int32_t channels,
                                   uint8_t* out, size_t out_bytes, size_t* written) {
  if (!pixels || !written || width <= 0 || height <= 0 || (channels != 3 && channels != 4))
    return fail(VT_EINVAL, "bad argument");
  char head[64];
  const int hl = snprintf(head, sizeof(head), "PF\n%d %d\n-1.0\n", width, height);
  const size_t need = (size_t)hl + (size_t)width * height * 12;
  *written = need;
  if (!out) return VT_OK;   // size query
  if (out_bytes < need) return fail(VT_EINVAL, "output buffer smaller than %zu bytes", need);
  memcpy(out, head, (size_t)hl);
  uint8_t* o = out + hl;
  for (int32_t y = 0; y < height; ++y)     // rows bottom first, in memory and in the file
    for (int32_t x = 0; x < width; ++x)
      for (int c = 0; c < 3; ++c) {
        const float f = pixels[((size_t)y * width + x) * channels + c];
        uint32_t u;
        memcpy(&u, &f, 4);
        o[0] = (uint8_t)u; o[1] = (uint8_t)(u >> 8); o[2] = (uint8_t)(u >> 16); o[3] = (uint8_t)(u >> 24);
        o += 4;
      }
  return VT_OK;
}

// Radiance RGBE (Ward, "Real Pixels", Graphics Gems II, 1991): the shared
// exponent of the largest channel, each channel's mantissa scaled to 8 bits.
// Negative and NaN channels are written as 0; infinities as the largest value.
static void to_rgbe(float r, float g, float b, uint8_t* o) {
  const float big = 1.0e38f;   // below 2^127, the largest shared exponent a byte holds
  auto clean = [big](float v) { return v > 0.0f ? (v < big ? v : big) : 0.0f; };   // NaN fails v > 0
  r = clean(r); g = clean(g); b = clean(b);
  const float v = std::max(r, std::max(g, b));
  if (v < 1e-32f) { o[0] = o[1] = o[2] = o[3] = 0; return; }
  int e = 0;
  const double m = std::frexp((double)v, &e);   // v = m * 2^e, m in [0.5, 1)
  const double scale = m * 256.0 / (double)v;
  o[0] = (uint8_t)std::min(255.0, (double)r * scale);
  o[1] = (uint8_t)std::min(255.0, (double)g * scale);
  o[2] = (uint8_t)std::min(255.0, (double)b * scale);
  o[3] = (uint8_t)(e + 128);
}

extern "C" int vt_image_encode_hdr(const float* pixels, int32_t width, int32_t height, int32_t channels,
                                   uint8_t* out, size_t out_bytes, size_t* written) {
  if (!pixels || !written || width <= 0 || height <= 0 || (channels != 3 && channels != 4))
    return fail(VT_EINVAL, "bad argument");
  char head[128];
  const int hl = snprintf(head, sizeof(head), "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n", height, width);
  const size_t need = (size_t)hl + (size_t)width * height * 4;
  *written = need;
  if (!out) return VT_OK;   // size query
  if (out_bytes < need) return fail(VT_EINVAL, "output buffer smaller than %zu bytes", need);
  memcpy(out, head, (size_t)hl);
  uint8_t* o = out + hl;
  for (int32_t y = height - 1; y >= 0; --y)   // rows bottom first in memory, top first in the file
    for (int32_t x = 0; x < width; ++x, o += 4) {
      const float* px = pixels + ((size_t)y * width + x) * channels;
      to_rgbe(px[0], px[1], px[2], o);
    }
  return VT_OK;
}
