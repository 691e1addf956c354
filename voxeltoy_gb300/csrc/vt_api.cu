// vt_api.cu — host runtime behind the C ABI (include/vt.h, include/vt_diag.h):
// contexts with a device-memory budget, scenes, environment images, jobs,
// batched rendering and the camera math of the reference Renderer.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/vt.h"
#include "../../include/vt_diag.h"
#include "vt_builtins.h"
#include "vt_internal.h"
#include "vt_kernels.h"
#include "vt_runtime.h"

using namespace vt;

// ------------------------------------------------------------------ errors
static thread_local std::string g_last_error;

int vt::fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int vt::cuda_fail(cudaError_t e, const char* what) {
  return fail(e == cudaErrorMemoryAllocation ? VT_ENOMEM : VT_EDEVICE, "%s: %s", what, cudaGetErrorString(e));
}

extern "C" const char* vt_last_error(void) { return g_last_error.c_str(); }

#define VT_CHECK_ARG(cond, msg) \
  do { if (!(cond)) return fail(VT_EINVAL, "%s", msg); } while (0)
#define VT_CUDA(call, what) \
  do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return cuda_fail(e_, what); } while (0)

// ----------------------------------------------------------------- context
void vt_context::log(const char* fmt, ...) {
  if (!log_fn) return;
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  log_fn(buf, log_user);
}

// Frees cached blocks, largest first, until at most `keep` bytes stay cached
// (the caller holds mu).
static uint64_t trim_locked(vt_context* ctx, uint64_t keep) {
  uint64_t freed = 0;
  if (ctx->cached > keep) cudaSetDevice(ctx->device);
  while (ctx->cached > keep && !ctx->cache.empty()) {
    auto it = std::prev(ctx->cache.end());
    cudaFree(it->second);
    ctx->cached -= it->first;
    freed += it->first;
    ctx->cache.erase(it);
  }
  return freed;
}

int vt_context::alloc(void** ptr, size_t bytes) {
  *ptr = nullptr;
  if (bytes == 0) bytes = 16;
  bytes = (bytes + 511) / 512 * 512;
  std::lock_guard<std::mutex> g(mu);
  if (budget && in_use + bytes > budget)
    return fail(VT_EBUDGET, "device-memory budget exceeded: %llu + %llu > %llu bytes",
                (unsigned long long)in_use, (unsigned long long)bytes, (unsigned long long)budget);
  auto hit = cache.lower_bound(bytes);
  if (hit != cache.end() && hit->first <= bytes + bytes / 4 && (!budget || in_use + hit->first <= budget)) {
    *ptr = hit->second;
    sizes[*ptr] = hit->first;
    in_use += hit->first;
    cached -= hit->first;
    cache.erase(hit);
    return VT_OK;
  }
  if (budget) trim_locked(this, in_use + bytes <= budget ? budget - in_use - bytes : 0);
  cudaSetDevice(device);
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e == cudaErrorMemoryAllocation && cached) {   // the cache first, then the device
    cudaGetLastError();
    trim_locked(this, 0);
    e = cudaMalloc(ptr, bytes);
  }
  if (e != cudaSuccess) { *ptr = nullptr; return cuda_fail(e, "cudaMalloc"); }
  sizes[*ptr] = bytes;
  in_use += bytes;
  return VT_OK;
}

void vt_context::release(void* ptr) {
  if (!ptr) return;
  std::lock_guard<std::mutex> g(mu);
  auto it = sizes.find(ptr);
  if (it == sizes.end()) { cudaFree(ptr); return; }
  const size_t sz = it->second;
  in_use -= sz;
  sizes.erase(it);
  cudaSetDevice(device);
  if (!caching || sz > cache_limit || !stream) { cudaFree(ptr); return; }
  // no kernel of this context still uses the block when another takes it
  if (cudaStreamSynchronize(stream) != cudaSuccess) { cudaGetLastError(); cudaFree(ptr); return; }
  cache.emplace(sz, ptr);
  cached += sz;
  trim_locked(this, cache_limit);
}

uint64_t vt_context::trim(uint64_t keep) {
  std::lock_guard<std::mutex> g(mu);
  return trim_locked(this, keep);
}

int vt_context::ensure_scratch(size_t bytes) {
  if (scratch_bytes >= bytes) return VT_OK;
  release(scratch);
  scratch = nullptr;
  scratch_bytes = 0;
  int rc = alloc(&scratch, bytes);
  if (rc != VT_OK) return rc;
  scratch_bytes = bytes;
  return VT_OK;
}

static uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

int vt_context::ensure_noise() {
  if (noise) return VT_OK;
  const size_t n = (size_t)kNoiseW * kNoiseH * 4;
  std::vector<float> host(n);
  for (size_t i = 0; i < n; ++i) host[i] = (float)(splitmix64((uint64_t)i) >> 40) * 5.9604644775390625e-8f;
  int rc = alloc((void**)&noise, n * sizeof(float));
  if (rc != VT_OK) return rc;
  VT_CUDA(cudaMemcpy(noise, host.data(), n * sizeof(float), cudaMemcpyHostToDevice), "noise table upload");
  return VT_OK;
}

extern "C" int vt_create(const vt_device_opts* opts, vt_context** out) {
  VT_CHECK_ARG(out, "out is null");
  *out = nullptr;
  int dev = opts ? opts->device : 0;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0)
    return fail(VT_EDEVICE, "no CUDA device available (%s)", cudaGetErrorString(e));
  VT_CHECK_ARG(dev >= 0 && dev < count, "device ordinal out of range");
  VT_CUDA(cudaSetDevice(dev), "cudaSetDevice");
  cudaDeviceProp prop;
  VT_CUDA(cudaGetDeviceProperties(&prop, dev), "cudaGetDeviceProperties");
  if (prop.major < 10) return fail(VT_EUNSUPPORTED, "device %s (sm_%d%d) is not Blackwell", prop.name, prop.major, prop.minor);
  vt_context* c = new vt_context();
  c->device = dev;
  c->budget = opts ? opts->hbm_budget_bytes : 0;
  c->caching = !(opts && (opts->flags & VT_DEVICE_NO_ALLOC_CACHE));
  c->sm_count = prop.multiProcessorCount;
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaStreamCreate"); }
  int rc = c->alloc((void**)&c->d_counters, sizeof(unsigned long long) * C_NUM);
  if (rc == VT_OK) rc = c->alloc((void**)&c->d_queue, sizeof(unsigned long long) * 4);
  if (rc == VT_OK) rc = c->alloc((void**)&c->d_error, sizeof(int32_t) * 4);
  if (rc != VT_OK) { vt_destroy(c); return rc; }
  cudaMemset(c->d_error, 0, sizeof(int32_t) * 4);
  // vt_render_batch_fixed's device array: loaded and located now, with this
  // device current, instead of at that entry point's first call.  A failure
  // here is not fatal to the context; the entry point retries and reports it.
  if (fixed_scratch_setup(dev) != VT_OK)
    c->log("vt_render_batch_fixed's device array is not available on device %d: %s", dev, vt_last_error());
  *out = c;
  return VT_OK;
}

// Every device buffer, host staging word, graph, event and stream a context
// owns (the context object itself stays).
void vt::release_context(vt_context* ctx) {
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->release(ctx->noise);
  ctx->release(ctx->scratch);
  ctx->release(ctx->d_counters);
  ctx->release(ctx->d_queue);
  ctx->release(ctx->d_error);
  ctx->release(ctx->d_jobs);
  ctx->release(ctx->d_grids);
  ctx->release(ctx->wf_mem);
  ctx->release(ctx->sbuf);
  ctx->release(ctx->wf_ctl);
  ctx->trim(0);
  if (ctx->h_live) cudaFreeHost(ctx->h_live);
  if (ctx->rounds_exec) cudaGraphExecDestroy(ctx->rounds_exec);
  if (ctx->lane_ready) cudaEventDestroy(ctx->lane_ready);
  for (int l = 0; l < vt_context::kMaxLanes - 1; ++l) {
    if (ctx->lane_done[l]) cudaEventDestroy(ctx->lane_done[l]);
    if (ctx->lane_stream[l]) cudaStreamDestroy(ctx->lane_stream[l]);
  }
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  ctx->h_live = nullptr;
  ctx->rounds_exec = nullptr;
  ctx->lane_ready = nullptr;
  for (int l = 0; l < vt_context::kMaxLanes - 1; ++l) {
    ctx->lane_done[l] = nullptr;
    ctx->lane_stream[l] = nullptr;
  }
  ctx->stream = nullptr;
}

extern "C" int vt_context_trim(vt_context* ctx, uint64_t* released) {
  VT_CHECK_ARG(ctx, "null argument");
  const uint64_t n = ctx->trim(0);
  if (released) *released = n;
  return VT_OK;
}

extern "C" int vt_destroy(vt_context* ctx) {
  if (!ctx) return VT_OK;
  release_context(ctx);
  delete ctx;
  return VT_OK;
}

extern "C" int vt_set_log_callback(vt_context* ctx, vt_log_fn fn, void* user) {
  VT_CHECK_ARG(ctx, "context is null");
  ctx->log_fn = fn;
  ctx->log_user = user;
  return VT_OK;
}

extern "C" int vt_context_memory(const vt_context* ctx, uint64_t* bytes) {
  VT_CHECK_ARG(ctx && bytes, "null argument");
  *bytes = ctx->in_use;
  return VT_OK;
}

// ---------------------------------------------------------------- palette
// One 16-byte record of eight IEEE halves.
static int pack_material(const vt_material& m, uint4* out) {
  if (m.type < 0 || m.type > 2) return fail(VT_EINVAL, "unknown material type %d", m.type);
  uint16_t h[8];
  h[0] = vtb::f2h((float)m.type);
  for (int i = 0; i < 3; ++i) h[1 + i] = vtb::f2h(m.emission[i]);
  for (int i = 0; i < 3; ++i) h[4 + i] = vtb::f2h(m.albedo[i]);
  h[7] = vtb::f2h(m.roughness);
  out->x = (uint32_t)h[0] | ((uint32_t)h[1] << 16);
  out->y = (uint32_t)h[2] | ((uint32_t)h[3] << 16);
  out->z = (uint32_t)h[4] | ((uint32_t)h[5] << 16);
  out->w = (uint32_t)h[6] | ((uint32_t)h[7] << 16);
  return VT_OK;
}

// ------------------------------------------------------------------ scenes
vt_scene::~vt_scene() {
  if (!ctx) return;
  ctx->release(grid);
  ctx->release(bricks);
  ctx->release(palette);
  ctx->release(emissive);
}

// Volume bounds of createVoxelDataTexture (renderer.cpp:845-850, 928-931).
static BrickShape scene_shape(const vt_scene* s) {
  BrickShape b;
  b.sx = s->bsh[0]; b.sy = s->bsh[1]; b.sz = s->bsh[2];
  return b;
}

static void scene_bounds(vt_scene* s) {
  const float voxel = 1000.0f / (float)std::max(s->res[0], std::max(s->res[1], s->res[2]));
  for (int i = 0; i < 3; ++i) {
    const float size = voxel * (float)s->res[i];
    s->bmin[i] = -size * 0.5f;
    s->bmax[i] = size * 0.5f;
    s->vsize[i] = (s->bmax[i] - s->bmin[i]) / (float)s->res[i];
    s->bdim[i] = (s->res[i] + (1 << s->bsh[i]) - 1) >> s->bsh[i];
  }
}

// Emissive-list pruning with the reference's swap-with-last removal order
// (Renderer::pruneInteriorEmissiveVoxels, src/renderer/import.cpp:180-203);
// the neighbour tests run on the GPU.
// `on_device` (nullable): the same list already in device memory.
static int prune_emissive(vt_context* ctx, vt_scene* s, std::vector<int32_t>& list,
                          const int32_t* on_device = nullptr) {
  if (list.empty()) return VT_OK;
  const int64_t n = (int64_t)list.size();
  int32_t* d_list = nullptr;
  uint8_t* d_keep = nullptr;
  int rc = VT_OK;
  if (!on_device) {
    rc = ctx->alloc((void**)&d_list, sizeof(int32_t) * n);
    if (rc != VT_OK) return rc;
  }
  rc = ctx->alloc((void**)&d_keep, (size_t)n);
  if (rc != VT_OK) { ctx->release(d_list); return rc; }
  std::vector<uint8_t> keep(n);
  cudaError_t e = cudaSuccess;
  if (!on_device)
    e = cudaMemcpyAsync(d_list, list.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, ctx->stream);
  const int32_t* dl = on_device ? on_device : d_list;
  if (e == cudaSuccess) e = launch_emissive_flags(s->grid, s->res[0], s->res[1], s->res[2], dl, n, d_keep, ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(keep.data(), d_keep, (size_t)n, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  ctx->release(d_list);
  ctx->release(d_keep);
  if (e != cudaSuccess) return cuda_fail(e, "emissive pruning");
  // The flag of an element travels with it when it is swapped into place.
  std::vector<int32_t> v = list;
  std::vector<uint8_t> k = keep;
  size_t removed = 0;
  for (int64_t i = 0; i < (int64_t)v.size(); ++i) {
    if (!k[i]) {
      v[i] = v.back();
      k[i] = k.back();
      v.pop_back();
      k.pop_back();
      --i;
      ++removed;
    }
  }
  ctx->log("Pruned emissive voxels: %zu/%lld", removed, (long long)n);
  list.swap(v);
  return VT_OK;
}

// The scene's emissive list: discovered from the palette
// (VT_SCENE_AUTO_EMISSIVE, in voxel order) or the caller's indices, pruned
// when VT_SCENE_PRUNE_EMISSIVE asks, uploaded in place of the previous list.
static int scene_emissive(vt_context* ctx, vt_scene* s, const int32_t* emissive, int64_t n_emissive,
                          uint32_t flags) {
  const int64_t nvox = (int64_t)s->res[0] * s->res[1] * s->res[2];
  const int32_t n_palette = s->n_palette;
  const vt_material* palette = s->host_palette.data();
  int rc = VT_OK;
  std::vector<int32_t> list;
  if (flags & VT_SCENE_AUTO_EMISSIVE) {
    uint8_t em[256] = {0};
    for (int i = 0; i < n_palette; ++i) {
      const vt_material& m = palette[i];
      // emissive when the quantised emission is non-zero (VoxLoader::getMaterialEmisiveness)
      const float e = vtb::h2f(vtb::f2h(m.emission[0])) + vtb::h2f(vtb::f2h(m.emission[1])) +
                      vtb::h2f(vtb::f2h(m.emission[2]));
      em[i + 1] = e > 0.0f ? 1 : 0;
    }
    bool lit = false;   // no emitting entry: an empty list without a pass over the grid
    for (int i = 1; i <= n_palette; ++i) lit = lit || em[i] != 0;
    // voxel order, found on the device (two passes over the grid)
    const int64_t chunks = lit ? emissive_chunks(nvox) : 0;
    void* tmp = nullptr;
    rc = ctx->alloc(&tmp, 256 + sizeof(uint32_t) * (size_t)(chunks + 1));
    if (rc != VT_OK) return rc;
    uint8_t* d_em = (uint8_t*)tmp;
    uint32_t* d_counts = (uint32_t*)((char*)tmp + 256);
    uint32_t total = 0;   // pageable: the read has completed when the copy returns
    cudaError_t e = cudaSuccess;
    if (lit) {
      e = cudaMemcpyAsync(d_em, em, 256, cudaMemcpyHostToDevice, ctx->stream);
      if (e == cudaSuccess) e = launch_emissive_count(s->grid, nvox, d_em, d_counts, ctx->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(&total, d_counts + chunks, sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream);
    }
    int32_t* d_out = nullptr;
    if (e == cudaSuccess && total > 0) {
      rc = ctx->alloc((void**)&d_out, sizeof(int32_t) * (size_t)total);
      if (rc != VT_OK) { ctx->release(tmp); return rc; }
      list.resize(total);
      e = launch_emissive_write(s->grid, nvox, d_em, d_counts, d_out, ctx->stream);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(list.data(), d_out, sizeof(int32_t) * (size_t)total, cudaMemcpyDeviceToHost, ctx->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    }
    if (e == cudaSuccess && (flags & VT_SCENE_PRUNE_EMISSIVE)) rc = prune_emissive(ctx, s, list, d_out);
    ctx->release(d_out);
    ctx->release(tmp);
    if (e != cudaSuccess) return cuda_fail(e, "emissive discovery");
    if (rc != VT_OK) return rc;
  } else if (n_emissive > 0) {
    VT_CHECK_ARG(emissive, "emissive_indices is null");
    list.assign(emissive, emissive + n_emissive);
    for (int32_t v : list)
      if (v < 0 || (int64_t)v >= nvox) return fail(VT_EINVAL, "emissive index %d out of range", v);
    if (flags & VT_SCENE_PRUNE_EMISSIVE) {
      rc = prune_emissive(ctx, s, list);
      if (rc != VT_OK) return rc;
    }
  }
  ctx->release(s->emissive);
  s->emissive = nullptr;
  s->n_emissive = (int64_t)list.size();
  rc = ctx->alloc((void**)&s->emissive, sizeof(int32_t) * std::max<size_t>(list.size(), 1));
  if (rc != VT_OK) return rc;
  if (!list.empty())
    VT_CUDA(cudaMemcpyAsync(s->emissive, list.data(), sizeof(int32_t) * list.size(), cudaMemcpyHostToDevice,
                            ctx->stream), "emissive upload");
  return VT_OK;
}

// Palette, bit-bricks (unless the voxelizer built them: s->bricks set and
// every voxel's entry known to be within the palette) and emissive list.
static int scene_finish(vt_context* ctx, vt_scene* s, const vt_material* palette, int32_t n_palette,
                        const int32_t* emissive, int64_t n_emissive, uint32_t flags, bool bricks_built = false) {
  const int64_t nvox = (int64_t)s->res[0] * s->res[1] * s->res[2];
  // palette
  std::vector<uint4> pal(std::max(n_palette, 1));
  for (int i = 0; i < n_palette; ++i) {
    int rc = pack_material(palette[i], &pal[i]);
    if (rc != VT_OK) return rc;
  }
  s->n_palette = n_palette;
  s->host_palette.assign(palette, palette + n_palette);
  // the palette as the reference's flat material table, entry after entry
  s->mat_table.clear();
  s->mat_offset.assign(n_palette, -1);
  for (int i = 0; i < n_palette; ++i) {
    const vt_material& m = palette[i];
    s->mat_offset[i] = (int64_t)s->mat_table.size();
    s->mat_table.push_back((float)m.type);
    s->mat_table.insert(s->mat_table.end(), m.emission, m.emission + 3);
    s->mat_table.insert(s->mat_table.end(), m.albedo, m.albedo + 3);
    if (m.type != VT_MATERIAL_LAMBERT) s->mat_table.push_back(m.roughness);
  }
  int rc = ctx->alloc((void**)&s->palette, sizeof(uint4) * pal.size());
  if (rc != VT_OK) return rc;
  VT_CUDA(cudaMemcpyAsync(s->palette, pal.data(), sizeof(uint4) * pal.size(), cudaMemcpyHostToDevice, ctx->stream),
          "palette upload");
  // bit-bricks
  const int64_t nb = (int64_t)(s->bdim[0] + 2) * (s->bdim[1] + 2) * (s->bdim[2] + 2);
  if (!bricks_built) {
    rc = ctx->alloc((void**)&s->bricks, sizeof(unsigned long long) * nb);
    if (rc != VT_OK) return rc;
    // the bricks pass also finds the largest palette entry the volume uses
    unsigned long long* d_top = ctx->d_queue + 1;
    VT_CUDA(cudaMemsetAsync(d_top, 0, sizeof(unsigned long long), ctx->stream), "brick build");
    VT_CUDA(launch_build_bricks(s->grid, s->res[0], s->res[1], s->res[2], s->bricks, s->bdim[0], s->bdim[1],
                                s->bdim[2], scene_shape(s), d_top, ctx->stream), "brick build");
    unsigned long long top = 0;   // pageable: the read has completed when the copy returns
    VT_CUDA(cudaMemcpyAsync(&top, d_top, sizeof(top), cudaMemcpyDeviceToHost, ctx->stream), "brick build");
    if (top > (unsigned long long)n_palette)
      return fail(VT_EINVAL, "voxel uses palette entry %d of %d", (int)top, n_palette);
  }
  s->flags = flags;
  rc = scene_emissive(ctx, s, emissive, n_emissive, flags);
  if (rc != VT_OK) return rc;
  VT_CUDA(cudaStreamSynchronize(ctx->stream), "scene upload");
  s->bytes = (uint64_t)nvox + sizeof(unsigned long long) * nb + sizeof(uint4) * pal.size() +
             sizeof(int32_t) * std::max<int64_t>(s->n_emissive, 1);
  return VT_OK;
}

static int scene_alloc(vt_context* ctx, int32_t rx, int32_t ry, int32_t rz, vt_scene** out, vt_scene** s_out) {
  VT_CHECK_ARG(ctx && out, "null argument");
  VT_CHECK_ARG(rx > 0 && ry > 0 && rz > 0, "resolution must be positive");
  VT_CHECK_ARG((int64_t)rx * ry * rz < ((int64_t)1 << 31), "volume exceeds 2^31 voxels");
  // the wavefront's packed segment ends hold positions -1 .. extent
  VT_CHECK_ARG(rx <= (1 << 20) - 2 && ry <= (1 << 20) - 2 && rz <= (1 << 19) - 2,
               "volume extent beyond 1048574 (x, y) or 524286 (z) voxels");
  *out = nullptr;
  vt_scene* s = new vt_scene();
  s->ctx = ctx;
  s->res[0] = rx; s->res[1] = ry; s->res[2] = rz;
  scene_bounds(s);
  const int64_t nvox = (int64_t)rx * ry * rz;
  int rc = ctx->alloc((void**)&s->grid, (size_t)nvox);
  if (rc != VT_OK) { delete s; return rc; }
  *s_out = s;
  return VT_OK;
}

extern "C" int vt_scene_create(vt_context* ctx, int32_t rx, int32_t ry, int32_t rz, const uint8_t* voxels,
                               const vt_material* palette, int32_t n_palette, const int32_t* emissive_indices,
                               int64_t n_emissive, uint32_t flags, vt_scene** out) {
  vt::Range nvtx_range("vt.scene_build");
  VT_CHECK_ARG(voxels && palette, "voxels/palette is null");
  VT_CHECK_ARG(n_palette >= 1 && n_palette <= 255, "n_palette must be in [1, 255]");
  VT_CHECK_ARG(n_emissive >= 0, "n_emissive < 0");
  vt_scene* s = nullptr;
  int rc = scene_alloc(ctx, rx, ry, rz, out, &s);
  if (rc != VT_OK) return rc;
  const int64_t nvox = (int64_t)rx * ry * rz;
  cudaError_t e = cudaMemcpyAsync(s->grid, voxels, (size_t)nvox, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) { delete s; return cuda_fail(e, "grid upload"); }
  rc = scene_finish(ctx, s, palette, n_palette, emissive_indices, n_emissive, flags);
  if (rc != VT_OK) { delete s; return rc; }
  *out = s;
  return VT_OK;
}

extern "C" int vt_scene_create_from_offsets(vt_context* ctx, int32_t rx, int32_t ry, int32_t rz,
                                            const int32_t* offsets, const float* table, int64_t table_size,
                                            const int32_t* emissive_indices, int64_t n_emissive, uint32_t flags,
                                            vt_scene** out) {
  VT_CHECK_ARG(offsets && table, "offsets/table is null");
  VT_CHECK_ARG(rx > 0 && ry > 0 && rz > 0, "resolution must be positive");
  const int64_t nvox = (int64_t)rx * ry * rz;
  // distinct record offsets, in ascending order, become palette entries
  std::vector<int32_t> used;
  {
    std::vector<int32_t> tmp;
    for (int64_t i = 0; i < nvox; ++i)
      if (offsets[i] >= 0) tmp.push_back(offsets[i]);
    std::sort(tmp.begin(), tmp.end());
    tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
    used.swap(tmp);
  }
  if (used.size() > 255) return fail(VT_EINVAL, "%zu distinct materials referenced (at most 255)", used.size());
  std::vector<vt_material> pal;
  std::unordered_map<int32_t, uint8_t> entry;
  for (int32_t off : used) {
    if ((int64_t)off >= table_size) return fail(VT_EINVAL, "material offset %d outside the table", off);
    vt_material m;
    m.type = (int32_t)table[off];
    const int64_t need = (m.type == 0) ? 7 : 8;   // type + LambertMaterialData / Metal / Plastic
    if (m.type < 0 || m.type > 2) return fail(VT_EINVAL, "unknown material type %g at offset %d", table[off], off);
    if ((int64_t)off + need > table_size) return fail(VT_EINVAL, "material record at %d truncated", off);
    for (int i = 0; i < 3; ++i) { m.emission[i] = table[off + 1 + i]; m.albedo[i] = table[off + 4 + i]; }
    m.roughness = (m.type == 0) ? 0.0f : table[off + 7];
    entry[off] = (uint8_t)(pal.size() + 1);
    pal.push_back(m);
  }
  if (pal.empty()) {
    vt_material m = {0, {0, 0, 0}, {0, 0, 0}, 0};
    pal.push_back(m);
  }
  std::vector<uint8_t> vox((size_t)nvox);
  for (int64_t i = 0; i < nvox; ++i) vox[i] = offsets[i] >= 0 ? entry[offsets[i]] : 0;
  const int rc = vt_scene_create(ctx, rx, ry, rz, vox.data(), pal.data(), (int32_t)pal.size(), emissive_indices,
                                 n_emissive, flags, out);
  if (rc == VT_OK) {   // the caller's table and offsets stay the material table
    vt_scene* s = *out;
    s->mat_table.assign(table, table + table_size);
    s->mat_offset.assign(s->n_palette, -1);
    for (size_t k = 0; k < used.size(); ++k) s->mat_offset[k] = used[k];
  }
  return rc;
}

extern "C" int vt_scene_voxelize_mesh(vt_context* ctx, const float* vertices, int64_t n_vertices,
                                      const uint32_t* indices, int64_t n_triangles, int32_t rx, int32_t ry,
                                      int32_t rz, int32_t mode, int32_t placement, const vt_material* palette,
                                      int32_t n_palette, vt_scene** out) {
  vt::Range nvtx_range("vt.voxelize");
  VT_CHECK_ARG(ctx && out, "null argument");
  VT_CHECK_ARG(n_triangles == 0 || (vertices && indices), "vertices/indices is null");
  VT_CHECK_ARG(n_vertices >= 0 && n_triangles >= 0, "negative counts");
  VT_CHECK_ARG((mode & ~VT_VOXELIZE_REFERENCE_BOUNDS) == VT_VOXELIZE_THIN ||
                   (mode & ~VT_VOXELIZE_REFERENCE_BOUNDS) == VT_VOXELIZE_FAT,
               "unknown voxelization mode");
  VT_CHECK_ARG(palette && n_palette >= 1 && n_palette <= 255, "palette needs 1..255 entries");
  vt_scene* s = nullptr;
  int rc = scene_alloc(ctx, rx, ry, rz, out, &s);
  if (rc != VT_OK) return rc;
  const int64_t nvox = (int64_t)rx * ry * rz;
  // mesh and the large-triangle list through the budgeted allocator; the
  // indices are checked and computeMeshTransform (import.cpp:46-64) applied
  // on the device, and the voxelizer sets the brick bits itself, so no
  // host pass over the mesh and no separate brick pass follow
  float* d_v = nullptr;
  uint32_t* d_i = nullptr;
  const int64_t nb = (int64_t)(s->bdim[0] + 2) * (s->bdim[1] + 2) * (s->bdim[2] + 2);
  rc = ctx->alloc((void**)&d_v, sizeof(float) * 3 * std::max<int64_t>(n_vertices, 1));
  if (rc == VT_OK) rc = ctx->alloc((void**)&d_i, sizeof(uint32_t) * 3 * std::max<int64_t>(n_triangles, 1));
  if (rc == VT_OK) rc = ctx->ensure_scratch(voxelize_scratch_bytes(n_triangles));
  if (rc == VT_OK) rc = ctx->alloc((void**)&s->bricks, sizeof(unsigned long long) * nb);
  if (rc != VT_OK) { ctx->release(d_v); ctx->release(d_i); delete s; return rc; }
  cudaError_t e = cudaMemsetAsync(s->grid, 0, (size_t)nvox, ctx->stream);
  if (e == cudaSuccess)
    e = launch_bricks_init(s->bricks, rx, ry, rz, s->bdim[0], s->bdim[1], s->bdim[2], scene_shape(s), ctx->stream);
  if (e == cudaSuccess && n_vertices)
    e = cudaMemcpyAsync(d_v, vertices, sizeof(float) * 3 * n_vertices, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess && n_triangles)
    e = cudaMemcpyAsync(d_i, indices, sizeof(uint32_t) * 3 * n_triangles, cudaMemcpyHostToDevice, ctx->stream);
  MeshPrep* prep = voxelize_prep_record(ctx->scratch, n_triangles);
  if (e == cudaSuccess)
    e = launch_mesh_prep(d_v, n_vertices, d_i, n_triangles, placement == VT_MESH_FIT_UNIT_CUBE, rx, ry, rz, prep,
                         ctx->sm_count, ctx->stream);
  if (e == cudaSuccess)
    e = launch_voxelize(d_v, n_vertices, d_i, n_triangles, rx, ry, rz, mode & 1,
                        (mode & VT_VOXELIZE_REFERENCE_BOUNDS) != 0, s->grid, 1, s->bricks, s->bdim[0], s->bdim[1],
                        scene_shape(s), ctx->scratch, ctx->sm_count * 4, ctx->stream);
  unsigned long long bad = 0ull;   // pageable destination: written when the copy returns
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, &prep->bad, sizeof(bad), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  ctx->release(d_v);
  ctx->release(d_i);
  if (e != cudaSuccess) { delete s; return cuda_fail(e, "voxelization"); }
  if (bad) {
    delete s;
    return fail(VT_EINVAL, "triangle index %u out of range (%lld vertices)", (unsigned)(bad & 0xffffffffu),
                (long long)n_vertices);
  }
  rc = scene_finish(ctx, s, palette, n_palette, nullptr, 0, VT_SCENE_AUTO_EMISSIVE | VT_SCENE_PRUNE_EMISSIVE,
                    /*bricks_built=*/true);
  if (rc != VT_OK) { delete s; return rc; }
  *out = s;
  return VT_OK;
}

extern "C" int vt_scene_get_info(const vt_scene* s, vt_scene_info* info) {
  VT_CHECK_ARG(s && info, "null argument");
  for (int i = 0; i < 3; ++i) {
    info->resolution[i] = s->res[i];
    info->bounds_min[i] = s->bmin[i];
    info->bounds_max[i] = s->bmax[i];
    info->voxel_size[i] = s->vsize[i];
  }
  info->n_emissive = s->n_emissive;
  info->n_palette = s->n_palette;
  info->device_bytes = s->bytes;
  return VT_OK;
}

extern "C" int vt_scene_read_voxels(const vt_scene* s, uint8_t* out, size_t bytes) {
  VT_CHECK_ARG(s && out, "null argument");
  const size_t n = (size_t)s->res[0] * s->res[1] * s->res[2];
  VT_CHECK_ARG(bytes >= n, "output buffer too small");
  cudaSetDevice(s->ctx->device);
  VT_CUDA(cudaMemcpy(out, s->grid, n, cudaMemcpyDeviceToHost), "grid readback");
  return VT_OK;
}

extern "C" int vt_scene_read_emissive(const vt_scene* s, int32_t* out, int64_t capacity, int64_t* n) {
  VT_CHECK_ARG(s && n, "null argument");
  *n = s->n_emissive;
  if (out && capacity > 0 && s->n_emissive > 0) {
    cudaSetDevice(s->ctx->device);
    VT_CUDA(cudaMemcpy(out, s->emissive, sizeof(int32_t) * std::min(capacity, s->n_emissive), cudaMemcpyDeviceToHost),
            "emissive readback");
  }
  return VT_OK;
}

extern "C" int vt_scene_read_material_table(const vt_scene* s, float* out, int64_t capacity, int64_t* size) {
  VT_CHECK_ARG(s && size, "null argument");
  *size = (int64_t)s->mat_table.size();
  if (!out) return VT_OK;
  if (capacity < *size)
    return fail(VT_EINVAL, "capacity %lld < %lld floats", (long long)capacity, (long long)*size);
  std::copy(s->mat_table.begin(), s->mat_table.end(), out);
  return VT_OK;
}

// Floats of the record at `at` (type + data), 0 for an unknown type.
static int64_t record_floats(const std::vector<float>& t, int64_t at) {
  if (at < 0 || at >= (int64_t)t.size()) return 0;
  const float type = t[(size_t)at];
  if (type == 0.0f) return 7;
  if (type == 1.0f || type == 2.0f) return 8;
  return 0;
}

// Emits light: the quantised emission is non-zero (VoxLoader::getMaterialEmisiveness).
static bool emits(const vt_material& m) {
  return vtb::h2f(vtb::f2h(m.emission[0])) + vtb::h2f(vtb::f2h(m.emission[1])) +
         vtb::h2f(vtb::f2h(m.emission[2])) > 0.0f;
}

extern "C" int vt_scene_write_material_table(vt_scene* s, int64_t off, const float* values, int32_t n) {
  VT_CHECK_ARG(s && values && n > 0, "bad argument");
  vt_context* ctx = s->ctx;
  const std::vector<float>& t = s->mat_table;
  // the record holding [off, off + n): a palette entry's, or any record of
  // the table walked as getMaterials walks it
  int64_t rec = -1;
  for (int64_t o : s->mat_offset) {
    const int64_t len = record_floats(t, o);
    if (len && off > o && off + n <= o + len) { rec = o; break; }
  }
  for (int64_t at = 0; rec < 0 && at < (int64_t)t.size();) {
    const int64_t len = record_floats(t, at);
    if (!len) break;
    if (off > at && off + n <= at + len) rec = at;
    at += len;
  }
  if (rec < 0)
    return fail(VT_EINVAL, "floats [%lld, %lld) are not inside the data of one material record", (long long)off,
                (long long)(off + n));
  for (int32_t i = 0; i < n; ++i) s->mat_table[(size_t)(off + i)] = values[i];
  cudaSetDevice(ctx->device);
  bool relist = false;
  for (int32_t k = 0; k < s->n_palette; ++k) {
    if (s->mat_offset[k] != rec) continue;
    vt_material m = s->host_palette[k];
    const float* r = &s->mat_table[(size_t)rec];
    for (int c = 0; c < 3; ++c) { m.emission[c] = r[1 + c]; m.albedo[c] = r[4 + c]; }
    m.roughness = m.type == VT_MATERIAL_LAMBERT ? 0.0f : r[7];
    uint4 q;
    const int rc = pack_material(m, &q);
    if (rc != VT_OK) return rc;
    relist = relist || emits(m) != emits(s->host_palette[k]);
    s->host_palette[k] = m;
    // pageable source: staged before the call returns; ordered after earlier passes
    VT_CUDA(cudaMemcpyAsync(s->palette + k, &q, sizeof(q), cudaMemcpyHostToDevice, ctx->stream), "material update");
  }
  if (relist && (s->flags & VT_SCENE_AUTO_EMISSIVE)) {
    const int rc = scene_emissive(ctx, s, nullptr, 0, s->flags);
    if (rc != VT_OK) return rc;
    s->generation++;   // jobs pick up the new list before their next pass
  }
  return VT_OK;
}

extern "C" int vt_scene_destroy(vt_scene* s) {
  if (!s) return VT_OK;
  cudaSetDevice(s->ctx->device);
  cudaStreamSynchronize(s->ctx->stream);
  delete s;
  return VT_OK;
}

// ------------------------------------------------------------- environment
vt_env::~vt_env() {
  if (!ctx) return;
  ctx->release(texels);
  ctx->release(cdf_u);
  ctx->release(cdf_v);
}

// Scratch layout of an environment build: nine offsets into one buffer.
static size_t env_scratch_bytes(int32_t w, int32_t h, size_t (&offs)[9]) {
  const size_t n = (size_t)w * h;
  size_t o = 0;
  auto take = [&](size_t bytes) { size_t at = o; o += (bytes + 255) & ~(size_t)255; return at; };
  offs[0] = take(sizeof(float) * n);                 // lum
  offs[1] = take(sizeof(float) * n);                 // tmp
  offs[2] = take(sizeof(float) * n);                 // func
  offs[3] = take(sizeof(float) * h);                 // sin
  offs[4] = take(sizeof(double) * (size_t)h * (w + 1));  // row prefixes
  offs[5] = take(sizeof(double) * h);                // row integrals
  offs[6] = take(sizeof(double) * (h + 1));          // marginal prefixes
  offs[7] = take(sizeof(float) * 3 * n);             // rgb input
  offs[8] = take(2 * sizeof(uint32_t));              // integral, first non-finite texel
  return o;
}

static EnvScratch env_scratch(void* base, const size_t* offs) {
  char* b = (char*)base;
  EnvScratch S;
  S.lum = (float*)(b + offs[0]);
  S.tmp = (float*)(b + offs[1]);
  S.func = (float*)(b + offs[2]);
  S.sin_theta = (float*)(b + offs[3]);
  S.row_pre = (double*)(b + offs[4]);
  S.row_int = (double*)(b + offs[5]);
  S.marg_pre = (double*)(b + offs[6]);
  return S;
}

// The reference's CDF image size (calculateCDF, image.cpp:14, 314-317): at
// most 512 texels on the long axis, by its float arithmetic.
static void reference_cdf_size(int32_t w, int32_t h, int32_t* cw, int32_t* ch) {
  const unsigned m = (unsigned)std::max(w, h);
  if (m <= 512u) { *cw = w; *ch = h; return; }
  *cw = (int32_t)(unsigned)((float)(unsigned)w / (float)m * 512.0f);
  *ch = (int32_t)(unsigned)((float)(unsigned)h / (float)m * 512.0f);
}

extern "C" int vt_env_create_image(vt_context* ctx, const float* rgb, int32_t w, int32_t h, vt_env** out) {
  return vt_env_create_image_ex(ctx, rgb, w, h, 0u, out);
}

extern "C" int vt_env_create_image_ex(vt_context* ctx, const float* rgb, int32_t w, int32_t h, uint32_t flags,
                                      vt_env** out) {
  vt::Range nvtx_range("vt.env_build");
  VT_CHECK_ARG(ctx && rgb && out, "null argument");
  VT_CHECK_ARG(w > 0 && h > 0 && (int64_t)w * h < ((int64_t)1 << 28), "bad image size");
  VT_CHECK_ARG((flags & ~(uint32_t)VT_ENV_CDF_REFERENCE_SIZE) == 0, "unknown environment flags");
  *out = nullptr;
  vt_env* env = new vt_env();
  env->ctx = ctx;
  env->w = w;
  env->h = h;
  env->cdf_w = w;
  env->cdf_h = h;
  if (flags & VT_ENV_CDF_REFERENCE_SIZE) reference_cdf_size(w, h, &env->cdf_w, &env->cdf_h);
  const int32_t cw = env->cdf_w, ch = env->cdf_h;
  VT_CHECK_ARG(cw > 0 && ch > 0, "the shrunk CDF image is empty");
  const size_t n = (size_t)w * h;
  int rc = ctx->alloc((void**)&env->texels, sizeof(uint2) * n);
  if (rc == VT_OK) rc = ctx->alloc((void**)&env->cdf_u, sizeof(float) * (size_t)(cw + 1) * ch);
  if (rc == VT_OK) rc = ctx->alloc((void**)&env->cdf_v, sizeof(float) * (size_t)(ch + 1));
  size_t offs[9];
  const size_t sb = env_scratch_bytes(w, h, offs);
  if (rc == VT_OK) rc = ctx->ensure_scratch(sb);   // kept by the context for the next build
  if (rc != VT_OK) { delete env; return rc; }
  void* scratch = ctx->scratch;
  EnvScratch S = env_scratch(scratch, offs);
  // row weights sin(pi (y + 0.5) / h) of the CDF image, as calculateImageIntegral computes them (image.cpp:366)
  std::vector<float> sin_theta(ch);
  for (int y = 0; y < ch; ++y) sin_theta[y] = (float)std::sin(M_PI * (double)((float)y + 0.5f) / (double)(float)ch);
  float* d_rgb = (float*)((char*)scratch + offs[7]);
  uint32_t* d_out = (uint32_t*)((char*)scratch + offs[8]);   // integral bits, first non-finite texel
  uint32_t res[2] = {0u, 0u};   // pageable: the read has completed when the copy returns
  cudaError_t e = cudaMemcpyAsync(d_rgb, rgb, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(S.sin_theta, sin_theta.data(), sizeof(float) * ch, cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_out + 1, 0xff, sizeof(uint32_t), ctx->stream);
  if (e == cudaSuccess)
    e = launch_env_build(d_rgb, w, h, cw, ch, S, env->texels, env->cdf_u, env->cdf_v, (float*)d_out, d_out + 1,
                         ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(res, d_out, sizeof(res), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) { delete env; return cuda_fail(e, "environment build"); }
  if (res[1] != 0xffffffffu) {
    delete env;
    return fail(VT_EINVAL, "environment texel %lld is not finite", (long long)res[1]);
  }
  float integral;
  memcpy(&integral, &res[0], sizeof(integral));
  env->integral = integral;
  *out = env;
  return VT_OK;
}

extern "C" int vt_env_read_cdf(const vt_env* env, float* cdf_u, size_t cu_bytes, float* cdf_v, size_t cv_bytes,
                               float* integral) {
  VT_CHECK_ARG(env, "env is null");
  cudaSetDevice(env->ctx->device);
  const size_t nu = sizeof(float) * (size_t)(env->cdf_w + 1) * env->cdf_h, nv = sizeof(float) * (size_t)(env->cdf_h + 1);
  if (cdf_u) { VT_CHECK_ARG(cu_bytes >= nu, "cdf_u too small"); VT_CUDA(cudaMemcpy(cdf_u, env->cdf_u, nu, cudaMemcpyDeviceToHost), "cdf_u"); }
  if (cdf_v) { VT_CHECK_ARG(cv_bytes >= nv, "cdf_v too small"); VT_CUDA(cudaMemcpy(cdf_v, env->cdf_v, nv, cudaMemcpyDeviceToHost), "cdf_v"); }
  if (integral) *integral = env->integral;
  return VT_OK;
}

extern "C" int vt_env_get_info(const vt_env* env, int32_t* size) {
  VT_CHECK_ARG(env && size, "null argument");
  size[0] = env->w; size[1] = env->h; size[2] = env->cdf_w; size[3] = env->cdf_h;
  return VT_OK;
}

extern "C" int vt_env_destroy(vt_env* env) {
  if (!env) return VT_OK;
  cudaSetDevice(env->ctx->device);
  cudaStreamSynchronize(env->ctx->stream);
  delete env;
  return VT_OK;
}

// ------------------------------------------------------------------ camera
static void v3_sub(const float* a, const float* b, float* r) { for (int i = 0; i < 3; ++i) r[i] = a[i] - b[i]; }
static float v3_dot(const float* a, const float* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
static void v3_cross(const float* a, const float* b, float* r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}
static float v3_len(const float* a) { return std::sqrt(v3_dot(a, a)); }
static void v3_normalized(const float* a, float* r) {
  const float l = v3_len(a);
  if (l == 0.0f) { r[0] = r[1] = r[2] = 0.0f; return; }
  for (int i = 0; i < 3; ++i) r[i] = a[i] / l;
}
// CameraParameters::getBasis (cameraParameters.cpp:43-50).
static void cam_basis(const vt_camera* c, float* fwd, float* right, float* up) {
  float d[3];
  v3_sub(c->target, c->eye, d);
  v3_normalized(d, fwd);
  const float y[3] = {0.0f, 1.0f, 0.0f};
  float r[3];
  v3_cross(y, fwd, r);
  v3_normalized(r, right);
  v3_cross(fwd, right, up);
}
static void sph(float theta, float phi, float* r) {
  const float st = std::sin(theta);
  r[0] = st * std::cos(phi); r[1] = std::cos(theta); r[2] = st * std::sin(phi);
}

extern "C" int vt_camera_default(vt_camera* cam) {
  VT_CHECK_ARG(cam, "camera is null");
  // target (0,0,0), eye at distance 100 along -forward with forward = +Z
  cam->target[0] = cam->target[1] = cam->target[2] = 0.0f;
  cam->eye[0] = 0.0f; cam->eye[1] = 0.0f; cam->eye[2] = -100.0f;
  cam->near_distance = 0.1f;
  cam->far_distance = 10000.0f;
  cam->focal_distance = 99999999.0f;   // focal-distance buffer initial value (renderer.cpp:711-720)
  cam->lens_radius = 0.0f;
  cam->lens_model = VT_LENS_PINHOLE;
  // setFocalLength(50) with a 36 mm film: fovY = 2 atan2(18, 50)
  cam->fov_y = std::atan2(36.0f * 0.5f, 50.0f) * 2.0f;
  return VT_OK;
}

extern "C" int vt_camera_orbit(vt_camera* cam, float theta, float phi) {
  VT_CHECK_ARG(cam, "camera is null");
  float d[3], s[3];
  v3_sub(cam->target, cam->eye, d);
  const float r = v3_len(d);
  sph(theta, phi, s);
  for (int i = 0; i < 3; ++i) cam->eye[i] = cam->target[i] - r * s[i];
  return VT_OK;
}

extern "C" int vt_camera_orbit_eye(vt_camera* cam, float theta, float phi) {
  VT_CHECK_ARG(cam, "camera is null");
  float d[3], s[3];
  v3_sub(cam->target, cam->eye, d);
  const float r = v3_len(d);
  sph(theta, phi, s);
  for (int i = 0; i < 3; ++i) cam->target[i] = cam->eye[i] + r * s[i];
  return VT_OK;
}

extern "C" int vt_camera_set_distance(vt_camera* cam, float distance) {
  VT_CHECK_ARG(cam, "camera is null");
  float f[3], r[3], u[3];
  cam_basis(cam, f, r, u);
  for (int i = 0; i < 3; ++i) cam->eye[i] = cam->target[i] - f[i] * distance;
  return VT_OK;
}

// Film size of Renderer::render / resizeFrame (renderer.cpp:573-580).
static void film_size(int32_t w, int32_t h, float* fw, float* fh) {
  const float a = (float)w / (float)h;
  if (a >= 1.0f) { *fw = 36.0f; *fh = 36.0f / a; }
  else { *fw = 36.0f * a; *fh = 36.0f; }
}

extern "C" int vt_camera_set_focal_length(vt_camera* cam, float f_mm, int32_t w, int32_t h) {
  VT_CHECK_ARG(cam && w > 0 && h > 0 && f_mm > 0.0f, "bad argument");
  float fw, fh;
  film_size(w, h, &fw, &fh);
  cam->fov_y = std::atan2(fh * 0.5f, f_mm) * 2.0f;
  return VT_OK;
}

extern "C" int vt_camera_set_fstop(vt_camera* cam, float fstop, int32_t w, int32_t h) {
  VT_CHECK_ARG(cam && w > 0 && h > 0, "bad argument");
  float fw, fh;
  film_size(w, h, &fw, &fh);
  const float focal = fh / (2.0f * std::tan(0.5f * cam->fov_y));
  cam->lens_radius = (focal / std::max(1e-4f, fstop)) * 0.5f;
  return VT_OK;
}

extern "C" int vt_camera_focus_on_bounds(vt_camera* cam, const float bmin[3], const float bmax[3]) {
  VT_CHECK_ARG(cam && bmin && bmax, "null argument");
  float f[3], r[3], u[3];
  cam_basis(cam, f, r, u);
  float size[3], center[3];
  for (int i = 0; i < 3; ++i) { size[i] = bmax[i] - bmin[i]; center[i] = (bmin[i] + bmax[i]) / 2.0f; }
  const float dist = v3_len(size) / (2.0f * std::tan(cam->fov_y / 2.0f));
  for (int i = 0; i < 3; ++i) { cam->eye[i] = center[i] - f[i] * dist; cam->target[i] = center[i]; }
  return VT_OK;
}

static float rotation_theta(const vt_camera* c) { float f[3], r[3], u[3]; cam_basis(c, f, r, u); return std::acos(f[1]); }
static float rotation_phi(const vt_camera* c) { float f[3], r[3], u[3]; cam_basis(c, f, r, u); return std::atan2(f[2], f[0]); }

extern "C" int vt_camera_orbit_mouse(vt_camera* cam, float dx, float dy, int32_t buttons) {
  VT_CHECK_ARG(cam, "camera is null");
  if (buttons & VT_BUTTON_ROTATE) {
    const float theta = dy * (float)M_PI * 1.0f + rotation_theta(cam);
    const float phi = -dx * 2.0f * (float)M_PI * 1.0f + rotation_phi(cam);
    return vt_camera_orbit(cam, theta, phi);
  }
  if (buttons & VT_BUTTON_PAN) {
    float d[3];
    v3_sub(cam->target, cam->eye, d);
    const float dist = v3_len(d);
    return vt_camera_set_distance(cam, dy > 0 ? dist * 1.05f : dist / 1.05f);
  }
  return VT_OK;
}

extern "C" int vt_camera_fly_mouse(vt_camera* cam, float dx, float dy, int32_t buttons) {
  VT_CHECK_ARG(cam, "camera is null");
  if (buttons & VT_BUTTON_ROTATE) {
    const float theta = dy * (float)M_PI * 1.0f + rotation_theta(cam);
    const float phi = -dx * 2.0f * (float)M_PI * 1.0f + rotation_phi(cam);
    return vt_camera_orbit_eye(cam, theta, phi);
  }
  if (buttons & VT_BUTTON_PAN) {
    float f[3], r[3], u[3];
    cam_basis(cam, f, r, u);
    for (int i = 0; i < 3; ++i) { const float m = dy * u[i] * 100.0f; cam->eye[i] += m; cam->target[i] += m; }
  }
  return VT_OK;
}

extern "C" int vt_camera_fly_key(vt_camera* cam, int32_t key) {
  VT_CHECK_ARG(cam, "camera is null");
  float f[3], r[3], u[3];
  cam_basis(cam, f, r, u);
  const float* dir = (key == VT_KEY_FORWARD || key == VT_KEY_BACK) ? f : r;
  const float sgn = (key == VT_KEY_FORWARD || key == VT_KEY_RIGHT) ? 1.0f : -1.0f;
  VT_CHECK_ARG(key >= 0 && key <= 3, "unknown key");
  for (int i = 0; i < 3; ++i) { const float m = dir[i] * 100.0f; cam->eye[i] += sgn * m; cam->target[i] += sgn * m; }
  return VT_OK;
}

// Gauss-Jordan inversion with partial pivoting (the algorithm of
// Imath::Matrix44::gjInverse that M44f::inverse falls back to for
// non-affine matrices, used at renderer.cpp:396-397).  Returns false if singular.
static bool gj_inverse(const float* m, float* out) {
  float t[4][4], s[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) { t[i][j] = m[4 * i + j]; s[i][j] = (i == j) ? 1.0f : 0.0f; }
  for (int i = 0; i < 3; ++i) {
    int pivot = i;
    float pivotsize = std::fabs(t[i][i]);
    for (int j = i + 1; j < 4; ++j) {
      const float tmp = std::fabs(t[j][i]);
      if (tmp > pivotsize) { pivot = j; pivotsize = tmp; }
    }
    if (pivotsize == 0.0f) return false;
    if (pivot != i)
      for (int j = 0; j < 4; ++j) { std::swap(t[i][j], t[pivot][j]); std::swap(s[i][j], s[pivot][j]); }
    for (int j = i + 1; j < 4; ++j) {
      const float f = t[j][i] / t[i][i];
      for (int k = 0; k < 4; ++k) { t[j][k] = t[j][k] - f * t[i][k]; s[j][k] = s[j][k] - f * s[i][k]; }
    }
  }
  for (int i = 3; i >= 0; --i) {
    const float f = t[i][i];
    if (f == 0.0f) return false;
    for (int j = 0; j < 4; ++j) { t[i][j] = t[i][j] / f; s[i][j] = s[i][j] / f; }
    for (int j = 0; j < i; ++j) {
      const float g = t[j][i];
      for (int k = 0; k < 4; ++k) { t[j][k] = t[j][k] - g * t[i][k]; s[j][k] = s[j][k] - g * s[i][k]; }
    }
  }
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) out[4 * i + j] = s[i][j];
  return true;
}

// Renderer::updateCamera (renderer.cpp:343-397).
extern "C" int vt_camera_compute_uniforms(const vt_camera* cam, int32_t w, int32_t h, vt_camera_uniforms* u) {
  VT_CHECK_ARG(cam && u && w > 0 && h > 0, "bad argument");
  float f[3], r[3], up[3];
  cam_basis(cam, f, r, up);
  const float* eye = cam->eye;
  float mv[16] = {r[0], r[1], r[2], -v3_dot(eye, r),
                  up[0], up[1], up[2], -v3_dot(eye, up),
                  -f[0], -f[1], -f[2], v3_dot(eye, f),
                  0.0f, 0.0f, 0.0f, 1.0f};
  float pm[16];
  const float a = (float)w / (float)h;
  if (cam->lens_model == VT_LENS_ORTHOGRAPHIC) {
    float d[3];
    v3_sub(cam->target, cam->eye, d);
    const float dist = v3_len(d);
    const float left = -std::tan(cam->fov_y / 2) * dist;
    const float right = -left;
    const float bottom = -std::tan(cam->fov_y / 2) * dist / a;
    const float top = -bottom;
    const float n = -cam->near_distance;
    const float fr = -cam->far_distance;
    const float tx = -(right + left) / (right - left);
    const float ty = -(top + bottom) / (top - bottom);
    const float tz = -(fr + n) / (fr - n);
    const float p[16] = {2.0f / (right - left), 0, 0, tx,
                         0, 2.0f / (top - bottom), 0, ty,
                         0, 0, -2.0f / (fr - n), tz,
                         0, 0, 0, 1};
    memcpy(pm, p, sizeof(pm));
  } else {
    const float n = cam->near_distance, fr = cam->far_distance;
    const float e = 1.0f / std::tan(cam->fov_y / 2);
    const float p[16] = {e / a, 0, 0, 0,
                         0, e, 0, 0,
                         0, 0, (fr + n) / (n - fr), 2.0f * fr * n / (n - fr),
                         0, 0, -1.0f, 0};
    memcpy(pm, p, sizeof(pm));
  }
  if (!gj_inverse(mv, u->inv_model_view)) return fail(VT_EINVAL, "singular model-view matrix");
  if (!gj_inverse(pm, u->inv_proj)) return fail(VT_EINVAL, "singular projection matrix");
  memcpy(u->proj, pm, sizeof(pm));
  u->viewport[0] = 0.0f; u->viewport[1] = 0.0f; u->viewport[2] = (float)w; u->viewport[3] = (float)h;
  return VT_OK;
}

// ---------------------------------------------------------------- settings
extern "C" int vt_settings_default(vt_render_settings* s) {
  VT_CHECK_ARG(s, "settings is null");
  memset(s, 0, sizeof(*s));
  s->max_bounces = 1;
  s->max_samples = 2048 * 2048;
  s->rr_start_bounce = -1;
  s->gamma = 2.2f;
  s->exposure = 1.0f;
  s->nee_emission_scale = 10.0f;
  s->wireframe_opacity = 0.0f;
  s->wireframe_thickness = 0.01f;
  // pathTracer.fs:25-26
  s->background_top[0] = 153.0f / 255 * 2; s->background_top[1] = 187.0f / 255 * 2; s->background_top[2] = 201.0f / 255 * 2;
  s->background_bottom[0] = 77.0f / 255; s->background_bottom[1] = 64.0f / 255; s->background_bottom[2] = 50.0f / 255;
  s->background_rotation = 0.0f;
  s->selected_voxel[0] = s->selected_voxel[1] = s->selected_voxel[2] = 0;
  s->select_enabled = 0;
  s->ground_material = 0;
  s->quirks = VT_QUIRKS_REFERENCE;
  s->rng_mode = VT_RNG_PHILOX;
  s->seed = 0;
  return VT_OK;
}

static int check_settings(const vt_render_settings* s, const vt_scene* scene) {
  VT_CHECK_ARG(s->max_bounces >= 0 && s->max_bounces <= 1024, "max_bounces out of range");
  VT_CHECK_ARG(s->max_samples >= 1, "max_samples must be >= 1");
  VT_CHECK_ARG(s->gamma > 0.0f, "gamma must be > 0");
  VT_CHECK_ARG(s->rng_mode == VT_RNG_PHILOX || s->rng_mode == VT_RNG_NOISE_TABLE, "unknown rng_mode");
  VT_CHECK_ARG(!scene || (s->ground_material >= 0 && s->ground_material < scene->n_palette),
               "ground_material outside the palette");
  return VT_OK;
}

// -------------------------------------------------------------------- jobs
vt_job::~vt_job() {
  if (!ctx) return;
  ctx->release(sum);
  ctx->release(comp);
  ctx->release(staging);
}

int vt::build_frame(vt_job* j) {
  Frame& F = j->frame;
  memset(&F, 0, sizeof(F));
  const vt_scene* s = j->scene;
  for (int i = 0; i < 3; ++i) {
    F.res[i] = s->res[i];
    F.bmin[i] = s->bmin[i];
    F.bmax[i] = s->bmax[i];
    F.vsize[i] = s->vsize[i];
    F.vext[i] = 1.0f / (s->bmax[i] - s->bmin[i]);
    F.bdim[i] = s->bdim[i];
    F.bsh[i] = s->bsh[i];
  }
  const float len = std::sqrt(((float)s->res[0] * (float)s->res[0] + (float)s->res[1] * (float)s->res[1]) +
                              (float)s->res[2] * (float)s->res[2]);
  F.max_steps = (int32_t)(2.0f * std::ceil(len));
  F.m_res0 = udiv_magic((uint32_t)s->res[0]);
  F.m_res01 = udiv_magic((uint32_t)s->res[0] * (uint32_t)s->res[1]);
  F.m_width = udiv_magic((uint32_t)j->w);
  F.m_pixels = udiv_magic((uint32_t)j->w * (uint32_t)j->h);
  vt_camera_uniforms U;
  int rc = vt_camera_compute_uniforms(&j->cam, j->w, j->h, &U);
  if (rc != VT_OK) return rc;
  memcpy(F.viewport, U.viewport, sizeof(F.viewport));
  memcpy(F.proj, U.proj, sizeof(F.proj));
  memcpy(F.inv_proj, U.inv_proj, sizeof(F.inv_proj));
  memcpy(F.inv_mv, U.inv_model_view, sizeof(F.inv_mv));
  F.frag_z = 0.5f * j->cam.near_distance + 0.5f;
  // screen_to_eye_persp's depth terms at frag_z, in its operation order
  F.persp_ndc_z = ((2.0f * F.frag_z - 0.0f) - 1.0f) / (1.0f - 0.0f);
  F.persp_cw = F.proj[11] / (F.persp_ndc_z - (F.proj[10] / F.proj[14]));
  F.lens_radius = j->cam.lens_radius;
  F.focal_distance = j->cam.focal_distance;
  F.lens_model = j->cam.lens_model;
  const vt_render_settings& S = j->set;
  for (int i = 0; i < 3; ++i) { F.bg_top[i] = S.background_top[i]; F.bg_bottom[i] = S.background_bottom[i]; }
  F.bg_rot = S.background_rotation;
  F.use_image = j->env ? 1 : 0;
  F.env_integral = j->env ? j->env->integral : 0.0f;
  F.env_w = j->env ? j->env->w : 0;
  F.env_h = j->env ? j->env->h : 0;
  F.env_cdf_w = j->env ? j->env->cdf_w : 0;
  F.env_cdf_h = j->env ? j->env->cdf_h : 0;
  F.n_emissive = (int32_t)s->n_emissive;
  F.n_palette = s->n_palette;
  F.max_bounces = S.max_bounces;
  F.rr_start = S.rr_start_bounce;
  F.inv_gamma = 1.0f / S.gamma;
  F.exposure = S.exposure;
  F.nee_scale = S.nee_emission_scale;
  F.wire_opacity = S.wireframe_opacity;
  F.wire_thickness = S.wireframe_thickness;
  for (int i = 0; i < 3; ++i) F.sel[i] = S.selected_voxel[i];
  F.sel_enabled = S.select_enabled;
  F.ground_mat = S.ground_material;
  F.quirks = S.quirks;
  F.rng_mode = S.rng_mode;
  F.seed = S.seed;
  F.width = j->w;
  F.height = j->h;
  F.integrator = j->integrator;
  j->scene_generation = s->generation;
  JobDev& D = j->dev;
  D.grid = s->grid;
  D.bricks = s->bricks;
  D.palette = s->palette;
  D.emissive = s->emissive;
  D.env_texels = j->env ? j->env->texels : nullptr;
  D.cdf_u = j->env ? j->env->cdf_u : nullptr;
  D.cdf_v = j->env ? j->env->cdf_v : nullptr;
  D.noise = j->ctx->noise;
  D.sum = j->sum;
  D.comp = j->comp;
  return VT_OK;
}

static int job_buffers(vt_job* j) {
  j->ctx->release(j->sum);
  j->ctx->release(j->comp);
  j->ctx->release(j->staging);
  j->sum = j->comp = j->staging = nullptr;
  const size_t n = (size_t)j->w * j->h;
  int rc = j->ctx->alloc((void**)&j->sum, sizeof(float4) * n);
  if (rc == VT_OK) rc = j->ctx->alloc((void**)&j->comp, sizeof(float4) * n);
  if (rc != VT_OK) return rc;
  return vt_job_reset(j);
}

extern "C" int vt_job_create(vt_context* ctx, const vt_scene* scene, const vt_env* env, const vt_camera* cam,
                             const vt_render_settings* settings, int32_t w, int32_t h, vt_job** out) {
  VT_CHECK_ARG(ctx && scene && cam && settings && out, "null argument");
  VT_CHECK_ARG(w > 0 && h > 0 && (int64_t)w * h <= ((int64_t)1 << 28), "bad image size");
  *out = nullptr;
  int rc = check_settings(settings, scene);
  if (rc != VT_OK) return rc;
  if (settings->rng_mode == VT_RNG_NOISE_TABLE) {
    rc = ctx->ensure_noise();
    if (rc != VT_OK) return rc;
  }
  vt_job* j = new vt_job();
  j->ctx = ctx;
  j->scene = scene;
  j->env = env;
  j->cam = *cam;
  j->set = *settings;
  j->w = w;
  j->h = h;
  rc = job_buffers(j);
  if (rc == VT_OK) rc = build_frame(j);
  if (rc != VT_OK) { delete j; return rc; }
  *out = j;
  return VT_OK;
}

extern "C" int vt_job_set_camera(vt_job* j, const vt_camera* cam) {
  VT_CHECK_ARG(j && cam, "null argument");
  j->cam = *cam;
  int rc = build_frame(j);
  if (rc != VT_OK) return rc;
  return vt_job_reset(j);
}

extern "C" int vt_job_set_settings(vt_job* j, const vt_render_settings* s) {
  VT_CHECK_ARG(j && s, "null argument");
  int rc = check_settings(s, j->scene);
  if (rc != VT_OK) return rc;
  if (s->rng_mode == VT_RNG_NOISE_TABLE) {
    rc = j->ctx->ensure_noise();
    if (rc != VT_OK) return rc;
  }
  j->set = *s;
  rc = build_frame(j);
  if (rc != VT_OK) return rc;
  return vt_job_reset(j);
}

extern "C" int vt_job_set_scene(vt_job* j, const vt_scene* scene, const vt_env* env) {
  VT_CHECK_ARG(j && scene, "null argument");
  int rc = check_settings(&j->set, scene);
  if (rc != VT_OK) return rc;
  j->scene = scene;
  j->env = env;
  rc = build_frame(j);
  if (rc != VT_OK) return rc;
  return vt_job_reset(j);
}

extern "C" int vt_job_resize(vt_job* j, int32_t w, int32_t h) {
  VT_CHECK_ARG(j && w > 0 && h > 0, "bad argument");
  j->w = w;
  j->h = h;
  int rc = job_buffers(j);
  if (rc != VT_OK) return rc;
  return build_frame(j);
}

extern "C" int vt_job_reset(vt_job* j) {
  VT_CHECK_ARG(j, "job is null");
  const size_t n = (size_t)j->w * j->h;
  cudaSetDevice(j->ctx->device);
  VT_CUDA(cudaMemsetAsync(j->sum, 0, sizeof(float4) * n, j->ctx->stream), "reset");
  VT_CUDA(cudaMemsetAsync(j->comp, 0, sizeof(float4) * n, j->ctx->stream), "reset");
  j->samples = 0;
  return VT_OK;
}

extern "C" int vt_job_set_integrator(vt_job* j, int32_t integrator) {
  VT_CHECK_ARG(j, "job is null");
  VT_CHECK_ARG(integrator == VT_INTEGRATOR_PATH_TRACER || integrator == VT_INTEGRATOR_EDIT_MODE,
               "unknown integrator");
  if (integrator == j->integrator) return VT_OK;
  j->integrator = integrator;
  j->frame.integrator = integrator;
  return vt_job_reset(j);   // the reference restarts the accumulation on a switch (renderer.cpp:678-683)
}

// Launch `passes` samples per pixel for a set of jobs with the selected kernel.
int vt::refresh_job(vt_job* j) {
  if (j->scene && j->scene_generation != j->scene->generation) return build_frame(j);
  return VT_OK;
}

int vt::render_jobs(vt_context* ctx, vt_job* const* jobs, int32_t n, const int32_t* passes, int kernel,
                    int path_slots, int blocks_per_sm, bool count) {
  vt::Range nvtx_range("vt.render");
  cudaSetDevice(ctx->device);
  for (int32_t i = 0; i < n; ++i) {
    const int rc = refresh_job(jobs[i]);
    if (rc != VT_OK) return rc;
  }
  if (count) VT_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(unsigned long long) * C_NUM, ctx->stream), "counters");
  // the plain kernel: every job when asked for, and edit-mode jobs always
  std::vector<vt_job*> wf_jobs;
  std::vector<int32_t> wf_passes;
  for (int i = 0; i < n; ++i) {
    vt_job* j = jobs[i];
    if (kernel != 1 && j->integrator == VT_INTEGRATOR_PATH_TRACER) {
      wf_jobs.push_back(j);
      wf_passes.push_back(passes[i]);
      continue;
    }
    for (int k = 0; k < passes[i]; ++k)
      VT_CUDA(launch_plain(j->frame, j->dev, j->samples + k, 1, count ? ctx->d_counters : nullptr, ctx->stream),
              "plain render");
    ctx->launches += (uint64_t)passes[i];
  }
  if (wf_jobs.empty()) return VT_OK;
  return render_wavefront(ctx, wf_jobs.data(), (int32_t)wf_jobs.size(), wf_passes.data(), path_slots, blocks_per_sm,
                          count);
}

// Device buffers of the wavefront for `slots` path slots and `items` samples.
static int wf_reserve(vt_context* ctx, int64_t slots, int64_t items) {
  if (ctx->wf_slots < slots) {
    ctx->release(ctx->wf_mem);
    ctx->wf_mem = nullptr;
    ctx->wf_slots = 0;
    // two path streams, segment ends, hit records, two segment queues (layout of wf_carve)
    int rc = ctx->alloc(&ctx->wf_mem, (size_t)slots * kWfSlotBytes);
    if (rc != VT_OK) return rc;
    ctx->wf_slots = slots;
  }
  if (ctx->sbuf_items < items) {
    ctx->release(ctx->sbuf);
    ctx->sbuf = nullptr;
    ctx->sbuf_items = 0;
    int rc = ctx->alloc((void**)&ctx->sbuf, sizeof(float4) * (size_t)items);
    if (rc != VT_OK) return rc;
    ctx->sbuf_items = items;
  }
  if (!ctx->wf_ctl) {
    int rc = ctx->alloc((void**)&ctx->wf_ctl, vt_context::kMaxLanes * kCtlBytes);
    if (rc != VT_OK) return rc;
  }
  if (!ctx->lane_ready) {
    cudaError_t e = cudaEventCreateWithFlags(&ctx->lane_ready, cudaEventDisableTiming);
    for (int l = 0; l < vt_context::kMaxLanes - 1 && e == cudaSuccess; ++l) {
      e = cudaStreamCreateWithFlags(&ctx->lane_stream[l], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->lane_done[l], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) return cuda_fail(e, "lane streams");
  }
  if (!ctx->h_live) {
    cudaError_t e = cudaHostAlloc((void**)&ctx->h_live, 64, cudaHostAllocDefault);
    if (e != cudaSuccess) return cuda_fail(e, "cudaHostAlloc");
  }
  return VT_OK;
}

// One wavefront launch over `entries` (tile_begin = first item of each job).
static int wf_launch(vt_context* ctx, std::vector<JobEntry>& entries, const std::vector<Grid>& grids,
                     int64_t items, int64_t slots_cap, int blocks_per_sm, bool count) {
  vt::Range nvtx_range("vt.wavefront_launch");
  const int64_t slots = std::max<int64_t>(32, std::min<int64_t>(items, slots_cap));
  int rc = wf_reserve(ctx, slots, items);
  if (rc != VT_OK) return rc;
  const size_t jbytes = sizeof(JobEntry) * entries.size();
  if (ctx->d_jobs_bytes < jbytes) {
    ctx->release(ctx->d_jobs);
    ctx->d_jobs = nullptr;
    ctx->d_jobs_bytes = 0;
    rc = ctx->alloc((void**)&ctx->d_jobs, jbytes);
    if (rc != VT_OK) return rc;
    ctx->d_jobs_bytes = jbytes;
  }
  const size_t gbytes = sizeof(Grid) * grids.size();
  if (ctx->d_grids_bytes < gbytes) {
    ctx->release(ctx->d_grids);
    ctx->d_grids = nullptr;
    ctx->d_grids_bytes = 0;
    rc = ctx->alloc((void**)&ctx->d_grids, gbytes);
    if (rc != VT_OK) return rc;
    ctx->d_grids_bytes = gbytes;
  }
  cudaStream_t st = ctx->stream;
  VT_CUDA(cudaMemcpyAsync(ctx->d_jobs, entries.data(), jbytes, cudaMemcpyHostToDevice, st), "job table");
  VT_CUDA(cudaMemcpyAsync(ctx->d_grids, grids.data(), gbytes, cudaMemcpyHostToDevice, st), "grid table");
  WfJobTable table;
  const WfJobTable* T = nullptr;
  if (entries.size() <= (size_t)kWfParamJobs) {
    memset(&table, 0, sizeof(table));
    for (size_t i = 0; i < entries.size(); ++i) {
      table.e[i] = entries[i];
      table.g[i] = grids[i];
    }
    T = &table;
  }
  bool all_444 = true;   // the DDA kernel's fixed-shape form applies
  for (const Grid& g : grids) all_444 = all_444 && g.shx == 2 && g.shy == 2 && g.shz == 2;
  // Lanes: independent wavefronts over equal shares of the items, each with
  // its share of the path slots and its own stream, so that one lane's
  // memory-bound shading overlaps another's ALU-bound DDA.
  int lanes = ctx->lanes;
  while (lanes > 1 && (items < 4096 * (int64_t)lanes || slots < 1024 * (int64_t)lanes)) --lanes;
  const size_t lane_slots = lanes > 1 ? ((size_t)slots / lanes) & ~(size_t)31 : (size_t)slots;   // 256-byte lane bases
  cudaStream_t lane_st[vt_context::kMaxLanes] = {st, ctx->lane_stream[0], ctx->lane_stream[1], ctx->lane_stream[2]};
  WfParams P[vt_context::kMaxLanes];
  for (int l = 0; l < lanes; ++l) {
    memset(&P[l], 0, sizeof(P[l]));
    P[l].jobs = ctx->d_jobs;
    P[l].n_jobs = (int32_t)entries.size();
    P[l].grids = ctx->d_grids;
    wf_carve((char*)ctx->wf_mem + (size_t)l * lane_slots * kWfSlotBytes, lane_slots, P[l]);
    P[l].n_slots = (int32_t)lane_slots;
    P[l].ctl = ctx->wf_ctl + (size_t)l * (kCtlBytes / sizeof(uint32_t));
    P[l].next_item = (unsigned long long*)(P[l].ctl + kCtlNextItem);
    P[l].n_items = (unsigned long long)(l + 1 == lanes ? items : items / lanes * (l + 1));
    P[l].sbuf = ctx->sbuf;
    P[l].counters = count ? ctx->d_counters : nullptr;
    P[l].trace_chunk = (uint32_t)ctx->trace_chunk;
    P[l].refill_min = ctx->refill_min;
    P[l].bricks_444 = all_444 ? 1 : 0;
    P[l].trace_form = ctx->trace_form;
  }
  // control words zero (first stream empty), item counters at each lane's first item
  VT_CUDA(cudaMemsetAsync(ctx->wf_ctl, 0, vt_context::kMaxLanes * kCtlBytes, st), "wavefront control");
  for (int l = 1; l < lanes; ++l) {
    const unsigned long long begin = (unsigned long long)(items / lanes * l);
    VT_CUDA(cudaMemcpyAsync(P[l].next_item, &begin, sizeof(begin), cudaMemcpyHostToDevice, st),
            "lane items");   // pageable source: read when the call returns
  }
  if (ctx->trace_occupancy <= 0) ctx->trace_occupancy = std::max(1, wf_trace_blocks_per_sm());
  int bps = blocks_per_sm > 0 ? blocks_per_sm
                              : (ctx->trace_blocks_per_sm > 0 ? ctx->trace_blocks_per_sm : ctx->trace_occupancy);
  if (lanes > 1 && blocks_per_sm <= 0 && ctx->trace_blocks_per_sm <= 0) bps = std::max(1, bps * 2 / 3);
  const int trace_blocks = ctx->sm_count * bps;
  // Eight rounds of every lane: per round and lane its counters cleared,
  // shade + hit + regen, trace.  The other lanes' streams fork from the
  // first and join it again, so the group is one unit of work on `st` (one
  // CUDA graph when graphs are on); within it the lanes run free of each
  // other.
  auto group = [&]() -> cudaError_t {
    cudaError_t e = cudaSuccess;
    if (lanes > 1) e = cudaEventRecord(ctx->lane_ready, st);
    for (int l = 1; l < lanes && e == cudaSuccess; ++l) e = cudaStreamWaitEvent(lane_st[l], ctx->lane_ready, 0);
    for (int r = 0; r < 8 && e == cudaSuccess; ++r) {
      const int par = r & 1;
      for (int l = 0; l < lanes && e == cudaSuccess; ++l) {
        e = cudaMemsetAsync(P[l].ctl + ctl_index(par, 0), 0, CTL_PER_PARITY * kCtlStride * sizeof(uint32_t),
                            lane_st[l]);
        if (e == cudaSuccess) e = launch_wf_shade(P[l], par, ctx->sm_count * 8, count, lane_st[l], T);
        if (e == cudaSuccess) e = launch_wf_trace(P[l], par, trace_blocks, ctx->trace_steps, count, lane_st[l], T);
      }
    }
    for (int l = 1; l < lanes && e == cudaSuccess; ++l) {
      e = cudaEventRecord(ctx->lane_done[l - 1], lane_st[l]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ctx->lane_done[l - 1], 0);
    }
    return e;
  };
  if (ctx->use_graphs) {
    cudaGraph_t graph = nullptr;
    VT_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "capture rounds");
    const cudaError_t ce = group();
    const cudaError_t ee = cudaStreamEndCapture(st, &graph);
    if (ce != cudaSuccess || ee != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      return cuda_fail(ce != cudaSuccess ? ce : ee, "capture rounds");
    }
    cudaGraphExec_t& exec = ctx->rounds_exec;
    bool updated = false;
    if (exec) {
      cudaGraphExecUpdateResultInfo info;
      updated = cudaGraphExecUpdate(exec, graph, &info) == cudaSuccess;
      if (!updated) {
        cudaGetLastError();
        cudaGraphExecDestroy(exec);
        exec = nullptr;
      }
    }
    if (!updated) {
      const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
      if (ie != cudaSuccess) {
        cudaGraphDestroy(graph);
        exec = nullptr;
        return cuda_fail(ie, "instantiate rounds");
      }
    }
    cudaGraphDestroy(graph);
  }
  // Groups run until every lane's next stream is empty (its items are done;
  // a finished lane's rounds find nothing to do).  A path ends within
  // max_bounces + 2 rounds of its start, so every such span of rounds frees
  // a full lane's slots for new paths while items remain: a lane drains
  // within (items / slots + 2) * (max_bounces + 2) rounds.  Four times that
  // bounds the loop, so a fault in the kernels' bookkeeping ends the call
  // with an error instead of looping.
  int32_t max_b = 0;
  for (const JobEntry& e : entries) max_b = std::max(max_b, e.F.max_bounces);
  const int64_t lane_items = (items + lanes - 1) / lanes;
  const int64_t drain_rounds = (lane_items / (int64_t)lane_slots + 2) * ((int64_t)max_b + 2);
  const int64_t max_groups = 4 * (drain_rounds + 7) / 8 + 4;
  for (int64_t group_n = 0;; ++group_n) {
    if (group_n >= max_groups)
      return fail(VT_EDEVICE, "wavefront did not drain within %lld rounds", (long long)(8 * max_groups));
    vt::Range rounds_range("vt.rounds");   // eight rounds of every lane, then the live-count check
    if (ctx->use_graphs) {
      VT_CUDA(cudaGraphLaunch(ctx->rounds_exec, st), "wavefront rounds");
    } else {
      VT_CUDA(group(), "wavefront rounds");
    }
    ctx->launches += (uint64_t)lanes * 8 * 4;
    for (int l = 0; l < lanes; ++l)
      VT_CUDA(cudaMemcpyAsync(ctx->h_live + l, P[l].ctl + ctl_index(1, CTL_NEXT_N), sizeof(uint32_t),
                              cudaMemcpyDeviceToHost, st),
              "stream length");
    VT_CUDA(cudaStreamSynchronize(st), "wavefront rounds");
    bool any = false;
    for (int l = 0; l < lanes; ++l) any = any || ((volatile uint32_t*)ctx->h_live)[l] != 0;
    if (!any) break;
  }
  long long max_pixels = 0;
  for (const JobEntry& e : entries) max_pixels = std::max<long long>(max_pixels, e.n_pixels);
  vt::Range acc_range("vt.accumulate");
  VT_CUDA(launch_wf_accumulate(ctx->d_jobs, (int)entries.size(), max_pixels, ctx->sbuf, st), "accumulate");
  ctx->launches += 1;
  return VT_OK;
}

// Wavefront rendering of passes[i] samples per pixel for each job, split in
// launches whose sample buffers stay within ctx->max_items.
int vt::render_wavefront(vt_context* ctx, vt_job* const* jobs, int32_t n, const int32_t* passes, int slots,
                         int blocks_per_sm, bool count) {
  if (n > kWfMaxJobs) {   // launches of at most kWfMaxJobs jobs
    for (int32_t i = 0; i < n; i += kWfMaxJobs) {
      const int rc = render_wavefront(ctx, jobs + i, std::min<int32_t>(kWfMaxJobs, n - i), passes + i, slots,
                                      blocks_per_sm, count);
      if (rc != VT_OK) return rc;
    }
    return VT_OK;
  }
  std::vector<int32_t> done(n, 0);
  const int64_t slots_cap = slots > 0 ? slots : ctx->max_slots;
  for (;;) {
    int64_t pix_left = 0;
    for (int i = 0; i < n; ++i)
      if (done[i] < passes[i]) pix_left += (int64_t)jobs[i]->w * jobs[i]->h;
    if (pix_left == 0) break;
    const int32_t q = (int32_t)std::max<int64_t>(1, ctx->max_items / pix_left);
    std::vector<JobEntry> entries;
    std::vector<Grid> grids;
    int64_t items = 0;
    for (int i = 0; i < n; ++i) {
      const int32_t p = std::min(q, passes[i] - done[i]);
      if (p <= 0) continue;
      JobEntry e;
      memset(&e, 0, sizeof(e));
      e.F = jobs[i]->frame;
      e.J = jobs[i]->dev;
      e.sample_base = jobs[i]->samples + done[i];
      e.passes = p;
      e.tile_begin = items;
      e.n_pixels = (int64_t)jobs[i]->w * jobs[i]->h;
      items += e.n_pixels * p;
      entries.push_back(e);
      grids.push_back(make_grid(jobs[i]->frame, jobs[i]->dev.bricks));
      done[i] += p;
    }
    if (items >= ((int64_t)1 << 32)) return fail(VT_EINVAL, "more than 2^32 samples in one launch");
    int rc = wf_launch(ctx, entries, grids, items, slots_cap, blocks_per_sm, count);
    if (rc != VT_OK) return rc;
  }
  return VT_OK;
}

static int job_passes(const vt_job* j, int32_t want) {
  const int left = j->set.max_samples - j->samples;
  return std::max(0, std::min(want, left));
}

extern "C" int vt_job_render(vt_job* j, int32_t passes, int32_t* result) {
  VT_CHECK_ARG(j && passes >= 0, "bad argument");
  const int32_t n = job_passes(j, passes);
  int rc = render_jobs(j->ctx, &j, 1, &n, j->ctx->kernel, 0, 0, false);
  if (rc != VT_OK) return rc;
  j->samples += n;
  if (result) *result = j->samples >= j->set.max_samples ? VT_FINISHED_RENDERING : VT_SAMPLES_PENDING;
  return VT_OK;
}

extern "C" int vt_job_synchronize(vt_job* j) {
  VT_CHECK_ARG(j, "job is null");
  cudaSetDevice(j->ctx->device);
  VT_CUDA(cudaStreamSynchronize(j->ctx->stream), "synchronize");
  return VT_OK;
}

extern "C" int vt_job_sample_count(const vt_job* j, int32_t* samples) {
  VT_CHECK_ARG(j && samples, "null argument");
  *samples = j->samples;
  return VT_OK;
}

extern "C" int vt_job_readback(vt_job* j, float* rgba, size_t bytes, uint32_t flags) {
  vt::Range nvtx_range("vt.readback");
  VT_CHECK_ARG(j && rgba, "null argument");
  const size_t n = (size_t)j->w * j->h;
  VT_CHECK_ARG(bytes >= n * sizeof(float4), "output buffer too small");
  cudaSetDevice(j->ctx->device);
  if (!j->staging) {
    int rc = j->ctx->alloc((void**)&j->staging, sizeof(float4) * n);
    if (rc != VT_OK) return rc;
  }
  VT_CUDA(launch_resolve(j->sum, j->w, j->h, j->samples, j->set.exposure, 1.0f / j->set.gamma, flags, j->staging,
                         j->ctx->stream), "resolve");
  VT_CUDA(cudaMemcpyAsync(rgba, j->staging, sizeof(float4) * n, cudaMemcpyDeviceToHost, j->ctx->stream), "readback");
  VT_CUDA(cudaStreamSynchronize(j->ctx->stream), "readback");
  return VT_OK;
}

extern "C" int vt_job_snapshot(const vt_job* j, float* sum, float* comp, size_t bytes_each, int32_t* samples) {
  VT_CHECK_ARG(j && sum && comp && samples, "null argument");
  const size_t n = (size_t)j->w * j->h;
  VT_CHECK_ARG(bytes_each >= n * sizeof(float4), "output buffers too small: width*height*4 floats each");
  cudaSetDevice(j->ctx->device);
  VT_CUDA(cudaMemcpyAsync(sum, j->sum, sizeof(float4) * n, cudaMemcpyDeviceToHost, j->ctx->stream), "snapshot");
  VT_CUDA(cudaMemcpyAsync(comp, j->comp, sizeof(float4) * n, cudaMemcpyDeviceToHost, j->ctx->stream), "snapshot");
  VT_CUDA(cudaStreamSynchronize(j->ctx->stream), "snapshot");
  *samples = j->samples;
  return VT_OK;
}

extern "C" int vt_job_restore(vt_job* j, const float* sum, const float* comp, size_t bytes_each, int32_t samples) {
  VT_CHECK_ARG(j && sum && comp, "null argument");
  const size_t n = (size_t)j->w * j->h;
  VT_CHECK_ARG(bytes_each >= n * sizeof(float4), "input buffers too small: width*height*4 floats each");
  VT_CHECK_ARG(samples >= 0 && samples <= j->set.max_samples, "sample count out of range [0, max_samples]");
  cudaSetDevice(j->ctx->device);
  VT_CUDA(cudaMemcpyAsync(j->sum, sum, sizeof(float4) * n, cudaMemcpyHostToDevice, j->ctx->stream), "restore");
  VT_CUDA(cudaMemcpyAsync(j->comp, comp, sizeof(float4) * n, cudaMemcpyHostToDevice, j->ctx->stream), "restore");
  VT_CUDA(cudaStreamSynchronize(j->ctx->stream), "restore");
  j->samples = samples;
  return VT_OK;
}

extern "C" int vt_job_device_buffer(vt_job* j, void** sums, int32_t* samples) {
  VT_CHECK_ARG(j, "job is null");
  if (sums) *sums = j->sum;
  if (samples) *samples = j->samples;
  return VT_OK;
}

extern "C" int vt_job_pick(vt_job* j, float x, float y, float* distance, int32_t voxel[3]) {
  VT_CHECK_ARG(j && distance, "null argument");
  {
    const int rc0 = refresh_job(j);
    if (rc0 != VT_OK) return rc0;
  }
  cudaSetDevice(j->ctx->device);
  int rc = j->ctx->ensure_scratch(64);
  if (rc != VT_OK) return rc;
  float* d_dist = (float*)j->ctx->scratch;
  int32_t* d_vox = (int32_t*)((char*)j->ctx->scratch + 16);
  VT_CUDA(launch_pick(j->frame, j->dev, x, y, d_dist, d_vox, j->ctx->stream), "pick");
  int32_t v[3];
  VT_CUDA(cudaMemcpyAsync(distance, d_dist, sizeof(float), cudaMemcpyDeviceToHost, j->ctx->stream), "pick");
  VT_CUDA(cudaMemcpyAsync(v, d_vox, sizeof(v), cudaMemcpyDeviceToHost, j->ctx->stream), "pick");
  VT_CUDA(cudaStreamSynchronize(j->ctx->stream), "pick");
  if (voxel) { voxel[0] = v[0]; voxel[1] = v[1]; voxel[2] = v[2]; }
  return VT_OK;
}

// ------------------------------------------------------------- voxel edits
extern "C" int vt_scene_set_voxel(vt_scene* s, int32_t x, int32_t y, int32_t z, int32_t entry) {
  VT_CHECK_ARG(s, "scene is null");
  VT_CHECK_ARG(x >= 0 && y >= 0 && z >= 0 && x < s->res[0] && y < s->res[1] && z < s->res[2],
               "voxel outside the volume");
  VT_CHECK_ARG(entry >= 0 && entry <= s->n_palette, "entry outside the palette");
  vt_context* ctx = s->ctx;
  cudaSetDevice(ctx->device);
  const int64_t idx = (int64_t)x + (int64_t)s->res[0] * ((int64_t)y + (int64_t)s->res[1] * z);
  VT_CUDA(launch_set_voxel(s->grid, s->bricks, s->res[0], s->res[1], s->bdim[0], s->bdim[1], scene_shape(s), x, y,
                           z, (uint8_t)entry, ctx->stream), "voxel edit");
  int rc = VT_OK;
  if (s->flags & VT_SCENE_AUTO_EMISSIVE) {
    rc = scene_emissive(ctx, s, nullptr, 0, s->flags);          // rediscover from the palette
  } else if (s->n_emissive > 0 && entry == 0) {
    std::vector<int32_t> list((size_t)s->n_emissive);           // an emptied voxel leaves the caller's list
    VT_CUDA(cudaMemcpyAsync(list.data(), s->emissive, sizeof(int32_t) * list.size(), cudaMemcpyDeviceToHost,
                            ctx->stream), "emissive list");
    VT_CUDA(cudaStreamSynchronize(ctx->stream), "emissive list");
    list.erase(std::remove(list.begin(), list.end(), (int32_t)idx), list.end());
    if ((int64_t)list.size() != s->n_emissive) rc = scene_emissive(ctx, s, list.data(), (int64_t)list.size(), 0);
  }
  if (rc != VT_OK) return rc;
  VT_CUDA(cudaStreamSynchronize(ctx->stream), "voxel edit");
  s->generation += 1;
  return VT_OK;
}

// RendererServiceSelectActiveVoxel (selectVoxel.vs:35-69).
static int select_voxel(vt_job* j, float x, float y, int32_t voxel[3], float normal[3], bool* hit) {
  vt_context* ctx = j->ctx;
  cudaSetDevice(ctx->device);
  int rc = refresh_job(j);
  if (rc != VT_OK) return rc;
  rc = ctx->ensure_scratch(64);
  if (rc != VT_OK) return rc;
  int32_t* d = (int32_t*)ctx->scratch;
  VT_CUDA(launch_select(j->frame, j->dev, x, y, j->cam.near_distance, d, ctx->stream), "select voxel");
  int32_t out[8];
  VT_CUDA(cudaMemcpyAsync(out, d, sizeof(out), cudaMemcpyDeviceToHost, ctx->stream), "select voxel");
  VT_CUDA(cudaStreamSynchronize(ctx->stream), "select voxel");
  for (int i = 0; i < 3; ++i) {
    voxel[i] = out[i];
    memcpy(&normal[i], &out[4 + i], sizeof(float));
  }
  *hit = out[3] != 0;
  return VT_OK;
}

extern "C" int vt_job_select_voxel(vt_job* j, float x, float y, int32_t voxel[3], float normal[3]) {
  VT_CHECK_ARG(j && voxel && normal, "null argument");
  bool hit = false;
  return select_voxel(j, x, y, voxel, normal, &hit);
}

static bool inside(const vt_scene* s, const int32_t v[3]) {
  return v[0] >= 0 && v[1] >= 0 && v[2] >= 0 && v[0] < s->res[0] && v[1] < s->res[1] && v[2] < s->res[2];
}

// GLSL step(a, b) * step(c, b) * sign(b) per component: the dominant axes of v.
static void axis_mask(const float v[3], float out[3]) {
  const float a[3] = {std::fabs(v[0]), std::fabs(v[1]), std::fabs(v[2])};
  const float mx = (!(a[0] < a[1]) && !(a[0] < a[2])) ? 1.0f : 0.0f;
  const float my = (!(a[1] < a[0]) && !(a[1] < a[2])) ? 1.0f : 0.0f;
  const float mz = (!(a[2] < a[0]) && !(a[2] < a[1])) ? 1.0f : 0.0f;
  out[0] = mx * vtb::gsign(v[0]); out[1] = my * vtb::gsign(v[1]); out[2] = mz * vtb::gsign(v[2]);
}

extern "C" int vt_job_add_voxel(vt_job* j, float x, float y, float dx, float dy, int32_t restart,
                                int32_t voxel[3]) {
  VT_CHECK_ARG(j && voxel, "null argument");
  int32_t sel[3];
  float n[3];
  bool hit = false;
  int rc = select_voxel(j, x, y, sel, n, &hit);
  if (rc != VT_OK) return rc;
  voxel[0] = voxel[1] = voxel[2] = -1;
  if (!hit) return VT_OK;
  // addVoxel.vs:16-41: with screen-space motion, the axis of the camera's
  // right / up vector nearest the dominant motion; otherwise the hit normal
  if (dx != 0.0f || dy != 0.0f) {
    const float* M = j->frame.inv_mv;   // row-major: columns are the camera axes
    const float right[3] = {M[0], M[4], M[8]}, up[3] = {M[1], M[5], M[9]};
    float ar[3], au[3];
    axis_mask(right, ar);
    axis_mask(up, au);
    const float ax = std::fabs(dx), ay = std::fabs(dy);
    const float mdx = (!(ax < ay) ? 1.0f : 0.0f) * vtb::gsign(dx);
    const float mdy = (!(ay < ax) ? 1.0f : 0.0f) * vtb::gsign(dy);
    for (int i = 0; i < 3; ++i) n[i] = ar[i] * mdx + au[i] * mdy;
  }
  int32_t c[3];
  for (int i = 0; i < 3; ++i) c[i] = sel[i] + (int32_t)n[i];
  if (!inside(j->scene, c)) return VT_OK;       // imageStore outside the image writes nothing
  // the new voxel copies the selected voxel's material (the ground's below the volume)
  int32_t entry = j->set.ground_material + 1;
  if (inside(j->scene, sel)) {
    const int64_t idx = (int64_t)sel[0] + (int64_t)j->scene->res[0] * ((int64_t)sel[1] + (int64_t)j->scene->res[1] * sel[2]);
    uint8_t e = 0;
    VT_CUDA(cudaMemcpyAsync(&e, j->scene->grid + idx, 1, cudaMemcpyDeviceToHost, j->ctx->stream), "selected voxel");
    VT_CUDA(cudaStreamSynchronize(j->ctx->stream), "selected voxel");
    if (e) entry = e;
  }
  rc = vt_scene_set_voxel(const_cast<vt_scene*>(j->scene), c[0], c[1], c[2], entry);
  if (rc != VT_OK) return rc;
  for (int i = 0; i < 3; ++i) voxel[i] = c[i];
  if (restart) rc = vt_job_reset(j);
  return rc;
}

extern "C" int vt_job_remove_voxel(vt_job* j, float x, float y, int32_t restart, int32_t voxel[3]) {
  VT_CHECK_ARG(j && voxel, "null argument");
  int32_t sel[3];
  float n[3];
  bool hit = false;
  int rc = select_voxel(j, x, y, sel, n, &hit);
  if (rc != VT_OK) return rc;
  voxel[0] = voxel[1] = voxel[2] = -1;
  if (!hit || !inside(j->scene, sel)) return VT_OK;   // nothing, or the implicit ground
  rc = vt_scene_set_voxel(const_cast<vt_scene*>(j->scene), sel[0], sel[1], sel[2], 0);
  if (rc != VT_OK) return rc;
  for (int i = 0; i < 3; ++i) voxel[i] = sel[i];
  if (restart) rc = vt_job_reset(j);
  return rc;
}

extern "C" int vt_job_destroy(vt_job* j) {
  if (!j) return VT_OK;
  cudaSetDevice(j->ctx->device);
  cudaStreamSynchronize(j->ctx->stream);
  delete j;
  return VT_OK;
}

// ---------------------------------------------------------------- batching
extern "C" int vt_render_batch(vt_context* ctx, vt_job* const* jobs, int32_t n_jobs, int32_t passes,
                               const vt_batch_opts* opts, int32_t* results) {
  VT_CHECK_ARG(ctx && (n_jobs == 0 || jobs) && n_jobs >= 0 && passes >= 0, "bad argument");
  std::vector<int32_t> np(n_jobs);
  for (int i = 0; i < n_jobs; ++i) {
    VT_CHECK_ARG(jobs[i] && jobs[i]->ctx == ctx, "job is null or belongs to another context");
    np[i] = job_passes(jobs[i], passes);
  }
  const int kernel = (opts && opts->kernel) ? opts->kernel : ctx->kernel;
  int rc = render_jobs(ctx, jobs, n_jobs, np.data(), kernel, opts ? opts->path_slots : 0,
                       opts ? opts->blocks_per_sm : 0, false);
  if (rc != VT_OK) return rc;
  for (int i = 0; i < n_jobs; ++i) {
    jobs[i]->samples += np[i];
    if (results) results[i] = jobs[i]->samples >= jobs[i]->set.max_samples ? VT_FINISHED_RENDERING : VT_SAMPLES_PENDING;
  }
  return VT_OK;
}

// ------------------------------------------------------------- diagnostics
extern "C" int vt_diag_trace_rays(vt_job* j, const float* origins, const float* dirs, int64_t n, int32_t* out) {
  VT_CHECK_ARG(j && (n == 0 || (origins && dirs && out)) && n >= 0, "bad argument");
  {
    const int rc0 = refresh_job(j);
    if (rc0 != VT_OK) return rc0;
  }
  if (n == 0) return VT_OK;
  vt_context* ctx = j->ctx;
  cudaSetDevice(ctx->device);
  const size_t bin = sizeof(float) * 3 * n, bout = sizeof(int32_t) * 4 * n;
  int rc = ctx->ensure_scratch(2 * bin + bout + 512);
  if (rc != VT_OK) return rc;
  char* base = (char*)ctx->scratch;
  float* d_o = (float*)base;
  float* d_d = (float*)(base + ((bin + 255) & ~(size_t)255));
  int32_t* d_out = (int32_t*)(base + 2 * ((bin + 255) & ~(size_t)255));
  VT_CUDA(cudaMemcpyAsync(d_o, origins, bin, cudaMemcpyHostToDevice, ctx->stream), "rays");
  VT_CUDA(cudaMemcpyAsync(d_d, dirs, bin, cudaMemcpyHostToDevice, ctx->stream), "rays");
  VT_CUDA(launch_trace_rays(j->frame, j->dev, d_o, d_d, n, d_out, ctx->stream), "trace rays");
  VT_CUDA(cudaMemcpyAsync(out, d_out, bout, cudaMemcpyDeviceToHost, ctx->stream), "rays");
  VT_CUDA(cudaStreamSynchronize(ctx->stream), "rays");
  return VT_OK;
}

extern "C" int vt_diag_samples(vt_job* j, int32_t sample, float* rgba, int32_t* hits, uint64_t* counters) {
  VT_CHECK_ARG(j && rgba && sample >= 0, "bad argument");
  {
    const int rc0 = refresh_job(j);
    if (rc0 != VT_OK) return rc0;
  }
  vt_context* ctx = j->ctx;
  cudaSetDevice(ctx->device);
  const size_t n = (size_t)j->w * j->h;
  const size_t b1 = (sizeof(float4) * n + 255) & ~(size_t)255;
  int rc = ctx->ensure_scratch(b1 + sizeof(HitRecord) * n + 256);
  if (rc != VT_OK) return rc;
  float4* d_out = (float4*)ctx->scratch;
  HitRecord* d_hits = (HitRecord*)((char*)ctx->scratch + b1);
  VT_CUDA(cudaMemsetAsync(ctx->d_counters, 0, sizeof(unsigned long long) * C_NUM, ctx->stream), "counters");
  VT_CUDA(launch_diag(j->frame, j->dev, sample, d_out, d_hits, ctx->d_counters, ctx->stream), "diag samples");
  VT_CUDA(cudaMemcpyAsync(rgba, d_out, sizeof(float4) * n, cudaMemcpyDeviceToHost, ctx->stream), "diag");
  if (hits) VT_CUDA(cudaMemcpyAsync(hits, d_hits, sizeof(HitRecord) * n, cudaMemcpyDeviceToHost, ctx->stream), "diag");
  if (counters)
    VT_CUDA(cudaMemcpyAsync(counters, ctx->d_counters, sizeof(unsigned long long) * C_NUM, cudaMemcpyDeviceToHost,
                            ctx->stream), "diag");
  VT_CUDA(cudaStreamSynchronize(ctx->stream), "diag");
  return VT_OK;
}

extern "C" int vt_diag_render_counted(vt_job* j, int32_t passes, uint64_t* counters, int32_t* result) {
  VT_CHECK_ARG(j && counters && passes >= 0, "bad argument");
  const int32_t n = job_passes(j, passes);
  int rc = render_jobs(j->ctx, &j, 1, &n, j->ctx->kernel, 0, 0, true);
  if (rc != VT_OK) return rc;
  j->samples += n;
  VT_CUDA(cudaMemcpyAsync(counters, j->ctx->d_counters, sizeof(unsigned long long) * C_NUM, cudaMemcpyDeviceToHost,
                          j->ctx->stream), "counters");
  VT_CUDA(cudaStreamSynchronize(j->ctx->stream), "counters");
  if (result) *result = j->samples >= j->set.max_samples ? VT_FINISHED_RENDERING : VT_SAMPLES_PENDING;
  return VT_OK;
}

extern "C" int vt_diag_set_lanes(vt_context* ctx, int32_t lanes) {
  VT_CHECK_ARG(ctx && lanes >= 1 && lanes <= vt_context::kMaxLanes, "lanes must be 1 to 4");
  ctx->lanes = lanes;
  return VT_OK;
}

extern "C" int vt_diag_set_graphs(vt_context* ctx, int32_t enabled) {
  VT_CHECK_ARG(ctx, "context is null");
  ctx->use_graphs = enabled != 0;
  return VT_OK;
}

extern "C" int vt_diag_set_kernel(vt_context* ctx, int32_t kernel) {
  VT_CHECK_ARG(ctx && (kernel == 1 || kernel == 2), "kernel must be 1 (plain) or 2 (wavefront)");
  ctx->kernel = kernel;
  return VT_OK;
}

extern "C" int vt_diag_builtins(vt_context* ctx, int32_t fn, const float* a, const float* b, float* out, int64_t n) {
  VT_CHECK_ARG(ctx && a && out && n >= 0, "bad argument");
  if (n == 0) return VT_OK;
  cudaSetDevice(ctx->device);
  const size_t bytes = sizeof(float) * n, al = (bytes + 255) & ~(size_t)255;
  int rc = ctx->ensure_scratch(3 * al);
  if (rc != VT_OK) return rc;
  float* da = (float*)ctx->scratch;
  float* db = (float*)((char*)ctx->scratch + al);
  float* dout = (float*)((char*)ctx->scratch + 2 * al);
  VT_CUDA(cudaMemcpyAsync(da, a, bytes, cudaMemcpyHostToDevice, ctx->stream), "builtins");
  VT_CUDA(cudaMemcpyAsync(db, b ? b : a, bytes, cudaMemcpyHostToDevice, ctx->stream), "builtins");
  VT_CUDA(launch_builtins(fn, da, db, dout, n, ctx->stream), "builtins");
  VT_CUDA(cudaMemcpyAsync(out, dout, bytes, cudaMemcpyDeviceToHost, ctx->stream), "builtins");
  VT_CUDA(cudaStreamSynchronize(ctx->stream), "builtins");
  return VT_OK;
}

extern "C" int vt_scene_set_brick_shape(vt_scene* s, int32_t sx, int32_t sy, int32_t sz) {
  VT_CHECK_ARG(s, "scene is null");
  // every extent at least 2: the padded border is then at least two voxels
  // deep, which the DDA's look-ahead by one cell beyond an exit relies on
  VT_CHECK_ARG(sx >= 1 && sy >= 1 && sz >= 1 && sx <= 4 && sy <= 4 && sz <= 4 && sx + sy + sz == 6,
               "brick shape: log2 extents in [1, 4] that sum to 6 (64 voxels a brick)");
  if (sx == s->bsh[0] && sy == s->bsh[1] && sz == s->bsh[2]) return VT_OK;
  vt_context* ctx = s->ctx;
  cudaSetDevice(ctx->device);
  const int32_t old[3] = {s->bsh[0], s->bsh[1], s->bsh[2]};
  s->bsh[0] = sx; s->bsh[1] = sy; s->bsh[2] = sz;
  int32_t bdim[3];
  for (int i = 0; i < 3; ++i) bdim[i] = (s->res[i] + (1 << s->bsh[i]) - 1) >> s->bsh[i];
  const int64_t nb = (int64_t)(bdim[0] + 2) * (bdim[1] + 2) * (bdim[2] + 2);
  unsigned long long* bricks = nullptr;
  int rc = ctx->alloc((void**)&bricks, sizeof(unsigned long long) * nb);
  if (rc != VT_OK) { for (int i = 0; i < 3; ++i) s->bsh[i] = old[i]; return rc; }
  cudaError_t e = launch_build_bricks(s->grid, s->res[0], s->res[1], s->res[2], bricks, bdim[0], bdim[1], bdim[2],
                                      scene_shape(s), nullptr, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    ctx->release(bricks);
    for (int i = 0; i < 3; ++i) s->bsh[i] = old[i];
    return cuda_fail(e, "brick rebuild");
  }
  const int64_t old_nb = (int64_t)(s->bdim[0] + 2) * (s->bdim[1] + 2) * (s->bdim[2] + 2);
  ctx->release(s->bricks);
  s->bricks = bricks;
  for (int i = 0; i < 3; ++i) s->bdim[i] = bdim[i];
  s->bytes = s->bytes - sizeof(unsigned long long) * (uint64_t)old_nb + sizeof(unsigned long long) * (uint64_t)nb;
  s->generation++;   // jobs on this scene rebuild their frames before their next pass
  return VT_OK;
}

extern "C" int vt_scene_get_brick_shape(const vt_scene* s, int32_t* shape) {
  VT_CHECK_ARG(s && shape, "null argument");
  for (int i = 0; i < 3; ++i) shape[i] = s->bsh[i];
  return VT_OK;
}

extern "C" int vt_diag_scene_bricks(const vt_scene* s, uint64_t* out, size_t bytes, int64_t* n_words) {
  VT_CHECK_ARG(s && n_words, "null argument");
  const int64_t nb = (int64_t)(s->bdim[0] + 2) * (s->bdim[1] + 2) * (s->bdim[2] + 2);
  *n_words = nb;
  if (!out) return VT_OK;
  VT_CHECK_ARG(bytes >= sizeof(uint64_t) * (size_t)nb, "output buffer too small");
  cudaSetDevice(s->ctx->device);
  VT_CUDA(cudaMemcpy(out, s->bricks, sizeof(uint64_t) * (size_t)nb, cudaMemcpyDeviceToHost), "brick readback");
  return VT_OK;
}

extern "C" int vt_diag_check_word(vt_context* ctx, uint32_t* word, int32_t* enabled) {
  VT_CHECK_ARG(ctx && word && enabled, "null argument");
  cudaSetDevice(ctx->device);
  VT_CUDA(cudaStreamSynchronize(ctx->stream), "check word");
  bool on = false;
  VT_CUDA(read_check_word(word, &on, true), "check word");
  *enabled = on ? 1 : 0;
  return VT_OK;
}

extern "C" int vt_diag_l2_read_bandwidth(vt_context* ctx, int64_t bytes, int32_t reps, double* gbs) {
  VT_CHECK_ARG(ctx && gbs && reps > 0 && bytes >= (1 << 20) && bytes <= ((int64_t)1 << 30) && bytes % 16 == 0,
               "bytes must be a multiple of 16 in [1 MiB, 1 GiB] and reps > 0");
  cudaSetDevice(ctx->device);
  const int blocks = ctx->sm_count * 4;
  const size_t out_bytes = (size_t)blocks * 512 * sizeof(uint4);
  void* buf = nullptr;
  void* out = nullptr;
  int rc = ctx->alloc(&buf, (size_t)bytes);
  if (rc != VT_OK) return rc;
  rc = ctx->alloc(&out, out_bytes);
  if (rc != VT_OK) { ctx->release(buf); return rc; }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float ms = 0.0f;
  cudaError_t e = cudaMemsetAsync(buf, 0x5a, (size_t)bytes, ctx->stream);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  const uint32_t n = (uint32_t)(bytes / 16);
  // one warm sweep brings the buffer into L2, then the timed launch
  if (e == cudaSuccess) e = launch_l2_read((const uint4*)buf, n, 1, (uint4*)out, blocks, ctx->stream);
  if (e == cudaSuccess) e = cudaEventRecord(e0, ctx->stream);
  if (e == cudaSuccess) e = launch_l2_read((const uint4*)buf, n, reps, (uint4*)out, blocks, ctx->stream);
  if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  ctx->release(out);
  ctx->release(buf);
  if (e != cudaSuccess) return cuda_fail(e, "l2 read sweep");
  *gbs = (double)bytes * reps / (ms * 1e-3) / 1e9;
  return VT_OK;
}

extern "C" int vt_diag_cdf_from_function(vt_context* ctx, const float* func, int32_t w, int32_t h, float* cdf_u,
                                         float* cdf_v, float* integral) {
  VT_CHECK_ARG(ctx && func && cdf_u && cdf_v && w > 0 && h > 0, "bad argument");
  cudaSetDevice(ctx->device);
  size_t offs[9];
  const size_t sb = env_scratch_bytes(w, h, offs);
  const size_t extra = ((sizeof(float) * (size_t)(w + 1) * h + 255) & ~(size_t)255) +
                       ((sizeof(float) * (size_t)(h + 2) + 255) & ~(size_t)255) + 256;
  int rc = ctx->ensure_scratch(sb + extra);
  if (rc != VT_OK) return rc;
  EnvScratch S = env_scratch(ctx->scratch, offs);
  float* d_cu = (float*)((char*)ctx->scratch + sb);
  float* d_cv = (float*)((char*)d_cu + ((sizeof(float) * (size_t)(w + 1) * h + 255) & ~(size_t)255));
  float* d_int = d_cv + (h + 1);
  VT_CUDA(cudaMemcpyAsync(S.func, func, sizeof(float) * (size_t)w * h, cudaMemcpyHostToDevice, ctx->stream), "cdf");
  VT_CUDA(launch_cdf(S.func, w, h, S, d_cu, d_cv, d_int, ctx->stream), "cdf");
  VT_CUDA(cudaMemcpyAsync(cdf_u, d_cu, sizeof(float) * (size_t)(w + 1) * h, cudaMemcpyDeviceToHost, ctx->stream), "cdf");
  VT_CUDA(cudaMemcpyAsync(cdf_v, d_cv, sizeof(float) * (size_t)(h + 1), cudaMemcpyDeviceToHost, ctx->stream), "cdf");
  float iv = 0.0f;
  VT_CUDA(cudaMemcpyAsync(&iv, d_int, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream), "cdf");
  VT_CUDA(cudaStreamSynchronize(ctx->stream), "cdf");
  if (integral) *integral = iv;
  return VT_OK;
}

extern "C" int vt_diag_set_tuning(vt_context* ctx, int64_t slots, int32_t blocks_per_sm, int32_t steps,
                                  int64_t max_items) {
  VT_CHECK_ARG(ctx, "context is null");
  if (slots > 0) ctx->max_slots = std::max<int64_t>(32, std::min<int64_t>(slots, (int64_t)1 << 26));
  if (blocks_per_sm >= 0) ctx->trace_blocks_per_sm = blocks_per_sm;
  if (steps > 0) ctx->trace_steps = steps <= 4 ? 4 : (steps <= 8 ? 8 : (steps <= 16 ? 16 : 32));
  if (max_items > 0) ctx->max_items = std::max<int64_t>(1024, max_items);
  return VT_OK;
}

extern "C" int vt_diag_set_trace_form(vt_context* ctx, int32_t form) {
  VT_CHECK_ARG(ctx && (form == 0 || form == 1), "trace form must be 0 (per-lane set-up) or 1 (pooled set-up)");
  ctx->trace_form = form;
  return VT_OK;
}

extern "C" int vt_diag_set_trace_tuning(vt_context* ctx, int32_t queue_chunk, int32_t refill_min) {
  VT_CHECK_ARG(ctx, "context is null");
  VT_CHECK_ARG(queue_chunk <= 0 || (queue_chunk >= 32 && queue_chunk <= 1024 && queue_chunk % 32 == 0),
               "queue_chunk must be a multiple of 32 in [32, 1024]");
  VT_CHECK_ARG(refill_min < 0 || refill_min <= 32, "refill_min must be in [0, 32]");
  if (queue_chunk > 0) ctx->trace_chunk = queue_chunk;
  if (refill_min >= 0) ctx->refill_min = refill_min;
  return VT_OK;
}

extern "C" int vt_diag_launch_count(const vt_context* ctx, uint64_t* launches) {
  VT_CHECK_ARG(ctx && launches, "null argument");
  *launches = ctx->launches;
  return VT_OK;
}

extern "C" int vt_diag_stream(vt_context* ctx, void** stream) {
  VT_CHECK_ARG(ctx && stream, "null argument");
  *stream = (void*)ctx->stream;
  return VT_OK;
}

extern "C" int vt_diag_env_texels(const vt_env* env, uint16_t* out, size_t bytes) {
  VT_CHECK_ARG(env && out, "null argument");
  const size_t n = sizeof(uint2) * (size_t)env->w * env->h;
  VT_CHECK_ARG(bytes >= n, "output buffer too small");
  cudaSetDevice(env->ctx->device);
  VT_CUDA(cudaMemcpy(out, env->texels, n, cudaMemcpyDeviceToHost), "texels");
  return VT_OK;
}

extern "C" int vt_diag_set_noise_table(vt_context* ctx, const float* rgba, size_t bytes) {
  VT_CHECK_ARG(ctx && rgba, "null argument");
  const size_t n = sizeof(float) * 4 * kNoiseW * kNoiseH;
  VT_CHECK_ARG(bytes >= n, "table must hold 1024*1024 RGBA floats");
  int rc = ctx->ensure_noise();
  if (rc != VT_OK) return rc;
  VT_CUDA(cudaMemcpy(ctx->noise, rgba, n, cudaMemcpyHostToDevice), "noise table");
  return VT_OK;
}

extern "C" int vt_diag_get_noise_table(vt_context* ctx, float* rgba, size_t bytes) {
  VT_CHECK_ARG(ctx && rgba, "null argument");
  const size_t n = sizeof(float) * 4 * kNoiseW * kNoiseH;
  VT_CHECK_ARG(bytes >= n, "table must hold 1024*1024 RGBA floats");
  int rc = ctx->ensure_noise();
  if (rc != VT_OK) return rc;
  VT_CUDA(cudaMemcpy(rgba, ctx->noise, n, cudaMemcpyDeviceToHost), "noise table");
  return VT_OK;
}
