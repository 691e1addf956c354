// vt_render.cu — path-tracing kernels.
//
//   k_plain       one thread per pixel, `passes` samples per launch; the
//                 reference's one-pass-per-draw structure (renderer.cpp:584-611)
//   wavefront     many jobs and passes per launch, in rounds of two kernels:
//                 k_wf_shade (one thread per path slot: segment results ->
//                 shading -> new segments appended to a queue by warp
//                 ballot, new items started as paths finish) and k_wf_trace
//                 (DDA of every queued segment with per-warp refill from the
//                 queue); per-sample outputs land in a sample buffer that
//                 k_wf_accumulate reduces in sample order.
//   k_diag        per-sample output and first-hit record (parity tests)
//   k_trace_rays  DDA of caller-supplied rays (parity tests)
//   k_pick        focal-distance pick of one pixel (focalDistance.vs:45-81)
//   k_resolve     average = sum / n (+ tonemap / flip) for readback
#include "vt_kernels.h"
#include "vt_shade.cuh"

namespace vt {

template <bool kCount>
__device__ __forceinline__ void flush_counters(Cnt<kCount>& cnt, unsigned long long* out) {
  if (!kCount || out == nullptr) return;
#pragma unroll
  for (int i = 0; i < C_NUM; ++i) {
    unsigned long long v = cnt.c[i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&out[i], v);
  }
}

// ------------------------------------------------------------------ plain
template <bool kCount>
__global__ void __launch_bounds__(128) k_plain(const Frame F, const JobDev J, int sample_base, int passes,
                                               unsigned long long* counters) {
  Cnt<kCount> cnt;
#pragma unroll
  for (int i = 0; i < C_NUM; ++i) cnt.c[i] = 0;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = F.width * F.height;
  if (idx < n) {
    const int px = idx % F.width, py = idx / F.width;
    float4 sum = J.sum[idx], comp = J.comp[idx];
    for (int k = 0; k < passes; ++k) {
      const float4 v = trace_sample(F, J, px, py, sample_base + k, cnt, (HitRecord*)nullptr);
      kahan_add(sum, comp, v);
    }
    J.sum[idx] = sum;
    J.comp[idx] = comp;
  }
  flush_counters(cnt, counters);
}

cudaError_t launch_plain(const Frame& F, const JobDev& J, int sample_base, int passes,
                         unsigned long long* counters, cudaStream_t st) {
  const int n = F.width * F.height;
  const int threads = 128;
  const int blocks = (n + threads - 1) / threads;
  if (counters) k_plain<true><<<blocks, threads, 0, st>>>(F, J, sample_base, passes, counters);
  else k_plain<false><<<blocks, threads, 0, st>>>(F, J, sample_base, passes, nullptr);
  return cudaGetLastError();
}

// ------------------------------------------------------------------- diag
__global__ void k_diag(const Frame F, const JobDev J, int sample, float4* out, HitRecord* hits,
                       unsigned long long* counters) {
  Cnt<true> cnt;
#pragma unroll
  for (int i = 0; i < C_NUM; ++i) cnt.c[i] = 0;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = F.width * F.height;
  if (idx < n) {
    const int px = idx % F.width, py = idx / F.width;
    HitRecord h;
    const float4 v = trace_sample(F, J, px, py, sample, cnt, &h);
    out[idx] = v;
    if (hits) hits[idx] = h;
  }
  flush_counters(cnt, counters);
}

cudaError_t launch_diag(const Frame& F, const JobDev& J, int sample, float4* out, HitRecord* hits,
                        unsigned long long* counters, cudaStream_t st) {
  const int n = F.width * F.height;
  k_diag<<<(n + 127) / 128, 128, 0, st>>>(F, J, sample, out, hits, counters);
  return cudaGetLastError();
}

// -------------------------------------------------------------- wavefront
// Slot flags.
enum : uint32_t {
  SL_BOUNCES = 0xffu,
  SL_PRIMARY = 1u << 8,
  SL_HAS_CONT = 1u << 9,
  SL_EXT = 1u << 10,      // an extension segment was traced for this slot
  SL_SHADOW = 1u << 11,   // a shadow segment was traced for this slot
  SL_ACTIVE = 1u << 12,   // a path (0: an empty position of the stream)
  // bits 14..16: non-finite throughput components of the pending light sample
  // bits 17..31: job of the path
};
constexpr int kSlotJobShift = 17;
static_assert(kWfMaxJobs == (1 << (32 - kSlotJobShift)), "job bits of the slot flags");

__device__ __forceinline__ v3 xyz4(float4 v) { return mk3(v.x, v.y, v.z); }
__device__ __forceinline__ float4 pack4(v3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

// Job and grid records: from the global tables, or (WfJobTable) from the
// kernel's parameter block.
struct WfNoTable {
  int unused;
};
__device__ __forceinline__ const JobEntry& job_entry(const WfParams& P, const WfNoTable&, uint32_t j) {
  return P.jobs[j];
}
__device__ __forceinline__ const JobEntry& job_entry(const WfParams&, const WfJobTable& T, uint32_t j) {
  return T.e[j];
}
__device__ __forceinline__ const Grid& grid_entry(const WfParams& P, const WfNoTable&, uint32_t j) {
  return P.grids[j];
}
__device__ __forceinline__ const Grid& grid_entry(const WfParams&, const WfJobTable& T, uint32_t j) {
  return T.g[j];
}
__device__ __forceinline__ const JobEntry& job_entry(const WfParams&, const WfOneJob& T, uint32_t) { return T.e; }
__device__ __forceinline__ const Grid& grid_entry(const WfParams&, const WfOneJob& T, uint32_t) { return T.g; }

// Job of a global item index (binary search over tile_begin).
__device__ __forceinline__ int job_of(const WfParams&, const WfOneJob&, unsigned long long) { return 0; }
template <class Tab>
__device__ __forceinline__ int job_of(const WfParams& P, const Tab& T, unsigned long long item) {
  int lo = 0, hi = P.n_jobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((unsigned long long)job_entry(P, T, (uint32_t)mid).tile_begin <= item) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Path state (WfState): a0 = (ro, -), a1 = (rd, item), a3 = (L, rng),
// a4 = (T, bsdf_pdf), a5 = (nee_P, light) for paths with a shadow segment;
// the job, bounces and flag bits live in `flags`, and pixel and sample
// follow from the item.
// k_wf_shade reads what ending a segment needs (a1, a3, a4, a5 for a shadow
// result, a0 for a hit it keeps) and copies kept hits into hit records;
// k_wf_hit reads only the hit records.
__device__ __forceinline__ void load_flags(uint32_t fl, Path& p) {
  p.bounces = (int)(fl & SL_BOUNCES);
  p.primary = (fl & SL_PRIMARY) ? 1 : 0;
  p.has_cont = (fl & SL_HAS_CONT) ? 1 : 0;
  p.nee_nf = (int)((fl >> 14) & 7u);
}

__device__ __forceinline__ void load_for_shade(const WfState& st, int i, uint32_t fl, Path& p, uint32_t& item,
                                               float& rng_word) {
  const float4 a1 = st.a1[i], a3 = st.a3[i], a4 = st.a4[i];
  p.rd = xyz4(a1);
  item = __float_as_uint(a1.w);
  p.L = xyz4(a3);
  rng_word = a3.w;
  p.T = xyz4(a4); p.bsdf_pdf = a4.w;
  if (fl & SL_SHADOW) {
    const float4 a5 = st.a5[i];
    p.nee_P = xyz4(a5); p.light = __float_as_int(a5.w);
  }
  load_flags(fl, p);
}

__device__ __forceinline__ void rng_from_item(const JobEntry& E, uint32_t item, uint32_t rng, Path& p) {
  // item - tile_begin = pass * n_pixels + pixel (< 2^32 items per launch)
  const uint32_t r = item - (uint32_t)E.tile_begin;
  const uint32_t np = (uint32_t)E.n_pixels;   // = width * height
  const uint32_t pass = udiv(r, E.F.m_pixels);
  p.rng.pixel = r - pass * np;
  p.rng.sample = (uint32_t)E.sample_base + pass;
  if (E.F.rng_mode == 1) { p.rng.ox = (int32_t)(rng & 0xffffu); p.rng.oy = (int32_t)(rng >> 16); p.rng.call = 0; }
  else { p.rng.call = rng; p.rng.ox = p.rng.oy = 0; }
}

// The state the next round's shading reads (the shadow direction is only
// needed for the segment record written beside it, so it is not stored).
__device__ __forceinline__ void store_path(const WfState& st, int i, const Frame& F, const Path& p, uint32_t item,
                                           bool shadow) {
  const uint32_t rng = (F.rng_mode == 1) ? ((uint32_t)p.rng.ox | ((uint32_t)p.rng.oy << 16)) : p.rng.call;
  st.a0[i] = pack4(p.ro, 0.0f);
  st.a1[i] = pack4(p.rd, __uint_as_float(item));
  st.a3[i] = pack4(p.L, __uint_as_float(rng));
  st.a4[i] = pack4(p.T, p.bsdf_pdf);
  if (shadow) st.a5[i] = pack4(p.nee_P, __int_as_float(p.light));
}

// Block-wide reservation on N counters with one atomic per counter and
// block instead of per warp: `n[i]` is this thread's count for counter i;
// returns in base[i] the first entry of the thread's warp (the offsets of
// the thread within its warp come from ballots).  Every thread of the block
// must call it (three barriers).
constexpr int kWfWarps = 4;   // warps per shade / hit / regen block (128 threads)
template <int N>
__device__ __forceinline__ void block_reserve(uint32_t* const (&ctr)[N], const uint32_t (&n)[N], uint32_t (&base)[N]) {
  __shared__ uint32_t s_n[N][kWfWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    uint32_t v = n[i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) s_n[i][warp] = v;
  }
  __syncthreads();
  if (threadIdx.x < N) {
    const int i = threadIdx.x;
    uint32_t t = 0, pre[kWfWarps];
#pragma unroll
    for (int w = 0; w < kWfWarps; ++w) { pre[w] = t; t += s_n[i][w]; }
    const uint32_t b0 = t ? atomicAdd(ctr[i], t) : 0u;
#pragma unroll
    for (int w = 0; w < kWfWarps; ++w) s_n[i][w] = b0 + pre[w];
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < N; ++i) base[i] = s_n[i][warp];
  __syncthreads();   // the next call may overwrite s_n
}

// Write this warp's next segments (queue entries from `base`) as 32-byte ray
// records {vo.xyz, inc.x} {inc.yz, slot << 1 | kind, job}: the origin in
// voxel space and the reciprocal direction as seg_rec gives them to the DDA
// set-up, computed here in coherent warps rather than by the DDA kernel's
// lanes as they start segments at different times.  The warp's extension
// records first, then its shadow records.  emit: 1 extension (from
// `ext_o`), 2 shadow.
__device__ __forceinline__ void write_segments(const WfParams& P, int par, uint32_t base, uint32_t emit, int slot,
                                               uint32_t job, v3 ext_o, const Path& p, const Frame& F) {
  const unsigned FULL = 0xffffffffu;
  const unsigned lt = (1u << (threadIdx.x & 31)) - 1u;
  const uint32_t n1 = (emit & 1u) ? 1u : 0u, n2 = (emit & 2u) ? 1u : 0u;
  const unsigned b1 = __ballot_sync(FULL, n1), b2 = __ballot_sync(FULL, n2);
  float4* q = P.queue[par];
  if (n1) {
    const size_t at = 2 * (size_t)(base + __popc(b1 & lt));
    const SegRec sr = seg_rec(F, ext_o, p.rd);
    q[at] = make_float4(sr.vo.x, sr.vo.y, sr.vo.z, sr.inc.x);
    q[at + 1] = make_float4(sr.inc.y, sr.inc.z, __uint_as_float((uint32_t)slot << 1), __uint_as_float(job));
  }
  if (n2) {
    const size_t at = 2 * (size_t)(base + __popc(b1) + __popc(b2 & lt));
    const SegRec sr = seg_rec(F, p.ro, p.sd);
    q[at] = make_float4(sr.vo.x, sr.vo.y, sr.vo.z, sr.inc.x);
    q[at + 1] = make_float4(sr.inc.y, sr.inc.z, __uint_as_float(((uint32_t)slot << 1) | 1u), __uint_as_float(job));
  }
}

__device__ __forceinline__ uint32_t slot_flags(const Path& p, uint32_t emit, uint32_t job) {
  return SL_ACTIVE | (uint32_t)(p.bounces & 0xff) | (p.primary ? SL_PRIMARY : 0u) | (p.has_cont ? SL_HAS_CONT : 0u) |
         ((emit & 1u) ? SL_EXT : 0u) | ((emit & 2u) ? SL_SHADOW : 0u) | ((uint32_t)(p.nee_nf & 7) << 14) |
         (job << kSlotJobShift);
}

// A round has four kernels over the stream x[par] (n paths, written by the
// previous round) and builds the stream x[par ^ 1]:
//   k_wf_shade  every position: shadow results (NEE added if visible),
//               extension results (miss -> environment, bounce limit,
//               selection), finished paths -> sample buffer; surviving hits
//               -> hit records, Lambert hits from the front of the list, the
//               others from its back, so that k_wf_hit's warps mostly run one
//               BSDF
//   k_wf_hit    the hit records: vertex shading, light and BSDF samples;
//               writes its paths to positions [0, hits) of the next stream
//               and their next segments to the queue; reserves the first
//               items of the new paths
//   k_wf_regen  new paths in positions [hits, capacity) of the next stream,
//               primary segments to the queue after the hit kernel's
//   k_wf_trace  the queue: DDA of every segment, ends stored by position
// Every state access is to consecutive positions.  k_wf_hit keeps eight
// resident blocks per SM (64 registers): the extra warps hide more of the
// load latency than the few spills cost; the lighter k_wf_shade and (with one
// job) k_wf_regen fit twelve.
template <bool kCount, class Tab>
__global__ void __launch_bounds__(128, 12) k_wf_shade(const WfParams P, const __grid_constant__ Tab T, int par) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  if (blockIdx.x == 0 && threadIdx.x == 0)    // items taken before this round, for k_wf_regen
    *(unsigned long long*)&P.ctl[ctl_index(par, CTL_ITEM_SNAP)] = *(volatile unsigned long long*)P.next_item;
  const uint32_t n = *(volatile uint32_t*)&P.ctl[ctl_index(par ^ 1, CTL_NEXT_N)];
  if (blockIdx.x * blockDim.x >= n) return;   // the whole block lies beyond the stream
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const WfState& src = P.x[par];
  Cnt<kCount> cnt;
#pragma unroll
  for (int k = 0; k < C_NUM; ++k) cnt.c[k] = 0;
  const uint32_t fl = (uint32_t)i < n ? src.flags[i] : 0u;
  bool hit = false;
  int cls = 0;
  Path p;
  uint32_t item = 0;
  float rng_word = 0.0f;
  SegEnd e;
  e.x = e.y = e.z = e.state = 0;
  if (fl & SL_ACTIVE) {
    cnt.add(C_POSITIONS, 1);
    const uint32_t job = fl >> kSlotJobShift;
    const JobEntry& E = job_entry(P, T, job);
    // every load of the position is issued before any of them is used (the
    // origin is read for every extension, whether or not it hits)
    const unsigned long long hs = (fl & SL_SHADOW) ? P.hits[(size_t)P.n_slots + i] : 0ull;
    const unsigned long long he = (fl & SL_EXT) ? P.hits[i] : 0ull;
    const float4 a0v = (fl & SL_EXT) ? src.a0[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    load_for_shade(src, i, fl, p, item, rng_word);
    if (fl & SL_SHADOW) shadow_end(E.F, p, unpack_end(hs));
    if (fl & SL_EXT) {
      e = unpack_end(he);
      hit = ext_resolve(E.F, E.J, p, e, cnt);
      if (hit) cls = hit_class(E.F, E.J, e);
    }
    if (hit) p.ro = xyz4(a0v);
    else if (chk(item < P.n_items, CHK_SAMPLE)) P.sbuf[item] = path_output(E.F, p);
  }
  uint32_t* const ctr[2] = {&P.ctl[ctl_index(par, CTL_HITS_LAMBERT)], &P.ctl[ctl_index(par, CTL_HITS_OTHER)]};
  const uint32_t cnt_l = (hit && cls == 0) ? 1u : 0u, cnt_o = (hit && cls != 0) ? 1u : 0u;
  const uint32_t nn[2] = {cnt_l, cnt_o};
  uint32_t base[2];
  block_reserve<2>(ctr, nn, base);
  const unsigned bl = __ballot_sync(FULL, cnt_l), bo = __ballot_sync(FULL, cnt_o);
  if (hit) {
    const uint32_t j = cnt_l ? base[0] + __popc(bl & lt) : (uint32_t)P.n_slots - 1u - (base[1] + __popc(bo & lt));
    P.hr.h0[j] = pack4(p.ro, __uint_as_float(item));
    P.hr.h1[j] = pack4(p.rd, __uint_as_float(slot_flags(p, 1u, fl >> kSlotJobShift)));
    P.hr.h2[j] = pack4(p.L, rng_word);
    P.hr.h3[j] = pack4(p.T, p.bsdf_pdf);
    P.hr.h4[j] = pack_end(e.x, e.y, e.z, e.state);
  }
  flush_counters(cnt, P.counters);
}

// The hit records of this round: list entry v (Lambert entries [0, nl), then
// the others, stored from the back) becomes position v of the next stream.
// A block-uniform grid-stride loop.
template <bool kCount, class Tab>
__global__ void __launch_bounds__(128, 8) k_wf_hit(const WfParams P, const __grid_constant__ Tab T, int par) {
  const uint32_t nl = *(volatile uint32_t*)&P.ctl[ctl_index(par, CTL_HITS_LAMBERT)];
  const uint32_t no = *(volatile uint32_t*)&P.ctl[ctl_index(par, CTL_HITS_OTHER)];
  const uint32_t n_hits = nl + no;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // items [taken, taken + m) go to k_wf_regen's m positions, position k
    // taking item taken + k first; its lanes claim further items only after
    const unsigned long long taken = *(volatile unsigned long long*)&P.ctl[ctl_index(par, CTL_ITEM_SNAP)];
    const unsigned long long left = P.n_items > taken ? P.n_items - taken : 0ull;
    const uint32_t m = (uint32_t)min((unsigned long long)((uint32_t)P.n_slots - n_hits), left);
    if (m) atomicAdd(P.next_item, (unsigned long long)m);
  }
  const WfState& dst = P.x[par ^ 1];
  Cnt<kCount> cnt;
#pragma unroll
  for (int k = 0; k < C_NUM; ++k) cnt.c[k] = 0;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t b0 = blockIdx.x * blockDim.x; b0 < n_hits; b0 += stride) {   // block-uniform
    const uint32_t v = b0 + threadIdx.x;
    const bool mine = v < n_hits;
    Path p;
    uint32_t job = 0, item = 0;
    uint32_t emit = 0;
    if (mine) {
      const uint32_t j = v < nl ? v : (uint32_t)P.n_slots - 1u - (v - nl);
      const float4 h0 = P.hr.h0[j], h1 = P.hr.h1[j], h2 = P.hr.h2[j], h3 = P.hr.h3[j];
      const unsigned long long h4 = P.hr.h4[j];
      const uint32_t fl = __float_as_uint(h1.w);
      job = fl >> kSlotJobShift;
      const JobEntry& E = job_entry(P, T, job);
      p.ro = xyz4(h0);
      item = __float_as_uint(h0.w);
      p.rd = xyz4(h1);
      p.L = xyz4(h2);
      p.T = xyz4(h3); p.bsdf_pdf = h3.w;
      load_flags(fl, p);
      rng_from_item(E, item, __float_as_uint(h2.w), p);
      const SegEnd e = unpack_end(h4);
      ext_hit(E.F, E.J, p, e, cnt);
      emit = 2u | (p.has_cont ? 1u : 0u);
    }
    uint32_t* const ctr[1] = {&P.ctl[ctl_index(par, CTL_QCOUNT)]};
    const uint32_t nn[1] = {(emit & 1u) + (emit >> 1)};
    uint32_t base[1];
    block_reserve<1>(ctr, nn, base);
    write_segments(P, par, base[0], emit, (int)v, job, p.ro, p, job_entry(P, T, job).F);
    if (mine) {
      store_path(dst, (int)v, job_entry(P, T, job).F, p, item, (emit & 2u) != 0);
      dst.flags[v] = slot_flags(p, emit, job);
    }
  }
  flush_counters(cnt, P.counters);
}

// New paths at positions [hits, hits + m) of the next stream, m = the free
// capacity or the items left, whichever is smaller.  Position k starts with
// item taken + k (reserved by k_wf_hit); a lane whose path misses its job's
// volume (finished at once) claims further items with one atomic per warp,
// until a path enters the volume or the items run out (the position stays
// empty).  The primary segment starts at the volume entry point; position
// k's queue record is entry QCOUNT + k of the round's queue (the hit
// kernel's records come first), a record without a segment for an empty
// position, so that the kernel needs no block-wide reservation.
// Resident blocks the new-path kernel is compiled for: twelve with one job
// (40 registers, no spill), eight with a job table (whose records need more).
template <class Tab> struct RegenBlocks { static constexpr int value = 8; };
template <> struct RegenBlocks<WfOneJob> { static constexpr int value = 12; };

template <bool kCount, class Tab>
__global__ void __launch_bounds__(128, RegenBlocks<Tab>::value) k_wf_regen(const WfParams P, const __grid_constant__ Tab T, int par) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const uint32_t n_hits = *(volatile uint32_t*)&P.ctl[ctl_index(par, CTL_HITS_LAMBERT)] +
                          *(volatile uint32_t*)&P.ctl[ctl_index(par, CTL_HITS_OTHER)];
  const unsigned long long taken = *(volatile unsigned long long*)&P.ctl[ctl_index(par, CTL_ITEM_SNAP)];
  const unsigned long long left = P.n_items > taken ? P.n_items - taken : 0ull;
  const uint32_t m = (uint32_t)min((unsigned long long)((uint32_t)P.n_slots - n_hits), left);
  const uint32_t qbase = *(volatile uint32_t*)&P.ctl[ctl_index(par, CTL_QCOUNT)];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    P.ctl[ctl_index(par, CTL_NEXT_N)] = n_hits + m;
    P.ctl[ctl_index(par, CTL_REGEN_N)] = m;
  }
  const WfState& dst = P.x[par ^ 1];
  float4* const q = P.queue[par];
  Cnt<kCount> cnt;
#pragma unroll
  for (int k = 0; k < C_NUM; ++k) cnt.c[k] = 0;
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t b0 = blockIdx.x * blockDim.x; b0 < m; b0 += stride) {   // block-uniform
    const uint32_t k = b0 + threadIdx.x;
    const bool mine = k < m;
    const uint32_t pos = n_hits + k;
    unsigned long long my = taken + k;
    bool need_new = mine, active = false;
    Path p;
    uint32_t job = 0, item = 0;
    float t_enter = 0.0f;
    for (;;) {
      if (need_new) {
        if (my >= P.n_items) {
          need_new = false;   // no items left: the position stays empty
        } else {
          item = (uint32_t)my;
          job = (uint32_t)job_of(P, T, my);
          const JobEntry& E = job_entry(P, T, job);
          const uint32_t r = (uint32_t)(my - (unsigned long long)E.tile_begin);   // < 2^32 items per launch
          const uint32_t np = (uint32_t)E.n_pixels;   // = width * height
          const uint32_t pass = udiv(r, E.F.m_pixels);
          const uint32_t pixel = r - pass * np;
          const uint32_t w = (uint32_t)E.F.width;
          const int py = (int)udiv(pixel, E.F.m_width), px = (int)(pixel - (uint32_t)py * w);
          if (path_start(E.F, E.J, p, px, py, E.sample_base + (int)pass, cnt, t_enter)) {
            active = true;
            need_new = false;
          } else {
            if (chk(item < P.n_items, CHK_SAMPLE))
              P.sbuf[item] = path_output(E.F, p);   // missed the volume: finished, take another item
          }
        }
      }
      const unsigned want = __ballot_sync(FULL, need_new);
      if (!want) break;
      const int leader = __ffs(want) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(P.next_item, (unsigned long long)__popc(want));
      base = __shfl_sync(FULL, base, leader);
      my = base + __popc(want & lt);
    }
    if (mine) {
      const size_t at = 2 * (size_t)(qbase + k);
      if (active) {
        const v3 o = p.ro + t_enter * p.rd;   // the primary segment starts at the volume entry point
        const SegRec sr = seg_rec(job_entry(P, T, job).F, o, p.rd);
        q[at] = make_float4(sr.vo.x, sr.vo.y, sr.vo.z, sr.inc.x);
        q[at + 1] = make_float4(sr.inc.y, sr.inc.z, __uint_as_float((uint32_t)pos << 1), __uint_as_float(job));
        store_path(dst, (int)pos, job_entry(P, T, job).F, p, item, false);   // a primary path has no shadow segment
        dst.flags[pos] = slot_flags(p, 1u, job);
      } else {
        q[at + 1] = make_float4(0.0f, 0.0f, __uint_as_float(kNoSegment), 0.0f);
        dst.flags[pos] = 0u;
      }
    }
  }
  flush_counters(cnt, P.counters);
}

// The grid record of a lane's current segment: a register copy, or with one
// job the record in the parameter block itself (constant operands).
template <class Tab>
struct GridHold {
  Grid g;
  __device__ __forceinline__ void set(const WfParams& P, const Tab& T, uint32_t job) { g = grid_entry(P, T, job); }
  __device__ __forceinline__ const Grid& get(const Tab&) const { return g; }
};
template <>
struct GridHold<WfOneJob> {
  __device__ __forceinline__ void set(const WfParams&, const WfOneJob&, uint32_t) {}
  __device__ __forceinline__ const Grid& get(const WfOneJob& T) const { return T.g; }
};

// One round of tracing: every queued segment runs its DDA to the end.  Each
// warp takes chunks of P.trace_chunk queue records with one atomic and hands
// them to its lanes; every lane keeps the record of its next segment loaded
// while it steps the current one, so starting a segment never waits on
// memory, and lanes pick up a new segment every kTraceSteps steps as theirs
// finish (with kVote also as soon as fewer than P.refill_min lanes step).
// Resident blocks the trace kernel is compiled for: six with one job (its
// grid record is constant), five with a job table, whose per-lane grid
// record would otherwise spill at six blocks' 40 registers.
template <class Tab> struct TraceBlocks { static constexpr int value = 5; };
template <> struct TraceBlocks<WfOneJob> { static constexpr int value = 6; };

template <bool kCount, int kTraceSteps, bool kVote, bool k444, class Tab>
__global__ void __launch_bounds__(256, TraceBlocks<Tab>::value) k_wf_trace(const WfParams P, const __grid_constant__ Tab T, int par) {
  static_assert(kTraceSteps % 4 == 0, "the 4x4x4 loop steps four at a time");
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  const uint32_t n = *(volatile uint32_t*)&P.ctl[ctl_index(par, CTL_QCOUNT)] +
                     *(volatile uint32_t*)&P.ctl[ctl_index(par, CTL_REGEN_N)];   // hit, then new-path records
  if (n == 0) return;
  const float4* q = P.queue[par];
  Cnt<kCount> cnt;
#pragma unroll
  for (int i = 0; i < C_NUM; ++i) cnt.c[i] = 0;
  uint32_t pool = 0, pool_end = 0;
  bool exhausted = false, have = false, have_next = false;
  float4 na = make_float4(0.f, 0.f, 0.f, 0.f), nb = na;
  GridHold<Tab> gh;
  Dda s;
  uint32_t tag = 0;   // position << 1 | kind of the current segment
  for (;;) {
    if (!have && have_next) {            // start the prefetched segment
      have_next = false;
      tag = __float_as_uint(nb.z);
      if (tag != kNoSegment) {
        gh.set(P, T, __float_as_uint(nb.w));
        dda_begin_rec(gh.get(T), s, mk3(na.x, na.y, na.z), mk3(na.w, nb.x, nb.y));
        if (s.state == DDA_RUNNING) have = true;
        else P.hits[(size_t)(tag & 1u) * P.n_slots + (tag >> 1)] = pack_end(s.x, s.y, s.z, s.state);
      }
    }
    unsigned need = __ballot_sync(FULL, !have_next);
    while (need && !exhausted) {          // prefetch next records
      if (pool >= pool_end) {
        uint32_t c = 0;
        if (lane == 0) c = atomicAdd(&P.ctl[ctl_index(par, CTL_QHEAD)], P.trace_chunk);
        c = __shfl_sync(FULL, c, 0);
        if (c >= n) { exhausted = true; break; }
        pool = c;
        pool_end = min(c + P.trace_chunk, n);
      }
      const uint32_t avail = pool_end - pool;
      const uint32_t r = __popc(need & lt);
      if (!have_next && r < avail) {
        na = __ldg(&q[2 * (size_t)(pool + r)]);
        nb = __ldg(&q[2 * (size_t)(pool + r) + 1]);
        have_next = true;
      }
      pool += min(avail, (uint32_t)__popc(need));
      need = __ballot_sync(FULL, !have_next);
    }
    if (__ballot_sync(FULL, have || have_next) == 0u) break;
    if (have) {
      if constexpr (!kCount && k444) dda_steps_444<kVote>(gh.get(T), s, kTraceSteps, P.refill_min);
      else dda_steps<kCount, kVote, k444>(gh.get(T), s, kTraceSteps, cnt, P.refill_min);
      if (s.state != DDA_RUNNING) {
        P.hits[(size_t)(tag & 1u) * P.n_slots + (tag >> 1)] = pack_end(s.x, s.y, s.z, s.state);
        have = false;
      }
    }
  }
  flush_counters(cnt, P.counters);
}

// One round of tracing, pooled form: each warp keeps up to kPoolSegs
// segments set up and ready to step in shared memory.  The segment set-up
// (dda_begin: nudge, divisions, floor, bounds test) runs for a warp's worth
// of queue records at once, every lane busy; a lane whose segment ended takes
// a ready one after each batch of kTraceSteps steps, so lanes rarely wait
// for a set-up.  Same segments, same ends, same bits as k_wf_trace.
constexpr int kPoolSegs = 64;
constexpr int kTraceWarps = 8;   // 256-thread blocks

__device__ __forceinline__ int32_t pack_signs(const Dda& t) {
  return (t.sx + 1) | ((t.sy + 1) << 2) | ((t.sz + 1) << 4);
}

template <bool kCount, int kTraceSteps, bool k444, class Tab>
__global__ void __launch_bounds__(256, 4) k_wf_trace_pool(const WfParams P, const __grid_constant__ Tab T, int par) {
  static_assert(kTraceSteps % 4 == 0, "the 4x4x4 loop steps four at a time");
  __shared__ int32_t s_i[4][kTraceWarps][kPoolSegs];    // x, y, z, packed signs
  __shared__ float s_f[6][kTraceWarps][kPoolSegs];      // dx, dy, dz, ax, ay, az
  __shared__ uint32_t s_u[2][kTraceWarps][kPoolSegs];   // position << 1 | kind, job
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lt = (1u << lane) - 1u;
  const uint32_t n = *(volatile uint32_t*)&P.ctl[ctl_index(par, CTL_QCOUNT)] +
                     *(volatile uint32_t*)&P.ctl[ctl_index(par, CTL_REGEN_N)];   // hit, then new-path records
  if (n == 0) return;
  const float4* q = P.queue[par];
  Cnt<kCount> cnt;
#pragma unroll
  for (int i = 0; i < C_NUM; ++i) cnt.c[i] = 0;
  uint32_t chunk = 0, chunk_end = 0;
  bool exhausted = false, active = false;
  int count = 0;   // ready segments in this warp's pool (the same in every lane)
  GridHold<Tab> gh;
  Dda s;
  uint32_t tag = 0;
  for (;;) {
    // set up new segments, a warp's worth at a time, while the pool has room
    while (count <= kPoolSegs - 32 && !exhausted) {
      if (chunk >= chunk_end) {
        uint32_t c = 0;
        if (lane == 0) c = atomicAdd(&P.ctl[ctl_index(par, CTL_QHEAD)], P.trace_chunk);
        c = __shfl_sync(FULL, c, 0);
        if (c >= n) { exhausted = true; break; }
        chunk = c;
        chunk_end = min(c + P.trace_chunk, n);
      }
      const uint32_t rec = chunk + (uint32_t)lane;
      chunk = min(chunk + 32u, chunk_end);
      bool run = false;
      Dda t;
      uint32_t ttag = 0, tjob = 0;
      if (rec < chunk_end && __float_as_uint(__ldg(&q[2 * (size_t)rec + 1]).z) != kNoSegment) {
        const float4 a = __ldg(&q[2 * (size_t)rec]), b = __ldg(&q[2 * (size_t)rec + 1]);
        ttag = __float_as_uint(b.z);
        tjob = __float_as_uint(b.w);
        GridHold<Tab> tg;
        tg.set(P, T, tjob);
        dda_begin_rec(tg.get(T), t, mk3(a.x, a.y, a.z), mk3(a.w, b.x, b.y));
        run = t.state == DDA_RUNNING;
        if (!run) P.hits[(size_t)(ttag & 1u) * P.n_slots + (ttag >> 1)] = pack_end(t.x, t.y, t.z, t.state);
      }
      const unsigned rm = __ballot_sync(FULL, run);
      if (run) {
        const int at = count + __popc(rm & lt);
        s_i[0][warp][at] = t.x; s_i[1][warp][at] = t.y; s_i[2][warp][at] = t.z; s_i[3][warp][at] = pack_signs(t);
        s_f[0][warp][at] = t.dx; s_f[1][warp][at] = t.dy; s_f[2][warp][at] = t.dz;
        s_f[3][warp][at] = t.ax; s_f[4][warp][at] = t.ay; s_f[5][warp][at] = t.az;
        s_u[0][warp][at] = ttag; s_u[1][warp][at] = tjob;
      }
      count += __popc(rm);
    }
    __syncwarp();
    // lanes without a segment take ready ones, from the top of the pool
    const unsigned need = __ballot_sync(FULL, !active);
    const int take = min(__popc(need), count);
    if (!active) {
      const int r = __popc(need & lt);
      if (r < take) {
        const int at = count - 1 - r;
        s.x = s_i[0][warp][at]; s.y = s_i[1][warp][at]; s.z = s_i[2][warp][at];
        const int32_t sg = s_i[3][warp][at];
        s.sx = (sg & 3) - 1; s.sy = ((sg >> 2) & 3) - 1; s.sz = ((sg >> 4) & 3) - 1;
        s.dx = s_f[0][warp][at]; s.dy = s_f[1][warp][at]; s.dz = s_f[2][warp][at];
        s.ax = s_f[3][warp][at]; s.ay = s_f[4][warp][at]; s.az = s_f[5][warp][at];
        s.steps = 0; s.cb = -1; s.bits = 0ull; s.state = DDA_RUNNING;
        tag = s_u[0][warp][at];
        gh.set(P, T, s_u[1][warp][at]);
        active = true;
      }
    }
    count -= take;
    __syncwarp();
    if (!__any_sync(FULL, active)) break;   // pool empty and queue exhausted
    if (active) {
      if constexpr (!kCount && k444) dda_steps_444<false>(gh.get(T), s, kTraceSteps, 0);
      else dda_steps<kCount, false, k444>(gh.get(T), s, kTraceSteps, cnt, 0);
      if (s.state != DDA_RUNNING) {
        P.hits[(size_t)(tag & 1u) * P.n_slots + (tag >> 1)] = pack_end(s.x, s.y, s.z, s.state);
        active = false;
      }
    }
  }
  flush_counters(cnt, P.counters);
}

// Ordered reduction of the per-sample outputs into each pixel's Kahan sums:
// sample order within a pixel is the same as one sample per launch.
__global__ void k_wf_accumulate(const JobEntry* jobs, const float4* sbuf) {
  const JobEntry& E = jobs[blockIdx.y];
  const long long px = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (px >= E.n_pixels || E.passes <= 0) return;
  float4 sum = E.J.sum[px], comp = E.J.comp[px];
  for (int k = 0; k < E.passes; ++k) kahan_add(sum, comp, sbuf[E.tile_begin + (long long)k * E.n_pixels + px]);
  E.J.sum[px] = sum;
  E.J.comp[px] = comp;
}

template <class Tab>
static void wf_shade(const WfParams& P, const Tab& T, int par, int persist_blocks, bool count, cudaStream_t st) {
  const int blocks = (P.n_slots + 127) / 128;
  if (count) {
    k_wf_shade<true, Tab><<<blocks, 128, 0, st>>>(P, T, par);
    k_wf_hit<true, Tab><<<persist_blocks, 128, 0, st>>>(P, T, par);
    k_wf_regen<true, Tab><<<persist_blocks / 8 * RegenBlocks<Tab>::value, 128, 0, st>>>(P, T, par);
  } else {
    k_wf_shade<false, Tab><<<blocks, 128, 0, st>>>(P, T, par);
    k_wf_hit<false, Tab><<<persist_blocks, 128, 0, st>>>(P, T, par);
    k_wf_regen<false, Tab><<<persist_blocks / 8 * RegenBlocks<Tab>::value, 128, 0, st>>>(P, T, par);
  }
}

static WfOneJob one_job(const WfJobTable& T) {
  WfOneJob o;
  o.e = T.e[0];
  o.g = T.g[0];
  return o;
}

cudaError_t launch_wf_shade(const WfParams& P, int par, int persist_blocks, bool count, cudaStream_t st,
                            const WfJobTable* T) {
  if (T && P.n_jobs == 1) wf_shade(P, one_job(*T), par, persist_blocks, count, st);
  else if (T && P.n_jobs <= kWfParamJobs) wf_shade(P, *T, par, persist_blocks, count, st);
  else wf_shade(P, WfNoTable{0}, par, persist_blocks, count, st);
  return cudaGetLastError();
}

template <bool kVote, bool k444, class Tab>
static void wf_trace_steps(const WfParams& P, const Tab& T, int par, int blocks, int steps, cudaStream_t st) {
  if (steps <= 8) k_wf_trace<false, 8, kVote, k444, Tab><<<blocks, 256, 0, st>>>(P, T, par);
  else if (steps <= 16) k_wf_trace<false, 16, kVote, k444, Tab><<<blocks, 256, 0, st>>>(P, T, par);
  else k_wf_trace<false, 32, kVote, k444, Tab><<<blocks, 256, 0, st>>>(P, T, par);
}

template <bool k444, class Tab>
static void wf_trace_shape(const WfParams& P, const Tab& T, int par, int blocks, int steps, bool count,
                           cudaStream_t st) {
  if (P.trace_form == 1) {   // pooled set-up
    if (count) k_wf_trace_pool<true, 8, k444, Tab><<<blocks, 256, 0, st>>>(P, T, par);
    else if (steps <= 4) k_wf_trace_pool<false, 4, k444, Tab><<<blocks, 256, 0, st>>>(P, T, par);
    else if (steps <= 8) k_wf_trace_pool<false, 8, k444, Tab><<<blocks, 256, 0, st>>>(P, T, par);
    else k_wf_trace_pool<false, 16, k444, Tab><<<blocks, 256, 0, st>>>(P, T, par);
    return;
  }
  if (count) k_wf_trace<true, 16, false, k444, Tab><<<blocks, 256, 0, st>>>(P, T, par);
  else if (P.refill_min > 0) wf_trace_steps<true, k444>(P, T, par, blocks, steps, st);
  else wf_trace_steps<false, k444>(P, T, par, blocks, steps, st);
}

template <class Tab>
static void wf_trace(const WfParams& P, const Tab& T, int par, int blocks, int steps, bool count, cudaStream_t st) {
  if (P.bricks_444) wf_trace_shape<true>(P, T, par, blocks, steps, count, st);
  else wf_trace_shape<false>(P, T, par, blocks, steps, count, st);
}

cudaError_t launch_wf_trace(const WfParams& P, int par, int blocks, int steps, bool count, cudaStream_t st,
                            const WfJobTable* T) {
  if (T && P.n_jobs == 1) wf_trace(P, one_job(*T), par, blocks, steps, count, st);
  else if (T && P.n_jobs <= kWfParamJobs) wf_trace(P, *T, par, blocks, steps, count, st);
  else wf_trace(P, WfNoTable{0}, par, blocks, steps, count, st);
  return cudaGetLastError();
}

cudaError_t launch_wf_accumulate(const JobEntry* jobs, int n_jobs, long long max_pixels, const float4* sbuf,
                                 cudaStream_t st) {
  if (n_jobs <= 0 || max_pixels <= 0) return cudaSuccess;
  dim3 grid((unsigned)((max_pixels + 255) / 256), (unsigned)n_jobs);
  k_wf_accumulate<<<grid, 256, 0, st>>>(jobs, sbuf);
  return cudaGetLastError();
}

void wf_carve(void* mem, size_t S, WfParams& P) {
  float4* f = (float4*)mem;
  for (int s = 0; s < 2; ++s) {
    WfState& x = P.x[s];
    x.a0 = f; x.a1 = f + S; x.a3 = f + 2 * S; x.a4 = f + 3 * S; x.a5 = f + 4 * S;
    f += 5 * S;
  }
  P.hr.h0 = f; P.hr.h1 = f + S; P.hr.h2 = f + 2 * S; P.hr.h3 = f + 3 * S;
  f += 4 * S;
  P.queue[0] = f;
  P.queue[1] = f + 4 * S;
  f += 8 * S;
  unsigned long long* h = (unsigned long long*)f;
  P.hits = h;
  P.hr.h4 = h + 2 * S;
  uint32_t* u = (uint32_t*)(h + 3 * S);
  P.x[0].flags = u;
  P.x[1].flags = u + S;
}

int wf_trace_blocks_per_sm() {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_wf_trace<false, 8, false, true, WfOneJob>, 256, 0);
  return n;
}

// ------------------------------------------------------------- trace rays
// out[4*i] = voxel x, y, z, flags (hit << 8 | ground << 9 | normal code).
__global__ void k_trace_rays(const Frame F, const JobDev J, const float* origins, const float* dirs,
                             int64_t n, int32_t* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Cnt<false> cnt;
  const v3 o = mk3(origins[3 * i], origins[3 * i + 1], origins[3 * i + 2]);
  const v3 d = mk3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]);
  Dda s;
  const Grid g = grid_of(F, J);
  dda_begin(g, s, o, d);
  if (s.state == DDA_RUNNING) dda_advance(g, s, 0x7fffffff, cnt);
  const bool h = dda_hit(F, s);
  int flags = (h ? 1 : 0) << 8 | ((h && s.state != DDA_HIT) ? 1 : 0) << 9 | (s.steps << 10);
  if (h) {
    const Basis b = voxel_basis(F, s.x, s.y, s.z, o, d);
    flags |= ((int)b.normal.x + 1) | (((int)b.normal.y + 1) << 2) | (((int)b.normal.z + 1) << 4);
  }
  out[4 * i] = s.x; out[4 * i + 1] = s.y; out[4 * i + 2] = s.z; out[4 * i + 3] = flags;
}

cudaError_t launch_trace_rays(const Frame& F, const JobDev& J, const float* origins, const float* dirs,
                              int64_t n, int32_t* out, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_trace_rays<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(F, J, origins, dirs, n, out);
  return cudaGetLastError();
}

// ------------------------------------------------------------------- pick
// focalDistance.vs:45-81: generateRay with rngOffset (0,0) and no pixel
// jitter consumption difference (the pinhole draws its jitter from the
// sequence start), AABB clip, traverse, exact voxel distance.
__global__ void k_pick(const Frame F, const JobDev J, float x, float y, float* out_dist, int32_t* out_voxel) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Cnt<false> cnt;
  Rng rng;
  rng.pixel = 0; rng.sample = 0; rng.call = 0; rng.ox = 0; rng.oy = 0;
  v3 o, d;
  generate_ray(F, J, mk3(x, y, 0.0f), rng, o, d);
  *out_dist = kInfinity;
  out_voxel[0] = out_voxel[1] = out_voxel[2] = -1;
  const float t = ray_aabb(o, d, ld3(F.bmin), ld3(F.bmax));
  if (t < 0.0f) return;
  Dda s;
  const Grid g = grid_of(F, J);
  dda_begin(g, s, o + t * d, d);
  if (s.state == DDA_RUNNING) dda_advance(g, s, 0x7fffffff, cnt);
  if (!dda_hit(F, s)) return;
  const v3 vs = ld3(F.vsize);
  const v3 vmin = mk3((float)s.x, (float)s.y, (float)s.z) * vs + ld3(F.bmin);
  *out_dist = ray_aabb(o, d, vmin, vmin + vs);
  out_voxel[0] = s.x; out_voxel[1] = s.y; out_voxel[2] = s.z;
}

// selectVoxel.vs:35-69: generateRay at window depth frag_z (the shader
// passes cameraNear), AABB clip, traverse, and the basis normal of the hit
// (voxelSpaceToWorldSpace).  Nothing hit: out[3] = 0.
__global__ void k_select(const Frame F, const JobDev J, float x, float y, float frag_z, int32_t* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Cnt<false> cnt;
  Rng rng;
  rng.pixel = 0; rng.sample = 0; rng.call = 0; rng.ox = 0; rng.oy = 0;
  v3 o, d;
  generate_ray(F, J, mk3(x, y, frag_z), rng, o, d);
  out[0] = out[1] = out[2] = -1;
  out[3] = 0;
  float* nrm = (float*)(out + 4);
  nrm[0] = nrm[1] = nrm[2] = 0.0f;
  const float t = ray_aabb(o, d, ld3(F.bmin), ld3(F.bmax));
  if (t < 0.0f) return;
  Dda s;
  const Grid g = grid_of(F, J);
  dda_begin(g, s, o + t * d, d);
  if (s.state == DDA_RUNNING) dda_advance(g, s, 0x7fffffff, cnt);
  if (!dda_hit(F, s)) return;
  const Basis b = voxel_basis(F, s.x, s.y, s.z, o, d);
  out[0] = s.x; out[1] = s.y; out[2] = s.z; out[3] = 1;
  nrm[0] = b.normal.x; nrm[1] = b.normal.y; nrm[2] = b.normal.z;
}

cudaError_t launch_select(const Frame& F, const JobDev& J, float x, float y, float frag_z, int32_t* out,
                          cudaStream_t st) {
  k_select<<<1, 32, 0, st>>>(F, J, x, y, frag_z, out);
  return cudaGetLastError();
}

cudaError_t launch_pick(const Frame& F, const JobDev& J, float x, float y, float* out_dist,
                        int32_t* out_voxel, cudaStream_t st) {
  k_pick<<<1, 32, 0, st>>>(F, J, x, y, out_dist, out_voxel);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- resolve
__global__ void k_resolve(const float4* sum, int32_t w, int32_t h, int32_t samples, float exposure,
                          float inv_gamma, uint32_t flags, float4* out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)w * h) return;
  const int x = (int)(i % w), y = (int)(i / w);
  float4 v = sum[i];
  const float n = samples > 0 ? (float)samples : 1.0f;
  v.x = v.x / n; v.y = v.y / n; v.z = v.z / n; v.w = v.w / n;
  if (flags & 2u) {
    v.x = vtb::vpow(v.x * exposure, inv_gamma);
    v.y = vtb::vpow(v.y * exposure, inv_gamma);
    v.z = vtb::vpow(v.z * exposure, inv_gamma);
  }
  const int oy = (flags & 1u) ? (h - 1 - y) : y;
  out[(int64_t)oy * w + x] = v;
}

cudaError_t launch_resolve(const float4* sum, int32_t w, int32_t h, int32_t samples, float exposure,
                           float inv_gamma, uint32_t flags, float4* out, cudaStream_t st) {
  const int64_t n = (int64_t)w * h;
  if (n <= 0) return cudaSuccess;
  k_resolve<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(sum, w, h, samples, exposure, inv_gamma, flags, out);
  return cudaGetLastError();
}

// --------------------------------------------------------------- builtins
__global__ void k_builtins(int32_t fn, const float* a, const float* b, float* out, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float x = a[i];
  float r;
  switch (fn) {
    case 0: r = vtb::vsin(x); break;
    case 1: r = vtb::vcos(x); break;
    case 2: r = vtb::vpow(x, b[i]); break;
    case 3: r = vtb::vacos(x); break;
    case 4: r = vtb::vatan2(x, b[i]); break;
    case 5: r = vtb::vlog2(x); break;
    case 6: r = vtb::vexp2(x); break;
    case 7: r = vtb::h2f(vtb::f2h(x)); break;
    default: r = 0.0f; break;
  }
  out[i] = r;
}

cudaError_t launch_builtins(int32_t fn, const float* a, const float* b, float* out, int64_t n,
                            cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_builtins<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(fn, a, b, out, n);
  return cudaGetLastError();
}

// ------------------------------------------------------ L2 read bandwidth
// `reps` sweeps of an L2-resident buffer in one launch, loads bypassing L1
// (ld.global.cg), four independent 16-byte loads in flight per thread; the
// XOR of everything read is stored per thread so that no load is dropped.
// Each sweep starts one grid-width further on, so a thread does not read
// the same lines in consecutive sweeps.
__global__ void __launch_bounds__(512) k_l2_read(const uint4* __restrict__ buf, uint32_t n, int32_t reps,
                                                 uint4* __restrict__ out) {
  const uint32_t T = gridDim.x * blockDim.x;
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  uint4 acc = make_uint4(0u, 0u, 0u, 0u);
  for (int32_t r = 0; r < reps; ++r) {
    const uint32_t base = (uint32_t)(((uint64_t)r * T + t) % n);
    uint32_t i = 0;
    for (; i + 3 * T < n; i += 4 * T) {
      uint4 v[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        uint32_t j = base + i + (uint32_t)k * T;
        if (j >= n) j -= n;
        v[k] = __ldcg(&buf[j]);
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) { acc.x ^= v[k].x; acc.y ^= v[k].y; acc.z ^= v[k].z; acc.w ^= v[k].w; }
    }
    for (; i < n; i += T) {
      uint32_t j = base + i;
      if (j >= n) j -= n;
      const uint4 v = __ldcg(&buf[j]);
      acc.x ^= v.x; acc.y ^= v.y; acc.z ^= v.z; acc.w ^= v.w;
    }
  }
  out[t] = acc;
}

cudaError_t launch_l2_read(const uint4* buf, uint32_t n, int32_t reps, uint4* out, int blocks, cudaStream_t st) {
  if (n == 0 || reps <= 0 || blocks <= 0) return cudaSuccess;
  k_l2_read<<<blocks, 512, 0, st>>>(buf, n, reps, out);
  return cudaGetLastError();
}

}  // namespace vt

namespace vt {
// The check word of the bounds-checked build (0 and enabled = false in a
// release build); reset clears it after reading.
cudaError_t read_check_word(uint32_t* word, bool* enabled, bool reset) {
#ifdef VT_CHECKED
  *enabled = true;
  cudaError_t e = cudaMemcpyFromSymbol(word, g_check_word, sizeof(uint32_t));
  if (e == cudaSuccess && reset) {
    const uint32_t zero = 0;
    e = cudaMemcpyToSymbol(g_check_word, &zero, sizeof(uint32_t));
  }
  return e;
#else
  *enabled = false;
  *word = 0;
  (void)reset;
  return cudaSuccess;
#endif
}
}  // namespace vt
