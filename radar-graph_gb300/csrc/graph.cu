// Device graph image, scans, frontier compaction and the degree-sort relabel.
//
// Degree sort (preprocessGraph, IO.h:843-895): the reference sorts
// pair<degree, id> with std::greater, i.e. degree descending and ties by
// DEScending original id, and gives rank r to the r-th pair.  Here a stable
// LSD radix sort on the 32-bit key ~degree runs over ids laid out in
// descending order, which yields exactly that order (the sort is stable, so
// equal degrees keep the descending-id input order).  Neighbour lists are then
// relabelled in place order (IO.h:877-895 keeps the order, it does not
// re-sort).

#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "rg_device.cuh"

namespace rg {

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local char g_err[512] = "";

rg_status fail(rg_status s, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return s;
}
void clear_error() { g_err[0] = 0; }
const char* last_error() { return g_err; }

rg_status cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  const char* f = strrchr(file, '/');
  fail(e == cudaErrorMemoryAllocation ? RG_ENOMEM : RG_ECUDA, "%s: %s (%s:%d)",
       cudaGetErrorString(e), what, f ? f + 1 : file, line);
  cudaGetLastError();  // clear a sticky-free error so the context stays usable
  return e == cudaErrorMemoryAllocation ? RG_ENOMEM : RG_ECUDA;
}

rg_status DevBuf::reserve(size_t b) {
  if (b <= bytes && p) return RG_OK;
  release();
  size_t want = b < 256 ? 256 : b;
  if (pooled) {  // usable from every stream once the allocating stream has it
    RG_CUDA(cudaMallocAsync(&p, want, 0));
    RG_CUDA(cudaStreamSynchronize(0));
  } else {
    RG_CUDA(cudaMalloc(&p, want));
  }
  bytes = want;
  return RG_OK;
}

Workspace::~Workspace() {
  if (h_info) cudaFreeHost(h_info);
  if (h_small) cudaFreeHost(h_small);
}

__global__ void read_small_kernel(const unsigned char* __restrict__ src, volatile unsigned char* dst, size_t bytes) {
  for (size_t i = threadIdx.x; i < bytes; i += blockDim.x) dst[i] = src[i];
  __threadfence_system();
}

rg_status read_small(const void* d_src, void* h_dst, size_t bytes, cudaStream_t st) {
  if (bytes == 0) return RG_OK;
  Ctx* c = nullptr;
  RG_TRY(get_ctx(&c));
  Workspace& ws = c->ws;
  if (bytes > kSmallRead || !ws.h_small_dev) {
    RG_CUDA(cudaMemcpyAsync(h_dst, d_src, bytes, cudaMemcpyDeviceToHost, st));
    RG_CUDA(cudaStreamSynchronize(st));
    return RG_OK;
  }
  read_small_kernel<<<1, 256, 0, st>>>(static_cast<const unsigned char*>(d_src), ws.h_small_dev, bytes);
  RG_CUDA(cudaGetLastError());
  RG_CUDA(cudaStreamSynchronize(st));
  memcpy(h_dst, ws.h_small, bytes);
  return RG_OK;
}

static thread_local Ctx* t_ctx = nullptr;

rg_status get_ctx(Ctx** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(RG_ENODEV, "no CUDA device: %s", cudaGetErrorString(e));
  }
  if (t_ctx && t_ctx->device == dev) {
    *out = t_ctx;
    return RG_OK;
  }
  // a thread that switches devices keeps one context per process lifetime of
  // the last device used; the old one is released
  delete t_ctx;
  t_ctx = nullptr;
  Ctx* c = new (std::nothrow) Ctx();
  if (!c) return fail(RG_ENOMEM, "host allocation failed");
  c->device = dev;
  {  // freed pool blocks stay mapped for reuse (graph images are large)
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    cudaGetLastError();
  }
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      cudaHostAlloc((void**)&c->ws.h_info, 64, cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer((void**)&c->ws.h_info_dev, c->ws.h_info, 0) != cudaSuccess ||
      cudaHostAlloc((void**)&c->ws.h_small, kSmallRead, cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer((void**)&c->ws.h_small_dev, c->ws.h_small, 0) != cudaSuccess ||
      c->ws.counters.reserve(4096) != RG_OK) {
    cudaGetLastError();
    delete c;
    return fail(RG_ECUDA, "stream/event/pinned allocation failed");
  }
  cudaMemset(c->ws.counters.p, 0, 4096);
  c->stream = c->own_stream;
  t_ctx = c;
  *out = c;
  return RG_OK;
}

Ctx& ctx() { return *t_ctx; }

// Binary search, degrees non-increasing: the first v with at most t entries.
__global__ void find_pull_split(const uint32_t* __restrict__ off, uint32_t n, uint32_t t, uint32_t* out) {
  uint32_t lo = 0, hi = n;
  while (lo < hi) {
    const uint32_t mid = lo + (hi - lo) / 2;
    if (off[mid + 1] - off[mid] <= t) hi = mid;
    else lo = mid + 1;
  }
  *out = lo;
}

uint32_t pull_split(const rg_graph* g, const DevGraph& pull_g, cudaStream_t st) {
  int64_t v = g->pull_split.load(std::memory_order_relaxed);
  if (v >= 0) return (uint32_t)v;
  Ctx* c = nullptr;
  if (get_ctx(&c) != RG_OK) return pull_g.n;  // a hint only: one group size for every vertex
  Workspace& ws = c->ws;
  uint32_t* d = reinterpret_cast<uint32_t*>(ws.counters.as<uint64_t>() + 8);  // a free scratch word
  find_pull_split<<<1, 1, 0, st>>>(pull_g.off, pull_g.n, 8u, d);
  uint32_t h = pull_g.n;
  if (cudaGetLastError() != cudaSuccess || read_small(d, &h, 4, st) != RG_OK) {
    cudaGetLastError();
    return pull_g.n;  // a hint only: one group size for every vertex
  }
  g->pull_split.store(h, std::memory_order_relaxed);
  return h;
}

rg_status copy_stream(cudaStream_t* out) {
  Ctx* c = nullptr;
  RG_TRY(get_ctx(&c));
  if (!c->copy_stream) RG_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
  *out = c->copy_stream;
  return RG_OK;
}

}  // namespace rg

extern "C" rg_status rg_set_stream(void* stream) {
  rg::Ctx* c = nullptr;
  RG_TRY(rg::get_ctx(&c));
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return RG_OK;
}

namespace rg {

// ---------------------------------------------------------------------------
// exclusive scan of uint32 (three kernels: tile sums, scan of sums, apply)
// ---------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

template <int kThreads>
__device__ __forceinline__ uint32_t block_exclusive_sum(uint32_t v, uint32_t* total) {
  __shared__ uint32_t warp_tot[kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_tot[w] = inc;
  __syncthreads();
  if (w == 0) {
    uint32_t t = lane < kThreads / 32 ? warp_tot[lane] : 0;
    uint32_t ti = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t u = __shfl_up_sync(0xffffffffu, ti, o);
      if (lane >= o) ti += u;
    }
    if (lane < kThreads / 32) warp_tot[lane] = ti - t;
    if (lane == kThreads / 32 - 1) *total = ti;
  }
  __syncthreads();
  uint32_t r = warp_tot[w] + inc - v;
  __syncthreads();
  return r;
}

__global__ void scan_tile_sums(const uint32_t* __restrict__ in, int64_t n, uint32_t* __restrict__ sums) {
  int64_t base = (int64_t)blockIdx.x * kScanTile;
  uint32_t s = 0;
  for (int i = 0; i < kScanItems; i++) {
    int64_t idx = base + (int64_t)i * kScanThreads + threadIdx.x;
    if (idx < n) s += in[idx];
  }
  __shared__ uint32_t tot;
  block_exclusive_sum<kScanThreads>(s, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// One block scans `nt` tile sums in place (exclusive) and writes the total.
__global__ void scan_sums(uint32_t* sums, int64_t nt, uint32_t* total_out) {
  __shared__ uint32_t carry_s, tot;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  for (int64_t base = 0; base < nt; base += kScanThreads) {
    int64_t i = base + threadIdx.x;
    uint32_t v = i < nt ? sums[i] : 0;
    uint32_t ex = block_exclusive_sum<kScanThreads>(v, &tot);
    uint32_t c = carry_s;
    if (i < nt) sums[i] = c + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry_s = c + tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total_out = carry_s;
}

__global__ void scan_apply(const uint32_t* __restrict__ in, int64_t n, const uint32_t* __restrict__ sums,
                           uint32_t* __restrict__ out) {
  // each thread scans kScanItems consecutive elements
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    int64_t idx = base + i;
    v[i] = idx < n ? in[idx] : 0;
    s += v[i];
  }
  __shared__ uint32_t tot;
  uint32_t ex = block_exclusive_sum<kScanThreads>(s, &tot) + sums[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; i++) {
    int64_t idx = base + i;
    if (idx < n) out[idx] = ex;
    ex += v[i];
  }
}

rg_status scan_u32(Workspace& ws, const uint32_t* in, uint32_t* out, int64_t n, cudaStream_t st) {
  int64_t nt = (n + kScanTile - 1) / kScanTile;
  if (nt == 0) nt = 1;
  RG_TRY(ws.scan_tmp.reserve(sizeof(uint32_t) * (nt + 1)));
  uint32_t* sums = ws.scan_tmp.as<uint32_t>();
  if (n > 0) scan_tile_sums<<<(unsigned)nt, kScanThreads, 0, st>>>(in, n, sums);
  else RG_CUDA(cudaMemsetAsync(sums, 0, 4, st));
  scan_sums<<<1, kScanThreads, 0, st>>>(sums, nt, out + n);
  if (n > 0) scan_apply<<<(unsigned)nt, kScanThreads, 0, st>>>(in, n, sums, out);
  RG_CUDA(cudaGetLastError());
  return RG_OK;
}

// ---------------------------------------------------------------------------
// bitmap -> ascending queue + degree scan (ligra.h:161-192 compaction,
// vertexSubset.h:196-211 toSparse)
// ---------------------------------------------------------------------------
constexpr int kCompThreads = 256;
// Words per lane: a warp emits its non-zero words one after another, each
// step waiting on its offsets, so fewer words per warp means more warps to
// hide that latency (RMAT s24 four-app step: 8 words 50.2 ms, 2 words
// 49.1 ms, 1 word 49.5 ms).
constexpr int kCompWords = 2;
constexpr int kCompTile = kCompThreads * kCompWords;  // words per block
constexpr int kCompWarps = kCompThreads / 32;
constexpr int kWarpWords = kCompWords * 32;  // consecutive words per warp

// Count and degree sum of the set bits of word x (vertices vb .. vb+31).  The
// degrees of a run of consecutive set bits [a, e) telescope to
// off[vb+e] - off[vb+a], so a dense word costs two loads, not 64.  Bits at
// or above n are never set, so vb + e <= n.
__device__ __forceinline__ void word_count_deg(uint32_t x, uint32_t vb, const uint32_t* __restrict__ off,
                                               uint32_t& c, uint32_t& d) {
  c += __popc(x);
  uint32_t starts = x & ~(x << 1);
  while (starts) {
    const int a = __ffs(starts) - 1;
    starts &= starts - 1;
    const uint32_t rest = ~x >> a;  // bit 0 is clear: bit a of x is set
    const int e = rest ? a + __ffs(rest) - 1 : 32;
    d += off[vb + e] - off[vb + a];
  }
}

// A warp owns kWarpWords consecutive words, lane l the words l, l+32, ...
// (coalesced loads of the bitmap).
__device__ __forceinline__ void warp_words(const uint32_t* __restrict__ bits, int64_t nwords, int64_t wbase,
                                           uint32_t (&xs)[kCompWords]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int i = 0; i < kCompWords; i++) {
    const int64_t w = wbase + i * 32 + lane;
    xs[i] = w < nwords ? bits[w] : 0u;
  }
}

__global__ void comp_count(const uint32_t* __restrict__ bits, int64_t nwords, const uint32_t* __restrict__ off,
                           uint32_t* __restrict__ part_c, uint32_t* __restrict__ part_d) {
  const int lane = threadIdx.x & 31;
  const int64_t wbase = (int64_t)blockIdx.x * kCompTile + (int64_t)(threadIdx.x >> 5) * kWarpWords;
  uint32_t xs[kCompWords];
  warp_words(bits, nwords, wbase, xs);
  uint32_t c = 0, d = 0;
#pragma unroll
  for (int i = 0; i < kCompWords; i++) {
    if (xs[i]) word_count_deg(xs[i], (uint32_t)((wbase + i * 32 + lane) * 32), off, c, d);
  }
  __shared__ uint32_t tc, td;
  block_exclusive_sum<kCompThreads>(c, &tc);
  block_exclusive_sum<kCompThreads>(d, &td);
  if (threadIdx.x == 0) {
    part_c[blockIdx.x] = tc;
    part_d[blockIdx.x] = td;
  }
}

// Also writes (count, degsum) straight into the caller's mapped host words
// `host_info`, so a level's host sync needs no copy (none on a copy engine
// another stream may be using).
__global__ void comp_scan(uint32_t* part_c, uint32_t* part_d, int64_t nt, uint64_t* info,
                          uint32_t* qoff_total_slot_base, volatile uint64_t* host_info) {
  __shared__ uint32_t cc, cd, tc, td;
  if (threadIdx.x == 0) { cc = 0; cd = 0; }
  __syncthreads();
  for (int64_t base = 0; base < nt; base += kCompThreads) {
    int64_t i = base + threadIdx.x;
    uint32_t vc = i < nt ? part_c[i] : 0, vd = i < nt ? part_d[i] : 0;
    uint32_t ec = block_exclusive_sum<kCompThreads>(vc, &tc);
    uint32_t ed = block_exclusive_sum<kCompThreads>(vd, &td);
    uint32_t c0 = cc, d0 = cd;
    if (i < nt) { part_c[i] = c0 + ec; part_d[i] = d0 + ed; }
    __syncthreads();
    if (threadIdx.x == 0) { cc = c0 + tc; cd = d0 + td; }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    info[0] = cc;
    info[1] = cd;
    // qoff[count] = degsum: the slot sits right after the last queue entry
    if (qoff_total_slot_base) qoff_total_slot_base[cc] = cd;
    host_info[0] = cc;
    host_info[1] = cd;
    __threadfence_system();
  }
}

// Emission: the warp walks its non-zero words in order, one word per step
// with lane b on bit b, so the queue, qoff and depth stores of a word are
// consecutive (coalesced) and its degrees come from 33 consecutive offsets.
__global__ void comp_emit(const uint32_t* __restrict__ bits, int64_t nwords, const uint32_t* __restrict__ off,
                          const uint32_t* __restrict__ part_c, const uint32_t* __restrict__ part_d,
                          uint32_t* __restrict__ queue, uint32_t* __restrict__ qoff, int32_t* depth,
                          int32_t level, uint32_t* or_into) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t wbase = (int64_t)blockIdx.x * kCompTile + (int64_t)warp * kWarpWords;
  uint32_t xs[kCompWords];
  warp_words(bits, nwords, wbase, xs);
  uint32_t c = 0, d = 0;
#pragma unroll
  for (int i = 0; i < kCompWords; i++) {
    if (xs[i]) {
      const int64_t w = wbase + i * 32 + lane;
      word_count_deg(xs[i], (uint32_t)(w * 32), off, c, d);
      if (or_into) or_into[w] |= xs[i];
    }
  }
  // the warp's place in the block, after the block's place in the frontier
  __shared__ uint32_t wc[kCompWarps], wd[kCompWarps];
  c = __reduce_add_sync(0xffffffffu, c);
  d = __reduce_add_sync(0xffffffffu, d);
  if (lane == 0) {
    wc[warp] = c;
    wd[warp] = d;
  }
  __syncthreads();
  uint32_t pc = part_c[blockIdx.x], pd = part_d[blockIdx.x];
  for (int j = 0; j < warp; j++) {
    pc += wc[j];
    pd += wd[j];
  }
  const uint32_t below_mask = (1u << lane) - 1u;
#pragma unroll
  for (int i = 0; i < kCompWords; i++) {
    unsigned nz = __ballot_sync(0xffffffffu, xs[i] != 0u);
    while (nz) {
      const int j = __ffs(nz) - 1;
      nz &= nz - 1;
      const uint32_t x = __shfl_sync(0xffffffffu, xs[i], j);
      const uint32_t v = (uint32_t)((wbase + i * 32 + j) * 32) + (uint32_t)lane;
      const bool set = (x >> lane) & 1u;
      const uint32_t dg = set ? off[v + 1] - off[v] : 0u;
      uint32_t inc = dg;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
      }
      if (set) {
        const uint32_t at = pc + (uint32_t)__popc(x & below_mask);
        queue[at] = v;
        qoff[at] = pd + inc - dg;
        if (depth) depth[v] = level;
      }
      pc += (uint32_t)__popc(x);
      pd += __shfl_sync(0xffffffffu, inc, 31);
    }
  }
}

rg_status compact_bits(const rg_graph* g, Frontier& f, cudaStream_t st, bool sync, int32_t* depth,
                       int32_t level, uint32_t* or_into, uint32_t* queue_out, uint32_t* qoff_out,
                       const uint32_t* deg_off) {
  Workspace& ws = ctx().ws;
  const uint32_t* doff = deg_off ? deg_off : g->off.as<uint32_t>();
  const int64_t nwords = (g->n + 31) / 32;
  const int64_t nt = (nwords + kCompTile - 1) / kCompTile;
  RG_TRY(ws.scan_partials.reserve(sizeof(uint32_t) * 2 * (nt + 1)));
  uint32_t* pc = ws.scan_partials.as<uint32_t>();
  uint32_t* pd = pc + nt + 1;
  uint32_t* q = queue_out ? queue_out : f.queue.as<uint32_t>();
  uint32_t* qo = qoff_out ? qoff_out : f.qoff.as<uint32_t>();
  uint64_t* info = ws.counters.as<uint64_t>();
  comp_count<<<(unsigned)nt, kCompThreads, 0, st>>>(f.bits.as<uint32_t>(), nwords, doff, pc, pd);
  comp_scan<<<1, kCompThreads, 0, st>>>(pc, pd, nt, info, qo, ws.h_info_dev);
  comp_emit<<<(unsigned)nt, kCompThreads, 0, st>>>(f.bits.as<uint32_t>(), nwords, doff, pc, pd, q, qo, depth,
                                                   level, or_into);
  RG_CUDA(cudaGetLastError());
  f.queue_valid = (queue_out == nullptr);
  f.bits_valid = true;
  if (sync) {
    RG_CUDA(cudaStreamSynchronize(st));
    f.count = (int64_t)ws.h_info[0];
    f.degsum = (int64_t)ws.h_info[1];
  }
  return RG_OK;
}

rg_status frontier_alloc(const rg_graph* g, Frontier& f) {
  const int64_t nwords = (g->n + 31) / 32;
  RG_TRY(f.queue.reserve(sizeof(uint32_t) * (g->n + 64)));
  RG_TRY(f.qoff.reserve(sizeof(uint32_t) * (g->n + 65)));
  RG_TRY(f.bits.reserve(sizeof(uint32_t) * (nwords + 8)));
  return RG_OK;
}

__global__ void set_bits_from_queue(const uint32_t* __restrict__ q, int64_t k, uint32_t* bits) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) atomicOr(bits + (q[i] >> 5), 1u << (q[i] & 31));
}

rg_status frontier_bits_from_queue(const rg_graph* g, Frontier& f, cudaStream_t st) {
  const int64_t nwords = (g->n + 31) / 32;
  RG_CUDA(cudaMemsetAsync(f.bits.p, 0, sizeof(uint32_t) * nwords, st));
  if (f.count > 0) {
    set_bits_from_queue<<<(unsigned)((f.count + 255) / 256), 256, 0, st>>>(f.queue.as<uint32_t>(), f.count,
                                                                          f.bits.as<uint32_t>());
  }
  RG_CUDA(cudaGetLastError());
  f.bits_valid = true;
  return RG_OK;
}

__global__ void lookup_kernel(const uint32_t* __restrict__ new_ids, const uint32_t* __restrict__ off,
                              const uint32_t* __restrict__ ids, int64_t k, uint32_t* __restrict__ out_id,
                              uint32_t* __restrict__ out_deg) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) {
    const uint32_t v = new_ids ? new_ids[ids[i]] : ids[i];
    out_id[i] = v;
    out_deg[i] = off[v + 1] - off[v];
  }
}

rg_status host_arrays(const rg_graph* g) {
  std::lock_guard<std::mutex> lk(g->host_mu);
  if (g->host_ready) return RG_OK;
  const int64_t n = g->n;
  HostU32 off(n + 1);
  RG_CUDA(cudaMemcpy(off.data(), g->off.p, 4 * (n + 1), cudaMemcpyDeviceToHost));
  g->h_deg.resize(n);
#pragma omp parallel for
  for (int64_t v = 0; v < n; v++) g->h_deg[v] = off[v + 1] - off[v];
  if (g->sorted) {
    g->h_new_ids.resize(n);
    RG_CUDA(cudaMemcpy(g->h_new_ids.data(), g->new_ids.p, 4 * n, cudaMemcpyDeviceToHost));
  }
  if (g->directed) {
    RG_CUDA(cudaMemcpy(off.data(), g->in_off.p, 4 * (n + 1), cudaMemcpyDeviceToHost));
    g->h_in_deg.resize(n);
#pragma omp parallel for
    for (int64_t v = 0; v < n; v++) g->h_in_deg[v] = off[v + 1] - off[v];
  }
  g->host_ready = true;
  return RG_OK;
}

rg_status lookup_ids(const rg_graph* g, const uint32_t* ids, int64_t k, bool orig, uint32_t* internal_out,
                     uint32_t* deg_out, bool in_degree) {
  in_degree = in_degree && g->directed;
  for (int64_t i = 0; i < k; i++) {
    if (ids[i] >= (uint64_t)g->n) return fail(RG_EINVAL, "vertex id %u >= n", ids[i]);
  }
  const bool map = orig && g->sorted;
  bool ready;
  {
    std::lock_guard<std::mutex> lk(g->host_mu);
    ready = g->host_ready;
  }
  if (ready || k > 4096) {
    RG_TRY(host_arrays(g));
    if ((in_degree ? g->h_in_deg : g->h_deg).size() != (size_t)g->n || (map && g->h_new_ids.size() != (size_t)g->n))
      return fail(RG_EUNSUPPORTED, "host degree arrays missing");
    for (int64_t i = 0; i < k; i++) {
      const uint32_t v = map ? g->h_new_ids[ids[i]] : ids[i];
      if (internal_out) internal_out[i] = v;
      if (deg_out) deg_out[i] = in_degree ? g->h_in_deg[v] : g->h_deg[v];
    }
    return RG_OK;
  }
  if (k == 0) return RG_OK;
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  cudaStream_t st = cx->stream;
  RG_TRY(cx->ws.lookup.reserve(12 * (size_t)k));
  uint32_t* d = cx->ws.lookup.as<uint32_t>();
  std::vector<uint32_t> back(2 * k);
  RG_CUDA(cudaMemcpyAsync(d, ids, 4 * k, cudaMemcpyHostToDevice, st));
  lookup_kernel<<<(unsigned)((k + 255) / 256), 256, 0, st>>>(map ? g->new_ids.as<uint32_t>() : nullptr,
                                                             (in_degree ? g->in_off : g->off).as<uint32_t>(), d, k,
                                                             d + k, d + 2 * k);
  RG_CUDA(cudaGetLastError());
  RG_TRY(read_small(d + k, back.data(), 8 * (size_t)k, st));
  for (int64_t i = 0; i < k; i++) {
    if (internal_out) internal_out[i] = back[i];
    if (deg_out) deg_out[i] = back[k + i];
  }
  return RG_OK;
}

rg_status frontier_from_host(const rg_graph* g, Frontier& f, const uint32_t* ids, int64_t k,
                             cudaStream_t st) {
  RG_TRY(frontier_alloc(g, f));
  if (k > g->n + 64) return fail(RG_EINVAL, "frontier larger than n+64 entries");
  std::vector<uint32_t> qo(k + 1), deg(k);
  RG_TRY(lookup_ids(g, ids, k, false, nullptr, deg.data()));
  uint64_t acc = 0;
  for (int64_t i = 0; i < k; i++) {
    qo[i] = (uint32_t)acc;
    acc += deg[i];
  }
  qo[k] = (uint32_t)acc;
  if (k) RG_CUDA(cudaMemcpyAsync(f.queue.p, ids, 4 * k, cudaMemcpyHostToDevice, st));
  RG_CUDA(cudaMemcpyAsync(f.qoff.p, qo.data(), 4 * (k + 1), cudaMemcpyHostToDevice, st));
  f.count = k;
  f.degsum = (int64_t)acc;
  f.queue_valid = true;
  RG_TRY(frontier_bits_from_queue(g, f, st));
  // the host vector must outlive the async copy
  RG_CUDA(cudaStreamSynchronize(st));
  return RG_OK;
}

__global__ void fill_all_bits(uint32_t* bits, int64_t n) {
  int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t nwords = (n + 31) / 32;
  if (w < nwords) {
    int64_t rem = n - w * 32;
    bits[w] = rem >= 32 ? 0xffffffffu : ((1u << rem) - 1u);
  }
}

rg_status frontier_set_all(const rg_graph* g, Frontier& f, cudaStream_t st) {
  RG_TRY(frontier_alloc(g, f));
  const int64_t nwords = (g->n + 31) / 32;
  fill_all_bits<<<(unsigned)((nwords + 255) / 256), 256, 0, st>>>(f.bits.as<uint32_t>(), g->n);
  RG_CUDA(cudaGetLastError());
  f.bits_valid = true;
  return compact_bits(g, f, st, true);
}

// ---------------------------------------------------------------------------
// graph image
// ---------------------------------------------------------------------------

// chunk_v[c] = source vertex of edge min(c*kSweepChunk, m-1), c = 0..nchunks.
__global__ void build_chunk_starts(const uint32_t* __restrict__ off, uint32_t n, uint32_t m, int64_t nchunks,
                                   uint32_t* __restrict__ chunk_v) {
  int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c > nchunks) return;
  uint64_t e = (uint64_t)c * kSweepChunk;
  if (e >= m) e = m - 1;
  chunk_v[c] = upper_index(off, 0u, n - 1, (uint32_t)e);
}

static rg_status finish_graph(rg_graph* g) {
  cudaStream_t st = ctx().stream;
  if (g->m > 0) {
    g->nchunks = (g->m + kSweepChunk - 1) / kSweepChunk;
    RG_TRY(g->chunk_v.reserve(sizeof(uint32_t) * (g->nchunks + 1)));
    build_chunk_starts<<<(unsigned)((g->nchunks + 1 + 255) / 256), 256, 0, st>>>(
        g->off.as<uint32_t>(), (uint32_t)g->n, (uint32_t)g->m, g->nchunks, g->chunk_v.as<uint32_t>());
    RG_CUDA(cudaGetLastError());
    if (g->directed) {
      RG_TRY(g->in_chunk_v.reserve(sizeof(uint32_t) * (g->nchunks + 1)));
      build_chunk_starts<<<(unsigned)((g->nchunks + 1 + 255) / 256), 256, 0, st>>>(
          g->in_off.as<uint32_t>(), (uint32_t)g->n, (uint32_t)g->m, g->nchunks, g->in_chunk_v.as<uint32_t>());
      RG_CUDA(cudaGetLastError());
    }
  }
  RG_CUDA(cudaStreamSynchronize(st));
  return RG_OK;
}

static rg_status new_graph(rg_graph** out) {
  Ctx* c = nullptr;
  RG_TRY(get_ctx(&c));
  rg_graph* g = new (std::nothrow) rg_graph();
  if (!g) return fail(RG_ENOMEM, "host allocation failed");
  static std::atomic<uint64_t> next_uid{1};
  g->uid = next_uid++;
  g->device = c->device;
  *out = g;
  return RG_OK;
}

}  // namespace rg

rg_graph::~rg_graph() {}

using namespace rg;

static rg_status graph_create_common(int64_t n, int64_t m, const uint32_t* off, const uint32_t* adj,
                                     cudaMemcpyKind kind, rg_graph** out) {
  if (!out || n <= 0 || m < 0 || !off || (m > 0 && !adj)) {
    return fail(RG_EINVAL, "rg_graph_create: bad arguments");
  }
  if (m >= 0xFFFFFFFFll || n >= 0xFFFFFFFFll) {
    return fail(RG_EUNSUPPORTED, "rg_graph_create: >= 2^32 edges or vertices");
  }
  HostU32 dev_off_copy;  // a host copy of the offsets only when they live on the device
  const uint32_t* h_off = off;
  if (kind != cudaMemcpyHostToDevice) {
    dev_off_copy.resize(n + 1);
    RG_CUDA(cudaMemcpy(dev_off_copy.data(), off, 4 * (n + 1), cudaMemcpyDeviceToHost));
    h_off = dev_off_copy.data();
  }
  if (h_off[0] != 0 || h_off[n] != (uint32_t)m) return fail(RG_EINVAL, "offsets must start at 0 and end at m");
  rg_graph* g = nullptr;
  RG_TRY(new_graph(&g));
  g->n = n;
  g->m = m;
  g->h_deg.resize(n);
  rg_status s;
  if ((s = g->off.reserve(4 * (n + 1))) != RG_OK || (s = g->adj.reserve(4 * (m + 8))) != RG_OK) {
    delete g;
    return s;
  }
  // host degrees and the monotonicity check run on a helper thread (all
  // cores) while this thread uploads the CSR
  int64_t bad_at = -1;
  uint32_t mx = 0;
  std::thread degrees([&] {
    int64_t bad = INT64_MAX;
    uint32_t m_loc = 0;
#pragma omp parallel for reduction(max : m_loc) reduction(min : bad)
    for (int64_t v = 0; v < n; v++) {
      if (h_off[v + 1] < h_off[v]) bad = std::min(bad, v);
      const uint32_t d = h_off[v + 1] - h_off[v];
      g->h_deg[v] = d;
      m_loc = std::max(m_loc, d);
    }
    mx = m_loc;
    bad_at = bad == INT64_MAX ? -1 : bad;
  });
  cudaStream_t st = ctx().stream;
  cudaError_t e = cudaMemcpyAsync(g->off.p, off, 4 * (n + 1), kind, st);
  if (e == cudaSuccess && m > 0) e = cudaMemcpyAsync(g->adj.p, adj, 4 * m, kind, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(g->adj.as<uint32_t>() + m, 0, 32, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  degrees.join();
  if (e != cudaSuccess) {
    delete g;
    return cuda_fail(e, "graph upload", __FILE__, __LINE__);
  }
  if (bad_at >= 0) {
    delete g;
    return fail(RG_EINVAL, "offsets not monotone at %lld", (long long)bad_at);
  }
  g->max_deg = mx;
  g->host_ready = true;  // an uploaded graph's host degrees are complete (it has no permutation)
  if ((s = finish_graph(g)) != RG_OK) { delete g; return s; }
  *out = g;
  return RG_OK;
}

extern "C" rg_status rg_graph_create(int64_t n, int64_t m, const uint32_t* h_off, const uint32_t* h_adj,
                                     rg_graph** out) {
  return graph_create_common(n, m, h_off, h_adj, cudaMemcpyHostToDevice, out);
}

extern "C" rg_status rg_graph_create_device(int64_t n, int64_t m, const uint32_t* d_off,
                                            const uint32_t* d_adj, rg_graph** out) {
  return graph_create_common(n, m, d_off, d_adj, cudaMemcpyDeviceToDevice, out);
}

namespace rg {
void drop_hub_cache(const rg_graph* g);
}

extern "C" rg_status rg_graph_free(rg_graph* g) {
  if (!g) return RG_OK;
  rg::drop_hub_cache(g);
  // no work may still read the graph when its pooled buffers go back
  // (cudaFree would synchronize the device the same way)
  cudaDeviceSynchronize();
  delete g;
  return RG_OK;
}

extern "C" rg_status rg_graph_info(const rg_graph* g, int64_t* n, int64_t* m, int* sorted) {
  if (!g) return fail(RG_EINVAL, "null graph");
  if (n) *n = g->n;
  if (m) *m = g->m;
  if (sorted) *sorted = g->sorted ? 1 : 0;
  return RG_OK;
}

extern "C" rg_status rg_graph_download(const rg_graph* g, uint32_t* h_off, uint32_t* h_adj, uint32_t* h_new_ids) {
  if (!g) return fail(RG_EINVAL, "null graph");
  if (h_off) RG_CUDA(cudaMemcpy(h_off, g->off.p, 4 * (g->n + 1), cudaMemcpyDeviceToHost));
  if (h_adj && g->m) RG_CUDA(cudaMemcpy(h_adj, g->adj.p, 4 * g->m, cudaMemcpyDeviceToHost));
  if (h_new_ids) {
    if (g->sorted) RG_CUDA(cudaMemcpy(h_new_ids, g->new_ids.p, 4 * g->n, cudaMemcpyDeviceToHost));
    else for (int64_t i = 0; i < g->n; i++) h_new_ids[i] = (uint32_t)i;
  }
  return RG_OK;
}

// ---------------------------------------------------------------------------
// degree sort
// ---------------------------------------------------------------------------
namespace rg {

constexpr int kSortThreads = 256;
constexpr int kSortSub = 16;  // sub-tiles per block
constexpr int kSortTile = kSortThreads * kSortSub;

// key[i] = ~deg(id), val[i] = id with ids laid out in DESCENDING order.
__global__ void sort_init(const uint32_t* __restrict__ off, uint32_t n, uint32_t* key, uint32_t* val) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    uint32_t v = n - 1 - (uint32_t)i;
    key[i] = ~(off[v + 1] - off[v]);
    val[i] = v;
  }
}

__global__ void sort_hist(const uint32_t* __restrict__ key, int64_t n, int shift, int64_t nblocks,
                          uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  int64_t base = (int64_t)blockIdx.x * kSortTile;
  for (int s = 0; s < kSortSub; s++) {
    int64_t i = base + (int64_t)s * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(key[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: sub-tiles in order, threads in order within a sub-tile.
__global__ void sort_scatter(const uint32_t* __restrict__ key, const uint32_t* __restrict__ val, int64_t n,
                             int shift, int64_t nblocks, const uint32_t* __restrict__ hist_scan,
                             uint32_t* __restrict__ key_out, uint32_t* __restrict__ val_out) {
  constexpr int kWarps = kSortThreads / 32;
  __shared__ uint32_t running[256];
  __shared__ uint32_t wcount[kWarps][257];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  running[threadIdx.x] = hist_scan[(int64_t)threadIdx.x * nblocks + blockIdx.x];
  int64_t base = (int64_t)blockIdx.x * kSortTile;
  for (int s = 0; s < kSortSub; s++) {
    for (int d = threadIdx.x; d < kWarps * 257; d += kSortThreads) (&wcount[0][0])[d] = 0;
    __syncthreads();
    int64_t i = base + (int64_t)s * kSortThreads + threadIdx.x;
    bool valid = i < n;
    uint32_t k = valid ? key[i] : 0, v = valid ? val[i] : 0;
    uint32_t digit = valid ? ((k >> shift) & 255u) : 256u;
    uint32_t peers = __match_any_sync(0xffffffffu, digit);
    uint32_t rank = __popc(peers & ((1u << lane) - 1u));
    if (rank == 0) wcount[w][digit] = __popc(peers);
    __syncthreads();
    uint32_t pos = 0;
    if (valid) {
      pos = running[digit] + rank;
      for (int ww = 0; ww < w; ww++) pos += wcount[ww][digit];
    }
    __syncthreads();
    {
      uint32_t t = 0;
      for (int ww = 0; ww < kWarps; ww++) t += wcount[ww][threadIdx.x];
      running[threadIdx.x] += t;
    }
    if (valid) {
      key_out[pos] = k;
      val_out[pos] = v;
    }
    __syncthreads();
  }
}

__global__ void rank_to_ids(const uint32_t* __restrict__ sorted_ids, const uint32_t* __restrict__ off, uint32_t n,
                            uint32_t* __restrict__ new_ids, uint32_t* __restrict__ new_deg) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) {
    uint32_t v = sorted_ids[r];
    new_ids[v] = (uint32_t)r;
    new_deg[r] = off[v + 1] - off[v];
  }
}

// Edge-balanced relabel: every warp owns kSweepChunk consecutive edges of the
// original CSR (16-byte loads), finds each edge's source from the chunk
// partition, and writes new_ids[neighbour] at the source's new position.
// The neighbour array may be pinned host memory read over the host link
// (rg_graph_create_sorted); it then has no padding, so the last partial
// group of four is read entry by entry.
__global__ void __launch_bounds__(256) relabel_sweep(DevGraph g, const uint32_t* __restrict__ chunk_v,
                                                     uint32_t nchunks, const uint32_t* __restrict__ new_ids,
                                                     const uint32_t* __restrict__ new_off,
                                                     uint32_t* __restrict__ new_adj, unsigned int* bad_id) {
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t c = warp; c < nchunks; c += nwarps) {
    const uint32_t vlo = chunk_v[c], vhi = chunk_v[c + 1];
#pragma unroll
    for (int r = 0; r < kSweepChunk / 128; r++) {
      const uint32_t e = c * kSweepChunk + r * 128 + lane * 4;
      if (e >= g.m) continue;
      uint32_t dd[4];
      if (e + 4 <= g.m) {
        const uint4 d4 = __ldg(reinterpret_cast<const uint4*>(g.adj + e));
        dd[0] = d4.x;
        dd[1] = d4.y;
        dd[2] = d4.z;
        dd[3] = d4.w;
      } else {
#pragma unroll
        for (int i = 0; i < 4; i++) dd[i] = e + i < g.m ? __ldg(g.adj + e + i) : 0u;
      }
      uint32_t s = upper_index(g.off, vlo, vhi, e);
      uint32_t nxt = g.off[s + 1];
      uint32_t base = new_off[new_ids[s]] - g.off[s];  // modulo 2^32; base + e is the new slot
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const uint32_t ee = e + i;
        if (ee >= g.m) break;
        if (ee >= nxt) {
          do { s++; nxt = g.off[s + 1]; } while (ee >= nxt);
          base = new_off[new_ids[s]] - g.off[s];
        }
        if (dd[i] < g.n) {
          new_adj[base + ee] = new_ids[dd[i]];
        } else {  // a neighbour id out of range: reported, never used as an index
          new_adj[base + ee] = 0u;
          atomicOr(bad_id, 1u);
        }
      }
    }
  }
}

}  // namespace rg

// in-degree of each rank's vertex (a directed graph's new in-lists)
__global__ void rank_in_deg(const uint32_t* __restrict__ sorted_ids, const uint32_t* __restrict__ in_off, uint32_t n,
                            uint32_t* __restrict__ new_in_deg) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < n) {
    const uint32_t v = sorted_ids[r];
    new_in_deg[r] = in_off[v + 1] - in_off[v];
  }
}

// Degree sort (IO.h:728-903): ranks by out-degree, or for a directed graph by
// in-degree unless by_out (-preprocess 1 / 0, IO.h:739-750); both lists of a
// directed graph are relabelled, their order kept.
static rg_status degree_sort_impl(const rg_graph* g, bool by_out, rg_graph** out, uint32_t* h_new_ids) {
  if (!g || !out) return fail(RG_EINVAL, "rg_graph_degree_sort: null argument");
  const int64_t n = g->n, m = g->m;
  const bool by_in = g->directed && !by_out;
  Ctx* c = nullptr;
  RG_TRY(get_ctx(&c));
  cudaStream_t st = c->stream;
  Workspace& ws = c->ws;
  // temporaries from the stream-ordered pool, released in order on `st`
  DevBuf k0{true, st}, v0{true, st}, k1{true, st}, v1{true, st}, hist{true, st}, new_deg{true, st}, bad{true, st};
  RG_TRY(bad.reserve(16));
  RG_CUDA(cudaMemsetAsync(bad.p, 0, 4, st));
  const int64_t nblocks = (n + kSortTile - 1) / kSortTile;
  RG_TRY(k0.reserve(4 * n)); RG_TRY(v0.reserve(4 * n));
  RG_TRY(k1.reserve(4 * n)); RG_TRY(v1.reserve(4 * n));
  RG_TRY(hist.reserve(4 * (256 * nblocks + 1)));
  sort_init<<<(unsigned)((n + 255) / 256), 256, 0, st>>>((by_in ? g->in_off : g->off).as<uint32_t>(), (uint32_t)n,
                                                        k0.as<uint32_t>(), v0.as<uint32_t>());
  // ~deg differs from 0xFFFFFFFF only in the low bits that max_deg spans
  // (in-degrees: all 32 bits, their maximum is not kept)
  int bits = 0;
  while (bits < 32 && (g->max_deg >> bits) != 0) bits++;
  if (by_in) bits = 32;
  int passes = (bits + 7) / 8;
  uint32_t *ka = k0.as<uint32_t>(), *va = v0.as<uint32_t>(), *kb = k1.as<uint32_t>(), *vb = v1.as<uint32_t>();
  for (int p = 0; p < passes; p++) {
    int shift = 8 * p;
    sort_hist<<<(unsigned)nblocks, kSortThreads, 0, st>>>(ka, n, shift, nblocks, hist.as<uint32_t>());
    RG_TRY(scan_u32(ws, hist.as<uint32_t>(), hist.as<uint32_t>(), 256 * nblocks, st));
    sort_scatter<<<(unsigned)nblocks, kSortThreads, 0, st>>>(ka, va, n, shift, nblocks, hist.as<uint32_t>(), kb,
                                                             vb);
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  RG_CUDA(cudaGetLastError());
  rg_graph* ng = nullptr;
  RG_TRY(new_graph(&ng));
  ng->n = n;
  ng->m = m;
  rg_status s;
  if ((s = ng->off.reserve(4 * (n + 1))) != RG_OK || (s = ng->adj.reserve(4 * (m + 8))) != RG_OK ||
      (s = ng->new_ids.reserve(4 * n)) != RG_OK || (s = new_deg.reserve(4 * n)) != RG_OK) {
    delete ng;
    return s;
  }
  rank_to_ids<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(va, g->off.as<uint32_t>(), (uint32_t)n,
                                                          ng->new_ids.as<uint32_t>(), new_deg.as<uint32_t>());
  if ((s = scan_u32(ws, new_deg.as<uint32_t>(), ng->off.as<uint32_t>(), n, st)) != RG_OK) {
    delete ng;
    return s;
  }
  ng->directed = g->directed;
  if (g->directed) {  // in-lists: offsets from the ranks' in-degrees (new_deg is free again after the scan)
    if ((s = ng->in_off.reserve(4 * (n + 1))) != RG_OK || (s = ng->in_adj.reserve(4 * (m + 8))) != RG_OK) {
      delete ng;
      return s;
    }
    rank_in_deg<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(va, g->in_off.as<uint32_t>(), (uint32_t)n,
                                                            new_deg.as<uint32_t>());
    if ((s = scan_u32(ws, new_deg.as<uint32_t>(), ng->in_off.as<uint32_t>(), n, st)) != RG_OK) {
      delete ng;
      return s;
    }
  }
  if (m > 0) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g->device);
    const int64_t blocks = std::min<int64_t>((g->nchunks * 32 + 255) / 256, (int64_t)std::max(sms, 1) * 8);
    relabel_sweep<<<(unsigned)blocks, 256, 0, st>>>(g->view(), g->chunk_v.as<uint32_t>(), (uint32_t)g->nchunks,
                                                    ng->new_ids.as<uint32_t>(), ng->off.as<uint32_t>(),
                                                    ng->adj.as<uint32_t>(), bad.as<unsigned int>());
    if (g->directed) {
      relabel_sweep<<<(unsigned)blocks, 256, 0, st>>>(g->in_view(), g->in_chunks(), (uint32_t)g->nchunks,
                                                      ng->new_ids.as<uint32_t>(), ng->in_off.as<uint32_t>(),
                                                      ng->in_adj.as<uint32_t>(), bad.as<unsigned int>());
    }
  }
  cudaError_t e = cudaMemsetAsync(ng->adj.as<uint32_t>() + m, 0, 32, st);
  if (e == cudaSuccess && g->directed) e = cudaMemsetAsync(ng->in_adj.as<uint32_t>() + m, 0, 32, st);
  unsigned int h_bad = 0;
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h_bad, bad.p, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    delete ng;
    return cuda_fail(e, "degree sort", __FILE__, __LINE__);
  }
  if (h_bad) {
    delete ng;
    return fail(RG_EINVAL, "rg_graph_degree_sort: a neighbour id is >= n");
  }
  ng->sorted = true;
  ng->max_deg = g->max_deg;  // host arrays: on first full use (host_arrays)
  if (h_new_ids) {
    e = cudaMemcpy(h_new_ids, ng->new_ids.p, 4 * n, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) { delete ng; return cuda_fail(e, "new_ids download", __FILE__, __LINE__); }
  }
  if ((s = finish_graph(ng)) != RG_OK) { delete ng; return s; }
  *out = ng;
  return RG_OK;
}

extern "C" rg_status rg_graph_degree_sort(const rg_graph* g, rg_graph** out, uint32_t* h_new_ids) {
  return degree_sort_impl(g, false, out, h_new_ids);
}

extern "C" rg_status rg_graph_degree_sort_by(const rg_graph* g, int by_out_degree, rg_graph** out,
                                             uint32_t* h_new_ids) {
  return degree_sort_impl(g, by_out_degree != 0, out, h_new_ids);
}

// ---------------------------------------------------------------------------
// CSR construction on the device (the symmetric loader's clean-up, IO.h:429-474,
// for an edge list): both directions of every edge become directed entries
// (a, b); two stable radix sorts order them by (a, b); self loops and repeats
// are dropped; a scan compacts the survivors into the neighbour array, and
// each vertex's offset is the position of its first entry.  The result is
// bit-identical to rg_csr_from_edges.
// ---------------------------------------------------------------------------
namespace rg {

__global__ void csr_keep(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b, int64_t k,
                         uint32_t* __restrict__ keep) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < k; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t ai = a[i], bi = b[i];
    keep[i] = (ai != bi && (i == 0 || a[i - 1] != ai || b[i - 1] != bi)) ? 1u : 0u;
  }
}

__global__ void csr_compact(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b,
                            const uint32_t* __restrict__ keep, const uint32_t* __restrict__ pos, int64_t k,
                            uint32_t* __restrict__ a_out, uint32_t* __restrict__ adj) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < k; i += (int64_t)gridDim.x * blockDim.x) {
    if (keep[i]) {
      a_out[pos[i]] = a[i];
      adj[pos[i]] = b[i];
    }
  }
}

// off[v] = first position whose source is >= v, for v in [0, n]: position p
// (0 <= p <= m) fills the vertices between the previous source and its own.
__global__ void csr_offsets(const uint32_t* __restrict__ a, int64_t m, int64_t n, uint32_t* __restrict__ off) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p <= m; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t lo = p == 0 ? 0 : (int64_t)a[p - 1] + 1;
    const int64_t hi = p == m ? n : min((int64_t)a[p], n);  // ids are < n; never write past off[n]
    for (int64_t v = lo; v <= hi; v++) off[v] = (uint32_t)p;
  }
}

__global__ void max_value(const uint32_t* __restrict__ x, int64_t k, unsigned int* out) {
  unsigned int mx = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < k; i += (int64_t)gridDim.x * blockDim.x) {
    mx = max(mx, x[i]);
  }
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, mx);
}

__global__ void max_degree(const uint32_t* __restrict__ off, int64_t n, unsigned int* out) {
  unsigned int mx = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    mx = max(mx, off[v + 1] - off[v]);
  }
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, mx);
}

// Stable LSD radix sort of k (key, val) pairs on the `bits` low key bits;
// the result ends in (key, val) (the buffers are swapped as needed).
static rg_status radix_pairs(Workspace& ws, DevBuf& key, DevBuf& val, DevBuf& key2, DevBuf& val2, int64_t k, int bits,
                             DevBuf& hist, cudaStream_t st) {
  const int64_t nblocks = (k + kSortTile - 1) / kSortTile;
  RG_TRY(hist.reserve(4 * (256 * nblocks + 1)));
  uint32_t *ka = key.as<uint32_t>(), *va = val.as<uint32_t>(), *kb = key2.as<uint32_t>(), *vb = val2.as<uint32_t>();
  const int passes = (bits + 7) / 8;
  for (int p = 0; p < passes; p++) {
    sort_hist<<<(unsigned)nblocks, kSortThreads, 0, st>>>(ka, k, 8 * p, nblocks, hist.as<uint32_t>());
    RG_TRY(scan_u32(ws, hist.as<uint32_t>(), hist.as<uint32_t>(), 256 * nblocks, st));
    sort_scatter<<<(unsigned)nblocks, kSortThreads, 0, st>>>(ka, va, k, 8 * p, nblocks, hist.as<uint32_t>(), kb, vb);
    std::swap(ka, kb);
    std::swap(va, vb);
  }
  RG_CUDA(cudaGetLastError());
  if (passes % 2) {  // the sorted pairs are in the second buffers: swap ownership
    std::swap(key.p, key2.p);
    std::swap(key.bytes, key2.bytes);
    std::swap(val.p, val2.p);
    std::swap(val.bytes, val2.bytes);
  }
  return RG_OK;
}

}  // namespace rg

namespace rg {
rg_status build_in_lists(rg_graph* g, cudaStream_t st);
}

// Shared by the symmetric and directed builders.  Symmetric: entries
// (a, b) = [src, dst] x [dst, src]; directed: (src, dst) only, and the
// in-lists are built afterwards.
static rg_status create_from_edges(const char* who, int64_t n, int64_t num_edges, const uint32_t* src,
                                   const uint32_t* dst, int on_device, bool directed, rg_graph** out) {
  if (!out || n <= 0 || num_edges < 0 || (num_edges > 0 && (!src || !dst))) {
    return fail(RG_EINVAL, "%s: bad arguments", who);
  }
  const int64_t k = directed ? num_edges : 2 * num_edges;
  if (n >= 0xFFFFFFFFll || k >= 0xFFFFFFFFll) {
    return fail(RG_EUNSUPPORTED, "%s: >= 2^32 vertices or directed entries", who);
  }
  Ctx* c = nullptr;
  RG_TRY(get_ctx(&c));
  cudaStream_t st = c->stream;
  int sms = 0;
  RG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
  // temporaries from the pool
  DevBuf a{true, st}, b{true, st}, a2{true, st}, b2{true, st}, hist{true, st}, info{true, st};
  RG_TRY(a.reserve(4 * (size_t)k));
  RG_TRY(b.reserve(4 * (size_t)k));
  RG_TRY(a2.reserve(4 * (size_t)k));
  RG_TRY(b2.reserve(4 * (size_t)k));
  RG_TRY(info.reserve(8));
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (num_edges > 0) {
    RG_CUDA(cudaMemcpyAsync(a.as<uint32_t>(), src, 4 * num_edges, kind, st));
    RG_CUDA(cudaMemcpyAsync(b.as<uint32_t>(), dst, 4 * num_edges, kind, st));
    if (!directed) {
      RG_CUDA(cudaMemcpyAsync(a.as<uint32_t>() + num_edges, dst, 4 * num_edges, kind, st));
      RG_CUDA(cudaMemcpyAsync(b.as<uint32_t>() + num_edges, src, 4 * num_edges, kind, st));
    }
  }
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((k + 255) / 256, (int64_t)sms * 32));
  if (k > 0) {  // every id must be < n: the offsets below are indexed by them
    uint32_t mx_id = 0;
    RG_CUDA(cudaMemsetAsync(info.p, 0, 4, st));
    max_value<<<blocks, 256, 0, st>>>(a.as<uint32_t>(), k, info.as<unsigned int>());
    RG_CUDA(cudaGetLastError());
    RG_CUDA(cudaMemcpyAsync(&mx_id, info.p, 4, cudaMemcpyDeviceToHost, st));
    RG_CUDA(cudaStreamSynchronize(st));
    if (mx_id >= (uint64_t)n) return fail(RG_EINVAL, "edge endpoint %u >= n", mx_id);
  }
  int bits = 1;
  while (bits < 32 && ((uint64_t)(n - 1) >> bits) != 0) bits++;
  uint32_t* keep = a2.as<uint32_t>();
  uint32_t* src_c = b2.as<uint32_t>();  // compacted sources
  DevBuf scan{true, st};                 // exclusive scan of keep, k+1 entries
  int64_t m = 0;
  if (k > 0) {
    // by (a, b): stable sort on b, then on a
    RG_TRY(radix_pairs(c->ws, b, a, b2, a2, k, bits, hist, st));
    RG_TRY(radix_pairs(c->ws, a, b, a2, b2, k, bits, hist, st));
    keep = a2.as<uint32_t>();  // a2/b2 are free again after the sorts
    src_c = b2.as<uint32_t>();
    csr_keep<<<blocks, 256, 0, st>>>(a.as<uint32_t>(), b.as<uint32_t>(), k, keep);
    RG_CUDA(cudaGetLastError());
    RG_TRY(scan.reserve(4 * (size_t)(k + 1)));
    RG_TRY(scan_u32(c->ws, keep, scan.as<uint32_t>(), k, st));
    uint32_t m32 = 0;
    RG_CUDA(cudaMemcpyAsync(&m32, scan.as<uint32_t>() + k, 4, cudaMemcpyDeviceToHost, st));
    RG_CUDA(cudaStreamSynchronize(st));
    m = (int64_t)m32;
  }
  rg_graph* g = nullptr;
  RG_TRY(new_graph(&g));
  g->n = n;
  g->m = m;
  rg_status s;
  if ((s = g->off.reserve(4 * (n + 1))) != RG_OK || (s = g->adj.reserve(4 * (m + 8))) != RG_OK) {
    delete g;
    return s;
  }
  cudaError_t e = cudaSuccess;
  if (k > 0) {
    csr_compact<<<blocks, 256, 0, st>>>(a.as<uint32_t>(), b.as<uint32_t>(), keep, scan.as<uint32_t>(), k, src_c,
                                       g->adj.as<uint32_t>());
  }
  const int oblocks = (int)std::max<int64_t>(1, std::min<int64_t>((m + 1 + 255) / 256, (int64_t)sms * 32));
  csr_offsets<<<oblocks, 256, 0, st>>>(src_c, m, n, g->off.as<uint32_t>());
  e = cudaMemsetAsync(g->adj.as<uint32_t>() + m, 0, 32, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(info.p, 0, 4, st);
  if (e == cudaSuccess) {
    const int dblocks = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)sms * 16));
    max_degree<<<dblocks, 256, 0, st>>>(g->off.as<uint32_t>(), n, info.as<unsigned int>());
    e = cudaGetLastError();
  }
  uint32_t mx = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&mx, info.p, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    delete g;
    return cuda_fail(e, "device CSR build", __FILE__, __LINE__);
  }
  g->max_deg = mx;  // host degree array: on first full use (host_arrays)
  if ((s = finish_graph(g)) != RG_OK) { delete g; return s; }
  if (directed) {
    g->directed = true;
    s = build_in_lists(g, st);          // uses the out-list partition
    if (s == RG_OK) s = finish_graph(g);  // partitions of both lists
    if (s != RG_OK) {
      rg_graph_free(g);
      return s;
    }
  }
  *out = g;
  return RG_OK;
}

extern "C" rg_status rg_graph_create_from_edges(int64_t n, int64_t num_edges, const uint32_t* src, const uint32_t* dst,
                                                int on_device, rg_graph** out) {
  return create_from_edges("rg_graph_create_from_edges", n, num_edges, src, dst, on_device, false, out);
}

extern "C" rg_status rg_graph_create_directed_from_edges(int64_t n, int64_t num_edges, const uint32_t* src,
                                                         const uint32_t* dst, int on_device, rg_graph** out) {
  return create_from_edges("rg_graph_create_directed_from_edges", n, num_edges, src, dst, on_device, true, out);
}

// ---------------------------------------------------------------------------
// directed graphs: the in-lists (the reference's CSC, IO.h:287-345) built on
// the device.  The out-list entries are already ordered by source, so one
// stable radix sort by target leaves every in-list's sources ascending.
// ---------------------------------------------------------------------------
namespace rg {

__global__ void __launch_bounds__(256) expand_rows(DevGraph g, const uint32_t* __restrict__ chunk_v,
                                                   uint32_t nchunks, uint32_t* __restrict__ row) {
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t c = warp; c < nchunks; c += nwarps) {
    const uint32_t vlo = chunk_v[c], vhi = chunk_v[c + 1];
    for (int r = 0; r < kSweepChunk / 32; r++) {
      const uint32_t e = c * kSweepChunk + r * 32 + lane;
      if (e >= g.m) break;
      row[e] = upper_index(g.off, vlo, vhi, e);
    }
  }
}

rg_status build_in_lists(rg_graph* g, cudaStream_t st) {
  const int64_t n = g->n, m = g->m;
  RG_TRY(g->in_off.reserve(4 * (n + 1)));
  RG_TRY(g->in_adj.reserve(4 * (m + 8)));
  RG_CUDA(cudaMemsetAsync(g->in_adj.as<uint32_t>() + m, 0, 32, st));
  int sms = 0;
  RG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, g->device));
  if (m == 0) {
    RG_CUDA(cudaMemsetAsync(g->in_off.p, 0, 4 * (n + 1), st));
    return RG_OK;
  }
  DevBuf key{true, st}, val{true, st}, key2{true, st}, val2{true, st}, hist{true, st};
  RG_TRY(key.reserve(4 * (size_t)m));
  RG_TRY(val.reserve(4 * (size_t)m));
  RG_TRY(key2.reserve(4 * (size_t)m));
  RG_TRY(val2.reserve(4 * (size_t)m));
  RG_CUDA(cudaMemcpyAsync(key.p, g->adj.p, 4 * m, cudaMemcpyDeviceToDevice, st));
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>((g->nchunks * 32 + 255) / 256, (int64_t)sms * 8));
  expand_rows<<<(unsigned)blocks, 256, 0, st>>>(g->view(), g->chunk_v.as<uint32_t>(), (uint32_t)g->nchunks,
                                                val.as<uint32_t>());
  RG_CUDA(cudaGetLastError());
  int bits = 1;
  while (bits < 32 && ((uint64_t)(n - 1) >> bits) != 0) bits++;
  RG_TRY(radix_pairs(ctx().ws, key, val, key2, val2, m, bits, hist, st));
  RG_CUDA(cudaMemcpyAsync(g->in_adj.p, val.p, 4 * m, cudaMemcpyDeviceToDevice, st));
  const int oblocks = (int)std::max<int64_t>(1, std::min<int64_t>((m + 1 + 255) / 256, (int64_t)sms * 32));
  csr_offsets<<<oblocks, 256, 0, st>>>(key.as<uint32_t>(), m, n, g->in_off.as<uint32_t>());
  RG_CUDA(cudaGetLastError());
  RG_CUDA(cudaStreamSynchronize(st));
  return RG_OK;
}

}  // namespace rg

extern "C" rg_status rg_graph_create_directed(int64_t n, int64_t m, const uint32_t* h_off, const uint32_t* h_adj,
                                              rg_graph** out) {
  rg_graph* g = nullptr;
  RG_TRY(rg_graph_create(n, m, h_off, h_adj, &g));
  g->directed = true;
  g->host_ready = false;  // host in-degrees come with the in-lists (host_arrays)
  rg_status s = build_in_lists(g, ctx().stream);
  if (s == RG_OK) s = finish_graph(g);  // partitions of both lists
  if (s != RG_OK) {
    rg_graph_free(g);
    return s;
  }
  *out = g;
  return RG_OK;
}

extern "C" rg_status rg_graph_is_directed(const rg_graph* g, int* directed) {
  if (!g || !directed) return fail(RG_EINVAL, "null argument");
  *directed = g->directed ? 1 : 0;
  return RG_OK;
}

// ---------------------------------------------------------------------------
// readGraph + preprocessGraph in one call (symmetric graphs): only the
// offsets are uploaded; the ranking runs on them while nothing else waits,
// and the relabel reads the neighbour array straight from page-locked host
// memory over the host link, writing the relabelled array into HBM.  The
// unsorted neighbour array never lands on the device, which saves one full
// pass over it.  Host memory the device cannot read in place (pageable, or
// not 16-byte aligned) takes the copy-then-sort path.
// ---------------------------------------------------------------------------
namespace rg {

__global__ void check_offsets(const uint32_t* __restrict__ off, int64_t n, uint32_t m, unsigned int* bad) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v <= n; v += (int64_t)gridDim.x * blockDim.x) {
    const bool ok = (v == 0 ? off[0] == 0u : off[v - 1] <= off[v]) && (v < n || off[n] == m);
    if (!ok) atomicOr(bad, 1u);
  }
}

}  // namespace rg

extern "C" rg_status rg_graph_create_sorted(int64_t n, int64_t m, const uint32_t* h_off, const uint32_t* h_adj,
                                            rg_graph** out, uint32_t* h_new_ids) {
  if (!out || n <= 0 || m < 0 || !h_off || (m > 0 && !h_adj)) return fail(RG_EINVAL, "rg_graph_create_sorted: bad arguments");
  if (n >= 0xFFFFFFFFll || m >= 0xFFFFFFFFll) return fail(RG_EUNSUPPORTED, ">= 2^32 vertices or edges");
  Ctx* c = nullptr;
  RG_TRY(get_ctx(&c));
  cudaStream_t st = c->stream;
  const uint32_t* d_adj = nullptr;
  if (m > 0) {
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, h_adj) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer &&
        ((uintptr_t)pa.devicePointer & 15u) == 0) {
      d_adj = static_cast<const uint32_t*>(pa.devicePointer);
    }
    cudaGetLastError();  // an unregistered pointer is not an error here
  }
  if (m > 0 && !d_adj) {  // copy, then sort
    rg_graph* g0 = nullptr;
    RG_TRY(rg_graph_create(n, m, h_off, h_adj, &g0));
    const rg_status s = rg_graph_degree_sort(g0, out, h_new_ids);
    rg_graph_free(g0);
    return s;
  }
  rg_graph* g0 = nullptr;
  RG_TRY(new_graph(&g0));
  g0->n = n;
  g0->m = m;
  DevBuf info(true, st);
  rg_status s = g0->off.reserve(4 * (n + 1));
  if (s == RG_OK) s = info.reserve(16);
  unsigned int h_info[2] = {0, 0};
  if (s == RG_OK) {
    cudaError_t e = cudaMemcpyAsync(g0->off.p, h_off, 4 * (n + 1), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(info.p, 0, 8, st);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
    const int64_t blocks = std::min<int64_t>((n + 256) / 256, (int64_t)std::max(sms, 1) * 16);
    if (e == cudaSuccess) {
      check_offsets<<<(unsigned)blocks, 256, 0, st>>>(g0->off.as<uint32_t>(), n, (uint32_t)m, info.as<unsigned int>());
      max_degree<<<(unsigned)blocks, 256, 0, st>>>(g0->off.as<uint32_t>(), n, info.as<unsigned int>() + 1);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_info, info.p, 8, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) s = cuda_fail(e, "graph offsets", __FILE__, __LINE__);
  }
  if (s == RG_OK && h_info[0]) s = fail(RG_EINVAL, "rg_graph_create_sorted: offsets not monotone or not ending at m");
  if (s == RG_OK) {
    g0->max_deg = h_info[1];
    g0->adj.p = const_cast<uint32_t*>(d_adj);  // borrowed: released below without freeing
    s = finish_graph(g0);                       // the chunk partition of the old CSR
    if (s == RG_OK) s = degree_sort_impl(g0, false, out, h_new_ids);
  }
  g0->adj.p = nullptr;
  g0->adj.bytes = 0;
  delete g0;
  return s;
}
