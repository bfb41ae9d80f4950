// PageRank (PageRank.C:120-189) on the device, in the reference's double
// precision.
//
// Per iteration, like the reference:
//   contrib[s] = p[s] / deg(s)            the IEEE double quotient PR_F forms
//                                         per edge (PageRank.C:48), formed once
//                                         per vertex
//   acc[d]    += contrib[s] over edges     PR_F's additions
//   p'[v]      = 0.85 * acc[v] + 0.15/n    PR_Vertex_F (fused multiply-add, as
//                                         the reference compiles it with FMA)
//   L1         = sum |p[v] - p'[v]|        PageRank.C:168-170, break at < 1e-7
// The edge pass differs from the reference only in how it adds.  The pull
// (every schedule the autotuner picks on large graphs, and the push-pull
// variant) forms each acc[d] EXACTLY, as a 128-bit fixed-point sum of the
// doubles (pr_exact.cuh), rounded to the nearest double once: the ranks are
// the correctly rounded sums of the reference's own terms, the same in every
// run.  The push (the reference's dense_forward schedule) adds with FP64
// atomics in arbitrary order, as the reference's CAS loop (utils.h:334-339)
// does; its per-CTA hub copies sum exactly and merge with one FP64 add.
// The L1 sum is exact too.  The L1 < 1e-7 break is taken on the device:
// every kernel of iteration i returns at once if iteration i-1 converged, so
// a whole run is enqueued without host round trips.

#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <utility>
#include <vector>

#include "app_common.cuh"
#include "pr_exact.cuh"

namespace rg {

namespace {

constexpr int kSweepThreads = 1024;  // push sweep CTA (one per SM with hub copies)
constexpr int kPullThreads = 256;
constexpr double kDamp = 0.85;       // PageRank.C:126
constexpr uint32_t kNoRow = 0xFFFFFFFFu;

// L1 of the previous iteration (exact) below 1e-7: this iteration is skipped.
__device__ __forceinline__ bool converged(const U128* l1_prev) {
  return l1_prev != nullptr && less128(*l1_prev, pr_eps_fx());
}

// acc[v] += x for a 128-bit sum shared with other warps: the low word's
// atomic returns the old value, so the carry out of it is known and goes into
// the high word.  Every carry is counted once, so the final sum is exact.
__device__ __forceinline__ void atomic_add128(U128* p, const U128& x) {
  const unsigned long long old = atomicAdd(&p->lo, x.lo);
  const unsigned long long hi = x.hi + (old + x.lo < old ? 1ull : 0ull);
  if (hi) atomicAdd(&p->hi, hi);
}

__device__ __forceinline__ void store128(U128* p, const U128& x) {
  asm volatile("st.global.v2.u64 [%0], {%1, %2};" ::"l"(p), "l"(x.lo), "l"(x.hi) : "memory");
}

__device__ __forceinline__ U128 shfl_up128(const U128& x, int o) {
  return U128{__shfl_up_sync(0xffffffffu, x.lo, o), __shfl_up_sync(0xffffffffu, x.hi, o)};
}

__device__ __forceinline__ U128 block_sum128(U128 v) {
  __shared__ U128 ws[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    add128(v, U128{__shfl_xor_sync(0xffffffffu, v.lo, o), __shfl_xor_sync(0xffffffffu, v.hi, o)});
  }
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
  __syncthreads();
  U128 t{0ull, 0ull};
  if (threadIdx.x < 32) {
    if (threadIdx.x < (blockDim.x >> 5)) t = ws[threadIdx.x];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      add128(t, U128{__shfl_xor_sync(0xffffffffu, t.lo, o), __shfl_xor_sync(0xffffffffu, t.hi, o)});
    }
  }
  return t;  // valid in thread 0
}

// p'/deg, the IEEE quotient of PR_F (PageRank.C:48), by degree class (the
// deg_quotient classes): the integer reciprocal is read only for degrees
// that need it, and degree-sorted graphs keep whole warps in one class.
__device__ __forceinline__ double pr_quotient(double pn, uint32_t d, const unsigned long long* __restrict__ rmag,
                                              int64_t v) {
  if (d == 0) return 0.0;
  if ((d & (d - 1)) == 0) return double_of(bits_of(pn) - ((unsigned long long)(31 - __clz(d)) << 52));
  return div_by_magic(pn, d, rmag[v]);
}

// p = 1/n, contrib = p/deg (PageRank.C:126-138), rmag = the integer
// reciprocal of each degree that is neither 0, 1 nor a power of two (for the
// later iterations' quotients); the accumulators start at 0.
__global__ void pr_init(uint32_t n, const uint32_t* __restrict__ off, double* p, double* contrib,
                        unsigned long long* rmag, double p0) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    p[v] = p0;
    const uint32_t d = off[v + 1] - off[v];
    const unsigned long long R = (d & (d - 1)) ? recip_magic(d) : 0ull;
    contrib[v] = deg_quotient(p0, d, R);
    rmag[v] = R;
  }
}

// Dense push over every edge (edgeMapDenseForward with a full frontier):
// acc[d] += contrib[s] with FP64 atomics, as the reference's CAS loop.  Each
// warp owns kSweepChunk consecutive edges read as 16-byte vectors; chunk_v
// gives the chunk's first source so a lane finds its source with a short
// search.  Hub copies (RADAR: ids < H; HUBDUP: bitmap + index map) are
// per-CTA shared-memory 128-bit exact sums, merged once per CTA with one FP64
// add each.
template <int kHub>
__global__ void __launch_bounds__(kSweepThreads) pr_push_sweep(DevGraph g, const uint32_t* __restrict__ chunk_v,
                                                               uint32_t nchunks, const double* __restrict__ contrib,
                                                               double* acc, HubInfo hub, const U128* l1_prev) {
  if (converged(l1_prev)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  U128* hs = reinterpret_cast<U128*>(smem_raw);
  if (kHub != kHubNone) {
    for (uint32_t h = threadIdx.x; h < hub.H; h += blockDim.x) hs[h] = U128{0ull, 0ull};
    __syncthreads();
  }
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t c = warp; c < nchunks; c += nwarps) {
    const uint32_t vlo = chunk_v[c], vhi = chunk_v[c + 1];
#pragma unroll
    for (int r = 0; r < kSweepChunk / 128; r++) {
      const uint32_t e = c * kSweepChunk + r * 128 + lane * 4;
      if (e >= g.m) continue;
      const uint4 d4 = __ldg(reinterpret_cast<const uint4*>(g.adj + e));
      uint32_t s = upper_index(g.off, vlo, vhi, e);
      uint32_t nxt = g.off[s + 1];
      double cs = contrib[s];
      const uint32_t dd[4] = {d4.x, d4.y, d4.z, d4.w};
#pragma unroll
      for (int i = 0; i < 4; i++) {
        const uint32_t ee = e + i;
        if (ee >= g.m) break;
        if (ee >= nxt) {
          do { s++; nxt = g.off[s + 1]; } while (ee >= nxt);
          cs = contrib[s];
        }
        const uint32_t d = dd[i];
        uint32_t slot;
        if (kHub != kHubNone && hub_slot<kHub>(hub, d, slot)) {
          const U128 x = fx_from_double(cs);
          const unsigned long long old = atomicAdd(&hs[slot].lo, x.lo);
          const unsigned long long hi = x.hi + (old + x.lo < old ? 1ull : 0ull);
          if (hi) atomicAdd(&hs[slot].hi, hi);
        } else {
          atomicAdd(acc + d, cs);
        }
      }
    }
  }
  if (kHub != kHubNone) {
    __syncthreads();
    for (uint32_t h = threadIdx.x; h < hub.H; h += blockDim.x) {
      const U128 x = hs[h];
      if (x.lo | x.hi) atomicAdd(acc + hub_vertex<kHub>(hub, h), fx_to_double(x));
    }
  }
}

// Dense pull over every vertex (edgeMapDense with a full frontier, the
// push-pull variant): acc[v] = the exact sum of contrib[u] over in-neighbours
// u.  Edge-balanced like the push sweep: each lane takes kItems consecutive
// edges of a warp step (one 16- or 32-byte load of the edge array) and
// gathers their contributions.  A row that starts and ends inside one lane
// is stored by that lane.  The first row of a lane may have started in an
// earlier lane and its last row may continue in a later one: those pieces
// are combined across the warp by a segmented scan (rows are non-decreasing
// across lanes); a row that starts and ends inside the warp step is then
// stored once, and only rows that cross a warp step's edge (at most two per
// step) are added with 128-bit atomics into the zeroed accumulator.
// The sweep is bound by the gathers' L2 requests, so kMode can stream the
// edge array past the caches (1) and also keep gathered lines in L1/L2 (2).
// kCache (degree-sorted graphs): the contributions of the H hubs (ids < H)
// are copied into shared memory once per CTA -- RADAR's duplication of hub
// data, used here for the reads of a pull instead of the writes of a push.
template <bool kCache, int kItems, int kMode>
__global__ void __launch_bounds__(kCache ? 1024 : kPullThreads)
    pr_pull_sweep(DevGraph g, const uint32_t* __restrict__ chunk_v, uint32_t nchunks,
                  const double* __restrict__ contrib, U128* acc, uint32_t H, const U128* l1_prev) {
  static_assert(kItems == 4 || kItems == 8 || kItems == 16, "4, 8 or 16 edges per lane");
  if (converged(l1_prev)) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double* hc = reinterpret_cast<double*>(smem_raw);
  if (kCache) {
    for (uint32_t h = threadIdx.x; h < H; h += blockDim.x) hc[h] = contrib[h];
    __syncthreads();
  }
  constexpr int kStep = 32 * kItems;  // edges per warp step
  const uint64_t first = kMode >= 1 ? policy_evict_first() : 0;
  const uint64_t keep = kMode == 2 ? policy_evict_last() : 0;
  const uint64_t* contrib_bits = reinterpret_cast<const uint64_t*>(contrib);
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t c = warp; c < nchunks; c += nwarps) {
    const uint32_t vlo = chunk_v[c], vhi = chunk_v[c + 1];
#pragma unroll
    for (int r = 0; r < kSweepChunk / kStep; r++) {
      const uint32_t s0 = c * kSweepChunk + r * kStep;  // this warp step's first edge
      const uint32_t e = s0 + lane * kItems;
      uint32_t row = kNoRow, head_row = kNoRow;
      U128 part{0ull, 0ull}, head{0ull, 0ull};
      bool cont = false;      // the lane's last row continues past the lane
      if (e < g.m) {
        // the lane's neighbour ids, all loaded up front: with 16 edges per
        // lane the second 32 bytes come from the L2 line the first just
        // brought in (loaded only when the second batch starts, the streamed,
        // evict-first line was often gone: RMAT s24 read 3.53 instead of 2.79
        // GB per sweep).  In bounds: adj is padded by 8 entries and 32-byte
        // aligned, and a group past the first is read only when it starts
        // before m.
        uint32_t uu[kItems];
        if (kItems >= 8 && kMode >= 1) {
#pragma unroll
          for (int h = 0; h < kItems / 8; h++) {
            const U32x8 w = (h == 0 || e + 8 * h < g.m) ? ld_stream_v8(g.adj + e + 8 * h) : U32x8{};
#pragma unroll
            for (int i = 0; i < 8; i++) uu[8 * h + i] = w.v[i];
          }
        } else {
#pragma unroll
          for (int h = 0; h < kItems / 4; h++) {
            uint4 w = make_uint4(0u, 0u, 0u, 0u);
            if (h < 2 || e + 4 * h < g.m) {
              w = kMode >= 1 ? ld_stream_v4(g.adj + e + 4 * h, first)
                             : __ldg(reinterpret_cast<const uint4*>(g.adj + e + 4 * h));
            }
            uu[4 * h] = w.x;
            uu[4 * h + 1] = w.y;
            uu[4 * h + 2] = w.z;
            uu[4 * h + 3] = w.w;
          }
        }
        uint32_t v = upper_index(g.off, vlo, vhi, e);
        uint32_t nxt = g.off[v + 1];
        const bool first_started_before = g.off[v] < e;
        row = v;
        bool at_first = true;
        // the gathers in batches of at most 8 per lane (16 edges per lane
        // halve the warp scans per edge without 16 values in flight at once)
        constexpr int kBatch = kItems > 8 ? 8 : kItems;
#pragma unroll
        for (int b = 0; b < kItems; b += kBatch) {
          if (e + b >= g.m) break;
          double x[kBatch];
#pragma unroll
          for (int j = 0; j < kBatch; j++) {
            const uint32_t u = uu[b + j];
            x[j] = (e + b + j < g.m) ? ((kCache && u < H) ? hc[u]
                                        : kMode == 2 ? __longlong_as_double((long long)ld_keep_u64(contrib_bits + u, keep))
                                                     : __ldg(contrib + u))
                                     : 0.0;
          }

#pragma unroll
          for (int j = 0; j < kBatch; j++) {
            const uint32_t ee = e + b + j;
            if (ee >= g.m) break;
            if (ee >= nxt) {
              // row `row` ends inside this lane: it is the lane's head piece
              // if it began in an earlier lane, else complete and stored here
              if (at_first && first_started_before) {
                head = part;
                head_row = row;
              } else {
                store128(acc + row, part);
              }
              at_first = false;
              part = U128{0ull, 0ull};
              do { v++; nxt = g.off[v + 1]; } while (ee >= nxt);
              row = v;
            }
            add128(part, fx_from_double(x[j]));
          }
        }
        cont = nxt > e + kItems;
      }
      // segmented inclusive scan of the lanes' last-row pieces
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const U128 t = shfl_up128(part, o);
        const uint32_t tr = __shfl_up_sync(0xffffffffu, row, o);
        if (lane >= o && tr == row) add128(part, t);
      }
      const uint32_t step_end = min(s0 + (uint32_t)kStep, g.m);
      // a head piece completes the row the previous lanes' pieces began
      const U128 prev = shfl_up128(part, 1);
      const uint32_t prev_row = __shfl_up_sync(0xffffffffu, row, 1);
      if (head_row != kNoRow) {
        if (lane > 0 && prev_row == head_row) add128(head, prev);
        if (g.off[head_row] >= s0) store128(acc + head_row, head);  // began inside this step
        else atomic_add128(acc + head_row, head);
      }
      // the last-row piece ends its segment where the row ends inside this
      // lane, or at the end of the step
      if (row != kNoRow && (!cont || lane == 31)) {
        if (!cont && g.off[row] >= s0 && g.off[row + 1] <= step_end) store128(acc + row, part);
        else atomic_add128(acc + row, part);
      }
    }
  }
}

using PullFn = void (*)(DevGraph, const uint32_t*, uint32_t, const double*, U128*, uint32_t, const U128*);

// The sweeps are picked at run time among their template instances: their
// dynamic shared memory limit is raised to the device maximum once per
// (kernel, device), under a lock (the per-instance form of
// allow_max_dyn_smem).
template <class K>
rg_status allow_pr_dyn_smem(K kern) {
  static std::mutex mu;
  static std::vector<std::pair<const void*, uint64_t>> done;  // kernel, device bits
  int dev = 0;
  RG_CUDA(cudaGetDevice(&dev));
  const uint64_t bit = 1ull << (dev & 63);
  const void* key = reinterpret_cast<const void*>(kern);
  std::lock_guard<std::mutex> lk(mu);
  auto it = std::find_if(done.begin(), done.end(), [&](const std::pair<const void*, uint64_t>& d) {
    return d.first == key;
  });
  if (it != done.end() && (it->second & bit)) return RG_OK;
  cudaFuncAttributes fa;
  RG_CUDA(cudaFuncGetAttributes(&fa, kern));
  RG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               max_dyn_smem() - (int)fa.sharedSizeBytes));
  if (it == done.end()) done.emplace_back(key, bit);
  else it->second |= bit;
  return RG_OK;
}


template <bool kCache>
PullFn pull_variant(int64_t shape) {
  switch (shape) {
    case 41: return pr_pull_sweep<kCache, 4, 1>;
    case 42: return pr_pull_sweep<kCache, 4, 2>;
    case 80: return pr_pull_sweep<kCache, 8, 0>;
    case 81: return pr_pull_sweep<kCache, 8, 1>;
    case 82: return pr_pull_sweep<kCache, 8, 2>;
    case 160: return pr_pull_sweep<kCache, 16, 0>;
    case 161: return pr_pull_sweep<kCache, 16, 1>;
    case 162: return pr_pull_sweep<kCache, 16, 2>;
    default: return pr_pull_sweep<kCache, 4, 0>;
  }
}

// vertexMap(PR_Vertex_F) + the L1 step + the reset, fused:
//   p' = fma(0.85, sum, 0.15/n);  L1 += |p - p'| (exact);  p = p';
//   acc = 0 where the next sweep adds instead of storing;  contrib = p'/deg.
// kExact: acc holds the pull's exact 128-bit sums; the pull stores every
// row that lies inside one warp step of `step` edges (pull_off: the rows it
// reads) and adds with atomics only into rows that cross a step, so only
// those are zeroed.  Else acc holds the push's FP64 sums, all zeroed.
template <bool kExact>
__global__ void __launch_bounds__(256) pr_finalize(uint32_t n, const uint32_t* __restrict__ off,
                                                   const uint32_t* __restrict__ pull_off, uint32_t step, U128* acc,
                                                   double* p, double* contrib,
                                                   const unsigned long long* __restrict__ rmag, double added,
                                                   U128* l1_out, const U128* l1_prev) {
  if (converged(l1_prev)) return;
  U128 local{0ull, 0ull};
  double* accd = reinterpret_cast<double*>(acc);
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    // the tests of zero and equality are integer compares (the FP64 pipe is
    // the scarce one): every value here is a nonnegative double, not NaN
    double sum;
    bool has;
    if (kExact) {
      const U128 a = acc[v];
      has = (a.lo | a.hi) != 0ull;
      sum = has ? fx_to_double(a) : 0.0;
      const uint32_t b = pull_off[v], e = pull_off[v + 1];
      if (e > b && b / step != (e - 1) / step) acc[v] = U128{0ull, 0ull};
    } else {
      sum = accd[v];
      has = (bits_of(sum) << 1) != 0ull;
      accd[v] = 0.0;
    }
    // fma(0.85, 0, added) is `added` exactly: vertices without in-edges skip it
    const double pn = has ? fma(kDamp, sum, added) : added;
    const double po = p[v];
    if (bits_of(po) != bits_of(pn)) add128(local, fx_from_double(fabs(po - pn)));
    p[v] = pn;
    contrib[v] = pr_quotient(pn, off[v + 1] - off[v], rmag, v);  // = pn / deg, correctly rounded
  }
  const U128 t = block_sum128(local);
  if (threadIdx.x == 0 && (t.lo | t.hi)) atomic_add128(l1_out, t);
}

// Ranks in original-id order when the graph is degree-sorted.
__global__ void pr_gather(const double* __restrict__ p, const uint32_t* __restrict__ new_ids, int64_t n,
                          double* __restrict__ out) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    out[v] = p[new_ids ? new_ids[v] : v];
  }
}

struct PrState {
  DevBuf acc, p, contrib, rmag, l1, out;
};

}  // namespace

rg_status pagerank_run(rg_graph* g, int variant, int64_t max_iters, double* h_ranks, int64_t* iters_out,
                       double* l1_out, uint32_t hub_h) {
  if (!g) return fail(RG_EINVAL, "null graph");
  if (variant < 0 || variant > 4) return fail(RG_EINVAL, "bad variant %d", variant);
  if (max_iters < 0) return fail(RG_EINVAL, "max_iters < 0");
  OptScope opt_scope(g, kAppPagerank);
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  cudaStream_t st = cx->stream;
  const int64_t n = g->n;
  static thread_local PrState S;
  RG_TRY(S.acc.reserve(sizeof(U128) * n));
  RG_TRY(S.p.reserve(8 * n));
  RG_TRY(S.contrib.reserve(8 * n));
  RG_TRY(S.rmag.reserve(8 * n));
  RG_TRY(S.l1.reserve(sizeof(U128) * (max_iters + 1)));
  RG_TRY(S.out.reserve(8 * n));
  // the reference's constants (PageRank.C:126-138)
  const double p0 = 1 / (double)n;
  const double added = (1 - kDamp) * (1 / (double)n);
  // hub set-up (host side, before the timed span).  The full sweeps run one
  // CTA per SM, so their hub copies may use the whole shared memory.
  // hub copies only with a shared-memory budget; the push kernel's hub mode is
  // the one actually set up (a HUBDUP map kernel needs the map's arrays)
  const int hm = g_opts.hub_smem_kb > 0 ? hub_mode_of(variant) : kHubNone;
  uint32_t pr_budget = (uint32_t)std::min<int64_t>((max_dyn_smem() - 1024) / (int)sizeof(U128), n);
  if (g_opts.hub_slots > 0) pr_budget = (uint32_t)std::min<int64_t>(pr_budget, g_opts.hub_slots);
  if (hub_h) pr_budget = std::min(pr_budget, hub_h);
  // pull: the push-pull variant (threshold 0, PageRank.C:122 in src/push-pull)
  // or the auto direction; RADAR's pull keeps the hubs' contributions in
  // shared memory, the others gather from global memory
  const bool pull = variant == RG_PUSH_PULL || g_opts.direction == 1;
  const bool cache = pull && variant == RG_RADAR && g->sorted && g_opts.hub_smem_kb > 0;
  HubInfo hub;
  size_t dyn = 0;
  if (!pull && hm != kHubNone) {
    if (hm == kHubPrefix) hub.H = pr_budget;
    else RG_TRY(hub_map(g, pr_budget, hub));
    dyn = sizeof(U128) * hub.H;
  }
  // the pull's hub cache holds hub_smem_kb KiB of contributions per CTA
  const uint32_t cacheH =
      cache ? (uint32_t)std::min<int64_t>({n, g_opts.hub_smem_kb * 1024 / (int64_t)sizeof(double),
                                           (max_dyn_smem() - 1024) / (int64_t)sizeof(double),
                                           g_opts.hub_slots > 0 ? g_opts.hub_slots : n, hub_h ? (int64_t)hub_h : n})
            : 0;
  const int push_hm = pull ? kHubNone : hm;
  auto sweep_fn = push_hm == kHubPrefix ? pr_push_sweep<kHubPrefix>
                  : push_hm == kHubMap  ? pr_push_sweep<kHubMap>
                                        : pr_push_sweep<kHubNone>;
  PullFn pull_fn = cache ? pull_variant<true>(g_opts.sweep_shape) : pull_variant<false>(g_opts.sweep_shape);
  // edges per warp step of the chosen pull (32 lanes x 4 or 8 edges, pull_variant's shapes)
  const uint32_t pull_step = 32u * (uint32_t)(g_opts.sweep_shape / 10);
  const int pull_threads = cache ? 1024 : kPullThreads;
  const size_t pull_dyn = sizeof(double) * cacheH;
  const int sms = device_sms();
  int sweep_grid = 1, per_sm = 0;
  // L1 caches the gathered contributions that shared memory does not: the
  // carve-out gives shared memory only what the resident CTAs need
  int smem_per_sm = 0;
  RG_CUDA(cudaDeviceGetAttribute(&smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, g->device));
  auto carveout = [&](size_t per_cta, int ctas) {
    const size_t need = (per_cta + 1024) * (size_t)ctas;
    return (int)std::min<size_t>(100, (need * 100 + (size_t)smem_per_sm - 1) / (size_t)std::max(smem_per_sm, 1));
  };
  if (pull) {
    if (pull_dyn) RG_TRY(allow_pr_dyn_smem(pull_fn));
    RG_CUDA(cudaFuncSetAttribute(pull_fn, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 cache ? carveout(pull_dyn, std::max(1, 2048 / pull_threads)) : 0));
    RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, pull_fn, pull_threads, pull_dyn));
    sweep_grid = (int)std::min<int64_t>((int64_t)sms * std::max(per_sm, 1),
                                        std::max<int64_t>((g->nchunks * 32 + pull_threads - 1) / pull_threads, 1));
  } else {
    if (dyn) RG_TRY(allow_pr_dyn_smem(sweep_fn));
    RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sweep_fn, kSweepThreads, dyn));
    sweep_grid = (int)std::min<int64_t>((int64_t)sms * std::max(per_sm, 1),
                                        std::max<int64_t>((g->nchunks * 32 + kSweepThreads - 1) / kSweepThreads, 1));
  }
  const int vblocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)sms * 16);

  CallTimer timer(g);
  U128* A = S.acc.as<U128>();
  double* P = S.p.as<double>();
  double* C = S.contrib.as<double>();
  unsigned long long* R = S.rmag.as<unsigned long long>();
  U128* L1 = S.l1.as<U128>();
  // The whole run (init + every iteration) is enqueued without host round
  // trips; it is captured once as a CUDA graph and replayed on later calls
  // with the same graph, buffers and schedule (not while per-kernel timing
  // is on, which needs the launches one by one).
  int64_t launches = 0, edge_launches = 0;
  auto enqueue = [&]() -> cudaError_t {
    cudaError_t e = cudaMemsetAsync(L1, 0, sizeof(U128) * (max_iters + 1), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(A, 0, sizeof(U128) * n, st);
    if (e != cudaSuccess) return e;
    pr_init<<<vblocks, 256, 0, st>>>((uint32_t)n, g->off.as<uint32_t>(), P, C, R, p0);
    launches++;
    // iteration i's kernels return at once when iteration i-1 already
    // reached L1 < 1e-7
    for (int64_t it = 0; it < max_iters; it++) {
      const U128* prev = it ? L1 + it - 1 : nullptr;
      if (g->m > 0) {
        kt_begin(st);
        if (pull) {
          pull_fn<<<sweep_grid, pull_threads, pull_dyn, st>>>(g->in_view(), g->in_chunks(), (uint32_t)g->nchunks, C,
                                                              A, cacheH, prev);
        } else {
          sweep_fn<<<sweep_grid, kSweepThreads, dyn, st>>>(g->view(), g->chunk_v.as<uint32_t>(),
                                                           (uint32_t)g->nchunks, C, reinterpret_cast<double*>(A), hub,
                                                           prev);
        }
        kt_end(st);
        launches++;
        edge_launches++;
      }
      if (pull) {
        pr_finalize<true><<<vblocks, 256, 0, st>>>((uint32_t)n, g->off.as<uint32_t>(), g->in_view().off, pull_step,
                                                   A, P, C, R, added, L1 + it, prev);
      } else {
        pr_finalize<false><<<vblocks, 256, 0, st>>>((uint32_t)n, g->off.as<uint32_t>(), g->off.as<uint32_t>(), 1u,
                                                    A, P, C, R, added, L1 + it, prev);
      }
      launches++;
    }
    return cudaGetLastError();
  };
  // the captured launches bake in every pointer below; the graph's uid keeps
  // a new graph whose buffers reuse a freed graph's addresses from matching
  struct GraphKey {
    uint64_t uid;
    const void *off, *adj, *chunk_v, *hub_bits, *hub_slot, *hub_vertex, *a, *p, *c, *r, *l1;
    int64_t n, m, iters;
    int variant, grid, pull, cacheH, hubH, hubmode, shape;
    bool operator==(const GraphKey& o) const { return memcmp(this, &o, sizeof *this) == 0; }
  };
  static thread_local GraphKey cached_key;
  static thread_local cudaGraphExec_t cached_exec = nullptr;
  static thread_local int64_t cached_launches = 0, cached_edge_launches = 0;
  GraphKey key;
  memset(&key, 0, sizeof key);  // memcmp compares the padding too: set fields one by one
  key.uid = g->uid;
  key.off = g->off.p;
  key.adj = g->adj.p;
  key.chunk_v = g->chunk_v.p;
  key.hub_bits = hub.bits;
  key.hub_slot = hub.slot;
  key.hub_vertex = hub.vertex;
  key.a = A;
  key.p = P;
  key.c = C;
  key.r = R;
  key.l1 = L1;
  key.n = n;
  key.m = g->m;
  key.iters = max_iters;
  key.variant = variant;
  key.grid = sweep_grid;
  key.pull = pull ? 1 : 0;
  key.cacheH = (int)cacheH;
  key.hubH = (int)hub.H;
  key.hubmode = push_hm;
  key.shape = (int)g_opts.sweep_shape;
  if (g_kernel_timing || max_iters == 0) {
    RG_CUDA(enqueue());
  } else {
    if (!cached_exec || !(key == cached_key)) {
      if (cached_exec) cudaGraphExecDestroy(cached_exec);
      cached_exec = nullptr;
      cudaGraph_t graph = nullptr;
      RG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      const cudaError_t e = enqueue();
      const cudaError_t e2 = cudaStreamEndCapture(st, &graph);
      if (e != cudaSuccess || e2 != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return cuda_fail(e != cudaSuccess ? e : e2, "PageRank graph capture", __FILE__, __LINE__);
      }
      const cudaError_t e3 = cudaGraphInstantiate(&cached_exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e3 != cudaSuccess) {
        cached_exec = nullptr;
        return cuda_fail(e3, "cudaGraphInstantiate", __FILE__, __LINE__);
      }
      cached_key = key;
      cached_launches = launches;
      cached_edge_launches = edge_launches;
    }
    RG_CUDA(cudaGraphLaunch(cached_exec, st));
    launches = cached_launches;
    edge_launches = cached_edge_launches;
  }
  g_timing.kernel_launches += launches;
  g_timing.edge_launches += edge_launches;
  RG_TRY(timer.stop());  // device work done; result copies are outside the timed span
  std::vector<U128> l1h(max_iters + 1, U128{0ull, 0ull});
  RG_TRY(read_small(L1, l1h.data(), sizeof(U128) * (max_iters + 1), st));
  int64_t done = max_iters;
  bool broke = false;
  const U128 eps = pr_eps_fx();
  for (int64_t it = 0; it < max_iters; it++) {
    if (less128(l1h[it], eps)) { done = it; broke = true; break; }
  }
  const int64_t last = broke ? done : max_iters - 1;
  if (h_ranks && g_opts.async_results) {
    RG_TRY(download_async<double>(h_ranks, n, st, [&](double* stage) -> rg_status {
      if (g->sorted) {
        pr_gather<<<vblocks, 256, 0, st>>>(P, g->new_ids.as<uint32_t>(), n, stage);
        RG_CUDA(cudaGetLastError());
      } else {
        RG_CUDA(cudaMemcpyAsync(stage, P, 8 * n, cudaMemcpyDeviceToDevice, st));
      }
      return RG_OK;
    }));
  } else if (h_ranks) {
    // P holds the last computed ranks (p_next after a break, p_curr after
    // the final reset and swap of a run that used every iteration)
    if (g->sorted) {
      pr_gather<<<vblocks, 256, 0, st>>>(P, g->new_ids.as<uint32_t>(), n, S.out.as<double>());
      RG_CUDA(cudaGetLastError());
      RG_CUDA(cudaMemcpyAsync(h_ranks, S.out.p, 8 * n, cudaMemcpyDeviceToHost, st));
    } else {
      RG_CUDA(cudaMemcpyAsync(h_ranks, P, 8 * n, cudaMemcpyDeviceToHost, st));
    }
    RG_CUDA(cudaStreamSynchronize(st));
  }
  const int64_t iters_run = broke ? done + 1 : max_iters;
  g_timing.edges_traversed = g->m * iters_run;
  g_timing.algorithmic_bytes = (4 * g->m + 4 * (n + 1) + 16 * n) * iters_run;
  if (iters_out) *iters_out = broke ? done + 1 : max_iters + 1;
  if (l1_out) *l1_out = max_iters ? fx_to_double(l1h[last]) : 0.0;
  return RG_OK;
}

}  // namespace rg

extern "C" rg_status rg_pagerank(rg_graph* g, rg_variant variant, int64_t max_iters, double* h_ranks,
                                 int64_t* iters_out, double* l1_out) {
  return rg::pagerank_run(g, variant, max_iters, h_ranks, iters_out, l1_out, 0);
}
