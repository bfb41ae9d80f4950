// Batched execution: many BFS sources per launch (64-wide bitmask frontiers)
// and many graphs per launch (a persistent kernel).
//
// Multi-source BFS keeps per vertex a 64-bit `seen` mask and a 64-bit
// frontier mask F: bit q of F[v] says v was reached from source q in the
// previous level.  A level ORs F[u] & ~seen[v] into N[v] over the edges --
// the same mask propagation as Radii_F (Radii.C:37-106), one bit per source --
// and every bit that arrives at v for the first time gives depth(q, v).  Each
// row q of the result equals a single-source BFS from source q (BFS.C), so
// up to 64 BFS queries cost one traversal.
//
// The persistent batch kernel runs, for every graph of a set, a 64-source BFS
// and a PageRank (the exact-sum arithmetic of pagerank.cu), each task owned by one
// CTA from start to finish: CTAs take tasks from an atomic counter (largest
// graphs first) and synchronise only with __syncthreads, never with each
// other, so no CTA ever waits on another.

#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "app_common.cuh"
#include "pr_exact.cuh"

namespace rg {

// ---------------------------------------------------------------------------
// multi-source BFS on one resident graph
// ---------------------------------------------------------------------------
namespace {

__global__ void ms_clear_frontier(const uint32_t* __restrict__ q, int64_t k, unsigned long long* F) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < k) F[q[j]] = 0ull;
}

// New frontier: the bits that arrived this level become F, join seen, and
// give depth(q, v) = level for every source bit q.
__global__ void ms_advance(const uint32_t* __restrict__ q, int64_t k, unsigned long long* N, unsigned long long* F,
                           unsigned long long* seen, int32_t* depth, int64_t n, int32_t level) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  const uint32_t v = q[j];
  const unsigned long long w = N[v] & ~seen[v];
  N[v] = 0ull;
  F[v] = w;
  seen[v] |= w;
  unsigned long long x = w;
  while (x) {
    const int b = __ffsll((long long)x) - 1;
    x &= x - 1;
    depth[(int64_t)b * n + v] = level;
  }
}

__global__ void ms_seed(const uint32_t* __restrict__ src, int k, int64_t n, unsigned long long* F,
                        unsigned long long* seen, int32_t* depth) {
  const int q = threadIdx.x;
  if (q < k) {
    const uint32_t s = src[q];
    atomicOr(F + s, 1ull << q);
    atomicOr(seen + s, 1ull << q);
    depth[(int64_t)q * n + s] = 0;
  }
}

// out[q*n + v] = in[q*n + new_ids[v]] (rows in original-id order)
__global__ void ms_gather(const int32_t* __restrict__ in, const uint32_t* __restrict__ new_ids, int64_t n, int k,
                          int32_t* __restrict__ out) {
  const int64_t total = n * k;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = i / n, v = i - q * n;
    out[i] = in[q * n + new_ids[v]];
  }
}

// Per-thread state sized by n; the k rows of depths (up to 64 n int32) are
// taken from the stream-ordered pool per call, so a serving worker does not
// keep them between batches.
struct MsState {
  DevBuf F, N, seen, src;
  Frontier f[2];
};

}  // namespace

rg_status bfs_multi_run(rg_graph* g, const uint32_t* src_orig, int k, int32_t* h_depths, int64_t* rounds_out,
                        int32_t* d_depths_out) {
  if (!g) return fail(RG_EINVAL, "null graph");
  if (k < 1 || k > 64 || !src_orig) return fail(RG_EINVAL, "need 1..64 sources");
  OptScope opt_scope(g, kAppBfs);
  for (int q = 0; q < k; q++) {
    if (src_orig[q] >= (uint64_t)g->n) return fail(RG_EINVAL, "source %u >= n", src_orig[q]);
  }
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  cudaStream_t st = cx->stream;
  const int64_t n = g->n;
  static thread_local MsState S;
  RG_TRY(S.F.reserve(8 * n));
  RG_TRY(S.N.reserve(8 * n));
  RG_TRY(S.seen.reserve(8 * n));
  DevBuf depth_rows(true, st), out_rows(true, st);
  RG_TRY(depth_rows.reserve(4 * n * k));
  RG_TRY(S.src.reserve(4 * 64));
  RG_TRY(frontier_alloc(g, S.f[0]));
  RG_TRY(frontier_alloc(g, S.f[1]));
  std::vector<uint32_t> src(k), sdeg(k), uniq;
  RG_TRY(lookup_ids(g, src_orig, k, true, src.data(), sdeg.data()));
  unsigned long long full = 0ull;  // the bits that can spread: sources with out-edges
  for (int q = 0; q < k; q++) full |= sdeg[q] ? (1ull << q) : 0ull;
  for (int q = 0; q < k; q++) {
    if (std::find(uniq.begin(), uniq.end(), src[q]) == uniq.end()) uniq.push_back(src[q]);
  }
  CallTimer timer(g);
  unsigned long long* F = S.F.as<unsigned long long>();
  unsigned long long* N = S.N.as<unsigned long long>();
  unsigned long long* seen = S.seen.as<unsigned long long>();
  int32_t* depth = depth_rows.as<int32_t>();
  RG_CUDA(cudaMemsetAsync(F, 0, 8 * n, st));
  RG_CUDA(cudaMemsetAsync(N, 0, 8 * n, st));
  RG_CUDA(cudaMemsetAsync(seen, 0, 8 * n, st));
  RG_CUDA(cudaMemsetAsync(depth, 0xFF, 4 * n * k, st));
  RG_CUDA(cudaMemcpyAsync(S.src.p, src.data(), 4 * k, cudaMemcpyHostToDevice, st));
  ms_seed<<<1, 64, 0, st>>>(S.src.as<uint32_t>(), k, n, F, seen, depth);
  g_timing.kernel_launches++;
  RG_TRY(frontier_from_host(g, S.f[0], uniq.data(), (int64_t)uniq.size(), st));
  FView cur = view_of(S.f[0]), nxt = view_of(S.f[1]);
  EmOpts o;
  o.variant = RG_PUSH;  // bitmask propagation: the push is already one atomic per edge and source set
  int64_t rounds = 0;
  const int64_t nwords = (n + 31) / 32;
  while (cur.count > 0) {
    rounds++;
    const bool dense = cur.count + cur.degsum > g->m / std::max<int64_t>(g_opts.dense_div, 1);
    if (dense && cur.degsum > 0) {
      RG_CUDA(cudaMemsetAsync(nxt.bits, 0, 4 * nwords, st));
      g_timing.edges_traversed += cur.degsum;
      // dense level: the bitmask pull over every edge (seen is stable during
      // the level; N receives only the new bits)
      RG_TRY(launch_mask_sweep(g, seen, N, nxt.bits, st, full));
      Frontier shell;
      shell.bits.p = nxt.bits;
      RG_TRY(compact_bits(g, shell, st, true, nullptr, 0, nullptr, nxt.queue, nxt.qoff));
      shell.bits.p = nullptr;
      nxt.count = shell.count;
      nxt.degsum = shell.degsum;
      g_timing.kernel_launches += 3;
    } else {
      RG_TRY(edge_map(g, cur, OpMsBfs{F, seen, N}, &nxt, o, st));
    }
    if (cur.count > 0) {
      ms_clear_frontier<<<(unsigned)((cur.count + 255) / 256), 256, 0, st>>>(cur.queue, cur.count, F);
      g_timing.kernel_launches++;
    }
    if (nxt.count > 0) {
      ms_advance<<<(unsigned)((nxt.count + 255) / 256), 256, 0, st>>>(nxt.queue, nxt.count, N, F, seen, depth, n,
                                                                      (int32_t)rounds);
      g_timing.kernel_launches++;
    }
    RG_CUDA(cudaGetLastError());
    std::swap(cur, nxt);
  }
  RG_TRY(timer.stop());
  const int32_t* res = depth;
  if (g->sorted && (h_depths || d_depths_out)) {
    RG_TRY(out_rows.reserve(4 * n * k));
    const int64_t blocks = std::min<int64_t>((n * k + 255) / 256, (int64_t)device_sms() * 32);
    ms_gather<<<(unsigned)blocks, 256, 0, st>>>(depth, g->new_ids.as<uint32_t>(), n, k, out_rows.as<int32_t>());
    RG_CUDA(cudaGetLastError());
    res = out_rows.as<int32_t>();
  }
  if (d_depths_out) RG_CUDA(cudaMemcpyAsync(d_depths_out, res, 4 * n * k, cudaMemcpyDeviceToDevice, st));
  if (h_depths) RG_CUDA(cudaMemcpyAsync(h_depths, res, 4 * n * k, cudaMemcpyDeviceToHost, st));
  RG_CUDA(cudaStreamSynchronize(st));
  g_timing.algorithmic_bytes = 4 * g_timing.edges_traversed + 4 * (n + 1) + 24 * n + 4 * n * k;
  if (rounds_out) *rounds_out = rounds;
  return RG_OK;
}

// ---------------------------------------------------------------------------
// many graphs, one persistent launch
// ---------------------------------------------------------------------------
namespace {

constexpr int kBatchThreads = 1024;
constexpr double kDamp = 0.85;  // PageRank.C:126

struct BatchDesc {
  const uint64_t* vbase;    // per graph: first vertex slot in the per-vertex arrays
  const uint64_t* ebase;    // per graph: first edge slot
  const uint32_t* nv;       // per graph: vertices
  const uint32_t* off;      // concatenated offsets (graph g at vbase[g] + g, n_g + 1 entries)
  const uint32_t* adj;      // concatenated neighbour lists
  const uint32_t* src;      // per graph: 64 sources (graph-local ids)
  int k;                    // sources per graph
  unsigned long long* F;    // per-vertex masks
  unsigned long long* N;
  unsigned long long* seen;
  int32_t* depth;           // per graph: k rows of n_g depths at 64 * vbase[g]
  double* p;                // PageRank ranks
  double* acc;              // the iteration's new ranks
  U128* contrib;            // p / deg, exact 128-bit fixed point
  double* ranks;            // results
  int32_t* pr_iters;        // per graph: iterations run (PageRank.C's iter)
  const int32_t* task;      // task list: graph * 2 + kind (0 BFS, 1 PageRank), largest first
  int ntasks;
  int64_t max_iters;
};

__device__ void batch_msbfs(const BatchDesc& D, int gi) {
  const uint64_t vb = D.vbase[gi];
  const uint32_t n = D.nv[gi];
  const uint32_t* off = D.off + vb + gi;
  const uint32_t* adj = D.adj + D.ebase[gi];
  unsigned long long* F = D.F + vb;
  unsigned long long* N = D.N + vb;
  unsigned long long* seen = D.seen + vb;
  int32_t* depth = D.depth + 64 * vb;
  const int k = D.k;
  const unsigned long long all = k == 64 ? ~0ull : ((1ull << k) - 1ull);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = kBatchThreads / 32;
  __shared__ int s_any;
  __shared__ unsigned int s_front;
  for (uint32_t v = threadIdx.x; v < n; v += kBatchThreads) { F[v] = 0; N[v] = 0; seen[v] = 0; }
  for (int64_t i = threadIdx.x; i < (int64_t)k * n; i += kBatchThreads) depth[i] = -1;
  __syncthreads();
  if (threadIdx.x < k) {
    const uint32_t s = D.src[gi * 64 + threadIdx.x];
    atomicOr(F + s, 1ull << threadIdx.x);
    atomicOr(seen + s, 1ull << threadIdx.x);
    depth[(int64_t)threadIdx.x * n + s] = 0;
  }
  __syncthreads();
  for (int32_t level = 1;; level++) {
    if (threadIdx.x == 0) { s_any = 0; s_front = 0; }
    __syncthreads();
    // frontier size decides push or pull for this level
    unsigned int fc = 0;
    for (uint32_t v = threadIdx.x; v < n; v += kBatchThreads) fc += F[v] != 0ull;
    fc = warp_sum(fc);
    if (lane == 0) atomicAdd(&s_front, fc);
    __syncthreads();
    if (s_front * 16u > n) {
      // pull: a warp per vertex still missing bits, early exit once complete
      for (uint32_t v = warp; v < n; v += nw) {
        const unsigned long long sv = seen[v];
        if (sv == all) continue;
        unsigned long long a = 0;
        for (uint32_t j0 = off[v]; j0 < off[v + 1]; j0 += 32) {
          const uint32_t j = j0 + lane;
          if (j < off[v + 1]) a |= F[adj[j]];
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) a |= __shfl_xor_sync(0xffffffffu, a, o);
          if ((a | sv) == all) break;
        }
        if (lane == 0) N[v] = a & ~sv;
      }
    } else {
      // push: a warp per frontier vertex
      for (uint32_t u = warp; u < n; u += nw) {
        const unsigned long long fu = F[u];
        if (!fu) continue;
        for (uint32_t j = off[u] + lane; j < off[u + 1]; j += 32) {
          const uint32_t d = adj[j];
          const unsigned long long w = fu & ~seen[d];
          if (w) atomicOr(N + d, w);
        }
      }
    }
    __syncthreads();
    for (uint32_t v = threadIdx.x; v < n; v += kBatchThreads) {
      const unsigned long long w = N[v] & ~seen[v];
      N[v] = 0;
      F[v] = w;
      if (w) {
        seen[v] |= w;
        s_any = 1;
        unsigned long long x = w;
        while (x) {
          const int b = __ffsll((long long)x) - 1;
          x &= x - 1;
          depth[(int64_t)b * n + v] = level;
        }
      }
    }
    __syncthreads();
    const int any = s_any;
    __syncthreads();  // every thread has read the flag before thread 0 resets it
    if (!any) break;
  }
}

// One graph's PageRank inside the persistent kernel, with the arithmetic of
// pagerank.cu's pull (pr_exact.cuh): FP64 contributions p/deg, each
// vertex's sum formed exactly (128-bit fixed point) and rounded once,
// p' = fma(0.85, sum, 0.15/n), exact L1.  Sums do not depend on the order of
// the additions, so the ranks equal rg_pagerank's bit for bit.
// p'/deg by degree class, as pagerank.cu's pr_quotient: no out-edges, a
// power of two (exact exponent shift) or the IEEE division.  Every branch
// gives the correctly rounded quotient.
__device__ __forceinline__ double batch_quotient(double pn, uint32_t d) {
  if (d == 0) return 0.0;
  if ((d & (d - 1)) == 0) return double_of(bits_of(pn) - ((unsigned long long)(31 - __clz(d)) << 52));
  return pn / (double)d;
}

// One graph's PageRank inside the persistent kernel, with the arithmetic of
// pagerank.cu's pull (pr_exact.cuh): FP64 contributions p/deg, kept as their
// exact 128-bit fixed-point values, each vertex's sum formed exactly and
// rounded once, p' = fma(0.85, sum, 0.15/n), exact L1.  Sums do not depend on
// the order of the additions, so the ranks equal rg_pagerank's bit for bit.
// Rows are pulled by groups of 8 lanes (the batched graphs' rows are short).
__device__ void batch_pagerank(const BatchDesc& D, int gi) {
  const uint64_t vb = D.vbase[gi];
  const uint32_t n = D.nv[gi];
  const uint32_t* off = D.off + vb + gi;
  const uint32_t* adj = D.adj + D.ebase[gi];
  double* p = D.p + vb;
  double* acc = D.acc + vb;
  U128* contrib = D.contrib + vb;
  constexpr int kG = 8;  // lanes per row
  const int lane = threadIdx.x & 31, gl = lane & (kG - 1);
  const unsigned gmask = 0xFFu << (lane & ~(kG - 1));
  const uint32_t group = threadIdx.x / kG, ngroups = kBatchThreads / kG;
  // the reference's constants (PageRank.C:126-138)
  const double p0 = 1 / (double)n;
  const double added = (1 - kDamp) * (1 / (double)n);
  const U128 eps = pr_eps_fx();
  __shared__ U128 s_l1;
  for (uint32_t v = threadIdx.x; v < n; v += kBatchThreads) {
    p[v] = p0;
    contrib[v] = fx_from_double(batch_quotient(p0, off[v + 1] - off[v]));
  }
  __syncthreads();
  int64_t it = 0;
  bool broke = false;
  while (it < D.max_iters) {
    it++;
    if (threadIdx.x == 0) s_l1 = U128{0ull, 0ull};
    __syncthreads();
    U128 l1{0ull, 0ull};
    for (uint32_t v = group; v < n; v += ngroups) {  // pull: a group of lanes per row
      U128 s{0ull, 0ull};
      for (uint32_t j = off[v] + gl; j < off[v + 1]; j += kG) add128(s, contrib[adj[j]]);
#pragma unroll
      for (int o = kG / 2; o > 0; o >>= 1) {
        add128(s, U128{__shfl_xor_sync(gmask, s.lo, o), __shfl_xor_sync(gmask, s.hi, o)});
      }
      if (gl == 0) {
        const double pn = (s.lo | s.hi) ? fma(kDamp, fx_to_double(s), added) : added;
        const double po = p[v];
        if (po != pn) add128(l1, fx_from_double(fabs(po - pn)));
        acc[v] = pn;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      add128(l1, U128{__shfl_xor_sync(0xffffffffu, l1.lo, o), __shfl_xor_sync(0xffffffffu, l1.hi, o)});
    }
    if (lane == 0 && (l1.lo | l1.hi)) {
      const unsigned long long old = atomicAdd(&s_l1.lo, l1.lo);
      const unsigned long long hi = l1.hi + (old + l1.lo < old ? 1ull : 0ull);
      if (hi) atomicAdd(&s_l1.hi, hi);
    }
    __syncthreads();
    for (uint32_t v = threadIdx.x; v < n; v += kBatchThreads) {
      const double pn = acc[v];
      p[v] = pn;
      contrib[v] = fx_from_double(batch_quotient(pn, off[v + 1] - off[v]));
    }
    __syncthreads();
    const bool conv = less128(s_l1, eps);
    __syncthreads();  // every thread has read the sum before thread 0 resets it
    if (conv) { broke = true; break; }
  }
  for (uint32_t v = threadIdx.x; v < n; v += kBatchThreads) D.ranks[vb + v] = p[v];
  if (threadIdx.x == 0) D.pr_iters[gi] = (int32_t)(broke ? it : D.max_iters + 1);
}

__global__ void __launch_bounds__(kBatchThreads) batch_persistent(BatchDesc D, int* next_task) {
  __shared__ int s_task;
  for (;;) {
    if (threadIdx.x == 0) s_task = atomicAdd(next_task, 1);
    __syncthreads();
    const int t = s_task;
    __syncthreads();
    if (t >= D.ntasks) return;
    const int code = D.task[t];
    if ((code & 1) == 0) batch_msbfs(D, code >> 1);
    else batch_pagerank(D, code >> 1);
    __syncthreads();
  }
}

}  // namespace
}  // namespace rg

struct rg_batch {
  int ngraphs = 0;
  std::vector<uint32_t> nv;
  std::vector<uint64_t> vbase, ebase;
  uint64_t total_v = 0, total_e = 0;
  rg::DevBuf d_vbase, d_ebase, d_nv, d_off, d_adj, d_src, d_F, d_N, d_seen, d_depth, d_p, d_acc, d_contrib,
      d_ranks, d_iters, d_task, d_counter;
};

using namespace rg;

extern "C" rg_status rg_bfs_multi(rg_graph* g, const uint32_t* h_sources, int k, int32_t* h_depths,
                                  int64_t* rounds_out) {
  return bfs_multi_run(g, h_sources, k, h_depths, rounds_out, nullptr);
}

extern "C" rg_status rg_batch_create(int ngraphs, const int64_t* ns, const int64_t* ms, const uint32_t* const* h_offs,
                                     const uint32_t* const* h_adjs, rg_batch** out) {
  if (ngraphs < 1 || !ns || !ms || !h_offs || !h_adjs || !out) return fail(RG_EINVAL, "rg_batch_create: bad arguments");
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  rg_batch* b = new (std::nothrow) rg_batch();
  if (!b) return fail(RG_ENOMEM, "host allocation failed");
  b->ngraphs = ngraphs;
  b->nv.resize(ngraphs);
  b->vbase.resize(ngraphs);
  b->ebase.resize(ngraphs);
  for (int i = 0; i < ngraphs; i++) {
    if (ns[i] <= 0 || ns[i] >= (1ll << 31) || ms[i] < 0 || !h_offs[i] || (ms[i] > 0 && !h_adjs[i]) ||
        h_offs[i][0] != 0 || h_offs[i][ns[i]] != (uint32_t)ms[i]) {
      delete b;
      return fail(RG_EINVAL, "rg_batch_create: graph %d is not a valid CSR", i);
    }
    b->nv[i] = (uint32_t)ns[i];
    b->vbase[i] = b->total_v;
    b->ebase[i] = b->total_e;
    b->total_v += ns[i];
    b->total_e += ms[i];
  }
  // concatenated host images, uploaded once
  std::vector<uint32_t> off(b->total_v + ngraphs), adj(b->total_e + 4, 0);
  for (int i = 0; i < ngraphs; i++) {
    memcpy(off.data() + b->vbase[i] + i, h_offs[i], 4 * (ns[i] + 1));
    if (ms[i]) memcpy(adj.data() + b->ebase[i], h_adjs[i], 4 * ms[i]);
  }
  const uint64_t V = b->total_v;
  rg_status s;
  if ((s = b->d_vbase.reserve(8 * ngraphs)) != RG_OK || (s = b->d_ebase.reserve(8 * ngraphs)) != RG_OK ||
      (s = b->d_nv.reserve(4 * ngraphs)) != RG_OK || (s = b->d_off.reserve(4 * off.size())) != RG_OK ||
      (s = b->d_adj.reserve(4 * adj.size())) != RG_OK || (s = b->d_src.reserve(4 * 64 * ngraphs)) != RG_OK ||
      (s = b->d_F.reserve(8 * V)) != RG_OK || (s = b->d_N.reserve(8 * V)) != RG_OK ||
      (s = b->d_seen.reserve(8 * V)) != RG_OK || (s = b->d_depth.reserve(4 * 64 * V)) != RG_OK ||
      (s = b->d_p.reserve(8 * V)) != RG_OK || (s = b->d_acc.reserve(8 * V)) != RG_OK ||
      (s = b->d_contrib.reserve(16 * V)) != RG_OK || (s = b->d_ranks.reserve(8 * V)) != RG_OK ||
      (s = b->d_iters.reserve(4 * ngraphs)) != RG_OK || (s = b->d_task.reserve(4 * 2 * ngraphs)) != RG_OK ||
      (s = b->d_counter.reserve(64)) != RG_OK) {
    delete b;
    return s;
  }
  cudaError_t e = cudaMemcpy(b->d_vbase.p, b->vbase.data(), 8 * ngraphs, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_ebase.p, b->ebase.data(), 8 * ngraphs, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_nv.p, b->nv.data(), 4 * ngraphs, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_off.p, off.data(), 4 * off.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_adj.p, adj.data(), 4 * adj.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    delete b;
    return cuda_fail(e, "batch upload", __FILE__, __LINE__);
  }
  *out = b;
  return RG_OK;
}

extern "C" rg_status rg_batch_free(rg_batch* b) {
  delete b;
  return RG_OK;
}

extern "C" rg_status rg_batch_run(rg_batch* b, const uint32_t* h_sources, int k, int64_t pr_iters, int32_t* h_depths,
                                  double* h_ranks, int32_t* h_pr_iters, double* device_ms) {
  if (!b || !h_sources || k < 1 || k > 64 || pr_iters < 0) return fail(RG_EINVAL, "rg_batch_run: bad arguments");
  for (int i = 0; i < b->ngraphs; i++) {
    for (int q = 0; q < k; q++) {
      if (h_sources[i * k + q] >= b->nv[i]) return fail(RG_EINVAL, "rg_batch_run: source out of range in graph %d", i);
    }
  }
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  cudaStream_t st = cx->stream;
  // sources padded to 64 per graph; tasks: both tasks of every graph, largest
  // graphs first so the tail of the launch holds the small ones
  std::vector<uint32_t> src(64 * (size_t)b->ngraphs, 0);
  for (int i = 0; i < b->ngraphs; i++) memcpy(src.data() + 64 * (size_t)i, h_sources + (size_t)i * k, 4 * k);
  std::vector<int> order(b->ngraphs);
  std::iota(order.begin(), order.end(), 0);
  std::vector<uint64_t> work(b->ngraphs);
  for (int i = 0; i < b->ngraphs; i++) {
    const uint64_t m = (i + 1 < b->ngraphs ? b->ebase[i + 1] : b->total_e) - b->ebase[i];
    work[i] = m + b->nv[i];
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return work[a] > work[c]; });
  std::vector<int32_t> tasks;
  tasks.reserve(2 * b->ngraphs);
  for (int i : order) {
    tasks.push_back(i * 2 + 0);
    tasks.push_back(i * 2 + 1);
  }
  RG_CUDA(cudaMemcpyAsync(b->d_src.p, src.data(), 4 * src.size(), cudaMemcpyHostToDevice, st));
  RG_CUDA(cudaMemcpyAsync(b->d_task.p, tasks.data(), 4 * tasks.size(), cudaMemcpyHostToDevice, st));
  RG_CUDA(cudaMemsetAsync(b->d_counter.p, 0, 64, st));
  BatchDesc D;
  D.vbase = b->d_vbase.as<uint64_t>();
  D.ebase = b->d_ebase.as<uint64_t>();
  D.nv = b->d_nv.as<uint32_t>();
  D.off = b->d_off.as<uint32_t>();
  D.adj = b->d_adj.as<uint32_t>();
  D.src = b->d_src.as<uint32_t>();
  D.k = k;
  D.F = b->d_F.as<unsigned long long>();
  D.N = b->d_N.as<unsigned long long>();
  D.seen = b->d_seen.as<unsigned long long>();
  D.depth = b->d_depth.as<int32_t>();
  D.p = b->d_p.as<double>();
  D.acc = b->d_acc.as<double>();
  D.contrib = b->d_contrib.as<U128>();
  D.ranks = b->d_ranks.as<double>();
  D.pr_iters = b->d_iters.as<int32_t>();
  D.task = b->d_task.as<int32_t>();
  D.ntasks = (int)tasks.size();
  D.max_iters = pr_iters;
  int per_sm = 0;
  RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_persistent, kBatchThreads, 0));
  const int grid = device_sms() * std::max(per_sm, 1);
  RG_CUDA(cudaEventRecord(cx->ev0, st));
  batch_persistent<<<grid, kBatchThreads, 0, st>>>(D, b->d_counter.as<int>());
  RG_CUDA(cudaGetLastError());
  RG_CUDA(cudaEventRecord(cx->ev1, st));
  RG_CUDA(cudaEventSynchronize(cx->ev1));
  float ms = 0;
  RG_CUDA(cudaEventElapsedTime(&ms, cx->ev0, cx->ev1));
  if (device_ms) *device_ms = ms;
  // results: depths graph by graph (k rows of n_g each), ranks, iterations
  if (h_depths) {
    size_t o = 0;
    for (int i = 0; i < b->ngraphs; i++) {
      const size_t cnt = (size_t)k * b->nv[i];
      RG_CUDA(cudaMemcpyAsync(h_depths + o, b->d_depth.as<int32_t>() + 64 * b->vbase[i], 4 * cnt,
                              cudaMemcpyDeviceToHost, st));
      o += cnt;
    }
  }
  if (h_ranks) RG_CUDA(cudaMemcpyAsync(h_ranks, b->d_ranks.p, 8 * b->total_v, cudaMemcpyDeviceToHost, st));
  if (h_pr_iters) RG_CUDA(cudaMemcpyAsync(h_pr_iters, b->d_iters.p, 4 * b->ngraphs, cudaMemcpyDeviceToHost, st));
  RG_CUDA(cudaStreamSynchronize(st));
  return RG_OK;
}
