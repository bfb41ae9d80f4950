// PageRankDelta (PageRankDelta.C:98-155) on the device.
//
// Each round pushes (or, in push-pull, pulls) the frontier's deltas through
// the engine -- nghSum[d] += Delta[s]/deg(s) -- and then one vertex kernel
// applies the round's filter to every vertex (PR_Vertex_F_FirstRound in round
// 1, PR_Vertex_F after), resets nghSum, forms the next frontier's
// contributions and bitmap, and sums |Delta| for the L1 stop (< 1e-7).  The
// arithmetic is FP64 like the reference: the deltas shrink geometrically,
// past what the fixed point of the PageRank pipeline resolves.

#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "app_common.cuh"

namespace rg {

namespace {

constexpr double kDamping = 0.85;
constexpr double kEps = 0.0000001;
constexpr double kEps2 = 0.01;

__global__ void prd_init(uint32_t n, const uint32_t* __restrict__ off, double* p, double* delta, double* ngh,
                         double* c, double one_over_n) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    p[v] = 0.0;
    delta[v] = one_over_n;
    ngh[v] = 0.0;
    const uint32_t d = off[v + 1] - off[v];
    c[v] = d ? one_over_n / d : 0.0;
  }
}

// vertexFilter over all vertices with the round's functor, fused with the
// L1 terms, the nghSum reset (PR_Vertex_Reset) and the next contributions.
// Each warp owns 32 consecutive vertices = one bitmap word (grid stride in
// whole warps), so the active set is written with a ballot, no atomics.
template <bool kFirst>
__global__ void __launch_bounds__(256) prd_filter(uint32_t n, const uint32_t* __restrict__ off, double* p,
                                                  double* delta, double* ngh, double* c, double one_over_n,
                                                  double added, uint32_t* next_bits, double* l1_out) {
  const int lane = threadIdx.x & 31;
  double local = 0.0;
  const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w * 32 < n; w += warps) {
    const uint64_t v = w * 32 + lane;
    bool act = false;
    if (v < n) {
      double pv = p[v], d;
      if (kFirst) {  // PageRankDelta.C:46-61
        d = __dadd_rn(__dmul_rn(kDamping, ngh[v]), added);
        pv = __dadd_rn(pv, d);
        d = __dsub_rn(d, one_over_n);
        act = fabs(d) > __dmul_rn(kEps2, pv);
      } else {  // PageRankDelta.C:63-76
        d = __dmul_rn(ngh[v], kDamping);
        act = fabs(d) > __dmul_rn(kEps2, pv);
        if (act) pv = __dadd_rn(pv, d);
      }
      p[v] = pv;
      delta[v] = d;
      ngh[v] = 0.0;
      const uint32_t deg = off[v + 1] - off[v];
      c[v] = (act && deg) ? __ddiv_rn(d, (double)deg) : 0.0;
      local += fabs(d);
    }
    const unsigned bits = __ballot_sync(0xffffffffu, act);
    if (lane == 0) next_bits[w] = bits;
  }
  local = warp_sum(local);
  __shared__ double ws[8];
  if (lane == 0) ws[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < 8 ? ws[threadIdx.x] : 0.0;
    t = warp_sum(t);
    if (threadIdx.x == 0) atomicAdd(l1_out, t);
  }
}

// Dense round as a pull over every edge: nghSum[v] = sum of c[u] over all
// neighbours.  c is 0 for vertices outside the frontier (the filter writes
// it so), so no frontier test is needed and the sum is the push's over the
// frontier.  Edge-balanced (8 edges per lane, edge array streamed), FP64
// sums in a fixed order, one add per row piece.
__global__ void __launch_bounds__(256) prd_pull_sweep(DevGraph g, const uint32_t* __restrict__ chunk_v,
                                                      uint32_t nchunks, const double* __restrict__ c, double* ngh) {
  constexpr int kItems = 8, kStep = 32 * kItems;
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t ch = warp; ch < nchunks; ch += nwarps) {
    const uint32_t vlo = chunk_v[ch], vhi = chunk_v[ch + 1];
#pragma unroll
    for (int r = 0; r < kSweepChunk / kStep; r++) {
      const uint32_t e = ch * kSweepChunk + r * kStep + lane * kItems;
      uint32_t row = kNone;
      double part = 0.0;
      if (e < g.m) {
        const U32x8 w = ld_stream_v8(g.adj + e);  // in bounds: adj is padded by 8 entries
        uint32_t v = upper_index(g.off, vlo, vhi, e);
        uint32_t nxt = g.off[v + 1];
        double x[kItems];
#pragma unroll
        for (int i = 0; i < kItems; i++) x[i] = (e + i < g.m) ? __ldg(c + w.v[i]) : 0.0;
        row = v;
#pragma unroll
        for (int i = 0; i < kItems; i++) {
          const uint32_t ee = e + i;
          if (ee >= g.m) break;
          if (ee >= nxt) {
            if (part != 0.0) atomicAdd(ngh + row, part);  // a row piece that ends in this lane
            part = 0.0;
            do { v++; nxt = g.off[v + 1]; } while (ee >= nxt);
            row = v;
          }
          part += x[i];
        }
      }
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const double t = __shfl_up_sync(0xffffffffu, part, o);
        const uint32_t tr = __shfl_up_sync(0xffffffffu, row, o);
        if (lane >= o && tr == row) part += t;
      }
      const uint32_t next_row = __shfl_down_sync(0xffffffffu, row, 1);
      if (row != kNone && (lane == 31 || next_row != row) && part != 0.0) atomicAdd(ngh + row, part);
    }
  }
}

struct PrdState {
  DevBuf p, delta, ngh, c, l1, tmp;
  Frontier f[2];
};

}  // namespace

rg_status pagerank_delta_run(rg_graph* g, int variant, int64_t max_iters, double* h_ranks, int64_t* iters_out,
                             double* l1_out) {
  if (!g) return fail(RG_EINVAL, "null graph");
  if (variant < 0 || variant > 4) return fail(RG_EINVAL, "bad variant %d", variant);
  if (max_iters < 0) return fail(RG_EINVAL, "max_iters < 0");
  OptScope opt_scope(g, kAppPagerank);  // the PageRank schedule: same kind of sweep
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  cudaStream_t st = cx->stream;
  const int64_t n = g->n;
  static thread_local PrdState S;
  RG_TRY(S.p.reserve(8 * n));
  RG_TRY(S.delta.reserve(8 * n));
  RG_TRY(S.ngh.reserve(8 * n));
  RG_TRY(S.c.reserve(8 * n));
  RG_TRY(S.l1.reserve(8));
  RG_TRY(frontier_alloc(g, S.f[0]));
  RG_TRY(frontier_alloc(g, S.f[1]));
  const double one_over_n = 1 / (double)n;
  const double added = (1 - kDamping) * one_over_n;  // PageRankDelta.C:55
  double* p = S.p.as<double>();
  double* delta = S.delta.as<double>();
  double* ngh = S.ngh.as<double>();
  double* c = S.c.as<double>();
  double* d_l1 = S.l1.as<double>();
  const int vblocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)device_sms() * 16);
  CallTimer timer(g);
  prd_init<<<vblocks, 256, 0, st>>>((uint32_t)n, g->off.as<uint32_t>(), p, delta, ngh, c, one_over_n);
  g_timing.kernel_launches++;
  RG_TRY(frontier_set_all(g, S.f[0], st));  // every vertex starts in the frontier
  FView cur = view_of(S.f[0]), nxt = view_of(S.f[1]);
  EmOpts o;
  o.variant = variant;
  o.dense_forward = variant != RG_PUSH_PULL;  // no_output | dense_forward; push-pull pulls
  Workspace& ws = cx->ws;
  int64_t round = 0;
  double l1 = 0.0;
  while (round++ < max_iters) {
    const bool dense = cur.count + cur.degsum > g->m / std::max<int64_t>(g_opts.dense_div, 1);
    if (dense && g->m > 0 && (variant == RG_PUSH_PULL || g_opts.direction == 1)) {
      static std::atomic<uint64_t> carveout_set{0};
      RG_TRY(once_per_device(carveout_set, [] {
        RG_CUDA(cudaFuncSetAttribute(prd_pull_sweep, cudaFuncAttributePreferredSharedMemoryCarveout, 0));
        return RG_OK;
      }));
      static std::atomic<int> resident{0};
      int per_sm = resident.load(std::memory_order_relaxed);
      if (!per_sm) {
        RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, prd_pull_sweep, 256, 0));
        per_sm = std::max(per_sm, 1);
        resident.store(per_sm, std::memory_order_relaxed);
      }
      const int64_t grid = std::min<int64_t>((int64_t)device_sms() * per_sm, (g->nchunks * 32 + 255) / 256);
      g_timing.edges_traversed += cur.degsum;
      kt_begin(st);
      prd_pull_sweep<<<(unsigned)std::max<int64_t>(grid, 1), 256, 0, st>>>(g->in_view(), g->in_chunks(),
                                                                             (uint32_t)g->nchunks, c, ngh);
      kt_end(st);
      RG_CUDA(cudaGetLastError());
      g_timing.kernel_launches++;
      g_timing.edge_launches++;
    } else {
      RG_TRY(edge_map(g, cur, OpPrDelta{c, ngh}, nullptr, o, st));
    }
    RG_CUDA(cudaMemsetAsync(d_l1, 0, 8, st));
    if (round == 1) {
      prd_filter<true><<<vblocks, 256, 0, st>>>((uint32_t)n, g->off.as<uint32_t>(), p, delta, ngh, c, one_over_n,
                                                added, nxt.bits, d_l1);
    } else {
      prd_filter<false><<<vblocks, 256, 0, st>>>((uint32_t)n, g->off.as<uint32_t>(), p, delta, ngh, c,
                                                 one_over_n, added, nxt.bits, d_l1);
    }
    RG_CUDA(cudaGetLastError());
    g_timing.kernel_launches++;
    RG_CUDA(cudaMemcpyAsync(&ws.h_info[4], d_l1, 8, cudaMemcpyDeviceToHost, st));
    Frontier shell;  // non-owning view of nxt for the compaction (which syncs)
    shell.bits.p = nxt.bits;
    RG_TRY(compact_bits(g, shell, st, true, nullptr, 0, nullptr, nxt.queue, nxt.qoff));
    shell.bits.p = nullptr;
    nxt.count = shell.count;
    nxt.degsum = shell.degsum;
    g_timing.kernel_launches += 3;
    memcpy(&l1, &ws.h_info[4], 8);
    if (l1 < kEps) break;  // PageRankDelta.C:144
    std::swap(cur, nxt);
  }
  RG_TRY(timer.stop());
  RG_TRY(download_orig<double>(g, p, h_ranks, S.tmp, st));
  RG_CUDA(cudaStreamSynchronize(st));
  // edge array + contribution per frontier edge; p, Delta, nghSum, c, the
  // degree and the bitmap per vertex per round
  g_timing.algorithmic_bytes = 12 * g_timing.edges_traversed + (int64_t)(44 * n + n / 8) * std::min(round, max_iters);
  if (iters_out) *iters_out = round;
  if (l1_out) *l1_out = l1;
  return RG_OK;
}

}  // namespace rg

extern "C" rg_status rg_pagerank_delta(rg_graph* g, rg_variant variant, int64_t max_iters, double* h_ranks,
                                       int64_t* iters_out, double* l1_out) {
  return rg::pagerank_delta_run(g, variant, max_iters, h_ranks, iters_out, l1_out);
}
