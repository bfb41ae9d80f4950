// Many Radii queries in one traversal: query q (its own <= 64 sample
// vertices) owns word q of a W-word mask per vertex, W = the query count
// rounded up to a power of two (<= 16).  A round propagates all words at
// once -- sparse rounds push over the union frontier with the engine's
// edge-balanced push, dense rounds pull every vertex's neighbour masks with
// an edge-balanced sweep, so one gather fetches all W words of a neighbour
// -- and radii[q][v] = round wherever word q of v changed (Radii.C:37-106,
// 140-218, applied per word).
//
// Each query's result equals its own single-query run: a vertex is in the
// union frontier when any word changed, and pushing a word that did not
// change adds nothing, because that word was pushed to every neighbour in the
// round it last changed.  The same argument lets the dense rounds skip the
// frontier test (as the single-query dense rounds do).

#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "app_common.cuh"

namespace rg {
namespace {

// Radii_F on W words: every word of s that adds bits to d is ORed into
// next[d]; d joins the next frontier when any word grew.
struct OpRadiiW {
  const unsigned long long* __restrict__ vis;
  unsigned long long* nvis;
  int W;
  using HubT = unsigned long long;  // no hub copies: the push runs without them
  static constexpr bool kOutput = true;
  __device__ __forceinline__ bool cond(uint32_t) const { return true; }
  __device__ __forceinline__ bool push(uint32_t s, uint32_t d) const {
    bool grew = false;
    for (int w = 0; w < W; w++) {
      const unsigned long long x = vis[(size_t)s * W + w] & ~vis[(size_t)d * W + w];
      if (x) {
        atomicOr(nvis + (size_t)d * W + w, x);
        grew = true;
      }
    }
    return grew;
  }
  __device__ static HubT hub_identity() { return 0ull; }
  __device__ __forceinline__ void hub_push(HubT*, uint32_t, uint32_t, uint32_t) const {}
  __device__ __forceinline__ bool hub_merge(uint32_t, HubT) const { return false; }
};

__global__ void rq_seed(const uint32_t* __restrict__ v, const unsigned long long* __restrict__ mask,
                        const int* __restrict__ word, int k, int W, int64_t n, unsigned long long* nvis,
                        int32_t* radii) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < k) {
    nvis[(size_t)v[j] * W + word[j]] = mask[j];
    radii[(int64_t)word[j] * n + v[j]] = 0;
  }
}

// Start of a round: the frontier's masks become current (vertexMap
// Radii_Vertex_F, Radii.C:78-86).
__global__ void rq_sync(const uint32_t* __restrict__ q, int64_t count, int W, unsigned long long* vis,
                        const unsigned long long* __restrict__ nvis) {
  const int64_t total = count * W;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = i / W;
    const size_t e = (size_t)q[j] * W + (i - j * W);
    vis[e] = nvis[e];
  }
}

// radii[w][v] = round for every word that grew at a new frontier vertex.
__global__ void rq_mark(const uint32_t* __restrict__ q, int64_t count, int W, int nq, int64_t n,
                        const unsigned long long* __restrict__ vis, const unsigned long long* __restrict__ nvis,
                        int32_t* radii, int32_t round) {
  const int64_t total = count * W;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = i / W;
    const int w = (int)(i - j * W);
    if (w >= nq) continue;
    const uint32_t v = q[j];
    const size_t e = (size_t)v * W + w;
    if (nvis[e] != vis[e]) radii[(int64_t)w * n + v] = round;
  }
}

// The bits each word can still receive (a query's samples with out-edges):
// a row whose W words hold them all cannot grow, and its edges are not
// gathered -- as in mask_pull_sweep, this skips most of the graph in the
// last dense rounds.  All zero: every row is gathered.
template <int W>
struct RowFull {
  unsigned long long w[W];
};

// Words per lane in the dense rounds: up to four (one 32-byte load), so the
// row walk and bookkeeping a lane repeats per item are shared by its words.
template <int W>
__host__ __device__ constexpr int rq_words_per_lane() {
  return W < 4 ? W : 4;
}

// A lane's kWL consecutive mask words (kWL*8-byte aligned) in one load.
template <int kWL>
__device__ __forceinline__ void rq_load_words(const unsigned long long* p, unsigned long long (&x)[kWL]) {
  if constexpr (kWL == 1) {
    x[0] = __ldg(p);
  } else if constexpr (kWL == 2) {
    const ulonglong2 t = __ldg(reinterpret_cast<const ulonglong2*>(p));
    x[0] = t.x;
    x[1] = t.y;
  } else {
    uint32_t r[8];
    asm("ld.global.nc.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
        : "l"(p));
#pragma unroll
    for (int h = 0; h < 4; h++) x[h] = ((unsigned long long)r[2 * h + 1] << 32) | r[2 * h];
  }
}

// One lane's words of a row piece: the new bits (not yet in vis) go into
// nvis, and the row is marked in next_bits once per slot.  The lanes of a
// slot walk the same rows and so reach every flush together; slot_mask names
// them.
template <int W, int kWL>
__device__ __forceinline__ void rq_flush_words(const unsigned long long* __restrict__ vis, unsigned long long* nvis,
                                               uint32_t* next_bits, uint32_t row, int w0, unsigned slot_mask,
                                               const unsigned long long (&part)[kWL]) {
  bool any = false;
#pragma unroll
  for (int i = 0; i < kWL; i++) any |= part[i] != 0ull;
  bool grew = false;
  if (any) {
    unsigned long long have[kWL];
    rq_load_words<kWL>(vis + (size_t)row * W + w0, have);
#pragma unroll
    for (int i = 0; i < kWL; i++) {
      const unsigned long long x = part[i] & ~have[i];
      if (x) {
        atomicOr(nvis + (size_t)row * W + w0 + i, x);
        grew = true;
      }
    }
  }
  const unsigned g = __ballot_sync(slot_mask, grew);
  if (g && w0 == 0) bit_set(next_bits, row);
}

// Dense round, W words: next[v] |= (OR of vis[u] over every neighbour u) &
// ~vis[v] per word.  Word lanes: a slot of W/kWL lanes walks 512*W/(32*kWL)
// consecutive edges of the warp's 512-edge chunk, and each lane gathers its
// kWL consecutive words of every neighbour's row in one load, so one gather
// instruction reads whole W-word rows (64 bytes at W = 8) of several edges.
// A lane skips the gather where its words of the row already hold every bit
// their queries can spread (`full`), and flushes a row piece where the row
// ends; the slots' last pieces are combined by a segmented OR scan across
// slots once per chunk.
template <int W>
__global__ void __launch_bounds__(256) rq_pull_sweep(DevGraph g, const uint32_t* __restrict__ chunk_v,
                                                     uint32_t nchunks, const unsigned long long* __restrict__ vis,
                                                     unsigned long long* nvis, uint32_t* next_bits, RowFull<W> full) {
  static_assert(W >= 1 && W <= 16 && (W & (W - 1)) == 0, "1..16 words, a power of two");
  constexpr int kWL = rq_words_per_lane<W>();
  constexpr int kLanes = W / kWL;              // lanes per slot
  constexpr int kSlots = 32 / kLanes;
  constexpr int kPer = kSweepChunk / kSlots;   // edges per slot per chunk
  constexpr int kGroup = kWL == 4 ? 4 : 8;     // edges per id load
  constexpr int kBatch = 8 / kWL;              // gathers in flight per lane at a time
  static_assert(kPer % kGroup == 0, "whole id groups per slot");
  const int lane = threadIdx.x & 31;
  const int slot = lane / kLanes;
  const int w0 = (lane % kLanes) * kWL;
  const unsigned slot_mask = (kLanes == 32 ? 0xffffffffu : ((1u << kLanes) - 1u)) << (slot * kLanes);
  unsigned long long fw[kWL];  // the bits each of the lane's words can still receive
#pragma unroll
  for (int i = 0; i < kWL; i++) {
    fw[i] = 0ull;
#pragma unroll
    for (int j = 0; j < W; j++) fw[i] = j == w0 + i ? full.w[j] : fw[i];
  }
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t c = warp; c < nchunks; c += nwarps) {
    const uint32_t vlo = chunk_v[c], vhi = chunk_v[c + 1];
    const uint32_t e0 = c * kSweepChunk + slot * kPer;  // the slot's first edge
    uint32_t row = kNone;
    unsigned long long part[kWL];
#pragma unroll
    for (int i = 0; i < kWL; i++) part[i] = 0ull;
    if (e0 < g.m) {
      uint32_t v = upper_index(g.off, vlo, vhi, e0);
      uint32_t nxt = g.off[v + 1];
      auto words_open = [&](uint32_t r) {
        unsigned long long have[kWL];
        rq_load_words<kWL>(vis + (size_t)r * W + w0, have);
        bool open = false;
#pragma unroll
        for (int i = 0; i < kWL; i++) open |= fw[i] != 0ull && (have[i] & fw[i]) != fw[i];
        return open;
      };
      bool open = words_open(v);
      row = v;
      for (int b = 0; b < kPer; b += kGroup) {
        if (e0 + b >= g.m) break;
        // the group's rows and which gathers this lane needs
        uint32_t rowj[kGroup];
        unsigned need = 0;
#pragma unroll
        for (int j = 0; j < kGroup; j++) {
          const uint32_t ee = e0 + b + j;
          if (ee < g.m && ee >= nxt) {
            do { v++; nxt = g.off[v + 1]; } while (ee >= nxt);
            open = words_open(v);
          }
          rowj[j] = v;
          if (ee < g.m && open) need |= 1u << j;
        }
        // in bounds: adj is padded by 8 entries and the group starts before m
        U32x8 ids;
        if constexpr (kGroup == 8) {
          ids = ld_stream_v8(g.adj + e0 + b);
        } else {
          const uint4 q = ld_stream_v4(g.adj + e0 + b, policy_evict_first());
          ids.v[0] = q.x;
          ids.v[1] = q.y;
          ids.v[2] = q.z;
          ids.v[3] = q.w;
        }
#pragma unroll
        for (int h = 0; h < kGroup; h += kBatch) {
          unsigned long long x[kBatch][kWL];
#pragma unroll
          for (int j = 0; j < kBatch; j++) {
            if ((need >> (h + j)) & 1u) {
              rq_load_words<kWL>(vis + (size_t)ids.v[h + j] * W + w0, x[j]);
            } else {
#pragma unroll
              for (int i = 0; i < kWL; i++) x[j][i] = 0ull;
            }
          }
#pragma unroll
          for (int j = 0; j < kBatch; j++) {
            if (e0 + b + h + j >= g.m) break;
            if (rowj[h + j] != row) {  // a row piece that ends in this slot
              rq_flush_words<W, kWL>(vis, nvis, next_bits, row, w0, slot_mask, part);
#pragma unroll
              for (int i = 0; i < kWL; i++) part[i] = 0ull;
              row = rowj[h + j];
            }
#pragma unroll
            for (int i = 0; i < kWL; i++) part[i] |= x[j][i];
          }
        }
      }
    }
    // segmented OR scan of the slots' last pieces (lanes of the same words)
#pragma unroll
    for (int o = 1; o < kSlots; o <<= 1) {
      const uint32_t tr = __shfl_up_sync(0xffffffffu, row, o * kLanes);
#pragma unroll
      for (int i = 0; i < kWL; i++) {
        const unsigned long long t = __shfl_up_sync(0xffffffffu, part[i], o * kLanes);
        if (slot >= o && tr == row) part[i] |= t;
      }
    }
    const uint32_t next_row = __shfl_down_sync(0xffffffffu, row, kLanes);
    if (row != kNone && (slot == kSlots - 1 || next_row != row)) {
      rq_flush_words<W, kWL>(vis, nvis, next_bits, row, w0, slot_mask, part);
    }
  }
}

template <int W>
rg_status launch_rq_sweep(rg_graph* g, const unsigned long long* vis, unsigned long long* nvis, uint32_t* bits,
                          cudaStream_t st, const unsigned long long* full_words) {
  RowFull<W> full;
  for (int w = 0; w < W; w++) full.w[w] = full_words[w];
  auto kern = rq_pull_sweep<W>;
  static std::atomic<int> resident{0};
  int per_sm = resident.load(std::memory_order_relaxed);
  if (!per_sm) {
    RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, 0));
    per_sm = std::max(per_sm, 1);
    resident.store(per_sm, std::memory_order_relaxed);
  }
  const int64_t grid = std::min<int64_t>((int64_t)device_sms() * per_sm, (g->nchunks * 32 + 255) / 256);
  kt_begin(st);
  kern<<<(unsigned)std::max<int64_t>(grid, 1), 256, 0, st>>>(g->in_view(), g->in_chunks(), (uint32_t)g->nchunks, vis,
                                                             nvis, bits, full);
  kt_end(st);
  RG_CUDA(cudaGetLastError());
  g_timing.kernel_launches++;
  g_timing.edge_launches++;
  return RG_OK;
}

rg_status rq_sweep(int W, rg_graph* g, const unsigned long long* vis, unsigned long long* nvis, uint32_t* bits,
                   cudaStream_t st, const unsigned long long* full_words) {
  switch (W) {
    case 1: return launch_rq_sweep<1>(g, vis, nvis, bits, st, full_words);
    case 2: return launch_rq_sweep<2>(g, vis, nvis, bits, st, full_words);
    case 4: return launch_rq_sweep<4>(g, vis, nvis, bits, st, full_words);
    case 8: return launch_rq_sweep<8>(g, vis, nvis, bits, st, full_words);
    default: return launch_rq_sweep<16>(g, vis, nvis, bits, st, full_words);
  }
}

inline unsigned grid_for(int64_t items) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>((items + 255) / 256, (int64_t)device_sms() * 32));
}

}  // namespace

rg_status radii_multi_run(rg_graph* g, const uint32_t* seeds_orig, int k, int nq, int32_t* h_radii,
                          int32_t* d_radii_out, int64_t* rounds_out) {
  if (!g) return fail(RG_EINVAL, "null graph");
  if (nq < 1 || nq > 16) return fail(RG_EINVAL, "need 1..16 queries");
  if (k < 0 || k > 64 || (k > 0 && !seeds_orig)) return fail(RG_EINVAL, "need 0..64 seeds per query");
  OptScope opt_scope(g, kAppRadii);
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  cudaStream_t st = cx->stream;
  const int64_t n = g->n;
  int W = 1;
  while (W < nq) W *= 2;
  // per query: seeding loop (Radii.C:162-169), NextVisited[v] = 1<<i is a
  // plain store, so on a collision the largest i wins
  std::vector<uint32_t> all(k * (size_t)nq), adeg(k * (size_t)nq), sv, sdeg, frontier;
  std::vector<unsigned long long> sm;
  std::vector<int> sw;
  RG_TRY(lookup_ids(g, seeds_orig, (int64_t)k * nq, true, all.data(), adeg.data()));
  for (int q = 0; q < nq; q++) {
    const size_t first = sv.size();
    for (int i = 0; i < k; i++) {
      const uint32_t v = all[(size_t)q * k + i];
      auto it = std::find(sv.begin() + first, sv.end(), v);
      if (it == sv.end()) {
        sv.push_back(v);
        sm.push_back(1ull << i);
        sw.push_back(q);
        sdeg.push_back(adeg[(size_t)q * k + i]);
      } else {
        sm[it - sv.begin()] = 1ull << i;
      }
    }
  }
  // per word, the bits that can spread: samples seeded at vertices with out-edges
  std::vector<unsigned long long> full(16, 0ull);
  for (size_t j = 0; j < sv.size(); j++) full[sw[j]] |= sdeg[j] ? sm[j] : 0ull;
  frontier = sv;
  std::sort(frontier.begin(), frontier.end());
  frontier.erase(std::unique(frontier.begin(), frontier.end()), frontier.end());
  DevBuf vis(true, st), nvis(true, st), radii(true, st), seedv(true, st), seedm(true, st), seedw(true, st),
      out(true, st);
  Frontier f[2];
  RG_TRY(vis.reserve(8 * (size_t)n * W));
  RG_TRY(nvis.reserve(8 * (size_t)n * W));
  RG_TRY(radii.reserve(4 * (size_t)n * nq));
  RG_TRY(frontier_alloc(g, f[0]));
  RG_TRY(frontier_alloc(g, f[1]));
  CallTimer timer(g);
  unsigned long long* pv = vis.as<unsigned long long>();
  unsigned long long* pn = nvis.as<unsigned long long>();
  int32_t* pr = radii.as<int32_t>();
  RG_CUDA(cudaMemsetAsync(pv, 0, 8 * (size_t)n * W, st));
  RG_CUDA(cudaMemsetAsync(pn, 0, 8 * (size_t)n * W, st));
  RG_CUDA(cudaMemsetAsync(pr, 0xFF, 4 * (size_t)n * nq, st));
  if (!sv.empty()) {
    RG_TRY(seedv.reserve(4 * sv.size()));
    RG_TRY(seedm.reserve(8 * sm.size()));
    RG_TRY(seedw.reserve(4 * sw.size()));
    RG_CUDA(cudaMemcpyAsync(seedv.p, sv.data(), 4 * sv.size(), cudaMemcpyHostToDevice, st));
    RG_CUDA(cudaMemcpyAsync(seedm.p, sm.data(), 8 * sm.size(), cudaMemcpyHostToDevice, st));
    RG_CUDA(cudaMemcpyAsync(seedw.p, sw.data(), 4 * sw.size(), cudaMemcpyHostToDevice, st));
    rq_seed<<<(unsigned)((sv.size() + 255) / 256), 256, 0, st>>>(seedv.as<uint32_t>(), seedm.as<unsigned long long>(),
                                                               seedw.as<int>(), (int)sv.size(), W, n, pn, pr);
    g_timing.kernel_launches++;
  }
  RG_TRY(frontier_from_host(g, f[0], frontier.data(), (int64_t)frontier.size(), st));
  FView cur = view_of(f[0]), nxt = view_of(f[1]);
  const int64_t nwords = (n + 31) / 32;
  const int64_t threshold = g->m / std::max<int64_t>(g_opts.dense_div, 1);
  int32_t round = 0;
  while (cur.count > 0) {
    round++;
    rq_sync<<<grid_for(cur.count * W), 256, 0, st>>>(cur.queue, cur.count, W, pv, pn);
    g_timing.kernel_launches++;
    RG_CUDA(cudaMemsetAsync(nxt.bits, 0, 4 * nwords, st));
    if (cur.degsum > 0) {
      g_timing.edges_traversed += cur.degsum;
      if (cur.count + cur.degsum > threshold) {
        RG_TRY(rq_sweep(W, g, pv, pn, nxt.bits, st, full.data()));
      } else {
        RG_TRY(launch_push<OpRadiiW, kHubNone>(g, g->view(), cur, OpRadiiW{pv, pn, W}, HubInfo{}, nxt.bits, st));
      }
    }
    Frontier shell;  // non-owning view of nxt for the compaction
    shell.bits.p = nxt.bits;
    RG_TRY(compact_bits(g, shell, st, true, nullptr, 0, nullptr, nxt.queue, nxt.qoff));
    shell.bits.p = nullptr;
    nxt.count = shell.count;
    nxt.degsum = shell.degsum;
    g_timing.kernel_launches += 3;
    if (nxt.count > 0) {
      rq_mark<<<grid_for(nxt.count * W), 256, 0, st>>>(nxt.queue, nxt.count, W, nq, n, pv, pn, pr, round);
      g_timing.kernel_launches++;
    }
    RG_CUDA(cudaGetLastError());
    std::swap(cur, nxt);
  }
  RG_TRY(timer.stop());
  const int32_t* res = pr;
  if (g->sorted) {  // rows in original-id order
    RG_TRY(out.reserve(4 * (size_t)n * nq));
    for (int q = 0; q < nq; q++) {
      gather_kernel<int32_t><<<grid_for(n), 256, 0, st>>>(pr + (size_t)q * n, g->new_ids.as<uint32_t>(), n,
                                                          out.as<int32_t>() + (size_t)q * n);
    }
    RG_CUDA(cudaGetLastError());
    res = out.as<int32_t>();
  }
  if (d_radii_out) RG_CUDA(cudaMemcpyAsync(d_radii_out, res, 4 * (size_t)n * nq, cudaMemcpyDeviceToDevice, st));
  if (h_radii) RG_CUDA(cudaMemcpyAsync(h_radii, res, 4 * (size_t)n * nq, cudaMemcpyDeviceToHost, st));
  RG_CUDA(cudaStreamSynchronize(st));
  g_timing.algorithmic_bytes = (4 + 8 * W) * g_timing.edges_traversed + (int64_t)(16 * W + 4 * nq) * n;
  if (rounds_out) *rounds_out = round;
  return RG_OK;
}

}  // namespace rg

extern "C" rg_status rg_radii_multi(rg_graph* g, const uint32_t* h_seeds, int k, int nq, int32_t* h_radii,
                                    int64_t* rounds_out) {
  return rg::radii_multi_run(g, h_seeds, k, nq, h_radii, nullptr, rounds_out);
}
