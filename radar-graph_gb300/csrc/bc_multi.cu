// Multi-source betweenness centrality: up to 64 independent single-source BC
// queries on one graph in one traversal.  The reference runs one source per
// Brandes pass (src/push-new-orig/Ligra/apps/BC-manyiter-v2.C:180-232); row q
// of this result equals that pass from sources[q] alone (rg_bc_sources with
// one source) up to floating-point summation order.
//
// Levels: one 64-wide bitmask BFS (OpMsBfs, bit q = source q) gives every
// level's queue and, per queued vertex, the mask of the sources for which it
// sits at that level.  Queues and masks are kept for the backward pass.
//
// Rows: per vertex kk = k rounded up to 4 columns of path counts sigma (u64:
// path counts are integers, summed exactly) and of dependencies D (double).
// Both passes push along the DAG edges of every source, one reduction in L2
// per (edge, source):
//   forward,  level r -> r+1: sigma[v][q] += sigma[u][q]   (BC_F :32-56)
//   backward, level r+1 -> r: D[v][q] += D[w][q], after D[v][q] = 1/sigma
//                             (BC_Back_F :58-80, BC_Back_Vertex_F :93-102)
//   result:   (D - 1/sigma) / (1/sigma), NaN where source q never reached the
//             vertex (:229-232)
// The adds run in the L2 atomic units, not in the SMs, whose FP64 issue rate
// on GB300 is one warp-instruction per 16 clocks.  Path counts are bounded
// before they are trusted: if the largest count pushed times the largest
// in-degree could pass 2^64, the call answers with one single-source pass per
// source instead.

#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <vector>

#include "app_common.cuh"

namespace rg {
namespace {

__global__ void mb_seed(const uint32_t* __restrict__ src, int k, int kk, unsigned long long* F,
                        unsigned long long* seen, unsigned long long* sig) {
  const int q = threadIdx.x;
  if (q < k) {
    const uint32_t s = src[q];
    atomicOr(F + s, 1ull << q);
    atomicOr(seen + s, 1ull << q);
    sig[(size_t)s * kk + q] = 1ull;
  }
}

// LM[j] = the sources whose level this is for queue[j]: level 0 reads F, a
// later level the bits that arrived (N & ~seen).
__global__ void mb_capture(const uint32_t* __restrict__ q, int64_t count, const unsigned long long* __restrict__ a,
                           const unsigned long long* __restrict__ not_b, unsigned long long* __restrict__ LM) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < count) {
    const uint32_t v = q[j];
    LM[j] = a[v] & (not_b ? ~not_b[v] : ~0ull);
  }
}

__global__ void mb_clear(const uint32_t* __restrict__ q, int64_t count, unsigned long long* a) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < count) a[q[j]] = 0ull;
}

__global__ void mb_scatter(const uint32_t* __restrict__ q, int64_t count, const unsigned long long* __restrict__ LM,
                           unsigned long long* a) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < count) a[q[j]] = LM[j];
}

// The level's bits become the frontier and join seen; N is cleared for them.
__global__ void mb_advance(const uint32_t* __restrict__ q, int64_t count, const unsigned long long* __restrict__ LM,
                           unsigned long long* N, unsigned long long* F, unsigned long long* seen) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < count) {
    const uint32_t v = q[j];
    N[v] = 0ull;
    F[v] = LM[j];
    seen[v] |= LM[j];
  }
}

// 1/s for a path count s >= 1, without FP64 arithmetic in the SMs but the
// final conversion: s as hi + lo floats (its top 24 bits and the next 24,
// each exact), the single-precision reciprocal r of hi, one Newton-Raphson
// step r' = r + r e with e = 1 - s r evaluated in float-float (hi*r split
// exactly by an FMA; 1 - p is exact for p near 1), then hi' + lo' in double.
// Relative error ~2^-46; deterministic, so the seed of D and the final
// transform see the same bits.
__device__ __forceinline__ double inv_count(unsigned long long s) {
  const int nb = 64 - __clzll((long long)s);
  const int sh = max(nb - 24, 0);
  const unsigned top = (unsigned)(s >> sh);
  const unsigned long long rem = s - ((unsigned long long)top << sh);
  const int sh2 = max(sh - 24, 0);
  const unsigned nxt = (unsigned)(rem >> sh2);
  const float hi = (float)top * __int_as_float((127 + sh) << 23);
  const float lo = (float)nxt * __int_as_float((127 + sh2) << 23);
  const float r = __frcp_rn(hi);
  const float p = hi * r;
  const float pe = fmaf(hi, r, -p);
  const float e = ((1.0f - p) - pe) - lo * r;
  const float c = r * e;
  const float h = r + c;
  return (double)h + (double)(c - (h - r));
}

// BC_Back_Vertex_F for a level: D[v][q] = 1/sigma[v][q] for its sources (the
// level above then pushes its dependencies into them).  One thread per
// (entry, column).
__global__ void mb_back_seed(const uint32_t* __restrict__ q, int64_t count, const unsigned long long* __restrict__ LM,
                             const unsigned long long* __restrict__ sig, double* __restrict__ D, int kk) {
  const int64_t total = count * kk;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = i / kk;
    const int c = (int)(i - j * kk);
    if (!((LM[j] >> c) & 1)) continue;
    const size_t e = (size_t)q[j] * kk + c;
    D[e] = inv_count(sig[e]);
  }
}

constexpr int kPushTile = 512;  // edges per warp task
constexpr int kStage = 4;       // edges per lane per round
constexpr unsigned kFull = 0xffffffffu;

// Push one level of either pass along g: for every queued vertex u (mask m =
// its sources at this level) and every neighbour x, each source q in
// m & lmask[x] adds u's value to x's, rows[x][q] += rows[u][q], as one
// reduction in L2: exact 64-bit integer adds for path counts, IEEE double
// adds for dependencies.  The values read (this level) and the values written
// (the next level: deeper in the forward pass, shallower in the backward
// pass) are disjoint entries.
//
// A warp walks a tile of kPushTile edges of the queue's degree scan (qoff)
// 128 at a time: lane l stages queue entry jc + l (start offset, vertex,
// mask, adjacency base), every lane finds the entries owning its four edges
// by a shuffle search over those starts and loads the four neighbours and
// their masks.  Narrow rows (kCols false): each lane then walks its four
// edges' sources together, two of each per step, so eight row loads are in
// flight per lane.  Wide rows (kCols true): the edges with work are taken
// four at a time by the whole warp, lane l moving columns l and l + 32, so
// one reduction instruction covers consecutive entries of a row, which L1
// merges into sector-sized requests to L2.
// Forward: the largest value pushed goes to *vmax (the overflow bound).
template <class T, bool kCols>
__global__ void __launch_bounds__(256) rows_push(DevGraph g, const uint32_t* __restrict__ queue,
                                                 const uint32_t* __restrict__ qoff,
                                                 const unsigned long long* __restrict__ qmask, uint32_t count,
                                                 uint32_t degsum, const uint32_t* __restrict__ tstart,
                                                 const unsigned long long* __restrict__ lmask, T* rows, int kk,
                                                 unsigned long long* vmax) {
  const int lane = threadIdx.x & 31;
  const uint32_t ntiles = (degsum + kPushTile - 1) / kPushTile;
  unsigned long long mx = 0ull;
  for (uint32_t t = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < ntiles;
       t += (gridDim.x * blockDim.x) >> 5) {
    const uint32_t e0 = t * kPushTile, e1 = min(e0 + kPushTile, degsum);
    uint32_t jc = tstart[t];  // the entry holding edge e0
    for (uint32_t eb = e0; eb < e1;) {
      // stage entries jc .. jc+31 (starts ascend; past the queue they read as +inf)
      const uint32_t js = jc + lane;
      uint32_t s = 0xFFFFFFFFu, v = 0, base = 0;
      unsigned long long m = 0ull;
      if (js <= count) s = qoff[js];
      if (js < count) {
        v = queue[js];
        m = qmask[js];
        base = g.off[v];
      }
      uint32_t end = __shfl_down_sync(kFull, s, 1);
      if (lane == 31) end = (jc + 32 <= count) ? qoff[jc + 32] : 0xFFFFFFFFu;
      const uint32_t stop = min(min(eb + 32 * kStage, e1), __shfl_sync(kFull, end, 31));
      uint32_t x[kStage], u[kStage];
      unsigned long long b[kStage];
#pragma unroll
      for (int i = 0; i < kStage; i++) {
        // owner of edge e: the largest staged p with start <= e (start 0 is <= eb)
        const uint32_t e = eb + 32 * i + lane;
        int p = 0;
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
          if (__shfl_sync(kFull, s, p + step) <= e) p += step;
        }
        const uint32_t ps = __shfl_sync(kFull, s, p), pb = __shfl_sync(kFull, base, p);
        u[i] = __shfl_sync(kFull, v, p);
        b[i] = __shfl_sync(kFull, m, p);
        x[i] = e < stop ? g.adj[pb + (e - ps)] : 0u;
        if (e >= stop) b[i] = 0ull;
      }
#pragma unroll
      for (int i = 0; i < kStage; i++) {
        if (b[i]) b[i] &= lmask[x[i]];
      }
      if constexpr (kCols) {
#pragma unroll
        for (int i = 0; i < kStage; i++) {
          unsigned act = __ballot_sync(kFull, b[i] != 0ull);
          while (act) {
            uint32_t xs[4], us[4];
            unsigned long long bs[4];
#pragma unroll
            for (int w = 0; w < 4; w++) {
              const bool ok = act != 0u;
              const int sl = ok ? __ffs(act) - 1 : 0;
              act &= act - 1u;
              xs[w] = __shfl_sync(kFull, x[i], sl);
              us[w] = __shfl_sync(kFull, u[i], sl);
              const unsigned long long bb = __shfl_sync(kFull, b[i], sl);
              bs[w] = ok ? bb : 0ull;
            }
            T v0[4], v1[4];
#pragma unroll
            for (int w = 0; w < 4; w++) {
              const T* row = rows + (size_t)us[w] * kk;
              v0[w] = ((bs[w] >> lane) & 1) ? row[lane] : T(0);
              v1[w] = ((bs[w] >> (lane + 32)) & 1) ? row[lane + 32] : T(0);
            }
#pragma unroll
            for (int w = 0; w < 4; w++) {
              T* row = rows + (size_t)xs[w] * kk;
              if ((bs[w] >> lane) & 1) atomicAdd(row + lane, v0[w]);
              if ((bs[w] >> (lane + 32)) & 1) atomicAdd(row + lane + 32, v1[w]);
              if constexpr (std::is_same<T, unsigned long long>::value) mx = max(mx, max(v0[w], v1[w]));
            }
          }
        }
        b[0] = b[1] = b[2] = b[3] = 0ull;
      }
      while (b[0] | b[1] | b[2] | b[3]) {
        int q[2 * kStage];
        T val[2 * kStage];
#pragma unroll
        for (int i = 0; i < 2 * kStage; i++) {
          unsigned long long& bi = b[i % kStage];
          q[i] = -1;
          if (bi) {
            q[i] = __ffsll((long long)bi) - 1;
            bi &= bi - 1;
            val[i] = rows[(size_t)u[i % kStage] * kk + q[i]];
          }
        }
#pragma unroll
        for (int i = 0; i < 2 * kStage; i++) {
          if (q[i] >= 0) {
            atomicAdd(rows + (size_t)x[i % kStage] * kk + q[i], val[i]);
            if constexpr (std::is_same<T, unsigned long long>::value) mx = max(mx, val[i]);
          }
        }
      }
      // the next round starts at the entry holding edge `stop`
      int nq = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        if (__shfl_sync(kFull, s, nq + step) <= stop) nq += step;
      }
      jc += (uint32_t)nq;
      eb = stop;
    }
  }
  if constexpr (std::is_same<T, unsigned long long>::value) {
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(kFull, mx, o));
    if (lane == 0 && mx) atomicMax(vmax, mx);
  }
}

// out[q*n + o] for original id o: (D - 1/sigma) / (1/sigma) (as
// (D - 1/sigma) * sigma: exactly 0 for a vertex with no successors), NaN
// where sigma = 0 (the source never reached the vertex).  A block takes 32
// consecutive original ids: their rows are read whole into shared memory,
// then each source's 32 results are written as one contiguous segment.
constexpr int kFinalIds = 32;
__global__ void __launch_bounds__(256) mb_final(const unsigned long long* __restrict__ sig,
                                                const double* __restrict__ D, int kk, int k, int64_t n,
                                                const uint32_t* __restrict__ new_ids, double* __restrict__ out) {
  __shared__ double res[kFinalIds][64 + 1];
  const int64_t ntiles = (n + kFinalIds - 1) / kFinalIds;
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t o0 = t * kFinalIds;
    for (int i = threadIdx.x; i < kFinalIds * kk; i += blockDim.x) {
      const int j = i / kk, q = i - j * kk;
      const int64_t o = o0 + j;
      if (o >= n || q >= k) continue;
      const uint32_t v = new_ids ? new_ids[o] : (uint32_t)o;
      const size_t e = (size_t)v * kk + q;
      const unsigned long long s = sig[e];
      double r = __longlong_as_double(0x7ff8000000000000ll);
      if (s) r = (D[e] - inv_count(s)) * (double)s;
      res[j][q] = r;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kFinalIds * k; i += blockDim.x) {
      const int q = i / kFinalIds, j = i - q * kFinalIds;
      const int64_t o = o0 + j;
      if (o < n) out[(int64_t)q * n + o] = res[j][q];
    }
    __syncthreads();
  }
}

__global__ void mb_max_degree(const uint32_t* __restrict__ off, int64_t n, unsigned int* out) {
  unsigned int mx = 0;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    mx = max(mx, off[v + 1] - off[v]);
  }
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(kFull, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, mx);
}

inline unsigned blocks_for(int64_t items, int per_block = 256) {
  return (unsigned)std::max<int64_t>(1, (items + per_block - 1) / per_block);
}

template <class T, bool kCols>
rg_status launch_push_as(const DevGraph& dg, const uint32_t* queue, const uint32_t* qoff,
                      const unsigned long long* qmask, int64_t count, int64_t degsum,
                      const unsigned long long* lmask, T* rows, int kk, unsigned long long* vmax, DevBuf& ts,
                      cudaStream_t st) {
  if (count <= 0 || degsum <= 0) return RG_OK;
  const int64_t tiles = (degsum + kPushTile - 1) / kPushTile;
  RG_TRY(ts.reserve(4 * (size_t)(tiles + 2)));
  tile_starts<<<(unsigned)((tiles + 1 + 255) / 256), 256, 0, st>>>(qoff, (uint32_t)count, (uint32_t)degsum,
                                                                    kPushTile, (uint32_t)tiles, ts.as<uint32_t>());
  const int64_t blocks = std::min<int64_t>((tiles + 7) / 8, (int64_t)device_sms() * 8);
  kt_begin(st);
  rows_push<T, kCols><<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, st>>>(
      dg, queue, qoff, qmask, (uint32_t)count, (uint32_t)degsum, ts.as<uint32_t>(), lmask, rows, kk, vmax);
  kt_end(st);
  RG_CUDA(cudaGetLastError());
  g_timing.kernel_launches += 2;
  g_timing.edge_launches++;
  g_timing.edges_traversed += degsum;
  return RG_OK;
}

// Rows of 16 or more columns move a row per warp (kCols); narrower rows, a
// source per lane.
template <class T>
rg_status launch_push(const DevGraph& dg, const uint32_t* queue, const uint32_t* qoff,
                      const unsigned long long* qmask, int64_t count, int64_t degsum,
                      const unsigned long long* lmask, T* rows, int kk, unsigned long long* vmax, DevBuf& ts,
                      cudaStream_t st) {
  if (kk >= 16) return launch_push_as<T, true>(dg, queue, qoff, qmask, count, degsum, lmask, rows, kk, vmax, ts, st);
  return launch_push_as<T, false>(dg, queue, qoff, qmask, count, degsum, lmask, rows, kk, vmax, ts, st);
}

// Level storage (queues, degree scans, masks of every level), grown by copy.
struct Levels {
  DevBuf q, qo, lm;
  int64_t cap = 0;
  explicit Levels(cudaStream_t st) : q(true, st), qo(true, st), lm(true, st) {}
  rg_status ensure(int64_t need, int64_t used, int64_t qo_used, cudaStream_t st) {
    if (need <= cap) return RG_OK;
    const int64_t ncap = std::max<int64_t>(need, cap + cap / 2);
    DevBuf q2(true, st), qo2(true, st), lm2(true, st);
    RG_TRY(q2.reserve(4 * (size_t)ncap));
    RG_TRY(qo2.reserve(4 * (size_t)(2 * ncap + 2)));
    RG_TRY(lm2.reserve(8 * (size_t)ncap));
    if (used > 0) {
      RG_CUDA(cudaMemcpyAsync(q2.p, q.p, 4 * (size_t)used, cudaMemcpyDeviceToDevice, st));
      RG_CUDA(cudaMemcpyAsync(lm2.p, lm.p, 8 * (size_t)used, cudaMemcpyDeviceToDevice, st));
    }
    if (qo_used > 0) RG_CUDA(cudaMemcpyAsync(qo2.p, qo.p, 4 * (size_t)qo_used, cudaMemcpyDeviceToDevice, st));
    std::swap(q.p, q2.p);
    std::swap(q.bytes, q2.bytes);
    std::swap(qo.p, qo2.p);
    std::swap(qo.bytes, qo2.bytes);
    std::swap(lm.p, lm2.p);
    std::swap(lm.bytes, lm2.bytes);
    cap = ncap;
    return RG_OK;
  }
};

}  // namespace

rg_status bc_multi_run(rg_graph* g, const uint32_t* src_orig, int k, double* h_out, double* d_out,
                       int64_t* levels_out) {
  if (!g) return fail(RG_EINVAL, "null graph");
  if (k < 1 || k > 64 || !src_orig) return fail(RG_EINVAL, "need 1..64 sources");
  for (int q = 0; q < k; q++) {
    if (src_orig[q] >= (uint64_t)g->n) return fail(RG_EINVAL, "source %u >= n", src_orig[q]);
  }
  if (g->m >= 0xFFFFFFFFll) return fail(RG_EUNSUPPORTED, ">= 2^32 edges");
  OptScope opt_scope(g, kAppBfs);  // the level discovery is a multi-source BFS
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  cudaStream_t st = cx->stream;
  const int64_t n = g->n;
  const int64_t nwords = (n + 31) / 32;
  const int kk = (k + 3) & ~3;
  const size_t cells = (size_t)n * kk;
  DevBuf F(true, st), N(true, st), seen(true, st), M(true, st), sig(true, st), D(true, st), src(true, st),
      info(true, st), inq(true, st), qdeg(true, st), bits0(true, st), bits1(true, st), res(true, st), tsb(true, st);
  RG_TRY(F.reserve(8 * n));
  RG_TRY(N.reserve(8 * n));
  RG_TRY(seen.reserve(8 * n));
  RG_TRY(M.reserve(8 * n));
  RG_TRY(sig.reserve(8 * cells));
  RG_TRY(D.reserve(8 * cells));
  RG_TRY(src.reserve(4 * 64));
  RG_TRY(info.reserve(16));
  RG_TRY(bits0.reserve(4 * (nwords + 8)));
  RG_TRY(bits1.reserve(4 * (nwords + 8)));
  if (g->directed) RG_TRY(inq.reserve(4 * (n + 66)));
  Levels L(st);
  RG_TRY(L.ensure(2 * n + 64, 0, 0, st));
  std::vector<uint32_t> s_int(k), s_deg(k), uniq;
  RG_TRY(lookup_ids(g, src_orig, k, true, s_int.data(), s_deg.data()));
  unsigned long long full = 0ull;  // the bits that can spread: sources with out-edges
  for (int q = 0; q < k; q++) full |= s_deg[q] ? (1ull << q) : 0ull;
  for (int q = 0; q < k; q++) {
    if (std::find(uniq.begin(), uniq.end(), s_int[q]) == uniq.end()) uniq.push_back(s_int[q]);
  }
  std::sort(uniq.begin(), uniq.end());
  std::vector<uint32_t> deg(uniq.size());
  RG_TRY(lookup_ids(g, uniq.data(), (int64_t)uniq.size(), false, nullptr, deg.data()));
  std::vector<uint32_t> qo0(uniq.size() + 1, 0);
  for (size_t j = 0; j < uniq.size(); j++) qo0[j + 1] = qo0[j] + deg[j];

  CallTimer timer(g);
  unsigned long long *pF = F.as<unsigned long long>(), *pN = N.as<unsigned long long>(),
                     *pS = seen.as<unsigned long long>(), *pM = M.as<unsigned long long>(),
                     *pSig = sig.as<unsigned long long>();
  double* pD = D.as<double>();
  unsigned long long* vmax = info.as<unsigned long long>();  // [0] largest count pushed, [1] largest in-degree
  RG_CUDA(cudaMemsetAsync(pF, 0, 8 * n, st));
  RG_CUDA(cudaMemsetAsync(pN, 0, 8 * n, st));
  RG_CUDA(cudaMemsetAsync(pS, 0, 8 * n, st));
  RG_CUDA(cudaMemsetAsync(pM, 0, 8 * n, st));
  RG_CUDA(cudaMemsetAsync(pSig, 0, 8 * cells, st));
  RG_CUDA(cudaMemsetAsync(vmax, 0, 16, st));
  RG_CUDA(cudaMemsetAsync(bits0.p, 0, 4 * nwords, st));
  RG_CUDA(cudaMemcpyAsync(src.p, s_int.data(), 4 * k, cudaMemcpyHostToDevice, st));
  RG_CUDA(cudaMemcpyAsync(L.q.p, uniq.data(), 4 * uniq.size(), cudaMemcpyHostToDevice, st));
  RG_CUDA(cudaMemcpyAsync(L.qo.p, qo0.data(), 4 * qo0.size(), cudaMemcpyHostToDevice, st));
  mb_seed<<<1, 64, 0, st>>>(src.as<uint32_t>(), k, kk, pF, pS, pSig);
  mb_capture<<<blocks_for((int64_t)uniq.size()), 256, 0, st>>>(L.q.as<uint32_t>(), (int64_t)uniq.size(), pF,
                                                                nullptr, L.lm.as<unsigned long long>());
  {
    const DevGraph ig = g->in_view();
    const int64_t mb = std::min<int64_t>((n + 255) / 256, (int64_t)device_sms() * 8);
    mb_max_degree<<<(unsigned)std::max<int64_t>(mb, 1), 256, 0, st>>>(ig.off, n, (unsigned int*)(vmax + 1));
  }
  g_timing.kernel_launches += 3;
  RG_CUDA(cudaStreamSynchronize(st));  // the host vectors above are staged
  // level r: entries [lstart[r], lstart[r] + lcount[r]) of L.q / L.lm, its
  // out-degree scan at L.qo + lstart[r] + r
  std::vector<int64_t> lstart{0}, lcount{(int64_t)uniq.size()}, ldeg{(int64_t)qo0.back()};
  int64_t qpos = (int64_t)uniq.size();
  uint32_t* cur_bits = bits0.as<uint32_t>();
  uint32_t* nxt_bits = bits1.as<uint32_t>();
  EmOpts o;
  o.variant = RG_PUSH;
  const int64_t threshold = g->m / std::max<int64_t>(g_opts.dense_div, 1);
  for (int64_t r = 0;; r++) {
    RG_TRY(L.ensure(qpos + n + 64, qpos, qpos + r + 1, st));
    uint32_t* LQ = L.q.as<uint32_t>();
    uint32_t* LQO = L.qo.as<uint32_t>();
    unsigned long long* LM = L.lm.as<unsigned long long>();
    FView cur{LQ + lstart[r], LQO + lstart[r] + r, cur_bits, lcount[r], ldeg[r]};
    FView nxt{LQ + qpos, LQO + qpos + r + 1, nxt_bits, 0, 0};
    // discovery: the bits that reach each vertex first at level r+1 go to N
    // (the 64-wide BFS of rg_bfs_multi)
    if (cur.count + cur.degsum > threshold && cur.degsum > 0) {
      RG_CUDA(cudaMemsetAsync(nxt.bits, 0, 4 * nwords, st));
      g_timing.edges_traversed += cur.degsum;
      RG_TRY(launch_mask_sweep(g, pS, pN, nxt.bits, st, full));
      Frontier shell;
      shell.bits.p = nxt.bits;
      RG_TRY(compact_bits(g, shell, st, true, nullptr, 0, nullptr, nxt.queue, nxt.qoff));
      shell.bits.p = nullptr;
      nxt.count = shell.count;
      nxt.degsum = shell.degsum;
      g_timing.kernel_launches += 3;
    } else {
      RG_TRY(edge_map(g, cur, OpMsBfs{pF, pS, pN}, &nxt, o, st));
    }
    if (nxt.count == 0) break;
    mb_capture<<<blocks_for(nxt.count), 256, 0, st>>>(nxt.queue, nxt.count, pN, pS, LM + qpos);
    g_timing.kernel_launches++;
    // sigma of level r+1: every DAG edge u -> v pushes sigma[u][q]
    RG_TRY(launch_push<unsigned long long>(g->view(), cur.queue, cur.qoff, LM + lstart[r], cur.count, cur.degsum, pN,
                                           pSig, kk, vmax, tsb, st));
    mb_clear<<<blocks_for(cur.count), 256, 0, st>>>(cur.queue, cur.count, pF);
    mb_advance<<<blocks_for(nxt.count), 256, 0, st>>>(nxt.queue, nxt.count, LM + qpos, pN, pF, pS);
    g_timing.kernel_launches += 2;
    RG_CUDA(cudaGetLastError());
    lstart.push_back(qpos);
    lcount.push_back(nxt.count);
    ldeg.push_back(nxt.degsum);
    qpos += nxt.count;
    std::swap(cur_bits, nxt_bits);
  }
  const int64_t R = (int64_t)lstart.size();  // levels 0..R-1
  // backward: every level is seeded with 1/sigma, then the level below it
  // (one step deeper) pushes its dependencies up along the DAG edges
  uint32_t* LQ = L.q.as<uint32_t>();
  uint32_t* LQO = L.qo.as<uint32_t>();
  unsigned long long* LM = L.lm.as<unsigned long long>();
  auto seed = [&](int64_t r) {
    const int64_t sb = std::min<int64_t>((lcount[r] * kk + 255) / 256, (int64_t)device_sms() * 32);
    mb_back_seed<<<(unsigned)std::max<int64_t>(sb, 1), 256, 0, st>>>(LQ + lstart[r], lcount[r], LM + lstart[r], pSig,
                                                                      pD, kk);
    g_timing.kernel_launches++;
  };
  seed(R - 1);
  for (int64_t r = R - 2; r >= 0; r--) {
    seed(r);
    mb_scatter<<<blocks_for(lcount[r]), 256, 0, st>>>(LQ + lstart[r], lcount[r], LM + lstart[r], pM);
    uint32_t* wq = LQ + lstart[r + 1];
    const uint32_t* w_qoff = LQO + lstart[r + 1] + r + 1;  // out-degrees = in-degrees when symmetric
    int64_t w_deg = ldeg[r + 1];
    if (g->directed) {  // the level's in-degrees: its predecessors lie on in-edges
      RG_TRY(requeue_degrees(g, wq, lcount[r + 1], g->in_off.as<uint32_t>(), inq.as<uint32_t>(), &w_deg, qdeg, st));
      w_qoff = inq.as<uint32_t>();
    }
    RG_TRY(launch_push<double>(g->in_view(), wq, w_qoff, LM + lstart[r + 1], lcount[r + 1], w_deg, pM, pD, kk,
                               nullptr, tsb, st));
    mb_clear<<<blocks_for(lcount[r]), 256, 0, st>>>(LQ + lstart[r], lcount[r], pM);
    g_timing.kernel_launches += 2;
    RG_CUDA(cudaGetLastError());
  }
  unsigned long long h_info[2] = {0, 0};
  RG_CUDA(cudaMemcpyAsync(h_info, vmax, 16, cudaMemcpyDeviceToHost, st));
  RG_CUDA(cudaStreamSynchronize(st));
  // no count can have wrapped if the largest pushed count times the largest
  // in-degree stays below 2^64 (a count is a sum of at most in-degree terms)
  const unsigned long long max_in = (unsigned int)h_info[1];
  const bool overflow = max_in > 0 && h_info[0] > ~0ull / max_in;
  double* result = d_out;
  if (!result) {
    RG_TRY(res.reserve(8 * (size_t)n * k));
    result = res.as<double>();
  }
  if (!overflow) {
    const int64_t blocks = std::min<int64_t>((n + kFinalIds - 1) / kFinalIds, (int64_t)device_sms() * 8);
    mb_final<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, st>>>(
        pSig, pD, kk, k, n, g->sorted ? g->new_ids.as<uint32_t>() : nullptr, result);
    RG_CUDA(cudaGetLastError());
    g_timing.kernel_launches++;
  }
  RG_TRY(timer.stop());
  if (overflow) {  // one single-source pass per source (timed by those calls)
    for (int q = 0; q < k; q++) RG_TRY(bc_run(g, RG_PUSH, &src_orig[q], 1, nullptr, nullptr, 0, result + q * n));
  }
  if (h_out) RG_CUDA(cudaMemcpyAsync(h_out, result, 8 * (size_t)n * k, cudaMemcpyDeviceToHost, st));
  RG_CUDA(cudaStreamSynchronize(st));
  g_timing.algorithmic_bytes = 4 * g_timing.edges_traversed + (int64_t)k * 16 * n + 24 * n;
  if (levels_out) *levels_out = R - 1;
  return RG_OK;
}

}  // namespace rg

extern "C" rg_status rg_bc_multi(rg_graph* g, const uint32_t* h_sources, int k, double* h_deps,
                                 int64_t* levels_out) {
  return rg::bc_multi_run(g, h_sources, k, h_deps, nullptr, levels_out);
}
