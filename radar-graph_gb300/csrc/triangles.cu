// Triangle counting (GAP tc_local, src/*/GAP/src/tc_local.cc:49-157) on the
// device.
//
// The graph is relabelled by degree (descending, ties by descending id, the
// order of builder.h:247-282 and of the degree sort) with every neighbour
// list sorted ascending; a triangle is then counted once, as u > v > w: for
// every edge (u, v) with v < u, the common neighbours w < v of u and v are
// found by merging u's list before v with v's list below v (or, when one is
// far longer, by searching the short one's elements in it).  In this order
// both lists hold only higher-degree neighbours, so they stay short even on
// skewed graphs.  Per-vertex counts (triangles containing each vertex) are
// returned by original id; the counts of the H highest-degree vertices
// (ids < H) are kept per CTA in shared memory and merged once per CTA -- the
// RADAR variant's per-thread copies of triangles[u] for u < numHubs
// (tc_local.cc:54-96).

#include <cuda_runtime.h>

#include <algorithm>

#include "app_common.cuh"

namespace rg {

namespace {

// a[j] = source row of edge j, b[j] = neighbour (edge-balanced: each warp owns
// kSweepChunk consecutive edges and finds their rows from the chunk starts)
__global__ void __launch_bounds__(256) expand_entries(DevGraph g, const uint32_t* __restrict__ chunk_v,
                                                      uint32_t nchunks, uint32_t* __restrict__ a,
                                                      uint32_t* __restrict__ b) {
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t c = warp; c < nchunks; c += nwarps) {
    const uint32_t vlo = chunk_v[c], vhi = chunk_v[c + 1];
    for (int r = 0; r < kSweepChunk / 32; r++) {
      const uint32_t e = c * kSweepChunk + r * 32 + lane;
      if (e >= g.m) break;
      a[e] = upper_index(g.off, vlo, vhi, e);
      b[e] = g.adj[e];
    }
  }
}

// lower[u] = number of u's (sorted) neighbours below u
__global__ void lower_degrees(DevGraph g, uint32_t* __restrict__ lower) {
  for (int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; u < g.n; u += (int64_t)gridDim.x * blockDim.x) {
    uint32_t lo = g.off[u], hi = g.off[u + 1];
    while (lo < hi) {
      const uint32_t mid = (lo + hi) >> 1;
      if (g.adj[mid] < (uint32_t)u) lo = mid + 1;
      else hi = mid;
    }
    lower[u] = lo - g.off[u];
  }
}

template <bool kHub>
__global__ void __launch_bounds__(256) count_triangles(DevGraph g, const uint32_t* __restrict__ chunk_v,
                                                       uint32_t nchunks, const uint32_t* __restrict__ lower,
                                                       unsigned long long* tri, uint32_t H,
                                                       unsigned long long* total) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned long long* hs = reinterpret_cast<unsigned long long*>(smem_raw);
  if (kHub) {
    for (uint32_t h = threadIdx.x; h < H; h += blockDim.x) hs[h] = 0ull;
    __syncthreads();
  }
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long found = 0;
  for (uint32_t c = warp; c < nchunks; c += nwarps) {
    const uint32_t vlo = chunk_v[c], vhi = chunk_v[c + 1];
    for (int r = 0; r < kSweepChunk / 32; r++) {
      const uint32_t e = c * kSweepChunk + r * 32 + lane;
      if (e >= g.m) break;
      const uint32_t u = upper_index(g.off, vlo, vhi, e);
      const uint32_t v = g.adj[e];
      if (v >= u) continue;  // each triangle once: u > v > w
      // u's neighbours before v (all < v) against v's neighbours below v:
      // merged, unless one list is far longer -- then each element of the
      // short one is searched in the long one (min * log(max) steps)
      uint32_t sa = g.off[u], ea = e, sb = g.off[v], eb = g.off[v] + lower[v];
      if (ea - sa > eb - sb) {
        const uint32_t t0 = sa, t1 = ea;
        sa = sb;
        ea = eb;
        sb = t0;
        eb = t1;
      }
      uint32_t cnt = 0;
      if (eb - sb > 16 * (ea - sa)) {
        uint32_t lo = sb;  // the short list ascends: each search starts past the last one
        for (uint32_t i = sa; i < ea && lo < eb; i++) {
          const uint32_t x = g.adj[i];
          uint32_t hi = eb;
          while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (g.adj[mid] < x) lo = mid + 1;
            else hi = mid;
          }
          if (lo < eb && g.adj[lo] == x) {
            cnt++;
            if (kHub && x < H) atomicAdd(hs + x, 1ull);
            else atomicAdd(tri + x, 1ull);
            lo++;
          }
        }
      } else {
        uint32_t ia = sa, ib = sb;
        while (ia < ea && ib < eb) {
          const uint32_t x = g.adj[ia], y = g.adj[ib];
          if (x == y) {
            cnt++;
            if (kHub && x < H) atomicAdd(hs + x, 1ull);
            else atomicAdd(tri + x, 1ull);
            ia++;
            ib++;
          } else if (x < y) {
            ia++;
          } else {
            ib++;
          }
        }
      }
      if (cnt) {
        if (kHub && u < H) atomicAdd(hs + u, (unsigned long long)cnt);
        else atomicAdd(tri + u, (unsigned long long)cnt);
        if (kHub && v < H) atomicAdd(hs + v, (unsigned long long)cnt);
        else atomicAdd(tri + v, (unsigned long long)cnt);
        found += cnt;
      }
    }
  }
  found = warp_sum(found);
  if (lane == 0 && found) atomicAdd(total, found);
  if (kHub) {
    __syncthreads();
    for (uint32_t h = threadIdx.x; h < H; h += blockDim.x) {
      if (hs[h]) atomicAdd(tri + h, hs[h]);
    }
  }
}

struct TcState {
  DevBuf a, b, lower, tri, total, out;
};

}  // namespace

rg_status triangle_run(rg_graph* g, uint64_t* h_counts, uint64_t* total_out) {
  if (!g) return fail(RG_EINVAL, "null graph");
  if (g->directed) return fail(RG_EUNSUPPORTED, "triangle counting needs an undirected graph (tc_local.cc:21-25)");
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  cudaStream_t st = cx->stream;
  const int64_t n = g->n, m = g->m;
  static thread_local TcState S;
  CallTimer timer(g);
  // degree order (the relabelled graph of the sort, or g itself when sorted)
  rg_graph* rs = g;
  rg_graph* tmp = nullptr;
  if (!g->sorted) {
    RG_TRY(rg_graph_degree_sort(g, &tmp, nullptr));
    rs = tmp;
  }
  // neighbour lists sorted: the device CSR builder over rs's entries (every
  // entry appears twice after symmetrising; the repeats are dropped)
  rg_graph* gt = nullptr;
  rg_status s = RG_OK;
  if (m > 0) {
    s = S.a.reserve(4 * (size_t)m);
    if (s == RG_OK) s = S.b.reserve(4 * (size_t)m);
    if (s == RG_OK) {
      const int64_t blocks = std::min<int64_t>((rs->nchunks * 32 + 255) / 256, (int64_t)device_sms() * 8);
      expand_entries<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, st>>>(
          rs->view(), rs->chunk_v.as<uint32_t>(), (uint32_t)rs->nchunks, S.a.as<uint32_t>(), S.b.as<uint32_t>());
      const cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) s = cuda_fail(e, "expand_entries", __FILE__, __LINE__);
    }
    if (s == RG_OK) s = rg_graph_create_from_edges(n, m, S.a.as<uint32_t>(), S.b.as<uint32_t>(), 1, &gt);
  } else {
    s = rg_graph_create_from_edges(n, 0, nullptr, nullptr, 1, &gt);
  }
  if (s != RG_OK) {
    if (tmp) rg_graph_free(tmp);
    return s;
  }
  auto cleanup = [&]() {
    rg_graph_free(gt);
    if (tmp) rg_graph_free(tmp);
  };
  if ((s = S.lower.reserve(4 * (size_t)n)) != RG_OK || (s = S.tri.reserve(8 * (size_t)n)) != RG_OK ||
      (s = S.total.reserve(8)) != RG_OK || (s = S.out.reserve(8 * (size_t)n)) != RG_OK) {
    cleanup();
    return s;
  }
  unsigned long long* tri = S.tri.as<unsigned long long>();
  unsigned long long* total = S.total.as<unsigned long long>();
  cudaError_t e = cudaMemsetAsync(tri, 0, 8 * n, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(total, 0, 8, st);
  if (e == cudaSuccess && gt->m > 0) {
    const int vblocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)device_sms() * 16);
    lower_degrees<<<vblocks, 256, 0, st>>>(gt->view(), S.lower.as<uint32_t>());
    // hub counters: as many of the first ids as a CTA's shared memory holds
    const bool hubs = g_opts.hub_smem_kb > 0;
    const uint32_t H = hubs ? (uint32_t)std::min<int64_t>(n, g_opts.hub_smem_kb * 1024 / 8) : 0;
    auto kern = hubs ? count_triangles<true> : count_triangles<false>;
    const size_t dyn = 8 * (size_t)H;
    static std::atomic<uint64_t> limit_set[2];  // count_triangles<false>, <true>
    e = allow_max_dyn_smem(limit_set[hubs ? 1 : 0], kern) == RG_OK ? cudaSuccess : cudaErrorInvalidValue;
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, dyn);
    const int64_t grid = std::min<int64_t>((gt->nchunks * 32 + 255) / 256, (int64_t)device_sms() * std::max(per_sm, 1));
    if (e == cudaSuccess) {
      kt_begin(st);
      kern<<<(unsigned)std::max<int64_t>(grid, 1), 256, dyn, st>>>(gt->view(), gt->chunk_v.as<uint32_t>(),
                                                                    (uint32_t)gt->nchunks, S.lower.as<uint32_t>(),
                                                                    tri, H, total);
      kt_end(st);
      e = cudaGetLastError();
      g_timing.kernel_launches += 2;
      g_timing.edge_launches++;
    }
  }
  uint64_t t = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&t, total, 8, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && h_counts) {  // by original id: rs's permutation maps g's ids to gt's
    const int64_t blocks = std::min<int64_t>((n + 255) / 256, (int64_t)device_sms() * 32);
    gather_kernel<unsigned long long><<<(unsigned)blocks, 256, 0, st>>>(
        tri, (g->sorted ? g : rs)->new_ids.as<uint32_t>(), n, S.out.as<unsigned long long>());
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_counts, S.out.p, 8 * n, cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cleanup();
  if (e != cudaSuccess) return cuda_fail(e, "triangle count", __FILE__, __LINE__);
  RG_TRY(timer.stop());
  g_timing.edges_traversed = m;
  if (total_out) *total_out = t;
  return RG_OK;
}

}  // namespace rg

extern "C" rg_status rg_triangle_count(rg_graph* g, uint64_t* h_counts, uint64_t* total_out) {
  return rg::triangle_run(g, h_counts, total_out);
}
