// App drivers (Compute of PageRank.C, BFS.C, BC-manyiter-v2.C, Radii.C) on
// the device engine, and the engine-level C ABI (rg_edgemap/rg_vertexmap).
//
// Every app keeps its arrays resident in HBM for the whole call, reads back
// only the per-level frontier size (one 16-byte copy per level, the same
// information the reference's edgeMapData gathers to choose a mode), and
// copies the result to the host once at the end.

#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <functional>
#include <mutex>
#include <random>
#include <vector>

#include "app_common.cuh"
#include "engine.cuh"
#include "rg_device.cuh"

namespace rg {

// ---------------------------------------------------------------------------
// per-call timing and launch accounting
// ---------------------------------------------------------------------------
thread_local rg_timing g_timing;
bool g_kernel_timing = false;
thread_local bool g_trace_on = false;
thread_local std::vector<rg_level_trace> g_trace;
thread_local std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_kt_events;
thread_local size_t g_kt_used = 0;

void kt_begin(cudaStream_t st) {
  if (!g_kernel_timing) return;
  if (g_kt_used == g_kt_events.size()) {
    cudaEvent_t a, b;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) return;
    g_kt_events.push_back({a, b});
  }
  cudaEventRecord(g_kt_events[g_kt_used].first, st);
}
void kt_end(cudaStream_t st) {
  if (!g_kernel_timing || g_kt_used >= g_kt_events.size()) return;
  cudaEventRecord(g_kt_events[g_kt_used].second, st);
  g_kt_used++;
}

CallTimer::CallTimer(rg_graph* gr) : g(gr) {
  memset(&g_timing, 0, sizeof g_timing);
  g_kt_used = 0;
  cudaEventRecord(ctx().ev0, ctx().stream);
}

rg_status CallTimer::stop() {
  Ctx& c = ctx();
  RG_CUDA(cudaEventRecord(c.ev1, c.stream));
  RG_CUDA(cudaEventSynchronize(c.ev1));
  float ms = 0;
  RG_CUDA(cudaEventElapsedTime(&ms, c.ev0, c.ev1));
  g_timing.total_ms = ms;
  double edge = 0;
  for (size_t i = 0; i < g_kt_used; i++) {
    float e = 0;
    RG_CUDA(cudaEventElapsedTime(&e, g_kt_events[i].first, g_kt_events[i].second));
    edge += e;
  }
  g_timing.edge_ms = edge;
  return RG_OK;
}

// Device properties, cached per device id (threads may drive different devices).
static int device_attr(std::atomic<int>* cache, cudaDeviceAttr attr) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::atomic<int>& c = cache[dev & 63];
  int v = c.load(std::memory_order_relaxed);
  if (!v) {
    cudaDeviceGetAttribute(&v, attr, dev);
    if (v <= 0) v = 1;
    c.store(v, std::memory_order_relaxed);
  }
  return v;
}
int device_sms() {
  static std::atomic<int> cache[64];
  return device_attr(cache, cudaDevAttrMultiProcessorCount);
}
int max_dyn_smem() {
  static std::atomic<int> cache[64];
  return device_attr(cache, cudaDevAttrMaxSharedMemoryPerBlockOptin);
}

// ---------------------------------------------------------------------------
// hubs (RADAR: ids < H after degree sort; HUBDUP: identifyHubs,
// hubdup/Ligra/ligra/IO.h:720-804, threshold = sorted_degree[H], hub iff
// degree > threshold)
// ---------------------------------------------------------------------------
struct HubCache {
  const rg_graph* g = nullptr;
  uint32_t requested = 0;  // H asked for
  uint32_t H = 0;          // hubs found (degree > sorted_degree[requested])
  DevBuf bits, slot, vertex;
};
static std::vector<HubCache*> g_hub_cache;

// Hub slots that fit the shared-memory budget for an element of `elem` bytes
// next to the push kernel's static staging arrays.
uint32_t hub_budget(size_t elem, int64_t n) {
  constexpr int kTile = kHubPushThreads * kPushItems;
  size_t static_bytes = sizeof(uint32_t) * (kTile + 3 * (kTile + 1)) + 256;
  size_t dyn = (size_t)max_dyn_smem() - static_bytes - 1024;
  dyn = std::min<size_t>(dyn, (size_t)std::max<int64_t>(g_opts.hub_smem_kb, 1) * 1024);
  uint64_t h = dyn / elem;
  if (g_opts.hub_slots > 0) h = std::min<uint64_t>(h, (uint64_t)g_opts.hub_slots);
  return (uint32_t)std::min<uint64_t>(h, (uint64_t)n);
}

thread_local Options g_opts;

static std::mutex g_hub_mu;  // the hub cache is shared by all threads

rg_status hub_map(const rg_graph* g, uint32_t H, HubInfo& info) {
  std::lock_guard<std::mutex> lk(g_hub_mu);
  HubCache* hc = nullptr;
  for (HubCache* c : g_hub_cache) if (c->g == g && c->requested == H) hc = c;
  if (!hc) {
    RG_TRY(host_arrays(g));
    std::vector<uint32_t> d(g->h_deg.begin(), g->h_deg.end());
    std::sort(d.begin(), d.end(), std::greater<uint32_t>());
    uint32_t thresh = H < (uint32_t)g->n ? d[H] : 0;
    int64_t nwords = (g->n + 31) / 32;
    std::vector<uint32_t> bits(nwords, 0), slot(g->n, 0), vert;
    for (int64_t v = 0; v < g->n; v++) {
      if (g->h_deg[v] > thresh) {
        bits[v >> 5] |= 1u << (v & 31);
        slot[v] = (uint32_t)vert.size();
        vert.push_back((uint32_t)v);
      }
    }
    hc = new HubCache();
    hc->g = g;
    hc->requested = H;
    hc->H = (uint32_t)vert.size();
    rg_status s;
    if ((s = hc->bits.reserve(4 * nwords)) != RG_OK || (s = hc->slot.reserve(4 * g->n)) != RG_OK ||
        (s = hc->vertex.reserve(4 * (vert.size() + 1))) != RG_OK) {
      delete hc;
      return s;
    }
    RG_CUDA(cudaMemcpy(hc->bits.p, bits.data(), 4 * nwords, cudaMemcpyHostToDevice));
    RG_CUDA(cudaMemcpy(hc->slot.p, slot.data(), 4 * g->n, cudaMemcpyHostToDevice));
    if (!vert.empty()) RG_CUDA(cudaMemcpy(hc->vertex.p, vert.data(), 4 * vert.size(), cudaMemcpyHostToDevice));
    g_hub_cache.push_back(hc);
  }
  info.H = hc->H;
  info.bits = hc->bits.as<uint32_t>();
  info.slot = hc->slot.as<uint32_t>();
  info.vertex = hc->vertex.as<uint32_t>();
  return RG_OK;
}

void drop_hub_cache(const rg_graph* g) {
  std::lock_guard<std::mutex> lk(g_hub_mu);
  for (auto it = g_hub_cache.begin(); it != g_hub_cache.end();) {
    if ((*it)->g == g) { delete *it; it = g_hub_cache.erase(it); }
    else ++it;
  }
}

int hub_mode_of(int variant) {
  return variant == RG_RADAR ? kHubPrefix : variant == RG_HUBDUP ? kHubMap : kHubNone;
}


constexpr double kDamping = 0.85;  // PR_Vertex_F damping (PageRank.C:126), engine-level vertexMap

// ---------------------------------------------------------------------------
// BFS (BFS.C:122-188)
// ---------------------------------------------------------------------------
__global__ void set_u32(uint32_t* a, uint32_t i, uint32_t v) { a[i] = v; }
__global__ void set_i32(int32_t* a, uint32_t i, int32_t v) { a[i] = v; }

struct BfsState {
  DevBuf parents, depth, visited, tmp;
  Frontier f[2];
};

rg_status bfs_run(rg_graph* g, int variant, uint32_t root_orig, uint32_t* h_parents, int32_t* h_depth,
                  int64_t* rounds_out, int64_t* reached_out, uint32_t hub_h, int32_t* d_depth_out) {
  if (!g) return fail(RG_EINVAL, "null graph");
  if (variant < 0 || variant > 4) return fail(RG_EINVAL, "bad variant %d", variant);
  if (root_orig >= (uint64_t)g->n) return fail(RG_EINVAL, "root %u >= n", root_orig);
  OptScope opt_scope(g, kAppBfs);
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  cudaStream_t st = cx->stream;
  const int64_t n = g->n;
  static thread_local BfsState S;
  RG_TRY(S.parents.reserve(4 * n));
  RG_TRY(S.depth.reserve(4 * n));
  RG_TRY(S.visited.reserve(4 * ((n + 31) / 32 + 8)));
  RG_TRY(frontier_alloc(g, S.f[0]));
  RG_TRY(frontier_alloc(g, S.f[1]));
  uint32_t root;
  RG_TRY(lookup_ids(g, &root_orig, 1, true, &root, nullptr));
  CallTimer timer(g);
  uint32_t* parents = S.parents.as<uint32_t>();
  int32_t* depth = S.depth.as<int32_t>();
  RG_CUDA(cudaMemsetAsync(parents, 0xFF, 4 * n, st));
  RG_CUDA(cudaMemsetAsync(depth, 0xFF, 4 * n, st));
  set_u32<<<1, 1, 0, st>>>(parents, root, root);
  set_i32<<<1, 1, 0, st>>>(depth, root, 0);
  g_timing.kernel_launches += 2;
  RG_TRY(frontier_from_host(g, S.f[0], &root, 1, st));
  FView cur = view_of(S.f[0]), nxt = view_of(S.f[1]);
  EmOpts o;
  o.variant = variant;
  o.dense_forward = variant != RG_PUSH_PULL;
  o.hub_h = hub_h;
  int64_t rounds = 0, reached = 1;
  uint32_t* visited = S.visited.as<uint32_t>();
  RG_CUDA(cudaMemsetAsync(visited, 0, 4 * ((n + 31) / 32), st));
  set_u32<<<1, 1, 0, st>>>(visited, root >> 5, 1u << (root & 31));
  OpBfs op{parents, visited, nullptr};
  while (cur.count > 0) {
    rounds++;
    op.next = nxt.bits;
    RG_TRY(edge_map(g, cur, op, &nxt, o, st, depth, (int32_t)rounds, visited));
    reached += nxt.count;
    std::swap(cur, nxt);
  }
  RG_TRY(timer.stop());
  if (d_depth_out) {  // device copy in original-id order
    if (g->sorted) {
      const int64_t blocks = std::min<int64_t>((n + 255) / 256, (int64_t)device_sms() * 32);
      gather_kernel<int32_t><<<(unsigned)blocks, 256, 0, st>>>(depth, g->new_ids.as<uint32_t>(), n, d_depth_out);
      RG_CUDA(cudaGetLastError());
    } else {
      RG_CUDA(cudaMemcpyAsync(d_depth_out, depth, 4 * n, cudaMemcpyDeviceToDevice, st));
    }
  }
  RG_TRY(download_orig<uint32_t>(g, parents, h_parents, S.tmp, st));
  RG_CUDA(cudaStreamSynchronize(st));
  RG_TRY(download_orig<int32_t>(g, depth, h_depth, S.tmp, st));
  RG_CUDA(cudaStreamSynchronize(st));
  // edges examined: the out-edges of every reached vertex
  g_timing.algorithmic_bytes = 4 * g_timing.edges_traversed + 4 * (n + 1) + 4 * n + 2 * ((n + 7) / 8) * rounds;
  if (rounds_out) *rounds_out = rounds;
  if (reached_out) *reached_out = reached;
  return RG_OK;
}

// ---------------------------------------------------------------------------
// BC (BC-manyiter-v2.C:205-367)
// ---------------------------------------------------------------------------
// inverseNumPaths (BC-manyiter-v2.C:324-325), kept beside the path counts.
__global__ void bc_invert(const double* __restrict__ sigma, double* __restrict__ inv, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i < n; i += (int64_t)gridDim.x * blockDim.x) inv[i] = 1 / sigma[i];
}
// BC_Back_Vertex_F over a level queue: visited[i] = 1; deps[i] += inv[i].
__global__ void bc_back_vertex(const uint32_t* __restrict__ q, int64_t k, uint32_t* visited, double* deps,
                               const double* __restrict__ inv) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < k) {
    uint32_t i = q[j];
    atomicOr(visited + (i >> 5), 1u << (i & 31));
    deps[i] += inv[i];
  }
}
// Final transform (BC-manyiter-v2.C:347-349): D = (D - 1/sigma) / (1/sigma),
// computed as (D - 1/sigma) * sigma: GB300 issues FP64 slowly and a divide is
// an iteration of several FP64 operations, a multiply one.  The two differ
// by a rounding of the last step (relative 1e-16); an unreached vertex
// (sigma 0, 1/sigma inf) still gives NaN.
__global__ void bc_final(double* deps, const double* __restrict__ inv, const double* __restrict__ sigma, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i < n; i += (int64_t)gridDim.x * blockDim.x) deps[i] = (deps[i] - inv[i]) * sigma[i];
}
__global__ void set_f64(double* a, uint32_t i, double v) { a[i] = v; }
// The next BC frontier after a forward push without marks: the unvisited
// vertices that now have paths (their counts were 0 before the push and only
// grow).  A warp writes one bitmap word, so no atomics.
__global__ void bc_mark_reached(const double* __restrict__ np, const uint32_t* __restrict__ visited,
                                uint32_t* __restrict__ next_bits, int64_t n) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; w * 32 < n; w += warps) {
    const int64_t v = w * 32 + lane;
    const bool r = v < n && !((visited[w] >> lane) & 1u) && np[v] != 0.0;
    const unsigned bits = __ballot_sync(0xffffffffu, r);
    if (lane == 0) next_bits[w] = bits;
  }
}

// qoff = exclusive scan of the degrees (from deg_off) of a queue's vertices,
// *degsum = their sum: a frontier's edge layout in another orientation.
__global__ void queue_degrees(const uint32_t* __restrict__ q, int64_t k, const uint32_t* __restrict__ deg_off,
                              uint32_t* __restrict__ deg) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < k) deg[j] = deg_off[q[j] + 1] - deg_off[q[j]];
}

rg_status requeue_degrees(const rg_graph* g, const uint32_t* queue, int64_t count, const uint32_t* deg_off,
                                 uint32_t* qoff, int64_t* degsum, DevBuf& tmp, cudaStream_t st) {
  if (count == 0) {
    *degsum = 0;
    return RG_OK;
  }
  RG_TRY(tmp.reserve(4 * (size_t)count));
  queue_degrees<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(queue, count, deg_off, tmp.as<uint32_t>());
  RG_CUDA(cudaGetLastError());
  RG_TRY(scan_u32(ctx().ws, tmp.as<uint32_t>(), qoff, count, st));
  uint32_t total = 0;
  RG_TRY(read_small(qoff + count, &total, 4, st));
  *degsum = total;
  return RG_OK;
}

struct BcState {
  DevBuf num_paths, inv_paths, deps, visited, levels_q, levels_qo, bits0, bits1, tmp, qdeg;
};

rg_status bc_run(rg_graph* g, int variant, const uint32_t* src_orig, int nsrc, double* h_deps, int64_t* levels_out,
                 uint32_t hub_h, double* d_deps_out) {
  if (!g) return fail(RG_EINVAL, "null graph");
  if (variant < 0 || variant > 4) return fail(RG_EINVAL, "bad variant %d", variant);
  if (nsrc < 0 || (nsrc > 0 && !src_orig)) return fail(RG_EINVAL, "bad source list");
  for (int i = 0; i < nsrc; i++) {
    if (src_orig[i] >= (uint64_t)g->n) return fail(RG_EINVAL, "source %u >= n", src_orig[i]);
  }
  OptScope opt_scope(g, kAppBc);
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  cudaStream_t st = cx->stream;
  const int64_t n = g->n;
  const int64_t nwords = (n + 31) / 32;
  static thread_local BcState S;
  RG_TRY(S.num_paths.reserve(8 * n));
  RG_TRY(S.inv_paths.reserve(8 * n));
  RG_TRY(S.deps.reserve(8 * n));
  RG_TRY(S.visited.reserve(4 * (nwords + 8)));
  RG_TRY(S.levels_q.reserve(4 * (n + 64)));
  RG_TRY(S.levels_qo.reserve(4 * (2 * n + 66)));
  RG_TRY(S.bits0.reserve(4 * (nwords + 8)));
  RG_TRY(S.bits1.reserve(4 * (nwords + 8)));
  CallTimer timer(g);
  double* np = S.num_paths.as<double>();
  double* inv = S.inv_paths.as<double>();
  double* deps = S.deps.as<double>();
  uint32_t* visited = S.visited.as<uint32_t>();
  uint32_t* LQ = S.levels_q.as<uint32_t>();
  uint32_t* LQO = S.levels_qo.as<uint32_t>();
  RG_CUDA(cudaMemsetAsync(deps, 0, 8 * n, st));
  EmOpts o;
  o.variant = variant;
  o.dense_forward = variant != RG_PUSH_PULL;
  o.hub_h = hub_h;
  const int vblocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)device_sms() * 16);
  int64_t total_levels = 0;
  std::vector<int64_t> lstart, lcount, ldeg;
  for (int it = 0; it < nsrc; it++) {
    // the reference transposes the graph before every backward phase and
    // never back (BC-manyiter-v2.C:334): on a directed graph source it's
    // forward phase runs on the graph transposed `it` times, its backward
    // phase on the opposite orientation (no-ops for symmetric graphs)
    const bool fwd_t = g->directed && (it % 2 == 1);
    EmOpts of = o, ob = o;
    of.hubs = g_opts.bc_fwd_hubs != 0;
    of.transpose = fwd_t;
    ob.transpose = g->directed && !fwd_t;
    uint32_t start, start_deg;
    RG_TRY(lookup_ids(g, &src_orig[it], 1, true, &start, &start_deg, fwd_t));
    RG_CUDA(cudaMemsetAsync(np, 0, 8 * n, st));
    set_f64<<<1, 1, 0, st>>>(np, start, 1.0);
    RG_CUDA(cudaMemsetAsync(visited, 0, 4 * nwords, st));
    set_u32<<<1, 1, 0, st>>>(visited, start >> 5, 1u << (start & 31));
    g_timing.kernel_launches += 2;
    // level 0 = {start}
    uint32_t q0[2] = {start, 0};
    uint32_t qo0[2] = {0, start_deg};
    RG_CUDA(cudaMemcpyAsync(LQ, q0, 4, cudaMemcpyHostToDevice, st));
    RG_CUDA(cudaMemcpyAsync(LQO, qo0, 8, cudaMemcpyHostToDevice, st));
    RG_CUDA(cudaMemsetAsync(S.bits0.p, 0, 4 * nwords, st));
    set_u32<<<1, 1, 0, st>>>(S.bits0.as<uint32_t>(), start >> 5, 1u << (start & 31));
    RG_CUDA(cudaStreamSynchronize(st));  // q0/qo0 live on this stack frame
    lstart.assign(1, 0);
    lcount.assign(1, 1);
    ldeg.assign(1, start_deg);
    FView cur{LQ, LQO, S.bits0.as<uint32_t>(), 1, (int64_t)start_deg};
    uint32_t* spare_bits = S.bits1.as<uint32_t>();
    int64_t round = 0, qpos = 1;
    OpBcFwd fop{np, visited};
    while (cur.count > 0) {
      round++;
      FView nxt{LQ + qpos, LQO + qpos + round, spare_bits, 0, 0};
      if (cur.degsum >= n / 4) {
        // a large level: one pass over the vertices finds the next frontier
        // for less than a bitmap test per edge
        RG_TRY(edge_map(g, cur, OpBcFwdT<false>{np, visited}, nullptr, of, st));
        bc_mark_reached<<<vblocks, 256, 0, st>>>(np, visited, nxt.bits, n);
        Frontier shell;  // non-owning view of nxt for the compaction (which syncs)
        shell.bits.p = nxt.bits;
        RG_TRY(compact_bits(g, shell, st, true, nullptr, 0, visited, nxt.queue, nxt.qoff,
                            (of.transpose && g->directed) ? g->in_off.as<uint32_t>() : nullptr));
        shell.bits.p = nullptr;
        nxt.count = shell.count;
        nxt.degsum = shell.degsum;
        g_timing.kernel_launches += 4;
      } else {
        RG_TRY(edge_map(g, cur, fop, &nxt, of, st, nullptr, 0, visited));
      }
      spare_bits = cur.bits;
      lstart.push_back(qpos);
      lcount.push_back(nxt.count);
      ldeg.push_back(nxt.degsum);
      qpos += nxt.count;
      cur = nxt;
    }
    total_levels += round;
    bc_invert<<<vblocks, 256, 0, st>>>(np, inv, n);
    RG_CUDA(cudaMemsetAsync(visited, 0, 4 * nwords, st));
    g_timing.kernel_launches++;
    auto level_view = [&](int64_t r) {
      return FView{LQ + lstart[r], LQO + lstart[r] + r, S.bits0.as<uint32_t>(), lcount[r], ldeg[r]};
    };
    auto back_vertex = [&](int64_t r) {
      if (lcount[r] > 0) {
        bc_back_vertex<<<(unsigned)((lcount[r] + 255) / 256), 256, 0, st>>>(LQ + lstart[r], lcount[r], visited, deps,
                                                                          inv);
        g_timing.kernel_launches++;
      }
    };
    back_vertex(round - 1);
    OpBcBwd bop{deps, visited};
    for (int64_t r = round - 2; r >= 0; r--) {
      FView lv = level_view(r + 1);
      if (g->directed) {  // the level's degrees in the backward orientation
        RG_TRY(requeue_degrees(g, lv.queue, lv.count, (ob.transpose ? g->in_off : g->off).as<uint32_t>(), lv.qoff,
                               &lv.degsum, S.qdeg, st));
      }
      // edge_map pulls a push-pull level above this size, and the pull reads
      // the level as a bitmap: build it with the same threshold
      const int64_t threshold = g->m / std::max<int64_t>(g_opts.dense_div, 1);
      if ((variant == RG_PUSH_PULL || g_opts.direction == 1) && lv.count + lv.degsum > threshold) {
        Frontier shell;
        shell.queue.p = lv.queue;
        shell.bits.p = lv.bits;
        shell.count = lv.count;
        RG_TRY(frontier_bits_from_queue(g, shell, st));
        shell.queue.p = nullptr;
        shell.bits.p = nullptr;
      }
      RG_TRY(edge_map(g, lv, bop, nullptr, ob, st));
      back_vertex(r);
    }
    bc_final<<<vblocks, 256, 0, st>>>(deps, inv, np, n);
    RG_CUDA(cudaGetLastError());
    g_timing.kernel_launches++;
  }
  RG_TRY(timer.stop());
  if (d_deps_out) {  // device copy in original-id order
    if (g->sorted) {
      const int64_t blocks = std::min<int64_t>((n + 255) / 256, (int64_t)device_sms() * 32);
      gather_kernel<double><<<(unsigned)blocks, 256, 0, st>>>(deps, g->new_ids.as<uint32_t>(), n, d_deps_out);
      RG_CUDA(cudaGetLastError());
    } else {
      RG_CUDA(cudaMemcpyAsync(d_deps_out, deps, 8 * n, cudaMemcpyDeviceToDevice, st));
    }
  }
  RG_TRY(download_orig<double>(g, deps, h_deps, S.tmp, st));
  RG_CUDA(cudaStreamSynchronize(st));
  g_timing.algorithmic_bytes =
      4 * g_timing.edges_traversed + (int64_t)nsrc * (8 * (n + 1) + 8 * n + n + 16 * n + 8 * n);
  if (levels_out) *levels_out = total_levels;
  return RG_OK;
}

// BC source selection (BC-manyiter-v2.C:253-271): mt19937(27491095),
// uniform_int_distribution<long>(0, n-1), redrawn while the vertex (original
// id) has degree 0.
rg_status bc_pick(const rg_graph* g, int k, uint32_t* out) {
  if (!g || k < 0 || (k > 0 && !out)) return fail(RG_EINVAL, "bad arguments");
  RG_TRY(host_arrays(g));
  if (g->h_deg.size() != (size_t)g->n || (g->directed && g->h_in_deg.size() != (size_t)g->n) ||
      (g->sorted && g->h_new_ids.size() != (size_t)g->n))
    return fail(RG_EUNSUPPORTED, "host degree arrays missing");
  bool any = false;
  for (int64_t v = 0; v < g->n && !any; v++) any = g->h_deg[v] > 0;
  if (!any && k > 0) return fail(RG_EINVAL, "graph has no edges; no BC source can be drawn");
  std::mt19937 rng(27491095);
  std::uniform_int_distribution<long> ud(0, g->n - 1);
  for (int i = 0; i < k; i++) {
    long s;
    // the reference checks the out-degree of the graph as it stands, and its
    // BC transposes a directed graph once per source (BC-manyiter-v2.C:264-270)
    const HostU32& deg = (g->directed && (i % 2)) ? g->h_in_deg : g->h_deg;
    do { s = ud(rng); } while (deg[g->sorted ? g->h_new_ids[s] : (uint32_t)s] == 0);
    out[i] = (uint32_t)s;
  }
  return RG_OK;
}

// Search roots by GAP's SourcePicker (GAP/src/benchmark.h:47-64): one
// mt19937(27491095) drives uniform_int_distribution<int32_t> (NodeID) over
// [0, n-1]; a pick is redrawn while the vertex (original id) has out-degree
// 0, and the k picks continue the same generator.
rg_status pick_roots(const rg_graph* g, int k, uint32_t* out) {
  if (!g || k < 0 || (k > 0 && !out)) return fail(RG_EINVAL, "bad arguments");
  if (g->n > 0x7FFFFFFFll) return fail(RG_EUNSUPPORTED, "SourcePicker draws int32 ids");
  RG_TRY(host_arrays(g));
  if (g->h_deg.size() != (size_t)g->n || (g->sorted && g->h_new_ids.size() != (size_t)g->n))
    return fail(RG_EUNSUPPORTED, "host degree arrays missing");
  bool any = false;
  for (int64_t v = 0; v < g->n && !any; v++) any = g->h_deg[v] > 0;
  if (!any && k > 0) return fail(RG_EINVAL, "graph has no edges; no root can be drawn");
  std::mt19937 rng(27491095);
  std::uniform_int_distribution<int32_t> ud(0, (int32_t)(g->n - 1));
  for (int i = 0; i < k; i++) {
    int32_t s;
    do { s = ud(rng); } while (g->h_deg[g->sorted ? g->h_new_ids[s] : (uint32_t)s] == 0);
    out[i] = (uint32_t)s;
  }
  return RG_OK;
}

// ---------------------------------------------------------------------------
// Radii (Radii.C:140-218)
// ---------------------------------------------------------------------------
__global__ void radii_sync(const uint32_t* __restrict__ q, int64_t k, unsigned long long* visited,
                           const unsigned long long* __restrict__ next_visited) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < k) {
    uint32_t i = q[j];
    visited[i] = next_visited[i];
  }
}
__global__ void radii_seed(const uint32_t* __restrict__ v, const unsigned long long* __restrict__ mask, int k,
                           unsigned long long* next_visited, int32_t* radii) {
  int j = threadIdx.x;
  if (j < k) {
    next_visited[v[j]] = mask[j];
    radii[v[j]] = 0;
  }
}

struct RadiiState {
  DevBuf visited, next_visited, radii, seedv, seedm, tmp;
  Frontier f[2];
};

rg_status radii_run(rg_graph* g, int variant, const uint32_t* seeds_orig, int k, int32_t* h_radii,
                    int64_t* rounds_out, uint32_t hub_h, int32_t* d_radii_out) {
  if (!g) return fail(RG_EINVAL, "null graph");
  if (variant < 0 || variant > 4) return fail(RG_EINVAL, "bad variant %d", variant);
  if (k < 0 || k > 64 || (k > 0 && !seeds_orig)) return fail(RG_EINVAL, "need 0..64 seeds");
  OptScope opt_scope(g, kAppRadii);
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  cudaStream_t st = cx->stream;
  const int64_t n = g->n;
  static thread_local RadiiState S;
  RG_TRY(S.visited.reserve(8 * n));
  RG_TRY(S.next_visited.reserve(8 * n));
  RG_TRY(S.radii.reserve(4 * n));
  RG_TRY(S.seedv.reserve(4 * 64));
  RG_TRY(S.seedm.reserve(8 * 64));
  RG_TRY(frontier_alloc(g, S.f[0]));
  RG_TRY(frontier_alloc(g, S.f[1]));
  // seeding loop (Radii.C:162-169): NextVisited[v] = 1<<i is a plain store, so
  // on a collision the largest i wins (the single-thread order)
  std::vector<uint32_t> starts(k), sdeg(k), uv, udeg;
  std::vector<unsigned long long> um;
  RG_TRY(lookup_ids(g, seeds_orig, k, true, starts.data(), sdeg.data()));
  for (int i = 0; i < k; i++) {
    const uint32_t v = starts[i];
    auto it = std::find(uv.begin(), uv.end(), v);
    if (it == uv.end()) { uv.push_back(v); um.push_back(1ull << i); udeg.push_back(sdeg[i]); }
    else um[it - uv.begin()] = 1ull << i;
  }
  // the bits that can spread: seeded at a vertex with out-edges
  unsigned long long full = 0ull;
  for (size_t j = 0; j < uv.size(); j++) full |= udeg[j] ? um[j] : 0ull;
  CallTimer timer(g);
  unsigned long long* vis = S.visited.as<unsigned long long>();
  unsigned long long* nvis = S.next_visited.as<unsigned long long>();
  int32_t* radii = S.radii.as<int32_t>();
  RG_CUDA(cudaMemsetAsync(vis, 0, 8 * n, st));
  RG_CUDA(cudaMemsetAsync(nvis, 0, 8 * n, st));
  RG_CUDA(cudaMemsetAsync(radii, 0xFF, 4 * n, st));
  if (!uv.empty()) {
    RG_CUDA(cudaMemcpyAsync(S.seedv.p, uv.data(), 4 * uv.size(), cudaMemcpyHostToDevice, st));
    RG_CUDA(cudaMemcpyAsync(S.seedm.p, um.data(), 8 * um.size(), cudaMemcpyHostToDevice, st));
    radii_seed<<<1, 64, 0, st>>>(S.seedv.as<uint32_t>(), S.seedm.as<unsigned long long>(), (int)uv.size(), nvis,
                                 radii);
    g_timing.kernel_launches++;
  }
  RG_TRY(frontier_from_host(g, S.f[0], starts.data(), k, st));  // keeps duplicates, like vertexSubset(n,64,starts)
  FView cur = view_of(S.f[0]), nxt = view_of(S.f[1]);
  EmOpts o;
  o.variant = variant;
  o.dense_forward = variant != RG_PUSH_PULL;
  o.hub_h = hub_h;
  int32_t round = 0;
  while (cur.count > 0) {
    round++;
    radii_sync<<<(unsigned)((cur.count + 255) / 256), 256, 0, st>>>(cur.queue, cur.count, vis, nvis);
    g_timing.kernel_launches++;
    const bool dense = cur.count + cur.degsum > g->m / std::max<int64_t>(g_opts.dense_div, 1);
    if (dense && g->m > 0 && (variant == RG_PUSH_PULL || g_opts.direction == 1)) {
      // dense round: pull over every edge (same next masks and frontier)
      RG_CUDA(cudaMemsetAsync(nxt.bits, 0, 4 * ((n + 31) / 32), st));
      g_timing.edges_traversed += cur.degsum;
      RG_TRY(launch_mask_sweep(g, vis, nvis, nxt.bits, st, full));
      Frontier shell;  // non-owning view of nxt for the compaction
      shell.bits.p = nxt.bits;
      RG_TRY(compact_bits(g, shell, st, true, radii, round, nullptr, nxt.queue, nxt.qoff));
      shell.bits.p = nullptr;
      nxt.count = shell.count;
      nxt.degsum = shell.degsum;
      g_timing.kernel_launches += 3;
    } else {
      OpRadii op{vis, nvis, radii, round};
      RG_TRY(edge_map(g, cur, op, &nxt, o, st, radii, round));  // radii[v] = round for the next frontier
    }
    std::swap(cur, nxt);
  }
  RG_TRY(timer.stop());
  if (d_radii_out) {  // device copy in original-id order
    if (g->sorted) {
      const int64_t blocks = std::min<int64_t>((n + 255) / 256, (int64_t)device_sms() * 32);
      gather_kernel<int32_t><<<(unsigned)blocks, 256, 0, st>>>(radii, g->new_ids.as<uint32_t>(), n, d_radii_out);
      RG_CUDA(cudaGetLastError());
    } else {
      RG_CUDA(cudaMemcpyAsync(d_radii_out, radii, 4 * n, cudaMemcpyDeviceToDevice, st));
    }
  }
  RG_TRY(download_orig<int32_t>(g, radii, h_radii, S.tmp, st));
  RG_CUDA(cudaStreamSynchronize(st));
  g_timing.algorithmic_bytes = 4 * g_timing.edges_traversed + 16 * n + 4 * n;
  if (rounds_out) *rounds_out = round;
  return RG_OK;
}

}  // namespace rg

using namespace rg;

extern "C" {

rg_status rg_bfs(rg_graph* g, rg_variant variant, uint32_t root, uint32_t* h_parents, int32_t* h_depth,
                 int64_t* rounds_out, int64_t* reached_out) {
  return bfs_run(g, variant, root, h_parents, h_depth, rounds_out, reached_out, 0);
}

rg_status rg_bc_pick_sources(const rg_graph* g, int k, uint32_t* h_sources) { return bc_pick(g, k, h_sources); }

rg_status rg_pick_roots(const rg_graph* g, int k, uint32_t* h_roots) { return pick_roots(g, k, h_roots); }

rg_status rg_bc(rg_graph* g, rg_variant variant, int max_iters, double* h_deps, int64_t* levels_out) {
  if (!g || max_iters < 0) return fail(RG_EINVAL, "bad arguments");
  std::vector<uint32_t> src(max_iters);
  RG_TRY(bc_pick(g, max_iters, src.data()));
  return bc_run(g, variant, src.data(), max_iters, h_deps, levels_out, 0);
}

rg_status rg_bc_sources(rg_graph* g, rg_variant variant, const uint32_t* h_sources, int nsrc, double* h_deps,
                        int64_t* levels_out) {
  return bc_run(g, variant, h_sources, nsrc, h_deps, levels_out, 0);
}

rg_status rg_radii(rg_graph* g, rg_variant variant, int32_t* h_radii, int64_t* rounds_out) {
  if (!g) return fail(RG_EINVAL, "null graph");
  int k = (int)std::min<int64_t>(g->n, 64);
  std::vector<uint32_t> seeds(k);
  for (int i = 0; i < k; i++) seeds[i] = (uint32_t)(hash_u64((uint64_t)i) % (uint64_t)g->n);
  return radii_run(g, variant, seeds.data(), k, h_radii, rounds_out, 0);
}

rg_status rg_radii_seeds(rg_graph* g, rg_variant variant, const uint32_t* h_seeds, int k, int32_t* h_radii,
                         int64_t* rounds_out) {
  return radii_run(g, variant, h_seeds, k, h_radii, rounds_out, 0);
}

rg_status rg_set_trace(int on) {
  g_trace_on = on != 0;
  if (!g_trace_on) g_trace.clear();
  return RG_OK;
}

rg_status rg_trace_take(rg_level_trace* h_out, int64_t cap, int64_t* count) {
  if (cap < 0 || (cap > 0 && !h_out) || !count) return fail(RG_EINVAL, "rg_trace_take: bad arguments");
  const int64_t k = std::min<int64_t>(cap, (int64_t)g_trace.size());
  std::copy(g_trace.begin(), g_trace.begin() + k, h_out);
  *count = k;
  g_trace.clear();
  return RG_OK;
}

rg_status rg_set_option(rg_option opt, int64_t value) {
  switch (opt) {
    case RG_OPT_DIRECTION:
      if (value != 0 && value != 1) return fail(RG_EINVAL, "direction must be 0 or 1");
      g_opts.direction = value;
      return RG_OK;
    case RG_OPT_HUB_SLOTS:
      if (value < 0) return fail(RG_EINVAL, "hub slots must be >= 0");
      g_opts.hub_slots = value;
      return RG_OK;
    case RG_OPT_HUB_SMEM_KB:
      if (value < 0 || value > 227) return fail(RG_EINVAL, "hub shared memory must be 0..227 KiB");
      g_opts.hub_smem_kb = value;
      return RG_OK;
    case RG_OPT_DENSE_DIV:
      if (value < 1) return fail(RG_EINVAL, "dense divisor must be >= 1");
      g_opts.dense_div = value;
      return RG_OK;
    case RG_OPT_SWEEP_SHAPE:
      if ((value / 10 != 4 && value / 10 != 8 && value / 10 != 16) || value % 10 > 2) {
        return fail(RG_EINVAL, "sweep shape must be 40..42, 80..82 or 160..162");
      }
      g_opts.sweep_shape = value;
      return RG_OK;
    case RG_OPT_BC_FWD_HUBS:
      if (value != 0 && value != 1) return fail(RG_EINVAL, "bc_fwd_hubs must be 0 or 1");
      g_opts.bc_fwd_hubs = value;
      return RG_OK;
    case RG_OPT_ASYNC_RESULTS:
      if (value != 0 && value != 1) return fail(RG_EINVAL, "async_results must be 0 or 1");
      g_opts.async_results = value;
      return RG_OK;
  }
  return fail(RG_EINVAL, "unknown option %d", (int)opt);
}

rg_status rg_get_option(rg_option opt, int64_t* value) {
  if (!value) return fail(RG_EINVAL, "null value");
  switch (opt) {
    case RG_OPT_DIRECTION: *value = g_opts.direction; return RG_OK;
    case RG_OPT_HUB_SLOTS: *value = g_opts.hub_slots; return RG_OK;
    case RG_OPT_HUB_SMEM_KB: *value = g_opts.hub_smem_kb; return RG_OK;
    case RG_OPT_DENSE_DIV: *value = g_opts.dense_div; return RG_OK;
    case RG_OPT_SWEEP_SHAPE: *value = g_opts.sweep_shape; return RG_OK;
    case RG_OPT_BC_FWD_HUBS: *value = g_opts.bc_fwd_hubs; return RG_OK;
    case RG_OPT_ASYNC_RESULTS: *value = g_opts.async_results; return RG_OK;
  }
  return fail(RG_EINVAL, "unknown option %d", (int)opt);
}

rg_status rg_set_kernel_timing(int on) {
  g_kernel_timing = on != 0;
  return RG_OK;
}

rg_status rg_last_timing(rg_timing* t) {
  if (!t) return fail(RG_EINVAL, "null");
  *t = g_timing;
  return RG_OK;
}

// ---- engine-level API ------------------------------------------------------

rg_status rg_frontier_create(const rg_graph* g, rg_frontier** out) {
  if (!g || !out) return fail(RG_EINVAL, "null argument");
  rg_frontier* f = new (std::nothrow) rg_frontier();
  if (!f) return fail(RG_ENOMEM, "host allocation failed");
  f->g = g;
  rg_status s = frontier_alloc(g, f->f);
  if (s != RG_OK) { delete f; return s; }
  RG_CUDA(cudaMemset(f->f.bits.p, 0, f->f.bits.bytes));
  RG_CUDA(cudaMemset(f->f.qoff.p, 0, 4));
  *out = f;
  return RG_OK;
}

rg_status rg_frontier_free(rg_frontier* f) {
  delete f;
  return RG_OK;
}

rg_status rg_frontier_set(rg_frontier* f, const uint32_t* h_ids, int64_t k) {
  if (!f || k < 0 || (k > 0 && !h_ids)) return fail(RG_EINVAL, "bad arguments");
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  return frontier_from_host(f->g, f->f, h_ids, k, cx->stream);
}

rg_status rg_frontier_set_all(rg_frontier* f) {
  if (!f) return fail(RG_EINVAL, "null frontier");
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  return frontier_set_all(f->g, f->f, cx->stream);
}

rg_status rg_frontier_count(const rg_frontier* f, int64_t* count) {
  if (!f || !count) return fail(RG_EINVAL, "null argument");
  *count = f->f.count;
  return RG_OK;
}

rg_status rg_frontier_get(const rg_frontier* f, uint8_t* h_member) {
  if (!f || !h_member) return fail(RG_EINVAL, "null argument");
  const int64_t n = f->g->n, nwords = (n + 31) / 32;
  std::vector<uint32_t> bits(nwords);
  RG_CUDA(cudaMemcpy(bits.data(), f->f.bits.p, 4 * nwords, cudaMemcpyDeviceToHost));
  for (int64_t v = 0; v < n; v++) h_member[v] = (bits[v >> 5] >> (v & 31)) & 1u;
  return RG_OK;
}

__global__ void contrib_kernel(uint32_t n, const uint32_t* __restrict__ off, const double* __restrict__ p,
                               double* __restrict__ c) {
  int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    uint32_t d = off[v + 1] - off[v];
    c[v] = d ? p[v] / (double)d : 0.0;
  }
}

rg_status rg_edgemap(rg_graph* g, rg_frontier* in, rg_op op, const rg_op_args* a, rg_frontier* out, uint32_t flags,
                     int64_t threshold, void* stream) {
  if (!g || !in || !a || in->g != g || (out && out->g != g)) return fail(RG_EINVAL, "bad arguments");
  if (in->f.count > g->n + 64) return fail(RG_EINVAL, "edgeMap: Sizes Don't match");
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  cudaStream_t st = stream ? (cudaStream_t)stream : cx->stream;
  memset(&g_timing, 0, sizeof g_timing);
  FView iv = view_of(in->f);
  const bool want_out = out && !(flags & RG_NO_OUTPUT);
  FView ov;
  if (want_out) ov = view_of(out->f);
  EmOpts o;
  o.variant = RG_PUSH;
  o.dense_forward = (flags & RG_DENSE_FORWARD) != 0;
  o.threshold = threshold;
  // the pull path reads the input bitmap; make sure it matches the queue
  if (!in->f.bits_valid) RG_TRY(frontier_bits_from_queue(g, in->f, st));
  rg_status s = RG_OK;
  switch (op) {
    case RG_OP_PAGERANK: {
      if (!a->p_curr || !a->p_next) return fail(RG_EINVAL, "PAGERANK needs p_curr, p_next");
      static thread_local DevBuf contrib;
      RG_TRY(contrib.reserve(8 * g->n));
      contrib_kernel<<<(unsigned)std::min<int64_t>((g->n + 255) / 256, 4096), 256, 0, st>>>(
          (uint32_t)g->n, g->off.as<uint32_t>(), a->p_curr, contrib.as<double>());
      s = edge_map(g, iv, OpPr{contrib.as<double>(), a->p_next}, nullptr, o, st);
      break;
    }
    case RG_OP_BFS:
      if (!a->parents) return fail(RG_EINVAL, "BFS needs parents");
      s = edge_map(g, iv, OpBfs{a->parents}, want_out ? &ov : nullptr, o, st);
      break;
    case RG_OP_BC_FWD:
      if (!a->num_paths || !a->visited_bits) return fail(RG_EINVAL, "BC_FWD needs num_paths, visited_bits");
      s = edge_map(g, iv, OpBcFwd{a->num_paths, a->visited_bits}, want_out ? &ov : nullptr, o, st);
      break;
    case RG_OP_BC_BWD:
      if (!a->deps || !a->visited_bits) return fail(RG_EINVAL, "BC_BWD needs deps, visited_bits");
      s = edge_map(g, iv, OpBcBwd{a->deps, a->visited_bits}, nullptr, o, st);
      break;
    case RG_OP_RADII:
      if (!a->visited || !a->next_visited || !a->radii) return fail(RG_EINVAL, "RADII needs visited, next_visited, radii");
      s = edge_map(g, iv,
                   OpRadii{(const unsigned long long*)a->visited, (unsigned long long*)a->next_visited, a->radii,
                           a->round},
                   want_out ? &ov : nullptr, o, st, want_out ? a->radii : nullptr, a->round);
      break;
    default:
      return fail(RG_EINVAL, "unknown op %d", (int)op);
  }
  if (s != RG_OK) return s;
  if (want_out) {
    out->f.count = ov.count;
    out->f.degsum = ov.degsum;
    out->f.queue_valid = true;
    out->f.bits_valid = true;
  }
  RG_CUDA(cudaStreamSynchronize(st));
  return RG_OK;
}

__global__ void vertexmap_kernel(const uint32_t* __restrict__ q, int64_t k, int vop, rg_op_args a, double c) {
  int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= k) return;
  uint32_t i = q[j];
  switch (vop) {
    case RG_VOP_PR_DAMP: a.p_next[i] = kDamping * a.p_next[i] + c; break;
    case RG_VOP_BC_VISIT: atomicOr(a.visited_bits + (i >> 5), 1u << (i & 31)); break;
    case RG_VOP_BC_BACK:
      atomicOr(a.visited_bits + (i >> 5), 1u << (i & 31));
      a.deps[i] += a.num_paths[i];
      break;
    case RG_VOP_RADII_SYNC: a.visited[i] = a.next_visited[i]; break;
  }
}

rg_status rg_vertexmap(rg_graph* g, rg_frontier* f, rg_vop vop, const rg_op_args* a, void* stream) {
  if (!g || !f || !a || f->g != g) return fail(RG_EINVAL, "bad arguments");
  if ((int)vop < 0 || (int)vop > 3) return fail(RG_EINVAL, "unknown vertex op");
  if ((vop == RG_VOP_PR_DAMP && !a->p_next) || (vop == RG_VOP_BC_VISIT && !a->visited_bits) ||
      (vop == RG_VOP_BC_BACK && (!a->visited_bits || !a->deps || !a->num_paths)) ||
      (vop == RG_VOP_RADII_SYNC && (!a->visited || !a->next_visited))) {
    return fail(RG_EINVAL, "vertex op is missing an array");
  }
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  cudaStream_t st = stream ? (cudaStream_t)stream : cx->stream;
  if (!f->f.queue_valid) RG_TRY(compact_bits(g, f->f, st, true));
  if (f->f.count > 0) {
    vertexmap_kernel<<<(unsigned)((f->f.count + 255) / 256), 256, 0, st>>>(
        f->f.queue.as<uint32_t>(), f->f.count, (int)vop, *a, (1 - kDamping) * (1 / (double)g->n));
    RG_CUDA(cudaGetLastError());
  }
  RG_CUDA(cudaStreamSynchronize(st));
  return RG_OK;
}

}  // extern "C"
