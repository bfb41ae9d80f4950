// Host-side helpers shared by the app drivers (apps.cu, pagerank.cu):
// per-call timing, device attributes, hub set-up, result download.
#pragma once

#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <utility>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "engine.cuh"
#include "rg_device.cuh"

namespace rg {

extern thread_local rg_timing g_timing;
extern bool g_kernel_timing;
// rg_set_trace: the calling thread's per-level edgeMap records
extern thread_local bool g_trace_on;
extern thread_local std::vector<rg_level_trace> g_trace;

// NVTX range for the lifetime of the object (no cost without a profiler)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

// rg_set_option values
// The calling thread's options (rg_set_option).  An app call on a graph that
// the autotuner has tuned runs with the graph's choice for that app instead.
extern thread_local Options g_opts;

enum App { kAppPagerank = 0, kAppBfs = 1, kAppBc = 2, kAppRadii = 3 };

struct OptScope {
  Options saved;
  OptScope(const rg_graph* g, int app) : saved(g_opts) {
    if (g && g->tuned[app]) {
      g_opts = g->topt[app];
      g_opts.async_results = saved.async_results;  // the thread's, not the schedule's
    }
  }
  ~OptScope() { g_opts = saved; }
};

// Events around one edge-kernel launch (only when rg_set_kernel_timing(1)).
void kt_begin(cudaStream_t st);
void kt_end(cudaStream_t st);

// CUDA events on the graph's stream around the device work of one app call.
struct CallTimer {
  rg_graph* g;
  explicit CallTimer(rg_graph* gr);
  rg_status stop();
};

int device_sms();     // of the calling thread's current device
int max_dyn_smem();   // opt-in shared memory per block, same device

// Runs fn (returning rg_status) once per device, however many threads call:
// kernel attributes are per device, and a flag without the device id would
// leave a second device unset.  `done` holds one bit per device id.
template <class Fn>
inline rg_status once_per_device(std::atomic<uint64_t>& done, Fn&& fn) {
  int dev = 0;
  RG_CUDA(cudaGetDevice(&dev));
  const uint64_t bit = 1ull << (dev & 63);
  if (done.load(std::memory_order_acquire) & bit) return RG_OK;
  const rg_status s = fn();
  if (s == RG_OK) done.fetch_or(bit, std::memory_order_acq_rel);
  return s;
}

// Lets `kern` take all the opt-in dynamic shared memory next to its static
// arrays, once per device.  Launches then pass their own size; setting the
// limit per call instead would let one thread lower it under another's
// launch.
template <class K>
inline rg_status allow_max_dyn_smem(std::atomic<uint64_t>& done, K kern) {
  return once_per_device(done, [&]() -> rg_status {
    cudaFuncAttributes fa;
    RG_CUDA(cudaFuncGetAttributes(&fa, kern));
    RG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 max_dyn_smem() - (int)fa.sharedSizeBytes));
    return RG_OK;
  });
}

// App drivers (pagerank.cu, apps.cu, multi.cu).  Host outputs are in original
// id order; the optional device outputs (d_*) receive the same arrays on the
// device (for serving, which keeps results resident until they are fetched).
rg_status pagerank_run(rg_graph* g, int variant, int64_t max_iters, double* h_ranks, int64_t* iters_out,
                       double* l1_out, uint32_t hub_h);
rg_status bfs_run(rg_graph* g, int variant, uint32_t root_orig, uint32_t* h_parents, int32_t* h_depth,
                  int64_t* rounds_out, int64_t* reached_out, uint32_t hub_h, int32_t* d_depth_out = nullptr);
rg_status bc_run(rg_graph* g, int variant, const uint32_t* src_orig, int nsrc, double* h_deps, int64_t* levels_out,
                 uint32_t hub_h, double* d_deps_out = nullptr);
rg_status radii_run(rg_graph* g, int variant, const uint32_t* seeds_orig, int k, int32_t* h_radii,
                    int64_t* rounds_out, uint32_t hub_h, int32_t* d_radii_out = nullptr);
rg_status bc_pick(const rg_graph* g, int k, uint32_t* out);
rg_status bfs_multi_run(rg_graph* g, const uint32_t* src_orig, int k, int32_t* h_depths, int64_t* rounds_out,
                        int32_t* d_depths_out = nullptr);
// k <= 64 independent single-source BCs in one traversal: h_out / d_out (either
// may be null) receive k rows of n doubles in original-id order (bc_multi.cu).
rg_status bc_multi_run(rg_graph* g, const uint32_t* src_orig, int k, double* h_out, double* d_out,
                       int64_t* levels_out);
// nq <= 16 Radii queries of k seeds each (seeds[q*k + i], ORIGINAL ids) in one
// traversal; h_radii / d_radii_out (either may be null): nq rows of n int32 in
// original-id order (radii_multi.cu).
rg_status radii_multi_run(rg_graph* g, const uint32_t* seeds_orig, int k, int nq, int32_t* h_radii,
                          int32_t* d_radii_out, int64_t* rounds_out);
// qoff = exclusive scan of the degrees (from deg_off) of a queue's vertices,
// *degsum = their sum: a frontier's edge layout in another orientation.
rg_status requeue_degrees(const rg_graph* g, const uint32_t* queue, int64_t count, const uint32_t* deg_off,
                          uint32_t* qoff, int64_t* degsum, DevBuf& tmp, cudaStream_t st);

// Hub slots that fit the push kernel's shared-memory budget (elem bytes each).
uint32_t hub_budget(size_t elem, int64_t n);
// HUBDUP hub set (identifyHubs): bitmap + vertex->slot + slot->vertex.
rg_status hub_map(const rg_graph* g, uint32_t H, HubInfo& info);
int hub_mode_of(int variant);

// out[v] = in[new_ids[v]]: results in original-id order (writeOutputToFile).
template <class T>
__global__ void gather_kernel(const T* __restrict__ in, const uint32_t* __restrict__ new_ids, int64_t n,
                              T* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i < n; i += (int64_t)gridDim.x * blockDim.x) out[i] = in[new_ids[i]];
}

// The thread's stream for asynchronous result copies (RG_OPT_ASYNC_RESULTS).
rg_status copy_stream(cudaStream_t* out);

// First vertex of a degree-sorted graph's pull lists with at most 8 entries
// (a schedule hint, computed once per graph; any value gives the same results).
uint32_t pull_split(const rg_graph* g, const DevGraph& pull_g, cudaStream_t st);

// Result download, asynchronous form: `fill(stage)` enqueues on `st` the
// work that writes the `count` results into a staging buffer; the copy into
// h_out then runs on the thread's copy stream once that work is done, and the
// staging buffer is released in stream order after the copy.  The call
// returns without waiting, and the caller may overwrite its own buffers at
// once.
template <class T, class Fill>
rg_status download_async(T* h_out, int64_t count, cudaStream_t st, Fill fill) {
  cudaStream_t cs = nullptr;
  RG_TRY(copy_stream(&cs));
  DevBuf stage(true, cs);
  RG_TRY(stage.reserve(sizeof(T) * (size_t)count));
  RG_TRY(fill(stage.as<T>()));
  cudaEvent_t ev = nullptr;
  RG_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(ev, st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(cs, ev, 0);
  cudaEventDestroy(ev);
  if (e == cudaSuccess) e = cudaMemcpyAsync(h_out, stage.p, sizeof(T) * (size_t)count, cudaMemcpyDeviceToHost, cs);
  if (e != cudaSuccess) return cuda_fail(e, "asynchronous result copy", __FILE__, __LINE__);
  return RG_OK;
}

template <class T>
rg_status download_orig(rg_graph* g, const T* d_arr, T* h_out, DevBuf& tmp, cudaStream_t st) {
  if (!h_out) return RG_OK;
  if (g_opts.async_results) {
    return download_async<T>(h_out, g->n, st, [&](T* stage) -> rg_status {
      if (g->sorted) {
        int64_t blocks = std::min<int64_t>((g->n + 255) / 256, (int64_t)device_sms() * 32);
        gather_kernel<T><<<(unsigned)blocks, 256, 0, st>>>(d_arr, g->new_ids.as<uint32_t>(), g->n, stage);
        RG_CUDA(cudaGetLastError());
        g_timing.kernel_launches++;
      } else {
        RG_CUDA(cudaMemcpyAsync(stage, d_arr, sizeof(T) * g->n, cudaMemcpyDeviceToDevice, st));
      }
      return RG_OK;
    });
  }
  const T* src = d_arr;
  if (g->sorted) {
    RG_TRY(tmp.reserve(sizeof(T) * g->n));
    int64_t blocks = std::min<int64_t>((g->n + 255) / 256, (int64_t)device_sms() * 32);
    gather_kernel<T><<<(unsigned)blocks, 256, 0, st>>>(d_arr, g->new_ids.as<uint32_t>(), g->n, tmp.as<T>());
    RG_CUDA(cudaGetLastError());
    g_timing.kernel_launches++;
    src = tmp.as<T>();
  }
  RG_CUDA(cudaMemcpyAsync(h_out, src, sizeof(T) * g->n, cudaMemcpyDeviceToHost, st));
  return RG_OK;
}

// ---------------------------------------------------------------------------
// frontier views and the edgeMap driver (edgeMapData, ligra.h:277-316)
// ---------------------------------------------------------------------------
struct FView {
  uint32_t* queue = nullptr;
  uint32_t* qoff = nullptr;
  uint32_t* bits = nullptr;
  int64_t count = 0, degsum = 0;
};

inline FView view_of(Frontier& f) {
  return FView{f.queue.as<uint32_t>(), f.qoff.as<uint32_t>(), f.bits.as<uint32_t>(), f.count, f.degsum};
}

struct EmOpts {
  int variant = RG_PUSH;
  bool dense_forward = true;
  int64_t threshold = -1;
  uint32_t hub_h = 0;  // 0 = budget
  bool hubs = true;    // false: this push runs without hub copies
  // run on the transposed graph (graph.h:78-86): pushes follow in-lists,
  // pulls read out-lists, the next frontier's degrees are in-degrees (a
  // no-op for symmetric graphs)
  bool transpose = false;
};

// Frontiers below this many edges skip hub privatisation: the shared-memory
// set-up and merge would cost more than the atomics they save.  Results do not
// depend on it.
constexpr int64_t kHubMinEdges = 1 << 16;

template <class Op, int kHub>
rg_status launch_push(rg_graph* g, const DevGraph& pg, const FView& in, const Op& op, const HubInfo& hub,
                      uint32_t* next_bits, cudaStream_t st) {
  constexpr int kT = kHub == kHubNone ? kPushThreads : kHubPushThreads;
  constexpr int kTile = kT * kPushItems;
  auto kern = push_lbs<Op, kHub, kT>;
  const int64_t tiles = (in.degsum + kTile - 1) / kTile;
  size_t dyn = kHub == kHubNone ? 0 : sizeof(typename Op::HubT) * hub.H;
  int grid;
  if (kHub == kHubNone) {
    grid = (int)std::min<int64_t>(tiles, (int64_t)device_sms() * 8);
  } else {
    static std::atomic<uint64_t> limit_set{0};
    RG_TRY(allow_max_dyn_smem(limit_set, kern));
    int per_sm = 0;
    RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kT, dyn));
    if (per_sm < 1) per_sm = 1;
    grid = (int)std::min<int64_t>(tiles, (int64_t)device_sms() * per_sm);
  }
  if (grid < 1) grid = 1;
  Workspace& ws = ctx().ws;
  RG_TRY(ws.tiles.reserve(sizeof(uint32_t) * (tiles + 2)));
  tile_starts<<<(unsigned)((tiles + 1 + 255) / 256), 256, 0, st>>>(in.qoff, (uint32_t)in.count,
                                                                    (uint32_t)in.degsum, kTile, (uint32_t)tiles,
                                                                    ws.tiles.as<uint32_t>());
  g_timing.kernel_launches++;
  kt_begin(st);
  kern<<<grid, kT, dyn, st>>>(pg, in.queue, in.qoff, ws.tiles.as<uint32_t>(), (uint32_t)in.degsum, op, hub,
                              next_bits);
  kt_end(st);
  RG_CUDA(cudaGetLastError());
  g_timing.kernel_launches++;
  g_timing.edge_launches++;
  return RG_OK;
}

// One dense bitmask round over every edge (mask_pull_sweep): next_bits must be
// cleared; the caller compacts it afterwards.
// `full`: the bits a vertex can still receive (mask_pull_sweep skips rows
// that hold them all; 0 = gather every row).  Edges per lane follow the
// thread's sweep shape (16 for shapes 160..162, else 8).
template <int kItems>
rg_status launch_mask_sweep_k(rg_graph* g, const unsigned long long* visited, unsigned long long* next,
                              uint32_t* next_bits, cudaStream_t st, unsigned long long full) {
  static std::atomic<uint64_t> carveout_set{0};  // one copy per translation unit and instance, like the kernel
  RG_TRY(once_per_device(carveout_set, [] {
    RG_CUDA(cudaFuncSetAttribute(mask_pull_sweep<kItems>, cudaFuncAttributePreferredSharedMemoryCarveout, 0));
    return RG_OK;
  }));
  static std::atomic<int> resident{0};
  int per_sm = resident.load(std::memory_order_relaxed);
  if (!per_sm) {
    RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mask_pull_sweep<kItems>, 256, 0));
    per_sm = std::max(per_sm, 1);
    resident.store(per_sm, std::memory_order_relaxed);
  }
  const int64_t grid = std::min<int64_t>((int64_t)device_sms() * per_sm, (g->nchunks * 32 + 255) / 256);
  kt_begin(st);
  mask_pull_sweep<kItems><<<(unsigned)std::max<int64_t>(grid, 1), 256, 0, st>>>(
      g->in_view(), g->in_chunks(), (uint32_t)g->nchunks, visited, next, next_bits, full);
  kt_end(st);
  RG_CUDA(cudaGetLastError());
  g_timing.kernel_launches++;
  g_timing.edge_launches++;
  return RG_OK;
}

static inline rg_status launch_mask_sweep(rg_graph* g, const unsigned long long* visited, unsigned long long* next,
                                          uint32_t* next_bits, cudaStream_t st, unsigned long long full = 0ull) {
  return g_opts.sweep_shape / 10 == 16 ? launch_mask_sweep_k<16>(g, visited, next, next_bits, st, full)
                                       : launch_mask_sweep_k<8>(g, visited, next, next_bits, st, full);
}

// One edgeMap.  `out` (may be null for no_output ops) receives the next
// frontier: its bitmap is cleared, filled, then compacted (which syncs).
template <class Op>
rg_status edge_map(rg_graph* g, const FView& in, const Op& op, FView* out, const EmOpts& o, cudaStream_t st,
                          int32_t* depth = nullptr, int32_t level = 0, uint32_t* or_into = nullptr) {
  const int64_t nwords = (g->n + 31) / 32;
  if (out) RG_CUDA(cudaMemsetAsync(out->bits, 0, 4 * nwords, st));
  int64_t threshold = o.threshold == -1 ? g->m / std::max<int64_t>(g_opts.dense_div, 1) : o.threshold;
  if (in.count > 0 && in.degsum > 0) {
    g_timing.edges_traversed += in.degsum;
    const bool dense = in.count + in.degsum > threshold;
    uint32_t* nb = out ? out->bits : nullptr;
    // direction 1 pulls dense levels whatever the variant (no atomics; BFS's
    // pull also exits at the first frontier neighbour)
    const bool pull = dense && (!o.dense_forward || g_opts.direction == 1);
    NvtxRange nvtx(pull ? "edgeMap pull" : dense ? "edgeMap dense-push" : "edgeMap sparse-push");
    if (g_trace_on) {
      const int hm_t = (!pull && o.hubs && in.degsum >= kHubMinEdges && g_opts.hub_smem_kb > 0) ? hub_mode_of(o.variant)
                                                                                                : kHubNone;
      g_trace.push_back(rg_level_trace{pull ? 2 : dense ? 1 : 0, hm_t, in.count, in.degsum, threshold});
    }
    const bool tr = o.transpose && g->directed;
    const DevGraph push_g = tr ? g->in_view() : g->view();
    const DevGraph pull_g = tr ? g->view() : g->in_view();
    if (pull) {
      // degree-sorted graphs: 8 lanes per vertex down to degree 8, then one
      // lane per vertex for the tail, where a group would mostly idle through
      // the dependent loads of a short list (RMAT s24 BFS: 8 lanes for every
      // vertex 1.62 ms, 2 for the tail 1.06, 1 for the tail 0.97)
      const uint32_t split = g->sorted ? pull_split(g, pull_g, st) : (uint32_t)g->n;
      auto blocks_for = [&](int64_t nv, int kg) {
        const int64_t groups_per_block = 256 / kg;
        return (unsigned)std::max<int64_t>(
            std::min<int64_t>((nv + groups_per_block - 1) / groups_per_block, (int64_t)device_sms() * 16), 1);
      };
      kt_begin(st);
      if (split > 0) pull_kernel<Op, 8><<<blocks_for(split, 8), 256, 0, st>>>(pull_g, in.bits, op, nb, 0u, split);
      if (split < (uint32_t)g->n) {
        pull_kernel<Op, 1><<<blocks_for(g->n - split, 1), 256, 0, st>>>(pull_g, in.bits, op, nb, split,
                                                                          (uint32_t)g->n);
      }
      kt_end(st);
      RG_CUDA(cudaGetLastError());
      g_timing.kernel_launches += (split > 0 ? 1 : 0) + (split < (uint32_t)g->n ? 1 : 0);
      g_timing.edge_launches++;
    } else {
      int hm = (o.hubs && in.degsum >= kHubMinEdges && g_opts.hub_smem_kb > 0) ? hub_mode_of(o.variant) : kHubNone;
      HubInfo hub;
      if (hm == kHubPrefix) {
        hub.H = o.hub_h ? std::min<uint32_t>(o.hub_h, hub_budget(sizeof(typename Op::HubT), g->n))
                        : hub_budget(sizeof(typename Op::HubT), g->n);
        RG_TRY(launch_push<Op, kHubPrefix>(g, push_g, in, op, hub, nb, st));
      } else if (hm == kHubMap) {
        uint32_t H = o.hub_h ? std::min<uint32_t>(o.hub_h, hub_budget(sizeof(typename Op::HubT), g->n))
                             : hub_budget(sizeof(typename Op::HubT), g->n);
        RG_TRY(hub_map(g, H, hub));
        RG_TRY(launch_push<Op, kHubMap>(g, push_g, in, op, hub, nb, st));
      } else {
        RG_TRY(launch_push<Op, kHubNone>(g, push_g, in, op, hub, nb, st));
      }
    }
  }
  if (out) {
    Frontier tmp;  // non-owning shell for compact_bits
    tmp.bits.p = out->bits;
    RG_TRY(compact_bits(g, tmp, st, true, depth, level, or_into, out->queue, out->qoff,
                        (o.transpose && g->directed) ? g->in_off.as<uint32_t>() : nullptr));
    tmp.bits.p = nullptr;
    out->count = tmp.count;
    out->degsum = tmp.degsum;
    g_timing.kernel_launches += 3;
  }
  return RG_OK;
}

// ---------------------------------------------------------------------------
// small vertex kernels
// ---------------------------------------------------------------------------

}  // namespace rg
