// Internal device-side declarations: the device graph image, the frontier,
// per-graph workspace, and small primitives (scan, block reductions).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <atomic>
#include <mutex>
#include <utility>
#include <vector>

#include "rg_host.h"

namespace rg {

constexpr uint32_t kNone = 0xFFFFFFFFu;  // UINT_E_MAX
constexpr int kSweepChunk = 512;         // edges per warp chunk of a full-graph sweep

rg_status cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define RG_CUDA(...)                                                                  \
  do {                                                                                \
    cudaError_t e_ = (__VA_ARGS__);                                                   \
    if (e_ != cudaSuccess) return ::rg::cuda_fail(e_, #__VA_ARGS__, __FILE__, __LINE__); \
  } while (0)
#define RG_TRY(...)                 \
  do {                              \
    rg_status s_ = (__VA_ARGS__);   \
    if (s_ != RG_OK) return s_;     \
  } while (0)

// Host arrays of n entries that are always overwritten in full: growing them
// does not zero the memory first (a 67 MB zero-fill per graph otherwise).
template <class T>
struct NoInit : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = NoInit<U>;
  };
  NoInit() = default;
  template <class U>
  NoInit(const NoInit<U>&) {}
  template <class U>
  void construct(U*) noexcept {}
  template <class U, class... A>
  void construct(U* p, A&&... a) {
    ::new ((void*)p) U(std::forward<A>(a)...);
  }
};
using HostU32 = std::vector<uint32_t, NoInit<uint32_t>>;

// Kernel view of a symmetric CSR graph.
struct DevGraph {
  uint32_t n;
  uint32_t m;
  const uint32_t* __restrict__ off;  // n+1
  const uint32_t* __restrict__ adj;  // m (+8 zero padding, 32-byte aligned)
};

// A device allocation that frees itself.  `pooled` buffers (a graph's CSR
// image) come from the device's stream-ordered pool, which keeps freed blocks
// mapped for the next graph instead of returning them to the driver; their
// owner makes sure no work still uses them when they are released.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  bool pooled = false;
  cudaStream_t free_stream = nullptr;  // pooled: the release is ordered after this stream's work
  DevBuf() = default;
  explicit DevBuf(bool from_pool, cudaStream_t stream = nullptr) : pooled(from_pool), free_stream(stream) {}
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) {
      if (pooled) cudaFreeAsync(p, free_stream);
      else cudaFree(p);
    }
    p = nullptr;
    bytes = 0;
  }
  // Grows (never shrinks) to at least `b` bytes; contents are not kept.
  rg_status reserve(size_t b);
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// Device frontier: compacted queue of ids (ascending when produced by the
// engine), the exclusive scan of their degrees (for edge-balanced push), and
// a bitmap.  `count`/`degsum` mirror the device values after a sync.
struct Frontier {
  DevBuf queue;   // n+64 ids
  DevBuf qoff;    // n+65 scan entries
  DevBuf bits;    // (n+31)/32 words (+pad)
  int64_t count = 0;
  int64_t degsum = 0;
  bool queue_valid = false;
  bool bits_valid = false;
};

// Scratch reused by every call on a graph (no per-level cudaMalloc).
struct Workspace {
  DevBuf scan_partials;  // scan / compaction block partials
  DevBuf scan_tmp;
  DevBuf tiles;          // push tile -> first frontier entry
  DevBuf counters;       // small device scalars
  DevBuf lookup;         // lookup_ids staging
  uint64_t* h_info = nullptr;      // pinned, mapped host mirror of level info (count, degsum, ...)
  uint64_t* h_info_dev = nullptr;  // the device's address of h_info (kernels write it directly)
  unsigned char* h_small = nullptr;      // pinned, mapped scratch for small reads (read_small)
  unsigned char* h_small_dev = nullptr;  // its device address
  ~Workspace();
};

}  // namespace rg

namespace rg {
// Scheduling options (RG_OPT_*); none of them changes a result.
struct Options {
  int64_t direction = 0;     // RG_OPT_DIRECTION
  int64_t hub_slots = 0;     // RG_OPT_HUB_SLOTS
  int64_t hub_smem_kb = 48;  // RG_OPT_HUB_SMEM_KB (0 = no hub copies in the frontier push)
  int64_t dense_div = 20;    // RG_OPT_DENSE_DIV
  int64_t sweep_shape = 161;  // RG_OPT_SWEEP_SHAPE
  int64_t bc_fwd_hubs = 1;   // RG_OPT_BC_FWD_HUBS
  int64_t async_results = 0;  // RG_OPT_ASYNC_RESULTS (per thread: a graph's tuning keeps the thread's)
};

// Per-thread execution context: the stream the calling thread's work goes
// to, two timing events and the scratch of the engine.  Graphs are shared
// read-only between threads, so several queries on one resident graph can be
// in flight on different threads (one stream each).
struct Ctx {
  int device = -1;
  cudaStream_t stream = nullptr;
  cudaStream_t own_stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // result copies of RG_OPT_ASYNC_RESULTS (created on first use)
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  Workspace ws;
};
// The calling thread's context for the current device (created on first use).
rg_status get_ctx(Ctx** out);
Ctx& ctx();  // only after a successful get_ctx on this thread
}  // namespace rg

struct rg_graph {
  int device = 0;
  uint64_t uid = 0;  // unique per graph in the process (device addresses can repeat)
  int64_t n = 0, m = 0;
  rg::DevBuf off{true}, adj{true};  // CSR on the device (out-lists)
  rg::DevBuf chunk_v{true};         // sweep partition: first vertex of every kSweepChunk edges
  int64_t nchunks = 0;
  // directed graphs: in-lists (CSC, sources ascending) and their partition;
  // a symmetric graph's in-lists are its out-lists
  bool directed = false;
  rg::DevBuf in_off{true}, in_adj{true}, in_chunk_v{true};
  bool sorted = false;
  rg::DevBuf new_ids{true};         // orig -> internal (when sorted)
  // Host copies of new_ids and of the degree by internal id.  An uploaded
  // graph has its degrees from creation; a degree-sorted graph copies both
  // on first full use (host_arrays) -- most calls need a few entries (a root,
  // the sources), which lookup_ids reads from the device instead.
  mutable rg::HostU32 h_new_ids;
  mutable rg::HostU32 h_deg;
  mutable rg::HostU32 h_in_deg;  // directed graphs: in-degree by internal id
  mutable bool host_ready = false;
  mutable std::mutex host_mu;
  uint32_t max_deg = 0;
  mutable std::atomic<int64_t> pull_split{-1};  // pull_split()'s cached value, -1 = not yet known
  bool tuned[4] = {false, false, false, false};  // per app: PageRank, BFS, BC, Radii
  rg::Options topt[4];                           // the autotuner's choice per app
  rg::DevGraph view() const {
    return rg::DevGraph{(uint32_t)n, (uint32_t)m, off.as<uint32_t>(), adj.as<uint32_t>()};
  }
  // the lists a pull reads (edges into each vertex) and their partition
  rg::DevGraph in_view() const {
    return directed ? rg::DevGraph{(uint32_t)n, (uint32_t)m, in_off.as<uint32_t>(), in_adj.as<uint32_t>()} : view();
  }
  const uint32_t* in_chunks() const { return directed ? in_chunk_v.as<uint32_t>() : chunk_v.as<uint32_t>(); }
  ~rg_graph();
};

struct rg_frontier {
  const rg_graph* g = nullptr;
  rg::Frontier f;
};

namespace rg {

// Reads `bytes` of device memory into host memory through a kernel that
// writes the thread's mapped scratch (up to kSmallRead bytes; larger reads
// copy): small reads on a level's critical path then never wait behind a
// large copy another stream has on a copy engine.  Syncs `st`.
constexpr size_t kSmallRead = 65536;
rg_status read_small(const void* d_src, void* h_dst, size_t bytes, cudaStream_t st);

// Exclusive scan of `n` uint32 values into out[0..n] (out[n] = total).
// Total must fit 32 bits.  Uses ws.scan_partials.  Async on `st`.
rg_status scan_u32(Workspace& ws, const uint32_t* in, uint32_t* out, int64_t n, cudaStream_t st);

// Builds frontier f (queue+qoff, ascending) from its bitmap.  Writes
// (count, degsum) into ws.h_info[0..1] and syncs the stream if `sync`.
// Optional epilogues: depth[v] = level for every member; or_into |= bits.
// Degrees (for qoff/degsum) come from deg_off (n+1 offsets; default: the
// out-lists).
rg_status compact_bits(const rg_graph* g, Frontier& f, cudaStream_t st, bool sync,
                       int32_t* depth = nullptr, int32_t level = 0, uint32_t* or_into = nullptr,
                       uint32_t* queue_out = nullptr, uint32_t* qoff_out = nullptr,
                       const uint32_t* deg_off = nullptr);

// Fills g's host arrays (h_new_ids when sorted, h_deg) if not yet there.
rg_status host_arrays(const rg_graph* g);
// For k host ids (ORIGINAL ids when `orig`, else internal): the internal id
// and/or the degree (either output may be null).  Few ids are gathered on
// the device; many, or a graph whose host arrays exist, use the host arrays.
// deg_out holds in-degrees when in_degree (directed graphs).
rg_status lookup_ids(const rg_graph* g, const uint32_t* ids, int64_t k, bool orig, uint32_t* internal_out,
                     uint32_t* deg_out, bool in_degree = false);

// Sets a frontier from host ids (queue + qoff from their degrees + bitmap).
rg_status frontier_from_host(const rg_graph* g, Frontier& f, const uint32_t* ids, int64_t k,
                             cudaStream_t st);
rg_status frontier_alloc(const rg_graph* g, Frontier& f);
rg_status frontier_set_all(const rg_graph* g, Frontier& f, cudaStream_t st);
// Bitmap from the current queue (clears first).
rg_status frontier_bits_from_queue(const rg_graph* g, Frontier& f, cudaStream_t st);

// ---- small device helpers ------------------------------------------------

__device__ __forceinline__ bool bit_test(const uint32_t* bits, uint32_t v) {
  return (bits[v >> 5] >> (v & 31)) & 1u;
}
// Sets bit v; skips the atomic when a plain read already shows it set.
__device__ __forceinline__ void bit_set(uint32_t* bits, uint32_t v) {
  uint32_t b = 1u << (v & 31);
  if (!(__ldcg(bits + (v >> 5)) & b)) atomicOr(bits + (v >> 5), b);
}

// ---- cache-policy loads ----------------------------------------------------
// The edge array is streamed once per sweep; the per-vertex values gathered
// through it are re-read many times (hubs most of all).  Streaming loads skip
// L1 and are first out of L2, so the gathered values keep the caches.
struct U32x8 {
  uint32_t v[8];
};
// 32 bytes (8 edges), 32-byte aligned: no L1 allocation, L2 evict-first.
__device__ __forceinline__ U32x8 ld_stream_v8(const uint32_t* p) {
  U32x8 r;
  asm("ld.global.nc.L1::no_allocate.L2::evict_first.v8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=r"(r.v[0]), "=r"(r.v[1]), "=r"(r.v[2]), "=r"(r.v[3]), "=r"(r.v[4]), "=r"(r.v[5]), "=r"(r.v[6]),
        "=r"(r.v[7])
      : "l"(p));
  return r;
}
// 16 bytes (4 edges), no L1 allocation, L2 policy `pol`.
__device__ __forceinline__ uint4 ld_stream_v4(const uint32_t* p, uint64_t pol) {
  uint4 r;
  asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
      : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
      : "l"(p), "l"(pol));
  return r;
}
// An L2 policy that lets lines go first (evict-first).
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t pol;
  asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
// An L2 policy that keeps lines (evict-last) for the loads that carry it.
__device__ __forceinline__ uint64_t policy_evict_last() {
  uint64_t pol;
  asm("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
  return pol;
}
// Read-only 8-byte gather kept in L1 (evict-last) and L2 (policy `pol`).
__device__ __forceinline__ unsigned long long ld_keep_u64(const uint64_t* p, uint64_t pol) {
  unsigned long long r;
  asm("ld.global.nc.L1::evict_last.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(r) : "l"(p), "l"(pol));
  return r;
}

// Largest i in [lo, hi] with a[i] <= x (a non-decreasing, a[lo] <= x).
template <class T>
__device__ __forceinline__ uint32_t upper_index(const T* a, uint32_t lo, uint32_t hi, uint32_t x) {
  while (lo < hi) {
    uint32_t mid = lo + ((hi - lo + 1) >> 1);
    if (a[mid] <= x) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

}  // namespace rg
