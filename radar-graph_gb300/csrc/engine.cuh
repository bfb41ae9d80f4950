// The frontier engine: device operators, edge-balanced push with optional
// shared-memory hub privatisation, pull with early exit, and the edgeMap mode
// switch.  Reference: ligra.h:61-316 (edgeMapDense / edgeMapDenseForward /
// edgeMapSparse / edgeMapData), vertex.h:12-79 (neighbour decode),
// app functors PageRank.C:29-72, BFS.C:28-99, BC-manyiter-v2.C:32-161,
// Radii.C:37-106.
//
// GPU mapping of the three reference modes:
//  * sparse push and dense push both run `push_lbs`: the frontier is a
//    compacted id queue with an exclusive scan of degrees (qoff); each CTA
//    owns a fixed tile of the frontier's concatenated out-edges, so hubs and
//    leaves cost the same per edge (load-balanced search).  The reference's
//    two push modes differ only in how the CPU finds active vertices; results
//    are identical.
//  * pull runs `pull_kernel`: a group of lanes per vertex scans its
//    in-neighbours against the frontier bitmap, with the early exit of
//    decodeInNghBreakEarly for BFS.
//  * HUBDUP/RADAR: the accumulators of hub vertices live in shared memory,
//    one private copy per CTA (the reference keeps one per OpenMP thread),
//    and are merged into global memory once per launch.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "rg_device.cuh"

namespace rg {

enum PullKind { kPullFirst = 0, kPullSum = 1, kPullOr = 2 };
enum HubMode { kHubNone = 0, kHubPrefix = 1, kHubMap = 2 };

// Hub lookup: RADAR -> hub iff id < H (ids are degree-sorted);
// HUBDUP -> bit in a hub bitmap, slot from an index map.
struct HubInfo {
  uint32_t H = 0;
  const uint32_t* bits = nullptr;   // kHubMap: n-bit hub bitmap
  const uint32_t* slot = nullptr;   // kHubMap: vertex -> slot
  const uint32_t* vertex = nullptr; // kHubMap: slot -> vertex
};

template <int kHub>
__device__ __forceinline__ bool hub_slot(const HubInfo& h, uint32_t d, uint32_t& slot) {
  if (kHub == kHubPrefix) {
    slot = d;
    return d < h.H;
  } else if (kHub == kHubMap) {
    if (!bit_test(h.bits, d)) return false;
    slot = h.slot[d];
    return true;
  }
  return false;
}
template <int kHub>
__device__ __forceinline__ uint32_t hub_vertex(const HubInfo& h, uint32_t slot) {
  return kHub == kHubMap ? h.vertex[slot] : slot;
}

// ---------------------------------------------------------------------------
// Operators.  push(): updateAtomic; returns true to activate d.  pull_*:
// edgeMapDense's update, reduced over the group of lanes owning d.
// ---------------------------------------------------------------------------

// PR_F (PageRank.C:30-72): p_next[d] += p_curr[s]/deg(s).  `contrib` holds
// p_curr[s]/deg(s) precomputed (the same IEEE quotient the reference forms
// per edge).
struct OpPr {
  const double* __restrict__ contrib;
  double* p_next;
  using HubT = double;
  static constexpr int kPull = kPullSum;
  static constexpr bool kOutput = false;
  __device__ __forceinline__ bool cond(uint32_t) const { return true; }
  __device__ __forceinline__ bool push(uint32_t s, uint32_t d) const {
    atomicAdd(p_next + d, contrib[s]);
    return false;
  }
  __device__ static HubT hub_identity() { return 0.0; }
  __device__ __forceinline__ void hub_push(HubT* hs, uint32_t slot, uint32_t s, uint32_t) const {
    atomicAdd(hs + slot, contrib[s]);
  }
  __device__ __forceinline__ bool hub_merge(uint32_t v, HubT x) const {
    if (x != 0.0) atomicAdd(p_next + v, x);
    return false;
  }
  using PullT = double;
  __device__ static PullT pull_identity() { return 0.0; }
  __device__ __forceinline__ PullT pull_val(uint32_t u) const { return contrib[u]; }
  __device__ static PullT combine(PullT a, PullT b) { return a + b; }
  __device__ __forceinline__ bool pull_apply(uint32_t v, PullT x) const {
    p_next[v] += x;
    return false;
  }
};

// BFS_F (BFS.C:28-99; push-pull cond/update src/push-pull/Ligra/apps/BFS.C:33-48).
struct OpBfs {
  uint32_t* parents;
  using HubT = uint32_t;
  static constexpr int kPull = kPullFirst;
  static constexpr bool kOutput = true;
  __device__ __forceinline__ bool cond(uint32_t d) const { return parents[d] == kNone; }
  __device__ __forceinline__ bool push(uint32_t s, uint32_t d) const {
    return atomicCAS(parents + d, kNone, s) == kNone;
  }
  __device__ static HubT hub_identity() { return kNone; }
  __device__ __forceinline__ void hub_push(HubT* hs, uint32_t slot, uint32_t s, uint32_t) const {
    if (hs[slot] == kNone) atomicCAS(hs + slot, kNone, s);
  }
  // mergeDuplicates (BFS.C:69-94): a private parent becomes the parent if the
  // vertex is still unvisited.
  __device__ __forceinline__ bool hub_merge(uint32_t v, HubT x) const {
    if (x == kNone || parents[v] != kNone) return false;
    return atomicCAS(parents + v, kNone, x) == kNone;
  }
  using PullT = uint32_t;
  __device__ static PullT pull_identity() { return kNone; }
  __device__ __forceinline__ bool pull_apply(uint32_t v, uint32_t u) const {
    parents[v] = u;
    return true;
  }
};

// BC_F (BC-manyiter-v2.C:32-101): num_paths[d] += num_paths[s] for unvisited
// d; d joins the next frontier when it receives its first paths.
struct OpBcFwd {
  double* num_paths;
  const uint32_t* __restrict__ visited;
  using HubT = double;
  static constexpr int kPull = kPullSum;
  static constexpr bool kOutput = true;
  __device__ __forceinline__ bool cond(uint32_t d) const { return !bit_test(visited, d); }
  __device__ __forceinline__ bool push(uint32_t s, uint32_t d) const {
    atomicAdd(num_paths + d, num_paths[s]);
    return true;  // every unvisited target joins the next frontier (bitmap dedups)
  }
  __device__ static HubT hub_identity() { return 0.0; }
  __device__ __forceinline__ void hub_push(HubT* hs, uint32_t slot, uint32_t s, uint32_t) const {
    atomicAdd(hs + slot, num_paths[s]);
  }
  __device__ __forceinline__ bool hub_merge(uint32_t v, HubT x) const {
    if (x == 0.0) return false;
    atomicAdd(num_paths + v, x);
    return true;
  }
  using PullT = double;
  __device__ static PullT pull_identity() { return 0.0; }
  __device__ __forceinline__ PullT pull_val(uint32_t u) const { return num_paths[u]; }
  __device__ static PullT combine(PullT a, PullT b) { return a + b; }
  __device__ __forceinline__ bool pull_apply(uint32_t v, PullT x) const {
    double o = num_paths[v];
    num_paths[v] = o + x;
    return x != 0.0 || o != 0.0;
  }
};

// BC_Back_F (BC-manyiter-v2.C:103-161): deps[d] += deps[s] for unvisited d.
struct OpBcBwd {
  double* deps;
  const uint32_t* __restrict__ visited;
  using HubT = double;
  static constexpr int kPull = kPullSum;
  static constexpr bool kOutput = false;
  __device__ __forceinline__ bool cond(uint32_t d) const { return !bit_test(visited, d); }
  __device__ __forceinline__ bool push(uint32_t s, uint32_t d) const {
    atomicAdd(deps + d, deps[s]);
    return false;
  }
  __device__ static HubT hub_identity() { return 0.0; }
  __device__ __forceinline__ void hub_push(HubT* hs, uint32_t slot, uint32_t s, uint32_t) const {
    atomicAdd(hs + slot, deps[s]);
  }
  __device__ __forceinline__ bool hub_merge(uint32_t v, HubT x) const {
    if (x != 0.0) atomicAdd(deps + v, x);
    return false;
  }
  using PullT = double;
  __device__ static PullT pull_identity() { return 0.0; }
  __device__ __forceinline__ PullT pull_val(uint32_t u) const { return deps[u]; }
  __device__ static PullT combine(PullT a, PullT b) { return a + b; }
  __device__ __forceinline__ bool pull_apply(uint32_t v, PullT x) const {
    deps[v] += x;
    return false;
  }
};

// Radii_F (Radii.C:37-106): OR the source's mask into next_visited[d] when it
// adds bits; radii[d] = round; d joins the next frontier.
struct OpRadii {
  const unsigned long long* __restrict__ visited;
  unsigned long long* next_visited;
  int32_t* radii;
  int32_t round;
  using HubT = unsigned long long;
  static constexpr int kPull = kPullOr;
  static constexpr bool kOutput = true;
  __device__ __forceinline__ bool cond(uint32_t) const { return true; }
  __device__ __forceinline__ bool push(uint32_t s, uint32_t d) const {
    unsigned long long vd = visited[d];
    unsigned long long w = vd | visited[s];
    if (w == vd) return false;
    atomicOr(next_visited + d, w);
    if (radii[d] != round) radii[d] = round;
    return true;
  }
  __device__ static HubT hub_identity() { return 0ull; }
  __device__ __forceinline__ void hub_push(HubT* hs, uint32_t slot, uint32_t s, uint32_t d) const {
    // the OR is privatised; the radius and the activation happen inline as in
    // Radii.C:62-76 (they are idempotent stores)
    unsigned long long vd = visited[d];
    unsigned long long w = vd | visited[s];
    if (w == vd) return;
    atomicOr(hs + slot, w);
  }
  __device__ __forceinline__ bool hub_changes(uint32_t s, uint32_t d) const {
    return (visited[d] | visited[s]) != visited[d];
  }
  __device__ __forceinline__ bool hub_merge(uint32_t v, HubT x) const {
    if (x == 0ull) return false;
    atomicOr(next_visited + v, x);
    return false;
  }
  using PullT = unsigned long long;
  __device__ static PullT pull_identity() { return 0ull; }
  __device__ __forceinline__ PullT pull_val(uint32_t u) const { return visited[u]; }
  __device__ static PullT combine(PullT a, PullT b) { return a | b; }
  __device__ __forceinline__ bool pull_apply(uint32_t v, PullT x) const {
    unsigned long long vd = visited[v];
    unsigned long long w = vd | x;
    if (w == vd) return false;
    next_visited[v] |= w;
    if (radii[v] != round) radii[v] = round;
    return true;
  }
};

template <class Op> struct IsRadii { static constexpr bool value = false; };
template <> struct IsRadii<OpRadii> { static constexpr bool value = true; };

// ---------------------------------------------------------------------------
// push over a compacted frontier, edge-balanced
// ---------------------------------------------------------------------------
constexpr int kPushThreads = 256;     // plain push
constexpr int kHubPushThreads = 1024; // hub push: one large CTA per SM keeps occupancy with big hub arrays
constexpr int kPushItems = 4;

template <class Op, int kHub, int kThreads>
__global__ void __launch_bounds__(kThreads) push_lbs(DevGraph g, const uint32_t* __restrict__ queue,
                                                         const uint32_t* __restrict__ qoff, uint32_t k,
                                                         uint32_t total, Op op, HubInfo hub,
                                                         uint32_t* __restrict__ next_bits) {
  constexpr int kPushTile = kThreads * kPushItems;
  constexpr int kPushCap = kPushTile + 1;  // staged frontier entries per tile
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using HubT = typename Op::HubT;
  HubT* hs = reinterpret_cast<HubT*>(smem_raw);
  __shared__ uint32_t s_i0, s_i1;
  __shared__ uint32_t s_q[kPushCap], s_qo[kPushCap], s_base[kPushCap];
  if (kHub != kHubNone) {
    for (uint32_t h = threadIdx.x; h < hub.H; h += blockDim.x) hs[h] = Op::hub_identity();
    __syncthreads();
  }
  for (uint64_t tile = blockIdx.x; tile * kPushTile < total; tile += gridDim.x) {
    const uint32_t e0 = (uint32_t)(tile * kPushTile);
    const uint32_t e1 = min(e0 + (uint32_t)kPushTile, total);
    if (threadIdx.x == 0) {
      uint32_t i0 = upper_index(qoff, 0u, k - 1, e0);
      s_i0 = i0;
      s_i1 = upper_index(qoff, i0, k - 1, e1 - 1);
    }
    __syncthreads();
    const uint32_t i0 = s_i0, i1 = s_i1, r = i1 - i0 + 1;
    const bool staged = r <= (uint32_t)kPushCap;
    if (staged) {
      for (uint32_t j = threadIdx.x; j < r; j += blockDim.x) {
        uint32_t s = queue[i0 + j];
        s_q[j] = s;
        s_qo[j] = qoff[i0 + j];
        s_base[j] = g.off[s];
      }
    }
    __syncthreads();
    for (uint32_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
      uint32_t s, pos;
      if (staged) {
        uint32_t li = upper_index(s_qo, 0u, r - 1, e);
        s = s_q[li];
        pos = s_base[li] + (e - s_qo[li]);
      } else {
        uint32_t gi = upper_index(qoff, i0, i1, e);
        s = queue[gi];
        pos = g.off[s] + (e - qoff[gi]);
      }
      const uint32_t d = g.adj[pos];
      if (!op.cond(d)) continue;
      uint32_t slot;
      if (kHub != kHubNone && hub_slot<kHub>(hub, d, slot)) {
        if constexpr (IsRadii<Op>::value) {
          if (op.hub_changes(s, d)) {
            op.hub_push(hs, slot, s, d);
            if (op.radii[d] != op.round) op.radii[d] = op.round;
            bit_set(next_bits, d);
          }
        } else {
          op.hub_push(hs, slot, s, d);
        }
      } else if (op.push(s, d) && Op::kOutput) {
        bit_set(next_bits, d);
      }
    }
    __syncthreads();
  }
  if (kHub != kHubNone) {
    __syncthreads();
    for (uint32_t h = threadIdx.x; h < hub.H; h += blockDim.x) {
      uint32_t v = hub_vertex<kHub>(hub, h);
      if (op.hub_merge(v, hs[h]) && Op::kOutput) bit_set(next_bits, v);
    }
  }
}

// ---------------------------------------------------------------------------
// pull (edgeMapDense + decodeInNghBreakEarly), a group of kG lanes per vertex
// ---------------------------------------------------------------------------
template <class Op, int kG>
__global__ void __launch_bounds__(256) pull_kernel(DevGraph g, const uint32_t* __restrict__ fbits, Op op,
                                                   uint32_t* __restrict__ next_bits) {
  const int lane = threadIdx.x & 31;
  const int gl = lane % kG;
  const unsigned gmask = (kG == 32) ? 0xffffffffu : (((1u << kG) - 1u) << (lane - gl));
  const uint64_t group = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / kG;
  const uint64_t ngroups = ((uint64_t)gridDim.x * blockDim.x) / kG;
  for (uint64_t vv = group; vv < g.n; vv += ngroups) {
    const uint32_t v = (uint32_t)vv;
    if (!op.cond(v)) continue;
    const uint32_t b = g.off[v], e = g.off[v + 1];
    if constexpr (Op::kPull == kPullFirst) {
      for (uint32_t j0 = b; j0 < e; j0 += kG) {
        const uint32_t j = j0 + gl;
        uint32_t u = 0;
        bool in = false;
        if (j < e) {
          u = g.adj[j];
          in = bit_test(fbits, u);
        }
        const unsigned bal = __ballot_sync(gmask, in) & gmask;
        if (bal) {
          const int first = __ffs(bal) - 1;
          const uint32_t pu = __shfl_sync(gmask, u, first);
          if (gl == 0 && op.pull_apply(v, pu)) bit_set(next_bits, v);
          break;
        }
      }
    } else {
      typename Op::PullT acc = Op::pull_identity();
      for (uint32_t j = b + gl; j < e; j += kG) {
        const uint32_t u = g.adj[j];
        if (bit_test(fbits, u)) acc = Op::combine(acc, op.pull_val(u));
      }
#pragma unroll
      for (int o = kG / 2; o > 0; o >>= 1) acc = Op::combine(acc, __shfl_xor_sync(gmask, acc, o));
      if (gl == 0) {
        bool has = true;
        if constexpr (Op::kPull == kPullOr) has = acc != 0ull;
        if (has && op.pull_apply(v, acc) && Op::kOutput) bit_set(next_bits, v);
      }
    }
  }
}

}  // namespace rg
