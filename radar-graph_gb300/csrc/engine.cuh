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
  // hub copies are FP64 like the reference's thread-private p_next_dup
  // (PageRank.C:42-70): shared-memory double adds, merged with one add
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
// With `visited` (union of all frontiers so far) and `next` (the bitmap being
// built) the unvisited test reads two L2-resident bitmaps instead of the
// parent array; without them it reads parents[d] like the reference's cond.
struct OpBfs {
  uint32_t* parents;
  const uint32_t* visited = nullptr;
  const uint32_t* next = nullptr;
  using HubT = uint32_t;
  static constexpr int kPull = kPullFirst;
  static constexpr bool kOutput = true;
  __device__ __forceinline__ bool cond(uint32_t d) const {
    if (visited) return !bit_test(visited, d) && !(next && (__ldcg(next + (d >> 5)) >> (d & 31) & 1u));
    return parents[d] == kNone;
  }
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

// PageRankDelta's PR_F (PageRankDelta.C:29-46): nghSum[d] += Delta[s]/deg(s),
// no output.  `c` holds Delta[s]/deg(s) for the frontier (the same IEEE
// quotient the reference forms per edge), 0 elsewhere.  FP64 like the
// reference: deltas shrink geometrically, below what fixed point resolves.
struct OpPrDelta {
  const double* __restrict__ c;
  double* ngh;
  using HubT = double;
  static constexpr int kPull = kPullSum;
  static constexpr bool kOutput = false;
  __device__ __forceinline__ bool cond(uint32_t) const { return true; }
  __device__ __forceinline__ bool push(uint32_t s, uint32_t d) const {
    atomicAdd(ngh + d, c[s]);
    return false;
  }
  __device__ static HubT hub_identity() { return 0.0; }
  __device__ __forceinline__ void hub_push(HubT* hs, uint32_t slot, uint32_t s, uint32_t) const {
    atomicAdd(hs + slot, c[s]);
  }
  __device__ __forceinline__ bool hub_merge(uint32_t v, HubT x) const {
    if (x != 0.0) atomicAdd(ngh + v, x);
    return false;
  }
  using PullT = double;
  __device__ static PullT pull_identity() { return 0.0; }
  __device__ __forceinline__ PullT pull_val(uint32_t u) const { return c[u]; }
  __device__ static PullT combine(PullT a, PullT b) { return a + b; }
  __device__ __forceinline__ bool pull_apply(uint32_t v, PullT x) const {
    ngh[v] += x;
    return false;
  }
};

// BC_F (BC-manyiter-v2.C:32-101): num_paths[d] += num_paths[s] for unvisited
// d; d joins the next frontier when it receives its first paths.  kMark
// false: the same adds without marking the next frontier, which the caller
// then reads off the counts (an unvisited vertex with paths was reached).
template <bool kMark>
struct OpBcFwdT {
  double* num_paths;
  const uint32_t* __restrict__ visited;
  using HubT = double;
  static constexpr int kPull = kPullSum;
  static constexpr bool kOutput = kMark;
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
using OpBcFwd = OpBcFwdT<true>;

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

// Multi-source BFS level (rg_bfs_multi, rg_bc_multi): bit q of F[s] says s is
// in source q's frontier; the bits that reach d for the first time are ORed
// into N[d] (Radii_F's mask propagation, one bit per source).
struct OpMsBfs {
  const unsigned long long* __restrict__ F;
  const unsigned long long* __restrict__ seen;
  unsigned long long* N;
  using HubT = unsigned long long;
  static constexpr int kPull = kPullOr;
  static constexpr bool kOutput = true;
  __device__ __forceinline__ bool cond(uint32_t) const { return true; }
  __device__ __forceinline__ bool push(uint32_t s, uint32_t d) const {
    const unsigned long long w = F[s] & ~seen[d];
    if (!w) return false;
    atomicOr(N + d, w);
    return true;
  }
  __device__ static HubT hub_identity() { return 0ull; }
  __device__ __forceinline__ void hub_push(HubT* hs, uint32_t slot, uint32_t s, uint32_t d) const {
    const unsigned long long w = F[s] & ~seen[d];
    if (w) atomicOr(hs + slot, w);
  }
  __device__ __forceinline__ bool hub_changes(uint32_t s, uint32_t d) const { return (F[s] & ~seen[d]) != 0; }
  __device__ __forceinline__ bool hub_merge(uint32_t v, HubT x) const {
    if (!x) return false;
    atomicOr(N + v, x);
    return true;
  }
  using PullT = unsigned long long;
  __device__ static PullT pull_identity() { return 0ull; }
  __device__ __forceinline__ PullT pull_val(uint32_t u) const { return F[u]; }
  __device__ static PullT combine(PullT a, PullT b) { return a | b; }
  __device__ __forceinline__ bool pull_apply(uint32_t v, PullT x) const {
    const unsigned long long w = x & ~seen[v];
    if (!w) return false;
    N[v] |= w;
    return true;
  }
};

// Radii_F (Radii.C:37-106): OR the source's mask into next_visited[d] when it
// adds bits; d joins the next frontier.  radii[d] = round is written for
// every member of the next frontier by the compaction that follows (the same
// set the reference's CAS on radii activates).
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
    return true;
  }
};

template <class Op> struct IsRadii { static constexpr bool value = false; };
template <> struct IsRadii<OpRadii> { static constexpr bool value = true; };

// ---------------------------------------------------------------------------
// push over a compacted frontier, edge-balanced
//
// Each CTA owns tiles of kThreads*kPushItems consecutive frontier edges.  The
// frontier entries overlapping a tile are staged in shared memory and every
// tile position learns its owning entry by a scatter (entry j marks the
// position where its edges start) followed by a block-wide max-scan, so a
// lane finds its source in O(1) instead of a binary search per edge.
// ---------------------------------------------------------------------------
constexpr int kPushThreads = 256;     // plain push
constexpr int kHubPushThreads = 256;  // hub push: small CTAs with a bounded hub array keep occupancy
constexpr int kPushItems = 4;
// push_lbs zeroes and max-scans a thread's owner slots as one uint4: one slot
// per edge the thread takes, so exactly four
static_assert(kPushItems == 4, "push_lbs's owner scan handles four slots per thread");

template <int kThreads>
__device__ __forceinline__ uint32_t block_max_scan_prefix(uint32_t v) {
  // returns max over threads < threadIdx.x (0 for thread 0)
  __shared__ uint32_t warp_max[kThreads / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc = max(inc, t);
  }
  if (lane == 31) warp_max[w] = inc;
  __syncthreads();
  if (w == 0) {
    uint32_t t = lane < kThreads / 32 ? warp_max[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t u = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t = max(t, u);
    }
    if (lane < kThreads / 32) warp_max[lane] = t;
  }
  __syncthreads();
  uint32_t ex = __shfl_up_sync(0xffffffffu, inc, 1);
  if (lane == 0) ex = 0;
  if (w > 0) ex = max(ex, warp_max[w - 1]);
  __syncthreads();
  return ex;
}

// ts[t] = the frontier entry holding edge t*tile (t < ntiles); ts[ntiles] =
// the entry holding the last edge.  One thread per tile, so the searches of
// all tiles overlap instead of stalling each CTA.
static __global__ void tile_starts(const uint32_t* __restrict__ qoff, uint32_t k, uint32_t total, uint32_t tile,
                            uint32_t ntiles, uint32_t* __restrict__ ts) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t > ntiles) return;
  const uint32_t e = t < ntiles ? t * tile : total - 1;
  ts[t] = upper_index(qoff, 0u, k - 1, e);
}

template <class Op, int kHub, int kThreads>
__global__ void __launch_bounds__(kThreads) push_lbs(DevGraph g, const uint32_t* __restrict__ queue,
                                                     const uint32_t* __restrict__ qoff,
                                                     const uint32_t* __restrict__ tstart, uint32_t total, Op op,
                                                     HubInfo hub, uint32_t* __restrict__ next_bits) {
  constexpr int kTile = kThreads * kPushItems;
  constexpr int kCap = kTile + 1;  // staged frontier entries per tile
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using HubT = typename Op::HubT;
  HubT* hs = reinterpret_cast<HubT*>(smem_raw);
  __shared__ __align__(16) uint32_t s_owner[kTile];
  __shared__ uint32_t s_q[kCap], s_qo[kCap], s_base[kCap];
  if (kHub != kHubNone) {
    for (uint32_t h = threadIdx.x; h < hub.H; h += kThreads) hs[h] = Op::hub_identity();
    __syncthreads();
  }
  for (uint64_t tile = blockIdx.x; tile * kTile < total; tile += gridDim.x) {
    const uint32_t e0 = (uint32_t)(tile * kTile);
    const uint32_t e1 = min(e0 + (uint32_t)kTile, total);
    // entries [i0, i1] cover the tile (i1 may be one past: an entry whose
    // edges start exactly at e1 is staged but never owns a position)
    const uint32_t i0 = tstart[tile], i1 = tstart[tile + 1], r = i1 - i0 + 1;
    reinterpret_cast<uint4*>(s_owner)[threadIdx.x] = make_uint4(0, 0, 0, 0);
    __syncthreads();
    const bool staged = r <= (uint32_t)kCap;
    if (staged) {
      for (uint32_t j = threadIdx.x; j < r; j += kThreads) {
        const uint32_t s = queue[i0 + j];
        const uint32_t qo = qoff[i0 + j];
        s_q[j] = s;
        s_qo[j] = qo;
        s_base[j] = g.off[s];
        if (j > 0 && qo < e1) atomicMax(&s_owner[qo - e0], j);
      }
      __syncthreads();
      // inclusive max-scan of the owner marks: position p -> last entry starting at or before p
      uint4 w4 = reinterpret_cast<uint4*>(s_owner)[threadIdx.x];
      w4.y = max(w4.y, w4.x);
      w4.z = max(w4.z, w4.y);
      w4.w = max(w4.w, w4.z);
      const uint32_t pre = block_max_scan_prefix<kThreads>(w4.w);
      w4.x = max(w4.x, pre);
      w4.y = max(w4.y, pre);
      w4.z = max(w4.z, pre);
      w4.w = max(w4.w, pre);
      reinterpret_cast<uint4*>(s_owner)[threadIdx.x] = w4;
      __syncthreads();
    }
    // A thread's kPushItems edges go through each stage together -- their
    // neighbour ids, then their cond tests, then the updates -- so the
    // scattered loads of one stage overlap instead of forming one chain per
    // edge.  cond is only a filter (the update itself decides, as with
    // Ligra's concurrent threads), so testing it before this thread's
    // earlier updates changes no result.
    uint32_t sv[kPushItems], dv[kPushItems];
    bool live[kPushItems];
#pragma unroll
    for (int i = 0; i < kPushItems; i++) {
      const uint32_t e = e0 + threadIdx.x + (uint32_t)i * kThreads;
      live[i] = e < e1;
      sv[i] = 0;
      dv[i] = 0;
      if (live[i]) {
        uint32_t s, pos;
        if (staged) {
          const uint32_t li = s_owner[e - e0];
          s = s_q[li];
          pos = s_base[li] + (e - s_qo[li]);
        } else {
          const uint32_t gi = upper_index(qoff, i0, i1, e);
          s = queue[gi];
          pos = g.off[s] + (e - qoff[gi]);
        }
        sv[i] = s;
        dv[i] = g.adj[pos];
      }
    }
#pragma unroll
    for (int i = 0; i < kPushItems; i++) live[i] = live[i] && op.cond(dv[i]);
#pragma unroll
    for (int i = 0; i < kPushItems; i++) {
      if (!live[i]) continue;
      const uint32_t s = sv[i], d = dv[i];
      uint32_t slot;
      if (kHub != kHubNone && hub_slot<kHub>(hub, d, slot)) {
        if constexpr (IsRadii<Op>::value) {
          if (op.hub_changes(s, d)) {
            op.hub_push(hs, slot, s, d);
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
    for (uint32_t h = threadIdx.x; h < hub.H; h += kThreads) {
      const uint32_t v = hub_vertex<kHub>(hub, h);
      if (op.hub_merge(v, hs[h]) && Op::kOutput) bit_set(next_bits, v);
    }
  }
}

// ---------------------------------------------------------------------------
// Dense round of a bitmask traversal (Radii, multi-source BFS) as a pull over
// every edge: next[v] |= (OR of visited[u] over all neighbours u) & ~visited[v],
// and v joins the next frontier when that adds bits.  `visited` is the mask
// each vertex had when the round began (Radii's synced Visited, the BFS
// `seen` set).  No frontier test is needed: a neighbour outside the frontier
// last changed two or more rounds ago and pushed its unchanged mask to v
// then, so its bits are already in visited[v]; the new bits and the next
// frontier are exactly those of the push over the frontier (Radii.C:51-76).
// Edge-balanced like the PageRank sweep: 8 or 16 edges per lane (streamed
// 32-byte id loads, gathers in batches of 8), row pieces combined by one
// segmented OR scan per warp step, one atomicOr and activation per row piece
// that adds bits.
// ---------------------------------------------------------------------------
static __device__ __forceinline__ void mask_flush(const unsigned long long* __restrict__ visited,
                                            unsigned long long* next_visited, uint32_t* next_bits, uint32_t row,
                                            unsigned long long part) {
  if (!part) return;
  const unsigned long long vd = __ldg(visited + row);
  const unsigned long long w = part & ~vd;
  if (!w) return;
  atomicOr(next_visited + row, w);
  bit_set(next_bits, row);
}

// `full`: the bits any vertex can still receive -- those of the sources that
// have out-edges (a source without them is no vertex's in-neighbour, so its
// bit never spreads; collisions that lost a bit drop it too).  A row whose
// mask already holds all of `full` cannot grow, so its edges are not
// gathered: in the last dense rounds that is most of the graph (RMAT s22,
// 64 samples: 64 % of the edges in round 4, 99.8 % in round 5), and the hub
// rows, which hold the most edges, fill first.  full = 0 gathers every row.
template <int kItems>
static __global__ void __launch_bounds__(256) mask_pull_sweep(DevGraph g, const uint32_t* __restrict__ chunk_v,
                                                        uint32_t nchunks, const unsigned long long* __restrict__ visited,
                                                        unsigned long long* next_visited, uint32_t* next_bits,
                                                        unsigned long long full) {
  static_assert(kItems == 8 || kItems == 16, "8 or 16 edges per lane");
  constexpr int kStep = 32 * kItems;
  constexpr int kBatch = 8;  // gathers in flight per lane at a time
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t c = warp; c < nchunks; c += nwarps) {
    const uint32_t vlo = chunk_v[c], vhi = chunk_v[c + 1];
#pragma unroll
    for (int r = 0; r < kSweepChunk / kStep; r++) {
      const uint32_t e = c * kSweepChunk + r * kStep + lane * kItems;
      uint32_t row = kNone;
      unsigned long long part = 0;
      if (e < g.m) {
        uint32_t v = upper_index(g.off, vlo, vhi, e);
        uint32_t nxt = g.off[v + 1];
        // the rows of the lane's edges first, then gathers only for rows
        // that can still grow.  8 edges per lane keep the rows in registers;
        // 16 walk them again while accumulating (the offsets hit L1), which
        // keeps the kernel at 8 gathers and 8 row ids per lane
        constexpr bool kKeepRows = kItems <= 8;
        uint32_t rowi[kKeepRows ? kItems : 1];
        unsigned need = 0;
        {
          uint32_t rv = v, rn = nxt;
          bool open = full == 0ull || (__ldg(visited + rv) & full) != full;
#pragma unroll
          for (int i = 0; i < kItems; i++) {
            const uint32_t ee = e + i;
            if (ee < g.m && ee >= rn) {
              do { rv++; rn = g.off[rv + 1]; } while (ee >= rn);
              open = full == 0ull || (__ldg(visited + rv) & full) != full;
            }
            if (kKeepRows) rowi[kKeepRows ? i : 0] = rv;
            if (ee < g.m && open) need |= 1u << i;
          }
        }
        row = v;
#pragma unroll
        for (int b = 0; b < kItems; b += kBatch) {
          if (e + b >= g.m) break;
          // this batch's neighbour ids (in bounds: adj is padded by 8
          // entries and the batch starts before m)
          const U32x8 w = ld_stream_v8(g.adj + e + b);
          unsigned long long x[kBatch];
#pragma unroll
          for (int j = 0; j < kBatch; j++) x[j] = ((need >> (b + j)) & 1u) ? __ldg(visited + w.v[j]) : 0ull;
#pragma unroll
          for (int j = 0; j < kBatch; j++) {
            const int i = b + j;
            const uint32_t ee = e + i;
            if (ee >= g.m) break;
            const bool ends = kKeepRows ? rowi[kKeepRows ? i : 0] != row : ee >= nxt;
            if (ends) {
              mask_flush(visited, next_visited, next_bits, row, part);  // a row piece that ends in this lane
              part = 0;
              if (kKeepRows) {
                row = rowi[kKeepRows ? i : 0];
              } else {
                do { v++; nxt = g.off[v + 1]; } while (ee >= nxt);
                row = v;
              }
            }
            part |= x[j];
          }
        }
      }
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned long long t = __shfl_up_sync(0xffffffffu, part, o);
        const uint32_t tr = __shfl_up_sync(0xffffffffu, row, o);
        if (lane >= o && tr == row) part |= t;
      }
      const uint32_t next_row = __shfl_down_sync(0xffffffffu, row, 1);
      if (row != kNone && (lane == 31 || next_row != row)) mask_flush(visited, next_visited, next_bits, row, part);
    }
  }
}

// ---------------------------------------------------------------------------
// pull (edgeMapDense + decodeInNghBreakEarly), a group of kG lanes per vertex
// ---------------------------------------------------------------------------
// Vertices [vlo, vhi), a group of kG lanes per vertex.
template <class Op, int kG>
__global__ void __launch_bounds__(256) pull_kernel(DevGraph g, const uint32_t* __restrict__ fbits, Op op,
                                                   uint32_t* __restrict__ next_bits, uint32_t vlo, uint32_t vhi) {
  const int lane = threadIdx.x & 31;
  const int gl = lane % kG;
  const unsigned gmask = (kG == 32) ? 0xffffffffu : (((1u << kG) - 1u) << (lane - gl));
  const uint64_t group = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / kG;
  const uint64_t ngroups = ((uint64_t)gridDim.x * blockDim.x) / kG;
  for (uint64_t vv = vlo + group; vv < vhi; vv += ngroups) {
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
