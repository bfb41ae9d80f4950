// Oracle: a CPU restatement of RADAR-Graph's edgeMap/vertexMap frontier engine
// and of the PageRank, BFS, BC and Radii apps that drive it.
//
// This file is TEST INFRASTRUCTURE.  Only the tests, the smoke check and the
// CPU-baseline leg of the benchmark load it, and only as the checker or as the
// timed CPU reference arm.  The product (the CUDA library) never calls it.
//
// Parity is pinned: the outputs of this restatement are compared against the
// reference's own OpenMP binaries (built from the reference sources by
// oracle/Makefile into oracle/_ref/) on seeded graphs; the resulting golden
// vectors live in tests/golden/ together with the script that made them.
//
// Every function cites the reference file:line it follows (paths are relative
// to the reference project root, RADAR variant unless another is named).
//
// Variants (argument `variant`):
//   0 push        src/push-new-orig : every app pushes (dense_forward)
//   1 push-pull   src/push-pull     : dense iterations pull (edgeMapDense)
//   2 degsort     src/degree-sorting: same as push; caller passes a sorted graph
//   3 hubdup      src/hubdup        : push + thread-private hub accumulators,
//                                     hubs found through a bitmap + index map
//   4 radar       src/RADAR         : push + thread-private hubs = ids < numHubs
//                                     (caller passes a degree-sorted graph)
// All variants compute the same results (depths/radii exactly, doubles within
// rounding), which is what the reference does too.

#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <algorithm>
#include <atomic>
#include <functional>
#include <random>
#include <utility>
#include <vector>

namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;  // UINT_E_MAX in Ligra (parallel.h:113-123)

enum Variant { kPush = 0, kPushPull = 1, kDegSort = 2, kHubDup = 3, kRadar = 4 };

// Out-edges (off/adj) and in-edges (in_off/in_adj; the same arrays for a
// symmetric graph).  Pushes follow out-edges, pulls read in-edges, and a
// transpose swaps the two (graph.h:78-86).
struct Csr {
  int64_t n, m;
  const uint32_t* off;  // n+1
  const uint32_t* adj;  // m
  const uint32_t* in_off = nullptr;
  const uint32_t* in_adj = nullptr;
  uint32_t deg(int64_t v) const { return off[v + 1] - off[v]; }
  Csr transposed() const { return Csr{n, m, in_off, in_adj, off, adj}; }
};

// In-edges for the next app calls on a directed graph (null: symmetric).
const uint32_t* g_in_off = nullptr;
const uint32_t* g_in_adj = nullptr;

Csr make_csr(int64_t n, const uint32_t* off, const uint32_t* adj) {
  Csr g{n, (int64_t)off[n], off, adj};
  g.in_off = g_in_off ? g_in_off : off;
  g.in_adj = g_in_off ? g_in_adj : adj;
  return g;
}

// ---------------------------------------------------------------------------
// Atomics.  The reference uses __sync CAS (utils.h:311-324) and a CAS loop for
// double addition (utils.h:334-339) and 64-bit OR (Radii.C:30-35).
// ---------------------------------------------------------------------------
inline bool cas_u32(uint32_t* p, uint32_t o, uint32_t nv) {
  return __atomic_compare_exchange_n(p, &o, nv, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED);
}
inline bool cas_i32(int32_t* p, int32_t o, int32_t nv) {
  return __atomic_compare_exchange_n(p, &o, nv, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED);
}
inline void add_f64(double* p, double v) {
  uint64_t* q = reinterpret_cast<uint64_t*>(p);
  uint64_t old = __atomic_load_n(q, __ATOMIC_RELAXED);
  for (;;) {
    double o; memcpy(&o, &old, 8);
    double nv = o + v;
    uint64_t nb; memcpy(&nb, &nv, 8);
    if (__atomic_compare_exchange_n(q, &old, nb, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return;
  }
}
// Returns the value before the add (the BC forward functor needs oldV, BC-manyiter-v2.C:63-68).
inline double add_f64_old(double* p, double v) {
  uint64_t* q = reinterpret_cast<uint64_t*>(p);
  uint64_t old = __atomic_load_n(q, __ATOMIC_RELAXED);
  for (;;) {
    double o; memcpy(&o, &old, 8);
    double nv = o + v;
    uint64_t nb; memcpy(&nb, &nv, 8);
    if (__atomic_compare_exchange_n(q, &old, nb, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return o;
  }
}
// Sets a shared flag byte, writing only when it is still clear (the
// reference's `if (doMerge[d] == false) CAS(...)`, BC-manyiter-v2.C:62-63):
// once set, the byte's cache line stays shared instead of bouncing between
// the threads that touch the same hub.
inline void set_flag(uint8_t* p) {
  if (!__atomic_load_n(p, __ATOMIC_RELAXED)) __atomic_store_n(p, (uint8_t)1, __ATOMIC_RELAXED);
}
inline void or_i64(int64_t* p, int64_t b) {
  int64_t old = __atomic_load_n(p, __ATOMIC_RELAXED);
  while ((old | b) != old &&
         !__atomic_compare_exchange_n(p, &old, old | b, false, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
  }
}

// Arrays the app drivers allocate per call, filled in parallel as the
// reference's parallel_for initialisations do (a serial fill of the hub
// copies alone is tens of MB on one core).
template <class V> void par_fill(V* p, int64_t n, V v) {
#pragma omp parallel for
  for (int64_t i = 0; i < n; i++) p[i] = v;
}
template <class V> struct Arr {
  V* p;
  int64_t n;
  Arr(int64_t n_, V v) : p(static_cast<V*>(malloc(sizeof(V) * (n_ > 0 ? n_ : 1)))), n(n_) { par_fill(p, n, v); }
  Arr(const Arr&) = delete;
  Arr& operator=(const Arr&) = delete;
  ~Arr() { free(p); }
  V& operator[](int64_t i) { return p[i]; }
  V* data() { return p; }
};
// Per-thread hub copies, each allocated and filled by its own thread.
template <class V> std::vector<std::vector<V>> make_dup(int threads, int64_t count, V init) {
  std::vector<std::vector<V>> d(count ? threads : 0);
#pragma omp parallel for schedule(static, 1)
  for (int t = 0; t < (int)d.size(); t++) d[t].assign(count, init);
  return d;
}

// Parallel pack of the indices of set bytes, in increasing order (the
// reference's pack_index, sequence.h, and the SlidingQueue compaction of
// ligra.h:161-192 produce the same set).
std::vector<uint32_t> pack_indices(const uint8_t* bits, int64_t n) {
  int T = omp_get_max_threads();
  std::vector<int64_t> cnt(T + 1, 0);
  std::vector<uint32_t> out;
#pragma omp parallel num_threads(T)
  {
    int t = omp_get_thread_num(), nt = omp_get_num_threads();
    int64_t b = n * t / nt, e = n * (t + 1) / nt, c = 0;
    for (int64_t i = b; i < e; i++) c += bits[i] != 0;
    cnt[t + 1] = c;
#pragma omp barrier
#pragma omp single
    {
      for (int i = 0; i < nt; i++) cnt[i + 1] += cnt[i];
      out.resize(cnt[nt]);
    }
    int64_t o = cnt[t];
    for (int64_t i = b; i < e; i++) if (bits[i]) out[o++] = (uint32_t)i;
  }
  return out;
}

// ---------------------------------------------------------------------------
// Frontier (vertexSubset.h:111-229): sparse id list or dense byte map.
// ---------------------------------------------------------------------------
struct Frontier {
  int64_t n = 0;
  int64_t count = 0;
  bool is_dense = false;
  std::vector<uint32_t> ids;   // sparse form
  std::vector<uint8_t> bits;   // dense form (one byte per vertex, like bool[n])
  bool has_ids = false, has_bits = false;

  static Frontier single(int64_t n, uint32_t v) {
    Frontier f; f.n = n; f.count = 1; f.ids = {v}; f.has_ids = true; return f;
  }
  static Frontier all(int64_t n) {
    Frontier f; f.n = n; f.count = n; f.bits.assign(n, 1); f.has_bits = true; f.is_dense = true;
    return f;
  }
  static Frontier from_ids(int64_t n, std::vector<uint32_t> v) {
    Frontier f; f.n = n; f.count = (int64_t)v.size(); f.ids = std::move(v); f.has_ids = true;
    return f;
  }
  static Frontier from_bits(int64_t n, std::vector<uint8_t> b) {
    Frontier f; f.n = n; f.bits = std::move(b); f.has_bits = true; f.is_dense = true;
    int64_t c = 0;
#pragma omp parallel for reduction(+ : c)
    for (int64_t i = 0; i < n; i++) c += f.bits[i];
    f.count = c;
    return f;
  }
  // toSparse (vertexSubset.h:196-211): pack the indices of set bytes in order.
  void to_sparse() {
    if (!has_ids && count > 0) {
      ids = pack_indices(bits.data(), n);
      has_ids = true;
    }
    is_dense = false;
  }
  // toDense (vertexSubset.h:214-221).
  void to_dense() {
    if (!has_bits) {
      bits.assign(n, 0);
#pragma omp parallel for
      for (int64_t i = 0; i < (int64_t)ids.size(); i++) bits[ids[i]] = 1;
      has_bits = true;
    }
    is_dense = true;
  }
  bool in(int64_t v) const { return bits[v] != 0; }
  template <class Fn> void for_each(Fn fn) {  // vertexMap (ligra.h:478-493)
    if (is_dense) {
#pragma omp parallel for
      for (int64_t i = 0; i < n; i++) if (bits[i]) fn((uint32_t)i);
    } else {
#pragma omp parallel for
      for (int64_t i = 0; i < (int64_t)ids.size(); i++) fn(ids[i]);
    }
  }
};

// ---------------------------------------------------------------------------
// edgeMap (ligra.h:277-316 mode switch; 130-196 sparse push; 90-128 dense
// push; 61-88 dense pull with vertex.h:12-41 early exit).
//
// The functor F provides:
//   bool cond(uint32_t d)
//   void update(uint32_t s, uint32_t d)              pull, non-atomic
//   void update_atomic(uint32_t s, uint32_t d, int tid)  push
//   void merge()                                     mergeDuplicates
//   uint8_t* next                                    next byte map or nullptr
// ---------------------------------------------------------------------------
// Edges traversed by edge_map calls (sum of the frontiers' out-degrees, the
// work the reference's edgeMap does), for the CPU baseline's edges/second.
std::atomic<int64_t> g_edges{0};

template <class F>
Frontier edge_map(const Csr& g, Frontier& fr, F& f, int64_t threshold, bool output,
                  bool dense_forward) {
  const int64_t n = g.n;
  if (threshold == -1) threshold = g.m / 20;  // ligra.h:283
  if (fr.count == 0) return Frontier::from_ids(n, {});
  fr.to_sparse();
  int64_t k = (int64_t)fr.ids.size();
  int64_t out_deg = 0;
#pragma omp parallel for reduction(+ : out_deg)
  for (int64_t i = 0; i < k; i++) out_deg += g.deg(fr.ids[i]);
  g_edges += out_deg;
  if (out_deg == 0) return Frontier::from_ids(n, {});  // ligra.h:301
  if (k + out_deg > threshold) {
    fr.to_dense();
    if (output) {
#pragma omp parallel for
      for (int64_t i = 0; i < n; i++) f.next[i] = 0;
    }
    if (dense_forward) {  // edgeMapDenseForward
#pragma omp parallel for schedule(dynamic, 64)
      for (int64_t s = 0; s < n; s++) {
        if (!fr.in(s)) continue;
        int tid = omp_get_thread_num();
        for (uint32_t j = g.off[s]; j < g.off[s + 1]; j++) {
          uint32_t d = g.adj[j];
          if (f.cond(d)) f.update_atomic((uint32_t)s, d, tid);
        }
      }
      f.merge();
    } else {  // edgeMapDense (pull) over in-edges
#pragma omp parallel for schedule(dynamic, 64)
      for (int64_t v = 0; v < n; v++) {
        if (!f.cond((uint32_t)v)) continue;
        for (uint32_t j = g.in_off[v]; j < g.in_off[v + 1]; j++) {
          uint32_t u = g.in_adj[j];
          if (fr.in(u)) f.update(u, (uint32_t)v);
          if (!f.cond((uint32_t)v)) break;
        }
      }
    }
  } else {  // edgeMapSparse
    if (output) {
#pragma omp parallel for
      for (int64_t i = 0; i < n; i++) f.next[i] = 0;
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t i = 0; i < k; i++) {
      uint32_t s = fr.ids[i];
      int tid = omp_get_thread_num();
      for (uint32_t j = g.off[s]; j < g.off[s + 1]; j++) {
        uint32_t d = g.adj[j];
        if (f.cond(d)) f.update_atomic(s, d, tid);
      }
    }
    f.merge();
    if (output) {  // compact the next byte map into an id list (ligra.h:161-192)
      return Frontier::from_ids(n, pack_indices(f.next, n));
    }
    return Frontier::from_ids(n, {});
  }
  if (output) return Frontier::from_bits(n, std::vector<uint8_t>(f.next, f.next + n));
  return Frontier::from_ids(n, {});
}

// ---------------------------------------------------------------------------
// Hub duplication (RADAR: hub <=> d < numHubs, PageRank.C:42-53; hubdup:
// hub <=> bit set in a bitmap, index through idxMap, hubdup/.../IO.h:720-804).
// numHubs = llcCap / (T*elem [+extra]) with llcCap = 1<<25 (PageRank.C:148-149,
// BFS.C:144-145, BC-manyiter-v2.C:232-233, Radii.C:172-173).  The reference
// reads and writes out of bounds when numHubs > n; this restatement caps it.
// ---------------------------------------------------------------------------
struct Hubs {
  int64_t count = 0;                 // number of hub slots
  std::vector<int32_t> slot_of;      // hubdup only: vertex -> slot or -1
  std::vector<uint32_t> vertex_of;   // slot -> vertex
  bool by_map = false;
  int32_t slot(uint32_t d) const {
    if (by_map) return slot_of[d];
    return (int64_t)d < count ? (int32_t)d : -1;
  }
};

Hubs make_hubs(const Csr& g, int variant, int nthreads, size_t elem, size_t extra) {
  Hubs h;
  if (variant != kHubDup && variant != kRadar) return h;
  const int64_t llc = 1 << 25;
  int64_t num = llc / (int64_t)(nthreads * elem + extra);
  if (variant == kRadar) {
    h.count = std::min<int64_t>(num, g.n);
    h.vertex_of.resize(h.count);
    for (int64_t i = 0; i < h.count; i++) h.vertex_of[i] = (uint32_t)i;
    return h;
  }
  // hubdup identifyHubs: threshold = sorted_degree[numHubs]; hubs are deg > thresh.
  std::vector<uint32_t> degs(g.n);
  for (int64_t v = 0; v < g.n; v++) degs[v] = g.deg(v);
  std::sort(degs.begin(), degs.end(), std::greater<uint32_t>());
  num = std::min<int64_t>(num, g.n - 1);
  uint32_t thresh = num >= 0 ? degs[num] : 0;
  h.by_map = true;
  h.slot_of.assign(g.n, -1);
  for (int64_t v = 0; v < g.n; v++) {
    if (g.deg(v) > thresh) {
      h.slot_of[v] = (int32_t)h.vertex_of.size();
      h.vertex_of.push_back((uint32_t)v);
    }
  }
  h.count = (int64_t)h.vertex_of.size();
  return h;
}

// ---------------------------------------------------------------------------
// PageRank (PageRank.C:29-189).
// ---------------------------------------------------------------------------
struct PrF {
  const Csr* g; double* p_curr; double* p_next; uint8_t* next = nullptr;
  const Hubs* hubs; std::vector<std::vector<double>>* dup;
  bool cond(uint32_t) const { return true; }
  void update(uint32_t s, uint32_t d) { p_next[d] += p_curr[s] / g->deg(s); }
  void update_atomic(uint32_t s, uint32_t d, int tid) {
    int32_t h = hubs->slot(d);
    if (h >= 0) (*dup)[tid][h] += p_curr[s] / g->deg(s);
    else add_f64(&p_next[d], p_curr[s] / g->deg(s));
  }
  void merge() {
    if (hubs->count == 0) return;
    int T = (int)dup->size();
#pragma omp parallel for
    for (int64_t h = 0; h < hubs->count; h++) {
      uint32_t d = hubs->vertex_of[h];
      for (int t = 0; t < T; t++) { p_next[d] += (*dup)[t][h]; (*dup)[t][h] = 0.0; }
    }
  }
};

// ---------------------------------------------------------------------------
// PageRankDelta (PageRankDelta.C:29-155; RADAR hubs :44-85, hubdup hubs
// src/hubdup/Ligra/apps/PageRankDelta.C:53-91).  nghSum[d] += Delta[s]/deg(s).
// ---------------------------------------------------------------------------
struct PrDeltaF {
  const Csr* g; const double* delta; double* ngh; uint8_t* next = nullptr;
  const Hubs* hubs; std::vector<std::vector<double>>* dup; std::vector<uint8_t>* do_merge;
  bool cond(uint32_t) const { return true; }
  void update(uint32_t s, uint32_t d) { ngh[d] += delta[s] / g->deg(s); }
  void update_atomic(uint32_t s, uint32_t d, int tid) {
    int32_t h = hubs->slot(d);
    if (h >= 0) {
      (*dup)[tid][h] += delta[s] / g->deg(s);
      set_flag(&(*do_merge)[h]);
    } else {
      add_f64(&ngh[d], delta[s] / g->deg(s));
    }
  }
  void merge() {  // only hubs some thread wrote (doMerge), then reset the copies
    if (hubs->count == 0) return;
    int T = (int)dup->size();
#pragma omp parallel for
    for (int64_t h = 0; h < hubs->count; h++) {
      if (!(*do_merge)[h]) continue;
      (*do_merge)[h] = 0;
      uint32_t d = hubs->vertex_of[h];
      for (int t = 0; t < T; t++) { ngh[d] += (*dup)[t][h]; (*dup)[t][h] = 0.0; }
    }
  }
};

// ---------------------------------------------------------------------------
// BFS (BFS.C:28-188; push-pull variant src/push-pull/Ligra/apps/BFS.C:28-48).
// ---------------------------------------------------------------------------
struct BfsF {
  uint32_t* parents; uint8_t* next;
  const Hubs* hubs; std::vector<std::vector<uint32_t>>* dup;
  std::vector<uint8_t>* do_merge; bool pull_cond;
  bool cond(uint32_t d) const { return pull_cond ? parents[d] == kNone : true; }
  void update(uint32_t s, uint32_t d) {
    if (parents[d] == kNone) { parents[d] = s; next[d] = 1; }
  }
  void update_atomic(uint32_t s, uint32_t d, int tid) {
    int32_t h = hubs->slot(d);
    if (h >= 0) {
      if ((*dup)[tid][h] == kNone) {
        (*dup)[tid][h] = s;
        set_flag(&(*do_merge)[h]);
      }
    } else if (parents[d] == kNone) {
      if (cas_u32(&parents[d], kNone, s)) next[d] = 1;
    }
  }
  void merge() {  // BFS.C:69-94: first non-MAX private copy wins
    if (hubs->count == 0) return;
    int T = (int)dup->size();
#pragma omp parallel for
    for (int64_t h = 0; h < hubs->count; h++) {
      if (!(*do_merge)[h]) continue;
      (*do_merge)[h] = 0;
      uint32_t d = hubs->vertex_of[h];
      if (parents[d] != kNone) continue;
      for (int t = 0; t < T; t++) {
        if ((*dup)[t][h] != kNone) { parents[d] = (*dup)[t][h]; next[d] = 1; break; }
      }
    }
  }
};

// ---------------------------------------------------------------------------
// BC (BC-manyiter-v2.C:32-183).
// ---------------------------------------------------------------------------
struct BcF {
  double* num_paths; uint8_t* visited; uint8_t* next;
  const Hubs* hubs; std::vector<std::vector<double>>* dup; std::vector<uint8_t>* do_merge;
  bool cond(uint32_t d) const { return visited[d] == 0; }
  void update(uint32_t s, uint32_t d) {
    double o = num_paths[d];
    num_paths[d] += num_paths[s];
    if (o == 0.0) next[d] = 1;
  }
  void update_atomic(uint32_t s, uint32_t d, int tid) {
    int32_t h = hubs->slot(d);
    if (h >= 0) {
      (*dup)[tid][h] += num_paths[s];
      set_flag(&(*do_merge)[h]);
    } else {
      double o = add_f64_old(&num_paths[d], num_paths[s]);
      if (o == 0.0) next[d] = 1;
    }
  }
  void merge() {
    if (hubs->count == 0) return;
    int T = (int)dup->size();
#pragma omp parallel for
    for (int64_t h = 0; h < hubs->count; h++) {
      if (!(*do_merge)[h]) continue;
      (*do_merge)[h] = 0;
      uint32_t d = hubs->vertex_of[h];
      bool upd = false;
      for (int t = 0; t < T; t++) {
        num_paths[d] += (*dup)[t][h];
        if ((*dup)[t][h] != 0.0) { upd = true; (*dup)[t][h] = 0.0; }
      }
      if (upd) next[d] = 1;
    }
  }
};

struct BcBackF {
  double* deps; uint8_t* visited; uint8_t* next = nullptr;
  const Hubs* hubs; std::vector<std::vector<double>>* dup; std::vector<uint8_t>* do_merge;
  bool cond(uint32_t d) const { return visited[d] == 0; }
  void update(uint32_t s, uint32_t d) { deps[d] += deps[s]; }
  void update_atomic(uint32_t s, uint32_t d, int tid) {
    int32_t h = hubs->slot(d);
    if (h >= 0) {
      (*dup)[tid][h] += deps[s];
      set_flag(&(*do_merge)[h]);
    } else {
      add_f64(&deps[d], deps[s]);
    }
  }
  void merge() {
    if (hubs->count == 0) return;
    int T = (int)dup->size();
#pragma omp parallel for
    for (int64_t h = 0; h < hubs->count; h++) {
      if (!(*do_merge)[h]) continue;
      (*do_merge)[h] = 0;
      uint32_t d = hubs->vertex_of[h];
      for (int t = 0; t < T; t++) { deps[d] += (*dup)[t][h]; (*dup)[t][h] = 0.0; }
    }
  }
};

// ---------------------------------------------------------------------------
// Radii (Radii.C:37-117).
// ---------------------------------------------------------------------------
struct RadiiF {
  int64_t* visited; int64_t* next_visited; int32_t* radii; int32_t round; uint8_t* next;
  const Hubs* hubs; std::vector<std::vector<int64_t>>* dup; std::vector<uint8_t>* do_merge;
  bool cond(uint32_t) const { return true; }
  void update(uint32_t s, uint32_t d) {
    int64_t w = visited[d] | visited[s];
    if (visited[d] != w) {
      next_visited[d] |= w;
      if (radii[d] != round) { radii[d] = round; next[d] = 1; }
    }
  }
  void update_atomic(uint32_t s, uint32_t d, int tid) {
    int64_t w = visited[d] | visited[s];
    if (visited[d] == w) return;
    int32_t h = hubs->slot(d);
    if (h >= 0) {
      (*dup)[tid][h] |= w;
      set_flag(&(*do_merge)[h]);
    } else {
      or_i64(&next_visited[d], w);
    }
    int32_t old = radii[d];
    if (old != round && cas_i32(&radii[d], old, round)) next[d] = 1;
  }
  void merge() {
    if (hubs->count == 0) return;
    int T = (int)dup->size();
#pragma omp parallel for
    for (int64_t h = 0; h < hubs->count; h++) {
      if (!(*do_merge)[h]) continue;
      (*do_merge)[h] = 0;
      uint32_t d = hubs->vertex_of[h];
      for (int t = 0; t < T; t++) {
        if ((*dup)[t][h]) { next_visited[d] |= (*dup)[t][h]; (*dup)[t][h] = 0; }
      }
    }
  }
};

struct ThreadScope {
  int saved;
  explicit ThreadScope(int t) : saved(omp_get_max_threads()) { if (t > 0) omp_set_num_threads(t); }
  ~ThreadScope() { omp_set_num_threads(saved); }
};

// Ligra's 64-bit hashInt (utils.h:350-358); a published integer mixing hash
// whose constants decide which vertices Radii samples, so they must match.
inline uint64_t hash_u64(uint64_t a) {
  a = (a + 0x7ed55d166bef7a1dULL) + (a << 12);
  a = (a ^ 0xc761c23c510fa2ddULL) ^ (a >> 9);
  a = (a + 0x165667b183a9c0e1ULL) + (a << 59);
  a = (a + 0xd3a2646cab3487e3ULL) ^ (a << 49);
  a = (a + 0xfd7046c5ef9ab54cULL) + (a << 3);
  a = (a ^ 0xb55a4f090dd4a67bULL) ^ (a >> 32);
  return a;
}

}  // namespace

extern "C" {

// Symmetric-graph clean-up of the Ligra text loader (IO.h:429-474): for every
// vertex sort its neighbour list, drop duplicates and self-loops, repack.
// `off` has n entries (start offsets, as in the AdjacencyGraph file).
// Returns the new edge count; out_off has n+1 entries.
int64_t orc_dedup_symmetric(int64_t n, int64_t m, const uint32_t* off, const uint32_t* adj,
                            uint32_t* out_off, uint32_t* out_adj) {
  std::vector<uint32_t> tmp(adj, adj + m);
  std::vector<uint32_t> nd(n);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; i++) {
    uint32_t b = off[i], e = (i == n - 1) ? (uint32_t)m : off[i + 1];
    uint32_t* s = tmp.data() + b;
    std::sort(s, tmp.data() + e);
    uint32_t* ne = std::unique(s, tmp.data() + e);
    ne = std::remove(s, ne, (uint32_t)i);
    nd[i] = (uint32_t)(ne - s);
  }
  uint64_t acc = 0;
  for (int64_t i = 0; i < n; i++) { out_off[i] = (uint32_t)acc; acc += nd[i]; }
  out_off[n] = (uint32_t)acc;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; i++) memcpy(out_adj + out_off[i], tmp.data() + off[i], 4ull * nd[i]);
  return (int64_t)acc;
}

// Degree sort of a symmetric graph (IO.h:843-895): sort (degree, id) pairs with
// std::greater -- degree descending, ties by DEScending original id -- and give
// rank r to the r-th pair.  Neighbour lists are relabelled but keep their order.
void orc_degree_sort(int64_t n, const uint32_t* off, const uint32_t* adj, uint32_t* new_ids,
                     uint32_t* new_off, uint32_t* new_adj) {
  std::vector<std::pair<uint32_t, uint32_t>> p(n);
  for (int64_t v = 0; v < n; v++) p[v] = {off[v + 1] - off[v], (uint32_t)v};
  std::sort(p.begin(), p.end(), std::greater<std::pair<uint32_t, uint32_t>>());
  for (int64_t r = 0; r < n; r++) new_ids[p[r].second] = (uint32_t)r;
  uint64_t acc = 0;
  for (int64_t r = 0; r < n; r++) { new_off[r] = (uint32_t)acc; acc += p[r].first; }
  new_off[n] = (uint32_t)acc;
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t v = 0; v < n; v++) {
    uint32_t r = new_ids[v];
    uint32_t o = new_off[r];
    for (uint32_t j = off[v]; j < off[v + 1]; j++) new_adj[o + (j - off[v])] = new_ids[adj[j]];
  }
}

// PageRank Compute (PageRank.C:120-189).  push-pull passes threshold 0 and no
// dense_forward (src/push-pull/Ligra/apps/PageRank.C:122), i.e. always pull.
// `ranks` receives the final rank vector: p_curr after a run that used all
// max_iters iterations (the last swap leaves the ranks there), p_next after an
// L1 < 1e-7 break.
int orc_pagerank(int64_t n, const uint32_t* off, const uint32_t* adj, int variant,
                 int64_t max_iters, int nthreads, double* ranks, int64_t* iters_out,
                 double* l1_out) {
  ThreadScope ts(nthreads);
  Csr g = make_csr(n, off, adj);
  const double damping = 0.85, eps = 0.0000001;
  Arr<double> a(n, 1.0 / (double)n), b(n, 0.0);
  double* p_curr = a.data();
  double* p_next = b.data();
  int T = omp_get_max_threads();
  Hubs hubs = make_hubs(g, variant, T, sizeof(double), variant == kHubDup ? 5 : 0);
  std::vector<std::vector<double>> dup = make_dup(T, hubs.count, 0.0);
  Frontier fr = Frontier::all(n);
  const double added = (1 - damping) * (1 / (double)n);
  int64_t iter = 0;
  double l1 = 0.0;
  bool broke = false;
  while (iter++ < max_iters) {
    PrF f{&g, p_curr, p_next, nullptr, &hubs, &dup};
    if (variant == kPushPull) edge_map(g, fr, f, 0, false, false);
    else edge_map(g, fr, f, -1, false, true);
    fr.for_each([&](uint32_t i) { p_next[i] = damping * p_next[i] + added; });
#pragma omp parallel for
    for (int64_t i = 0; i < n; i++) p_curr[i] = fabs(p_curr[i] - p_next[i]);
    l1 = 0.0;
#pragma omp parallel for reduction(+ : l1)
    for (int64_t i = 0; i < n; i++) l1 += p_curr[i];
    if (l1 < eps) { broke = true; break; }
    fr.for_each([&](uint32_t i) { p_curr[i] = 0.0; });
    std::swap(p_curr, p_next);
  }
  memcpy(ranks, broke ? p_next : p_curr, 8 * n);
  if (iters_out) *iters_out = iter;
  if (l1_out) *l1_out = l1;
  return 0;
}

// PageRankDelta Compute (PageRankDelta.C:98-155).  The first round filters with
// PR_Vertex_F_FirstRound (:46-61), later rounds with PR_Vertex_F (:63-76); the
// L1 norm is the sum of |Delta| over all vertices (:140-143) and the run stops
// when it drops below 1e-7.  push-pull pulls its dense rounds (no
// dense_forward, src/push-pull/Ligra/apps/PageRankDelta.C:130).
// iters_out = the reference's printed round count.
int orc_pagerank_delta(int64_t n, const uint32_t* off, const uint32_t* adj, int variant,
                       int64_t max_iters, int nthreads, double* ranks, int64_t* iters_out,
                       double* l1_out) {
  ThreadScope ts(nthreads);
  Csr g = make_csr(n, off, adj);
  const double damping = 0.85, eps = 0.0000001, eps2 = 0.01;
  const double one_over_n = 1 / (double)n;
  const double added = (1 - damping) * one_over_n;
  Arr<double> p(n, 0.0), delta(n, one_over_n), ngh(n, 0.0);
  int T = omp_get_max_threads();
  Hubs hubs = make_hubs(g, variant, T, sizeof(double), variant == kHubDup ? 6 : 1);
  std::vector<std::vector<double>> dup = make_dup(T, hubs.count, 0.0);
  std::vector<uint8_t> do_merge(hubs.count, 0);
  std::vector<uint8_t> active(n);
  Frontier fr = Frontier::all(n);
  int64_t round = 0;
  double l1 = 0.0;
  while (round++ < max_iters) {
    PrDeltaF f{&g, delta.data(), ngh.data(), nullptr, &hubs, &dup, &do_merge};
    edge_map(g, fr, f, g.m / 20, false, variant != kPushPull);
    if (round == 1) {
#pragma omp parallel for
      for (int64_t i = 0; i < n; i++) {
        delta[i] = damping * ngh[i] + added;
        p[i] += delta[i];
        delta[i] -= one_over_n;
        active[i] = fabs(delta[i]) > eps2 * p[i];
      }
    } else {
#pragma omp parallel for
      for (int64_t i = 0; i < n; i++) {
        delta[i] = ngh[i] * damping;
        active[i] = fabs(delta[i]) > eps2 * p[i];
        if (active[i]) p[i] += delta[i];
      }
    }
    l1 = 0.0;
#pragma omp parallel for reduction(+ : l1)
    for (int64_t i = 0; i < n; i++) l1 += fabs(delta[i]);
    if (l1 < eps) break;
#pragma omp parallel for
    for (int64_t i = 0; i < n; i++) ngh[i] = 0.0;
    fr = Frontier::from_bits(n, active);
  }
  memcpy(ranks, p.data(), 8 * n);
  if (iters_out) *iters_out = round;
  if (l1_out) *l1_out = l1;
  return 0;
}

// BFS Compute (BFS.C:122-188).  `root` is an internal id.  Parents are internal
// ids, UINT32_MAX for unreached.  rounds_out = number of edgeMap calls.
int orc_bfs(int64_t n, const uint32_t* off, const uint32_t* adj, int variant, uint32_t root,
            int nthreads, uint32_t* parents, int64_t* rounds_out) {
  ThreadScope ts(nthreads);
  Csr g = make_csr(n, off, adj);
  par_fill(parents, n, kNone);
  parents[root] = root;
  int T = omp_get_max_threads();
  Hubs hubs = make_hubs(g, variant, T, sizeof(uint32_t), 1 + (variant == kHubDup ? 5 : 0));
  std::vector<std::vector<uint32_t>> dup = make_dup(T, hubs.count, kNone);
  // RADAR seeds the private copies from Parents (BFS.C:154-156); with hub
  // slot == vertex id that marks the root's slot as already set, which is
  // harmless because the root already has its parent.
  std::vector<uint8_t> do_merge(hubs.count, 0);
  Arr<uint8_t> next(n, 0);
  Frontier fr = Frontier::single(n, root);
  int64_t rounds = 0;
  while (fr.count > 0) {
    BfsF f{parents, next.data(), &hubs, &dup, &do_merge, variant == kPushPull};
    fr = edge_map(g, fr, f, -1, true, variant != kPushPull);
    rounds++;
  }
  if (rounds_out) *rounds_out = rounds;
  return 0;
}

// BC Compute (BC-manyiter-v2.C:205-352) over the given source list (internal
// ids, already picked).  `deps` is zeroed once and chained across sources,
// exactly as the reference does: each source's final transform
// D = (D - 1/sigma) / (1/sigma) feeds the next source's backward phase.
int orc_bc(int64_t n, const uint32_t* off, const uint32_t* adj, int variant,
           const uint32_t* sources, int nsrc, int nthreads, double* deps, int64_t* levels_out) {
  ThreadScope ts(nthreads);
  const Csr g0 = make_csr(n, off, adj);
  int T = omp_get_max_threads();
  Hubs hubs = make_hubs(g0, variant, T, sizeof(double), 1 + (variant == kHubDup ? 5 : 0));
  std::vector<std::vector<double>> dup = make_dup(T, hubs.count, 0.0);
  std::vector<uint8_t> do_merge(hubs.count, 0);
  Arr<double> num_paths(n, 0.0);
  Arr<uint8_t> visited(n, 0), next(n, 0);
  par_fill(deps, n, 0.0);
  int64_t total_levels = 0;
  for (int it = 0; it < nsrc; it++) {
    // the reference transposes the graph before every backward phase and
    // never back (BC-manyiter-v2.C:334): source it's forward phase runs on
    // the graph transposed `it` times (a no-op for symmetric graphs)
    const Csr gf = (it % 2) ? g0.transposed() : g0;
    const Csr& g = gf;
    const Csr gb = gf.transposed();
    uint32_t start = sources[it];
    par_fill(num_paths.data(), n, 0.0);
    num_paths[start] = 1.0;
    par_fill(visited.data(), n, (uint8_t)0);
    visited[start] = 1;
    std::vector<Frontier> levels;
    Frontier fr = Frontier::single(n, start);
    levels.push_back(fr);
    int64_t round = 0;
    while (fr.count > 0) {
      round++;
      BcF f{num_paths.data(), visited.data(), next.data(), &hubs, &dup, &do_merge};
      Frontier out = edge_map(g, fr, f, -1, true, variant != kPushPull);
      out.for_each([&](uint32_t i) { visited[i] = 1; });
      levels.push_back(out);
      fr = out;
    }
    total_levels += round;
    double* inv = num_paths.data();  // inverted in place (BC-manyiter-v2.C:324-325)
#pragma omp parallel for
    for (int64_t i = 0; i < n; i++) inv[i] = 1 / inv[i];
    par_fill(visited.data(), n, (uint8_t)0);
    auto back_vertex = [&](uint32_t i) { visited[i] = 1; deps[i] += inv[i]; };
    Frontier cur = levels[round - 1];
    cur.for_each(back_vertex);
    for (int64_t r = round - 2; r >= 0; r--) {
      BcBackF f{deps, visited.data(), nullptr, &hubs, &dup, &do_merge};
      edge_map(gb, cur, f, -1, false, variant != kPushPull);
      cur = levels[r];
      cur.for_each(back_vertex);
    }
#pragma omp parallel for
    for (int64_t i = 0; i < n; i++) deps[i] = (deps[i] - inv[i]) / inv[i];
  }
  if (levels_out) *levels_out = total_levels;
  return 0;
}

// Radii Compute (Radii.C:140-218).  seeds[i] is the internal id that gets bit i
// (hashInt(i) % n mapped through new_ids).  When two seeds collide the seeding
// loop's plain store leaves one bit; this restatement keeps the bit of the
// larger i, which is what the reference does with one thread.
int orc_radii(int64_t n, const uint32_t* off, const uint32_t* adj, int variant,
              const uint32_t* seeds, int nseeds, int nthreads, int32_t* radii,
              int64_t* rounds_out) {
  ThreadScope ts(nthreads);
  Csr g = make_csr(n, off, adj);
  Arr<int64_t> visited(n, 0), next_visited(n, 0);
  par_fill(radii, n, -1);
  std::vector<uint32_t> starts(nseeds);
  for (int i = 0; i < nseeds; i++) {
    uint32_t v = seeds[i];
    radii[v] = 0;
    starts[i] = v;
    next_visited[v] = (int64_t)(1ULL << i);
  }
  int T = omp_get_max_threads();
  Hubs hubs = make_hubs(g, variant, T, sizeof(int64_t), 1 + (variant == kHubDup ? 5 : 0));
  std::vector<std::vector<int64_t>> dup = make_dup(T, hubs.count, (int64_t)0);
  std::vector<uint8_t> do_merge(hubs.count, 0);
  Arr<uint8_t> next(n, 0);
  Frontier fr = Frontier::from_ids(n, starts);
  int32_t round = 0;
  while (fr.count > 0) {
    round++;
    fr.for_each([&](uint32_t i) { visited[i] = next_visited[i]; });
    RadiiF f{visited.data(), next_visited.data(), radii, round, next.data(), &hubs, &dup,
             &do_merge};
    fr = edge_map(g, fr, f, -1, true, variant != kPushPull);
  }
  if (rounds_out) *rounds_out = round;
  return 0;
}

// Triangle counting, GAP tc_local (src/*/GAP/src/tc_local.cc:49-125 OrderedCount
// on the graph relabelled by degree, builder.h:247-282 RelabelByDegree: degree
// descending, ties by descending id, neighbour lists sorted).  A triangle is
// counted once, as u > v > w in the relabelled ids; counts[x] is the number
// of triangles containing x, returned by ORIGINAL id (it does not depend on
// the labelling).  Needs a cleaned symmetric graph (sorted, no repeats, no
// self loops), which is what the loaders produce.
int orc_triangles(int64_t n, const uint32_t* off, const uint32_t* adj, int nthreads, uint64_t* counts,
                  uint64_t* total_out) {
  ThreadScope ts(nthreads);
  std::vector<std::pair<uint32_t, uint32_t>> p(n);
  for (int64_t v = 0; v < n; v++) p[v] = {off[v + 1] - off[v], (uint32_t)v};
  std::sort(p.begin(), p.end(), std::greater<std::pair<uint32_t, uint32_t>>());
  std::vector<uint32_t> ids(n), roff(n + 1), radj(off[n]);
  for (int64_t r = 0; r < n; r++) ids[p[r].second] = (uint32_t)r;
  uint64_t acc = 0;
  for (int64_t r = 0; r < n; r++) { roff[r] = (uint32_t)acc; acc += p[r].first; }
  roff[n] = (uint32_t)acc;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t v = 0; v < n; v++) {
    const uint32_t r = ids[v];
    uint32_t* row = radj.data() + roff[r];
    for (uint32_t j = off[v]; j < off[v + 1]; j++) row[j - off[v]] = ids[adj[j]];
    std::sort(row, row + (off[v + 1] - off[v]));
  }
  std::vector<uint64_t> tri(n, 0);
  uint64_t total = 0;
#pragma omp parallel for reduction(+ : total) schedule(dynamic, 64)
  for (int64_t u = 0; u < n; u++) {
    for (uint32_t j = roff[u]; j < roff[u + 1]; j++) {
      const uint32_t v = radj[j];
      if (v > u) break;
      uint32_t it = roff[u];
      for (uint32_t k = roff[v]; k < roff[v + 1]; k++) {
        const uint32_t w = radj[k];
        if (w > v) break;
        while (radj[it] < w) it++;  // stops at v (< u, in u's list) at the latest
        if (radj[it] == w) {
          total++;
          __atomic_fetch_add(&tri[u], 1, __ATOMIC_RELAXED);
          __atomic_fetch_add(&tri[v], 1, __ATOMIC_RELAXED);
          __atomic_fetch_add(&tri[w], 1, __ATOMIC_RELAXED);
        }
      }
    }
  }
  for (int64_t v = 0; v < n; v++) counts[v] = tri[ids[v]];
  if (total_out) *total_out = total;
  return 0;
}

// In-edges (in_off n+1, in_adj m) for the following calls on a directed
// graph; null pointers return to symmetric graphs.
void orc_set_in_edges(const uint32_t* in_off, const uint32_t* in_adj) {
  g_in_off = in_off;
  g_in_adj = in_adj;
}

// Directed clean-up of the text loader (IO.h:287-474 without symmetry):
// every out-list sorted, repeats and self loops dropped.  `off` has n
// entries (start offsets).  Returns the new edge count; out_off has n+1.
int64_t orc_dedup_directed(int64_t n, int64_t m, const uint32_t* off, const uint32_t* adj, uint32_t* out_off,
                           uint32_t* out_adj) {
  return orc_dedup_symmetric(n, m, off, adj, out_off, out_adj);  // the per-list rule is the same
}

// In-edges of a CSR (the reference's CSC, IO.h:287-345): in_adj lists the
// sources of each vertex in increasing order.
void orc_transpose(int64_t n, const uint32_t* off, const uint32_t* adj, uint32_t* in_off, uint32_t* in_adj) {
  const int64_t m = off[n];
  std::vector<uint32_t> cnt(n + 1, 0);
  for (int64_t j = 0; j < m; j++) cnt[adj[j] + 1]++;
  for (int64_t v = 0; v < n; v++) cnt[v + 1] += cnt[v];
  for (int64_t v = 0; v <= n; v++) in_off[v] = cnt[v];
  for (int64_t s = 0; s < n; s++)
    for (uint32_t j = off[s]; j < off[s + 1]; j++) in_adj[cnt[adj[j]]++] = (uint32_t)s;
}

// Edges traversed by every edge_map since the last call (then reset).
int64_t orc_take_edges() { return g_edges.exchange(0); }

// BC source selection (BC-manyiter-v2.C:253-271, 279-280): mt19937 seeded with
// 27491095, uniform_int_distribution<long>(0, n-1), redrawn while the vertex has
// degree 0; draws are original ids, mapped through new_ids when the graph was
// degree-sorted.  `deg_orig` is the degree by ORIGINAL id.
void orc_bc_sources(int64_t n, const uint32_t* deg_orig, int k, uint32_t* out_orig) {
  std::mt19937 rng(27491095);
  std::uniform_int_distribution<long> ud(0, n - 1);
  for (int i = 0; i < k; i++) {
    long s;
    do { s = ud(rng); } while (deg_orig[s] == 0);
    out_orig[i] = (uint32_t)s;
  }
}

// Radii seeds (Radii.C:159-169): vertex hashInt((ulong)i) % n for i < min(n,64).
// The same draws on a directed graph: the reference checks the out-degree of
// the graph as it stands, and its BC transposes the graph once per source
// (BC-manyiter-v2.C:264-270, :334), so draw i rejects on out-degree for even
// i and in-degree for odd i.
void orc_bc_sources_directed(int64_t n, const uint32_t* outdeg_orig, const uint32_t* indeg_orig, int k,
                             uint32_t* out_orig) {
  std::mt19937 rng(27491095);
  std::uniform_int_distribution<long> ud(0, n - 1);
  for (int i = 0; i < k; i++) {
    const uint32_t* deg = (i % 2) ? indeg_orig : outdeg_orig;
    long s;
    do { s = ud(rng); } while (deg[s] == 0);
    out_orig[i] = (uint32_t)s;
  }
}

int orc_radii_seeds(int64_t n, uint32_t* out_orig) {
  int k = (int)std::min<int64_t>(n, 64);
  for (int i = 0; i < k; i++) out_orig[i] = (uint32_t)(hash_u64((uint64_t)i) % (uint64_t)n);
  return k;
}

// BFS depths from a parent array (used to compare BFS results bit-exactly).
void orc_depths_from_parents(int64_t n, const uint32_t* parents, int32_t* depth) {
  for (int64_t i = 0; i < n; i++) depth[i] = -2;
  for (int64_t i = 0; i < n; i++) {
    if (parents[i] == kNone) { depth[i] = -1; continue; }
    // walk up until a known depth or the root
    int64_t v = i, steps = 0;
    while (depth[v] == -2 && parents[v] != (uint32_t)v && steps <= n) { v = parents[v]; steps++; }
    int32_t base = depth[v] >= 0 ? depth[v] : (parents[v] == (uint32_t)v ? 0 : -3);
    if (depth[v] == -2) depth[v] = base;
    // second pass assigns depths along the path
    int64_t u = i; int32_t d = base + (int32_t)steps;
    while (u != v) { depth[u] = d--; u = parents[u]; }
  }
}

// Reference BFS depths by a plain serial level-synchronous BFS (textbook), the
// bit-exact quantity all variants agree on.
void orc_bfs_depths(int64_t n, const uint32_t* off, const uint32_t* adj, uint32_t root,
                    int32_t* depth) {
  for (int64_t i = 0; i < n; i++) depth[i] = -1;
  std::vector<uint32_t> q; q.reserve(n);
  depth[root] = 0; q.push_back(root);
  for (size_t h = 0; h < q.size(); h++) {
    uint32_t u = q[h];
    for (uint32_t j = off[u]; j < off[u + 1]; j++) {
      uint32_t v = adj[j];
      if (depth[v] < 0) { depth[v] = depth[u] + 1; q.push_back(v); }
    }
  }
}


// Seeded edge list of the GAP generator (GAP/src/generator.h:52-114), so the
// oracle builds the benchmark's graphs without the product library.
// R-MAT (uniform = 0): per edge, `scale` draws of a float in [0,1) pick one of
// four quadrants with A=0.57, B=0.19, C=0.19 (generator.h:82-105); edges come
// in 2^18-edge blocks and block b's mt19937 is seeded with seed + b
// (generator.h:90), then every id goes through a permutation made by
// shuffling 0..n-1 with mt19937(seed) (PermuteIDs, generator.h:52-62).
// Erdos-Renyi (uniform = 1): both endpoints uniform over [0, n-1] from
// uniform_int_distribution<int32_t> (NodeID), same blocks, no permutation
// (MakeUniformEL, generator.h:64-79).  GAP seeds with kRandSeed; the
// benchmark passes its own seed.
int orc_generate_edges(int scale, int edge_factor, uint64_t seed, int uniform, uint32_t* src, uint32_t* dst) {
  if (scale < 1 || scale > 31 || edge_factor < 1) return 1;
  const int64_t n = int64_t(1) << scale;
  const int64_t ne = n * edge_factor;
  const int64_t block = int64_t(1) << 18;  // generator.h:152
  const int64_t nblocks = (ne + block - 1) / block;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t b = 0; b < nblocks; b++) {
    std::mt19937 rng((uint32_t)(seed + (uint64_t)b));
    const int64_t lo = b * block, hi = std::min(ne, lo + block);
    if (uniform) {
      std::uniform_int_distribution<int32_t> pick(0, (int32_t)(n - 1));
      for (int64_t e = lo; e < hi; e++) {
        const int32_t u = pick(rng);  // sequenced: u is drawn before v
        const int32_t v = pick(rng);
        src[e] = (uint32_t)u;
        dst[e] = (uint32_t)v;
      }
      continue;
    }
    std::uniform_real_distribution<float> unit(0, 1.0f);
    const float a = 0.57f, ab = 0.57f + 0.19f, abc = 0.57f + 0.19f + 0.19f;
    for (int64_t e = lo; e < hi; e++) {
      uint32_t u = 0, v = 0;
      for (int d = 0; d < scale; d++) {
        const float x = unit(rng);
        const bool right = x < ab ? (x > a) : (x > abc);
        u = (u << 1) | (x < ab ? 0u : 1u);
        v = (v << 1) | (right ? 1u : 0u);
      }
      src[e] = u;
      dst[e] = v;
    }
  }
  if (!uniform) {
    std::vector<uint32_t> perm(n);
    for (int64_t i = 0; i < n; i++) perm[i] = (uint32_t)i;
    std::mt19937 rng((uint32_t)seed);
    std::shuffle(perm.begin(), perm.end(), rng);
#pragma omp parallel for
    for (int64_t e = 0; e < ne; e++) {
      src[e] = perm[src[e]];
      dst[e] = perm[dst[e]];
    }
  }
  return 0;
}

// Symmetric CSR of an edge list: both directions of every edge bucketed by
// source, then the symmetric loader's clean-up (sort, unique, drop self
// loops; IO.h:429-474) through orc_dedup_symmetric.  out_off: n+1 entries;
// out_adj: room for 2 * num_edges entries.  Returns m, or -1 when an id is out
// of range or m does not fit in 32 bits.
int64_t orc_csr_from_edges(int64_t n, int64_t num_edges, const uint32_t* src, const uint32_t* dst,
                           uint32_t* out_off, uint32_t* out_adj) {
  std::vector<std::atomic<uint32_t>> cnt(n);
  for (auto& c : cnt) c.store(0, std::memory_order_relaxed);
  bool bad = false;
#pragma omp parallel for reduction(|| : bad)
  for (int64_t e = 0; e < num_edges; e++) {
    if (src[e] >= n || dst[e] >= n) { bad = true; continue; }
    cnt[src[e]].fetch_add(1, std::memory_order_relaxed);
    cnt[dst[e]].fetch_add(1, std::memory_order_relaxed);
  }
  if (bad || 2 * num_edges >= (int64_t)0xFFFFFFFFu) return -1;
  std::vector<uint32_t> start(n);
  uint64_t acc = 0;
  for (int64_t v = 0; v < n; v++) { start[v] = (uint32_t)acc; acc += cnt[v].load(std::memory_order_relaxed); }
  std::vector<std::atomic<uint32_t>> cur(n);
  for (int64_t v = 0; v < n; v++) cur[v].store(start[v], std::memory_order_relaxed);
  std::vector<uint32_t> raw(2 * num_edges);
#pragma omp parallel for
  for (int64_t e = 0; e < num_edges; e++) {
    raw[cur[src[e]].fetch_add(1, std::memory_order_relaxed)] = dst[e];
    raw[cur[dst[e]].fetch_add(1, std::memory_order_relaxed)] = src[e];
  }
  return orc_dedup_symmetric(n, 2 * num_edges, start.data(), raw.data(), out_off, out_adj);
}

// GAP's SourcePicker (GAP/src/benchmark.h:47-64): one mt19937 seeded with
// kRandSeed (27491095, util.h:22) drives uniform_int_distribution<int32_t>
// (NodeID) over [0, n-1]; each pick redraws until the vertex has out-degree
// > 0, and k successive picks continue the same generator.  deg_orig is
// indexed by the ids the picks are in.
void orc_source_picker(int64_t n, const uint32_t* deg_orig, int k, uint32_t* out) {
  std::mt19937 rng(27491095u);
  std::uniform_int_distribution<int32_t> pick(0, (int32_t)(n - 1));
  for (int i = 0; i < k; i++) {
    int32_t v;
    do { v = pick(rng); } while (deg_orig[v] == 0);
    out[i] = (uint32_t)v;
  }
}

}  // extern "C"
