// Host-side graph input: seeded generator, Ligra file formats, symmetric
// clean-up into CSR.  These feed the device graph image (rg_graph_create).
//
// Generator: GAP/src/generator.h:52-114 (R-MAT A=0.57 B=0.19 C=0.19 with
// 2^18-edge blocks each drawn from mt19937 seeded with seed+block, then an
// id permutation from an mt19937(seed) shuffle; Erdos-Renyi draws uniform
// endpoint pairs with the same blocking and no permutation).
// Text format: IO.h:231-268.  Binary format: IO.h:477-626.
// Symmetric clean-up: IO.h:429-474 (per vertex sort, unique, drop self-loop).

#include <omp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <random>
#include <string>
#include <vector>

#include "rg_host.h"

namespace rg {

namespace {

constexpr int64_t kGenBlock = 1 << 18;  // generator.h:152

// Parallel exclusive prefix sum of uint32 counts into n+1 uint32 offsets.
// Returns false if the total does not fit in 32 bits.
bool prefix_u32(const std::vector<uint32_t>& cnt, uint32_t* out) {
  int64_t n = (int64_t)cnt.size();
  int T = omp_get_max_threads();
  std::vector<uint64_t> part(T + 1, 0);
#pragma omp parallel num_threads(T)
  {
    int t = omp_get_thread_num(), nt = omp_get_num_threads();
    int64_t b = n * t / nt, e = n * (t + 1) / nt;
    uint64_t s = 0;
    for (int64_t i = b; i < e; i++) s += cnt[i];
    part[t + 1] = s;
#pragma omp barrier
#pragma omp single
    for (int i = 0; i < nt; i++) part[i + 1] += part[i];
    uint64_t a = part[t];
    for (int64_t i = b; i < e; i++) { out[i] = (uint32_t)a; a += cnt[i]; }
  }
  if (part[T] > 0xFFFFFFFFull) return false;
  out[n] = (uint32_t)part[T];
  return true;
}

}  // namespace

rg_status generate_edges(int scale, int edge_factor, uint64_t seed, int uniform, uint32_t* src,
                         uint32_t* dst) {
  if (scale < 1 || scale > 31 || edge_factor < 1 || !src || !dst) {
    return fail(RG_EINVAL, "rg_generate_edges: bad scale/edge_factor/pointer");
  }
  const int64_t nn = int64_t(1) << scale;
  const int64_t ne = nn * edge_factor;
  const int64_t nblocks = (ne + kGenBlock - 1) / kGenBlock;
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t blk = 0; blk < nblocks; blk++) {
    std::mt19937 rng((uint32_t)(seed + (uint64_t)blk));
    const int64_t e0 = blk * kGenBlock, e1 = std::min(e0 + kGenBlock, ne);
    if (uniform) {
      std::uniform_int_distribution<int32_t> ud(0, (int32_t)(nn - 1));
      for (int64_t e = e0; e < e1; e++) {
        int32_t a = ud(rng);
        int32_t b = ud(rng);
        src[e] = (uint32_t)a;
        dst[e] = (uint32_t)b;
      }
    } else {
      const float A = 0.57f, B = 0.19f, C = 0.19f;
      std::uniform_real_distribution<float> ud(0, 1.0f);
      for (int64_t e = e0; e < e1; e++) {
        uint32_t s = 0, d = 0;
        for (int depth = 0; depth < scale; depth++) {
          float r = ud(rng);
          s <<= 1;
          d <<= 1;
          if (r < A + B) {
            if (r > A) d++;
          } else {
            s++;
            if (r > A + B + C) d++;
          }
        }
        src[e] = s;
        dst[e] = d;
      }
    }
  }
  if (!uniform) {  // PermuteIDs (generator.h:52-62)
    std::vector<uint32_t> perm(nn);
    for (int64_t i = 0; i < nn; i++) perm[i] = (uint32_t)i;
    std::mt19937 rng((uint32_t)seed);
    std::shuffle(perm.begin(), perm.end(), rng);
#pragma omp parallel for
    for (int64_t e = 0; e < ne; e++) {
      src[e] = perm[src[e]];
      dst[e] = perm[dst[e]];
    }
  }
  return RG_OK;
}

// Per-vertex sort + unique + self-loop removal over a scattered adjacency
// (`off` n+1, `tmp` holds the raw lists), then repack into exact arrays.
static rg_status clean_and_pack(int64_t n, const std::vector<uint32_t>& off, std::vector<uint32_t>& tmp,
                                uint32_t** off_out, uint32_t** adj_out, int64_t* m_out) {
  std::vector<uint32_t> nd(n);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < n; i++) {
    uint32_t* b = tmp.data() + off[i];
    uint32_t* e = tmp.data() + off[i + 1];
    std::sort(b, e);
    uint32_t* ne = std::unique(b, e);
    ne = std::remove(b, ne, (uint32_t)i);
    nd[i] = (uint32_t)(ne - b);
  }
  uint32_t* o = (uint32_t*)malloc(sizeof(uint32_t) * (n + 1));
  if (!o) return fail(RG_ENOMEM, "host malloc of offsets failed");
  if (!prefix_u32(nd, o)) { free(o); return fail(RG_EUNSUPPORTED, "graph has >= 2^32 edges"); }
  const int64_t m = o[n];
  uint32_t* a = (uint32_t*)malloc(sizeof(uint32_t) * (m + 4));  // +4: room for 16-byte tails
  if (!a) { free(o); return fail(RG_ENOMEM, "host malloc of edges failed"); }
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < n; i++) memcpy(a + o[i], tmp.data() + off[i], 4ull * nd[i]);
  memset(a + m, 0, 16);
  *off_out = o;
  *adj_out = a;
  *m_out = m;
  return RG_OK;
}

rg_status csr_from_edges(int64_t n, int64_t ne, const uint32_t* src, const uint32_t* dst,
                         uint32_t** off_out, uint32_t** adj_out, int64_t* m_out) {
  if (n <= 0 || ne < 0 || (ne > 0 && (!src || !dst)) || !off_out || !adj_out || !m_out) {
    return fail(RG_EINVAL, "rg_csr_from_edges: bad arguments");
  }
  if (2 * ne > 0xFFFFFFFFll) return fail(RG_EUNSUPPORTED, "rg_csr_from_edges: >= 2^32 entries");
  std::vector<std::atomic<uint32_t>> cnt(n);
#pragma omp parallel for
  for (int64_t i = 0; i < n; i++) cnt[i].store(0, std::memory_order_relaxed);
  bool bad = false;
#pragma omp parallel for reduction(|| : bad)
  for (int64_t e = 0; e < ne; e++) {
    if (src[e] >= (uint64_t)n || dst[e] >= (uint64_t)n) { bad = true; continue; }
    cnt[src[e]].fetch_add(1, std::memory_order_relaxed);
    cnt[dst[e]].fetch_add(1, std::memory_order_relaxed);
  }
  if (bad) return fail(RG_EINVAL, "rg_csr_from_edges: endpoint >= n");
  std::vector<uint32_t> c(n);
#pragma omp parallel for
  for (int64_t i = 0; i < n; i++) c[i] = cnt[i].load(std::memory_order_relaxed);
  std::vector<uint32_t> off(n + 1);
  prefix_u32(c, off.data());
  std::vector<std::atomic<uint32_t>>& pos = cnt;
#pragma omp parallel for
  for (int64_t i = 0; i < n; i++) pos[i].store(off[i], std::memory_order_relaxed);
  std::vector<uint32_t> tmp(2 * ne);
#pragma omp parallel for
  for (int64_t e = 0; e < ne; e++) {
    tmp[pos[src[e]].fetch_add(1, std::memory_order_relaxed)] = dst[e];
    tmp[pos[dst[e]].fetch_add(1, std::memory_order_relaxed)] = src[e];
  }
  return clean_and_pack(n, off, tmp, off_out, adj_out, m_out);
}

rg_status write_adjacency(const char* path, int64_t n, int64_t m, const uint32_t* off,
                          const uint32_t* adj) {
  if (!path || n <= 0 || m < 0 || !off || (m > 0 && !adj)) {
    return fail(RG_EINVAL, "rg_write_adjacency: bad arguments");
  }
  FILE* f = fopen(path, "w");
  if (!f) return fail(RG_EIO, "rg_write_adjacency: cannot open %s", path);
  std::string buf;
  buf.reserve(1 << 20);
  auto flush = [&]() { fwrite(buf.data(), 1, buf.size(), f); buf.clear(); };
  char tmp[32];
  buf += "AdjacencyGraph\n";
  snprintf(tmp, sizeof tmp, "%lld\n", (long long)n); buf += tmp;
  snprintf(tmp, sizeof tmp, "%lld\n", (long long)m); buf += tmp;
  for (int64_t i = 0; i < n; i++) {
    snprintf(tmp, sizeof tmp, "%u\n", off[i]); buf += tmp;
    if (buf.size() > (1u << 20)) flush();
  }
  for (int64_t i = 0; i < m; i++) {
    snprintf(tmp, sizeof tmp, "%u\n", adj[i]); buf += tmp;
    if (buf.size() > (1u << 20)) flush();
  }
  flush();
  bool ok = fclose(f) == 0;
  return ok ? RG_OK : fail(RG_EIO, "rg_write_adjacency: write failed");
}

namespace {

bool read_file(const char* path, std::vector<char>& out) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  fseek(f, 0, SEEK_END);
  long sz = ftell(f);
  fseek(f, 0, SEEK_SET);
  out.resize(sz > 0 ? sz : 0);
  size_t got = sz > 0 ? fread(out.data(), 1, sz, f) : 0;
  fclose(f);
  return (long)got == sz;
}

inline bool is_space(char c) { return c == ' ' || c == '\n' || c == '\r' || c == '\t' || c == '\0'; }

}  // namespace

rg_status read_graph(const char* path, int symmetric, int binary, int64_t* n_out, int64_t* m_out,
                     uint32_t** off_out, uint32_t** adj_out) {
  if (!path || !n_out || !m_out || !off_out || !adj_out) {
    return fail(RG_EINVAL, "rg_read_graph: null argument");
  }
  // a directed graph's out-lists get the same per-list clean-up as a
  // symmetric one's (IO.h:287-474); its in-lists are built on the device
  (void)symmetric;
  if (binary) {  // IO.h:477-626: .config holds n, .adj uint32 edges, .idx uint32 offsets
    std::string base(path);
    FILE* cf = fopen((base + ".config").c_str(), "r");
    if (!cf) return fail(RG_EIO, "rg_read_graph: cannot open %s.config", path);
    long long n = -1;
    int got = fscanf(cf, "%lld", &n);
    fclose(cf);
    if (got != 1 || n <= 0) return fail(RG_EFORMAT, "rg_read_graph: bad .config");
    std::vector<char> adjb, idxb;
    if (!read_file((base + ".adj").c_str(), adjb)) return fail(RG_EIO, "cannot read %s.adj", path);
    if (!read_file((base + ".idx").c_str(), idxb)) return fail(RG_EIO, "cannot read %s.idx", path);
    if ((long long)(idxb.size() / 4) != n || idxb.size() % 4 || adjb.size() % 4) {
      return fail(RG_EFORMAT, "rg_read_graph: File size wrong");
    }
    int64_t m = (int64_t)(adjb.size() / 4);
    uint32_t* o = (uint32_t*)malloc(4 * (n + 1));
    uint32_t* a = (uint32_t*)malloc(4 * (m + 4));
    if (!o || !a) { free(o); free(a); return fail(RG_ENOMEM, "host malloc failed"); }
    memcpy(o, idxb.data(), 4 * n);
    o[n] = (uint32_t)m;
    memcpy(a, adjb.data(), 4 * m);
    memset(a + m, 0, 16);
    for (int64_t i = 0; i < n; i++) {
      if (o[i] > o[i + 1]) { free(o); free(a); return fail(RG_EFORMAT, "offsets not monotone"); }
    }
    for (int64_t i = 0; i < m; i++) {
      if (a[i] >= (uint64_t)n) { free(o); free(a); return fail(RG_EFORMAT, "edge id >= n"); }
    }
    *n_out = n; *m_out = m; *off_out = o; *adj_out = a;
    return RG_OK;
  }
  std::vector<char> s;
  if (!read_file(path, s)) return fail(RG_EIO, "rg_read_graph: Unable to open file: %s", path);
  s.push_back('\0');
  size_t p = 0, len = s.size() - 1;
  auto next_word = [&](size_t& b, size_t& e) -> bool {
    while (p < len && is_space(s[p])) p++;
    if (p >= len) return false;
    b = p;
    while (p < len && !is_space(s[p])) p++;
    e = p;
    return true;
  };
  size_t b, e;
  if (!next_word(b, e) || std::string(&s[b], e - b) != "AdjacencyGraph") {
    return fail(RG_EFORMAT, "rg_read_graph: Bad input file (header)");
  }
  auto next_num = [&](uint64_t& v) -> bool {
    size_t bb, ee;
    if (!next_word(bb, ee)) return false;
    uint64_t x = 0;
    for (size_t i = bb; i < ee; i++) {
      if (s[i] < '0' || s[i] > '9') return false;
      x = x * 10 + (uint64_t)(s[i] - '0');
    }
    v = x;
    return true;
  };
  uint64_t n = 0, m = 0;
  if (!next_num(n) || !next_num(m) || n == 0) return fail(RG_EFORMAT, "rg_read_graph: Bad input file (n/m)");
  if (m > 0xFFFFFFFFull) return fail(RG_EUNSUPPORTED, "rg_read_graph: >= 2^32 edges");
  std::vector<uint32_t> off(n + 1);
  std::vector<uint32_t> tmp(m);
  for (uint64_t i = 0; i < n; i++) {
    uint64_t v;
    if (!next_num(v) || v > m) return fail(RG_EFORMAT, "rg_read_graph: Bad input file (offsets)");
    off[i] = (uint32_t)v;
  }
  off[n] = (uint32_t)m;
  for (uint64_t i = 0; i < m; i++) {
    uint64_t v;
    if (!next_num(v) || v >= n) return fail(RG_EFORMAT, "rg_read_graph: Bad input file (edges)");
    tmp[i] = (uint32_t)v;
  }
  uint64_t extra;
  if (next_num(extra)) return fail(RG_EFORMAT, "rg_read_graph: Bad input file (trailing data)");
  for (uint64_t i = 0; i < n; i++) {
    if (off[i] > off[i + 1]) return fail(RG_EFORMAT, "rg_read_graph: offsets not monotone");
  }
  *n_out = (int64_t)n;
  return clean_and_pack((int64_t)n, off, tmp, off_out, adj_out, m_out);
}

// GAP serialized graph (.sg, GAP/src/reader.h:251-304, written by
// writer.h): bool directed; int64 num_edges (directed entries); int64
// num_nodes; int64 offsets[num_nodes+1]; int32 neighbours[num_edges]; a
// directed graph may follow with its in-lists in the same layout (reader.h:
// 290-295).  GAP's builder has already sorted and deduplicated the lists
// (builder.h:188-244), so the out-lists are taken as is after bounds checks;
// in-lists are rebuilt on the device (rg_graph_create_directed).  Directed
// files are refused when the caller passes no directed_out.
rg_status read_sg(const char* path, int* directed_out, int64_t* n_out, int64_t* m_out, uint32_t** off_out,
                  uint32_t** adj_out) {
  if (!path || !n_out || !m_out || !off_out || !adj_out) return fail(RG_EINVAL, "rg_read_sg: null argument");
  std::vector<char> f;
  if (!read_file(path, f)) return fail(RG_EIO, "rg_read_sg: cannot open %s", path);
  const size_t head = 1 + 8 + 8;
  if (f.size() < head) return fail(RG_EFORMAT, "rg_read_sg: file too short");
  const bool directed = f[0] != 0;
  int64_t m = 0, n = 0;
  memcpy(&m, f.data() + 1, 8);
  memcpy(&n, f.data() + 9, 8);
  if (directed && !directed_out) return fail(RG_EUNSUPPORTED, "rg_read_sg: directed graph (pass directed_out)");
  if (n <= 0 || m < 0) return fail(RG_EFORMAT, "rg_read_sg: bad node or edge count");
  if (n >= 0xFFFFFFFFll || m >= 0xFFFFFFFFll) return fail(RG_EUNSUPPORTED, "rg_read_sg: >= 2^32 nodes or edges");
  const size_t need = head + 8 * (size_t)(n + 1) + 4 * (size_t)m;
  const bool with_inverse = directed && f.size() == head + 2 * (need - head);
  if (f.size() != need && !with_inverse) {
    return fail(RG_EFORMAT, "rg_read_sg: file size %zu, expected %zu", f.size(), need);
  }
  uint32_t* o = (uint32_t*)malloc(4 * (n + 1));
  uint32_t* a = (uint32_t*)malloc(4 * (m + 4));
  if (!o || !a) { free(o); free(a); return fail(RG_ENOMEM, "host malloc failed"); }
  const char* offs = f.data() + head;
  const char* nbrs = offs + 8 * (n + 1);
  bool bad = false;
  for (int64_t i = 0; i <= n && !bad; i++) {
    int64_t x;
    memcpy(&x, offs + 8 * i, 8);
    bad = x < 0 || x > m || (i > 0 && (uint32_t)x < o[i - 1]) || (i == 0 && x != 0) || (i == n && x != m);
    o[i] = (uint32_t)x;
  }
  for (int64_t j = 0; j < m && !bad; j++) {
    int32_t v;
    memcpy(&v, nbrs + 4 * j, 4);
    bad = v < 0 || v >= n;
    a[j] = (uint32_t)v;
  }
  if (bad) { free(o); free(a); return fail(RG_EFORMAT, "rg_read_sg: offsets or neighbour ids out of range"); }
  memset(a + m, 0, 16);
  if (directed_out) *directed_out = directed ? 1 : 0;
  *n_out = n; *m_out = m; *off_out = o; *adj_out = a;
  return RG_OK;
}

// GAP text edge lists (GAP/src/reader.h:50-248), chosen by the file suffix:
//   .el     "u v" pairs, ids as written                       (ReadInEL)
//   .wel    "u v w", weight ignored                             (ReadInWEL)
//   .gr     DIMACS: lines "a u v w" only, ids as written        (ReadInGR)
//   .graph  METIS: '%' comments, header "n m [fmt]" (fmt 1: weighted
//           lists, 0 or 100: plain), then line u (from 0) lists its
//           neighbours 1-based, weights after each when fmt is 1 (ReadInMetis)
//   .mtx    MatrixMarket "matrix coordinate pattern|real|double|integer
//           symmetric|general|skew-symmetric", '%' comments, "rows cols nnz"
//           (square), entries "i j [w]" 1-based; symmetric adds (j, i) too
//           (ReadInMTX)
// The vertex count is the largest id + 1, as GAP's builder takes it
// (builder.h:74-83); the edges are returned as read, for rg_csr_from_edges
// or the device builders to clean up (builder.h:188-244's squish).
namespace {

struct TextScan {
  const char* p;
  const char* end;
  void skip_blank() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\r')) p++;
  }
  void skip_space() {
    while (p < end && is_space(*p)) p++;
  }
  bool at_eol() const { return p >= end || *p == '\n'; }
  void next_line() {
    while (p < end && *p != '\n') p++;
    if (p < end) p++;
  }
  // an integer token (optional sign); a real token's integer part is read
  // and the rest of the token skipped (weights are not used)
  bool integer(int64_t& v) {
    bool neg = false;
    if (p < end && (*p == '-' || *p == '+')) neg = *p++ == '-';
    if (p >= end || *p < '0' || *p > '9') return false;
    int64_t x = 0;
    while (p < end && *p >= '0' && *p <= '9') {
      x = x * 10 + (*p - '0');
      if (x > (int64_t)1 << 40) return false;
      p++;
    }
    while (p < end && !is_space(*p)) p++;
    v = neg ? -x : x;
    return true;
  }
  bool skip_token() {  // a weight: any non-blank token
    if (p >= end || is_space(*p)) return false;
    while (p < end && !is_space(*p)) p++;
    return true;
  }
  std::string word() {
    skip_space();
    const char* b = p;
    while (p < end && !is_space(*p)) p++;
    return std::string(b, p - b);
  }
};

}  // namespace

rg_status read_edges(const char* path, int64_t* n_out, int64_t* ne_out, uint32_t** src_out, uint32_t** dst_out) {
  if (!path || !n_out || !ne_out || !src_out || !dst_out) return fail(RG_EINVAL, "rg_read_edges: null argument");
  const std::string name(path);
  const size_t dot = name.rfind('.');
  const std::string suffix = dot == std::string::npos ? "" : name.substr(dot);
  if (suffix != ".el" && suffix != ".wel" && suffix != ".gr" && suffix != ".graph" && suffix != ".mtx") {
    return fail(RG_EINVAL, "rg_read_edges: unrecognized suffix '%s' (.el .wel .gr .graph .mtx)", suffix.c_str());
  }
  std::vector<char> buf;
  if (!read_file(path, buf)) return fail(RG_EIO, "rg_read_edges: cannot open %s", path);
  TextScan t{buf.data(), buf.data() + buf.size()};
  std::vector<uint32_t> src, dst;
  int64_t max_id = -1;
  auto add = [&](int64_t u, int64_t v) -> bool {
    if (u < 0 || v < 0 || u >= 0xFFFFFFFFll || v >= 0xFFFFFFFFll) return false;
    src.push_back((uint32_t)u);
    dst.push_back((uint32_t)v);
    max_id = std::max(max_id, std::max(u, v));
    return true;
  };
  auto bad = [&](const char* what) { return fail(RG_EFORMAT, "rg_read_edges: %s in %s", what, path); };
  if (suffix == ".el" || suffix == ".wel") {
    const int per = suffix == ".el" ? 2 : 3;
    for (;;) {
      t.skip_space();
      if (t.p >= t.end) break;
      int64_t x[2];
      for (int k = 0; k < 2; k++) {
        t.skip_space();
        if (!t.integer(x[k])) return bad("malformed edge");
      }
      if (per == 3) {
        t.skip_space();
        if (!t.skip_token()) return bad("malformed weight");
      }
      if (!add(x[0], x[1])) return bad("vertex id out of range");
    }
  } else if (suffix == ".gr") {
    while (t.p < t.end) {
      if (*t.p == 'a') {
        t.p++;
        int64_t u, v;
        t.skip_blank();
        if (!t.integer(u)) return bad("malformed arc");
        t.skip_blank();
        if (!t.integer(v)) return bad("malformed arc");
        t.skip_blank();
        if (!t.skip_token()) return bad("malformed arc weight");
        if (!add(u, v)) return bad("vertex id out of range");
      }
      t.next_line();
    }
  } else if (suffix == ".graph") {
    while (t.p < t.end && *t.p == '%') t.next_line();
    int64_t nn, mm, fmt = 0;
    t.skip_blank();
    if (!t.integer(nn)) return bad("malformed METIS header");
    t.skip_blank();
    if (!t.integer(mm)) return bad("malformed METIS header");
    t.skip_blank();
    if (!t.at_eol() && !t.integer(fmt)) return bad("malformed METIS header");
    if (fmt != 0 && fmt != 1 && fmt != 100) return fail(RG_EUNSUPPORTED, "rg_read_edges: METIS fmt %lld", (long long)fmt);
    t.next_line();
    for (int64_t u = 0; u < nn && t.p < t.end;) {
      if (*t.p == '%') {
        t.next_line();
        continue;
      }
      for (;;) {
        t.skip_blank();
        if (t.at_eol()) break;
        int64_t v;
        if (!t.integer(v)) return bad("malformed METIS list");
        if (fmt == 1) {
          t.skip_blank();
          if (!t.skip_token()) return bad("malformed METIS weight");
        }
        if (!add(u, v - 1)) return bad("vertex id out of range");
      }
      t.next_line();
      u++;
    }
  } else {  // .mtx
    if (t.word() != "%%MatrixMarket") return bad(".mtx file did not start with %%MatrixMarket");
    const std::string object = t.word(), format = t.word(), field = t.word(), symmetry = t.word();
    if (object != "matrix" || format != "coordinate") return bad("only matrix coordinate format for .mtx");
    bool weights;
    if (field == "pattern") weights = false;
    else if (field == "real" || field == "double" || field == "integer") weights = true;
    else return bad("unsupported .mtx field type");
    bool undirected;
    if (symmetry == "symmetric") undirected = true;
    else if (symmetry == "general" || symmetry == "skew-symmetric") undirected = false;
    else return bad("unsupported .mtx symmetry type");
    t.next_line();
    while (t.p < t.end && *t.p == '%') t.next_line();
    int64_t rows, cols, nnz;
    t.skip_space();
    if (!t.integer(rows)) return bad("malformed .mtx size line");
    t.skip_blank();
    if (!t.integer(cols)) return bad("malformed .mtx size line");
    t.skip_blank();
    if (!t.integer(nnz)) return bad("malformed .mtx size line");
    if (rows != cols) return bad("matrix must be square for .mtx");
    t.next_line();
    while (t.p < t.end) {
      t.skip_blank();
      if (t.at_eol()) {
        t.next_line();
        continue;
      }
      int64_t i, j;
      if (!t.integer(i)) return bad("malformed .mtx entry");
      t.skip_blank();
      if (!t.integer(j)) return bad("malformed .mtx entry");
      if (weights) {
        t.skip_blank();
        if (!t.skip_token()) return bad("malformed .mtx weight");
      }
      if (!add(i - 1, j - 1)) return bad("vertex id out of range");
      if (undirected && !add(j - 1, i - 1)) return bad("vertex id out of range");
      t.next_line();
    }
  }
  const int64_t ne = (int64_t)src.size();
  if (max_id + 1 >= 0xFFFFFFFFll) return fail(RG_EUNSUPPORTED, "rg_read_edges: >= 2^32 vertices");
  uint32_t* s_out = (uint32_t*)malloc(4 * (size_t)std::max<int64_t>(ne, 1));
  uint32_t* d_out = (uint32_t*)malloc(4 * (size_t)std::max<int64_t>(ne, 1));
  if (!s_out || !d_out) { free(s_out); free(d_out); return fail(RG_ENOMEM, "host malloc failed"); }
  if (ne) {
    memcpy(s_out, src.data(), 4 * (size_t)ne);
    memcpy(d_out, dst.data(), 4 * (size_t)ne);
  }
  *n_out = max_id + 1;
  *ne_out = ne;
  *src_out = s_out;
  *dst_out = d_out;
  return RG_OK;
}

}  // namespace rg
