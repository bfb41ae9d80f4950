// Command-line front end shared by the PageRank, BFS, BC and Radii binaries.
//
// Each binary keeps the reference app's command line and run shape
// (ligra.h:556-651, parseCommandLine.h:47-100):
//
//   <App> [-s] [-b] [-rounds R] [-preprocess p] [-r root] [-maxiters k]
//         [-variant push|push-pull|degree-sorting|hubdup|radar] [-out file] <graph>
//
// The graph file is read (Ligra AdjacencyGraph text, or the binary
// .config/.adj/.idx triple with -b; symmetric with -s, else directed),
// uploaded to the GPU and, when -preprocess
// is 0 or 1 (the default of the degree-sorting and RADAR variants), degree
// sorted on the device.  Compute(G, P) then runs 1 + rounds times, each timed,
// as parallel_main does.  Results go through the C ABI in
// include/radar_graph.h; -out writes the last round's per-vertex result in
// original-id order, one value per line (17 significant digits for doubles).

#pragma once

#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <chrono>
#include <string>
#include <type_traits>
#include <vector>

#include "radar_graph.h"

namespace rg_cli {

// Flags and the trailing input file, looked up like commandLine in
// parseCommandLine.h:47-100 (a flag's value is the argument after it).
class commandLine {
 public:
  commandLine(int argc, char** argv) : argv_(argv + 1, argv + argc) {}
  bool getOption(const char* flag) const { return find(flag) >= 0; }
  const char* getOptionValue(const char* flag, const char* dflt) const {
    const int i = find(flag);
    return (i >= 0 && i + 1 < (int)argv_.size()) ? argv_[i + 1] : dflt;
  }
  long getOptionLongValue(const char* flag, long dflt) const {
    const char* v = getOptionValue(flag, nullptr);
    return v ? strtol(v, nullptr, 10) : dflt;
  }
  // the input file: the last argument (parseCommandLine.h:50-53)
  const char* getArgument() const { return argv_.empty() ? nullptr : argv_.back(); }

 private:
  int find(const char* flag) const {
    for (int i = 0; i + 1 < (int)argv_.size(); i++)  // the last argument is the file
      if (strcmp(argv_[i], flag) == 0) return i;
    return -1;
  }
  std::vector<char*> argv_;
};

struct Graph {
  rg_graph* g = nullptr;
  rg_variant variant = RG_RADAR;
  int64_t n = 0, m = 0;
  bool sorted = false;
  const char* file = "";
  const char* variant_name = "radar";
  double peak_gbs = 0;    // HBM roofline denominator of the JSON line
  const char* peak_kind = "nominal";
};

inline void die(const char* what) {
  fprintf(stderr, "%s: %s\n", what, rg_last_error());
  exit(1);
}

// GAP's text edge-list suffixes (GAP/src/reader.h:219-248)
inline bool gap_edge_list(const char* path) {
  const char* dot = strrchr(path, '.');
  if (!dot) return false;
  for (const char* sfx : {".el", ".wel", ".gr", ".graph", ".mtx"}) {
    if (strcmp(dot, sfx) == 0) return true;
  }
  return false;
}

inline rg_variant parse_variant(const char* s) {
  if (!strcmp(s, "push") || !strcmp(s, "push-new-orig")) return RG_PUSH;
  if (!strcmp(s, "push-pull")) return RG_PUSH_PULL;
  if (!strcmp(s, "degree-sorting") || !strcmp(s, "degsort")) return RG_DEGSORT;
  if (!strcmp(s, "hubdup")) return RG_HUBDUP;
  if (!strcmp(s, "radar") || !strcmp(s, "RADAR")) return RG_RADAR;
  fprintf(stderr, "unknown variant '%s'\n", s);
  exit(2);
}

class Timer {
 public:
  void start() { t0_ = std::chrono::steady_clock::now(); }
  double stop() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
  }

 private:
  std::chrono::steady_clock::time_point t0_;
};

template <class T>
void write_output(const commandLine& P, const std::vector<T>& v) {
  const char* path = P.getOptionValue("-out", nullptr);
  if (!path) return;
  FILE* f = fopen(path, "w");
  if (!f) {
    fprintf(stderr, "cannot write %s\n", path);
    exit(1);
  }
  for (const T& x : v) {
    if constexpr (std::is_floating_point<T>::value) {
      fprintf(f, "%.17g\n", (double)x);
    } else {
      fprintf(f, "%lld\n", (long long)x);
    }
  }
  fclose(f);
}

// JSON string body: the path with quotes, backslashes and control bytes escaped
inline void json_str(FILE* f, const char* x) {
  fputc('"', f);
  for (const unsigned char* c = (const unsigned char*)x; *c; c++) {
    if (*c == '"' || *c == '\\') fprintf(f, "\\%c", *c);
    else if (*c < 0x20) fprintf(f, "\\u%04x", *c);
    else fputc(*c, f);
  }
  fputc('"', f);
}

// The reference's "Run Time(sec)" line (PageRank.C:185-186 and the other
// apps' ends), then one JSON result line: app, variant, graph, size, time,
// GTEPS and the fraction of the HBM roofline the call's algorithmic bytes
// reached (peak: -hbm-gbs or $RG_HBM_GBS, e.g. a measured copy bandwidth;
// else the device's nominal figure).
inline void report(const char* app, const Graph& G, double secs) {
  rg_timing t;
  if (rg_last_timing(&t) != RG_OK) memset(&t, 0, sizeof t);
  const double gteps = t.total_ms > 0 ? (double)t.edges_traversed / (t.total_ms * 1e6) : 0.0;
  printf("Run Time(sec) : %.6f   [%s, %s graph, device %.3f ms, %lld edges, %.2f GTEPS]\n", secs, app,
         G.sorted ? "degree-sorted" : "original", t.total_ms, (long long)t.edges_traversed, gteps);
  char gpu[256] = "";
  rg_device_info(gpu, sizeof gpu, nullptr, nullptr);
  const double gbs = t.total_ms > 0 ? (double)t.algorithmic_bytes / (t.total_ms * 1e6) : 0.0;
  printf("{\"app\": \"%s\", \"variant\": \"%s\", \"graph\": ", app, G.variant_name);
  json_str(stdout, G.file);
  printf(", \"n\": %lld, \"m\": %lld, \"degree_sorted\": %s, \"run_time_s\": %.6f, \"device_ms\": %.4f, "
         "\"edges\": %lld, \"gteps\": %.6g, \"algorithmic_bytes\": %lld, \"achieved_gbs\": %.6g, "
         "\"hbm_peak_gbs\": %.1f, \"peak_kind\": \"%s\", \"hbm_frac\": %.6g, \"gpu\": ",
         (long long)G.n, (long long)G.m, G.sorted ? "true" : "false", secs, t.total_ms,
         (long long)t.edges_traversed, gteps, (long long)t.algorithmic_bytes, gbs, G.peak_gbs, G.peak_kind,
         G.peak_gbs > 0 ? gbs / G.peak_gbs : 0.0);
  json_str(stdout, gpu);
  printf("}\n");
  fflush(stdout);
}

using ComputeFn = void (*)(Graph&, commandLine&);

// parallel_main (ligra.h:556-651): load, optional degree sort, 1 + rounds runs.
inline int run(int argc, char** argv, ComputeFn compute) {
  commandLine P(argc, argv);
  const char* file = P.getArgument();
  if (argc < 2 || !file || file[0] == '-') {
    fprintf(stderr,
            "usage: %s [-s] [-b] [-rounds R] [-preprocess p] [-r root] [-maxiters k] "
            "[-variant push|push-pull|degree-sorting|hubdup|radar] [-out file] [-hbm-gbs GB/s] <graph>\n",
            argv[0]);
    return 2;
  }
  Graph G;
  G.file = file;
  G.variant_name = P.getOptionValue("-variant", "radar");
  G.variant = parse_variant(G.variant_name);
  const char* peak = P.getOptionValue("-hbm-gbs", getenv("RG_HBM_GBS"));
  if (peak && atof(peak) > 0) {
    G.peak_gbs = atof(peak);
    G.peak_kind = "given";
  } else {
    rg_device_info(nullptr, 0, nullptr, &G.peak_gbs);  // nominal; 0 without a device
  }
  const bool symmetric = P.getOption("-s");  // without -s the graph is directed
  const long rounds = P.getOptionLongValue("-rounds", 3);
  // degree-sorting and RADAR sort by default (-preprocess 1); the others do not
  const bool sorts_by_default = G.variant == RG_DEGSORT || G.variant == RG_RADAR;
  const long pre = P.getOptionLongValue("-preprocess", sorts_by_default ? 1 : -1);
  rg_graph* g0 = nullptr;
  const char* dot = strrchr(file, '.');
  if (dot && strcmp(dot, ".sg") == 0) {
    // GAP serialized graph: cleaned lists; the file says whether it is directed
    uint32_t *off = nullptr, *adj = nullptr;
    int directed = 0;
    if (rg_read_sg(file, &G.n, &G.m, &off, &adj, &directed) != RG_OK) die("read");
    const rg_status up = directed ? rg_graph_create_directed(G.n, G.m, off, adj, &g0)
                                  : rg_graph_create(G.n, G.m, off, adj, &g0);
    if (up != RG_OK) die("upload");
    rg_host_free(off);
    rg_host_free(adj);
  } else if (gap_edge_list(file)) {
    // GAP text edge lists (.el .wel .gr .graph .mtx): read as written, then
    // cleaned up on the device (both directions with -s, as GAP's -s does)
    int64_t ne = 0;
    uint32_t *src = nullptr, *dst = nullptr;
    if (rg_read_edges(file, &G.n, &ne, &src, &dst) != RG_OK) die("read");
    const rg_status up = symmetric ? rg_graph_create_from_edges(G.n, ne, src, dst, 0, &g0)
                                   : rg_graph_create_directed_from_edges(G.n, ne, src, dst, 0, &g0);
    if (up != RG_OK) die("build");
    rg_host_free(src);
    rg_host_free(dst);
    int64_t m = 0;
    if (rg_graph_info(g0, nullptr, &m, nullptr) != RG_OK) die("info");
    G.m = m;
  } else {
    uint32_t *off = nullptr, *adj = nullptr;
    if (rg_read_graph(file, symmetric ? 1 : 0, P.getOption("-b") ? 1 : 0, &G.n, &G.m, &off, &adj) != RG_OK) {
      die("read");
    }
    const rg_status up = symmetric ? rg_graph_create(G.n, G.m, off, adj, &g0)
                                   : rg_graph_create_directed(G.n, G.m, off, adj, &g0);
    if (up != RG_OK) die("upload");
    rg_host_free(off);
    rg_host_free(adj);
  }
  if (pre == 0 || pre == 1) {  // 0: out-degree, 1: in-degree (the same when symmetric)
    Timer t;
    t.start();
    if (rg_graph_degree_sort_by(g0, pre == 0 ? 1 : 0, &G.g, nullptr) != RG_OK) die("degree sort");
    rg_synchronize();
    printf("DegSort Time : %.6f\n", t.stop());
    rg_graph_free(g0);
    G.sorted = true;
  } else {
    G.g = g0;
  }
  for (long r = 0; r <= rounds; r++) compute(G, P);
  rg_graph_free(G.g);
  return 0;
}

}  // namespace rg_cli
