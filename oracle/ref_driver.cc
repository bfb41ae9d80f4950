// Driver that runs ONE of the reference's own, unmodified app sources (chosen
// at compile time with -DRG_APP="<path to src/<variant>/Ligra/apps/<App>.C>")
// and captures its per-vertex result arrays.
//
// This is test infrastructure that exists only where the reference sources
// are present: oracle/Makefile compiles it into oracle/_ref/, and the golden
// vector script in tests/golden/ runs it.  Nothing in the product uses it.
//
// How it works without touching the reference sources:
//  * parallel.h is included first and `parallel_main` is renamed, so the
//    reference's main (ligra.h:556-651) becomes ref_parallel_main and this
//    file supplies the real main with the same load/preprocess steps
//    (ligra.h:597-604), but calls Compute once and then dumps.
//  * Before the app file is included, Ligra's `newA` allocation macro
//    (utils.h:45) is redirected to a size-recording malloc, and `free` to a
//    hook that copies the block out before releasing it.  The apps free their
//    result arrays at the end of Compute (PageRank.C:179, BFS.C:187,
//    BC-manyiter-v2.C:353-355, Radii.C:199-218), so the captured blocks are
//    the final results.  Every per-vertex output dump in the apps is
//    commented out (PageRank.C:178 ...), which is why this is needed.
//
// Usage: <bin> [-s] [-preprocess p] [-maxiters k] [-r root] -dump <out> <graph>
// Output file: repeated records {u64 nbytes; bytes}: the loaded graph's CSR
// offsets (n+1 x u32) and neighbours (m x u32) -- followed, for a directed
// graph (no -s), by the in-lists in the same form -- the new_ids permutation
// (n x u32), then every captured block in free() order.

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <random>
#include <string>
#include <vector>

#include "parallel.h"
#undef parallel_main
#define parallel_main ref_parallel_main
#include "ligra.h"

namespace rgref {
std::map<void*, size_t> g_sizes;
std::vector<std::vector<char>> g_captured;
void* alloc(size_t bytes) {
  void* p = malloc(bytes);
  g_sizes[p] = bytes;
  return p;
}
void release(void* p) {
  auto it = g_sizes.find(p);
  if (it != g_sizes.end()) {
    const char* c = static_cast<const char*>(p);
    g_captured.emplace_back(c, c + it->second);
    g_sizes.erase(it);
  }
  std::free(p);
}
}  // namespace rgref

#undef newA
#define newA(__E, __n) (__E*)rgref::alloc((__n) * sizeof(__E))
#define free(p) rgref::release((void*)(p))
#include RG_APP
#undef free

static void put(FILE* f, const void* p, uint64_t nbytes) {
  fwrite(&nbytes, 8, 1, f);
  if (nbytes) fwrite(p, 1, nbytes, f);
}

// Loads, optionally degree-sorts, runs Compute once and dumps (templated on
// the reference's vertex type: symmetricVertex, or asymmetricVertex for a
// directed graph, whose in-lists are dumped after the out-lists).
template <class vertex>
int run(commandLine& P, char* iFile, bool symmetric, bool binary, int preprocess, const char* dump) {
  graph<vertex> G = readGraph<vertex>(iFile, false, symmetric, binary, false);
  pvector<uintE> new_ids(G.n, 0);
  FILE* f = fopen(dump, "wb");
  {  // the loaded (cleaned) graph: out-lists as CSR, then (directed) in-lists
    for (int in = 0; in < (symmetric ? 1 : 2); in++) {
      std::vector<uint32_t> off(G.n + 1), adj;
      adj.reserve(G.m);
      for (long v = 0; v < G.n; v++) {
        off[v] = (uint32_t)adj.size();
        const uintT d = in ? G.V[v].getInDegree() : G.V[v].getOutDegree();
        for (uintT j = 0; j < d; j++) adj.push_back(in ? G.V[v].getInNeighbor(j) : G.V[v].getOutNeighbor(j));
      }
      off[G.n] = (uint32_t)adj.size();
      put(f, off.data(), 4ull * off.size());
      put(f, adj.data(), 4ull * adj.size());
    }
  }
  if (preprocess == 0 || preprocess == 1) {
    graph<vertex> newG = preprocessGraph<vertex>(G, symmetric, (preprocess == 0), new_ids);
    G.del();
    put(f, new_ids.data(), 4ull * newG.n);
    Compute(newG, P, new_ids);
    newG.del();
  } else {
    put(f, new_ids.data(), 4ull * G.n);
    Compute(G, P, new_ids);
    G.del();
  }
  for (auto& b : rgref::g_captured) put(f, b.data(), b.size());
  fclose(f);
  return 0;
}

int main(int argc, char* argv[]) {
  commandLine P(argc, argv, " [-s] -dump <out> <inFile>");
  char* iFile = P.getArgument(0);
  bool symmetric = P.getOptionValue("-s");
  bool binary = P.getOptionValue("-b");
  char* dump = P.getOptionValue("-dump");
  int preprocess = P.getOptionIntValue("-preprocess", -1);
  if (dump == nullptr) {
    fprintf(stderr, "ref_driver: needs -dump\n");
    return 2;
  }
  if (symmetric) return run<symmetricVertex>(P, iFile, true, binary, preprocess, dump);
  return run<asymmetricVertex>(P, iFile, false, binary, preprocess, dump);
}
