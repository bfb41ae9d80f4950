// BFS (BFS.C:122-188): -r root (original id, default 0).  -out writes depths
// (-1 unreached); parents are in the internal id space like the reference's.
#include "cli.h"

using namespace rg_cli;

void Compute(Graph& G, commandLine& P) {
  const long root = P.getOptionLongValue("-r", 0);
  if (root < 0 || root >= G.n) {
    fprintf(stderr, "root %ld out of range\n", root);
    exit(2);
  }
  std::vector<int32_t> depth(G.n);
  int64_t rounds = 0, reached = 0;
  Timer t;
  t.start();
  if (rg_bfs(G.g, G.variant, (uint32_t)root, nullptr, depth.data(), &rounds, &reached) != RG_OK) die("bfs");
  const double secs = t.stop();
  printf("BFS: %lld vertices reached in %lld rounds\n", (long long)reached, (long long)rounds);
  report("BFS", G, secs);
  write_output(P, depth);
}

int main(int argc, char** argv) { return run(argc, argv, Compute); }
