// Triangle counting (GAP tc_local): prints the total; -out writes the number
// of triangles containing each vertex.  The degree order tc_local relabels
// to is built internally whatever -preprocess says.
#include "cli.h"

using namespace rg_cli;

void Compute(Graph& G, commandLine& P) {
  std::vector<uint64_t> counts(G.n);
  uint64_t total = 0;
  Timer t;
  t.start();
  if (rg_triangle_count(G.g, counts.data(), &total) != RG_OK) die("triangle count");
  const double secs = t.stop();
  printf("%llu triangles\n", (unsigned long long)total);
  report("TriangleCount", G, secs);
  write_output(P, counts);
}

int main(int argc, char** argv) { return run(argc, argv, Compute); }
