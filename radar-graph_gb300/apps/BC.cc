// BC (BC-manyiter-v2.C:205-367): -maxiters k sources (default 16) drawn like
// the reference; dependencies chained across sources, NaN where unreached.
#include "cli.h"

using namespace rg_cli;

void Compute(Graph& G, commandLine& P) {
  const long k = P.getOptionLongValue("-maxiters", 16);
  std::vector<double> deps(G.n);
  int64_t levels = 0;
  Timer t;
  t.start();
  if (rg_bc(G.g, G.variant, (int)k, deps.data(), &levels) != RG_OK) die("bc");
  const double secs = t.stop();
  printf("BC: %ld sources, %lld forward levels\n", k, (long long)levels);
  report("BC", G, secs);
  write_output(P, deps);
}

int main(int argc, char** argv) { return run(argc, argv, Compute); }
