// PageRank (PageRank.C:120-189): -maxiters k (default 100), stop at L1 < 1e-7.
#include "cli.h"

using namespace rg_cli;

void Compute(Graph& G, commandLine& P) {
  const long max_iters = P.getOptionLongValue("-maxiters", 100);
  std::vector<double> ranks(G.n);
  int64_t iters = 0;
  double l1 = 0;
  Timer t;
  t.start();
  if (rg_pagerank(G.g, G.variant, max_iters, ranks.data(), &iters, &l1) != RG_OK) die("pagerank");
  const double secs = t.stop();
  printf("PageRank: %lld iterations, L1 %.3e\n", (long long)iters, l1);
  report("PageRank", G, secs);
  write_output(P, ranks);
}

int main(int argc, char** argv) { return run(argc, argv, Compute); }
