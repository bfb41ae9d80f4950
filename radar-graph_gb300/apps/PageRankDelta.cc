// PageRankDelta (PageRankDelta.C:98-155): -maxiters k (default 100), stop
// when the sum of |Delta| drops below 1e-7.
#include "cli.h"

using namespace rg_cli;

void Compute(Graph& G, commandLine& P) {
  const long max_iters = P.getOptionLongValue("-maxiters", 100);
  std::vector<double> ranks(G.n);
  int64_t iters = 0;
  double l1 = 0;
  Timer t;
  t.start();
  if (rg_pagerank_delta(G.g, G.variant, max_iters, ranks.data(), &iters, &l1) != RG_OK) die("pagerank delta");
  const double secs = t.stop();
  printf("PageRankDelta: %lld rounds, L1 %.3e\n", (long long)iters, l1);
  report("PageRankDelta", G, secs);
  write_output(P, ranks);
}

int main(int argc, char** argv) { return run(argc, argv, Compute); }
