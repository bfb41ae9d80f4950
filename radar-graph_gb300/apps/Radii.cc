// Radii (Radii.C:140-218): 64 samples hashInt(i) % n, 64-bit masks.
#include "cli.h"

using namespace rg_cli;

void Compute(Graph& G, commandLine& P) {
  std::vector<int32_t> radii(G.n);
  int64_t rounds = 0;
  Timer t;
  t.start();
  if (rg_radii(G.g, G.variant, radii.data(), &rounds) != RG_OK) die("radii");
  const double secs = t.stop();
  printf("Radii: %lld rounds\n", (long long)rounds);
  report("Radii", G, secs);
  write_output(P, radii);
}

int main(int argc, char** argv) { return run(argc, argv, Compute); }
