// Gather ceiling of a graph: the time to stream the graph's edge array and
// gather one 8-byte value per edge (value[adj[e]]), with perfect balance and
// nothing else -- no row bookkeeping, no reduction beyond one sum per warp.
// Every pull over the graph (the PageRank sweep, the bitmask sweeps) does at
// least this work, so it is the achievable ceiling those kernels are measured
// against, next to the HBM copy bandwidth.
//
// A measurement aid, not part of the engine: it is built into its own
// library (librg_probe.so, linked against librg.so for the graph handle and
// the thread's stream) that only the benchmark loads; librg.so does not
// export it.

#include <cuda_runtime.h>

#include <algorithm>

#include "app_common.cuh"

namespace rg {
namespace {

__global__ void __launch_bounds__(256) gather_probe(const uint32_t* __restrict__ adj, uint32_t m,
                                                    const uint64_t* __restrict__ value, unsigned long long* out) {
  constexpr int kItems = 8;
  unsigned long long acc = 0;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * kItems;
  for (uint64_t e = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) * kItems; e < m; e += stride) {
    const U32x8 w = ld_stream_v8(adj + e);  // in bounds: adj is padded by 8 entries
#pragma unroll
    for (int i = 0; i < kItems; i++) acc += (e + i < m) ? __ldg(value + w.v[i]) : 0ull;
  }
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

}  // namespace
}  // namespace rg

using namespace rg;

extern "C" rg_status rg_probe_gather_ceiling(rg_graph* g, int reps, double* best_ms) {
  if (!g || reps < 1 || !best_ms) return fail(RG_EINVAL, "rg_probe_gather_ceiling: bad arguments");
  if (g->m == 0) return fail(RG_EINVAL, "rg_probe_gather_ceiling: graph has no edges");
  Ctx* cx = nullptr;
  RG_TRY(get_ctx(&cx));
  cudaStream_t st = cx->stream;
  DevBuf value, out;
  RG_TRY(value.reserve(8 * (size_t)g->n));
  RG_TRY(out.reserve(8));
  RG_CUDA(cudaMemsetAsync(value.p, 0, 8 * (size_t)g->n, st));
  int per_sm = 0;
  RG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gather_probe, 256, 0));
  RG_CUDA(cudaFuncSetAttribute(gather_probe, cudaFuncAttributePreferredSharedMemoryCarveout, 0));
  const int64_t grid = std::min<int64_t>((int64_t)device_sms() * std::max(per_sm, 1), (g->m + 2047) / 2048);
  double best = 1e30;
  for (int r = 0; r <= reps; r++) {  // the first run warms up
    RG_CUDA(cudaEventRecord(cx->ev0, st));
    gather_probe<<<(unsigned)std::max<int64_t>(grid, 1), 256, 0, st>>>(g->adj.as<uint32_t>(), (uint32_t)g->m,
                                                                       value.as<uint64_t>(),
                                                                       out.as<unsigned long long>());
    RG_CUDA(cudaGetLastError());
    RG_CUDA(cudaEventRecord(cx->ev1, st));
    RG_CUDA(cudaEventSynchronize(cx->ev1));
    float ms = 0;
    RG_CUDA(cudaEventElapsedTime(&ms, cx->ev0, cx->ev1));
    if (r > 0) best = std::min(best, (double)ms);
  }
  *best_ms = best;
  return RG_OK;
}
