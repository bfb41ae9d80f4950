// rg_bfs_depth_noalloc: BFS depths for callers that cannot allocate device
// memory.
//
// Some callers of this library must not call cudaMalloc: code that runs
// inside another framework's memory pool (its caching allocator owns the
// device memory, so a stray cudaMalloc can fail or fragment the pool), and
// latency-critical serving loops, where cudaMalloc/cudaFree synchronize the
// device and stall every other stream.  This entry point takes the graph and
// the output as device pointers the caller owns and keeps all of its working
// memory -- two frontier queues, a visited bitmap and a level counter -- in
// one file-scope __device__ array of a fixed size.  Every GPU that loads the
// library holds that array (kScratchBytes) until the process exits.
//
// It is the level-synchronous push BFS of the engine (BFS_F, BFS.C:28-99:
// the first update of an unvisited vertex claims it) reduced to depths.

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "rg_device.cuh"

namespace rg {
namespace {

// Largest graph this entry point accepts, and the scratch it needs:
// 2 queues of kMaxVertices ids + a kMaxVertices-bit bitmap + 256 B counters.
constexpr int64_t kMaxVertices = int64_t(1) << 21;  // 2,097,152
constexpr size_t kQueueBytes = sizeof(uint32_t) * kMaxVertices;
constexpr size_t kBitmapBytes = kMaxVertices / 8;
constexpr size_t kCounterBytes = 256;
constexpr size_t kScratchBytes = 2 * kQueueBytes + kBitmapBytes + kCounterBytes;  // 16.25 MiB + 256 B

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of the scratch array for the current device.  The symbol's
// host-side name is only a stand-in; the address must come from
// cudaGetSymbolAddress with the device current.  It is looked up on every
// call (a cheap driver query next to the per-level host syncs), so a context
// that was reset and re-created never leaves a stale address behind.
rg_status scratch_address(unsigned char** out) {
  void* p = nullptr;
  RG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  *out = static_cast<unsigned char*>(p);
  return RG_OK;
}

__global__ void noalloc_init(int32_t* depth, uint32_t n, uint32_t root, uint32_t* visited, uint32_t* queue0) {
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
    depth[v] = v == root ? 0 : -1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    visited[root >> 5] = 1u << (root & 31);
    queue0[0] = root;
  }
}

// One warp per frontier vertex; the first claim of a neighbour's visited bit
// gives it depth `level` and a slot in the next queue.  A neighbour id >= n
// (a malformed CSR the caller passed as device pointers) is skipped, so it
// can reach neither the bitmap, the queues nor depth[].
__global__ void __launch_bounds__(256) noalloc_expand(const uint32_t* __restrict__ off, const uint32_t* __restrict__ adj,
                                                      const uint32_t* __restrict__ q, uint32_t k, uint32_t n,
                                                      uint32_t* visited, uint32_t* nq, uint32_t* ncount, int32_t* depth,
                                                      int32_t level) {
  const int lane = threadIdx.x & 31;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < k; i += nwarps) {
    const uint32_t s = q[i];
    const uint32_t b = off[s], e = off[s + 1];
    for (uint32_t j = b + lane; j < e; j += 32) {
      const uint32_t d = adj[j];
      if (d >= n) continue;
      const uint32_t bit = 1u << (d & 31);
      if (visited[d >> 5] & bit) continue;
      if (atomicOr(visited + (d >> 5), bit) & bit) continue;
      depth[d] = level;
      nq[atomicAdd(ncount, 1u)] = d;
    }
  }
}

}  // namespace
}  // namespace rg

using namespace rg;

extern "C" rg_status rg_bfs_depth_noalloc(const uint32_t* d_off, const uint32_t* d_adj, int64_t n, int64_t m,
                                          uint32_t root, int32_t* d_depth, void* stream, int64_t* rounds_out) {
  if (!d_off || (m > 0 && !d_adj) || !d_depth) return fail(RG_EINVAL, "rg_bfs_depth_noalloc: null pointer");
  if (n <= 0 || m < 0) return fail(RG_EINVAL, "rg_bfs_depth_noalloc: bad n/m");
  if (n > kMaxVertices) {
    return fail(RG_EINVAL, "rg_bfs_depth_noalloc: n = %lld exceeds the fixed scratch limit of %lld vertices",
                (long long)n, (long long)kMaxVertices);
  }
  if (m >= 0xFFFFFFFFll) return fail(RG_EUNSUPPORTED, "rg_bfs_depth_noalloc: >= 2^32 edges");
  if (root >= (uint64_t)n) return fail(RG_EINVAL, "rg_bfs_depth_noalloc: root %u >= n", root);
  cudaStream_t st = (cudaStream_t)stream;
  unsigned char* base = nullptr;
  RG_TRY(scratch_address(&base));
  uint32_t* q[2] = {reinterpret_cast<uint32_t*>(base), reinterpret_cast<uint32_t*>(base + kQueueBytes)};
  uint32_t* visited = reinterpret_cast<uint32_t*>(base + 2 * kQueueBytes);
  uint32_t* counter = reinterpret_cast<uint32_t*>(base + 2 * kQueueBytes + kBitmapBytes);
  // the array keeps the previous call's contents: clear what must start at zero
  RG_CUDA(cudaMemsetAsync(visited, 0, (size_t)((n + 31) / 32) * 4, st));
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, 4096);
  noalloc_init<<<blocks, 256, 0, st>>>(d_depth, (uint32_t)n, root, visited, q[0]);
  RG_CUDA(cudaGetLastError());
  uint32_t k = 1;
  int64_t rounds = 0;
  int cur = 0;
  while (k > 0) {
    rounds++;
    RG_CUDA(cudaMemsetAsync(counter, 0, 4, st));
    const int eb = (int)std::min<int64_t>(((int64_t)k * 32 + 255) / 256, 8192);
    noalloc_expand<<<eb, 256, 0, st>>>(d_off, d_adj, q[cur], k, (uint32_t)n, visited, q[1 - cur], counter, d_depth, (int32_t)rounds);
    RG_CUDA(cudaGetLastError());
    uint32_t next = 0;
    RG_CUDA(cudaMemcpyAsync(&next, counter, 4, cudaMemcpyDeviceToHost, st));
    RG_CUDA(cudaStreamSynchronize(st));
    k = next;
    cur = 1 - cur;
  }
  if (rounds_out) *rounds_out = rounds;
  return RG_OK;
}
