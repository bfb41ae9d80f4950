// Host-side helpers shared by the app drivers (apps.cu, pagerank.cu):
// per-call timing, device attributes, hub set-up, result download.
#pragma once

#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <utility>
#include <vector>

#include "engine.cuh"
#include "rg_device.cuh"

namespace rg {

extern thread_local rg_timing g_timing;
extern bool g_kernel_timing;

// rg_set_option values
struct Options {
  int64_t direction = 0;     // RG_OPT_DIRECTION
  int64_t hub_slots = 0;     // RG_OPT_HUB_SLOTS
  int64_t hub_smem_kb = 48;  // RG_OPT_HUB_SMEM_KB
  int64_t dense_div = 20;    // RG_OPT_DENSE_DIV
};
extern Options g_opts;

// Events around one edge-kernel launch (only when rg_set_kernel_timing(1)).
void kt_begin(cudaStream_t st);
void kt_end(cudaStream_t st);

// CUDA events on the graph's stream around the device work of one app call.
struct CallTimer {
  rg_graph* g;
  explicit CallTimer(rg_graph* gr);
  rg_status stop();
};

int device_sms();
int max_dyn_smem();

// Hub slots that fit the push kernel's shared-memory budget (elem bytes each).
uint32_t hub_budget(size_t elem, int64_t n);
// HUBDUP hub set (identifyHubs): bitmap + vertex->slot + slot->vertex.
rg_status hub_map(const rg_graph* g, uint32_t H, HubInfo& info);
int hub_mode_of(int variant);
uint32_t to_internal(const rg_graph* g, uint32_t orig);

// out[v] = in[new_ids[v]]: results in original-id order (writeOutputToFile).
template <class T>
__global__ void gather_kernel(const T* __restrict__ in, const uint32_t* __restrict__ new_ids, int64_t n,
                              T* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (; i < n; i += (int64_t)gridDim.x * blockDim.x) out[i] = in[new_ids[i]];
}

template <class T>
rg_status download_orig(rg_graph* g, const T* d_arr, T* h_out, DevBuf& tmp, cudaStream_t st) {
  if (!h_out) return RG_OK;
  const T* src = d_arr;
  if (g->sorted) {
    RG_TRY(tmp.reserve(sizeof(T) * g->n));
    int64_t blocks = std::min<int64_t>((g->n + 255) / 256, (int64_t)device_sms() * 32);
    gather_kernel<T><<<(unsigned)blocks, 256, 0, st>>>(d_arr, g->new_ids.as<uint32_t>(), g->n, tmp.as<T>());
    RG_CUDA(cudaGetLastError());
    g_timing.kernel_launches++;
    src = tmp.as<T>();
  }
  RG_CUDA(cudaMemcpyAsync(h_out, src, sizeof(T) * g->n, cudaMemcpyDeviceToHost, st));
  return RG_OK;
}

}  // namespace rg
