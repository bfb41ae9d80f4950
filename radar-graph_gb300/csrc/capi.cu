// C ABI glue: error strings, host-side format entry points, device buffers.

#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>

#include "rg_device.cuh"

namespace rg {
const char* last_error();
void drop_hub_cache(const rg_graph* g);
}  // namespace rg

using namespace rg;

extern "C" {

const char* rg_last_error(void) { return last_error(); }

const char* rg_status_str(rg_status s) {
  switch (s) {
    case RG_OK: return "ok";
    case RG_EINVAL: return "invalid argument";
    case RG_ENOMEM: return "out of memory";
    case RG_ECUDA: return "CUDA error";
    case RG_EIO: return "I/O error";
    case RG_EFORMAT: return "bad input format";
    case RG_EUNSUPPORTED: return "unsupported";
    case RG_ETIMEOUT: return "wait timed out";
    case RG_ENODEV: return "no CUDA device";
    case RG_ECANCELED: return "cancelled";
  }
  return "unknown status";
}

const char* rg_version(void) { return "radar-graph-gb300 0.1 sm_103a"; }

rg_status rg_generate_edges(int scale, int edge_factor, uint64_t seed, int uniform, uint32_t* h_src,
                            uint32_t* h_dst) {
  return generate_edges(scale, edge_factor, seed, uniform, h_src, h_dst);
}

rg_status rg_csr_from_edges(int64_t n, int64_t num_edges, const uint32_t* h_src, const uint32_t* h_dst,
                            uint32_t** h_off_out, uint32_t** h_adj_out, int64_t* m_out) {
  return csr_from_edges(n, num_edges, h_src, h_dst, h_off_out, h_adj_out, m_out);
}

rg_status rg_write_adjacency(const char* path, int64_t n, int64_t m, const uint32_t* h_off, const uint32_t* h_adj) {
  return write_adjacency(path, n, m, h_off, h_adj);
}

rg_status rg_read_graph(const char* path, int symmetric, int binary, int64_t* n_out, int64_t* m_out,
                        uint32_t** h_off_out, uint32_t** h_adj_out) {
  return read_graph(path, symmetric, binary, n_out, m_out, h_off_out, h_adj_out);
}

rg_status rg_read_sg(const char* path, int64_t* n_out, int64_t* m_out, uint32_t** h_off_out,
                     uint32_t** h_adj_out, int* directed_out) {
  return read_sg(path, directed_out, n_out, m_out, h_off_out, h_adj_out);
}

rg_status rg_read_edges(const char* path, int64_t* n_out, int64_t* num_edges_out, uint32_t** h_src_out,
                        uint32_t** h_dst_out) {
  return read_edges(path, n_out, num_edges_out, h_src_out, h_dst_out);
}

void rg_host_free(void* p) { free(p); }

rg_status rg_device_alloc(size_t bytes, void** d_ptr) {
  if (!d_ptr || bytes == 0) return fail(RG_EINVAL, "rg_device_alloc: bad arguments");
  RG_CUDA(cudaMalloc(d_ptr, bytes));
  RG_CUDA(cudaMemset(*d_ptr, 0, bytes));
  return RG_OK;
}

rg_status rg_device_free(void* d_ptr) {
  if (d_ptr) RG_CUDA(cudaFree(d_ptr));
  return RG_OK;
}

rg_status rg_copy_to_device(void* d_dst, const void* h_src, size_t bytes) {
  if ((!d_dst || !h_src) && bytes) return fail(RG_EINVAL, "null pointer");
  RG_CUDA(cudaMemcpy(d_dst, h_src, bytes, cudaMemcpyHostToDevice));
  return RG_OK;
}

rg_status rg_copy_to_host(void* h_dst, const void* d_src, size_t bytes) {
  if ((!h_dst || !d_src) && bytes) return fail(RG_EINVAL, "null pointer");
  RG_CUDA(cudaMemcpy(h_dst, d_src, bytes, cudaMemcpyDeviceToHost));
  return RG_OK;
}

rg_status rg_device_info(char* name, int name_len, int32_t* sms, double* nominal_hbm_gbs) {
  int dev = 0;
  RG_CUDA(cudaGetDevice(&dev));
  if (name && name_len > 0) {
    cudaDeviceProp p;
    RG_CUDA(cudaGetDeviceProperties(&p, dev));
    snprintf(name, (size_t)name_len, "%s", p.name);
  }
  if (sms) RG_CUDA(cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev));
  if (nominal_hbm_gbs) {
    int khz = 0, bits = 0;
    RG_CUDA(cudaDeviceGetAttribute(&khz, cudaDevAttrMemoryClockRate, dev));
    RG_CUDA(cudaDeviceGetAttribute(&bits, cudaDevAttrGlobalMemoryBusWidth, dev));
    *nominal_hbm_gbs = 2.0 * (double)khz * 1e3 * (double)bits / 8.0 / 1e9;
  }
  return RG_OK;
}

rg_status rg_synchronize(void) {
  RG_CUDA(cudaDeviceSynchronize());
  return RG_OK;
}

}  // extern "C"
