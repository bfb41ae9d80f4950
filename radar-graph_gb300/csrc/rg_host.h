// Internal host-side declarations shared by the library's translation units.
#pragma once

#include <stdint.h>

#include "../../include/radar_graph.h"

namespace rg {

// Records a one-line message for rg_last_error() and returns `s`.
rg_status fail(rg_status s, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
void clear_error();

rg_status generate_edges(int scale, int edge_factor, uint64_t seed, int uniform, uint32_t* src,
                         uint32_t* dst);
rg_status csr_from_edges(int64_t n, int64_t ne, const uint32_t* src, const uint32_t* dst,
                         uint32_t** off_out, uint32_t** adj_out, int64_t* m_out);
rg_status write_adjacency(const char* path, int64_t n, int64_t m, const uint32_t* off,
                          const uint32_t* adj);
rg_status read_sg(const char* path, int* directed_out, int64_t* n_out, int64_t* m_out, uint32_t** off_out,
                  uint32_t** adj_out);
rg_status read_edges(const char* path, int64_t* n_out, int64_t* ne_out, uint32_t** src_out, uint32_t** dst_out);
rg_status read_graph(const char* path, int symmetric, int binary, int64_t* n_out, int64_t* m_out,
                     uint32_t** off_out, uint32_t** adj_out);

// Ligra's 64-bit hashInt (utils.h:350-358), a published integer mix whose
// constants decide which vertices Radii samples, so they must be the same.
inline uint64_t hash_u64(uint64_t a) {
  a = (a + 0x7ed55d166bef7a1dULL) + (a << 12);
  a = (a ^ 0xc761c23c510fa2ddULL) ^ (a >> 9);
  a = (a + 0x165667b183a9c0e1ULL) + (a << 59);
  a = (a + 0xd3a2646cab3487e3ULL) ^ (a << 49);
  a = (a + 0xfd7046c5ef9ab54cULL) + (a << 3);
  a = (a ^ 0xb55a4f090dd4a67bULL) ^ (a >> 32);
  return a;
}

}  // namespace rg
