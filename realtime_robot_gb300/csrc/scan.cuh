// scan.cuh — device-wide exclusive scan of uint32 (counts on host or device).
#pragma once
#include "common.cuh"

namespace rtr {

int scan_tiles(int n_cap);  // scratch entries needed for the tile sums
// out[i] = sum_{j<i} in[i]; *d_total (optional) = sum of all.  in == out is allowed.
void scan_exclusive(const uint32_t* in, uint32_t* out, uint32_t* tile_sums, int n_cap, int n_host,
                    const int* d_n, uint32_t* d_total, cudaStream_t st);

}  // namespace rtr
