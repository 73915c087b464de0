// scan.cu — reduce-then-scan exclusive prefix sum (three launches).
#include "scan.cuh"

namespace rtr {

constexpr int SC_BLOCK = 256;
constexpr int SC_ITEMS = 16;
constexpr int SC_TILE = SC_BLOCK * SC_ITEMS;

__device__ __forceinline__ int sc_count(int n_host, const int* d_n) { return d_n ? *d_n : n_host; }

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t ws[SC_BLOCK / 32 + 1];  // warp offsets + block total
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) ws[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < SC_BLOCK / 32 ? ws[lane] : 0u, wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < SC_BLOCK / 32) ws[lane] = wi - w;
    if (lane == SC_BLOCK / 32 - 1) ws[SC_BLOCK / 32] = wi;  // block total (uses slot past the warps)
  }
  __syncthreads();
  const uint32_t r = ws[warp] + incl - v;
  if (total) *total = ws[SC_BLOCK / 32];
  return r;
}

__global__ void __launch_bounds__(SC_BLOCK) k_scan_sums(const uint32_t* __restrict__ in, int n_host,
                                                        const int* d_n, uint32_t* __restrict__ sums) {
  __shared__ uint32_t red[SC_BLOCK / 32];
  const int n = sc_count(n_host, d_n);
  const int base = blockIdx.x * SC_TILE + threadIdx.x * SC_ITEMS;
  uint32_t s = 0;
#pragma unroll
  for (int j = 0; j < SC_ITEMS; ++j)
    if (base + j < n) s += in[base + j];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < SC_BLOCK / 32; ++w) t += red[w];
    sums[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(1024) k_scan_top(uint32_t* __restrict__ h, int total, uint32_t* d_total) {
  __shared__ uint32_t wsum[33];
  const int per = (total + 1023) / 1024;
  const int beg = min(total, (int)threadIdx.x * per), end = min(total, beg + per);
  uint32_t s = 0;
  for (int i = beg; i < end; ++i) s += h[i];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t incl = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) wsum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = wsum[lane], wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    wsum[lane] = wi - w;
    if (lane == 31) wsum[32] = wi;
  }
  __syncthreads();
  uint32_t run = wsum[warp] + incl - s;
  for (int i = beg; i < end; ++i) {
    uint32_t v = h[i];
    h[i] = run;
    run += v;
  }
  if (threadIdx.x == 0 && d_total) *d_total = wsum[32];
}

__global__ void __launch_bounds__(SC_BLOCK) k_scan_apply(const uint32_t* __restrict__ in,
                                                         uint32_t* __restrict__ out, int n_host,
                                                         const int* d_n, const uint32_t* __restrict__ sums) {
  const int n = sc_count(n_host, d_n);
  const int base = blockIdx.x * SC_TILE + threadIdx.x * SC_ITEMS;
  uint32_t v[SC_ITEMS];
  uint32_t s = 0;
#pragma unroll
  for (int j = 0; j < SC_ITEMS; ++j) {
    v[j] = (base + j < n) ? in[base + j] : 0u;
    s += v[j];
  }
  uint32_t run = block_excl_scan(s, nullptr) + sums[blockIdx.x];
#pragma unroll
  for (int j = 0; j < SC_ITEMS; ++j) {
    if (base + j < n) out[base + j] = run;
    run += v[j];
  }
}

int scan_tiles(int n_cap) {
  int t = (n_cap + SC_TILE - 1) / SC_TILE;
  return t < 1 ? 1 : t;
}

void scan_exclusive(const uint32_t* in, uint32_t* out, uint32_t* tile_sums, int n_cap, int n_host,
                    const int* d_n, uint32_t* d_total, cudaStream_t st) {
  const int nt = scan_tiles(n_cap);
  k_scan_sums<<<nt, SC_BLOCK, 0, st>>>(in, n_host, d_n, tile_sums);
  k_scan_top<<<1, 1024, 0, st>>>(tile_sums, nt, d_total);
  k_scan_apply<<<nt, SC_BLOCK, 0, st>>>(in, out, n_host, d_n, tile_sums);
  RTR_LAUNCHED(3);
}

}  // namespace rtr
