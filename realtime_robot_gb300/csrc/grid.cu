// grid.cu — stable LSD radix sort and the uniform-grid build.
#include <math.h>

#include "grid.cuh"

namespace rtr {

constexpr int RS_BLOCK = 256;
constexpr int RS_WARPS = RS_BLOCK / 32;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_BLOCK * RS_ITEMS;  // 4096 keys per block
constexpr int RS_RADIX = 256;

__device__ __forceinline__ int count_of(int n_host, const int* d_n) { return d_n ? *d_n : n_host; }

// Sorts of at most this many tiles skip the scan kernel: each scatter block
// sums the tile-major histogram itself (nb rows of 1 KB from L2).
constexpr int RS_FUSE_TILES = 128;

// Per-tile digit histogram, written digit-major, hist[d * nb + tile], or
// tile-major, hist[tile * 256 + d] (TILE_MAJOR, read by k_rs_scatter_own).
template <bool TILE_MAJOR>
__global__ void __launch_bounds__(RS_BLOCK) k_rs_hist(const uint32_t* __restrict__ keys, int n_host,
                                                      const int* d_n, int shift,
                                                      uint32_t* __restrict__ hist, int nb) {
  __shared__ uint32_t cnt[RS_RADIX];
  const int n = count_of(n_host, d_n);
  for (int i = threadIdx.x; i < RS_RADIX; i += RS_BLOCK) cnt[i] = 0;
  __syncthreads();
  const int base = blockIdx.x * RS_TILE;
#pragma unroll 4
  for (int j = 0; j < RS_ITEMS; ++j) {
    int i = base + j * RS_BLOCK + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & (RS_RADIX - 1)], 1u);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RS_RADIX; d += RS_BLOCK)
    hist[TILE_MAJOR ? blockIdx.x * RS_RADIX + d : d * nb + blockIdx.x] = cnt[d];
}

// In-place exclusive scan of `total` entries by one block of 1024 threads,
// in chunks of 8192 entries staged through shared memory with coalesced
// loads and stores (eight per thread), a carry between chunks.
__global__ void __launch_bounds__(1024) k_rs_scan(uint32_t* __restrict__ h, int total) {
  constexpr int PER = 8, CH = 1024 * PER;
  __shared__ uint32_t sh[CH];
  __shared__ uint32_t wsum[32];
  __shared__ uint32_t s_carry;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_carry = 0;
  for (int c0 = 0; c0 < total; c0 += CH) {
    const int cn = min(CH, total - c0);
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int i = k * 1024 + threadIdx.x;
      sh[i] = i < cn ? h[c0 + i] : 0u;
    }
    __syncthreads();
    // thread t owns sh[t*PER .. t*PER+PER)
    uint32_t v[PER], s = 0;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      v[k] = sh[threadIdx.x * PER + k];
      s += v[k];
    }
    uint32_t incl = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    if (warp == 0) {
      const uint32_t w = wsum[lane];
      uint32_t wi = w;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
        if (lane >= o) wi += t;
      }
      wsum[lane] = wi - w;
    }
    __syncthreads();
    uint32_t run = s_carry + wsum[warp] + incl - s;
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      sh[threadIdx.x * PER + k] = run;
      run += v[k];
    }
    __syncthreads();
    if (threadIdx.x == 1023) s_carry = run;  // the last thread ends with the chunk's total
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const int i = k * 1024 + threadIdx.x;
      if (i < cn) h[c0 + i] = sh[i];
    }
    __syncthreads();
  }
}

// This block's output offset of each digit from the tile-major histogram:
// the keys of smaller digits in every tile plus those of the same digit in
// earlier tiles (thread d owns digit d; a block-wide exclusive scan of the
// digit totals).
__device__ __forceinline__ void rs_own_offsets(const uint32_t* __restrict__ hist, int nb, uint32_t* boff,
                                               uint32_t* wsum) {
  static_assert(RS_BLOCK == RS_RADIX, "one thread per digit");
  const int d = threadIdx.x, lane = d & 31, warp = d >> 5;
  const int b = blockIdx.x;
  uint32_t tot = 0, pre = 0;
  int t = 0;
  for (; t + 4 <= nb; t += 4) {
    const uint32_t a0 = hist[(t + 0) * RS_RADIX + d], a1 = hist[(t + 1) * RS_RADIX + d];
    const uint32_t a2 = hist[(t + 2) * RS_RADIX + d], a3 = hist[(t + 3) * RS_RADIX + d];
    tot += a0 + a1 + a2 + a3;
    pre += (t + 0 < b ? a0 : 0u) + (t + 1 < b ? a1 : 0u) + (t + 2 < b ? a2 : 0u) + (t + 3 < b ? a3 : 0u);
  }
  for (; t < nb; ++t) {
    const uint32_t a0 = hist[t * RS_RADIX + d];
    tot += a0;
    pre += t < b ? a0 : 0u;
  }
  uint32_t inc = tot;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += v;
  }
  if (lane == 31) wsum[warp] = inc;
  __syncthreads();
  uint32_t wpre = 0;
#pragma unroll
  for (int w = 0; w < RS_WARPS; ++w) wpre += w < warp ? wsum[w] : 0u;
  boff[d] = wpre + inc - tot + pre;
}

// Stable scatter.  Warp w of a block owns a contiguous run of RS_ITEMS*32 keys
// and walks it 32 at a time, so (warp, step, lane) is the input order; ranks
// inside a step come from __match_any_sync, so equal digits keep their order.
// OWN: the block computes its offsets from the tile-major histogram
// (rs_own_offsets); otherwise it reads them from the scanned digit-major one.
template <bool OWN>
__global__ void __launch_bounds__(RS_BLOCK) k_rs_scatter(const uint32_t* __restrict__ kin,
                                                         const uint32_t* __restrict__ vin,
                                                         uint32_t* __restrict__ kout,
                                                         uint32_t* __restrict__ vout, int n_host,
                                                         const int* d_n, int shift,
                                                         const uint32_t* __restrict__ hist, int nb) {
  __shared__ uint32_t wcnt[RS_WARPS][RS_RADIX];
  __shared__ uint32_t boff[RS_RADIX];
  __shared__ uint32_t wsum[RS_WARPS];
  const int n = count_of(n_host, d_n);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < RS_WARPS * RS_RADIX; i += RS_BLOCK) (&wcnt[0][0])[i] = 0;
  if (OWN) {
    if (blockIdx.x * RS_TILE >= n) return;  // whole tile empty (uniform per block)
    rs_own_offsets(hist, nb, boff, wsum);
  } else {
    for (int d = threadIdx.x; d < RS_RADIX; d += RS_BLOCK) boff[d] = hist[d * nb + blockIdx.x];
  }
  __syncthreads();
  const int base = blockIdx.x * RS_TILE + warp * (RS_ITEMS * 32);
  if (blockIdx.x * RS_TILE >= n) return;  // whole tile empty (uniform per block)
  const unsigned lt = lanemask_lt();
  uint32_t key[RS_ITEMS];
  uint32_t loc[RS_ITEMS];
#pragma unroll
  for (int j = 0; j < RS_ITEMS; ++j) {
    const int i = base + j * 32 + lane;
    const bool valid = i < n;
    const uint32_t k = valid ? kin[i] : 0u;
    key[j] = k;
    const uint32_t d = valid ? ((k >> shift) & (RS_RADIX - 1)) : RS_RADIX;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    uint32_t before = valid ? wcnt[warp][d] : 0u;
    __syncwarp();
    if (valid && (peers & lt) == 0) wcnt[warp][d] = before + __popc(peers);
    __syncwarp();
    loc[j] = before + __popc(peers & lt);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < RS_RADIX; d += RS_BLOCK) {
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; ++w) {
      uint32_t t = wcnt[w][d];
      wcnt[w][d] = run;
      run += t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < RS_ITEMS; ++j) {
    const int i = base + j * 32 + lane;
    if (i < n) {
      const uint32_t d = (key[j] >> shift) & (RS_RADIX - 1);
      const uint32_t pos = boff[d] + wcnt[warp][d] + loc[j];
      kout[pos] = key[j];
      vout[pos] = vin ? vin[i] : (uint32_t)i;
    }
  }
}

int radix_hist_entries(int n_cap) {
  int nb = (n_cap + RS_TILE - 1) / RS_TILE;
  if (nb < 1) nb = 1;
  return nb * RS_RADIX;
}

void radix_sort_pairs(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, uint32_t* hist,
                      int n_cap, int n_host, const int* d_n, int bits, bool vals_iota,
                      cudaStream_t st, uint32_t** k_out, uint32_t** v_out) {
  int nb = (n_cap + RS_TILE - 1) / RS_TILE;
  if (nb < 1) nb = 1;
  int passes = (bits + 7) / 8;
  if (passes < 1) passes = 1;
  for (int p = 0; p < passes; ++p) {
    const int shift = 8 * p;
    const bool even = (p & 1) == 0;
    uint32_t* ki = even ? k0 : k1;
    uint32_t* vi = even ? ((p == 0 && vals_iota) ? nullptr : v0) : v1;
    uint32_t* ko = even ? k1 : k0;
    uint32_t* vo = even ? v1 : v0;
    if (nb <= RS_FUSE_TILES) {
      k_rs_hist<true><<<nb, RS_BLOCK, 0, st>>>(ki, n_host, d_n, shift, hist, nb);
      k_rs_scatter<true><<<nb, RS_BLOCK, 0, st>>>(ki, vi, ko, vo, n_host, d_n, shift, hist, nb);
    } else {
      k_rs_hist<false><<<nb, RS_BLOCK, 0, st>>>(ki, n_host, d_n, shift, hist, nb);
      k_rs_scan<<<1, 1024, 0, st>>>(hist, nb * RS_RADIX);
      k_rs_scatter<false><<<nb, RS_BLOCK, 0, st>>>(ki, vi, ko, vo, n_host, d_n, shift, hist, nb);
    }
  }
  RTR_LAUNCHED((nb <= RS_FUSE_TILES ? 2 : 3) * passes);
  const bool odd = (passes & 1) != 0;
  *k_out = odd ? k1 : k0;
  *v_out = odd ? v1 : v0;
}

// ---------------------------------------------------------------------------
// grid build
// ---------------------------------------------------------------------------

__global__ void k_bbox_init(GridMeta* m) {
  if (threadIdx.x < 3) {
    m->bmin[threadIdx.x] = 0xffffffffu;
    m->bmax[threadIdx.x] = 0u;
  }
}

// Launched with 256 threads and at most bbox_blocks(n) blocks.
__global__ void __launch_bounds__(256) k_bbox(const float4* __restrict__ pts, int n_host,
                                              const int* d_n, GridMeta* m) {
  const int n = count_of(n_host, d_n);
  unsigned mn[3] = {0xffffffffu, 0xffffffffu, 0xffffffffu}, mx[3] = {0u, 0u, 0u};
#pragma unroll 4
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float4 p = pts[i];
    // a point with a non-finite coordinate does not size the grid: it sits in
    // a clamped border cell and never matches (its d^2 is NaN or inf)
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) continue;
    unsigned u[3] = {float_to_ordered(p.x), float_to_ordered(p.y), float_to_ordered(p.z)};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      mn[a] = min(mn[a], u[a]);
      mx[a] = max(mx[a], u[a]);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mn[a] = min(mn[a], __shfl_xor_sync(0xffffffffu, mn[a], o));
      mx[a] = max(mx[a], __shfl_xor_sync(0xffffffffu, mx[a], o));
    }
  }
  // the block's extremes, then six atomics per block (atomics from every
  // warp on the same six words serialise: 39 us for 1216 blocks)
  __shared__ unsigned s_mn[3][8], s_mx[3][8];
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      s_mn[a][warp] = mn[a];
      s_mx[a][warp] = mx[a];
    }
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    const int a = threadIdx.x;
    unsigned lo = s_mn[a][0], hi = s_mx[a][0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      lo = min(lo, s_mn[a][w]);
      hi = max(hi, s_mx[a][w]);
    }
    atomicMin(&m->bmin[a], lo);
    atomicMax(&m->bmax[a], hi);
  }
}

__global__ void k_grid_setup(GridMeta* m, float h_req, unsigned cell_cap, int n_host,
                             const int* d_n) {
  const int n = count_of(n_host, d_n);
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    if (n > 0) {
      lo[a] = ordered_to_float(m->bmin[a]);
      hi[a] = ordered_to_float(m->bmax[a]);
    } else {
      lo[a] = hi[a] = 0.f;
    }
    // non-finite coordinates (NaN / inf points) must not size the grid: such
    // points land in a clamped border cell and never match (d^2 is NaN/inf)
    if (!isfinite(lo[a]) || !isfinite(hi[a]) || !(hi[a] >= lo[a])) {
      lo[a] = isfinite(lo[a]) ? lo[a] : (isfinite(hi[a]) ? hi[a] : 0.f);
      hi[a] = isfinite(hi[a]) && hi[a] >= lo[a] ? hi[a] : lo[a];
    }
  }
  float h = h_req;
  if (!(h > 0.f)) {
    // automatic edge: twice the mean spacing of n points spread over the box
    double vol = 1.0;
    for (int a = 0; a < 3; ++a) vol *= fmax((double)(hi[a] - lo[a]), 1e-3);
    h = (float)(2.0 * cbrt(vol / (double)(n > 0 ? n : 1)));
  }
  int dims[3];
  for (int tries = 0; tries < 64; ++tries) {
    double cells = 1.0;
    for (int a = 0; a < 3; ++a) {
      double e = floor((double)(hi[a] - lo[a]) / (double)h) + 1.0;
      if (e > 2.0e9) e = 2.0e9;
      dims[a] = (int)e;
      cells *= e;
    }
    if (cells <= (double)cell_cap) break;
    h = (float)(h * cbrt(cells / (double)cell_cap) * 1.001);
  }
  m->ox = lo[0];
  m->oy = lo[1];
  m->oz = lo[2];
  m->h = h;
  m->inv_h = 1.0f / h;
  m->nx = dims[0];
  m->ny = dims[1];
  m->nz = dims[2];
  m->n = n;
  m->ncells = (unsigned)dims[0] * (unsigned)dims[1] * (unsigned)dims[2];
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__device__ __forceinline__ int cell_of(float v, float o, float inv_h) {
  float f = __fmul_rn(__fsub_rn(v, o), inv_h);
  f = fminf(fmaxf(f, -1.0e8f), 1.0e8f);
  return (int)floorf(f);
}

__global__ void __launch_bounds__(256) k_grid_keys(const float4* __restrict__ pts, int n_host,
                                                   const int* d_n, const GridMeta* __restrict__ m,
                                                   uint32_t* __restrict__ keys) {
  const int n = count_of(n_host, d_n);
  const float ox = m->ox, oy = m->oy, oz = m->oz, ih = m->inv_h;
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float4 p = pts[i];
    int cx = clampi(cell_of(p.x, ox, ih), 0, nx - 1);
    int cy = clampi(cell_of(p.y, oy, ih), 0, ny - 1);
    int cz = clampi(cell_of(p.z, oz, ih), 0, nz - 1);
    keys[i] = ((uint32_t)cz * (uint32_t)ny + (uint32_t)cy) * (uint32_t)nx + (uint32_t)cx;
  }
}

__global__ void __launch_bounds__(256) k_grid_gather(const float4* __restrict__ pts,
                                                     const uint32_t* __restrict__ order, int n_host,
                                                     const int* d_n, float4* __restrict__ out,
                                                     int* __restrict__ idx) {
  const int n = count_of(n_host, d_n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint32_t o = order[i];
    float4 p = pts[o];
    p.w = __int_as_float((int)o);  // original index travels with the point
    out[i] = p;
    idx[i] = (int)o;
  }
}

__global__ void __launch_bounds__(256) k_cells_clear(uint2* __restrict__ cells,
                                                     const GridMeta* __restrict__ m) {
  const unsigned nc = m->ncells;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < nc; i += gridDim.x * blockDim.x)
    cells[i] = make_uint2(0u, 0u);
}

__global__ void __launch_bounds__(256) k_cell_bounds(const uint32_t* __restrict__ sk, int n_host,
                                                     const int* d_n, uint2* __restrict__ cells) {
  const int n = count_of(n_host, d_n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint32_t k = sk[i];
    if (i == 0 || sk[i - 1] != k) cells[k].x = (unsigned)i;
    if (i == n - 1 || sk[i + 1] != k) cells[k].y = (unsigned)(i + 1);
  }
}

void grid_plan(ScratchPlan& plan, int n_cap, unsigned cell_cap) {
  int n = n_cap > 0 ? n_cap : 1;
  plan.add<GridMeta>(1);
  plan.add<float4>(n);
  plan.add<int>(n);
  plan.add<uint2>(cell_cap);
  for (int i = 0; i < 4; ++i) plan.add<uint32_t>(n);
  plan.add<uint32_t>(radix_hist_entries(n));
}

bool grid_take(Scratch& s, int n_cap, unsigned cell_cap, GridBufs* b) {
  int n = n_cap > 0 ? n_cap : 1;
  b->meta = s.take<GridMeta>(1);
  b->pts = s.take<float4>(n);
  b->idx = s.take<int>(n);
  b->cells = s.take<uint2>(cell_cap);
  b->k0 = s.take<uint32_t>(n);
  b->v0 = s.take<uint32_t>(n);
  b->k1 = s.take<uint32_t>(n);
  b->v1 = s.take<uint32_t>(n);
  b->hist = s.take<uint32_t>(radix_hist_entries(n));
  b->n_cap = n_cap;
  b->cell_cap = cell_cap;
  return b->meta && b->pts && b->idx && b->cells && b->k0 && b->v0 && b->k1 && b->v1 && b->hist;
}

static int grid_blocks(int n) {
  int b = (n + 255) / 256;
  if (b < 1) b = 1;
  if (b > 152 * 8) b = 152 * 8;
  return b;
}
// Blocks of a reduction to a few words: two per SM at most.
static int bbox_blocks(int n) {
  int b = (n + 255) / 256;
  if (b < 1) b = 1;
  if (b > 152 * 2) b = 152 * 2;
  return b;
}

void bbox_build(GridMeta* m, const float4* pts, int n, cudaStream_t st) { bbox_build(m, pts, n, nullptr, st); }

void bbox_build(GridMeta* m, const float4* pts, int n_cap, const int* d_n, cudaStream_t st) {
  k_bbox_init<<<1, 32, 0, st>>>(m);
  k_bbox<<<bbox_blocks(n_cap), 256, 0, st>>>(pts, n_cap, d_n, m);
  RTR_LAUNCHED(2);
}

void grid_build(const GridBufs& b, const float4* pts, int n_host, const int* d_n, float h_req,
                cudaStream_t st) {
  const int nb = grid_blocks(b.n_cap);
  k_bbox_init<<<1, 32, 0, st>>>(b.meta);
  k_bbox<<<bbox_blocks(b.n_cap), 256, 0, st>>>(pts, n_host, d_n, b.meta);
  k_grid_setup<<<1, 1, 0, st>>>(b.meta, h_req, b.cell_cap, n_host, d_n);
  k_grid_keys<<<nb, 256, 0, st>>>(pts, n_host, d_n, b.meta, b.k0);
  int bits = 1;
  while (bits < 32 && (1ull << bits) < (unsigned long long)b.cell_cap) ++bits;
  uint32_t *ks, *vs;
  radix_sort_pairs(b.k0, b.v0, b.k1, b.v1, b.hist, b.n_cap, n_host, d_n, bits, true, st, &ks, &vs);
  k_grid_gather<<<nb, 256, 0, st>>>(pts, vs, n_host, d_n, b.pts, b.idx);
  int cb = (int)((b.cell_cap + 255) / 256);
  if (cb > 152 * 16) cb = 152 * 16;
  k_cells_clear<<<cb, 256, 0, st>>>(b.cells, b.meta);
  k_cell_bounds<<<nb, 256, 0, st>>>(ks, n_host, d_n, b.cells);
  RTR_LAUNCHED(7);
}

}  // namespace rtr
