// grid.cuh — radix-sorted uniform grid (build on device, exact searches).
//
// A grid over n points with cell edge h: points are sorted by the linear index
// of their cell (x fastest) with a stable LSD radix sort, and a dense table
// gives each cell its [start, end) range in the sorted order.  Every size and
// every bound is computed on the device, so a build can sit inside a captured
// CUDA graph; capacities come from the host.
#pragma once
#include "common.cuh"

struct GridMeta {
  float ox, oy, oz;      // lower corner of cell (0,0,0)
  float h, inv_h;        // cell edge actually used (>= the requested edge)
  int nx, ny, nz;
  int n;                 // points in the grid
  unsigned ncells;       // nx*ny*nz
  unsigned bmin[3];      // bounding box as order-preserving unsigned
  unsigned bmax[3];
};

struct GridDev {
  const GridMeta* meta;  // device
  const float4* pts;     // points sorted by cell; w = original index (int bits)
  const int* idx;        // original index of each sorted point
  const uint2* cells;    // per cell {start, end}
};

namespace rtr {

struct GridBufs {
  GridMeta* meta;
  float4* pts;
  int* idx;
  uint2* cells;
  uint32_t *k0, *v0, *k1, *v1, *hist;
  int n_cap;
  unsigned cell_cap;
};

// Stable LSD radix sort of (key, value) pairs by the low `bits` bits of key.
// When vals_in is NULL the values are the element indices.  Ping-pongs
// between (k0,v0) and (k1,v1); *k_out/*v_out point at the sorted arrays.
int radix_hist_entries(int n_cap);
void radix_sort_pairs(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, uint32_t* hist,
                      int n_cap, int n_host, const int* d_n, int bits, bool vals_iota,
                      cudaStream_t st, uint32_t** k_out, uint32_t** v_out);

void grid_plan(ScratchPlan& plan, int n_cap, unsigned cell_cap);
bool grid_take(Scratch& s, int n_cap, unsigned cell_cap, GridBufs* b);
// Build the grid over pts[0..n) (n = *d_n when d_n != NULL).  h_req is the
// requested cell edge; if the bounding box needs more than cell_cap cells the
// edge grows until it fits (searches stay exact, only slower).
void grid_build(const GridBufs& b, const float4* pts, int n_host, const int* d_n, float h_req,
                cudaStream_t st);
// Bounding box only (fills m->bmin / m->bmax).
void bbox_build(GridMeta* m, const float4* pts, int n, cudaStream_t st);
// Same over the first *d_n (<= n_cap) points.
void bbox_build(GridMeta* m, const float4* pts, int n_cap, const int* d_n, cudaStream_t st);
inline GridDev grid_dev(const GridBufs& b) { return GridDev{b.meta, b.pts, b.idx, b.cells}; }
inline unsigned default_cell_cap(int n) {
  unsigned c = (unsigned)n * 8u;
  return c < (1u << 18) ? (1u << 18) : c;
}

}  // namespace rtr
