// search.cuh — exact grid searches (device functions).
//
// Ring search: cells are visited in rings of growing Chebyshev radius k around
// the query's cell.  After ring k every unvisited point lies outside the box of
// cells [c-k, c+k], so its distance is at least the distance lb from the query
// to that box's faces (faces on the grid boundary do not count: nothing lies
// beyond them).  The search stops once lb, shrunk by a rounding margin, is
// strictly larger than the current k-th best distance.  Cells whose box is
// farther than the current bound are skipped.  Candidates are compared as
// (d^2, original index), so ties go to the lowest index and the result does not
// depend on the visiting order.
#pragma once
#include <limits.h>

#include "grid.cuh"

struct GridView {
  float ox, oy, oz, h, inv_h;
  int nx, ny, nz;
  const float4* __restrict__ pts;
  const int* __restrict__ idx;
  const uint2* __restrict__ cells;
};

__device__ __forceinline__ GridView load_view(const GridDev& g) {
  GridView v;
  const GridMeta* m = g.meta;
  v.ox = m->ox;
  v.oy = m->oy;
  v.oz = m->oz;
  v.h = m->h;
  v.inv_h = m->inv_h;
  v.nx = m->nx;
  v.ny = m->ny;
  v.nz = m->nz;
  v.pts = g.pts;
  v.idx = g.idx;
  v.cells = g.cells;
  return v;
}

__device__ __forceinline__ int q_cell(float v, float o, float inv_h) {
  float f = __fmul_rn(__fsub_rn(v, o), inv_h);
  f = fminf(fmaxf(f, -1.0e8f), 1.0e8f);
  return (int)floorf(f);
}

// Conservative rounding margin (metres) for bounds near query q.
__device__ __forceinline__ float search_margin(const GridView& g, float4 q, int k) {
  float s = fmaxf(fmaxf(fabsf(q.x), fabsf(q.y)), fabsf(q.z));
  s = fmaxf(s, fmaxf(fmaxf(fabsf(g.ox), fabsf(g.oy)), fabsf(g.oz)));
  float ext = (float)(max(max(g.nx, g.ny), g.nz) + k + 2) * g.h;
  return 8.0e-6f * (1.0f + s + ext);
}

// True when every point at distance >= (lb - margin) has d^2 > bound.
__device__ __forceinline__ bool beyond(float lb, float margin, float bound) {
  float l = lb - margin;
  return l > 0.f && l * l > bound * 1.000001f + 1e-30f;
}

// Distance from q to the box of cell (x, y, z).
__device__ __forceinline__ float cell_box_dist(const GridView& g, float4 q, int x, int y, int z) {
  float lx = g.ox + (float)x * g.h, ly = g.oy + (float)y * g.h, lz = g.oz + (float)z * g.h;
  float dx = fmaxf(fmaxf(lx - q.x, q.x - (lx + g.h)), 0.f);
  float dy = fmaxf(fmaxf(ly - q.y, q.y - (ly + g.h)), 0.f);
  float dz = fmaxf(fmaxf(lz - q.z, q.z - (lz + g.h)), 0.f);
  return sqrtf(dx * dx + dy * dy + dz * dz);
}

// Lower bound on the distance to any point outside the ring box of radius k;
// returns +inf when the ring box already covers the whole grid.
__device__ __forceinline__ float ring_bound(const GridView& g, float4 q, int cx, int cy, int cz, int k) {
  float lb = __int_as_float(0x7f800000);
  if (cx - k > 0) lb = fminf(lb, q.x - (g.ox + (float)(cx - k) * g.h));
  if (cx + k < g.nx - 1) lb = fminf(lb, (g.ox + (float)(cx + k + 1) * g.h) - q.x);
  if (cy - k > 0) lb = fminf(lb, q.y - (g.oy + (float)(cy - k) * g.h));
  if (cy + k < g.ny - 1) lb = fminf(lb, (g.oy + (float)(cy + k + 1) * g.h) - q.y);
  if (cz - k > 0) lb = fminf(lb, q.z - (g.oz + (float)(cz - k) * g.h));
  if (cz + k < g.nz - 1) lb = fminf(lb, (g.oz + (float)(cz + k + 1) * g.h) - q.z);
  return lb;
}

__device__ __forceinline__ bool ring_covers(const GridView& g, int cx, int cy, int cz, int k) {
  return cx - k <= 0 && cx + k >= g.nx - 1 && cy - k <= 0 && cy + k >= g.ny - 1 && cz - k <= 0 &&
         cz + k >= g.nz - 1;
}

// Visits every in-grid cell at Chebyshev distance exactly k from (cx, cy, cz):
// rows on a z or y face of the ring are walked in full, the others only at
// x = cx - k and x = cx + k.  BODY sees the cell as (x, y, z).
#define RTR_FOR_RING(g, cx, cy, cz, k, ...)                                         \
  {                                                                                 \
    const int z0_ = max((cz) - (k), 0), z1_ = min((cz) + (k), (g).nz - 1);            \
    const int y0_ = max((cy) - (k), 0), y1_ = min((cy) + (k), (g).ny - 1);            \
    for (int z = z0_; z <= z1_; ++z) {                                              \
      const bool zedge_ = (z == (cz) - (k)) || (z == (cz) + (k));                   \
      for (int y = y0_; y <= y1_; ++y) {                                            \
        const bool edge_ = zedge_ || (y == (cy) - (k)) || (y == (cy) + (k));        \
        const int xs_ = edge_ ? max((cx) - (k), 0) : (cx) - (k);                     \
        const int xe_ = edge_ ? min((cx) + (k), (g).nx - 1) : (cx) + (k);            \
        const int st_ = edge_ ? 1 : 2 * (k);                                        \
        for (int x = xs_; x <= xe_; x += st_) {                                     \
          if (x < 0 || x >= (g).nx) continue;                                       \
          __VA_ARGS__                                                               \
        }                                                                           \
      }                                                                             \
    }                                                                               \
  }

__device__ __forceinline__ int first_ring(const GridView& g, int cx, int cy, int cz) {
  int k = 0;
  k = max(k, max(-cx, cx - (g.nx - 1)));
  k = max(k, max(-cy, cy - (g.ny - 1)));
  k = max(k, max(-cz, cz - (g.nz - 1)));
  return k;
}

// Exact 1-NN with d^2 <= r2max (r2max = +inf: unbounded).  Returns the
// original index (or -1) and the sorted position (for reading the point).
__device__ __forceinline__ void grid_nn1(const GridView& g, float4 q, float r2max, float& bd, int& bi,
                                         int& bpos) {
  bd = r2max;
  bi = INT_MAX;
  bpos = -1;
  const int cx = q_cell(q.x, g.ox, g.inv_h), cy = q_cell(q.y, g.oy, g.inv_h),
            cz = q_cell(q.z, g.oz, g.inv_h);
  for (int k = first_ring(g, cx, cy, cz);; ++k) {
    const float margin = search_margin(g, q, k);
    RTR_FOR_RING(g, cx, cy, cz, k, {
      const uint2 c = g.cells[((unsigned)z * (unsigned)g.ny + (unsigned)y) * (unsigned)g.nx + (unsigned)x];
      if (c.x < c.y && !beyond(cell_box_dist(g, q, x, y, z), margin, bd)) {
        for (unsigned j = c.x; j < c.y; ++j) {
          const float d2 = dist2_exact(q, g.pts[j]);
          if (d2 <= bd) {
            const int id = g.idx[j];
            if (d2 < bd || id < bi) {
              bd = d2;
              bi = id;
              bpos = (int)j;
            }
          }
        }
      }
    })
    if (ring_covers(g, cx, cy, cz, k)) break;
    if (beyond(ring_bound(g, q, cx, cy, cz, k), margin, bd)) break;
  }
  if (bi == INT_MAX) {
    bi = -1;
    bpos = -1;
    bd = __int_as_float(0x7f800000);
  }
}

// Exact K-NN (K compile-time), sorted by (d^2, index).  The K nearest by that
// order are unique, so any k <= K of them form the exact k-NN.
template <int K>
__device__ __forceinline__ void grid_knn(const GridView& g, float4 q, float (&bd)[K], int (&bi)[K]) {
#pragma unroll
  for (int s = 0; s < K; ++s) {
    bd[s] = __int_as_float(0x7f800000);
    bi[s] = INT_MAX;
  }
  const int cx = q_cell(q.x, g.ox, g.inv_h), cy = q_cell(q.y, g.oy, g.inv_h),
            cz = q_cell(q.z, g.oz, g.inv_h);
  for (int k = first_ring(g, cx, cy, cz);; ++k) {
    const float margin = search_margin(g, q, k);
    RTR_FOR_RING(g, cx, cy, cz, k, {
      const uint2 c = g.cells[((unsigned)z * (unsigned)g.ny + (unsigned)y) * (unsigned)g.nx + (unsigned)x];
      if (c.x < c.y && !beyond(cell_box_dist(g, q, x, y, z), margin, bd[K - 1])) {
        for (unsigned j = c.x; j < c.y; ++j) {
          const float d2 = dist2_exact(q, g.pts[j]);
          if (d2 > bd[K - 1]) continue;
          const int id = g.idx[j];
          if (d2 == bd[K - 1] && id >= bi[K - 1]) continue;
          bd[K - 1] = d2;
          bi[K - 1] = id;
#pragma unroll
          for (int s = K - 1; s > 0; --s) {
            const bool lt = bd[s] < bd[s - 1] || (bd[s] == bd[s - 1] && bi[s] < bi[s - 1]);
            const float da = bd[s], db = bd[s - 1];
            const int ia = bi[s], ib = bi[s - 1];
            bd[s] = lt ? db : da;
            bd[s - 1] = lt ? da : db;
            bi[s] = lt ? ib : ia;
            bi[s - 1] = lt ? ia : ib;
          }
        }
      }
    })
    if (ring_covers(g, cx, cy, cz, k)) break;
    if (beyond(ring_bound(g, q, cx, cy, cz, k), margin, bd[K - 1])) break;
  }
}
