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
//
// Sorted points carry their original index in the w lane (as int bits), so one
// 16-byte load gives both the coordinates and the tie-break key.
#pragma once
#include <limits.h>

#include "grid.cuh"

struct GridView {
  float ox, oy, oz, h, inv_h;
  int nx, ny, nz;
  const float4* __restrict__ pts;
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
  v.cells = g.cells;
  return v;
}

__device__ __forceinline__ int pt_index(float4 p) { return __float_as_int(p.w); }

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
// +inf when the ring box already covers the whole grid.
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

// Distance from q to the box spanned by the whole grid.
__device__ __forceinline__ float grid_box_dist(const GridView& g, float4 q) {
  const float hx = g.ox + (float)g.nx * g.h, hy = g.oy + (float)g.ny * g.h, hz = g.oz + (float)g.nz * g.h;
  const float dx = fmaxf(fmaxf(g.ox - q.x, q.x - hx), 0.f);
  const float dy = fmaxf(fmaxf(g.oy - q.y, q.y - hy), 0.f);
  const float dz = fmaxf(fmaxf(g.oz - q.z, q.z - hz), 0.f);
  return sqrtf(dx * dx + dy * dy + dz * dz);
}

__device__ __forceinline__ bool ring_covers(const GridView& g, int cx, int cy, int cz, int k) {
  return cx - k <= 0 && cx + k >= g.nx - 1 && cy - k <= 0 && cy + k >= g.ny - 1 && cz - k <= 0 &&
         cz + k >= g.nz - 1;
}

// Visits every in-grid cell at Chebyshev distance exactly k from (cx, cy, cz):
// rows on a z or y face of the ring are walked in full, the others only at
// x = cx - k and x = cx + k.  The body sees the cell as (x, y, z).
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

__device__ __forceinline__ void nn_take(float4 p, unsigned j, float4 q, float& bd, int& bi, int& bpos) {
  const float d2 = dist2_exact(q, p);
  const int id = pt_index(p);
  // a candidate at infinite (or NaN) d^2 is never a neighbour: points with a
  // non-finite coordinate never match
  if (d2 < bd || (d2 == bd && id < bi && d2 < __int_as_float(0x7f800000))) {
    bd = d2;
    bi = id;
    bpos = (int)j;
  }
}

// Exact 1-NN with d^2 <= r2max (r2max = +inf: unbounded), one thread per
// query.  Returns the original index (or -1) and the sorted position.
__device__ __forceinline__ void grid_nn1(const GridView& g, float4 q, float r2max, float& bd, int& bi,
                                         int& bpos) {
  bd = r2max;
  bi = INT_MAX;
  bpos = -1;
  const int cx = q_cell(q.x, g.ox, g.inv_h), cy = q_cell(q.y, g.oy, g.inv_h),
            cz = q_cell(q.z, g.oz, g.inv_h);
  // nothing of the grid within the bound: done before walking any ring
  if (beyond(grid_box_dist(g, q), search_margin(g, q, 0), r2max)) {
    bi = -1;
    bd = __int_as_float(0x7f800000);
    return;
  }
  for (int k = first_ring(g, cx, cy, cz);; ++k) {
    const float margin = search_margin(g, q, k);
    RTR_FOR_RING(g, cx, cy, cz, k, {
      const uint2 c = g.cells[((unsigned)z * (unsigned)g.ny + (unsigned)y) * (unsigned)g.nx + (unsigned)x];
      if (c.x < c.y && !beyond(cell_box_dist(g, q, x, y, z), margin, bd))
        for (unsigned j = c.x; j < c.y; ++j) nn_take(g.pts[j], j, q, bd, bi, bpos);
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

// Group reduction of (bd, bi, bpos) over the G lanes in gmask.
template <int G>
__device__ __forceinline__ void group_best(unsigned gmask, float& bd, int& bi, int& bpos) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    const float od = __shfl_xor_sync(gmask, bd, o);
    const int oi = __shfl_xor_sync(gmask, bi, o);
    const int op = __shfl_xor_sync(gmask, bpos, o);
    if (od < bd || (od == bd && oi < bi)) {
      bd = od;
      bi = oi;
      bpos = op;
    }
  }
}

// Same search with G lanes per query (G a power of two <= 32; the lanes of a
// group are contiguous and aligned).  A ring is walked as the (2k+1)^3 cube in
// chunks of 4G entries: each lane fetches four cell entries at once (interior
// and out-of-grid entries are dropped), the group ballots the surviving
// candidate cells and then scans each one's points with all G lanes.  After
// every ring the group agrees on the best (d^2, index), so the ring loop is
// uniform inside the group.  A lane skips a cell only when the cell is beyond
// its own best, which is never better than the group's.
// CP (cell-parallel): each lane scans its own candidate cells of a chunk,
// with the first two points of all four issued as independent loads, instead
// of the group scanning one candidate cell after another.  Same result.
template <int G, bool CP = false>
__device__ __forceinline__ void grid_nn1_group(const GridView& g, float4 q, float r2max, int lg,
                                               unsigned gmask, float& bd, int& bi, int& bpos) {
  bd = r2max;
  bi = INT_MAX;
  bpos = -1;
  const int cx = q_cell(q.x, g.ox, g.inv_h), cy = q_cell(q.y, g.oy, g.inv_h),
            cz = q_cell(q.z, g.oz, g.inv_h);
  const int gbase = (threadIdx.x & 31) & ~(G - 1);
  // nothing of the grid within the bound (uniform inside the group)
  if (beyond(grid_box_dist(g, q), search_margin(g, q, 0), r2max)) {
    bi = -1;
    bd = __int_as_float(0x7f800000);
    return;
  }
  for (int k = first_ring(g, cx, cy, cz);; ++k) {
    const float margin = search_margin(g, q, k);
    // the ring's cube clamped to the grid
    const int x0 = max(cx - k, 0), y0 = max(cy - k, 0), z0 = max(cz - k, 0);
    const int ex = min(cx + k, g.nx - 1) - x0 + 1, ey = min(cy + k, g.ny - 1) - y0 + 1,
              ez = min(cz + k, g.nz - 1) - z0 + 1;
    const int vol = (ex > 0 && ey > 0 && ez > 0) ? ex * ey * ez : 0;
    if (vol <= 512) {
      for (int m0 = 0; m0 < vol; m0 += 4 * G) {
        uint2 cc[4];
        bool cand[4];
#pragma unroll
        for (int s = 0; s < 4; ++s) {
          const int m = m0 + s * G + lg;
          cand[s] = false;
          cc[s] = make_uint2(0u, 0u);
          if (m < vol) {
            const int x = x0 + m % ex, y = y0 + (m / ex) % ey, z = z0 + m / (ex * ey);
            // the cell's box first: a cell beyond the current best is not fetched
            if (max(max(abs(x - cx), abs(y - cy)), abs(z - cz)) == k &&
                !beyond(cell_box_dist(g, q, x, y, z), margin, bd)) {
              cc[s] = g.cells[((unsigned)z * (unsigned)g.ny + (unsigned)y) * (unsigned)g.nx + (unsigned)x];
              cand[s] = cc[s].x < cc[s].y;
            }
          }
        }
        if (CP) {
          float4 p0[4], p1[4];
#pragma unroll
          for (int s = 0; s < 4; ++s) {
            const unsigned a = cc[s].x, e = cc[s].y;
            p0[s] = (cand[s] && a < e) ? g.pts[a] : q;
            p1[s] = (cand[s] && a + 1 < e) ? g.pts[a + 1] : q;
          }
#pragma unroll
          for (int s = 0; s < 4; ++s) {
            if (!cand[s]) continue;
            const unsigned a = cc[s].x, e = cc[s].y;
            if (a < e) nn_take(p0[s], a, q, bd, bi, bpos);
            if (a + 1 < e) nn_take(p1[s], a + 1, q, bd, bi, bpos);
            for (unsigned j = a + 2; j < e; ++j) nn_take(g.pts[j], j, q, bd, bi, bpos);
          }
        } else {
#pragma unroll
          for (int s = 0; s < 4; ++s) {
            unsigned bal = __ballot_sync(gmask, cand[s]) >> gbase;
            while (bal) {
              const int src = __ffs(bal) - 1;
              bal &= bal - 1;
              const unsigned b0 = __shfl_sync(gmask, cc[s].x, gbase + src);
              const unsigned b1 = __shfl_sync(gmask, cc[s].y, gbase + src);
              for (unsigned j = b0 + (unsigned)lg; j < b1; j += G) nn_take(g.pts[j], j, q, bd, bi, bpos);
            }
          }
        }
      }
    } else {
      // large rings: walk only the shell, all lanes on the same cell
      RTR_FOR_RING(g, cx, cy, cz, k, {
        const uint2 c = g.cells[((unsigned)z * (unsigned)g.ny + (unsigned)y) * (unsigned)g.nx + (unsigned)x];
        if (c.x < c.y && !beyond(cell_box_dist(g, q, x, y, z), margin, bd))
          for (unsigned j = c.x + (unsigned)lg; j < c.y; j += G) nn_take(g.pts[j], j, q, bd, bi, bpos);
      })
    }
    group_best<G>(gmask, bd, bi, bpos);
    if (ring_covers(g, cx, cy, cz, k)) break;
    if (beyond(ring_bound(g, q, cx, cy, cz, k), margin, bd)) break;
  }
  if (bi == INT_MAX) {
    bi = -1;
    bpos = -1;
    bd = __int_as_float(0x7f800000);
  }
}

// True when every point within sqrt(r2max) of any query lies in the 3x3x3
// cells around the query's cell: the cell edge exceeds the radius by 1 % and
// the grid is small enough (<= 4096 cells per axis) that the rounding of a
// cell index stays far below that slack.
__device__ __forceinline__ bool grid_near27_ok(const GridView& g, float r2max) {
  const float r = sqrtf(r2max);
  return r2max >= 0.f && isfinite(r) && g.h >= 1.01f * r && g.nx <= 4096 && g.ny <= 4096 && g.nz <= 4096;
}

// Offsets (-1, 0, +1 as bits 0, 1, 2) along one axis that stay in the grid
// (0 <= c + d < n) and, for d != 0, whose face lies within reach (squared
// face distance <= thr2).
__device__ __forceinline__ unsigned near_axis_mask(int c, int n, float fm2, float fp2, float thr2) {
  unsigned m = 0u;
  if (c - 1 >= 0 && c - 1 < n && !(fm2 > thr2)) m |= 1u;
  if (c >= 0 && c < n) m |= 2u;
  if (c + 1 >= 0 && c + 1 < n && !(fp2 > thr2)) m |= 4u;
  return m;
}
// Offset of the k-th set bit (k < popc(m)) of a 3-bit axis mask.
__device__ __forceinline__ int near_axis_pick(unsigned m, int k) {
  const int b0 = (int)(m & 1u), b1 = (int)((m >> 1) & 1u);
  return k < b0 ? -1 : (k < b0 + b1 ? 0 : 1);
}

// The query's position relative to its cell: squared distances to the six
// faces (clamped at 0; underestimates under rounding).
struct NearCell {
  int cx, cy, cz;
  float xm2, xp2, ym2, yp2, zm2, zp2;
};
__device__ __forceinline__ NearCell near_cell(const GridView& g, float4 q) {
  NearCell c;
  c.cx = q_cell(q.x, g.ox, g.inv_h);
  c.cy = q_cell(q.y, g.oy, g.inv_h);
  c.cz = q_cell(q.z, g.oz, g.inv_h);
  const float xl = g.ox + (float)c.cx * g.h, yl = g.oy + (float)c.cy * g.h, zl = g.oz + (float)c.cz * g.h;
  const float fxm = fmaxf(q.x - xl, 0.f), fxp = fmaxf(xl + g.h - q.x, 0.f);
  const float fym = fmaxf(q.y - yl, 0.f), fyp = fmaxf(yl + g.h - q.y, 0.f);
  const float fzm = fmaxf(q.z - zl, 0.f), fzp = fmaxf(zl + g.h - q.z, 0.f);
  c.xm2 = fxm * fxm;
  c.xp2 = fxp * fxp;
  c.ym2 = fym * fym;
  c.yp2 = fyp * fyp;
  c.zm2 = fzm * fzm;
  c.zp2 = fzp * fzp;
  return c;
}

// The neighbour cells a query must visit: every (dx, dy, dz) != 0 from the
// per-axis masks whose box is within reach; entry k (k = lg, lg + G, ...) of
// that list for lane lg.  thr2 must be the same in every lane of the group
// (the lists then agree).  Calls body(x, y, z) for each of the lane's cells.
template <int G, typename F>
__device__ __forceinline__ void near_neighbours(const GridView& g, const NearCell& c, float thr2, int lg, F body) {
  const unsigned mx = near_axis_mask(c.cx, g.nx, c.xm2, c.xp2, thr2);
  const unsigned my = near_axis_mask(c.cy, g.ny, c.ym2, c.yp2, thr2);
  const unsigned mz = near_axis_mask(c.cz, g.nz, c.zm2, c.zp2, thr2);
  const int nxo = __popc(mx), nyo = __popc(my), nzo = __popc(mz);
  const int total = nxo * nyo * nzo;
  for (int k = lg; k < total; k += G) {
    const int ix = k % nxo, iy = (k / nxo) % nyo, iz = k / (nxo * nyo);
    const int dx = near_axis_pick(mx, ix), dy = near_axis_pick(my, iy), dz = near_axis_pick(mz, iz);
    if ((dx | dy | dz) == 0) continue;  // the own cell
    const float b2 = (dx < 0 ? c.xm2 : (dx > 0 ? c.xp2 : 0.f)) + (dy < 0 ? c.ym2 : (dy > 0 ? c.yp2 : 0.f)) +
                     (dz < 0 ? c.zm2 : (dz > 0 ? c.zp2 : 0.f));
    if (b2 > thr2) continue;  // an edge or corner cell beyond reach
    body(c.cx + dx, c.cy + dy, c.cz + dz);
  }
}

// Exact 1-NN with d^2 <= r2max over the 27 cells around the query's cell
// (precondition: grid_near27_ok), G lanes per query as grid_nn1_group; same
// result.  The query's own cell is scanned first and the group agrees on its
// best; then only the neighbours whose box, measured through the query's
// distances to its own cell's faces (an underestimate), is within that best
// plus the rounding margin are fetched, spread over the group.  No ring
// bookkeeping and no square root per cell.
template <int G>
__device__ __forceinline__ void grid_nn1_near(const GridView& g, float4 q, float r2max, int lg, unsigned gmask,
                                              float& bd, int& bi, int& bpos) {
  bd = r2max;
  bi = INT_MAX;
  bpos = -1;
  const NearCell c = near_cell(g, q);
  if (c.cx >= 0 && c.cx < g.nx && c.cy >= 0 && c.cy < g.ny && c.cz >= 0 && c.cz < g.nz) {
    const uint2 e = g.cells[((unsigned)c.cz * (unsigned)g.ny + (unsigned)c.cy) * (unsigned)g.nx + (unsigned)c.cx];
    for (unsigned j = e.x + (unsigned)lg; j < e.y; j += G) nn_take(g.pts[j], j, q, bd, bi, bpos);
  }
  group_best<G>(gmask, bd, bi, bpos);
  const float t = search_margin(g, q, 1) + sqrtf(bd * 1.000001f + 1e-30f);
  const float thr2 = t * t * 1.00001f;
  near_neighbours<G>(g, c, thr2, lg, [&](int x, int y, int z) {
    const uint2 e = g.cells[((unsigned)z * (unsigned)g.ny + (unsigned)y) * (unsigned)g.nx + (unsigned)x];
    for (unsigned j = e.x; j < e.y; ++j) nn_take(g.pts[j], j, q, bd, bi, bpos);
  });
  group_best<G>(gmask, bd, bi, bpos);
  if (bi == INT_MAX) {
    bi = -1;
    bpos = -1;
    bd = __int_as_float(0x7f800000);
  }
}

// Whether any point lies within sqrt(r2) of q (d^2 <= r2, finite), over the
// 27 cells around q's cell (precondition: grid_near27_ok(g, r2)), G lanes
// per query; the same answer as grid_nn1_group finding a neighbour.  The own
// cell first, then the neighbours within reach; every lane stops once the
// group has found one.
template <int G>
__device__ __forceinline__ bool grid_any_near(const GridView& g, float4 q, float r2, int lg, unsigned gmask) {
  const NearCell c = near_cell(g, q);
  bool found = false;
  if (c.cx >= 0 && c.cx < g.nx && c.cy >= 0 && c.cy < g.ny && c.cz >= 0 && c.cz < g.nz) {
    const uint2 e = g.cells[((unsigned)c.cz * (unsigned)g.ny + (unsigned)c.cy) * (unsigned)g.nx + (unsigned)c.cx];
    for (unsigned j = e.x + (unsigned)lg; j < e.y && !found; j += G) found = dist2_exact(q, g.pts[j]) <= r2;
  }
  if (__any_sync(gmask, found)) return true;
  const float t = search_margin(g, q, 1) + sqrtf(r2 * 1.000001f + 1e-30f);
  const float thr2 = t * t * 1.00001f;
  near_neighbours<G>(g, c, thr2, lg, [&](int x, int y, int z) {
    if (found) return;
    const uint2 e = g.cells[((unsigned)z * (unsigned)g.ny + (unsigned)y) * (unsigned)g.nx + (unsigned)x];
    for (unsigned j = e.x; j < e.y && !found; ++j) found = dist2_exact(q, g.pts[j]) <= r2;
  });
  return __any_sync(gmask, found);
}

// Exact K-NN (K compile-time), sorted by (d^2, index).  The K nearest by that
// order are unique, so any k <= K of them form the exact k-NN.
template <int K>
__device__ __forceinline__ void knn_insert(float (&bd)[K], int (&bi)[K], float d2, int id) {
  // NaN and infinite d^2 never enter the list
  if (!(d2 < bd[K - 1]) && !(d2 == bd[K - 1] && id < bi[K - 1] && d2 < __int_as_float(0x7f800000))) return;
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
          const float4 p = g.pts[j];
          knn_insert<K>(bd, bi, dist2_exact(q, p), pt_index(p));
        }
      }
    })
    if (ring_covers(g, cx, cy, cz, k)) break;
    if (beyond(ring_bound(g, q, cx, cy, cz, k), margin, bd[K - 1])) break;
  }
}
