/*
 * harris.c — CPU restatement of the reference's keypoint detector (test
 * infrastructure: the checker of the GPU path, realtime_robot_gb300/csrc/
 * harris.cu).
 *
 *   ModelPoint::getKeypoint  model_point.h:99-156
 *   ScanPoint::getKeypoint   scan_point.h:57-113
 *   pcl::HarrisKeypoint3D, radius 0.05, threshold 0.01, non-maximum
 *   suppression on, refinement at its default (on)
 *
 * PCL 1.8.0 is absent, so parity with it is unpinned.  The detector is the
 * 3-D Harris operator on surface normals (Sipiran & Bustos 2011) with these
 * conventions, which the GPU path follows bit for bit:
 *
 *  - neighbours of a point: every point within the radius (squared distance
 *    ((dx*dx + dy*dy) + dz*dz) <= r*r in float), the point itself included,
 *    taken in ascending index order for every sum;
 *  - normal: smallest eigenvector (FP32 Jacobi, orc_eig3) of the FP32
 *    centred covariance of the neighbours (mean first, then the centred
 *    products, each sum in index order); its sign does not matter below;
 *  - M = (1/n) sum n_j n_j^T over the neighbours' normals (FP32, index
 *    order); response R = det(M) - k tr(M)^2 + k with k = 0.04.  For unit
 *    normals tr(M) = 1 and R = det(M): 0 on a face or an edge, up to 1/27 at
 *    a corner of three faces -- the normalisation under which the
 *    reference's threshold of 0.01 selects corners;
 *  - keypoint: R > threshold and R >= R_j of every neighbour j (ties keep
 *    both);
 *  - refinement: the position x moves to the least-squares intersection of
 *    the tangent planes of the points within r of x, argmin sum (n_j.(x -
 *    p_j))^2 (FP64 sums in index order, Cramer's rule), at most 10 times,
 *    while the system is well conditioned (det(A) > 1e-12 tr(A)^3) and the
 *    new position stays within r of the keypoint's point; it stops when it
 *    moves less than 1e-6 m.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

typedef struct {
  int* idx;
  int n, cap;
} hr_list;

static void hr_push(hr_list* L, int j) {
  if (L->n == L->cap) {
    L->cap = L->cap ? 2 * L->cap : 256;
    L->idx = (int*)realloc(L->idx, sizeof(int) * (size_t)L->cap);
  }
  L->idx[L->n++] = j;
}

static int hr_int_cmp(const void* a, const void* b) {
  const int x = *(const int*)a, y = *(const int*)b;
  return (x > y) - (x < y);
}

static float hr_d2(const float* q, const float* p) {
  const float dx = q[0] - p[0], dy = q[1] - p[1], dz = q[2] - p[2];
  const float xx = dx * dx, yy = dy * dy, zz = dz * dz;
  return (xx + yy) + zz;
}

/* the points within r of q, ascending index (brute force over the cells of
 * a uniform grid of edge r) */
typedef struct {
  float lo[3], inv;
  int n[3];
  int* start;
  int* order;
} hr_grid;

static int hr_cell(const hr_grid* g, float v, int a) {
  double f = floor(((double)v - (double)g->lo[a]) * (double)g->inv);
  if (!(f >= 0)) f = 0;
  if (f > g->n[a] - 1) f = g->n[a] - 1;
  return (int)f;
}

static void hr_grid_build(hr_grid* g, const float* pts, int n, float r) {
  float hi[3];
  for (int a = 0; a < 3; ++a) {
    g->lo[a] = n ? pts[a] : 0.f;
    hi[a] = g->lo[a];
  }
  for (int i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      if (pts[4 * i + a] < g->lo[a]) g->lo[a] = pts[4 * i + a];
      if (pts[4 * i + a] > hi[a]) hi[a] = pts[4 * i + a];
    }
  g->inv = 1.f / r;
  for (int a = 0; a < 3; ++a) {
    double e = floor(((double)hi[a] - g->lo[a]) * g->inv) + 1;
    g->n[a] = e > 4096 ? 4096 : (int)e;
  }
  const size_t nc = (size_t)g->n[0] * g->n[1] * g->n[2];
  g->start = (int*)calloc(nc + 1, sizeof(int));
  g->order = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  int* key = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  for (int i = 0; i < n; ++i) {
    const int c = (hr_cell(g, pts[4 * i + 2], 2) * g->n[1] + hr_cell(g, pts[4 * i + 1], 1)) * g->n[0] +
                  hr_cell(g, pts[4 * i], 0);
    key[i] = c;
    g->start[c + 1]++;
  }
  for (size_t c = 0; c < nc; ++c) g->start[c + 1] += g->start[c];
  int* fill = (int*)malloc(sizeof(int) * (nc + 1));
  memcpy(fill, g->start, sizeof(int) * (nc + 1));
  for (int i = 0; i < n; ++i) g->order[fill[key[i]]++] = i;
  free(fill);
  free(key);
}

static void hr_neighbours(const hr_grid* g, const float* pts, const float* q, float r2, hr_list* L) {
  L->n = 0;
  /* every cell that can hold a point within r: those of q -+ r (with a
   * margin) on each axis; the cell index is monotone in the coordinate */
  const double rr = (double)sqrtf(r2) * 1.0001 + 1e-6;
  int c0[3], c1[3];
  for (int a = 0; a < 3; ++a) {
    c0[a] = hr_cell(g, (float)((double)q[a] - rr), a);
    c1[a] = hr_cell(g, (float)((double)q[a] + rr), a);
  }
  for (int z = c0[2]; z <= c1[2]; ++z) {
    for (int y = c0[1]; y <= c1[1]; ++y) {
      for (int x = c0[0]; x <= c1[0]; ++x) {
        const int cell = (z * g->n[1] + y) * g->n[0] + x;
        for (int s = g->start[cell]; s < g->start[cell + 1]; ++s) {
          const int j = g->order[s];
          if (hr_d2(q, pts + 4 * (size_t)j) <= r2) hr_push(L, j);
        }
      }
    }
  }
  qsort(L->idx, (size_t)L->n, sizeof(int), hr_int_cmp);
}

static float hr_det3(const float* m) { /* m = {00, 01, 02, 11, 12, 22} */
  const float a = m[3] * m[5] - m[4] * m[4];
  const float b = m[1] * m[5] - m[4] * m[2];
  const float c = m[1] * m[4] - m[3] * m[2];
  return (m[0] * a - m[1] * b) + m[2] * c;
}

int orc_harris3d(const float* pts, int n, float r, float thr, int non_max, int refine, float* keys, int32_t* src) {
  const float r2 = r * r;
  hr_grid g;
  hr_grid_build(&g, pts, n, r);
  float* nrm = (float*)malloc(sizeof(float) * 3 * (size_t)(n > 0 ? n : 1));
  float* R = (float*)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
#pragma omp parallel
  {
    hr_list L = {NULL, 0, 0};
#pragma omp for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i) {
      hr_neighbours(&g, pts, pts + 4 * (size_t)i, r2, &L);
      float mx = 0.f, my = 0.f, mz = 0.f;
      for (int k = 0; k < L.n; ++k) {
        const float* p = pts + 4 * (size_t)L.idx[k];
        mx = mx + p[0];
        my = my + p[1];
        mz = mz + p[2];
      }
      const float cnt = (float)L.n;
      mx = mx / cnt;
      my = my / cnt;
      mz = mz / cnt;
      float C[6] = {0, 0, 0, 0, 0, 0};
      for (int k = 0; k < L.n; ++k) {
        const float* p = pts + 4 * (size_t)L.idx[k];
        const float dx = p[0] - mx, dy = p[1] - my, dz = p[2] - mz;
        C[0] = C[0] + dx * dx;
        C[1] = C[1] + dx * dy;
        C[2] = C[2] + dx * dz;
        C[3] = C[3] + dy * dy;
        C[4] = C[4] + dy * dz;
        C[5] = C[5] + dz * dz;
      }
      const float A[9] = {C[0], C[1], C[2], C[1], C[3], C[4], C[2], C[4], C[5]};
      float w[3], V[9];
      orc_eig3(A, w, V);
      nrm[3 * (size_t)i] = V[0];
      nrm[3 * (size_t)i + 1] = V[3];
      nrm[3 * (size_t)i + 2] = V[6];
    }
#pragma omp for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i) {
      hr_neighbours(&g, pts, pts + 4 * (size_t)i, r2, &L);
      float M[6] = {0, 0, 0, 0, 0, 0};
      for (int k = 0; k < L.n; ++k) {
        const float* v = nrm + 3 * (size_t)L.idx[k];
        M[0] = M[0] + v[0] * v[0];
        M[1] = M[1] + v[0] * v[1];
        M[2] = M[2] + v[0] * v[2];
        M[3] = M[3] + v[1] * v[1];
        M[4] = M[4] + v[1] * v[2];
        M[5] = M[5] + v[2] * v[2];
      }
      const float cnt = (float)L.n;
      for (int e = 0; e < 6; ++e) M[e] = M[e] / cnt;
      const float tr = (M[0] + M[3]) + M[5];
      R[i] = (hr_det3(M) - 0.04f * (tr * tr)) + 0.04f;
    }
    free(L.idx);
  }
  /* keypoints: threshold and (optional) non-maximum suppression */
  int K = 0;
  hr_list L = {NULL, 0, 0};
  for (int i = 0; i < n; ++i) {
    if (!(R[i] > thr)) continue;
    int ok = 1;
    if (non_max) {
      hr_neighbours(&g, pts, pts + 4 * (size_t)i, r2, &L);
      for (int k = 0; k < L.n && ok; ++k) ok = !(R[i] < R[L.idx[k]]);
    }
    if (!ok) continue;
    float x[3] = {pts[4 * (size_t)i], pts[4 * (size_t)i + 1], pts[4 * (size_t)i + 2]};
    if (refine) {
      for (int it = 0; it < 10; ++it) {
        hr_neighbours(&g, pts, x, r2, &L);
        double A[6] = {0, 0, 0, 0, 0, 0}, b[3] = {0, 0, 0};
        for (int k = 0; k < L.n; ++k) {
          const float* v = nrm + 3 * (size_t)L.idx[k];
          const float* p = pts + 4 * (size_t)L.idx[k];
          const double nx = v[0], ny = v[1], nz = v[2];
          const double d = (nx * p[0] + ny * p[1]) + nz * p[2];
          A[0] += nx * nx;
          A[1] += nx * ny;
          A[2] += nx * nz;
          A[3] += ny * ny;
          A[4] += ny * nz;
          A[5] += nz * nz;
          b[0] += nx * d;
          b[1] += ny * d;
          b[2] += nz * d;
        }
        const double c00 = A[3] * A[5] - A[4] * A[4], c01 = A[2] * A[4] - A[1] * A[5], c02 = A[1] * A[4] - A[2] * A[3];
        const double det = (A[0] * c00 + A[1] * c01) + A[2] * c02;
        const double tr = (A[0] + A[3]) + A[5];
        if (!(det > 1e-12 * tr * tr * tr)) break;
        const double c11 = A[0] * A[5] - A[2] * A[2], c12 = A[1] * A[2] - A[0] * A[4], c22 = A[0] * A[3] - A[1] * A[1];
        const double nxp = ((c00 * b[0] + c01 * b[1]) + c02 * b[2]) / det;
        const double nyp = ((c01 * b[0] + c11 * b[1]) + c12 * b[2]) / det;
        const double nzp = ((c02 * b[0] + c12 * b[1]) + c22 * b[2]) / det;
        const float y[3] = {(float)nxp, (float)nyp, (float)nzp};
        if (!(hr_d2(y, pts + 4 * (size_t)i) <= r2)) break;
        const float mv = hr_d2(y, x);
        x[0] = y[0];
        x[1] = y[1];
        x[2] = y[2];
        if (mv < 1e-12f) break;
      }
    }
    keys[4 * (size_t)K] = x[0];
    keys[4 * (size_t)K + 1] = x[1];
    keys[4 * (size_t)K + 2] = x[2];
    keys[4 * (size_t)K + 3] = R[i];
    if (src) src[K] = i;
    ++K;
  }
  free(L.idx);
  free(nrm);
  free(R);
  free(g.start);
  free(g.order);
  return K;
}
