/*
 * oracle.c — CPU restatement of the registration hot path (test
 * infrastructure: the checker and the timed CPU baseline, never the product).
 * Build: see oracle/Makefile (gcc -O2 -ffp-contract=off -fopenmp).
 */
#include "oracle.h"

#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

static inline float d2f(const float* q, const float* p) {
  float dx = q[0] - p[0], dy = q[1] - p[1], dz = q[2] - p[2];
  float xx = dx * dx, yy = dy * dy, zz = dz * dz;
  float s = xx + yy;
  return s + zz;
}

/* ------------------------------------------------------------------------ */
/* nearest neighbours                                                        */
/* ------------------------------------------------------------------------ */

/* PCL's ICP keeps a correspondence when its squared distance is <= max^2
 * (registration correspondence estimation); the kd-tree search is exact. */
void orc_nn1_brute(const float* q, int nq, const float* t, int nt, float r2max, int32_t* idx, float* d2) {
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < nq; ++i) {
    float bd = r2max;
    int bi = INT_MAX;
    for (int j = 0; j < nt; ++j) {
      float d = d2f(q + 4 * i, t + 4 * j);
      /* an infinite or NaN d^2 is never a neighbour */
      if (d < bd || (d == bd && j < bi && d < INFINITY)) {
        bd = d;
        bi = j;
      }
    }
    idx[i] = bi == INT_MAX ? -1 : bi;
    if (d2) d2[i] = bi == INT_MAX ? INFINITY : bd;
  }
}

typedef struct {
  double o[3], h;
  int n[3];
  int* start; /* ncells + 1 */
  int* order;
  const float* pts;
} cgrid;

static int cg_cell(const cgrid* g, double v, int a) {
  double f = floor((v - g->o[a]) / g->h);
  if (!(f >= -1e8)) f = -1e8; /* also NaN, as the GPU's fmaxf does */
  if (f > 1e8) f = 1e8;
  return (int)f;
}

static void cg_build(cgrid* g, const float* pts, int n, double h) {
  double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  int nf = 0;
  for (int i = 0; i < n; ++i) {
    /* points with a non-finite coordinate do not size the grid; they sit in
     * a border cell and never match (their d^2 is NaN or inf) */
    if (!(isfinite(pts[4 * i]) && isfinite(pts[4 * i + 1]) && isfinite(pts[4 * i + 2]))) continue;
    ++nf;
    for (int a = 0; a < 3; ++a) {
      if (pts[4 * i + a] < lo[a]) lo[a] = pts[4 * i + a];
      if (pts[4 * i + a] > hi[a]) hi[a] = pts[4 * i + a];
    }
  }
  if (nf == 0)
    for (int a = 0; a < 3; ++a) lo[a] = hi[a] = 0;
  if (!(h > 0)) {
    double vol = 1;
    for (int a = 0; a < 3; ++a) vol *= fmax(hi[a] - lo[a], 1e-3);
    h = 2.0 * cbrt(vol / (n > 0 ? n : 1));
  }
  double cap = 8.0 * n + 4096;
  for (;;) {
    double cells = 1;
    for (int a = 0; a < 3; ++a) cells *= floor((hi[a] - lo[a]) / h) + 1;
    if (cells <= cap) break;
    h *= cbrt(cells / cap) * 1.001;
  }
  g->h = h;
  for (int a = 0; a < 3; ++a) {
    g->o[a] = lo[a];
    g->n[a] = (int)floor((hi[a] - lo[a]) / h) + 1;
  }
  size_t nc = (size_t)g->n[0] * g->n[1] * g->n[2];
  g->start = (int*)calloc(nc + 1, sizeof(int));
  g->order = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
  g->pts = pts;
  int* key = (int*)malloc(sizeof(int) * (n > 0 ? n : 1));
  for (int i = 0; i < n; ++i) {
    int c[3];
    for (int a = 0; a < 3; ++a) {
      c[a] = cg_cell(g, pts[4 * i + a], a);
      if (c[a] < 0) c[a] = 0;
      if (c[a] >= g->n[a]) c[a] = g->n[a] - 1;
    }
    key[i] = (c[2] * g->n[1] + c[1]) * g->n[0] + c[0];
    g->start[key[i] + 1]++;
  }
  for (size_t c = 0; c < nc; ++c) g->start[c + 1] += g->start[c];
  int* fill = (int*)malloc(sizeof(int) * (nc + 1));
  memcpy(fill, g->start, sizeof(int) * (nc + 1));
  for (int i = 0; i < n; ++i) g->order[fill[key[i]]++] = i;
  free(fill);
  free(key);
}

static void cg_free(cgrid* g) {
  free(g->start);
  free(g->order);
}

/* lower bound on the distance from q to anything outside the ring box k */
static double cg_ring_lb(const cgrid* g, const double* q, const int* c, int k) {
  double lb = INFINITY;
  for (int a = 0; a < 3; ++a) {
    if (c[a] - k > 0) lb = fmin(lb, q[a] - (g->o[a] + (c[a] - k) * g->h));
    if (c[a] + k < g->n[a] - 1) lb = fmin(lb, (g->o[a] + (c[a] + k + 1) * g->h) - q[a]);
  }
  return lb;
}

static int cg_beyond(double lb, double bound) {
  double l = lb - 1e-7 * (1.0 + fabs(lb));
  return l > 0 && l * l > (double)bound * (1.0 + 1e-6) + 1e-30;
}

typedef struct {
  int k;
  float* bd;
  int* bi;
} topk;

static void cg_search(const cgrid* g, const float* qf, topk* T) {
  const double q[3] = {qf[0], qf[1], qf[2]};
  int c[3];
  for (int a = 0; a < 3; ++a) c[a] = cg_cell(g, q[a], a);
  int k0 = 0;
  for (int a = 0; a < 3; ++a) {
    if (-c[a] > k0) k0 = -c[a];
    if (c[a] - (g->n[a] - 1) > k0) k0 = c[a] - (g->n[a] - 1);
  }
  for (int k = k0;; ++k) {
    /* the ring's cells inside the grid: loops clamped to the grid (a query
     * far outside, or with a NaN coordinate, starts at a huge ring) */
    const int z0 = c[2] - k > 0 ? c[2] - k : 0, z1 = c[2] + k < g->n[2] - 1 ? c[2] + k : g->n[2] - 1;
    const int y0 = c[1] - k > 0 ? c[1] - k : 0, y1 = c[1] + k < g->n[1] - 1 ? c[1] + k : g->n[1] - 1;
    for (int z = z0; z <= z1; ++z) {
      for (int y = y0; y <= y1; ++y) {
        int edge = (z == c[2] - k || z == c[2] + k || y == c[1] - k || y == c[1] + k);
        const int xs = edge || k == 0 ? (c[0] - k > 0 ? c[0] - k : 0) : c[0] - k;
        const int xe = edge || k == 0 ? (c[0] + k < g->n[0] - 1 ? c[0] + k : g->n[0] - 1) : c[0] + k;
        for (int x = xs; x <= xe; x += (edge || k == 0) ? 1 : 2 * k) {
          if (x < 0 || x >= g->n[0]) continue;
          int cell = (z * g->n[1] + y) * g->n[0] + x;
          for (int s = g->start[cell]; s < g->start[cell + 1]; ++s) {
            int j = g->order[s];
            float d = d2f(qf, g->pts + 4 * j);
            int last = T->k - 1;
            /* an infinite or NaN distance is never taken */
            if (!(d < T->bd[last]) && !(d == T->bd[last] && j < T->bi[last] && d < INFINITY)) continue;
            int p = last;
            while (p > 0 && (d < T->bd[p - 1] || (d == T->bd[p - 1] && j < T->bi[p - 1]))) {
              T->bd[p] = T->bd[p - 1];
              T->bi[p] = T->bi[p - 1];
              --p;
            }
            T->bd[p] = d;
            T->bi[p] = j;
          }
        }
      }
    }
    int covers = 1;
    for (int a = 0; a < 3; ++a)
      if (c[a] - k > 0 || c[a] + k < g->n[a] - 1) covers = 0;
    if (covers) break;
    if (cg_beyond(cg_ring_lb(g, q, c, k), T->bd[T->k - 1])) break;
  }
}

static void cg_nn1(const cgrid* g, int nt, const float* q, int nq, float r2max, int32_t* idx, float* d2) {
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < nq; ++i) {
    float bd = r2max;
    int bi = INT_MAX;
    topk T = {1, &bd, &bi};
    if (nt > 0) cg_search(g, q + 4 * i, &T);
    idx[i] = bi == INT_MAX ? -1 : bi;
    if (d2) d2[i] = bi == INT_MAX ? INFINITY : bd;
  }
}

void orc_nn1_grid(const float* q, int nq, const float* t, int nt, float r2max, float cell, int32_t* idx,
                  float* d2) {
  cgrid g;
  cg_build(&g, t, nt, cell > 0 ? cell : (r2max < INFINITY ? 0.5 * sqrt(r2max) : -1));
  cg_nn1(&g, nt, q, nq, r2max, idx, d2);
  cg_free(&g);
}

/* A target grid kept across calls (the searches are exact, so their
 * results do not depend on the cell size or on reusing the grid). */
struct orc_grid {
  cgrid g;
  int n;
};

orc_grid* orc_grid_create(const float* pts, int n, float cell) {
  orc_grid* G = (orc_grid*)malloc(sizeof(orc_grid));
  cg_build(&G->g, pts, n, cell > 0 ? cell : -1.0);
  G->n = n;
  return G;
}

void orc_grid_destroy(orc_grid* G) {
  if (!G) return;
  cg_free(&G->g);
  free(G);
}

void orc_grid_nn1(const orc_grid* G, const float* q, int nq, float r2max, int32_t* idx, float* d2) {
  cg_nn1(&G->g, G->n, q, nq, r2max, idx, d2);
}

/* Fraction of every stride-th source point that lands, under each pose,
 * within r of the grid's points: scores[h] for poses16[16 h]. */
void orc_grid_inlier_fraction(const orc_grid* G, const float* src, int ns, int stride, const double* poses16,
                              int nh, float r, double* scores) {
  const int m = stride > 0 ? (ns + stride - 1) / stride : 0;
  float* sub = (float*)malloc(sizeof(float) * 4 * (m > 0 ? m : 1));
  float* tmp = (float*)malloc(sizeof(float) * 4 * (m > 0 ? m : 1));
  int32_t* idx = (int32_t*)malloc(sizeof(int32_t) * (m > 0 ? m : 1));
  for (int i = 0; i < m; ++i) memcpy(sub + 4 * i, src + 4 * (size_t)i * stride, 16);
  for (int h = 0; h < nh; ++h) {
    orc_transform_f32(poses16 + 16 * (size_t)h, sub, m, tmp);
    cg_nn1(&G->g, G->n, tmp, m, r * r, idx, NULL);
    int c = 0;
    for (int i = 0; i < m; ++i) c += idx[i] >= 0;
    scores[h] = (double)c / (double)(m > 0 ? m : 1);
  }
  free(sub);
  free(tmp);
  free(idx);
}

/* Fixed-radius (box = 0: d^2 <= r^2, d^2 as d2f) and box (box = 1: the
 * inclusive box [q - r, q + r] with the bounds formed in float, as
 * KeyPoint::getOccupiedGrid forms v_min / v_max, key_point.h:118-140) searches
 * by brute force: every target in ascending index; cnt[i] the true count, the
 * first maxk indices in idx[i * maxk ...], -1 past the count.  A query or
 * target with a non-finite coordinate never matches. */
void orc_range_search(const float* q, int nq, const float* t, int nt, float r, int box, int maxk, int32_t* idx,
                      int32_t* cnt) {
  const float r2 = r * r;
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < nq; ++i) {
    const float* qi = q + 4 * i;
    const int fin = isfinite(qi[0]) && isfinite(qi[1]) && isfinite(qi[2]);
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = qi[a] - r;
      hi[a] = qi[a] + r;
    }
    int c = 0;
    for (int j = 0; j < nt && fin; ++j) {
      const float* p = t + 4 * j;
      const int hit = box ? (p[0] >= lo[0] && p[1] >= lo[1] && p[2] >= lo[2] && p[0] <= hi[0] && p[1] <= hi[1] &&
                             p[2] <= hi[2])
                          : (d2f(qi, p) <= r2);
      if (!hit) continue;
      if (c < maxk) idx[(size_t)i * maxk + c] = j;
      ++c;
    }
    for (int s = c; s < maxk; ++s) idx[(size_t)i * maxk + s] = -1;
    cnt[i] = c;
  }
}

void orc_knn_brute(const float* q, int nq, const float* t, int nt, int k, int32_t* idx, float* d2) {
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < nq; ++i) {
    float bd[64];
    int bi[64];
    for (int s = 0; s < k; ++s) {
      bd[s] = INFINITY;
      bi[s] = INT_MAX;
    }
    for (int j = 0; j < nt; ++j) {
      float d = d2f(q + 4 * i, t + 4 * j);
      int last = k - 1;
      if (!(d < bd[last]) && !(d == bd[last] && j < bi[last] && d < INFINITY)) continue; /* nor inf */
      int p = last;
      while (p > 0 && (d < bd[p - 1] || (d == bd[p - 1] && j < bi[p - 1]))) {
        bd[p] = bd[p - 1];
        bi[p] = bi[p - 1];
        --p;
      }
      bd[p] = d;
      bi[p] = j;
    }
    for (int s = 0; s < k; ++s) {
      idx[(size_t)i * k + s] = bi[s] == INT_MAX ? -1 : bi[s];
      if (d2) d2[(size_t)i * k + s] = bi[s] == INT_MAX ? INFINITY : bd[s];
    }
  }
}

/* ------------------------------------------------------------------------ */
/* pose                                                                      */
/* ------------------------------------------------------------------------ */

void orc_transform_f32(const double* T, const float* in, int n, float* out) {
  float r[12];
  for (int k = 0; k < 12; ++k) r[k] = (float)T[k];
  for (int i = 0; i < n; ++i) {
    const float x = in[4 * i], y = in[4 * i + 1], z = in[4 * i + 2];
    float o[3];
    for (int a = 0; a < 3; ++a) {
      float m0 = r[4 * a] * x, m1 = r[4 * a + 1] * y, m2 = r[4 * a + 2] * z;
      float s = m0 + m1;
      s = s + m2;
      o[a] = s + r[4 * a + 3];
    }
    out[4 * i] = o[0];
    out[4 * i + 1] = o[1];
    out[4 * i + 2] = o[2];
    out[4 * i + 3] = 0.f;
  }
}

/* Cyclic Jacobi eigen-decomposition of a symmetric 4x4 (FP64). */
static void jacobi4(double A[4][4], double V[4][4], double w[4]) {
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) V[i][j] = (i == j);
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0, tot = 0;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        tot += A[i][j] * A[i][j];
        if (i != j) off += A[i][j] * A[i][j];
      }
    if (off <= 1e-32 * tot || off == 0) break;
    for (int p = 0; p < 3; ++p)
      for (int q = p + 1; q < 4; ++q) {
        if (A[p][q] == 0) continue;
        double theta = (A[q][q] - A[p][p]) / (2 * A[p][q]);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1));
        double c = 1 / sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < 4; ++k) {
          double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - s * akq;
          A[k][q] = s * akp + c * akq;
        }
        for (int k = 0; k < 4; ++k) {
          double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - s * aqk;
          A[q][k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 4; ++k) {
          double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - s * vkq;
          V[k][q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < 4; ++i) w[i] = A[i][i];
}

/* Horn (1987): the rotation maximising sum q_c . R p_c is the quaternion of
 * the largest eigenvalue of N built from S = sum p_c q_c^T.  It is the same
 * minimiser Umeyama's SVD form gives (PCL TransformationEstimationSVD). */
int orc_rigid_fit(const float* p, const float* q, const int32_t* corr, int n, double* T) {
  double mp[3] = {0, 0, 0}, mq[3] = {0, 0, 0};
  int m = 0;
  for (int i = 0; i < n; ++i) {
    int j = corr ? corr[i] : i;
    if (j < 0) continue;
    for (int a = 0; a < 3; ++a) {
      mp[a] += p[4 * i + a];
      mq[a] += q[4 * j + a];
    }
    ++m;
  }
  for (int k = 0; k < 16; ++k) T[k] = (k % 5 == 0);
  if (m < 3) return 0;
  for (int a = 0; a < 3; ++a) {
    mp[a] /= m;
    mq[a] /= m;
  }
  double S[3][3] = {{0}};
  for (int i = 0; i < n; ++i) {
    int j = corr ? corr[i] : i;
    if (j < 0) continue;
    double dp[3], dq[3];
    for (int a = 0; a < 3; ++a) {
      dp[a] = (double)p[4 * i + a] - mp[a];
      dq[a] = (double)q[4 * j + a] - mq[a];
    }
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) S[a][b] += dp[a] * dq[b];
  }
  double N[4][4] = {
      {S[0][0] + S[1][1] + S[2][2], S[1][2] - S[2][1], S[2][0] - S[0][2], S[0][1] - S[1][0]},
      {S[1][2] - S[2][1], S[0][0] - S[1][1] - S[2][2], S[0][1] + S[1][0], S[2][0] + S[0][2]},
      {S[2][0] - S[0][2], S[0][1] + S[1][0], -S[0][0] + S[1][1] - S[2][2], S[1][2] + S[2][1]},
      {S[0][1] - S[1][0], S[2][0] + S[0][2], S[1][2] + S[2][1], -S[0][0] - S[1][1] + S[2][2]}};
  double V[4][4], w[4];
  jacobi4(N, V, w);
  int b = 0;
  for (int i = 1; i < 4; ++i)
    if (w[i] > w[b]) b = i;
  double q0 = V[0][b], qx = V[1][b], qy = V[2][b], qz = V[3][b];
  double nrm = sqrt(q0 * q0 + qx * qx + qy * qy + qz * qz);
  q0 /= nrm; qx /= nrm; qy /= nrm; qz /= nrm;
  double R[9] = {q0 * q0 + qx * qx - qy * qy - qz * qz, 2 * (qx * qy - q0 * qz), 2 * (qx * qz + q0 * qy),
                 2 * (qy * qx + q0 * qz), q0 * q0 - qx * qx + qy * qy - qz * qz, 2 * (qy * qz - q0 * qx),
                 2 * (qz * qx - q0 * qy), 2 * (qz * qy + q0 * qx), q0 * q0 - qx * qx - qy * qy + qz * qz};
  for (int a = 0; a < 3; ++a) {
    for (int c = 0; c < 3; ++c) T[a * 4 + c] = R[a * 3 + c];
    T[a * 4 + 3] = mq[a] - (R[a * 3] * mp[0] + R[a * 3 + 1] * mp[1] + R[a * 3 + 2] * mp[2]);
  }
  return m;
}

static void mat4mul(const double* A, const double* B, double* C) {
  double T[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = 0;
      for (int k = 0; k < 4; ++k) s += A[i * 4 + k] * B[k * 4 + j];
      T[i * 4 + j] = s;
    }
  memcpy(C, T, sizeof(T));
}

/* One ICP iteration at pose P (PCL IterativeClosestPoint::computeTransformation:
 * transform source, correspondences by exact 1-NN with d^2 <= max^2, SVD
 * estimate on the transformed source, transformation = delta * transformation). */
static int icp_step(const float* src, int ns, const cgrid* g, const float* tgt, int nt, float r2max,
                    const double* P, int32_t* corr, float* tmp, double* Pnext, double* dT, double* fitness) {
  orc_transform_f32(P, src, ns, tmp);
  float* d2 = (float*)malloc(sizeof(float) * (ns > 0 ? ns : 1));
  cg_nn1(g, nt, tmp, ns, r2max, corr, d2);
  double fs = 0;
  int m = 0;
  for (int i = 0; i < ns; ++i)
    if (corr[i] >= 0) {
      fs += d2[i];
      ++m;
    }
  free(d2);
  if (m < 3) {
    memcpy(Pnext, P, 16 * sizeof(double));
    return m;
  }
  orc_rigid_fit(tmp, tgt, corr, ns, dT);
  mat4mul(dT, P, Pnext);
  *fitness = fs / m;
  return m;
}

static void icp_run(const float* src, int ns, const cgrid* g, const float* tgt, int nt, int max_it,
                    float max_dist, double eps_t, double eps_r, const double* init, orc_icp_out* out,
                    double* trace_pose, int32_t* trace_corr) {
  const float r2max = (max_dist > 0 && max_dist < 1e18f) ? max_dist * max_dist : INFINITY;
  double P[16];
  for (int k = 0; k < 16; ++k) P[k] = init ? init[k] : (k % 5 == 0);
  if (trace_pose) memcpy(trace_pose, P, sizeof(P));
  float* tmp = (float*)malloc(sizeof(float) * 4 * (ns > 0 ? ns : 1));
  int32_t* corr = (int32_t*)malloc(sizeof(int32_t) * (ns > 0 ? ns : 1));
  out->converged = 1;
  out->iterations = 0;
  out->fitness = 0;
  out->n_corr = 0;
  for (int it = 0; it < max_it; ++it) {
    double Pn[16], dT[16], fit = 0;
    int m = icp_step(src, ns, g, tgt, nt, r2max, P, corr, tmp, Pn, dT, &fit);
    if (trace_corr) memcpy(trace_corr + (size_t)it * ns, corr, sizeof(int32_t) * ns);
    out->iterations = it + 1;
    out->n_corr = m;
    if (m < 3) {
      out->converged = 0;
      break;
    }
    memcpy(P, Pn, sizeof(P));
    out->fitness = fit;
    if (trace_pose) memcpy(trace_pose + (size_t)(it + 1) * 16, P, sizeof(P));
    double cosang = 0.5 * (dT[0] + dT[5] + dT[10] - 1.0);
    double tsq = dT[3] * dT[3] + dT[7] * dT[7] + dT[11] * dT[11];
    if (eps_t > 0 && tsq < eps_t && (eps_r <= 0 || cosang > eps_r)) break;
  }
  memcpy(out->pose, P, sizeof(P));
  free(tmp);
  free(corr);
}

void orc_icp(const float* src, int ns, const float* tgt, int nt, int max_it, float max_dist, double eps_t,
             double eps_r, const double* init, orc_icp_out* out, double* trace_pose, int32_t* trace_corr) {
  /* the target grid is built once for all iterations */
  const float cell = (max_dist > 0 && max_dist < 1e18f) ? 0.5f * max_dist : -1.f;
  cgrid g;
  cg_build(&g, tgt, nt, cell);
  icp_run(src, ns, &g, tgt, nt, max_it, max_dist, eps_t, eps_r, init, out, trace_pose, trace_corr);
  cg_free(&g);
}

/* ICP against a kept grid (its points are the target). */
void orc_grid_icp(const orc_grid* G, const float* src, int ns, int max_it, float max_dist, double eps_t,
                  double eps_r, const double* init, orc_icp_out* out) {
  icp_run(src, ns, &G->g, G->g.pts, G->n, max_it, max_dist, eps_t, eps_r, init, out, NULL, NULL);
}

/* Several ICP problems of one source against a kept grid, one problem per
 * thread (each problem's searches then run on its own thread). */
void orc_grid_icp_multi(const orc_grid* G, const float* src, int ns, int max_it, float max_dist,
                        const double* inits16, int nh, orc_icp_out* outs) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int h = 0; h < nh; ++h)
    icp_run(src, ns, &G->g, G->g.pts, G->n, max_it, max_dist, 0.0, 0.0, inits16 + 16 * (size_t)h, outs + h,
            NULL, NULL);
}

void orc_icp_replay(const float* src, int ns, const float* tgt, int nt, float max_dist, const double* poses_in,
                    int iters, int32_t* corr_out, double* poses_out, int32_t* ncorr_out) {
  const float r2max = (max_dist > 0 && max_dist < 1e18f) ? max_dist * max_dist : INFINITY;
  const float cell = (max_dist > 0 && max_dist < 1e18f) ? 0.5f * max_dist : -1.f;
  float* tmp = (float*)malloc(sizeof(float) * 4 * (ns > 0 ? ns : 1));
  cgrid g;
  cg_build(&g, tgt, nt, cell);
  memcpy(poses_out, poses_in, 16 * sizeof(double));
  for (int it = 0; it < iters; ++it) {
    double dT[16], fit = 0;
    int m = icp_step(src, ns, &g, tgt, nt, r2max, poses_in + 16 * (size_t)it, corr_out + (size_t)it * ns, tmp,
                     poses_out + 16 * (size_t)(it + 1), dT, &fit);
    if (ncorr_out) ncorr_out[it] = m;
  }
  cg_free(&g);
  free(tmp);
}

/* ------------------------------------------------------------------------ */
/* TDF: kernel.cu:8-31 — voxel (x, y, z) with x fastest (kernel.cu:16-18),  */
/* start at 900, keep the minimum float(dx*dx + dy*dy + dz*dz).             */
/* ------------------------------------------------------------------------ */
void orc_tdf(const int32_t* occ, int n_occ, int dim, float* out) {
  const int vol = dim * dim * dim;
#pragma omp parallel for schedule(static)
  for (int v = 0; v < vol; ++v) {
    int z = v / (dim * dim);
    int y = (v - z * dim * dim) / dim;
    int x = v - z * dim * dim - y * dim;
    float best = 900;
    for (int i = 0; i < n_occ; ++i) {
      int dx = x - occ[3 * i], dy = y - occ[3 * i + 1], dz = z - occ[3 * i + 2];
      float t = (float)(dx * dx + dy * dy + dz * dz);
      if (t < best) best = t;
    }
    out[v] = best;
  }
}

/* ======================================================================== */
/* recognition stages                                                       */
/* ======================================================================== */

typedef struct {
  uint32_t key;
  int32_t idx;
} kv_t;

static int kv_cmp(const void* a, const void* b) {
  const kv_t* x = (const kv_t*)a;
  const kv_t* y = (const kv_t*)b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

/* Voxel keys floor(p * inv) relative to the minimum voxel; returns the number
 * of keys or -1 when the key space does not fit 32 bits.  kv sorted by
 * (key, index), i.e. a stable sort by key. */
/* Voxel keys floor(p * inv) relative to the minimum voxel, sorted by
 * (key, index) (a stable sort by key).  Points with a non-finite coordinate
 * get no voxel (PCL's VoxelGrid skips them in clouds that are not dense):
 * they are left out and the number of keyed points is returned.  -1 when a
 * finite point's voxel index reaches 10^9 or the key space does not fit in
 * 32 bits with one key (0xffffffff) to spare. */
static int voxel_keys(const float* pts, int n, float inv, kv_t* kv, int* ijk_out) {
  int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
  int m = 0;
  for (int i = 0; i < n; ++i) {
    const float* p = pts + 4 * i;
    if (!(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]))) continue;
    for (int a = 0; a < 3; ++a) {
      const float f = floorf(p[a] * inv);
      if (!(fabsf(f) < 1.0e9f)) return -1;
      const int v = (int)f;
      ijk_out[3 * i + a] = v;
      if (v < lo[a]) lo[a] = v;
      if (v > hi[a]) hi[a] = v;
    }
    kv[m++].idx = i;
  }
  if (m == 0) return 0;
  uint64_t d0 = (uint64_t)(hi[0] - lo[0] + 1), d1 = (uint64_t)(hi[1] - lo[1] + 1), d2 = (uint64_t)(hi[2] - lo[2] + 1);
  if (d0 * d1 > 0xffffffffull || d0 * d1 * d2 >= 0xffffffffull) return -1;
  for (int k = 0; k < m; ++k) {
    const int i = kv[k].idx;
    uint32_t x = (uint32_t)(ijk_out[3 * i] - lo[0]), y = (uint32_t)(ijk_out[3 * i + 1] - lo[1]),
             z = (uint32_t)(ijk_out[3 * i + 2] - lo[2]);
    kv[k].key = (z * (uint32_t)d1 + y) * (uint32_t)d0 + x;
  }
  qsort(kv, (size_t)m, sizeof(kv_t), kv_cmp);
  return m;
}

int orc_voxel_downsample(const float* pts, int n, float leaf, float* out) {
  const float inv = 1.0f / leaf;
  kv_t* kv = (kv_t*)malloc(sizeof(kv_t) * (n > 0 ? n : 1));
  int* ijk = (int*)malloc(sizeof(int) * 3 * (n > 0 ? n : 1));
  const int m = voxel_keys(pts, n, inv, kv, ijk);
  if (m < 0) {
    free(kv);
    free(ijk);
    return -1;
  }
  int v = 0;
  for (int s = 0; s < m;) {
    int e = s;
    float sx = 0.f, sy = 0.f, sz = 0.f;
    while (e < m && kv[e].key == kv[s].key) {
      const float* p = pts + 4 * kv[e].idx;
      sx = sx + p[0];
      sy = sy + p[1];
      sz = sz + p[2];
      ++e;
    }
    const float c = (float)(e - s);
    out[4 * v] = sx / c;
    out[4 * v + 1] = sy / c;
    out[4 * v + 2] = sz / c;
    out[4 * v + 3] = 0.f;
    ++v;
    s = e;
  }
  free(kv);
  free(ijk);
  return v;
}

/* Cyclic Jacobi for a symmetric 3x3 in FP32.  Every operation is a single
 * rounded IEEE op (compiled without contraction); the GPU performs the same
 * sequence, so results match bit for bit.  Eigenvalues ascending (stable),
 * eigenvectors in the columns of V. */
void orc_eig3(const float* A9, float* w, float* V) {
  float a[3][3], v[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      a[i][j] = A9[i * 3 + j];
      v[i][j] = (i == j) ? 1.f : 0.f;
    }
  for (int sweep = 0; sweep < 16; ++sweep) {
    float o01 = a[0][1] * a[0][1], o02 = a[0][2] * a[0][2], o12 = a[1][2] * a[1][2];
    float off = (o01 + o02) + o12;
    float d0 = a[0][0] * a[0][0], d1 = a[1][1] * a[1][1], d2 = a[2][2] * a[2][2];
    float dsum = (d0 + d1) + d2;
    if (!(off > 1e-12f * dsum)) break;
    for (int pq = 0; pq < 3; ++pq) {
      const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
      const float apq = a[p][q];
      if (apq == 0.f) continue;
      const float num = a[q][q] - a[p][p];
      const float den = 2.f * apq;
      const float theta = num / den;
      const float th2 = theta * theta;
      const float rt = sqrtf(th2 + 1.f);
      const float at = fabsf(theta) + rt;
      float t = 1.f / at;
      if (theta < 0.f) t = -t;
      const float t2 = t * t;
      const float c = 1.f / sqrtf(t2 + 1.f);
      const float s = t * c;
      for (int k = 0; k < 3; ++k) {
        const float akp = a[k][p], akq = a[k][q];
        const float m0 = c * akp, m1 = s * akq, m2 = s * akp, m3 = c * akq;
        a[k][p] = m0 - m1;
        a[k][q] = m2 + m3;
      }
      for (int k = 0; k < 3; ++k) {
        const float apk = a[p][k], aqk = a[q][k];
        const float m0 = c * apk, m1 = s * aqk, m2 = s * apk, m3 = c * aqk;
        a[p][k] = m0 - m1;
        a[q][k] = m2 + m3;
      }
      for (int k = 0; k < 3; ++k) {
        const float vkp = v[k][p], vkq = v[k][q];
        const float m0 = c * vkp, m1 = s * vkq, m2 = s * vkp, m3 = c * vkq;
        v[k][p] = m0 - m1;
        v[k][q] = m2 + m3;
      }
    }
  }
  int ord[3] = {0, 1, 2};
  /* stable ascending sort of the diagonal */
  for (int i = 1; i < 3; ++i) {
    int x = ord[i], j = i;
    while (j > 0 && a[ord[j - 1]][ord[j - 1]] > a[x][x]) {
      ord[j] = ord[j - 1];
      --j;
    }
    ord[j] = x;
  }
  for (int j = 0; j < 3; ++j) {
    w[j] = a[ord[j]][ord[j]];
    for (int i = 0; i < 3; ++i) V[i * 3 + j] = v[i][ord[j]];
  }
}

void orc_normals(const float* pts, int n, int k, const float* vp, float* out) {
  int32_t* nb = (int32_t*)malloc(sizeof(int32_t) * (size_t)n * k + 4);
  float* nd = (float*)malloc(sizeof(float) * (size_t)n * k + 4);
  cgrid g;
  cg_build(&g, pts, n, -1.0);
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < n; ++i) {
    float bd[64];
    int bi[64];
    for (int s = 0; s < k; ++s) {
      bd[s] = INFINITY;
      bi[s] = INT_MAX;
    }
    topk T = {k, bd, bi};
    cg_search(&g, pts + 4 * i, &T);
    int m = 0;
    for (int s = 0; s < k; ++s)
      if (bi[s] != INT_MAX) ++m;
    float mx = 0.f, my = 0.f, mz = 0.f;
    for (int s = 0; s < m; ++s) {
      const float* p = pts + 4 * bi[s];
      mx = mx + p[0];
      my = my + p[1];
      mz = mz + p[2];
    }
    const float fm = (float)m;
    mx = mx / fm;
    my = my / fm;
    mz = mz / fm;
    float c00 = 0.f, c01 = 0.f, c02 = 0.f, c11 = 0.f, c12 = 0.f, c22 = 0.f;
    for (int s = 0; s < m; ++s) {
      const float* p = pts + 4 * bi[s];
      const float dx = p[0] - mx, dy = p[1] - my, dz = p[2] - mz;
      const float xx = dx * dx, xy = dx * dy, xz = dx * dz, yy = dy * dy, yz = dy * dz, zz = dz * dz;
      c00 = c00 + xx;
      c01 = c01 + xy;
      c02 = c02 + xz;
      c11 = c11 + yy;
      c12 = c12 + yz;
      c22 = c22 + zz;
    }
    const float A[9] = {c00, c01, c02, c01, c11, c12, c02, c12, c22};
    float w[3], V[9];
    orc_eig3(A, w, V);
    float nx = V[0], ny = V[3], nz = V[6];
    const float* p = pts + 4 * i;
    const float vx = vp[0] - p[0], vy = vp[1] - p[1], vz = vp[2] - p[2];
    const float t0 = vx * nx, t1 = vy * ny, t2 = vz * nz;
    const float dotv = (t0 + t1) + t2;
    if (dotv < 0.f) {
      nx = -nx;
      ny = -ny;
      nz = -nz;
    }
    const float den = (w[0] + w[1]) + w[2];
    out[4 * i] = nx;
    out[4 * i + 1] = ny;
    out[4 * i + 2] = nz;
    out[4 * i + 3] = den != 0.f ? w[0] / den : 0.f;
  }
  cg_free(&g);
  free(nb);
  free(nd);
}

int orc_uniform_sample(const float* pts, int n, float r, int32_t* out_idx) {
  const float inv = 1.0f / r;
  kv_t* kv = (kv_t*)malloc(sizeof(kv_t) * (n > 0 ? n : 1));
  int* ijk = (int*)malloc(sizeof(int) * 3 * (n > 0 ? n : 1));
  const int m = voxel_keys(pts, n, inv, kv, ijk);
  if (m < 0) {
    free(kv);
    free(ijk);
    return -1;
  }
  int K = 0;
  for (int s = 0; s < m;) {
    int e = s, best = -1;
    float bd = INFINITY;
    while (e < m && kv[e].key == kv[s].key) {
      const int i = kv[e].idx;
      const float* p = pts + 4 * i;
      float c[3];
      for (int a = 0; a < 3; ++a) {
        const float fi = (float)ijk[3 * i + a];
        const float h = fi + 0.5f;
        c[a] = h * r;
      }
      const float dx = p[0] - c[0], dy = p[1] - c[1], dz = p[2] - c[2];
      const float xx = dx * dx, yy = dy * dy, zz = dz * dz;
      const float d = (xx + yy) + zz;
      if (d < bd || (d == bd && i < best)) {
        bd = d;
        best = i;
      }
      ++e;
    }
    out_idx[K++] = best;
    s = e;
  }
  free(kv);
  free(ijk);
  return K;
}

/* SHOT conventions (restated from the paper):
 *  support: points within radius R of the keypoint (d^2 <= R*R) whose
 *  oriented normal faces the keypoint's (n_j . n_k >= -0.2);
 *  LRF: M = sum (R - d) (p - k)(p - k)^T, x = eigenvector of the largest
 *  eigenvalue, z of the smallest; x flipped so that at least half of the
 *  support has (p - k).x >= 0, z flipped so that sum (R - d)(n_p . z) >= 0;
 *  y = z cross x;
 *  histogram: 2 radial shells (split at R/2) x 2 elevations x 8 azimuths x
 *  11 cosine bins of n_p . z, quadrilinear interpolation (azimuth circular,
 *  the others clamped at their ends), the keypoint itself excluded; the 352
 *  values are L2-normalised.
 * Arithmetic (the GPU kernel k_shot runs the same, so descriptors and LRFs
 * agree bit for bit): every per-point term is a fixed sequence of IEEE
 * single operations (no contraction: -ffp-contract=off); every sum over the
 * support is an integer sum of fixed-point terms, each rounded to an int32
 * (covariance terms in units of 2^-(30 - e3) with R^3 < 2^e3, z-sign terms
 * in units of 2^-(30 - e1) with R < 2^e1, summed in int64; histogram votes
 * in units of 2^-(31 - b), b the bit length of the support count, summed
 * in uint32), so the order of the support does not matter; sums convert
 * back by one int-to-float rounding and an exact power-of-two scale; angles
 * come from shot_atan2 below; the norm is summed as 32 lanes of 11 bins
 * each (lane l: bins l, l + 32, ...) closed by a xor butterfly. */
#define SHOT_PI 0x1.921fb6p+1f
#define SHOT_FACING (-0.2f)

/* Convention switches for probes of descriptor repeatability (0 = the
 * conventions the GPU path uses).  bit 0: keep support points facing away
 * (no n_j . n_k >= -0.2 filter); bit 1: sign of z by the paper's majority
 * rule over the support's offsets instead of agreement with the oriented
 * normals. */
static int g_shot_flags = 0;
void orc_set_shot_flags(int flags) { g_shot_flags = flags; }

/* atan2 by the reduction atan(a) = pi/6 + atan((sqrt(3) a - 1) / (a +
 * sqrt(3))) for a = min(|x|,|y|) / max(|x|,|y|) above tan(pi/12) (Cody and
 * Waite, Software Manual for the Elementary Functions, 1980, ch. 11), the
 * series u - u^3/3 + ... - u^11/11 on |u| <= tan(pi/12), then the octant and
 * the signs; atan2(0, 0) = 0 and -0 counts as positive. */
static float shot_atan2(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
  if (!(mx > 0.f)) return 0.f;
  const float a = mn / mx;
  float u = a, base = 0.f;
  if (a > 0x1.126146p-2f) {
    u = (a * 0x1.bb67aep+0f - 1.f) / (a + 0x1.bb67aep+0f);
    base = 0x1.0c1524p-1f;
  }
  const float z = u * u;
  float p = -0x1.745d18p-4f;
  p = p * z + 0x1.c71c72p-4f;
  p = p * z + -0x1.24924ap-3f;
  p = p * z + 0x1.99999ap-3f;
  p = p * z + -0x1.555556p-2f;
  p = p * z;
  float r = base + (u + u * p);
  if (ay > ax) r = 0x1.921fb6p+0f - r;
  if (x < 0.f) r = SHOT_PI - r;
  return y < 0.f ? -r : r;
}

float orc_shot_atan2(float y, float x) { return shot_atan2(y, x); }

static float dot3f(float a0, float a1, float a2, float b0, float b1, float b2) {
  const float p0 = a0 * b0, p1 = a1 * b1, p2 = a2 * b2;
  return (p0 + p1) + p2;
}

/* e with v < 2^e for a positive normal float v (frexp's exponent) */
static int shot_exp2_above(float v) {
  uint32_t u;
  memcpy(&u, &v, 4);
  return (int)((u >> 23) & 0xffu) - 126;
}


static void shot_bins(float pos, int nb, int circular, int* b0, float* w0, int* b1, float* w1) {
  const float fl = floorf(pos);
  int lo = (int)fl;
  const float f = pos - fl;
  if (circular) {
    *b0 = ((lo % nb) + nb) % nb;
    *b1 = (*b0 + 1) % nb;
    *w0 = 1.f - f;
    *w1 = f;
    return;
  }
  if (lo < 0) {
    *b0 = 0; *w0 = 1.f; *b1 = 0; *w1 = 0.f;
  } else if (lo >= nb - 1) {
    *b0 = nb - 1; *w0 = 1.f; *b1 = nb - 1; *w1 = 0.f;
  } else {
    *b0 = lo; *w0 = 1.f - f; *b1 = lo + 1; *w1 = f;
  }
}

void orc_shot352(const float* pts, const float* normals, int n, const int32_t* keys, int nk, float R,
                 float* desc, float* lrf_out) {
  cgrid g;
  cg_build(&g, pts, n, R);
  const float R2 = R * R;
  const int e_cov = 30 - shot_exp2_above(R2 * R), e_z = 30 - shot_exp2_above(R);
  const float cov_scale = ldexpf(1.f, e_cov), cov_unscale = ldexpf(1.f, -e_cov), z_scale = ldexpf(1.f, e_z);
#pragma omp parallel for schedule(dynamic, 16)
  for (int kk = 0; kk < nk; ++kk) {
    const float* kp = pts + 4 * keys[kk];
    const float* nkp = normals + 4 * keys[kk];
    float* D = desc + (size_t)kk * 352;
    /* gather support by walking the 27 cells around the keypoint */
    int cap = 256, cnt = 0;
    int* sup = (int*)malloc(sizeof(int) * cap);
    int c[3];
    for (int a = 0; a < 3; ++a) c[a] = cg_cell(&g, kp[a], a);
    for (int z = c[2] - 1; z <= c[2] + 1; ++z)
      for (int y = c[1] - 1; y <= c[1] + 1; ++y)
        for (int x = c[0] - 1; x <= c[0] + 1; ++x) {
          if (x < 0 || y < 0 || z < 0 || x >= g.n[0] || y >= g.n[1] || z >= g.n[2]) continue;
          const int cell = (z * g.n[1] + y) * g.n[0] + x;
          for (int s = g.start[cell]; s < g.start[cell + 1]; ++s) {
            const int j = g.order[s];
            const float* nj = normals + 4 * j;
            const float facing = dot3f(nj[0], nj[1], nj[2], nkp[0], nkp[1], nkp[2]);
            if (d2f(kp, pts + 4 * j) <= R2 && (facing >= SHOT_FACING || (g_shot_flags & 1))) {
              if (cnt == cap) {
                cap *= 2;
                sup = (int*)realloc(sup, sizeof(int) * cap);
              }
              sup[cnt++] = j;
            }
          }
        }
    long long m[6] = {0, 0, 0, 0, 0, 0};
    for (int s = 0; s < cnt; ++s) {
      const float* p = pts + 4 * sup[s];
      const float dx = p[0] - kp[0], dy = p[1] - kp[1], dz = p[2] - kp[2];
      const float w = R - sqrtf(d2f(p, kp));
      const float wx = w * dx, wy = w * dy, wz = w * dz;
      m[0] += lrintf(wx * dx * cov_scale); m[1] += lrintf(wx * dy * cov_scale);
      m[2] += lrintf(wx * dz * cov_scale); m[3] += lrintf(wy * dy * cov_scale);
      m[4] += lrintf(wy * dz * cov_scale); m[5] += lrintf(wz * dz * cov_scale);
    }
    const float m0 = (float)m[0] * cov_unscale, m1 = (float)m[1] * cov_unscale, m2 = (float)m[2] * cov_unscale,
                m3 = (float)m[3] * cov_unscale, m4 = (float)m[4] * cov_unscale, m5 = (float)m[5] * cov_unscale;
    const float M[9] = {m0, m1, m2, m1, m3, m4, m2, m4, m5};
    float ev[3], V[9];
    orc_eig3(M, ev, V);
    float X[3] = {V[2], V[5], V[8]}, Z[3] = {V[0], V[3], V[6]};
    int px = 0, nx = 0, pz = 0, nz = 0;
    long long zn = 0;
    for (int s = 0; s < cnt; ++s) {
      const float* p = pts + 4 * sup[s];
      const float* nv = normals + 4 * sup[s];
      const float dx = p[0] - kp[0], dy = p[1] - kp[1], dz = p[2] - kp[2];
      if (dot3f(dx, dy, dz, X[0], X[1], X[2]) >= 0.f) ++px; else ++nx;
      if (dot3f(dx, dy, dz, Z[0], Z[1], Z[2]) >= 0.f) ++pz; else ++nz;
      const float w = R - sqrtf(d2f(p, kp));
      zn += lrintf(w * dot3f(nv[0], nv[1], nv[2], Z[0], Z[1], Z[2]) * z_scale);
    }
    if (px < nx) for (int a = 0; a < 3; ++a) X[a] = -X[a];
    if ((g_shot_flags & 2) ? (pz < nz) : (zn < 0))
      for (int a = 0; a < 3; ++a) Z[a] = -Z[a];
    const float Y[3] = {Z[1] * X[2] - Z[2] * X[1], Z[2] * X[0] - Z[0] * X[2], Z[0] * X[1] - Z[1] * X[0]};
    if (lrf_out) {
      float* L = lrf_out + (size_t)kk * 9;
      for (int a = 0; a < 3; ++a) { L[a] = X[a]; L[3 + a] = Y[a]; L[6 + a] = Z[a]; }
    }
    uint32_t H[352];
    memset(H, 0, sizeof(H));
    int bits = 0;
    while (bits < 32 && (cnt >> bits) != 0) ++bits;
    const float hs = ldexpf(1.f, 31 - bits), hu = ldexpf(1.f, bits - 31);
    for (int s = 0; s < cnt; ++s) {
      const float* p = pts + 4 * sup[s];
      const float d2 = d2f(p, kp);
      if (!(d2 > 0.f)) continue;
      const float dx = p[0] - kp[0], dy = p[1] - kp[1], dz = p[2] - kp[2];
      const float lx = dot3f(dx, dy, dz, X[0], X[1], X[2]);
      const float ly = dot3f(dx, dy, dz, Y[0], Y[1], Y[2]);
      const float lz = dot3f(dx, dy, dz, Z[0], Z[1], Z[2]);
      const float* nv = normals + 4 * sup[s];
      float cs = dot3f(nv[0], nv[1], nv[2], Z[0], Z[1], Z[2]);
      cs = fminf(fmaxf(cs, -1.f), 1.f);
      const float d = sqrtf(d2);
      const float az = shot_atan2(ly, lx);
      const float lxx = lx * lx, lyy = ly * ly;
      const float el = shot_atan2(lz, sqrtf(lxx + lyy));
      int cb0, cb1, ab0, ab1, eb0, eb1, rb0, rb1;
      float cw0, cw1, aw0, aw1, ew0, ew1, rw0, rw1;
      shot_bins((cs + 1.f) * 5.5f - 0.5f, 11, 0, &cb0, &cw0, &cb1, &cw1);
      shot_bins((az + SHOT_PI) * 0x1.45f306p+0f - 0.5f, 8, 1, &ab0, &aw0, &ab1, &aw1);
      shot_bins((el + 0x1.921fb6p+0f) * 0x1.45f306p-1f - 0.5f, 2, 0, &eb0, &ew0, &eb1, &ew1);
      shot_bins(d / R * 2.f - 0.5f, 2, 0, &rb0, &rw0, &rb1, &rw1);
      const int cb[2] = {cb0, cb1}, ab[2] = {ab0, ab1}, eb[2] = {eb0, eb1}, rb[2] = {rb0, rb1};
      const float cw[2] = {cw0, cw1}, aw[2] = {aw0, aw1}, ew[2] = {ew0, ew1}, rw[2] = {rw0, rw1};
      for (int i0 = 0; i0 < 2; ++i0)
        for (int i1 = 0; i1 < 2; ++i1)
          for (int i2 = 0; i2 < 2; ++i2)
            for (int i3 = 0; i3 < 2; ++i3) {
              const float w = rw[i0] * ew[i1] * aw[i2] * cw[i3];
              if (w == 0.f) continue;
              H[((rb[i0] * 2 + eb[i1]) * 8 + ab[i2]) * 11 + cb[i3]] += (uint32_t)lrintf(w * hs);
            }
    }
    float hb[352], lanes[32];
    for (int b = 0; b < 352; ++b) hb[b] = (float)H[b] * hu;
    for (int l = 0; l < 32; ++l) {
      float s = 0.f;
      for (int k = 0; k < 11; ++k) s = s + hb[l + 32 * k] * hb[l + 32 * k];
      lanes[l] = s;
    }
    for (int o = 16; o > 0; o >>= 1) {
      float nxt[32];
      for (int l = 0; l < 32; ++l) nxt[l] = lanes[l] + lanes[l ^ o];
      memcpy(lanes, nxt, sizeof(lanes));
    }
    const float ss = lanes[0];
    const float inv = ss > 0.f ? 1.f / sqrtf(ss) : 0.f;
    for (int b = 0; b < 352; ++b) D[b] = hb[b] * inv;
    free(sup);
  }
  cg_free(&g);
}

/* Exact FP32 1-NN of descriptors: d^2 = sum over k in order of (a_k - b_k)^2,
 * each operation rounded separately, ties to the lowest row.  For speed the
 * database is read from a transposed copy, 16 rows x 4 queries at a time,
 * with GCC's generic vector types: every lane holds one (query, row) pair's
 * own running sum, added in the same k order, so each sum is bit-identical
 * to the scalar loop's (no reassociation; -ffp-contract=off keeps the
 * multiply and the add separate). */
typedef float orc_v4 __attribute__((vector_size(16)));
#define MATCH_RB 16
#define MATCH_QB 4
void orc_match(const float* q, int nq, const float* db, int ndb, int dim, int32_t* idx, float* d2) {
  const int nblk = (ndb + MATCH_RB - 1) / MATCH_RB;
  float* dbT = (float*)aligned_alloc(64, sizeof(float) * (size_t)(nblk > 0 ? nblk : 1) * dim * MATCH_RB);
  for (int b = 0; b < nblk; ++b)
    for (int k = 0; k < dim; ++k)
      for (int r = 0; r < MATCH_RB; ++r) {
        const int j = b * MATCH_RB + r;
        dbT[((size_t)b * dim + k) * MATCH_RB + r] = j < ndb ? db[(size_t)j * dim + k] : 0.f;
      }
  const int nqb = (nq + MATCH_QB - 1) / MATCH_QB;
#pragma omp parallel for schedule(dynamic, 8)
  for (int qb = 0; qb < nqb; ++qb) {
    const int q0 = qb * MATCH_QB;
    const float* a[MATCH_QB];
    float bd[MATCH_QB];
    int bi[MATCH_QB];
    for (int u = 0; u < MATCH_QB; ++u) {
      a[u] = q + (size_t)(q0 + u < nq ? q0 + u : q0) * dim;
      bd[u] = INFINITY;
      bi[u] = -1;
    }
    for (int b = 0; b < nblk; ++b) {
      const orc_v4* B = (const orc_v4*)(dbT + (size_t)b * dim * MATCH_RB);
      orc_v4 acc[MATCH_QB][MATCH_RB / 4];
      for (int u = 0; u < MATCH_QB; ++u)
        for (int v = 0; v < MATCH_RB / 4; ++v) acc[u][v] = (orc_v4){0.f, 0.f, 0.f, 0.f};
      for (int k = 0; k < dim; ++k) {
        const orc_v4* Bk = B + (size_t)k * (MATCH_RB / 4);
        for (int u = 0; u < MATCH_QB; ++u) {
          const float x = a[u][k];
          const orc_v4 xa = {x, x, x, x};
          for (int v = 0; v < MATCH_RB / 4; ++v) {
            const orc_v4 t = xa - Bk[v];
            const orc_v4 tt = t * t;
            acc[u][v] = acc[u][v] + tt;
          }
        }
      }
      for (int u = 0; u < MATCH_QB; ++u) {
        float sums[MATCH_RB];
        memcpy(sums, acc[u], sizeof(sums));
        for (int r = 0; r < MATCH_RB; ++r) {
          const int j = b * MATCH_RB + r;
          if (j < ndb && sums[r] < bd[u]) {
            bd[u] = sums[r];
            bi[u] = j;
          }
        }
      }
    }
    for (int u = 0; u < MATCH_QB && q0 + u < nq; ++u) {
      idx[q0 + u] = bi[u];
      if (d2) d2[q0 + u] = bd[u];
    }
  }
  free(dbT);
}

typedef struct {
  float d;
  int i;
} dk_t;

static int dk_cmp(const void* a, const void* b) {
  const dk_t* x = (const dk_t*)a;
  const dk_t* y = (const dk_t*)b;
  if (x->d != y->d) return x->d < y->d ? -1 : 1;
  return x->i < y->i ? -1 : (x->i > y->i);
}

/* Chen & Bhanu / PCL GeometricConsistencyGrouping: correspondences sorted by
 * descriptor distance (ties: input order); each not-yet-taken one seeds a
 * consensus set that admits, in the same order, every not-taken
 * correspondence whose model-side and scene-side distances to EVERY member
 * differ by at most gc_size; sets of at least gc_thresh members become
 * clusters and their members are taken.  Pose per cluster: least squares
 * model -> scene (FP64).  Returns the number of clusters. */
int orc_gc_group(const float* mk, const float* sk, const int32_t* cm, const int32_t* cs, const float* cd,
                 int nc, float gc_size, int gc_thresh, int max_clusters, int32_t* cluster_of,
                 double* poses16, int32_t* sizes) {
  dk_t* ord = (dk_t*)malloc(sizeof(dk_t) * (nc > 0 ? nc : 1));
  for (int i = 0; i < nc; ++i) {
    ord[i].d = cd[i];
    ord[i].i = i;
    cluster_of[i] = -1;
  }
  qsort(ord, (size_t)nc, sizeof(dk_t), dk_cmp);
  char* taken = (char*)calloc((size_t)nc + 1, 1);
  /* pass[b]: candidate ord[b] is consistent with the current seed — the
   * first member every candidate is tested against, computed for all
   * candidates in parallel; the in-order admission then tests the other
   * members only.  Same predicate, same order, same sets. */
  char* pass = (char*)malloc((size_t)nc + 1);
  int* set = (int*)malloc(sizeof(int) * (nc > 0 ? nc : 1));
  float* P = (float*)malloc(sizeof(float) * 4 * (nc > 0 ? nc : 1));
  float* Q = (float*)malloc(sizeof(float) * 4 * (nc > 0 ? nc : 1));
  int ncl = 0;
  /* clusters past max_clusters are not reported, and the walk that finds
   * the first max_clusters does not depend on later seeds: stop there */
  for (int a = 0; a < nc && ncl < max_clusters; ++a) {
    const int i = ord[a].i;
    if (taken[i]) continue;
    const float* mi = mk + 4 * cm[i];
    const float* si = sk + 4 * cs[i];
#pragma omp parallel for schedule(static, 4096)
    for (int b = 0; b < nc; ++b) {
      const int j = ord[b].i;
      const float dm = sqrtf(d2f(mi, mk + 4 * cm[j]));
      const float ds = sqrtf(d2f(si, sk + 4 * cs[j]));
      pass[b] = !(fabsf(dm - ds) > gc_size);
    }
    int ns = 0;
    set[ns++] = i;
    for (int b = 0; b < nc; ++b) {
      const int j = ord[b].i;
      if (j == i || taken[j] || !pass[b]) continue;
      int ok = 1;
      for (int s = 1; s < ns && ok; ++s) {
        const int m = set[s];
        const float dm = sqrtf(d2f(mk + 4 * cm[m], mk + 4 * cm[j]));
        const float ds = sqrtf(d2f(sk + 4 * cs[m], sk + 4 * cs[j]));
        if (fabsf(dm - ds) > gc_size) ok = 0;
      }
      if (ok) set[ns++] = j;
    }
    if (ns >= gc_thresh) {
      for (int s = 0; s < ns; ++s) {
        taken[set[s]] = 1;
        cluster_of[set[s]] = ncl;
      }
      for (int s = 0; s < ns; ++s) {
        memcpy(P + 4 * s, mk + 4 * cm[set[s]], 16);
        memcpy(Q + 4 * s, sk + 4 * cs[set[s]], 16);
      }
      orc_rigid_fit(P, Q, NULL, ns, poses16 + 16 * ncl);
      sizes[ncl] = ns;
      ++ncl;
    }
  }
  free(ord);
  free(taken);
  free(pass);
  free(set);
  free(P);
  free(Q);
  return ncl;
}
