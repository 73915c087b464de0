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
      if (d < bd || (d == bd && j < bi)) {
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
  if (f < -1e8) f = -1e8;
  if (f > 1e8) f = 1e8;
  return (int)f;
}

static void cg_build(cgrid* g, const float* pts, int n, double h) {
  double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  for (int i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      if (pts[4 * i + a] < lo[a]) lo[a] = pts[4 * i + a];
      if (pts[4 * i + a] > hi[a]) hi[a] = pts[4 * i + a];
    }
  if (n == 0)
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
    for (int z = c[2] - k; z <= c[2] + k; ++z) {
      if (z < 0 || z >= g->n[2]) continue;
      for (int y = c[1] - k; y <= c[1] + k; ++y) {
        if (y < 0 || y >= g->n[1]) continue;
        int edge = (z == c[2] - k || z == c[2] + k || y == c[1] - k || y == c[1] + k);
        for (int x = c[0] - k; x <= c[0] + k; x += (edge || k == 0) ? 1 : 2 * k) {
          if (x < 0 || x >= g->n[0]) continue;
          int cell = (z * g->n[1] + y) * g->n[0] + x;
          for (int s = g->start[cell]; s < g->start[cell + 1]; ++s) {
            int j = g->order[s];
            float d = d2f(qf, g->pts + 4 * j);
            int last = T->k - 1;
            if (d > T->bd[last] || (d == T->bd[last] && j >= T->bi[last])) continue;
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

void orc_nn1_grid(const float* q, int nq, const float* t, int nt, float r2max, float cell, int32_t* idx,
                  float* d2) {
  cgrid g;
  cg_build(&g, t, nt, cell > 0 ? cell : (r2max < INFINITY ? 0.5 * sqrt(r2max) : -1));
#pragma omp parallel for schedule(dynamic, 256)
  for (int i = 0; i < nq; ++i) {
    float bd = r2max;
    int bi = INT_MAX;
    topk T = {1, &bd, &bi};
    if (nt > 0) cg_search(&g, q + 4 * i, &T);
    idx[i] = bi == INT_MAX ? -1 : bi;
    if (d2) d2[i] = bi == INT_MAX ? INFINITY : bd;
  }
  cg_free(&g);
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
      if (d > bd[last] || (d == bd[last] && j >= bi[last])) continue;
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
static int icp_step(const float* src, int ns, const float* tgt, int nt, float r2max, float cell, const double* P,
                    int32_t* corr, float* tmp, double* Pnext, double* dT, double* fitness) {
  orc_transform_f32(P, src, ns, tmp);
  float* d2 = (float*)malloc(sizeof(float) * (ns > 0 ? ns : 1));
  orc_nn1_grid(tmp, ns, tgt, nt, r2max, cell, corr, d2);
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

void orc_icp(const float* src, int ns, const float* tgt, int nt, int max_it, float max_dist, double eps_t,
             double eps_r, const double* init, orc_icp_out* out, double* trace_pose, int32_t* trace_corr) {
  const float r2max = (max_dist > 0 && max_dist < 1e18f) ? max_dist * max_dist : INFINITY;
  const float cell = (max_dist > 0 && max_dist < 1e18f) ? 0.5f * max_dist : -1.f;
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
    int m = icp_step(src, ns, tgt, nt, r2max, cell, P, corr, tmp, Pn, dT, &fit);
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

void orc_icp_replay(const float* src, int ns, const float* tgt, int nt, float max_dist, const double* poses_in,
                    int iters, int32_t* corr_out, double* poses_out, int32_t* ncorr_out) {
  const float r2max = (max_dist > 0 && max_dist < 1e18f) ? max_dist * max_dist : INFINITY;
  const float cell = (max_dist > 0 && max_dist < 1e18f) ? 0.5f * max_dist : -1.f;
  float* tmp = (float*)malloc(sizeof(float) * 4 * (ns > 0 ? ns : 1));
  memcpy(poses_out, poses_in, 16 * sizeof(double));
  for (int it = 0; it < iters; ++it) {
    double dT[16], fit = 0;
    int m = icp_step(src, ns, tgt, nt, r2max, cell, poses_in + 16 * (size_t)it, corr_out + (size_t)it * ns, tmp,
                     poses_out + 16 * (size_t)(it + 1), dT, &fit);
    if (ncorr_out) ncorr_out[it] = m;
  }
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
