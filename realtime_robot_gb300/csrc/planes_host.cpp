// planes_host.cpp — the scalar steps of rtr_plane_segment / rtr_vector3d
// that run on the host between kernels (a few per extracted plane): the
// RANSAC stop rule, the 3x3 eigen-solve of the refit, the plane's 2-D basis,
// the horizontal / vertical classes and the hull's area and perimeter.
// Compiled with -ffp-contract=off: every operation is rounded as written,
// so the results equal the CPU oracle's (oracle/planes.c), which restates
// the same steps.
#include <float.h>
#include <math.h>
#include <string.h>

#include "planes_host.h"

namespace rtr {

int plane_ransac_walk(const int* valid, const int* count, int n_slots, int m, int max_iterations, PlaneWalk* w) {
  const double log_p = log(1.0 - 0.99);
  for (; w->slot < n_slots; ++w->slot) {
    if (w->done) return 1;
    if (!((double)w->iterations < w->k) || w->skipped >= 10 * max_iterations) {
      w->done = 1;
      return 1;
    }
    const int s = w->slot;
    if (!valid[s]) {
      ++w->skipped;
      continue;
    }
    if (count[s] > w->best_cnt) {
      w->best_cnt = count[s];
      w->best = w->base + s;
      const double f = (double)w->best_cnt / (double)m;
      double pno = 1.0 - f * f * f;
      if (pno < DBL_EPSILON) pno = DBL_EPSILON;
      if (pno > 1.0 - DBL_EPSILON) pno = 1.0 - DBL_EPSILON;
      w->k = log_p / log(pno);
    }
    if (++w->iterations >= max_iterations) {
      w->done = 1;
      return 1;
    }
  }
  return w->done;
}

// cyclic Jacobi on a symmetric 3x3 (FP64): eigenvalues ascending, vectors in
// the columns of V
static void jacobi3(const double* A0, double* w, double* V) {
  double A[9];
  memcpy(A, A0, sizeof(A));
  for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
  static const int P[3] = {0, 0, 1}, Q[3] = {1, 2, 2};
  for (int sweep = 0; sweep < 50; ++sweep) {
    const double off = (A[1] * A[1] + A[2] * A[2]) + A[5] * A[5];
    if (!(off > 0.0)) break;
    for (int r = 0; r < 3; ++r) {
      const int p = P[r], q = Q[r];
      const double apq = A[p * 3 + q];
      if (apq == 0.0) continue;
      const double theta = (A[q * 3 + q] - A[p * 3 + p]) / (2.0 * apq);
      const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
      const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
      for (int k = 0; k < 3; ++k) {
        const double akp = A[k * 3 + p], akq = A[k * 3 + q];
        A[k * 3 + p] = c * akp - s * akq;
        A[k * 3 + q] = s * akp + c * akq;
      }
      for (int k = 0; k < 3; ++k) {
        const double apk = A[p * 3 + k], aqk = A[q * 3 + k];
        A[p * 3 + k] = c * apk - s * aqk;
        A[q * 3 + k] = s * apk + c * aqk;
      }
      for (int k = 0; k < 3; ++k) {
        const double vkp = V[k * 3 + p], vkq = V[k * 3 + q];
        V[k * 3 + p] = c * vkp - s * vkq;
        V[k * 3 + q] = s * vkp + c * vkq;
      }
    }
  }
  int o[3] = {0, 1, 2};
  for (int i = 1; i < 3; ++i)
    for (int j = i; j > 0 && A[o[j] * 4] < A[o[j - 1] * 4]; --j) {
      const int t = o[j];
      o[j] = o[j - 1];
      o[j - 1] = t;
    }
  double W[9];
  for (int j = 0; j < 3; ++j) {
    w[j] = A[o[j] * 4];
    for (int k = 0; k < 3; ++k) W[k * 3 + j] = V[k * 3 + o[j]];
  }
  memcpy(V, W, sizeof(W));
}

void plane_refit(const double* sums9, int n, const float* c_in, float* c_out, int* flat) {
  memcpy(c_out, c_in, 4 * sizeof(float));
  *flat = 1;
  if (n < 3) return;
  const double inv = 1.0 / (double)n;
  const double mx = sums9[0] * inv, my = sums9[1] * inv, mz = sums9[2] * inv;
  double C[9];
  C[0] = sums9[3] * inv - mx * mx;
  C[1] = sums9[4] * inv - mx * my;
  C[2] = sums9[5] * inv - mx * mz;
  C[4] = sums9[6] * inv - my * my;
  C[5] = sums9[7] * inv - my * mz;
  C[8] = sums9[8] * inv - mz * mz;
  C[3] = C[1];
  C[6] = C[2];
  C[7] = C[5];
  double w[3], V[9];
  jacobi3(C, w, V);
  double nx = V[0], ny = V[3], nz = V[6];
  const double L = sqrt((nx * nx + ny * ny) + nz * nz);
  if (!(L > 0.0)) return;
  nx = nx / L;
  ny = ny / L;
  nz = nz / L;
  c_out[0] = (float)nx;
  c_out[1] = (float)ny;
  c_out[2] = (float)nz;
  c_out[3] = (float)(-((nx * mx + ny * my) + nz * mz));
  *flat = !(w[2] > 0.0) || (w[0] / w[2] < 1e-3);
}

void plane_basis(const float* c, float* e1, float* e2) {
  const float ax = fabsf(c[0]), ay = fabsf(c[1]), az = fabsf(c[2]);
  const int k = (ax <= ay && ax <= az) ? 0 : (ay <= az ? 1 : 2);
  const float a[3] = {k == 0 ? 1.f : 0.f, k == 1 ? 1.f : 0.f, k == 2 ? 1.f : 0.f};
  float x = c[1] * a[2] - c[2] * a[1], y = c[2] * a[0] - c[0] * a[2], z = c[0] * a[1] - c[1] * a[0];
  const float L = sqrtf((x * x + y * y) + z * z);
  x = x / L;
  y = y / L;
  z = z / L;
  e1[0] = x;
  e1[1] = y;
  e1[2] = z;
  e2[0] = c[1] * z - c[2] * y;
  e2[1] = c[2] * x - c[0] * z;
  e2[2] = c[0] * y - c[1] * x;
}

int plane_class(const float* c) {
  const float b = (c[0] * c[0] + c[1] * c[1]) + c[2] * c[2];
  const double cc = sqrt((double)b);
  const double e = (double)c[2] / cc;
  const double angle = acos(e);
  if ((angle > 2.9670597 && angle < 3.1415926) || (angle > 0 && angle < 0.1745329)) return 0;
  if (angle > 1.3962634 && angle < 1.7453292) return 1;
  return -1;
}

void hull_measure(const float* uv, int h, double* area, double* perim) {
  double A = 0.0, L = 0.0;
  for (int i = 0; i < h; ++i) {
    const int j = (i + 1) % h;
    const float au = uv[2 * i], av = uv[2 * i + 1], bu = uv[2 * j], bv = uv[2 * j + 1];
    A += (double)au * (double)bv - (double)bu * (double)av;
    const double du = (double)bu - (double)au, dv = (double)bv - (double)av;
    L += sqrt(du * du + dv * dv);
  }
  *area = h >= 3 ? 0.5 * fabs(A) : 0.0;
  *perim = h >= 2 ? L : 0.0;
}

}  // namespace rtr
