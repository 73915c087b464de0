// pose.cuh — FP64 closed-form rigid pose from a 3x3 cross-covariance
// (Umeyama 1991, without scale): H = sum (p - mp)(q - mq)^T = U S V^T,
// R = V diag(1, 1, det(V U^T)) U^T, t = mq - R mp.  The SVD is a one-sided
// Jacobi iteration on H (Hestenes): rotate column pairs of A = H V until they
// are orthogonal; then S = column norms, U = normalised columns.
#pragma once
#include <math.h>

#ifdef __CUDACC__
#define RTR_HD __host__ __device__ __forceinline__
#else
#define RTR_HD inline
#endif

RTR_HD void svd3_jacobi(const double H[9], double U[9], double S[3], double V[9]) {
  double A[9];
  for (int i = 0; i < 9; ++i) A[i] = H[i];
  for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 12; ++sweep) {
    double off = 0.0;
    for (int pq = 0; pq < 3; ++pq) {
      const int p = pq == 2 ? 1 : 0;
      const int q = pq == 0 ? 1 : 2;
      double alpha = 0, beta = 0, gamma = 0;
      for (int i = 0; i < 3; ++i) {
        alpha += A[i * 3 + p] * A[i * 3 + p];
        beta += A[i * 3 + q] * A[i * 3 + q];
        gamma += A[i * 3 + p] * A[i * 3 + q];
      }
      const double nrm = sqrt(alpha * beta);
      if (nrm == 0.0 || fabs(gamma) <= 1e-15 * nrm) continue;
      const double r = fabs(gamma) / nrm;
      off = r > off ? r : off;
      const double zeta = (beta - alpha) / (2.0 * gamma);
      const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
      const double c = 1.0 / sqrt(1.0 + t * t);
      const double s = c * t;
      for (int i = 0; i < 3; ++i) {
        const double ap = A[i * 3 + p], aq = A[i * 3 + q];
        A[i * 3 + p] = c * ap - s * aq;
        A[i * 3 + q] = s * ap + c * aq;
        const double vp = V[i * 3 + p], vq = V[i * 3 + q];
        V[i * 3 + p] = c * vp - s * vq;
        V[i * 3 + q] = s * vp + c * vq;
      }
    }
    if (off < 1e-15) break;
  }
  for (int j = 0; j < 3; ++j) {
    double n = 0;
    for (int i = 0; i < 3; ++i) n += A[i * 3 + j] * A[i * 3 + j];
    n = sqrt(n);
    S[j] = n;
    for (int i = 0; i < 3; ++i) U[i * 3 + j] = n > 0 ? A[i * 3 + j] / n : 0.0;
  }
  // complete U where a singular value vanished: column = cross of the other two
  for (int j = 0; j < 3; ++j) {
    const int a = (j + 1) % 3, b = (j + 2) % 3;
    const double smax = fmax(fmax(S[0], S[1]), S[2]);
    if (S[j] <= 1e-13 * smax && S[a] > 0 && S[b] > 0) {
      U[0 * 3 + j] = U[1 * 3 + a] * U[2 * 3 + b] - U[2 * 3 + a] * U[1 * 3 + b];
      U[1 * 3 + j] = U[2 * 3 + a] * U[0 * 3 + b] - U[0 * 3 + a] * U[2 * 3 + b];
      U[2 * 3 + j] = U[0 * 3 + a] * U[1 * 3 + b] - U[1 * 3 + a] * U[0 * 3 + b];
    }
  }
}

RTR_HD double det3(const double M[9]) {
  return M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) +
         M[2] * (M[3] * M[7] - M[4] * M[6]);
}

// R (3x3 row-major) from H; returns false when H is (numerically) zero.
RTR_HD bool umeyama_rotation(const double H[9], double R[9]) {
  double U[9], S[3], V[9];
  svd3_jacobi(H, U, S, V);
  if (!(S[0] + S[1] + S[2] > 0)) {
    for (int i = 0; i < 9; ++i) R[i] = (i % 4 == 0) ? 1.0 : 0.0;
    return false;
  }
  // D = diag(1,1,d) applied to the column of the smallest singular value
  int jmin = 0;
  for (int j = 1; j < 3; ++j)
    if (S[j] < S[jmin]) jmin = j;
  double VUt[9];
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) {
      double s = 0;
      for (int j = 0; j < 3; ++j) s += V[i * 3 + j] * U[k * 3 + j];
      VUt[i * 3 + k] = s;
    }
  const double d = det3(VUt) < 0 ? -1.0 : 1.0;
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) {
      double s = 0;
      for (int j = 0; j < 3; ++j) s += V[i * 3 + j] * (j == jmin ? d : 1.0) * U[k * 3 + j];
      R[i * 3 + k] = s;
    }
  return true;
}

// C = A * B for row-major 4x4.
RTR_HD void mat4_mul(const double A[16], const double B[16], double C[16]) {
  double T[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double s = 0;
      for (int k = 0; k < 4; ++k) s += A[i * 4 + k] * B[k * 4 + j];
      T[i * 4 + j] = s;
    }
  for (int i = 0; i < 16; ++i) C[i] = T[i];
}
