// pose.cuh — the rotation of the closed-form rigid pose from a 3x3
// cross-covariance (Umeyama 1991, without scale): R maximises tr(R H) over
// SO(3), t = mq - R mp follows.  An FP32 start (Newton iteration on the polar
// condition from the identity, an FP32 one-sided Jacobi SVD when that does
// not converge) is polished in FP64 by a whole warp.
#pragma once
#include <math.h>

// ---------------------------------------------------------------------------
// Fast FP64 rotation for the GPU.  FP64 instructions are scarce on GB300 (a
// dependent FP64 op costs ~30 cycles), so the SVD runs in FP32 and one FP64
// Newton step then solves the optimality condition exactly:
//   R maximises tr(R H) over SO(3)  <=>  S = H R is symmetric.
// With R = R0 (I + W), W = [w]x, the antisymmetric part of H R0 W is
// [(tr(S) I - S) w]x / 2 to first order, so
//   w = -2 (tr(S) I - S)^-1 vex(asym(H R0)),   R = R0 (I + W + W^2 / 2).
// The FP32 start is accurate to ~1e-6 rad, so one step leaves ~1e-12.
// ---------------------------------------------------------------------------
#ifdef __CUDACC__
__device__ __forceinline__ void svd3_jacobi_f32(const float H[9], float U[9], float S[3], float V[9]) {
  float A[9];
  for (int i = 0; i < 9; ++i) A[i] = H[i];
  for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.f : 0.f;
  for (int sweep = 0; sweep < 10; ++sweep) {
    float off = 0.f;
#pragma unroll
    for (int pq = 0; pq < 3; ++pq) {
      const int p = pq == 2 ? 1 : 0;
      const int q = pq == 0 ? 1 : 2;
      float alpha = 0.f, beta = 0.f, gamma = 0.f;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        alpha += A[i * 3 + p] * A[i * 3 + p];
        beta += A[i * 3 + q] * A[i * 3 + q];
        gamma += A[i * 3 + p] * A[i * 3 + q];
      }
      const float nrm2 = alpha * beta;
      if (!(nrm2 > 0.f) || gamma * gamma <= 1e-14f * nrm2) continue;
      off = fmaxf(off, gamma * gamma / nrm2);
      const float zeta = (beta - alpha) / (2.f * gamma);
      const float t = copysignf(1.f, zeta) / (fabsf(zeta) + sqrtf(1.f + zeta * zeta));
      const float c = rsqrtf(1.f + t * t);
      const float s = c * t;
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float ap = A[i * 3 + p], aq = A[i * 3 + q];
        A[i * 3 + p] = c * ap - s * aq;
        A[i * 3 + q] = s * ap + c * aq;
        const float vp = V[i * 3 + p], vq = V[i * 3 + q];
        V[i * 3 + p] = c * vp - s * vq;
        V[i * 3 + q] = s * vp + c * vq;
      }
    }
    if (off < 1e-13f) break;
  }
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float n = sqrtf(A[j] * A[j] + A[3 + j] * A[3 + j] + A[6 + j] * A[6 + j]);
    S[j] = n;
    const float inv = n > 0.f ? 1.f / n : 0.f;
#pragma unroll
    for (int i = 0; i < 3; ++i) U[i * 3 + j] = A[i * 3 + j] * inv;
  }
  for (int j = 0; j < 3; ++j) {
    const int a = (j + 1) % 3, b = (j + 2) % 3;
    const float smax = fmaxf(fmaxf(S[0], S[1]), S[2]);
    if (S[j] <= 1e-6f * smax && S[a] > 0.f && S[b] > 0.f) {
      U[0 * 3 + j] = U[1 * 3 + a] * U[2 * 3 + b] - U[2 * 3 + a] * U[1 * 3 + b];
      U[1 * 3 + j] = U[2 * 3 + a] * U[0 * 3 + b] - U[0 * 3 + a] * U[2 * 3 + b];
      U[2 * 3 + j] = U[0 * 3 + a] * U[1 * 3 + b] - U[1 * 3 + a] * U[0 * 3 + b];
    }
  }
}

// One FP32 Newton step on R (in place) for the condition "Hf R symmetric";
// returns |w| (or +inf when the step is undefined).
__device__ __forceinline__ float newton_f32(const float Hf[9], float R[9]) {
  float Sm[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) Sm[i * 3 + k] = Hf[i * 3 + 0] * R[k] + Hf[i * 3 + 1] * R[3 + k] + Hf[i * 3 + 2] * R[6 + k];
  const float b0 = 0.5f * (Sm[7] - Sm[5]), b1 = 0.5f * (Sm[2] - Sm[6]), b2 = 0.5f * (Sm[3] - Sm[1]);
  const float s01 = 0.5f * (Sm[1] + Sm[3]), s02 = 0.5f * (Sm[2] + Sm[6]), s12 = 0.5f * (Sm[5] + Sm[7]);
  const float tr = Sm[0] + Sm[4] + Sm[8];
  const float a00 = tr - Sm[0], a11 = tr - Sm[4], a22 = tr - Sm[8];
  const float a01 = -s01, a02 = -s02, a12 = -s12;
  const float c00 = a11 * a22 - a12 * a12, c01 = a02 * a12 - a01 * a22, c02 = a01 * a12 - a02 * a11;
  const float c11 = a00 * a22 - a02 * a02, c12 = a01 * a02 - a00 * a12, c22 = a00 * a11 - a01 * a01;
  const float det = a00 * c00 + a01 * c01 + a02 * c02;
  // on the maximising branch A = tr(S) I - S is positive definite
  // (Sylvester: a00 > 0, leading 2x2 minor c22 > 0, det > 0)
  if (!(det > 1e-6f) || !(a00 > 0.f) || !(c22 > 0.f) || !(a11 > 0.f) || !(a22 > 0.f))
    return __int_as_float(0x7f800000);
  const float f = -2.f * __frcp_rn(det);
  const float w0 = f * (c00 * b0 + c01 * b1 + c02 * b2);
  const float w1 = f * (c01 * b0 + c11 * b1 + c12 * b2);
  const float w2 = f * (c02 * b0 + c12 * b1 + c22 * b2);
  const float W[9] = {0.f, -w2, w1, w2, 0.f, -w0, -w1, w0, 0.f};
  // exact exponential (Rodrigues): E = I + (sin t / t) W + ((1 - cos t) / t^2) W^2,
  // so R stays a rotation however large the step
  const float th2 = w0 * w0 + w1 * w1 + w2 * w2;
  float sa, sb;
  if (th2 > 1e-6f) {
    const float th = sqrtf(th2);
    float sn, cs;
    sincosf(th, &sn, &cs);
    sa = sn / th;
    sb = (1.f - cs) / th2;
  } else {
    sa = 1.f - th2 * (1.f / 6.f);
    sb = 0.5f - th2 * (1.f / 24.f);
  }
  float E[9], Rn[9];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k)
      E[i * 3 + k] = (i == k ? 1.f : 0.f) + sa * W[i * 3 + k] +
                     sb * (W[i * 3 + 0] * W[k] + W[i * 3 + 1] * W[3 + k] + W[i * 3 + 2] * W[6 + k]);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) Rn[i * 3 + k] = R[i * 3 + 0] * E[k] + R[i * 3 + 1] * E[3 + k] + R[i * 3 + 2] * E[6 + k];
#pragma unroll
  for (int i = 0; i < 9; ++i) R[i] = Rn[i];
  return sqrtf(w0 * w0 + w1 * w1 + w2 * w2);
}

// Umeyama rotation, FP32 start: Newton from the identity (where ICP
// increments live), the FP32 Jacobi SVD when that does not converge.  Writes
// the start to R0 and the scale applied to H to *sc_out; false (R0 = I) when
// H is zero or not finite.
__device__ __forceinline__ bool umeyama_start_f32(const double H[9], double R0[9], float* sc_out) {
  float Hf[9];
  float hmax = 0.f;
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    Hf[i] = (float)H[i];
    hmax = fmaxf(hmax, fabsf(Hf[i]));
  }
  if (!(hmax > 0.f) || !isfinite(hmax)) {
    for (int i = 0; i < 9; ++i) R0[i] = (i % 4 == 0) ? 1.0 : 0.0;
    *sc_out = 0.f;
    return false;
  }
  const float sc = 1.f / hmax;
  *sc_out = sc;
#pragma unroll
  for (int i = 0; i < 9; ++i) Hf[i] *= sc;
  float Rf[9] = {1.f, 0.f, 0.f, 0.f, 1.f, 0.f, 0.f, 0.f, 1.f};
  bool ok = false;
  for (int step = 0; step < 6; ++step) {
    const float wn = newton_f32(Hf, Rf);
    if (!(wn < (step == 0 ? 0.35f : 0.5f))) break;  // far from the identity, or undefined
    if (wn < 3e-6f) {
      ok = true;
      break;
    }
  }
  if (ok) {
#pragma unroll
    for (int i = 0; i < 9; ++i) R0[i] = (double)Rf[i];
  } else {
    float U[9], S[3], V[9];
    svd3_jacobi_f32(Hf, U, S, V);
    int jmin = 0;
    for (int j = 1; j < 3; ++j)
      if (S[j] < S[jmin]) jmin = j;
    // det(V U^T) = det(V) det(U)
    const float dv = V[0] * (V[4] * V[8] - V[5] * V[7]) - V[1] * (V[3] * V[8] - V[5] * V[6]) +
                     V[2] * (V[3] * V[7] - V[4] * V[6]);
    const float du = U[0] * (U[4] * U[8] - U[5] * U[7]) - U[1] * (U[3] * U[8] - U[5] * U[6]) +
                     U[2] * (U[3] * U[7] - U[4] * U[6]);
    const float d = dv * du < 0.f ? -1.f : 1.f;
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k) {
        float s = 0.f;
        for (int j = 0; j < 3; ++j) s += V[i * 3 + j] * (j == jmin ? d : 1.f) * U[k * 3 + j];
        R0[i * 3 + k] = (double)s;
      }
  }
  return true;
}

// Entry e of a row-major 3x3 held in registers, e the same or different in
// every lane (unrolled selects: no local memory).
__device__ __forceinline__ double pick9(const double M[9], int e) {
  double v = M[0];
#pragma unroll
  for (int q = 1; q < 9; ++q)
    if (e == q) v = M[q];
  return v;
}

// The same rotation computed by a whole warp: every lane passes the same H
// and gets the same R.  GB300 issues FP64 at a small fraction of the FP32
// rate and charges per warp instruction, not per active lane, so the FP64
// 3x3 products run distributed, lane e (0..8) computing entry e from
// operands fetched with shuffles, and only the scalar chain of each Newton
// step (on the gathered S) runs on every lane.  The FP32 start is computed
// by every lane alike, so every branch is warp-uniform.
__device__ __forceinline__ bool umeyama_rotation_warp(const double H[9], double R[9]) {
  double R0[9];
  float sc;
  if (!umeyama_start_f32(H, R0, &sc)) {
    for (int i = 0; i < 9; ++i) R[i] = R0[i];
    return false;
  }
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int e = lane < 9 ? lane : 8, ei = e / 3, ek = e % 3;
  double r0 = pick9(R0, e);  // R0 distributed: entry e in lane e
  {  // Newton-Schulz: R0 <- R0 (3I - R0^T R0) / 2
    const double g = (ei == ek ? 1.5 : 0.0) -
                     0.5 * (__shfl_sync(full, r0, ei) * __shfl_sync(full, r0, ek) +
                            __shfl_sync(full, r0, 3 + ei) * __shfl_sync(full, r0, 3 + ek) +
                            __shfl_sync(full, r0, 6 + ei) * __shfl_sync(full, r0, 6 + ek));
    r0 = __shfl_sync(full, r0, ei * 3 + 0) * __shfl_sync(full, g, 0 * 3 + ek) +
         __shfl_sync(full, r0, ei * 3 + 1) * __shfl_sync(full, g, 1 * 3 + ek) +
         __shfl_sync(full, r0, ei * 3 + 2) * __shfl_sync(full, g, 2 * 3 + ek);
  }
  const double inv = (double)sc;
  const double h0 = pick9(H, ei * 3 + 0), h1 = pick9(H, ei * 3 + 1), h2 = pick9(H, ei * 3 + 2);
#pragma unroll 1
  for (int step = 0; step < 3; ++step) {
    const double sm = (h0 * __shfl_sync(full, r0, 0 * 3 + ek) + h1 * __shfl_sync(full, r0, 1 * 3 + ek) +
                       h2 * __shfl_sync(full, r0, 2 * 3 + ek)) * inv;
    double Sm[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) Sm[q] = __shfl_sync(full, sm, q);
    const double b0 = 0.5 * (Sm[7] - Sm[5]), b1 = 0.5 * (Sm[2] - Sm[6]), b2 = 0.5 * (Sm[3] - Sm[1]);
    const double s01 = 0.5 * (Sm[1] + Sm[3]), s02 = 0.5 * (Sm[2] + Sm[6]), s12 = 0.5 * (Sm[5] + Sm[7]);
    const double tr = Sm[0] + Sm[4] + Sm[8];
    const double a00 = tr - Sm[0], a11 = tr - Sm[4], a22 = tr - Sm[8];
    const double a01 = -s01, a02 = -s02, a12 = -s12;
    const double c00 = a11 * a22 - a12 * a12, c01 = a02 * a12 - a01 * a22, c02 = a01 * a12 - a02 * a11;
    const double c11 = a00 * a22 - a02 * a02, c12 = a01 * a02 - a00 * a12, c22 = a00 * a11 - a01 * a01;
    const double det = a00 * c00 + a01 * c01 + a02 * c02;
    if (!(fabs(det) > 1e-12)) break;
    // 1/det from the FP32 reciprocal and two FP64 Newton steps (each doubles
    // the correct bits: 24 -> 48 -> 96, so within an ulp of the division
    // and far cheaper than it on GB300's FP64 pipe)
    double rd = (double)__frcp_rn((float)det);
    rd = rd * (2.0 - det * rd);
    rd = rd * (2.0 - det * rd);
    const double f = -2.0 * rd;
    const double w0 = f * (c00 * b0 + c01 * b1 + c02 * b2);
    const double w1 = f * (c01 * b0 + c11 * b1 + c12 * b2);
    const double w2 = f * (c02 * b0 + c12 * b1 + c22 * b2);
    const double W[9] = {0.0, -w2, w1, w2, 0.0, -w0, -w1, w0, 0.0};
    // E = I + W + W^2 / 2, entry e
    const double ee = (ei == ek ? 1.0 : 0.0) + pick9(W, e) +
                      0.5 * (pick9(W, ei * 3 + 0) * pick9(W, 0 * 3 + ek) + pick9(W, ei * 3 + 1) * pick9(W, 1 * 3 + ek) +
                             pick9(W, ei * 3 + 2) * pick9(W, 2 * 3 + ek));
    r0 = __shfl_sync(full, r0, ei * 3 + 0) * __shfl_sync(full, ee, 0 * 3 + ek) +
         __shfl_sync(full, r0, ei * 3 + 1) * __shfl_sync(full, ee, 1 * 3 + ek) +
         __shfl_sync(full, r0, ei * 3 + 2) * __shfl_sync(full, ee, 2 * 3 + ek);
    // converged when |w|^2 < 1e-13 det / max(c00, c11, c22) (the cofactors
    // are positive on the maximising branch), tested without a division
    if ((w0 * w0 + w1 * w1 + w2 * w2) * fmax(fmax(c00, c11), c22) < 1e-13 * det) break;
  }
#pragma unroll
  for (int q = 0; q < 9; ++q) R[q] = __shfl_sync(full, r0, q);
  return true;
}
#endif

