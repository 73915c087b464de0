// eig3.cuh — symmetric 3x3 eigen-decomposition (cyclic Jacobi, FP32) with
// every operation a separately rounded IEEE op, in a fixed order.  The CPU
// oracle runs the same sequence, so normals and curvatures agree bit for bit.
// Eigenvalues ascending (stable on ties), eigenvectors in the columns of V.
#pragma once
#include "common.cuh"

#ifdef __CUDACC__
__device__ __forceinline__ void eig3_exact(const float* A9, float* w, float* V) {
  float a[3][3], v[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      a[i][j] = A9[i * 3 + j];
      v[i][j] = (i == j) ? 1.f : 0.f;
    }
#pragma unroll 1
  for (int sweep = 0; sweep < 16; ++sweep) {
    const float o01 = __fmul_rn(a[0][1], a[0][1]), o02 = __fmul_rn(a[0][2], a[0][2]),
                o12 = __fmul_rn(a[1][2], a[1][2]);
    const float off = __fadd_rn(__fadd_rn(o01, o02), o12);
    const float d0 = __fmul_rn(a[0][0], a[0][0]), d1 = __fmul_rn(a[1][1], a[1][1]),
                d2 = __fmul_rn(a[2][2], a[2][2]);
    const float dsum = __fadd_rn(__fadd_rn(d0, d1), d2);
    if (!(off > __fmul_rn(1e-12f, dsum))) break;
#pragma unroll
    for (int pq = 0; pq < 3; ++pq) {
      const int p = pq == 2 ? 1 : 0, q = pq == 0 ? 1 : 2;
      const float apq = a[p][q];
      if (apq == 0.f) continue;
      const float num = __fsub_rn(a[q][q], a[p][p]);
      const float den = __fmul_rn(2.f, apq);
      const float theta = __fdiv_rn(num, den);
      const float th2 = __fmul_rn(theta, theta);
      const float rt = __fsqrt_rn(__fadd_rn(th2, 1.f));
      const float at = __fadd_rn(fabsf(theta), rt);
      float t = __fdiv_rn(1.f, at);
      if (theta < 0.f) t = -t;
      const float t2 = __fmul_rn(t, t);
      const float c = __fdiv_rn(1.f, __fsqrt_rn(__fadd_rn(t2, 1.f)));
      const float s = __fmul_rn(t, c);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float akp = a[k][p], akq = a[k][q];
        a[k][p] = __fsub_rn(__fmul_rn(c, akp), __fmul_rn(s, akq));
        a[k][q] = __fadd_rn(__fmul_rn(s, akp), __fmul_rn(c, akq));
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float apk = a[p][k], aqk = a[q][k];
        a[p][k] = __fsub_rn(__fmul_rn(c, apk), __fmul_rn(s, aqk));
        a[q][k] = __fadd_rn(__fmul_rn(s, apk), __fmul_rn(c, aqk));
      }
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float vkp = v[k][p], vkq = v[k][q];
        v[k][p] = __fsub_rn(__fmul_rn(c, vkp), __fmul_rn(s, vkq));
        v[k][q] = __fadd_rn(__fmul_rn(s, vkp), __fmul_rn(c, vkq));
      }
    }
  }
  // stable ascending order of the diagonal (3-element insertion sort)
  const float e0 = a[0][0], e1 = a[1][1], e2 = a[2][2];
  int o0 = 0, o1 = 1, o2 = 2;
  float f0 = e0, f1 = e1, f2 = e2;
  if (f0 > f1) { float t = f0; f0 = f1; f1 = t; int u = o0; o0 = o1; o1 = u; }
  if (f1 > f2) {
    float t = f1; f1 = f2; f2 = t; int u = o1; o1 = o2; o2 = u;
    if (f0 > f1) { float t2 = f0; f0 = f1; f1 = t2; int u2 = o0; o0 = o1; o1 = u2; }
  }
  w[0] = f0;
  w[1] = f1;
  w[2] = f2;
  const int ord[3] = {o0, o1, o2};
#pragma unroll
  for (int j = 0; j < 3; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) V[i * 3 + j] = ord[j] == 0 ? v[i][0] : (ord[j] == 1 ? v[i][1] : v[i][2]);
}
#endif
