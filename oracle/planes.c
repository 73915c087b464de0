/*
 * planes.c — CPU restatement of the reference's plane segmentation and
 * plane-area descriptor (test infrastructure: the checker of the GPU path).
 *
 *   ModelPoint::getArea   model_point.h:170-245
 *   ScanPoint::get_Area   scan_point.h:117-188
 *   is_h_plane/is_v_plane model_point.h:48-79
 *   KeyPoint::get_Vector3D, getDistance   key_point.h:38-43, 87-111
 *
 * The reference runs these through PCL 1.8.0 (SACSegmentation with RANSAC,
 * ExtractIndices, ConvexHull over Qhull), which is absent here: parity with
 * PCL is unpinned.  The steps below restate the published methods with
 * conventions of our own, and the GPU path (realtime_robot_gb300/csrc/
 * planes.cu, planes_host.cpp) follows them bit for bit:
 *
 *  - the points with a non-finite coordinate are left out from the start;
 *  - a round runs while more than remain_frac of the points remain;
 *  - RANSAC (Fischler & Bolles 1981) with the adaptive sample count of
 *    Hartley & Zisserman: sample slot s of round r draws three positions
 *    in the remaining list from a SplitMix64 hash of (seed, r, s, k); a
 *    sample with a repeated position or collinear points is skipped
 *    (counted toward 10 x max_iterations skips); a valid sample's plane is
 *    the normalised cross product (float); its score is the number of
 *    remaining points within `distance` (float |n.p + d|); the first best
 *    sample wins; after every new best the needed count becomes
 *    log(1 - 0.99) / log(1 - w^3) (w = inlier fraction); at most
 *    max_iterations valid samples;
 *  - the plane is refitted by least squares to the best sample's inliers:
 *    FP64 sums in a fixed order (1024 strided partial sums, then a pairwise
 *    tree), the covariance's smallest eigenvector (cyclic Jacobi, FP64),
 *    rounded to float; the inliers are then selected again with the refitted
 *    plane; no inlier ends the segmentation, as in the reference;
 *  - the surface's area is the area of the 2-D convex hull (Andrew's
 *    monotone chain, exact orientation tests) of the inliers projected
 *    (float) onto the plane; its perimeter is reported too (for a hull
 *    Qhull treats as two-dimensional, PCL's getTotalArea reports Qhull's
 *    "area", which is that perimeter);
 *  - horizontal / vertical as is_h_plane / is_v_plane; kept when one of the
 *    two and area >= min_area (the reference's surface list);
 *  - the inliers leave the remaining list, whose order is kept.
 *
 * Compile with -ffp-contract=off (oracle/Makefile).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define PLANE_PARTIALS 1024

static uint64_t pl_mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static int pl_pick(uint64_t seed, int round, int slot, int k, int m) {
  const uint64_t key = seed ^ ((uint64_t)round << 48) ^ ((uint64_t)slot << 16) ^ (uint64_t)k;
  return (int)(pl_mix(key) % (uint64_t)m);
}

/* plane through three points (float); 0 when degenerate */
static int pl_from3(const float* p0, const float* p1, const float* p2, float* c) {
  const float ax = p1[0] - p0[0], ay = p1[1] - p0[1], az = p1[2] - p0[2];
  const float bx = p2[0] - p0[0], by = p2[1] - p0[1], bz = p2[2] - p0[2];
  const float t0 = ay * bz, t1 = az * by, t2 = az * bx, t3 = ax * bz, t4 = ax * by, t5 = ay * bx;
  float nx = t0 - t1, ny = t2 - t3, nz = t4 - t5;
  const float l2 = (nx * nx + ny * ny) + nz * nz;
  if (!(l2 > 0.f) || !(l2 < INFINITY)) return 0;
  const float L = sqrtf(l2);
  nx = nx / L;
  ny = ny / L;
  nz = nz / L;
  c[0] = nx;
  c[1] = ny;
  c[2] = nz;
  c[3] = -((nx * p0[0] + ny * p0[1]) + nz * p0[2]);
  return 1;
}

static int pl_within(const float* c, const float* p, float thr) {
  const float s = ((c[0] * p[0] + c[1] * p[1]) + c[2] * p[2]) + c[3];
  return fabsf(s) <= thr;
}

/* cyclic Jacobi on a symmetric 3x3 (FP64), eigenvalues ascending, vectors in
 * the columns of V */
static void pl_jacobi(const double* A0, double* w, double* V) {
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
      for (int k = 0; k < 3; ++k) {  /* A <- A J (columns p, q) */
        const double akp = A[k * 3 + p], akq = A[k * 3 + q];
        A[k * 3 + p] = c * akp - s * akq;
        A[k * 3 + q] = s * akp + c * akq;
      }
      for (int k = 0; k < 3; ++k) {  /* A <- J^T A (rows p, q) */
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

/* least-squares plane of the points within thr of c (over rem[0..m)), FP64
 * sums in the fixed strided order; writes the refitted float plane to out
 * and returns the number of points summed; *flat = smallest / largest
 * covariance eigenvalue below 1e-3 */
static int pl_refit(const float* pts, const int* rem, int m, const float* c, float thr, float* out, int* flat) {
  double part[PLANE_PARTIALS][9];
  int cnt[PLANE_PARTIALS];
  for (int t = 0; t < PLANE_PARTIALS; ++t) {
    for (int k = 0; k < 9; ++k) part[t][k] = 0.0;
    cnt[t] = 0;
    for (int j = t; j < m; j += PLANE_PARTIALS) {
      const float* p = pts + 4 * (size_t)rem[j];
      if (!pl_within(c, p, thr)) continue;
      const double x = p[0], y = p[1], z = p[2];
      part[t][0] += x;
      part[t][1] += y;
      part[t][2] += z;
      part[t][3] += x * x;
      part[t][4] += x * y;
      part[t][5] += x * z;
      part[t][6] += y * y;
      part[t][7] += y * z;
      part[t][8] += z * z;
      ++cnt[t];
    }
  }
  for (int width = PLANE_PARTIALS / 2; width >= 1; width /= 2)
    for (int t = 0; t < width; ++t) {
      for (int k = 0; k < 9; ++k) part[t][k] += part[t + width][k];
      cnt[t] += cnt[t + width];
    }
  const int n = cnt[0];
  memcpy(out, c, 4 * sizeof(float));
  *flat = 1;
  if (n < 3) return n;
  const double inv = 1.0 / (double)n;
  const double mx = part[0][0] * inv, my = part[0][1] * inv, mz = part[0][2] * inv;
  double C[9];
  C[0] = part[0][3] * inv - mx * mx;
  C[1] = part[0][4] * inv - mx * my;
  C[2] = part[0][5] * inv - mx * mz;
  C[4] = part[0][6] * inv - my * my;
  C[5] = part[0][7] * inv - my * mz;
  C[8] = part[0][8] * inv - mz * mz;
  C[3] = C[1];
  C[6] = C[2];
  C[7] = C[5];
  double w[3], V[9];
  pl_jacobi(C, w, V);
  double nx = V[0], ny = V[3], nz = V[6];
  const double L = sqrt((nx * nx + ny * ny) + nz * nz);
  if (!(L > 0.0)) return n;
  nx = nx / L;
  ny = ny / L;
  nz = nz / L;
  out[0] = (float)nx;
  out[1] = (float)ny;
  out[2] = (float)nz;
  out[3] = (float)(-((nx * mx + ny * my) + nz * mz));
  *flat = !(w[2] > 0.0) || (w[0] / w[2] < 1e-3);
  return n;
}

typedef struct {
  float u, v;
} pl_uv;

static int pl_uv_cmp(const void* a, const void* b) {
  const pl_uv* x = (const pl_uv*)a;
  const pl_uv* y = (const pl_uv*)b;
  if (x->u != y->u) return x->u < y->u ? -1 : 1;
  if (x->v != y->v) return x->v < y->v ? -1 : 1;
  return 0;
}

static double pl_cross(pl_uv o, pl_uv a, pl_uv b) {
  const double ax = (double)a.u - (double)o.u, ay = (double)a.v - (double)o.v;
  const double bx = (double)b.u - (double)o.u, by = (double)b.v - (double)o.v;
  return ax * by - ay * bx;
}

/* the plane's 2-D basis (float): e1 across the coordinate axis least
 * aligned with the normal, e2 = n x e1; a point projects to (p.e1, p.e2) */
void orc_plane_basis(const float* c, float* e1, float* e2) {
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

/* hull of the projected points: vertex count, area and perimeter */
static int pl_hull(pl_uv* P, int n, pl_uv* H, double* area, double* perim) {
  *area = 0.0;
  *perim = 0.0;
  if (n == 0) return 0;
  qsort(P, (size_t)n, sizeof(pl_uv), pl_uv_cmp);
  int h = 0;
  for (int i = 0; i < n; ++i) {
    while (h >= 2 && pl_cross(H[h - 2], H[h - 1], P[i]) <= 0.0) --h;
    H[h++] = P[i];
  }
  for (int i = n - 2, lo = h + 1; i >= 0; --i) {
    while (h >= lo && pl_cross(H[h - 2], H[h - 1], P[i]) <= 0.0) --h;
    H[h++] = P[i];
  }
  if (h > 1) --h; /* the last point repeats the first */
  orc_hull_measure(H, h, area, perim);
  return h;
}

void orc_hull_measure(const void* Hv, int h, double* area, double* perim) {
  const pl_uv* H = (const pl_uv*)Hv;
  double A = 0.0, L = 0.0;
  for (int i = 0; i < h; ++i) {
    const pl_uv a = H[i], b = H[(i + 1) % h];
    A += (double)a.u * (double)b.v - (double)b.u * (double)a.v;
    const double du = (double)b.u - (double)a.u, dv = (double)b.v - (double)a.v;
    L += sqrt(du * du + dv * dv);
  }
  *area = h >= 3 ? 0.5 * fabs(A) : 0.0;
  *perim = h >= 2 ? L : 0.0;
}

/* is_h_plane / is_v_plane (model_point.h:48-79): the angle between the
 * plane's normal and z, from float products and sums as the reference
 * computes them */
int orc_plane_class(const float* c) {
  const float b = (c[0] * c[0] + c[1] * c[1]) + c[2] * c[2];
  const double cc = sqrt((double)b);
  const double e = (double)c[2] / cc;
  const double angle = acos(e);
  if ((angle > 2.9670597 && angle < 3.1415926) || (angle > 0 && angle < 0.1745329)) return 0; /* horizontal */
  if (angle > 1.3962634 && angle < 1.7453292) return 1;                                       /* vertical */
  return -1;
}

int orc_plane_segment(const float* pts, int n, int max_iterations, float distance, double remain_frac,
                      double min_area, uint64_t seed, int max_planes, orc_surface* out, int* n_total) {
  int* rem = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  int* keep = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  pl_uv* P = (pl_uv*)malloc(sizeof(pl_uv) * (size_t)(n > 0 ? n : 1));
  pl_uv* H = (pl_uv*)malloc(sizeof(pl_uv) * (size_t)(2 * n + 2));
  int m = 0;
  for (int i = 0; i < n; ++i) {
    const float* p = pts + 4 * (size_t)i;
    if (isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2])) rem[m++] = i;
  }
  const int nr_points = m;
  const int n_slots = 11 * max_iterations;
  const double log_p = log(1.0 - 0.99);
  int np = 0, round = 0;
  while ((double)m > remain_frac * (double)nr_points && m >= 3) {
    /* RANSAC: samples in slot order, scored when the walk reaches them */
    int iterations = 0, skipped = 0, best_cnt = -1;
    float best[4] = {0.f, 0.f, 0.f, 0.f};
    double k = 1.0;
    for (int s = 0; s < n_slots && (double)iterations < k && skipped < 10 * max_iterations; ++s) {
      const int i0 = pl_pick(seed, round, s, 0, m), i1 = pl_pick(seed, round, s, 1, m),
                i2 = pl_pick(seed, round, s, 2, m);
      float cs[4];
      if (i0 == i1 || i0 == i2 || i1 == i2 ||
          !pl_from3(pts + 4 * (size_t)rem[i0], pts + 4 * (size_t)rem[i1], pts + 4 * (size_t)rem[i2], cs)) {
        ++skipped;
        continue;
      }
      int cnt = 0;
#pragma omp parallel for reduction(+ : cnt) schedule(static)
      for (int j = 0; j < m; ++j) cnt += pl_within(cs, pts + 4 * (size_t)rem[j], distance);
      if (cnt > best_cnt) {
        best_cnt = cnt;
        memcpy(best, cs, sizeof(cs));
        const double w = (double)best_cnt / (double)m;
        double pno = 1.0 - w * w * w;
        if (pno < DBL_EPSILON) pno = DBL_EPSILON;
        if (pno > 1.0 - DBL_EPSILON) pno = 1.0 - DBL_EPSILON;
        k = log_p / log(pno);
      }
      if (++iterations >= max_iterations) break;
    }
    if (best_cnt < 0) break;
    float c[4];
    int flat = 1;
    pl_refit(pts, rem, m, best, distance, c, &flat);
    int ni = 0, nk = 0;
    float e1[3], e2[3];
    orc_plane_basis(c, e1, e2);
    for (int j = 0; j < m; ++j) {
      const float* p = pts + 4 * (size_t)rem[j];
      if (pl_within(c, p, distance)) {
        const float u = (p[0] * e1[0] + p[1] * e1[1]) + p[2] * e1[2];
        const float v = (p[0] * e2[0] + p[1] * e2[1]) + p[2] * e2[2];
        P[ni].u = u + 0.f; /* -0 becomes +0 */
        P[ni].v = v + 0.f;
        ++ni;
      } else {
        keep[nk++] = rem[j];
      }
    }
    if (ni == 0) break;
    double area = 0.0, perim = 0.0;
    const int hv = pl_hull(P, ni, H, &area, &perim);
    if (np < max_planes) {
      orc_surface* S = out + np;
      S->area = area;
      S->perimeter = perim;
      memcpy(S->coeffs, c, sizeof(c));
      S->n_inliers = ni;
      S->hull_vertices = hv;
      S->flat = flat;
      const int cls = orc_plane_class(c);
      S->is_vertical = cls;
      S->kept = cls >= 0 && area >= min_area;
    }
    ++np;
    memcpy(rem, keep, sizeof(int) * (size_t)nk);
    m = nk;
    ++round;
  }
  if (n_total) *n_total = np;
  free(rem);
  free(keep);
  free(P);
  free(H);
  return np < max_planes ? np : max_planes;
}

/* KeyPoint::get_Vector3D (key_point.h:87-111) over the kept surfaces in list
 * order: the first horizontal one within 5 cm gives [0], the first two
 * vertical ones within 2 cm give [1] and [2] (sorted descending); defaults
 * 0.16.  The point-plane distance as getDistance computes it: float
 * expressions, the norm's sqrt of a float sum, divided in double. */
void orc_vector3d(const float* keys, int nk, const orc_surface* s, int ns, double* v3) {
  for (int k = 0; k < nk; ++k) {
    const float* p = keys + 4 * (size_t)k;
    double* v = v3 + 3 * (size_t)k;
    v[0] = v[1] = v[2] = 0.16;
    int vertical = 0, horizontal = 0;
    for (int i = 0; i < ns; ++i) {
      if (!s[i].kept) continue;
      const float* c = s[i].coeffs;
      const double d = (double)sqrtf((c[0] * c[0] + c[1] * c[1]) + c[2] * c[2]);
      const double dist = (double)fabsf(((c[0] * p[0] + c[1] * p[1]) + c[2] * p[2]) + c[3]) / d;
      if (s[i].is_vertical == 0 && horizontal == 0 && dist <= 0.05) {
        v[0] = s[i].area;
        ++horizontal;
      } else if (s[i].is_vertical == 1 && vertical <= 1 && dist <= 0.02) {
        v[1 + vertical] = s[i].area;
        ++vertical;
      }
    }
    if (v[1] < v[2]) {
      const double t = v[2];
      v[2] = v[1];
      v[1] = t;
    }
  }
}
