/*
 * refmatch.c — CPU restatement of the reference's own descriptor route
 * (test infrastructure: the checker of librtr's rtr_ref_* entry points and
 * their timed CPU baseline; never linked into librtr.so):
 *
 *   KeyPoint::getOccupiedGrid  key_point.h:112-161  -> orc_ref_occupancy
 *   KeyPoint::get_TSDF         key_point.h:251-334  -> orc_ref_tdf
 *   get_Distance               matching.h:122-222   -> orc_ref_distance
 *   match_by_height/area/occupied + the all-pairs loop
 *                              function.h:158-178, RealTimeRobot.cpp:70-102
 *                                                   -> orc_ref_correspond
 *   Ransac                     function.h:35-109    -> orc_ref_ransac
 *
 * The reference builds PCL 1.8.0 octrees for these (PCL is not part of the
 * reference; parity against PCL itself is unpinned).  Restated octree rules
 * (OctreePointCloud with a defined bounding box):
 *   - define: the cube has 2^depth leaves of edge res per axis, depth the
 *     fewest levels covering ceil((hi - lo - FLT_EPSILON) / res) leaves on the
 *     widest axis (at least 2); each axis is padded by the same amount on both
 *     sides to the cube edge (when that amount exceeds FLT_EPSILON);
 *   - a point outside (p < min or p >= max on some axis) grows the tree one
 *     level at a time until it fits: on every axis where the point is not
 *     above the box the old cube becomes the upper half (min -= old edge);
 *     then max = min + new edge - FLT_EPSILON.  Points are inserted in
 *     ascending index order (PCL inserts the box search's output, which
 *     comes in its own tree order);
 *   - leaf key = (unsigned)((p - min) / res) in double, against the final
 *     box; leaf centre = (float)((key + 0.5) * res + min);
 *   - occupied leaves are listed depth-first with child index
 *     (x bit << 2 | y bit << 1 | z bit), i.e. ascending Morton code with x
 *     the most significant bit of each level.
 *
 * Where the reference has undefined behaviour, the definitions here:
 *   - get_Distance reads grid_value[y*30 + z*900 + x] for any leaf the
 *     rotated cloud reaches; an index outside [0, 27000) reads 900 (the
 *     distance cap) here;
 *   - get_TSDF of a keypoint with no occupied leaf allocates a negative
 *     array; here its field is all 900 (no occupied voxel);
 *   - Ransac's bestMatrix is uninitialised when no pair has an inlier; here
 *     it is the identity;
 *   - a cloud that would grow the tree past 21 levels, or a non-finite
 *     keypoint: score NaN, identity.
 * get_Distance accumulates its running score in float, leaf by leaf in
 * tree order, never reset between rotations (matching.h:141,179-189):
 * float_order = 1 reproduces that and is what the GPU path matches bit for
 * bit.  float_order = 0 is a variant kept to measure the rounding: each
 * rotation's sum of squared field values exact (integers), the running
 * score in double.
 *
 * Arithmetic (compile with -ffp-contract=off): transforms are
 * ((m0*x + m1*y) + m2*z) + m3 per row in float; 4x4 float products sum
 * their four terms in index order.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define REF_PI 3.14159265358979323846 /* M_PI */
#define REF_MAX_DEPTH 21
#define REF_DIM 30

typedef struct {
  double min[3], max[3];
  int depth;
} OctBox;

static void oct_define(OctBox* b, const float lo[3], const float hi[3], double res) {
  unsigned mv = 2;
  for (int a = 0; a < 3; ++a) {
    const double k = ceil(((double)hi[a] - (double)lo[a] - FLT_EPSILON) / res);
    if (k > mv) mv = (unsigned)k;
  }
  int d = 0;
  while ((1u << d) < mv) ++d;
  const double side = (double)(1u << d) * res;
  for (int a = 0; a < 3; ++a) {
    b->min[a] = lo[a];
    b->max[a] = hi[a];
    const double over = (side - ((double)hi[a] - (double)lo[a])) / 2.0;
    if (over > FLT_EPSILON) {
      b->min[a] -= over;
      b->max[a] += over;
    }
  }
  b->depth = d;
}

/* Grow until p fits; 0 on success, -1 past REF_MAX_DEPTH levels. */
static int oct_fit(OctBox* b, const float p[3], double res) {
  for (;;) {
    int up[3], out = 0;
    for (int a = 0; a < 3; ++a) {
      up[a] = (double)p[a] >= b->max[a];
      out |= up[a] | ((double)p[a] < b->min[a]);
    }
    if (!out) return 0;
    if (b->depth >= REF_MAX_DEPTH) return -1;
    const double side = (double)(1u << b->depth) * res;
    for (int a = 0; a < 3; ++a)
      if (!up[a]) b->min[a] -= side;
    b->depth++;
    const double edge = (double)(1u << b->depth) * res - FLT_EPSILON;
    for (int a = 0; a < 3; ++a) b->max[a] = b->min[a] + edge;
  }
}

static void oct_key(const OctBox* b, const float p[3], double res, unsigned k[3]) {
  const unsigned top = (1u << b->depth) - 1u;
  for (int a = 0; a < 3; ++a) {
    unsigned v = (unsigned)(((double)p[a] - b->min[a]) / res);
    k[a] = v > top ? top : v;
  }
}

static uint64_t morton3(const unsigned k[3], int depth) {
  uint64_t m = 0;
  for (int l = depth - 1; l >= 0; --l)
    m = (m << 3) | ((uint64_t)((k[0] >> l) & 1u) << 2) | ((uint64_t)((k[1] >> l) & 1u) << 1) |
        (uint64_t)((k[2] >> l) & 1u);
  return m;
}

static float oct_centre(const OctBox* b, unsigned key, int a, double res) {
  return (float)(((double)key + 0.5) * res + b->min[a]);
}

typedef struct {
  uint64_t m;
  unsigned k[3];
} Leaf;

static int leaf_cmp(const void* x, const void* y) {
  const uint64_t a = ((const Leaf*)x)->m, b = ((const Leaf*)y)->m;
  return a < b ? -1 : a > b;
}

/* Sort by Morton code and drop duplicates; returns the number of leaves. */
static int leaves_unique(Leaf* L, int n) {
  if (n == 0) return 0;
  qsort(L, (size_t)n, sizeof(Leaf), leaf_cmp);
  int u = 1;
  for (int i = 1; i < n; ++i)
    if (L[i].m != L[u - 1].m) L[u++] = L[i];
  return u;
}

static void xf(const float M[16], const float p[3], float o[3]) {
  for (int a = 0; a < 3; ++a) {
    float s = M[4 * a] * p[0];
    s = s + M[4 * a + 1] * p[1];
    s = s + M[4 * a + 2] * p[2];
    o[a] = s + M[4 * a + 3];
  }
}

static void mm4(const float A[16], const float B[16], float C[16]) {
  float T[16];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      float s = A[4 * r] * B[c];
      s = s + A[4 * r + 1] * B[4 + c];
      s = s + A[4 * r + 2] * B[8 + c];
      s = s + A[4 * r + 3] * B[12 + c];
      T[4 * r + c] = s;
    }
  memcpy(C, T, sizeof(T));
}

static void eye4(float M[16]) {
  memset(M, 0, 16 * sizeof(float));
  M[0] = M[5] = M[10] = M[15] = 1.f;
}

/* ---- KeyPoint::getOccupiedGrid (key_point.h:112-161) -------------------- */
long long orc_ref_occupancy(const float* cloud, int n, const float* keys, int nk, float res, float half,
                            int32_t* number, int32_t* offsets, int32_t* indices, long long cap) {
  long long total = 0;
  offsets[0] = 0;
  int32_t* cnt = (int32_t*)calloc((size_t)(nk > 0 ? nk : 1), sizeof(int32_t));
#pragma omp parallel for schedule(dynamic, 4)
  for (int k = 0; k < nk; ++k) {
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = keys[4 * k + a] - half;
      hi[a] = keys[4 * k + a] + half;
    }
    OctBox b;
    oct_define(&b, lo, hi, (double)res);
    Leaf* L = (Leaf*)malloc(sizeof(Leaf) * (size_t)(n > 0 ? n : 1));
    int c = 0;
    for (int i = 0; i < n; ++i) {
      const float* p = cloud + 4 * (size_t)i;
      if (p[0] >= lo[0] && p[1] >= lo[1] && p[2] >= lo[2] && p[0] <= hi[0] && p[1] <= hi[1] && p[2] <= hi[2]) {
        oct_key(&b, p, (double)res, L[c].k);
        L[c].m = morton3(L[c].k, b.depth);
        ++c;
      }
    }
    cnt[k] = c;
    number[k] = leaves_unique(L, c);
    free(L);
  }
  for (int k = 0; k < nk; ++k) {
    total += cnt[k];
    offsets[k + 1] = (int32_t)total;
  }
  if (total <= cap && indices) {
#pragma omp parallel for schedule(dynamic, 4)
    for (int k = 0; k < nk; ++k) {
      float lo[3], hi[3];
      for (int a = 0; a < 3; ++a) {
        lo[a] = keys[4 * k + a] - half;
        hi[a] = keys[4 * k + a] + half;
      }
      int32_t w = offsets[k];
      for (int i = 0; i < n; ++i) {
        const float* p = cloud + 4 * (size_t)i;
        if (p[0] >= lo[0] && p[1] >= lo[1] && p[2] >= lo[2] && p[0] <= hi[0] && p[1] <= hi[1] && p[2] <= hi[2])
          indices[w++] = i;
      }
    }
  }
  free(cnt);
  return total;
}

/* ---- KeyPoint::get_TSDF (key_point.h:251-334) ---------------------------
 * Occupied leaves of the keypoint's occupancy cloud in the +-half box, the
 * first in tree order dropped (the loop starts at 1), each leaf centre made
 * an integer voxel (centre - box min) / res, then the distance field of
 * kernel.cu.  Returns dim = (int)(half / res * 2), or -1 when dim^3 > 27000. */
int orc_ref_tdf(const float* cloud, const float* keys, int nk, const int32_t* offsets, const int32_t* indices,
                float res, float half, float* tdf) {
  const int dim = (int)(half / res * 2);
  if (dim < 1 || dim * dim * dim > 27000) return -1;
  const size_t vol = (size_t)dim * dim * dim;
#pragma omp parallel for schedule(dynamic, 1)
  for (int k = 0; k < nk; ++k) {
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = keys[4 * k + a] - half;
      hi[a] = keys[4 * k + a] + half;
    }
    OctBox b;
    oct_define(&b, lo, hi, (double)res);
    const int beg = offsets[k], n = offsets[k + 1] - beg;
    Leaf* L = (Leaf*)malloc(sizeof(Leaf) * (size_t)(n > 0 ? n : 1));
    /* insertion (grows the tree only when the occupancy box is wider than
     * this one), then keys against the final box */
    int c = 0, bad = 0;
    for (int j = 0; j < n && !bad; ++j) bad = oct_fit(&b, cloud + 4 * (size_t)indices[beg + j], (double)res) != 0;
    for (int j = 0; j < n && !bad; ++j) {
      const float* p = cloud + 4 * (size_t)indices[beg + j];
      oct_key(&b, p, (double)res, L[c].k);
      L[c].m = morton3(L[c].k, b.depth);
      ++c;
    }
    const int u = leaves_unique(L, c);
    int32_t* occ = (int32_t*)malloc(sizeof(int32_t) * 3 * (size_t)(u > 1 ? u - 1 : 1));
    for (int i = 1; i < u; ++i)
      for (int a = 0; a < 3; ++a) {
        const float ctr = oct_centre(&b, L[i].k[a], a, (double)res);
        occ[3 * (i - 1) + a] = (int32_t)(((double)ctr - (double)lo[a]) / (double)res);
      }
    orc_tdf(occ, u > 1 ? u - 1 : 0, dim, tdf + (size_t)k * vol);
    free(occ);
    free(L);
  }
  return dim;
}

/* ---- get_Distance (matching.h:122-222) ---------------------------------- */
typedef struct {
  float c1, s1;            /* cos, sin of theta = (float)(pi / 18), float functions */
  float c2[36], s2[36];    /* (float)cos((double)(i * theta)), likewise sin */
} RotTables;

static void rot_tables(RotTables* t) {
  const float theta = (float)(REF_PI / 18);
  t->c1 = cosf(theta);
  t->s1 = sinf(theta);
  for (int i = 0; i < 36; ++i) {
    const float th = (float)i * theta;
    t->c2[i] = (float)cos((double)th);
    t->s2[i] = (float)sin((double)th);
  }
}

static float field_at(const float* grid, const OctBox* b, const unsigned k[3], const float border[3], float res,
                      double dres) {
  long long ix[3];
  for (int a = 0; a < 3; ++a) {
    const float ctr = oct_centre(b, k[a], a, dres);
    const float q = (ctr - border[a]) / res;
    if (!(q > -2147483648.f && q < 2147483648.f)) return 900.f;
    ix[a] = (long long)(int)q;
  }
  const long long idx = ix[1] * REF_DIM + ix[2] * REF_DIM * REF_DIM + ix[0];
  return (idx >= 0 && idx < REF_DIM * REF_DIM * REF_DIM) ? grid[idx] : 900.f;
}

static void ref_distance_one(const float* mcloud, const float* km, const int32_t* idx, int n, const float* grid,
                             const float* ks, float res, float half, int float_order, const RotTables* R,
                             Leaf* L, float* P, float* score, float* Tout) {
  const double dres = (double)res;
  if (!(isfinite(km[0]) && isfinite(km[1]) && isfinite(km[2]) && isfinite(ks[0]) && isfinite(ks[1]) &&
        isfinite(ks[2]))) {
    *score = NAN;
    eye4(Tout);
    return;
  }
  float t[3], lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    t[a] = km[a] - ks[a];
    lo[a] = km[a] - half;
    hi[a] = km[a] + half;
  }
  float Tm[16], T1[16], T3[16], Rs[16], M[16];
  eye4(Tm);
  Tm[3] = t[0], Tm[7] = t[1], Tm[11] = t[2];
  for (int j = 0; j < n; ++j) xf(Tm, mcloud + 4 * (size_t)idx[j], P + 3 * (size_t)j);
  eye4(T1);
  T1[3] = -km[0], T1[7] = -km[1];
  eye4(T3);
  T3[3] = km[0], T3[7] = km[1];
  eye4(Rs);
  Rs[0] = R->c1, Rs[4] = R->s1, Rs[1] = -R->s1, Rs[5] = R->c1;
  mm4(T3, Rs, M);
  mm4(M, T1, M);
  double dt = 0.0, best = 100000000.0;
  float dtf = 0.f, bestf = 100000000.f;
  int best_i = 0, bad = 0;
  for (int i = 0; i < 36 && !bad; ++i) {
    if (i != 0)
      for (int j = 0; j < n; ++j) {
        float o[3];
        xf(M, P + 3 * (size_t)j, o);
        memcpy(P + 3 * (size_t)j, o, sizeof(o));
      }
    OctBox b;
    oct_define(&b, lo, hi, dres);
    for (int j = 0; j < n && !bad; ++j) bad = oct_fit(&b, P + 3 * (size_t)j, dres) != 0;
    if (bad) break;
    for (int j = 0; j < n; ++j) {
      oct_key(&b, P + 3 * (size_t)j, dres, L[j].k);
      L[j].m = morton3(L[j].k, b.depth);
    }
    const int u = leaves_unique(L, n);
    const double div = u == 0 ? 18446744073709551615.0 : (double)(u - 1);
    if (float_order) {
      for (int p = 1; p < u; ++p) {
        const float v = field_at(grid, &b, L[p].k, lo, res, dres);
        dtf += v * v;
      }
      dtf /= (float)div;
      if (dtf < bestf) {
        bestf = dtf;
        best_i = i;
      }
    } else {
      long long s = 0;
      for (int p = 1; p < u; ++p) {
        const float v = field_at(grid, &b, L[p].k, lo, res, dres);
        s += (long long)v * (long long)v;
      }
      dt = (dt + (double)s) / div;
      if (dt < best) {
        best = dt;
        best_i = i;
      }
    }
  }
  if (bad) {
    *score = NAN;
    eye4(Tout);
    return;
  }
  *score = float_order ? bestf : (float)best;
  float S[16], R2[16], A[16];
  eye4(S);
  const float cs = km[2] / ks[2];
  S[0] = S[5] = S[10] = cs;
  eye4(R2);
  R2[0] = R->c2[best_i], R2[4] = R->s2[best_i], R2[1] = -R->s2[best_i], R2[5] = R->c2[best_i];
  mm4(S, T3, A);
  mm4(A, R2, A);
  mm4(A, T1, A);
  mm4(A, Tm, Tout);
}

/* Pairs (pair_m[p], pair_s[p]), or every (model, scan) pair model-major when
 * pair_m is NULL (np = nm * ns).  Writes score[p] and the 4x4 row-major T[16p]. */
void orc_ref_distance(const float* mcloud, const float* mkeys, const int32_t* moff, const int32_t* midx,
                      const float* mtdf, int nm, const float* skeys, int ns, const int32_t* pair_m,
                      const int32_t* pair_s, long long np, float res, float half, int float_order, float* score,
                      float* T) {
  RotTables R;
  rot_tables(&R);
  int nmax = 1;
  for (int m = 0; m < nm; ++m)
    if (moff[m + 1] - moff[m] > nmax) nmax = moff[m + 1] - moff[m];
#pragma omp parallel
  {
    Leaf* L = (Leaf*)malloc(sizeof(Leaf) * (size_t)nmax);
    float* P = (float*)malloc(sizeof(float) * 3 * (size_t)nmax);
#pragma omp for schedule(dynamic, 16)
    for (long long p = 0; p < np; ++p) {
      const int m = pair_m ? pair_m[p] : (int)(p / ns);
      const int s = pair_s ? pair_s[p] : (int)(p % ns);
      ref_distance_one(mcloud, mkeys + 4 * (size_t)m, midx + moff[m], moff[m + 1] - moff[m],
                       mtdf + (size_t)m * REF_DIM * REF_DIM * REF_DIM, skeys + 4 * (size_t)s, res, half,
                       float_order, &R, L, P, score + p, T + 16 * p);
    }
    free(L);
    free(P);
  }
}

/* ---- the all-pairs loop with its gates (RealTimeRobot.cpp:70-102,
 * function.h:158-178), as written: the height gate passes unless the ratio
 * is NaN (float(2/3) == 0), the area gate has no lower bound
 * (float(1/3) == 0), the occupancy ratio is an integer quotient.
 * v3 (3 doubles per keypoint) NULL = the KeyPoint default 0.16. */
int orc_ref_gates(const float* km, int nm_number, const double* mv3, const float* ks, int ns_number,
                  const double* sv3) {
  const float h = km[2] / ks[2];
  if (!(h >= 0.f || h <= 1.5f)) return 0;
  for (int a = 0; a < 3; ++a) {
    const double r = (mv3 ? mv3[a] : 0.16) / (sv3 ? sv3[a] : 0.16);
    if (r > 3 || r < 0.0) return 0;
  }
  if (ns_number == 0) return 0;
  const float q = (float)(nm_number / ns_number);
  if (q > 2 || q < 0.5) return 0;
  return 1;
}

long long orc_ref_correspond(const float* mkeys, const int32_t* mnum, const double* mv3, int nm, const float* skeys,
                             const int32_t* snum, const double* sv3, int ns, const float* score_all,
                             float max_score, int32_t* pair_idx, long long cap) {
  long long c = 0;
  for (int m = 0; m < nm; ++m)
    for (int s = 0; s < ns; ++s) {
      const long long p = (long long)m * ns + s;
      const int keep = (score_all[p] < max_score) &&
                       orc_ref_gates(mkeys + 4 * (size_t)m, mnum[m], mv3 ? mv3 + 3 * (size_t)m : NULL,
                                     skeys + 4 * (size_t)s, snum[s], sv3 ? sv3 + 3 * (size_t)s : NULL);
      if (keep) {
        if (c < cap) pair_idx[c] = (int32_t)p;
        ++c;
      }
    }
  return c;
}

/* ---- Ransac (function.h:35-109) -----------------------------------------
 * Every kept pair's transform T_i (its get_Distance transform) moves every
 * pair's scan keypoint; inliers = pairs j with |k_j - T_i sk_j| < inlier
 * (float distance, float sqrt) and score_j < max_des.  The first transform
 * with the most inliers (strictly more than 0) wins; identity otherwise.
 * Returns the winning position in the pair list or -1. */
int orc_ref_ransac(const float* mkeys, const float* skeys, int ns, const int32_t* pair_idx, int np,
                   const float* score_all, const float* T_all, float inlier, float max_des, float* T_out,
                   int32_t* best_inliers) {
  int32_t* cnt = (int32_t*)malloc(sizeof(int32_t) * (size_t)(np > 0 ? np : 1));
#pragma omp parallel for schedule(dynamic, 8)
  for (int i = 0; i < np; ++i) {
    const float* Ti = T_all + 16 * (size_t)pair_idx[i];
    int c = 0;
    for (int j = 0; j < np; ++j) {
      const long long p = pair_idx[j];
      const int m = (int)(p / ns), s = (int)(p % ns);
      float q[3];
      xf(Ti, skeys + 4 * (size_t)s, q);
      const float* k = mkeys + 4 * (size_t)m;
      const float dx = k[0] - q[0], dy = k[1] - q[1], dz = k[2] - q[2];
      float d2 = dx * dx;
      d2 = d2 + dy * dy;
      d2 = d2 + dz * dz;
      const float dis = sqrtf(d2);
      if ((double)dis < (double)inlier && score_all[p] < max_des) ++c;
    }
    cnt[i] = c;
  }
  int best = -1, bc = 0;
  for (int i = 0; i < np; ++i)
    if (cnt[i] > bc) {
      bc = cnt[i];
      best = i;
    }
  if (best >= 0)
    memcpy(T_out, T_all + 16 * (size_t)pair_idx[best], 16 * sizeof(float));
  else
    eye4(T_out);
  *best_inliers = bc;
  free(cnt);
  return best;
}
