/*
 * orient.c — outward normal orientation for full (360 degree) model clouds.
 * Test infrastructure: the checker's restatement of rtr_orient_normals_outward.
 *
 * A model cloud has no single viewpoint that sees every face, so
 * "flip towards the viewpoint" (PCL flipNormalTowardsViewpoint) orients some
 * faces inwards.  Rule used instead: count the cloud's points inside a
 * cylinder of radius rc along +n and along -n (axial distance in (gap, len]);
 * the normal points to the side with fewer points (the free side); ties keep
 * the sign.  Counts are integers, so the rule is exact.
 */
#include <math.h>

#include "oracle.h"

void orc_orient_outward(const float* pts, float* nrm, int n, float rc, float gap, float len) {
  const float rc2 = rc * rc;
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < n; ++i) {
    const float* p = pts + 4 * i;
    float* nv = nrm + 4 * i;
    int cp = 0, cm = 0;
    for (int j = 0; j < n; ++j) {
      const float dx = pts[4 * j] - p[0], dy = pts[4 * j + 1] - p[1], dz = pts[4 * j + 2] - p[2];
      const float ax0 = dx * nv[0], ax1 = dy * nv[1], ax2 = dz * nv[2];
      const float ax = (ax0 + ax1) + ax2;
      const float aa = fabsf(ax);
      if (!(aa > gap) || aa > len) continue;
      const float xx = dx * dx, yy = dy * dy, zz = dz * dz;
      const float r2 = ((xx + yy) + zz) - ax * ax;
      if (r2 > rc2) continue;
      if (ax > 0.f) ++cp; else ++cm;
    }
    if (cp > cm) {
      nv[0] = -nv[0];
      nv[1] = -nv[1];
      nv[2] = -nv[2];
    }
  }
}
