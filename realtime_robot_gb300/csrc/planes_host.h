// planes_host.h — host-side scalar steps of the plane segmentation
// (planes_host.cpp, compiled without floating-point contraction).
#pragma once

namespace rtr {

// State of the RANSAC walk over sample slots in order (slots come in
// batches; `base` is the first slot of the batch being walked).
struct PlaneWalk {
  int slot = 0;        // next slot of the current batch to look at
  int base = 0;        // global index of the batch's slot 0
  int iterations = 0;  // valid samples scored
  int skipped = 0;     // samples skipped (repeated positions, collinear)
  int best = -1;       // global slot of the first best sample
  int best_cnt = -1;
  double k = 1.0;      // samples needed for 99 % confidence
  int done = 0;
};

// Walks the batch's slots (valid flags and inlier counts) from w->slot;
// returns 1 when the walk has ended, 0 when it needs the next batch.
int plane_ransac_walk(const int* valid, const int* count, int n_slots, int m, int max_iterations, PlaneWalk* w);
// Least-squares plane from the FP64 sums (x, y, z, xx, xy, xz, yy, yz, zz)
// of n points; c_in when n < 3; *flat as PCL's hull dimension test.
void plane_refit(const double* sums9, int n, const float* c_in, float* c_out, int* flat);
// The plane's 2-D basis: e1 across the axis least aligned with the normal.
void plane_basis(const float* c, float* e1, float* e2);
// 0 horizontal, 1 vertical, -1 neither (is_h_plane / is_v_plane).
int plane_class(const float* c);
// Shoelace area and perimeter of a hull given as h (u, v) float pairs.
void hull_measure(const float* uv, int h, double* area, double* perim);

}  // namespace rtr
