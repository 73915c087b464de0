// recog.cuh — stage building blocks of the recognition chain (device-driven
// counts so a whole chain can be captured in a CUDA graph).
#pragma once
#include "grid.cuh"

namespace rtr {

// Voxel segmentation shared by the voxel-grid filter and uniform sampling:
// keys floor(p * inv_leaf) relative to the minimum voxel (x fastest), a
// stable radix sort, segment heads and starts.  seg_start[V] = n.
struct VoxMeta {
  int lo[3], hi[3];
  unsigned dx, dy, dz;
  int error;  // key space exceeds 2^32
  int n;
};

struct VoxSeg {
  VoxMeta* meta;
  uint32_t *k0, *v0, *k1, *v1, *hist;  // radix buffers
  uint32_t* flags;                      // heads, then their exclusive scan
  uint32_t* tile_sums;
  int* seg_start;                       // [n_cap + 1]
  int* d_nseg;                          // V (device)
  const uint32_t* keys;                 // sorted keys (after build)
  const uint32_t* order;                // original index per sorted position
  int n_cap;
};

void voxseg_plan(ScratchPlan& p, int n_cap);
bool voxseg_take(Scratch& s, int n_cap, VoxSeg* v);
void voxseg_build(VoxSeg& v, const float4* pts, int n_host, const int* d_n, float inv_leaf,
                  cudaStream_t st);

}  // namespace rtr
