// icp.cuh — problem descriptor of the persistent multi-problem ICP kernel.
#pragma once
#include <vector>

#include "grid.cuh"

namespace rtr {

struct IcpDev {
  GridDev grid;               // target grid
  const GridMeta* src_meta;   // bounding box of the source (centring)
  const float4* src;          // source points (any order; sorted by target cell is faster)
  const int* src_idx;         // original index of each source point (NULL: identity)
  int n_src;
  int max_it;
  float r2max;
  double eps_t, eps_r;
  double init[16];
  double* pose64;             // [16]
  float* posef;               // [12]
  float* partial;             // [nblk][32]
  int* pcount;                // [nblk]
  unsigned* arrive;
  unsigned* gen;
  rtr_icp_result* result;
  double* trace_pose;
  int* trace_corr;
  int* status;
  long long budget;
  int blk0, nblk;             // this problem's blocks in the launch
  const int* d_active;        // when set: the problem runs only if slot < *d_active
  int slot;
  // when set (the launch's first problem): ns of block 0's search, of the
  // last block's serial section and of block 0's wait, summed over the
  // iterations, the iteration count, and the serial section's time to the
  // end of its cross-block reduction and of its pose solve
  unsigned long long* prof;
};

struct IcpSpec {
  IcpDev dev;               // grid, src_meta, src, src_idx, n_src, max_it, r2max, eps, init, result, traces
  const double* init_dev;   // optional device initial pose (overrides dev.init)
};

int icp_max_blocks(rtr_context* ctx);
int icp_pick_group(const rtr_context* ctx, long long total_pts, int blocks);
void icp_multi_plan(ScratchPlan& p, int n_probs, int max_blocks);
// Runs every problem; specs are completed (blocks, state buffers) in place.
rtr_status icp_multi(rtr_context* ctx, Scratch& s, std::vector<IcpSpec>& specs, cudaStream_t st);

}  // namespace rtr
