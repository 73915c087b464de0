// pipeline.cu — model preparation and scene recognition (the chain driven by
// main, RealTimeRobot.cpp:39-105: model side, scene side, all-pairs
// correspondence, consensus, transform).
//
// rtr_recognize: voxel filter -> normals -> uniform keypoints (optional
// curvature gate / learned pruning) -> SHOT-352 -> 1-NN descriptor matching ->
// geometric-consistency grouping -> hypothesis verification (model inliers in
// the scene) -> batched ICP refinement of the best hypotheses -> final score
// and non-maximum suppression.  Every count stays on the device: no stage
// reads back to the host, so a warmed-up call can be captured in a CUDA graph.
#include <cuda_bf16.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "grid.cuh"
#include "pipeline.cuh"
#include "recog.cuh"
#include "scan.cuh"
#include "search.cuh"

namespace rtr {

rtr_status voxel_downsample_dev(rtr_context*, Scratch&, const float4*, int, const int*, float, float4*, int*, cudaStream_t);
rtr_status uniform_sample_dev(rtr_context*, Scratch&, const float4*, int, const int*, float, int*, int*, cudaStream_t);
rtr_status normals_dev(rtr_context*, Scratch&, const float4*, int, const int*, int, const float*, float, float4*, cudaStream_t);
rtr_status shot_dev(rtr_context*, Scratch&, const float4*, const float4*, int, const int*, const int*, int, const int*,
                    float, float*, float*, cudaStream_t);
rtr_status shot_on_grid(const GridBufs&, const float4*, const float4*, const int*, int, const int*, float, float*,
                        float*, cudaStream_t);
rtr_status match_exact_dev(const float*, int, const int*, const float*, int, int*, float*, cudaStream_t);
size_t match_tc_bf16_bytes(int rows);
void match_tc_plan(ScratchPlan& p, int nq_cap, bool with_db, int ndb);
rtr_status match_tc_prepare_db(const float* db, int ndb, __nv_bfloat16* hi, __nv_bfloat16* lo, float* norm2,
                               cudaStream_t st);
rtr_status match_tc_dev(rtr_context* ctx, Scratch& s, const float* q, int nq_cap, const int* d_nq, const float* db,
                        int ndb, const __nv_bfloat16* db_hi, const __nv_bfloat16* db_lo, const float* db_n2,
                        int* out_idx, float* out_d2, cudaStream_t st);
size_t gc_scratch_bytes(int C, int max_clusters);
rtr_status gc_group_async(rtr_context* ctx, Scratch& s, const float* d_model_kp, const float* d_scene_kp,
                          const int32_t* d_corr_m, const int32_t* d_corr_s, const float* d_corr_d, int C_cap,
                          const int* d_C, float gc_size, int gc_thresh, int max_clusters, int32_t* d_sizes,
                          double* d_poses, int* d_ncl, cudaStream_t st);
size_t mlp_infer_bytes(int n_cap);
rtr_status mlp_score_rows(rtr_context* ctx, Scratch& s, const rtr_mlp* m, const float* X, int n_cap, const int* d_n,
                          float* score, cudaStream_t st);
__global__ void k_orient_outward(const float4* __restrict__ pts, float4* __restrict__ nrm, int n_host, const int* d_n,
                                 float rc2, float gap, float len);
rtr_status gc_group_dev(rtr_context* ctx, Scratch& s, const float* d_model_kp, const float* d_scene_kp,
                        const int32_t* d_corr_m, const int32_t* d_corr_s, const float* d_corr_d, int n_corr,
                        float gc_size, int gc_thresh, int max_clusters, int max_members, int32_t* d_members,
                        int32_t* d_sizes, double* d_poses, int* h_n_clusters, cudaStream_t st);

static int nblocks(int n, int per = 256, int cap = 152 * 16) {
  int b = (n + per - 1) / per;
  if (b < 1) b = 1;
  return b > cap ? cap : b;
}

__device__ __forceinline__ int dcount(const int* d, int cap) {
  const int v = *d;
  return v < 0 ? 0 : (v > cap ? cap : v);
}

// keep[i] = keep keypoint i (curvature gate); writes 0/1 flags
__global__ void k_gate_flags(const int* __restrict__ keys, const int* d_nk, int cap, const float4* __restrict__ nrm,
                             float min_curv, uint32_t* __restrict__ flags) {
  const int nk = dcount(d_nk, cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x)
    flags[i] = (i < nk && nrm[keys[i]].w >= min_curv) ? 1u : 0u;
}

__global__ void k_compact_int(const int* __restrict__ in, const uint32_t* __restrict__ flags,
                              const uint32_t* __restrict__ pos, int cap, int* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x)
    if (flags[i]) out[pos[i]] = in[i];
}

// Learned pruning: sort keys putting higher credibility first (scores are
// in (0, 1); anything else sorts last), then flags for the first
// ceil(keep * K) keypoints of that order.
__global__ void k_score_keys(const float* __restrict__ score, const int* d_nk, int cap, uint32_t* __restrict__ keys) {
  const int nk = dcount(d_nk, cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nk; i += gridDim.x * blockDim.x) {
    const float v = score[i];
    keys[i] = (v >= 0.f && v <= 1.f) ? ~__float_as_uint(v) : 0xffffffffu;
  }
}

__global__ void k_mark_top(const uint32_t* __restrict__ order, const int* d_nk, int cap, float keep,
                           uint32_t* __restrict__ flags) {
  const int nk = dcount(d_nk, cap);
  int kk = (int)ceil((double)keep * (double)nk);
  kk = kk < nk ? kk : nk;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) {
    if (i < nk)
      flags[order[i]] = i < kk ? 1u : 0u;  // order is a permutation of [0, nk)
    else
      flags[i] = 0u;
  }
}

// Rows of a [cap][352] descriptor array kept by flags, packed in order (warp
// per row, float4 copies).
__global__ void k_compact_rows(const float* __restrict__ in, const uint32_t* __restrict__ flags,
                               const uint32_t* __restrict__ pos, const int* d_nk, int cap, float* __restrict__ out) {
  const int nk = dcount(d_nk, cap);
  const int lane = threadIdx.x & 31;
  for (int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < nk; r += gridDim.x * (blockDim.x >> 5)) {
    if (!flags[r]) continue;
    const float4* src = reinterpret_cast<const float4*>(in + (size_t)r * 352);
    float4* dst = reinterpret_cast<float4*>(out + (size_t)pos[r] * 352);
    for (int k = lane; k < 88; k += 32) dst[k] = src[k];
  }
}

// correspondences: scene keypoint slot i matched to model keypoint idx[i]
__global__ void k_corr_flags(const int* __restrict__ idx, const float* __restrict__ d2, const int* d_nk, int cap,
                             float max_d2, uint32_t* __restrict__ flags) {
  const int nk = dcount(d_nk, cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x)
    flags[i] = (i < nk && idx[i] >= 0 && d2[i] < max_d2) ? 1u : 0u;
}

__global__ void k_corr_scatter(const int* __restrict__ idx, const float* __restrict__ d2,
                               const uint32_t* __restrict__ flags, const uint32_t* __restrict__ pos, int cap,
                               int* __restrict__ cm, int* __restrict__ cs, float* __restrict__ cd) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x)
    if (flags[i]) {
      const int o = pos[i];
      cm[o] = idx[i];
      cs[o] = i;
      cd[o] = d2[i];
    }
}

__global__ void k_gather_kp(const float4* __restrict__ pts, const int* __restrict__ keys, const int* d_nk, int cap,
                            float4* __restrict__ out) {
  const int nk = dcount(d_nk, cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nk; i += gridDim.x * blockDim.x) out[i] = pts[keys[i]];
}

// Inlier count of a transformed model cloud in the scene grid: one block per
// hypothesis, G lanes per model point (exact bounded 1-NN; found = inlier).
constexpr int HV_G = 4;
// Inlier count of every hypothesis: model points (every stride-th) moved by
// the hypothesis pose with a scene point within sqrt(r2).  Blocks cover
// (hypothesis, run of HV_PPB points); counts are integers, so the order of
// the atomic adds does not matter.  Four blocks an SM (64 registers):
// more searches in flight beat the spills that costs.
constexpr int HV_PPB = 256;
__global__ void __launch_bounds__(256, 4) k_hv_count(GridDev gd, const float4* __restrict__ model, int n_model, int stride,
                                                  const double* __restrict__ poses, int n_hyp, const int* d_nhyp,
                                                  float r2, int bph, int* __restrict__ counts) {
  __shared__ int s_cnt;
  const int h = blockIdx.x / bph, part = blockIdx.x - h * bph;
  if (d_nhyp) n_hyp = min(*d_nhyp, n_hyp);
  if (h >= n_hyp) return;
  const GridView g = load_view(gd);
  const bool near27 = grid_near27_ok(g, r2);  // every inlier within the 27 cells around a point
  float T[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) T[k] = __double2float_rn(poses[(size_t)h * 16 + k]);
  if (threadIdx.x == 0) s_cnt = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, lg = lane & (HV_G - 1);
  const unsigned gmask = ((1u << HV_G) - 1u) << (lane & ~(HV_G - 1));
  int cnt = 0;
  const int total = (n_model + stride - 1) / stride;
  const int i1 = min(total, (part + 1) * HV_PPB);
  for (int i = part * HV_PPB + threadIdx.x / HV_G; i < i1; i += blockDim.x / HV_G) {
    const float4 p = xform_exact(T, model[(size_t)i * stride]);
    bool in;
    if (near27) {
      in = grid_any_near<HV_G>(g, p, r2, lg, gmask);
    } else {
      float d2;
      int bi, bp;
      grid_nn1_group<HV_G, true>(g, p, r2, lg, gmask, d2, bi, bp);
      in = bi >= 0;
    }
    if (lg == 0 && in) ++cnt;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if (lane == 0 && cnt) atomicAdd(&s_cnt, cnt);
  __syncthreads();
  if (threadIdx.x == 0 && s_cnt) atomicAdd(counts + h, s_cnt);
}

__global__ void k_hv_finish(const int* __restrict__ counts, int n_hyp, const int* d_nhyp, int total,
                            float* __restrict__ score) {
  if (d_nhyp) n_hyp = min(*d_nhyp, n_hyp);
  for (int h = blockIdx.x * blockDim.x + threadIdx.x; h < n_hyp; h += gridDim.x * blockDim.x)
    score[h] = total > 0 ? (float)counts[h] / (float)total : 0.f;
}

static rtr_status hv_score(GridDev gd, const float4* model, int n_model, int stride, const double* poses, int n_hyp,
                           const int* d_nhyp, float r2, int* counts, float* score, cudaStream_t st) {
  const int total = (n_model + stride - 1) / stride;
  const int bph = (total + HV_PPB - 1) / HV_PPB > 0 ? (total + HV_PPB - 1) / HV_PPB : 1;
  RTR_CUDA(cudaMemsetAsync(counts, 0, sizeof(int) * (size_t)n_hyp, st));
  k_hv_count<<<n_hyp * bph, 256, 0, st>>>(gd, model, n_model, stride, poses, n_hyp, d_nhyp, r2, bph, counts);
  k_hv_finish<<<(n_hyp + 255) / 256, 256, 0, st>>>(counts, n_hyp, d_nhyp, total, score);
  RTR_LAUNCHED(2);
  return RTR_OK;
}

// Top-m hypotheses by score (ties: lower hypothesis index) -> order[0..m),
// with n = min(*d_n, n_cap) hypotheses and m = min(n, m_cap); order[m..m_cap)
// = -1 and *d_m = m.  One warp, scores staged in shared memory (n <= 256).
__global__ void k_topm(const float* __restrict__ score, int n_cap, const int* d_n, int m_cap,
                       int* __restrict__ order, int* __restrict__ d_m) {
  __shared__ float s_sc[256];
  const int lane = threadIdx.x;
  if (lane >= 32) return;
  const int n = d_n ? min(*d_n, n_cap) : n_cap;
  const int m = min(n, m_cap);
  if (lane == 0) *d_m = m;
  for (int k = m + lane; k < m_cap; k += 32) order[k] = -1;
  for (int h = lane; h < 256; h += 32) s_sc[h] = h < n ? score[h] : 0.f;
  bool used[8] = {false, false, false, false, false, false, false, false};  // hypothesis lane + 32 q taken
  __syncwarp();
  for (int k = 0; k < m; ++k) {
    int best = -1;
    float bs = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int h = lane + 32 * q;
      if (h < n && !used[q] && (best < 0 || s_sc[h] > bs)) {
        best = h;
        bs = s_sc[h];
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const int ob = __shfl_xor_sync(0xffffffffu, best, o);
      const float os = __shfl_xor_sync(0xffffffffu, bs, o);
      if (ob >= 0 && (best < 0 || os > bs || (os == bs && ob < best))) {
        best = ob;
        bs = os;
      }
    }
    if (lane == 0) order[k] = best;
#pragma unroll
    for (int q = 0; q < 8; ++q)
      if (best == lane + 32 * q) used[q] = true;
  }
}

__global__ void k_select_poses(const double* __restrict__ poses, const int* __restrict__ order, int m,
                               double* __restrict__ out) {
  for (int i = threadIdx.x; i < m * 16; i += blockDim.x) {
    const int k = i / 16, e = i % 16;
    const int h = order[k];
    out[i] = h >= 0 ? poses[(size_t)h * 16 + e] : ((e % 5) == 0 ? 1.0 : 0.0);
  }
}

__global__ void k_copy_result_poses(const rtr_icp_result* __restrict__ r, int m, double* __restrict__ out) {
  for (int i = threadIdx.x; i < m * 16; i += blockDim.x) out[i] = r[i / 16].pose[i % 16];
}

// The result records of an empty scene: nothing found.
__global__ void k_result_empty(rtr_recog_result* __restrict__ out, int n) {
  const int words = (int)(sizeof(rtr_recog_result) / sizeof(int));
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n * words; i += gridDim.x * blockDim.x)
    reinterpret_cast<int*>(out)[i] = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) out[i].status = RTR_ERR_NOT_FOUND;
}

// Non-maximum suppression and the result record (one thread).
__global__ void k_finalize(const float* __restrict__ fscore, const double* __restrict__ refined,
                           const int* __restrict__ order, const int* __restrict__ cl_sizes, int m_cap,
                           const int* d_m, float accept, float nms2, int max_inst, const int* d_V, const int* d_K,
                           const int* d_C, const int* d_ncl, const int* d_status, rtr_recog_result* __restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int m = min(*d_m, m_cap), ncl = *d_ncl;
  int picked[RTR_MAX_INSTANCES];
  int np = 0;
  bool used[64];
  for (int k = 0; k < m && k < 64; ++k) used[k] = false;
  while (np < max_inst && np < RTR_MAX_INSTANCES) {
    int best = -1;
    for (int k = 0; k < m && k < 64; ++k) {
      if (used[k] || order[k] < 0) continue;
      if (best < 0 || fscore[k] > fscore[best]) best = k;
    }
    if (best < 0 || !(fscore[best] >= accept)) break;
    used[best] = true;
    bool dup = false;
    for (int j = 0; j < np; ++j) {
      const double* A = refined + (size_t)picked[j] * 16;
      const double* B = refined + (size_t)best * 16;
      const double dx = A[3] - B[3], dy = A[7] - B[7], dz = A[11] - B[11];
      if (dx * dx + dy * dy + dz * dz < (double)nms2) dup = true;
    }
    if (dup) continue;
    picked[np] = best;
    rtr_instance& I = out->inst[np];
    for (int e = 0; e < 16; ++e) I.pose[e] = refined[(size_t)best * 16 + e];
    I.score = fscore[best];
    I.hypothesis = order[best];
    I.cluster_size = cl_sizes[order[best]];
    ++np;
  }
  out->n_instances = np;
  out->n_voxels = *d_V;
  out->n_keypoints = *d_K;
  out->n_correspondences = d_C ? *d_C : 0;
  out->n_clusters = ncl;
  const int err = *d_status;  // a failed stage of this context (timeout, capacity)
  out->status = err ? err : (ncl > 0 ? RTR_OK : RTR_ERR_NOT_FOUND);
}

}  // namespace rtr

using namespace rtr;

struct rtr_model {
  int device = 0;
  int n_vox = 0, n_kp = 0;
  float4* vox = nullptr;    // voxel cloud
  float4* nrm = nullptr;    // outward normals
  int* keys = nullptr;      // keypoint indices into vox
  float4* kp = nullptr;     // keypoint positions
  float* desc = nullptr;    // [n_kp][352]
  GridMeta* vox_meta = nullptr;  // bbox of the voxel cloud (ICP centring)
  __nv_bfloat16* db_hi = nullptr;  // [n_kp][384] descriptor split for the tensor cores
  __nv_bfloat16* db_lo = nullptr;
  float* db_n2 = nullptr;          // [db_norm_floats(n_kp)] squared norms, their maximum, the all-zero answer
  uint64_t uid = 0;                // identity for captured recognitions (rtr::next_uid)
};

// rtr_mlp's identity, for the recognition graph's key (mlp.cu).
uint64_t rtr_mlp_uid(const rtr_mlp* m);

extern "C" {

void rtr_recog_default_params(rtr_recog_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->voxel_leaf = 0.01f;
  p->normal_k = 10;
  p->scene_keypoint_r = 0.02f;
  p->model_keypoint_r = 0.02f;
  p->descriptor_r = 0.04f;
  p->match_max_d2 = 0.25f;
  p->gc_size = 0.01f;
  p->gc_thresh = 5;
  p->max_clusters = 256;
  p->hv_inlier_r = 0.02f;
  p->hv_subsample = 4;
  p->refine_top = 16;
  p->icp_iterations = 30;
  p->icp_max_dist = 0.02f;
  p->accept_inlier_r = 0.01f;
  p->accept_score = 0.2f;
  p->nms_dist = 0.1f;
  p->max_instances = 8;
  p->viewpoint[0] = 0.f;
  p->viewpoint[1] = 0.f;
  p->viewpoint[2] = 0.f;
  p->keypoint_min_curvature = 0.f;
}

rtr_status rtr_model_create(rtr_context* ctx, const float* d_pts, int n, const rtr_recog_params* prm,
                            rtr_model** out) {
  RTR_CHECK_ARG(ctx && d_pts && n > 0 && prm && out, "rtr_model_create: bad arguments");
  *out = nullptr;
  RTR_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->host_stream;
  rtr_model* m = new rtr_model();
  m->uid = next_uid();
  m->device = ctx->device;
  auto cleanup = [&](rtr_status s) {
    rtr_model_destroy(m);
    return s;
  };
  if (cudaMalloc(&m->vox, (size_t)n * 16) != cudaSuccess || cudaMalloc(&m->nrm, (size_t)n * 16) != cudaSuccess ||
      cudaMalloc(&m->keys, (size_t)n * 4) != cudaSuccess || cudaMalloc(&m->vox_meta, sizeof(GridMeta)) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(fail(RTR_ERR_OOM, "rtr_model_create: device buffers"));
  }
  ScratchPlan plan;
  plan.add<int>(4);
  voxseg_plan(plan, n);
  grid_plan(plan, n, default_cell_cap(n));
  Scratch s;
  rtr_status r = ensure_scratch(ctx, plan.bytes, st, &s);
  if (r != RTR_OK) return cleanup(r);
  int* d_cnt = s.take<int>(4);  // counts first; the stages below reuse what follows
  const float4* p4 = reinterpret_cast<const float4*>(d_pts);
  Scratch sa = s;
  r = voxel_downsample_dev(ctx, sa, p4, n, nullptr, prm->voxel_leaf, m->vox, d_cnt, st);
  if (r != RTR_OK) return cleanup(r);
  if (cudaMemcpyAsync(ctx->h_pin, d_cnt, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return cleanup(fail(RTR_ERR_CUDA, "rtr_model_create: voxel count"));
  const int V = ctx->h_pin[0];
  if (V <= 0) return cleanup(fail(RTR_ERR_INVALID_ARG, "rtr_model_create: voxel filter produced %d points", V));
  m->n_vox = V;
  const float vp[3] = {0.f, 0.f, 0.f};
  Scratch sb = s;
  r = normals_dev(ctx, sb, m->vox, V, nullptr, prm->normal_k, vp, 2.f * prm->voxel_leaf, m->nrm, st);
  if (r != RTR_OK) return cleanup(r);
  r = rtr_orient_normals_outward(ctx, reinterpret_cast<float*>(m->vox), reinterpret_cast<float*>(m->nrm), V, 0.01f,
                                 0.005f, 1.0f, st);
  if (r != RTR_OK) return cleanup(r);
  Scratch sc = s;
  r = uniform_sample_dev(ctx, sc, m->vox, V, nullptr, prm->model_keypoint_r, m->keys, d_cnt + 1, st);
  if (r != RTR_OK) return cleanup(r);
  if (cudaMemcpyAsync(ctx->h_pin, d_cnt + 1, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return cleanup(fail(RTR_ERR_CUDA, "rtr_model_create: keypoint count"));
  const int K = ctx->h_pin[0];
  if (K <= 0) return cleanup(fail(RTR_ERR_INVALID_ARG, "rtr_model_create: no keypoints"));
  m->n_kp = K;
  if (cudaMalloc(&m->kp, (size_t)K * 16) != cudaSuccess ||
      cudaMalloc(&m->desc, (size_t)K * 352 * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(fail(RTR_ERR_OOM, "rtr_model_create: descriptor buffers"));
  }
  Scratch sd = s;
  r = shot_dev(ctx, sd, m->vox, m->nrm, V, nullptr, m->keys, K, nullptr, prm->descriptor_r, m->desc, nullptr, st);
  if (r != RTR_OK) return cleanup(r);
  k_gather_kp<<<nblocks(K), 256, 0, st>>>(m->vox, m->keys, d_cnt + 1, K, m->kp);
  bbox_build(m->vox_meta, m->vox, V, st);
  RTR_LAUNCHED(1);
  if (cudaMalloc(&m->db_hi, match_tc_bf16_bytes(K)) != cudaSuccess ||
      cudaMalloc(&m->db_lo, match_tc_bf16_bytes(K)) != cudaSuccess ||
      cudaMalloc(&m->db_n2, (size_t)db_norm_floats(K) * sizeof(float)) != cudaSuccess) {
    cudaGetLastError();
    return cleanup(fail(RTR_ERR_OOM, "rtr_model_create: tensor-core database"));
  }
  r = match_tc_prepare_db(m->desc, K, m->db_hi, m->db_lo, m->db_n2, st);
  if (r != RTR_OK) return cleanup(r);
  if (cudaStreamSynchronize(st) != cudaSuccess) return cleanup(fail(RTR_ERR_CUDA, "rtr_model_create: sync"));
  *out = m;
  return RTR_OK;
}

rtr_status rtr_model_destroy(rtr_model* m) {
  if (!m) return RTR_OK;
  cudaSetDevice(m->device);
  cudaFree(m->vox);
  cudaFree(m->nrm);
  cudaFree(m->keys);
  cudaFree(m->kp);
  cudaFree(m->desc);
  cudaFree(m->vox_meta);
  cudaFree(m->db_hi);
  cudaFree(m->db_lo);
  cudaFree(m->db_n2);
  delete m;
  return RTR_OK;
}

rtr_status rtr_model_info(const rtr_model* m, int* n_voxels, int* n_keypoints) {
  RTR_CHECK_ARG(m, "rtr_model_info: NULL model");
  if (n_voxels) *n_voxels = m->n_vox;
  if (n_keypoints) *n_keypoints = m->n_kp;
  return RTR_OK;
}

rtr_status rtr_model_buffers(const rtr_model* m, const float** d_vox, const float** d_normals, const int32_t** d_keys,
                             const float** d_kp, const float** d_desc) {
  RTR_CHECK_ARG(m, "rtr_model_buffers: NULL model");
  if (d_vox) *d_vox = reinterpret_cast<const float*>(m->vox);
  if (d_normals) *d_normals = reinterpret_cast<const float*>(m->nrm);
  if (d_keys) *d_keys = m->keys;
  if (d_kp) *d_kp = reinterpret_cast<const float*>(m->kp);
  if (d_desc) *d_desc = m->desc;
  return RTR_OK;
}

}  // extern "C"

namespace rtr {

// Scene-side buffers of one recognition: everything that depends on the
// scene alone, shared by every model recognised in it.
struct SceneBufs {
  int* cnt;                 // [0] V, [1] K (uniform), [2] K (gated), [3] K (pruned)
  float4 *sv, *sn;
  int *keys, *keys2;
  float* desc;
  uint32_t *flags, *pos, *tiles;
  GridBufs grid;            // scene voxels at the ICP distance (verification, refinement)
  GridBufs shot_grid;       // scene voxels at the descriptor radius (SHOT's support)
  Scratch aux;              // temporaries of the keypoint stage on the side stream
  int* keys_p;              // learned pruning: kept keypoints
  float* desc_p;            // and their descriptors
  // what goes on to matching (set by scene_stages)
  const int* keys_m;
  const int* d_nk;
  const float* desc_m;
  // recorded on the side stream once the scene grid is built: a stream waits
  // on it before the first stage that reads the grid (verification)
  cudaEvent_t grid_ready = nullptr;
};

// Model-side buffers: correspondences, hypotheses, refinement.
struct ModelBufs {
  int* cnt;                 // [0] C, [1] clusters, [2] hypotheses refined
  float4* skp;
  int *midx, *cm, *cs;
  float *md2, *cd;
  uint32_t *flags, *pos, *tiles;
  double *poses, *init, *refined;
  int *sizes, *order;
  float *hv, *fscore;
  int* hvcnt;
  rtr_icp_result* res;
};

// The keypoint stage's temporaries, which run beside the normals on the
// context's side stream and so need a region of their own.
static size_t aux_bytes(int n) {
  ScratchPlan t;
  voxseg_plan(t, n);
  return t.bytes + 256;
}

static void scene_plan(ScratchPlan& p, int n, bool learned) {
  p.add<int>(8);
  p.add<float4>(n);
  p.add<float4>(n);
  p.add<int>(n);
  p.add<int>(n);
  p.add<float>((size_t)n * 352);
  p.add<uint32_t>(n);
  p.add<uint32_t>(n);
  p.add<uint32_t>(scan_tiles(n));
  grid_plan(p, n, default_cell_cap(n));
  grid_plan(p, n, default_cell_cap(n));
  p.add<char>(aux_bytes(n));
  if (learned) {
    p.add<int>(n);
    p.add<float>((size_t)n * 352);
  }
}

static bool scene_take(Scratch& s, int n, bool learned, SceneBufs* b) {
  b->cnt = s.take<int>(8);
  b->sv = s.take<float4>(n);
  b->sn = s.take<float4>(n);
  b->keys = s.take<int>(n);
  b->keys2 = s.take<int>(n);
  b->desc = s.take<float>((size_t)n * 352);
  b->flags = s.take<uint32_t>(n);
  b->pos = s.take<uint32_t>(n);
  b->tiles = s.take<uint32_t>(scan_tiles(n));
  if (!b->tiles || !grid_take(s, n, default_cell_cap(n), &b->grid) ||
      !grid_take(s, n, default_cell_cap(n), &b->shot_grid))
    return false;
  b->aux.base = s.take<char>(aux_bytes(n));
  b->aux.off = 0;
  b->aux.cap = aux_bytes(n);
  if (!b->aux.base) return false;
  b->keys_p = nullptr;
  b->desc_p = nullptr;
  if (learned) {
    b->keys_p = s.take<int>(n);
    b->desc_p = s.take<float>((size_t)n * 352);
    return b->desc_p != nullptr;
  }
  return true;
}

static void model_plan(ScratchPlan& p, int n, const rtr_recog_params* q) {
  const int H = q->max_clusters, M = q->refine_top;
  p.add<int>(8);
  p.add<float4>(n);
  for (int i = 0; i < 3; ++i) p.add<int>(n);
  p.add<float>(n);
  p.add<float>(n);
  p.add<uint32_t>(n);
  p.add<uint32_t>(n);
  p.add<uint32_t>(scan_tiles(n));
  p.add<double>((size_t)H * 16);
  p.add<double>((size_t)M * 16);
  p.add<double>((size_t)M * 16);
  p.add<int>(H);
  p.add<int>(M);
  p.add<float>(H);
  p.add<float>(M);
  p.add<int>(H > M ? H : M);
  p.add<rtr_icp_result>(M);
}

static bool model_take(Scratch& s, int n, const rtr_recog_params* q, ModelBufs* b) {
  const int H = q->max_clusters, M = q->refine_top;
  b->cnt = s.take<int>(8);
  b->skp = s.take<float4>(n);
  b->midx = s.take<int>(n);
  b->cm = s.take<int>(n);
  b->cs = s.take<int>(n);
  b->md2 = s.take<float>(n);
  b->cd = s.take<float>(n);
  b->flags = s.take<uint32_t>(n);
  b->pos = s.take<uint32_t>(n);
  b->tiles = s.take<uint32_t>(scan_tiles(n));
  b->poses = s.take<double>((size_t)H * 16);
  b->init = s.take<double>((size_t)M * 16);
  b->refined = s.take<double>((size_t)M * 16);
  b->sizes = s.take<int>(H);
  b->order = s.take<int>(M);
  b->hv = s.take<float>(H);
  b->fscore = s.take<float>(M);
  b->hvcnt = s.take<int>(H > M ? H : M);
  b->res = s.take<rtr_icp_result>(M);
  return b->res != nullptr;
}

// Per-stage scratch: the largest of the stages' own needs.
static size_t stage_bytes(int n, const rtr_recog_params* q, bool learned) {
  size_t stage = 0;
  if (learned) {
    ScratchPlan t;
    t.add<float>(n);
    for (int i = 0; i < 4; ++i) t.add<uint32_t>(n);
    t.add<uint32_t>(radix_hist_entries(n));
    const size_t b = t.bytes + mlp_infer_bytes(n) + 512;
    stage = b > stage ? b : stage;
  }
  {
    ScratchPlan t;
    voxseg_plan(t, n);
    stage = t.bytes > stage ? t.bytes : stage;
  }
  {
    ScratchPlan t;
    grid_plan(t, n, default_cell_cap(n));
    stage = t.bytes > stage ? t.bytes : stage;
  }
  stage = gc_scratch_bytes(n, q->max_clusters) > stage ? gc_scratch_bytes(n, q->max_clusters) : stage;
  {
    ScratchPlan t;
    icp_multi_plan(t, q->refine_top, 152 * 16);
    stage = t.bytes > stage ? t.bytes : stage;
  }
  {
    ScratchPlan t;
    match_tc_plan(t, n, false, 0);
    stage = t.bytes > stage ? t.bytes : stage;
  }
  return stage;
}

size_t recognize_scratch_bytes(int n, const rtr_recog_params* q, bool learned) {
  ScratchPlan p;
  scene_plan(p, n, learned);
  model_plan(p, n, q);
  return p.bytes + stage_bytes(n, q, learned) + 4096;
}

// The scene's stages: voxels, normals, keypoints (gated), descriptors,
// learned pruning, the scene grid at the ICP distance.
static rtr_status scene_stages(rtr_context* ctx, const Scratch& stage, SceneBufs& b, const float4* scene, int n,
                               const rtr_recog_params* q, const rtr_mlp* mlp, float keep, cudaStream_t st) {
  int* dV = b.cnt;
  int* dK = b.cnt + 1;
  int* dKg = b.cnt + 2;
  const int nb = nblocks(n);
  {
    ProfScope ps(ctx, st, "voxel_downsample");
    Scratch t = stage;
    RTR_TRY(voxel_downsample_dev(ctx, t, scene, n, nullptr, q->voxel_leaf, b.sv, dV, st));
  }
  // The keypoints, the descriptors' grid and the scene grid need only the
  // voxels: they run on the context's side stream beside the normals, the
  // descriptors and pruning (small sort-bound kernels that leave most of the
  // GPU idle), joined before the descriptors and, for the scene grid (its
  // own buffers), before verification.
  RTR_TRY(side_stream_ready(ctx));
  cudaStream_t ax = ctx->side_stream;
  RTR_CUDA(cudaEventRecord(ctx->ev_side[0], st));
  RTR_CUDA(cudaStreamWaitEvent(ax, ctx->ev_side[0], 0));
  {
    ProfScope ps(ctx, ax, "keypoints");
    Scratch t = b.aux;
    RTR_TRY(uniform_sample_dev(ctx, t, b.sv, n, dV, q->scene_keypoint_r, b.keys, dK, ax));
  }
  {
    ProfScope ps(ctx, ax, "shot_grid");
    grid_build(b.shot_grid, b.sv, n, dV, q->descriptor_r, ax);
  }
  RTR_CUDA(cudaEventRecord(ctx->ev_side[1], ax));
  {
    ProfScope ps(ctx, ax, "scene_grid");
    // 1.5 x the ICP distance measured fastest for refinement and verification
    const float cell = ctx->tune_scene_grid_mm > 0 ? 1e-3f * (float)ctx->tune_scene_grid_mm : 1.5f * q->icp_max_dist;
    grid_build(b.grid, b.sv, n, dV, cell, ax);
  }
  RTR_CUDA(cudaEventRecord(ctx->ev_side[2], ax));
  {
    ProfScope ps(ctx, st, "normals");
    Scratch t = stage;
    // 5 leaves: the k-NN of a voxel (k = 10 at 1 cm) mostly resolves in its
    // own cell and the next ring; smaller cells cost more cell visits than
    // the extra points of larger ones (0.71 ms at 2 leaves, 0.41 ms at 5 on
    // the 213k-voxel room)
    const float cell = ctx->tune_normals_grid_mm > 0 ? 1e-3f * (float)ctx->tune_normals_grid_mm : 5.f * q->voxel_leaf;
    RTR_TRY(normals_dev(ctx, t, b.sv, n, dV, q->normal_k, q->viewpoint, cell, b.sn, st));
    if (q->scene_outward) {
      k_orient_outward<<<nblocks(n, 8, 152 * 16), 256, 0, st>>>(b.sv, b.sn, n, dV, 0.01f * 0.01f, 0.005f, 1.0f);
      RTR_LAUNCHED(1);
    }
  }
  RTR_CUDA(cudaStreamWaitEvent(st, ctx->ev_side[1], 0));  // the keypoints and the descriptors' grid
  const int* keys = b.keys;
  const int* dKeys = dK;
  if (q->keypoint_min_curvature > 0.f) {
    ProfScope ps(ctx, st, "keypoint_gate");
    k_gate_flags<<<nb, 256, 0, st>>>(b.keys, dK, n, b.sn, q->keypoint_min_curvature, b.flags);
    scan_exclusive(b.flags, b.pos, b.tiles, n, n, nullptr, reinterpret_cast<uint32_t*>(dKg), st);
    k_compact_int<<<nb, 256, 0, st>>>(b.keys, b.flags, b.pos, n, b.keys2);
    RTR_LAUNCHED(2);
    keys = b.keys2;
    dKeys = dKg;
  }
  {
    ProfScope ps(ctx, st, "shot352");
    RTR_TRY(shot_on_grid(b.shot_grid, b.sv, b.sn, keys, n, dKeys, q->descriptor_r, b.desc, nullptr, st));
  }
  const float* desc = b.desc;
  if (mlp) {
    // learned pruning: keep the ceil(keep * K) most credible keypoints (ties:
    // lower keypoint index), in their original order
    ProfScope ps(ctx, st, "prune");
    Scratch t = stage;
    float* score = t.take<float>(n);
    uint32_t* k0 = t.take<uint32_t>(n);
    uint32_t* v0 = t.take<uint32_t>(n);
    uint32_t* k1 = t.take<uint32_t>(n);
    uint32_t* v1 = t.take<uint32_t>(n);
    uint32_t* hist = t.take<uint32_t>(radix_hist_entries(n));
    if (!hist) return fail(RTR_ERR_CAPACITY, "rtr_recognize_learned: scratch carve");
    {
      ProfScope ps2(ctx, st, "prune_score");
      RTR_TRY(mlp_score_rows(ctx, t, mlp, b.desc, n, dKeys, score, st));
    }
    {
      ProfScope ps2(ctx, st, "prune_select");
      k_score_keys<<<nb, 256, 0, st>>>(score, dKeys, n, k0);
      uint32_t *ks, *vs;
      radix_sort_pairs(k0, v0, k1, v1, hist, n, n, dKeys, 32, true, st, &ks, &vs);
      k_mark_top<<<nb, 256, 0, st>>>(vs, dKeys, n, keep, b.flags);
    }
    ProfScope ps2(ctx, st, "prune_compact");
    scan_exclusive(b.flags, b.pos, b.tiles, n, n, nullptr, reinterpret_cast<uint32_t*>(b.cnt + 3), st);
    k_compact_int<<<nb, 256, 0, st>>>(keys, b.flags, b.pos, n, b.keys_p);
    k_compact_rows<<<nblocks(n, 8, 152 * 16), 256, 0, st>>>(b.desc, b.flags, b.pos, dKeys, n, b.desc_p);
    RTR_LAUNCHED(4);
    keys = b.keys_p;
    dKeys = b.cnt + 3;
    desc = b.desc_p;
  }
  b.grid_ready = ctx->ev_side[2];  // the scene grid: joined by model_stages
  b.keys_m = keys;
  b.d_nk = dKeys;
  b.desc_m = desc;
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

// One model against a scene whose stages are done: matching,
// correspondences, grouping, verification, ICP refinement, final scoring.
// Every count stays on the device (no host round trip): the stages are sized
// for their capacities (n correspondences, max_clusters hypotheses,
// refine_top refinements) and read the live counts.
static rtr_status model_stages(rtr_context* ctx, const Scratch& stage, const SceneBufs& sb, ModelBufs& b,
                               const rtr_model* m, int n, const rtr_recog_params* q, rtr_recog_result* out,
                               cudaStream_t st) {
  int* dC = b.cnt;
  int* dNcl = b.cnt + 1;
  int* dM = b.cnt + 2;
  const int nb = nblocks(n);
  {
    ProfScope ps(ctx, st, "match");
    Scratch t = stage;
    RTR_TRY(match_tc_dev(ctx, t, sb.desc_m, n, sb.d_nk, m->desc, m->n_kp, m->db_hi, m->db_lo, m->db_n2, b.midx,
                         b.md2, st));
  }
  {
    ProfScope ps(ctx, st, "correspondences");
    k_corr_flags<<<nb, 256, 0, st>>>(b.midx, b.md2, sb.d_nk, n, q->match_max_d2, b.flags);
    scan_exclusive(b.flags, b.pos, b.tiles, n, n, nullptr, reinterpret_cast<uint32_t*>(dC), st);
    k_corr_scatter<<<nb, 256, 0, st>>>(b.midx, b.md2, b.flags, b.pos, n, b.cm, b.cs, b.cd);
    k_gather_kp<<<nb, 256, 0, st>>>(sb.sv, sb.keys_m, sb.d_nk, n, b.skp);
    RTR_LAUNCHED(3);
  }
  {
    ProfScope ps(ctx, st, "gc_group");
    Scratch t = stage;
    RTR_TRY(gc_group_async(ctx, t, reinterpret_cast<const float*>(m->kp), reinterpret_cast<const float*>(b.skp), b.cm,
                           b.cs, b.cd, n, dC, q->gc_size, q->gc_thresh, q->max_clusters, b.sizes, b.poses, dNcl,
                           st));
  }
  const int H = q->max_clusters, M = q->refine_top;
  if (sb.grid_ready) RTR_CUDA(cudaStreamWaitEvent(st, sb.grid_ready, 0));  // the scene grid (side stream)
  {
    ProfScope ps(ctx, st, "verify");
    RTR_TRY(hv_score(grid_dev(sb.grid), m->vox, m->n_vox, q->hv_subsample > 0 ? q->hv_subsample : 1, b.poses, H,
                     dNcl, q->hv_inlier_r * q->hv_inlier_r, b.hvcnt, b.hv, st));
    k_topm<<<1, 32, 0, st>>>(b.hv, H, dNcl, M, b.order, dM);
    k_select_poses<<<1, 256, 0, st>>>(b.poses, b.order, M, b.init);
    RTR_LAUNCHED(2);
  }
  {
    ProfScope ps(ctx, st, "icp_refine");
    Scratch t = stage;
    std::vector<IcpSpec> specs((size_t)M);
    for (int k = 0; k < M; ++k) {
      IcpDev& d = specs[k].dev;
      memset(&d, 0, sizeof(d));
      d.grid = grid_dev(sb.grid);
      d.src_meta = m->vox_meta;
      d.src = m->vox;
      d.src_idx = nullptr;
      d.n_src = m->n_vox;
      d.max_it = q->icp_iterations;
      d.r2max = q->icp_max_dist * q->icp_max_dist;
      d.eps_t = 0.0;
      d.eps_r = 0.0;
      for (int e = 0; e < 16; ++e) d.init[e] = (e % 5) == 0 ? 1.0 : 0.0;
      d.result = b.res + k;
      d.d_active = dM;  // slots past the hypotheses found leave at once
      d.slot = k;
      specs[k].init_dev = b.init + 16 * k;
    }
    RTR_TRY(icp_multi(ctx, t, specs, st));
  }
  {
    ProfScope ps(ctx, st, "final_score");
    k_copy_result_poses<<<1, 256, 0, st>>>(b.res, M, b.refined);
    RTR_TRY(hv_score(grid_dev(sb.grid), m->vox, m->n_vox, 1, b.refined, M, dM,
                     q->accept_inlier_r * q->accept_inlier_r, b.hvcnt, b.fscore, st));
    const float nms2 = q->nms_dist * q->nms_dist;
    k_finalize<<<1, 32, 0, st>>>(b.fscore, b.refined, b.order, b.sizes, M, dM, q->accept_score, nms2,
                                 q->max_instances, sb.cnt, sb.d_nk, dC, dNcl, ctx->d_status, out);
    RTR_LAUNCHED(2);
  }
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

static rtr_status recognize_impl(rtr_context* ctx, const rtr_model* m, const float4* scene, int n,
                                 const rtr_recog_params* q, rtr_recog_result* out, cudaStream_t st,
                                 const rtr_mlp* mlp = nullptr, float keep = 1.f) {
  const bool learned = mlp != nullptr;
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, recognize_scratch_bytes(n, q, learned), st, &s));
  SceneBufs sb;
  ModelBufs mb;
  if (!scene_take(s, n, learned, &sb) || !model_take(s, n, q, &mb))
    return fail(RTR_ERR_CAPACITY, "rtr_recognize: scratch carve");
  const Scratch stage = s;  // everything after this point is per-stage scratch
  RTR_TRY(scene_stages(ctx, stage, sb, scene, n, q, mlp, keep, st));
  return model_stages(ctx, stage, sb, mb, m, n, q, out, st);
}

// Several models in one scene: the scene's stages once on the caller's
// stream, then each model's stages on a worker's stream (forked and joined
// with events), or all on the caller's stream with one worker.
static rtr_status recognize_multi_impl(rtr_context* ctx, const rtr_model* const* models, int nm, const float4* scene,
                                       int n, const rtr_recog_params* q, const rtr_mlp* mlp, float keep,
                                       rtr_recog_result* out, int nw, cudaStream_t st) {
  const bool learned = mlp != nullptr;
  const size_t stage_b = stage_bytes(n, q, learned);
  ScratchPlan sp;
  scene_plan(sp, n, learned);
  if (nw <= 1) model_plan(sp, n, q);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, sp.bytes + stage_b + 4096, st, &s));
  SceneBufs sb;
  if (!scene_take(s, n, learned, &sb)) return fail(RTR_ERR_CAPACITY, "rtr_recognize_multi: scratch carve");
  if (nw <= 1) {
    ModelBufs mb;
    if (!model_take(s, n, q, &mb)) return fail(RTR_ERR_CAPACITY, "rtr_recognize_multi: scratch carve");
    const Scratch stage = s;
    RTR_TRY(scene_stages(ctx, stage, sb, scene, n, q, mlp, keep, st));
    for (int i = 0; i < nm; ++i) RTR_TRY(model_stages(ctx, stage, sb, mb, models[i], n, q, out + i, st));
    return RTR_OK;
  }
  RTR_TRY(scene_stages(ctx, s, sb, scene, n, q, mlp, keep, st));
  RTR_CUDA(cudaStreamWaitEvent(st, sb.grid_ready, 0));  // joined before the workers fork
  RTR_TRY(batch_ensure_workers(ctx, nw));
  ScratchPlan mp;
  model_plan(mp, n, q);
  for (int wi = 0; wi < nw; ++wi) {  // sized before the fork: growing synchronises
    Scratch ws;
    RTR_TRY(ensure_scratch(ctx->workers[wi], mp.bytes + stage_b + 4096, ctx->workers[wi]->host_stream, &ws));
  }
  RTR_CUDA(cudaSetDevice(ctx->device));
  RTR_CUDA(cudaEventRecord(ctx->ev_fork, st));
  for (int wi = 0; wi < nw; ++wi) RTR_CUDA(cudaStreamWaitEvent(ctx->workers[wi]->host_stream, ctx->ev_fork, 0));
  for (int i = 0; i < nm; ++i) {
    rtr_context* w = ctx->workers[i % nw];
    Scratch ws;
    RTR_TRY(ensure_scratch(w, mp.bytes + stage_b + 4096, w->host_stream, &ws));
    ModelBufs mb;
    if (!model_take(ws, n, q, &mb)) return fail(RTR_ERR_CAPACITY, "rtr_recognize_multi: scratch carve");
    const rtr_status r = model_stages(w, ws, sb, mb, models[i], n, q, out + i, w->host_stream);
    if (r != RTR_OK) return fail(r, "rtr_recognize_multi: model %d: %s", i, rtr_last_error());
  }
  for (int wi = 0; wi < nw; ++wi) {
    rtr_context* w = ctx->workers[wi];
    RTR_CUDA(cudaEventRecord(w->ev_fork, w->host_stream));
    RTR_CUDA(cudaStreamWaitEvent(st, w->ev_fork, 0));
  }
  RTR_CUDA(cudaSetDevice(ctx->device));
  return RTR_OK;
}

// A recognition enqueued through the context's graph slot.  The first call
// with a key runs directly (sizing the arena); the second identical call
// captures the same enqueue sequence on a private stream into a CUDA graph
// and launches it on the caller's stream; later identical calls only launch
// the graph: the same kernels with the same arguments, without the host's
// per-launch cost (~150 launches a recognition).  Any change of key (inputs'
// addresses, parameters, model or network, arena, tuning) runs directly
// again.  Off while profiling, inside a caller's own capture, and on batch
// workers.
static rtr_status recognize_cached(rtr_context* ctx, const rtr_model* m, const float4* scene, int n,
                                   const rtr_recog_params* q, rtr_recog_result* out, cudaStream_t st,
                                   const rtr_mlp* mlp, float keep) {
  if (!ctx->auto_graph || ctx->profiling || stream_is_capturing(st))
    return recognize_impl(ctx, m, scene, n, q, out, st, mlp, keep);
  RecogGraphSlot& g = ctx->rgraph;
  const float* sc = reinterpret_cast<const float*>(scene);
  const bool same = g.model == m && g.model_uid == m->uid && g.mlp == mlp && g.mlp_uid == rtr_mlp_uid(mlp) &&
                    g.keep == keep && g.scene == sc && g.n == n && g.result == out &&
                    memcmp(&g.params, q, sizeof(*q)) == 0 && g.scratch_gen == ctx->scratch_gen &&
                    g.cfg_gen == ctx->cfg_gen;
  if (same && g.exec) {
    RTR_CUDA(cudaGraphLaunch(g.exec, st));
    RTR_LAUNCHED(g.launches);
    return RTR_OK;
  }
  if (!same) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = RecogGraphSlot();
    g.model = m;
    g.model_uid = m->uid;
    g.mlp = mlp;
    g.mlp_uid = rtr_mlp_uid(mlp);
    g.keep = keep;
    g.scene = sc;
    g.n = n;
    g.result = out;
    g.params = *q;
    g.cfg_gen = ctx->cfg_gen;
  }
  if (!g.armed || g.failed) {
    const rtr_status r = recognize_impl(ctx, m, scene, n, q, out, st, mlp, keep);
    g.armed = r == RTR_OK;
    g.scratch_gen = ctx->scratch_gen;  // after any growth of this call
    return r;
  }
  if (!ctx->cap_stream) RTR_CUDA(cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking));
  const uint64_t l0 = g_launches.load();
  RTR_CUDA(cudaStreamBeginCapture(ctx->cap_stream, cudaStreamCaptureModeThreadLocal));
  const rtr_status r = recognize_impl(ctx, m, scene, n, q, out, ctx->cap_stream, mlp, keep);
  cudaGraph_t graph = nullptr;
  const cudaError_t e = cudaStreamEndCapture(ctx->cap_stream, &graph);
  const uint64_t nl = g_launches.load() - l0;
  g_launches.fetch_sub(nl);  // captured, not launched
  cudaGraphExec_t x = nullptr;
  if (r == RTR_OK && e == cudaSuccess && graph && ctx->scratch_gen == g.scratch_gen &&
      cudaGraphInstantiate(&x, graph, 0) == cudaSuccess) {
    cudaGraphDestroy(graph);
    g.exec = x;
    g.launches = nl;
    RTR_CUDA(cudaGraphLaunch(g.exec, st));
    RTR_LAUNCHED(nl);
    return RTR_OK;
  }
  if (graph) cudaGraphDestroy(graph);
  cudaGetLastError();
  g.failed = true;
  return recognize_impl(ctx, m, scene, n, q, out, st, mlp, keep);
}

}  // namespace rtr

extern "C" {

rtr_status rtr_recognize(rtr_context* ctx, const rtr_model* model, const float* d_scene, int n,
                         const rtr_recog_params* p, rtr_recog_result* d_result, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && model && p && d_result && n >= 0, "rtr_recognize: bad arguments");
  RTR_CHECK_ARG(n == 0 || d_scene, "rtr_recognize: NULL scene");
  RTR_CHECK_ARG(p->max_clusters >= 1 && p->max_clusters <= 256 && p->refine_top >= 1 && p->refine_top <= 64 &&
                    p->max_instances >= 1 && p->max_instances <= RTR_MAX_INSTANCES && p->voxel_leaf > 0.f &&
                    p->descriptor_r > 0.f && p->scene_keypoint_r > 0.f && p->icp_iterations >= 1,
                "rtr_recognize: parameter out of range");
  RTR_CHECK_ARG(((uintptr_t)d_scene & 15) == 0, "rtr_recognize: scene must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (n == 0) {
    k_result_empty<<<1, 256, 0, st>>>(d_result, 1);
    RTR_LAUNCHED(1);
    RTR_CUDA(cudaGetLastError());
    return RTR_OK;
  }
  return recognize_cached(ctx, model, reinterpret_cast<const float4*>(d_scene), n, p, d_result, st, nullptr, 1.f);
}

rtr_status rtr_recognize_learned(rtr_context* ctx, const rtr_model* model, const rtr_mlp* mlp, float keep,
                                 const float* d_scene, int n, const rtr_recog_params* p, rtr_recog_result* d_result,
                                 rtr_stream_t stream) {
  RTR_CHECK_ARG(mlp && keep > 0.f && keep <= 1.f, "rtr_recognize_learned: need an MLP and keep in (0, 1]");
  RTR_CHECK_ARG(ctx && model && p && d_result && n >= 0, "rtr_recognize_learned: bad arguments");
  RTR_CHECK_ARG(n == 0 || d_scene, "rtr_recognize_learned: NULL scene");
  RTR_CHECK_ARG(p->max_clusters >= 1 && p->max_clusters <= 256 && p->refine_top >= 1 && p->refine_top <= 64 &&
                    p->max_instances >= 1 && p->max_instances <= RTR_MAX_INSTANCES && p->voxel_leaf > 0.f &&
                    p->descriptor_r > 0.f && p->scene_keypoint_r > 0.f && p->icp_iterations >= 1,
                "rtr_recognize_learned: parameter out of range");
  RTR_CHECK_ARG(((uintptr_t)d_scene & 15) == 0, "rtr_recognize_learned: scene must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (n == 0) {
    k_result_empty<<<1, 256, 0, st>>>(d_result, 1);
    RTR_LAUNCHED(1);
    RTR_CUDA(cudaGetLastError());
    return RTR_OK;
  }
  return recognize_cached(ctx, model, reinterpret_cast<const float4*>(d_scene), n, p, d_result, st, mlp, keep);
}

rtr_status rtr_recognize_multi(rtr_context* ctx, const rtr_model* const* h_models, int n_models, const rtr_mlp* mlp,
                               float keep, const float* d_scene, int n, const rtr_recog_params* p,
                               rtr_recog_result* d_results, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && p && n >= 0 && n_models >= 0 && (n_models == 0 || (h_models && d_results)),
                "rtr_recognize_multi: bad arguments");
  for (int i = 0; i < n_models; ++i) RTR_CHECK_ARG(h_models[i], "rtr_recognize_multi: model %d is NULL", i);
  RTR_CHECK_ARG(!mlp || (keep > 0.f && keep <= 1.f), "rtr_recognize_multi: keep must be in (0, 1]");
  RTR_CHECK_ARG(n == 0 || d_scene, "rtr_recognize_multi: NULL scene");
  RTR_CHECK_ARG(p->max_clusters >= 1 && p->max_clusters <= 256 && p->refine_top >= 1 && p->refine_top <= 64 &&
                    p->max_instances >= 1 && p->max_instances <= RTR_MAX_INSTANCES && p->voxel_leaf > 0.f &&
                    p->descriptor_r > 0.f && p->scene_keypoint_r > 0.f && p->icp_iterations >= 1,
                "rtr_recognize_multi: parameter out of range");
  RTR_CHECK_ARG(((uintptr_t)d_scene & 15) == 0, "rtr_recognize_multi: scene must be 16-byte aligned");
  if (n_models == 0) return RTR_OK;
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (n == 0) {
    k_result_empty<<<1, 256, 0, st>>>(d_results, n_models);
    RTR_LAUNCHED(1);
    RTR_CUDA(cudaGetLastError());
    RTR_CUDA(cudaStreamSynchronize(st));
    return RTR_OK;
  }
  const int nw = batch_worker_count(ctx, n_models);
  RTR_TRY(recognize_multi_impl(ctx, h_models, n_models, reinterpret_cast<const float4*>(d_scene), n, p, mlp, keep,
                               d_results, nw, st));
  RTR_CUDA(cudaStreamSynchronize(st));
  RTR_TRY(rtr_context_check(ctx, st));
  return nw > 1 ? batch_check_workers(ctx, nw) : RTR_OK;
}

rtr_status rtr_recognize_host(rtr_context* ctx, const rtr_model* model, const float* h_scene, int n,
                              const rtr_recog_params* p, rtr_recog_result* h_result) {
  RTR_CHECK_ARG(ctx && model && p && h_result && h_scene && n > 0, "rtr_recognize_host: bad arguments");
  RTR_CUDA(cudaSetDevice(ctx->device));
  const size_t bs = ((size_t)n * 16 + 255) & ~size_t(255);
  RTR_TRY(ensure_io(ctx, bs + sizeof(rtr_recog_result) + 256));
  char* io = static_cast<char*>(ctx->io);
  float* d_scene = reinterpret_cast<float*>(io);
  rtr_recog_result* d_res = reinterpret_cast<rtr_recog_result*>(io + bs);
  cudaStream_t st = ctx->host_stream;
  RTR_CUDA(cudaMemcpyAsync(d_scene, h_scene, (size_t)n * 16, cudaMemcpyHostToDevice, st));
  RTR_TRY(rtr_recognize(ctx, model, d_scene, n, p, d_res, st));
  RTR_CUDA(cudaMemcpyAsync(h_result, d_res, sizeof(rtr_recog_result), cudaMemcpyDeviceToHost, st));
  return rtr_context_check(ctx, st);
}

rtr_status rtr_pose_inliers(rtr_context* ctx, const float* d_model, int n_model, const float* d_scene, int n_scene,
                            const double* d_poses, int n_poses, float radius, int32_t* d_counts,
                            rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n_model >= 0 && n_scene >= 0 && n_poses >= 0, "rtr_pose_inliers: bad arguments");
  RTR_CHECK_ARG(radius > 0.f && radius < 1.0e18f, "rtr_pose_inliers: radius must be finite and > 0");
  if (n_poses == 0) return RTR_OK;
  RTR_CHECK_ARG(d_poses && d_counts, "rtr_pose_inliers: NULL poses or counts");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (n_model == 0 || n_scene == 0) {
    RTR_CUDA(cudaMemsetAsync(d_counts, 0, sizeof(int32_t) * (size_t)n_poses, st));
    return RTR_OK;
  }
  RTR_CHECK_ARG(d_model && d_scene, "rtr_pose_inliers: NULL model or scene");
  const unsigned cap = default_cell_cap(n_scene);
  ScratchPlan plan;
  grid_plan(plan, n_scene, cap);
  plan.add<float>(n_poses);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  GridBufs gb;
  if (!grid_take(s, n_scene, cap, &gb)) return fail(RTR_ERR_CAPACITY, "rtr_pose_inliers: scratch");
  float* score = s.take<float>(n_poses);
  if (!score) return fail(RTR_ERR_CAPACITY, "rtr_pose_inliers: scratch");
  ProfScope ps(ctx, st, "pose_inliers");
  // a cell 1.5 x the radius: the counts take the 27-cell existence search
  grid_build(gb, reinterpret_cast<const float4*>(d_scene), n_scene, nullptr, 1.5f * radius, st);
  RTR_TRY(hv_score(grid_dev(gb), reinterpret_cast<const float4*>(d_model), n_model, 1, d_poses, n_poses, nullptr,
                   radius * radius, d_counts, score, st));
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

}  // extern "C"
