// match.cu — descriptor 1-NN (scene keypoint -> nearest model keypoint).
//
// Distances are FP32 sums over the 352 dimensions in index order, each term
// ((a_k - b_k) * (a_k - b_k)) and each addition rounded separately, ties to
// the lowest model index: the rule of the CPU oracle, so indices and distances
// agree bit for bit.  This is the exact SIMT kernel; it also re-ranks the
// tensor-core candidates.
#include "common.cuh"

namespace rtr {

constexpr int MT_DIM = 352;
constexpr int MT_Q = 32;   // queries per block
constexpr int MT_T = 32;   // database descriptors per tile (one per lane)
constexpr int MT_WARPS = 8;

__device__ __forceinline__ int mcount(int n_host, const int* d_n) { return d_n ? *d_n : n_host; }

__global__ void __launch_bounds__(MT_WARPS * 32) k_match_exact(const float* __restrict__ q, int nq_host,
                                                               const int* d_nq, const float* __restrict__ db,
                                                               int ndb, int* __restrict__ out_idx,
                                                               float* __restrict__ out_d2) {
  extern __shared__ float sm[];
  float* sq = sm;                       // [MT_Q][MT_DIM]
  float* st = sm + MT_Q * MT_DIM;       // [MT_DIM][MT_T] (k-major: conflict-free per lane)
  const int nq = mcount(nq_host, d_nq);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int q0 = blockIdx.x * MT_Q; q0 < nq; q0 += gridDim.x * MT_Q) {
    __syncthreads();
    for (int i = threadIdx.x; i < MT_Q * MT_DIM; i += blockDim.x) {
      const int r = i / MT_DIM;
      sq[i] = (q0 + r < nq) ? q[(size_t)(q0 + r) * MT_DIM + (i - r * MT_DIM)] : 0.f;
    }
    float bd[MT_Q / MT_WARPS];
    int bi[MT_Q / MT_WARPS];
#pragma unroll
    for (int s = 0; s < MT_Q / MT_WARPS; ++s) {
      bd[s] = __int_as_float(0x7f800000);
      bi[s] = 0x7fffffff;
    }
    for (int t0 = 0; t0 < ndb; t0 += MT_T) {
      __syncthreads();
      for (int i = threadIdx.x; i < MT_T * MT_DIM; i += blockDim.x) {
        const int r = i / MT_DIM, k = i - r * MT_DIM;
        st[k * MT_T + r] = (t0 + r < ndb) ? db[(size_t)(t0 + r) * MT_DIM + k] : 0.f;
      }
      __syncthreads();
      const int j = t0 + lane;
#pragma unroll
      for (int s = 0; s < MT_Q / MT_WARPS; ++s) {
        const float* a = sq + (wid * (MT_Q / MT_WARPS) + s) * MT_DIM;
        float acc = 0.f;
#pragma unroll 8
        for (int k = 0; k < MT_DIM; ++k) {
          const float t = __fsub_rn(a[k], st[k * MT_T + lane]);
          acc = __fadd_rn(acc, __fmul_rn(t, t));
        }
        if (j < ndb && acc < bd[s]) {
          bd[s] = acc;
          bi[s] = j;
        }
      }
    }
#pragma unroll
    for (int s = 0; s < MT_Q / MT_WARPS; ++s) {
      float d = bd[s];
      int i = bi[s];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float od = __shfl_xor_sync(0xffffffffu, d, o);
        const int oi = __shfl_xor_sync(0xffffffffu, i, o);
        if (od < d || (od == d && oi < i)) {
          d = od;
          i = oi;
        }
      }
      const int qi = q0 + wid * (MT_Q / MT_WARPS) + s;
      if (lane == 0 && qi < nq) {
        out_idx[qi] = i == 0x7fffffff ? -1 : i;
        if (out_d2) out_d2[qi] = d;
      }
    }
  }
}

rtr_status match_exact_dev(const float* q, int nq_cap, const int* d_nq, const float* db, int ndb, int* idx,
                           float* d2, cudaStream_t st) {
  const size_t smem = (size_t)(MT_Q + MT_T) * MT_DIM * sizeof(float);
  // per call: the attribute is per device, and calls may come from several threads
  RTR_CUDA(cudaFuncSetAttribute(k_match_exact, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int blocks = (nq_cap + MT_Q - 1) / MT_Q;
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  k_match_exact<<<blocks, MT_WARPS * 32, smem, st>>>(q, nq_cap, d_nq, db, ndb, idx, d2);
  RTR_LAUNCHED(1);
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

}  // namespace rtr

using namespace rtr;

extern "C" rtr_status rtr_match_exact(rtr_context* ctx, const float* d_query, int n_query, const float* d_db,
                                      int n_db, int32_t* d_idx, float* d_d2, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n_query >= 0 && n_db >= 0, "rtr_match_exact: bad arguments");
  if (n_query == 0) return RTR_OK;
  RTR_CHECK_ARG(d_query && d_idx, "rtr_match_exact: NULL query or output");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (n_db == 0) {
    RTR_CUDA(cudaMemsetAsync(d_idx, 0xff, (size_t)n_query * 4, st));
    return RTR_OK;
  }
  RTR_CHECK_ARG(d_db != nullptr, "rtr_match_exact: NULL database");
  ProfScope ps(ctx, st, "match_exact");
  return match_exact_dev(d_query, n_query, nullptr, d_db, n_db, d_idx, d_d2, st);
}
