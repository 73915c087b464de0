// tdf.cu — truncated distance field of occupied voxels.
//
// Replaces ComputeTDF / ComputeTDFWithCuda (kernel.cu:8-106).  For every voxel
// v = (x, y, z) of a dim^3 grid (x fastest), value = min(900, min_i |v - o_i|^2)
// over the integer occupied voxels o_i, stored as float (kernel.cu:20-30).
// All values are integers below 2^24, so the float result is exact and equal to
// the reference's.
//
// Layout here: one CTA per keypoint; the occupied list is staged through shared
// memory in chunks; thread (y, z) owns the whole x-row of dim voxels in
// registers, so dy^2 + dz^2 is computed once per occupied voxel per row.
#include <string.h>

#include "common.cuh"

namespace rtr {

constexpr int TDF_MAXDIM = 32;
constexpr int TDF_CHUNK = 2048;
constexpr int TDF_THREADS = 1024;

__global__ void __launch_bounds__(TDF_THREADS) k_tdf(const int* __restrict__ occ,
                                                     const int* __restrict__ offsets, int dim,
                                                     float* __restrict__ out) {
  __shared__ int s_occ[TDF_CHUNK * 3];
  const int key = blockIdx.x;
  const int beg = offsets[key], end = offsets[key + 1];
  const int rows = dim * dim;
  const size_t vol = (size_t)dim * dim * dim;
  float* o = out + (size_t)key * vol;
  for (int r0 = 0; r0 < rows; r0 += TDF_THREADS) {
    const int row = r0 + (int)threadIdx.x;
    const int y = row % dim, z = row / dim;
    int best[TDF_MAXDIM];
#pragma unroll
    for (int x = 0; x < TDF_MAXDIM; ++x) best[x] = 900;
    for (int c0 = beg; c0 < end; c0 += TDF_CHUNK) {
      const int cn = min(TDF_CHUNK, end - c0);
      __syncthreads();
      for (int i = threadIdx.x; i < cn * 3; i += TDF_THREADS) s_occ[i] = occ[(size_t)c0 * 3 + i];
      __syncthreads();
      if (row < rows) {
        for (int i = 0; i < cn; ++i) {
          const int ox = s_occ[3 * i], oy = s_occ[3 * i + 1], oz = s_occ[3 * i + 2];
          const int dy = y - oy, dz = z - oz;
          const int dyz = dy * dy + dz * dz;
          if (dyz >= 900) continue;
#pragma unroll
          for (int x = 0; x < TDF_MAXDIM; ++x) {
            const int dx = x - ox;
            best[x] = min(best[x], dx * dx + dyz);
          }
        }
      }
    }
    if (row < rows) {
#pragma unroll
      for (int x = 0; x < TDF_MAXDIM; ++x)
        if (x < dim) o[(size_t)row * dim + x] = (float)best[x];
    }
  }
}

// The reference kernel's guard lets thread dim^3 write the voxel (0, 0, dim).
__global__ void k_tdf_extra(const int* __restrict__ occ, int n_occ, int dim, float* __restrict__ out) {
  int best = 900;
  for (int i = threadIdx.x; i < n_occ; i += blockDim.x) {
    const int dx = 0 - occ[3 * i], dy = 0 - occ[3 * i + 1], dz = dim - occ[3 * i + 2];
    best = min(best, dx * dx + dy * dy + dz * dz);
  }
  for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, o));
  if (threadIdx.x == 0) out[(size_t)dim * dim * dim] = (float)best;
}

// Device buffers of the host-pointer shim, kept between calls (one host
// thread at a time, as with the reference).
struct TdfShim {
  int* occ = nullptr;
  size_t occ_cap = 0;
  float* tdf = nullptr;
  int* offs = nullptr;
};
static TdfShim g_tdf;

}  // namespace rtr

using namespace rtr;

extern "C" {

rtr_status rtr_tdf_batch(rtr_context* ctx, const int* d_occ, const int* d_offsets, int n_keys, int dim,
                         float* d_tdf, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n_keys >= 0, "rtr_tdf_batch: bad arguments");
  RTR_CHECK_ARG(dim >= 1 && dim <= TDF_MAXDIM, "rtr_tdf_batch: dim must be in [1, %d]", TDF_MAXDIM);
  if (n_keys == 0) return RTR_OK;
  RTR_CHECK_ARG(d_offsets && d_tdf, "rtr_tdf_batch: NULL offsets or output");
  RTR_CUDA(cudaSetDevice(ctx->device));
  ProfScope ps(ctx, (cudaStream_t)stream, "tdf");
  RTR_LAUNCHED(1);
  k_tdf<<<n_keys, TDF_THREADS, 0, (cudaStream_t)stream>>>(d_occ, d_offsets, dim, d_tdf);
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

int ComputeTDFWithCuda(const int* voxel_grid_occ, float* voxel_grid_TDF, int voxel_grid_dim,
                       int num_occ) {
  const int dim = voxel_grid_dim;
  if (dim < 1 || (long long)dim * dim * dim > 27000 || num_occ < 0 || !voxel_grid_TDF ||
      (num_occ > 0 && !voxel_grid_occ)) {
    set_error("ComputeTDFWithCuda: dim^3 must be in [1, 27000] and num_occ >= 0");
    return (int)cudaErrorInvalidValue;
  }
  cudaError_t e = cudaSetDevice(0);
  if (e != cudaSuccess) return (int)e;
  TdfShim& S = g_tdf;
  if ((size_t)num_occ > S.occ_cap || !S.occ) {
    if (S.occ) cudaFree(S.occ);
    S.occ = nullptr;
    size_t cap = (size_t)(num_occ > 4096 ? num_occ : 4096);
    if ((e = cudaMalloc(&S.occ, cap * 3 * sizeof(int))) != cudaSuccess) return (int)e;
    S.occ_cap = cap;
  }
  if (!S.tdf && (e = cudaMalloc(&S.tdf, 27001 * sizeof(float))) != cudaSuccess) return (int)e;
  if (!S.offs && (e = cudaMalloc(&S.offs, 2 * sizeof(int))) != cudaSuccess) return (int)e;
  const int offs[2] = {0, num_occ};
  if ((e = cudaMemcpy(S.offs, offs, sizeof(offs), cudaMemcpyHostToDevice)) != cudaSuccess) return (int)e;
  if (num_occ > 0 &&
      (e = cudaMemcpy(S.occ, voxel_grid_occ, (size_t)num_occ * 3 * sizeof(int), cudaMemcpyHostToDevice)) !=
          cudaSuccess)
    return (int)e;
  const int vol = dim * dim * dim;
  k_tdf<<<1, TDF_THREADS>>>(S.occ, S.offs, dim, S.tdf);
  const bool extra = vol < 27000;
  if (extra) k_tdf_extra<<<1, 32>>>(S.occ, num_occ, dim, S.tdf);
  RTR_LAUNCHED(extra ? 2 : 1);
  if ((e = cudaGetLastError()) != cudaSuccess) return (int)e;
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return (int)e;
  e = cudaMemcpy(voxel_grid_TDF, S.tdf, (size_t)(vol + (extra ? 1 : 0)) * sizeof(float),
                 cudaMemcpyDeviceToHost);
  return (int)e;
}

}  // extern "C"
