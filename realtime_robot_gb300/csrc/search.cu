// search.cu — rtr_knn1 / rtr_knn entry points over the radix-sorted grid.
#include <string.h>

#include <mutex>

#include "search.cuh"

namespace rtr {

constexpr int KNN1_G = 8;  // lanes per query

__global__ void __launch_bounds__(128) k_knn1(GridDev gd, const float4* __restrict__ q, int nq,
                                              float r2max, int* __restrict__ out_idx,
                                              float* __restrict__ out_d2) {
  const GridView g = load_view(gd);
  constexpr int G = KNN1_G;
  const int lane = threadIdx.x & 31, lg = lane & (G - 1);
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));
  const int qpb = blockDim.x / G;
  for (int i = blockIdx.x * qpb + threadIdx.x / G; i < nq; i += gridDim.x * qpb) {
    float d2;
    int bi, bp;
    grid_nn1_group<G>(g, q[i], r2max, lg, gmask, d2, bi, bp);
    if (lg == 0) {
      out_idx[i] = bi;
      if (out_d2) out_d2[i] = d2;
    }
  }
}

template <int K>
__global__ void __launch_bounds__(128) k_knn(GridDev gd, const float4* __restrict__ q, int nq, int k,
                                             int* __restrict__ out_idx, float* __restrict__ out_d2) {
  const GridView g = load_view(gd);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x) {
    float bd[K];
    int bi[K];
    grid_knn<K>(g, q[i], bd, bi);
#pragma unroll
    for (int s = 0; s < K; ++s) {
      if (s < k) {
        const bool ok = bi[s] != INT_MAX;
        out_idx[(size_t)i * k + s] = ok ? bi[s] : -1;
        if (out_d2) out_d2[(size_t)i * k + s] = ok ? bd[s] : __int_as_float(0x7f800000);
      }
    }
  }
}

static int search_blocks(int n) {
  int b = (n + 127) / 128;
  return b < 1 ? 1 : b;
}

// Fixed grid storage of rtr_knn1_static: the grid of up to
// RTR_KNN1_STATIC_MAX_TARGET points with the default cell table
// (8 cells per point) needs about 6.6 MB.
constexpr size_t KNN1_STATIC_BYTES = size_t(7) << 20;
static __device__ __align__(256) unsigned char g_knn1_static[KNN1_STATIC_BYTES];

constexpr int KNN1_STATIC_DEVICES = 64;
static std::mutex g_knn1_static_mu;
static void* g_knn1_static_ptr[KNN1_STATIC_DEVICES];

// A pointer rtr_knn1_static may hand to its kernel on device `dev`: device
// memory of that device, or managed memory.  cudaPointerGetAttributes reads
// the driver's records and allocates nothing.
static bool on_device(const void* p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace rtr

using namespace rtr;

extern "C" {

rtr_status rtr_knn1(rtr_context* ctx, const float* d_query, int n_query, const float* d_target,
                    int n_target, float max_dist, int32_t* d_out_idx, float* d_out_d2,
                    rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n_query >= 0 && n_target >= 0, "rtr_knn1: bad arguments");
  if (n_query == 0) return RTR_OK;
  RTR_CHECK_ARG(d_query && d_out_idx, "rtr_knn1: NULL query or output");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (n_target == 0) {
    RTR_CUDA(cudaMemsetAsync(d_out_idx, 0xff, (size_t)n_query * 4, st));
    return RTR_OK;  // d_out_d2 left as is: every index is -1
  }
  RTR_CHECK_ARG(d_target != nullptr, "rtr_knn1: NULL target");
  const unsigned cap = default_cell_cap(n_target);
  ScratchPlan plan;
  grid_plan(plan, n_target, cap);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  GridBufs gb;
  if (!grid_take(s, n_target, cap, &gb)) return fail(RTR_ERR_CAPACITY, "rtr_knn1: scratch");
  const bool bounded = max_dist > 0.f && max_dist < 1e18f;
  grid_build(gb, reinterpret_cast<const float4*>(d_target), n_target, nullptr,
             bounded ? 0.5f * max_dist : -1.f, st);
  ProfScope ps(ctx, st, "knn1");
  RTR_LAUNCHED(1);
  k_knn1<<<search_blocks(n_query * KNN1_G), 128, 0, st>>>(grid_dev(gb), reinterpret_cast<const float4*>(d_query),
                                                 n_query, bounded ? max_dist * max_dist : __builtin_inff(),
                                                 d_out_idx, d_out_d2);
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

rtr_status rtr_knn1_static(const float* d_query, int n_query, const float* d_target,
                           int n_target, float max_dist, int32_t* d_out_idx, float* d_out_d2,
                           rtr_stream_t stream) {
  RTR_CHECK_ARG(n_query >= 0 && n_target >= 0, "rtr_knn1_static: bad arguments");
  if (n_target > RTR_KNN1_STATIC_MAX_TARGET)
    return fail(RTR_ERR_CAPACITY,
                "rtr_knn1_static: n_target %d exceeds the fixed maximum %d (use rtr_knn1)",
                n_target, RTR_KNN1_STATIC_MAX_TARGET);
  if (n_query == 0) return RTR_OK;
  RTR_CHECK_ARG(d_query && d_out_idx, "rtr_knn1_static: NULL query or output");
  cudaStream_t st = (cudaStream_t)stream;
  if (n_target == 0) {
    RTR_CUDA(cudaMemsetAsync(d_out_idx, 0xff, (size_t)n_query * 4, st));
    return RTR_OK;  // d_out_d2 left as is: every index is -1
  }
  RTR_CHECK_ARG(d_target != nullptr, "rtr_knn1_static: NULL target");
  int dev = 0;
  RTR_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= KNN1_STATIC_DEVICES)
    return fail(RTR_ERR_INVALID_ARG, "rtr_knn1_static: device %d beyond the supported %d", dev,
                KNN1_STATIC_DEVICES);
  // the kernel runs on the current device: every buffer must live there
  if (!on_device(d_query, dev) || !on_device(d_target, dev) || !on_device(d_out_idx, dev) ||
      (d_out_d2 && !on_device(d_out_d2, dev)))
    return fail(RTR_ERR_INVALID_ARG,
                "rtr_knn1_static: a buffer is not device memory of the current device %d", dev);
  void* base = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_knn1_static_mu);
    if (!g_knn1_static_ptr[dev]) {
      void* p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_knn1_static);
      if (e != cudaSuccess || !p) {
        (void)cudaGetLastError();
        return fail(RTR_ERR_CUDA, "rtr_knn1_static: cudaGetSymbolAddress failed on device %d: %s",
                    dev, cudaGetErrorString(e));
      }
      g_knn1_static_ptr[dev] = p;
    }
    base = g_knn1_static_ptr[dev];
  }
  // the same cell table as rtr_knn1 builds for this target count (at most
  // the maximum target count's, which the array is sized for)
  const unsigned cap = default_cell_cap(n_target);
  ScratchPlan plan;
  grid_plan(plan, n_target, cap);
  if (plan.bytes > KNN1_STATIC_BYTES)
    return fail(RTR_ERR_CAPACITY, "rtr_knn1_static: grid needs %zu bytes, fixed array holds %zu",
                plan.bytes, KNN1_STATIC_BYTES);
  Scratch s;
  s.base = static_cast<char*>(base);
  s.cap = KNN1_STATIC_BYTES;
  GridBufs gb;
  if (!grid_take(s, n_target, cap, &gb)) return fail(RTR_ERR_CAPACITY, "rtr_knn1_static: scratch");
  const bool bounded = max_dist > 0.f && max_dist < 1e18f;
  grid_build(gb, reinterpret_cast<const float4*>(d_target), n_target, nullptr,
             bounded ? 0.5f * max_dist : -1.f, st);
  RTR_LAUNCHED(1);
  k_knn1<<<search_blocks(n_query * KNN1_G), 128, 0, st>>>(grid_dev(gb), reinterpret_cast<const float4*>(d_query),
                                                 n_query, bounded ? max_dist * max_dist : __builtin_inff(),
                                                 d_out_idx, d_out_d2);
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

rtr_status rtr_knn(rtr_context* ctx, const float* d_query, int n_query, const float* d_target,
                   int n_target, int k, int32_t* d_out_idx, float* d_out_d2, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n_query >= 0 && n_target >= 0, "rtr_knn: bad arguments");
  RTR_CHECK_ARG(k >= 1 && k <= 32, "rtr_knn: k must be in [1, 32]");
  if (n_query == 0) return RTR_OK;
  RTR_CHECK_ARG(d_query && d_out_idx, "rtr_knn: NULL query or output");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (n_target == 0) {
    RTR_CUDA(cudaMemsetAsync(d_out_idx, 0xff, (size_t)n_query * k * 4, st));
    return RTR_OK;
  }
  RTR_CHECK_ARG(d_target != nullptr, "rtr_knn: NULL target");
  const unsigned cap = default_cell_cap(n_target);
  ScratchPlan plan;
  grid_plan(plan, n_target, cap);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  GridBufs gb;
  if (!grid_take(s, n_target, cap, &gb)) return fail(RTR_ERR_CAPACITY, "rtr_knn: scratch");
  grid_build(gb, reinterpret_cast<const float4*>(d_target), n_target, nullptr, -1.f, st);
  const float4* q = reinterpret_cast<const float4*>(d_query);
  const int nb = search_blocks(n_query);
  ProfScope ps(ctx, st, "knn");
  RTR_LAUNCHED(1);
  if (k <= 8)
    k_knn<8><<<nb, 128, 0, st>>>(grid_dev(gb), q, n_query, k, d_out_idx, d_out_d2);
  else if (k <= 16)
    k_knn<16><<<nb, 128, 0, st>>>(grid_dev(gb), q, n_query, k, d_out_idx, d_out_d2);
  else
    k_knn<32><<<nb, 128, 0, st>>>(grid_dev(gb), q, n_query, k, d_out_idx, d_out_d2);
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

}  // extern "C"
