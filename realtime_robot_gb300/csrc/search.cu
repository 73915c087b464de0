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

// Fixed-radius and box searches: every target within reach of a query, in
// ascending target index.  One warp per query.  The grid's cell edge is at
// least 1.01 x the reach, so the cube of cells around the query's reach
// (widened by a rounding margin) spans at most 3 cells per axis: lane k
// owns cells k and k + 32 of that cube.  A cell's points are stored in
// ascending original index (the grid's sort is stable), so the warp merges
// the cells' hit sequences by repeated minimum: the output comes out sorted
// and a cut at max_per_query keeps the lowest indices.  A cube of more than
// 64 cells (coordinates so large that the margin exceeds the cell's slack)
// takes a slower path that scans the cube once per output.
template <bool BOX>
__device__ __forceinline__ bool range_hit(float4 q, float4 p, float r2, float4 lo, float4 hi) {
  if (BOX) return p.x >= lo.x && p.y >= lo.y && p.z >= lo.z && p.x <= hi.x && p.y <= hi.y && p.z <= hi.z;
  return dist2_exact(q, p) <= r2;
}

template <bool BOX>
__device__ __forceinline__ int range_advance(const GridView& g, unsigned& j, unsigned e, float4 q, float r2,
                                             float4 lo, float4 hi) {
  while (j < e && !range_hit<BOX>(q, g.pts[j], r2, lo, hi)) ++j;
  return j < e ? pt_index(g.pts[j]) : INT_MAX;
}

__device__ __forceinline__ int warp_min_int(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

template <bool BOX>
__global__ void __launch_bounds__(128) k_range(GridDev gd, const float4* __restrict__ qs, int nq, float reach,
                                               int maxk, int* __restrict__ out_idx, int* __restrict__ out_cnt) {
  const GridView g = load_view(gd);
  const int lane = threadIdx.x & 31;
  const float r2 = reach * reach;
  for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < nq; i += gridDim.x * (blockDim.x >> 5)) {
    const float4 q = qs[i];
    // the box as the reference forms it: centre -/+ half extent in FP32
    const float4 lo = make_float4(__fsub_rn(q.x, reach), __fsub_rn(q.y, reach), __fsub_rn(q.z, reach), 0.f);
    const float4 hi = make_float4(__fadd_rn(q.x, reach), __fadd_rn(q.y, reach), __fadd_rn(q.z, reach), 0.f);
    // cells of the cube [q - e, q + e], e = reach + a margin above the
    // rounding of the distance, the bounds and the cell index
    const float mag = fmaxf(fmaxf(fabsf(q.x), fabsf(q.y)), fabsf(q.z));
    const float e = reach + 1.0e-4f * reach + 4.0e-7f * mag + 1.0e-30f;
    int x0 = q_cell(q.x - e, g.ox, g.inv_h), x1 = q_cell(q.x + e, g.ox, g.inv_h);
    int y0 = q_cell(q.y - e, g.oy, g.inv_h), y1 = q_cell(q.y + e, g.oy, g.inv_h);
    int z0 = q_cell(q.z - e, g.oz, g.inv_h), z1 = q_cell(q.z + e, g.oz, g.inv_h);
    x0 = max(x0, 0);
    y0 = max(y0, 0);
    z0 = max(z0, 0);
    x1 = min(x1, g.nx - 1);
    y1 = min(y1, g.ny - 1);
    z1 = min(z1, g.nz - 1);
    const bool finite_q = isfinite(q.x) && isfinite(q.y) && isfinite(q.z);
    const int ex = x1 - x0 + 1, ey = y1 - y0 + 1, ez = z1 - z0 + 1;
    const int nc = (finite_q && ex > 0 && ey > 0 && ez > 0) ? ex * ey * ez : 0;
    auto cell_range = [&](int k) -> uint2 {
      const int x = x0 + k % ex, y = y0 + (k / ex) % ey, z = z0 + k / (ex * ey);
      return g.cells[((unsigned)z * (unsigned)g.ny + (unsigned)y) * (unsigned)g.nx + (unsigned)x];
    };
    // the true count
    int cnt = 0;
    for (int k = lane; k < nc; k += 32) {
      const uint2 c = cell_range(k);
      for (unsigned j = c.x; j < c.y; ++j) cnt += range_hit<BOX>(q, g.pts[j], r2, lo, hi) ? 1 : 0;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (lane == 0 && out_cnt) out_cnt[i] = cnt;
    const int nout = min(cnt, maxk);
    int* out = out_idx ? out_idx + (size_t)i * maxk : nullptr;
    if (out && nc <= 64) {
      uint2 ra = make_uint2(0u, 0u), rb = ra;
      if (lane < nc) ra = cell_range(lane);
      if (lane + 32 < nc) rb = cell_range(lane + 32);
      int ha = range_advance<BOX>(g, ra.x, ra.y, q, r2, lo, hi);
      int hb = range_advance<BOX>(g, rb.x, rb.y, q, r2, lo, hi);
      for (int o = 0; o < nout; ++o) {
        const int m = warp_min_int(min(ha, hb));
        if (lane == 0) out[o] = m;
        if (ha == m) {  // indices are unique: one run of one lane holds it
          ++ra.x;
          ha = range_advance<BOX>(g, ra.x, ra.y, q, r2, lo, hi);
        } else if (hb == m) {
          ++rb.x;
          hb = range_advance<BOX>(g, rb.x, rb.y, q, r2, lo, hi);
        }
      }
    } else if (out) {
      int last = -1;
      for (int o = 0; o < nout; ++o) {
        int best = INT_MAX;
        for (int k = lane; k < nc; k += 32) {
          const uint2 c = cell_range(k);
          for (unsigned j = c.x; j < c.y; ++j) {
            const float4 p = g.pts[j];
            const int id = pt_index(p);
            if (id > last && id < best && range_hit<BOX>(q, p, r2, lo, hi)) best = id;
          }
        }
        best = warp_min_int(best);
        if (lane == 0) out[o] = best;
        last = best;
      }
    }
    if (out)
      for (int o = nout + lane; o < maxk; o += 32) out[o] = -1;
  }
}

static rtr_status range_search(rtr_context* ctx, const char* who, bool box, const float* d_query, int n_query,
                               const float* d_target, int n_target, float reach, int max_per_query,
                               int32_t* d_out_idx, int32_t* d_out_count, cudaStream_t st) {
  RTR_CHECK_ARG(ctx && n_query >= 0 && n_target >= 0 && max_per_query >= 0, "%s: bad arguments", who);
  RTR_CHECK_ARG(reach >= 0.f && reach < 1.0e18f, "%s: the radius / half extent must be finite and >= 0", who);
  RTR_CHECK_ARG(max_per_query == 0 || d_out_idx, "%s: NULL index output with max_per_query > 0", who);
  if (n_query == 0) return RTR_OK;
  RTR_CHECK_ARG(d_query != nullptr, "%s: NULL query", who);
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (n_target == 0) {
    if (d_out_count) RTR_CUDA(cudaMemsetAsync(d_out_count, 0, (size_t)n_query * 4, st));
    if (max_per_query > 0) RTR_CUDA(cudaMemsetAsync(d_out_idx, 0xff, (size_t)n_query * max_per_query * 4, st));
    return RTR_OK;
  }
  RTR_CHECK_ARG(d_target != nullptr, "%s: NULL target", who);
  const unsigned cap = default_cell_cap(n_target);
  ScratchPlan plan;
  grid_plan(plan, n_target, cap);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  GridBufs gb;
  if (!grid_take(s, n_target, cap, &gb)) return fail(RTR_ERR_CAPACITY, "%s: scratch", who);
  // cell edge 1.01 x the reach (the table's size limit may widen it)
  const float h = reach > 0.f ? 1.01f * reach : 1.0e-3f;
  grid_build(gb, reinterpret_cast<const float4*>(d_target), n_target, nullptr, h, st);
  const float4* q = reinterpret_cast<const float4*>(d_query);
  int nb = (n_query + 3) / 4;
  if (nb > 152 * 16) nb = 152 * 16;
  ProfScope ps(ctx, st, box ? "box_search" : "radius_search");
  int* oi = max_per_query > 0 ? d_out_idx : nullptr;
  if (box)
    k_range<true><<<nb, 128, 0, st>>>(grid_dev(gb), q, n_query, reach, max_per_query, oi, d_out_count);
  else
    k_range<false><<<nb, 128, 0, st>>>(grid_dev(gb), q, n_query, reach, max_per_query, oi, d_out_count);
  RTR_LAUNCHED(1);
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
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

rtr_status rtr_radius_search(rtr_context* ctx, const float* d_query, int n_query, const float* d_target,
                             int n_target, float radius, int max_per_query, int32_t* d_out_idx,
                             int32_t* d_out_count, rtr_stream_t stream) {
  return range_search(ctx, "rtr_radius_search", false, d_query, n_query, d_target, n_target, radius, max_per_query,
                      d_out_idx, d_out_count, (cudaStream_t)stream);
}

rtr_status rtr_box_search(rtr_context* ctx, const float* d_query, int n_query, const float* d_target,
                          int n_target, float half_extent, int max_per_query, int32_t* d_out_idx,
                          int32_t* d_out_count, rtr_stream_t stream) {
  return range_search(ctx, "rtr_box_search", true, d_query, n_query, d_target, n_target, half_extent,
                      max_per_query, d_out_idx, d_out_count, (cudaStream_t)stream);
}

}  // extern "C"
