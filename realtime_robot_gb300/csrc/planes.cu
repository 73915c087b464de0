// planes.cu — plane segmentation with convex-hull areas, and the plane-area
// vector of keypoints: the reference's ModelPoint::getArea /
// ScanPoint::get_Area (model_point.h:170-245, scan_point.h:117-188) and
// KeyPoint::get_Vector3D (key_point.h:87-111), which the reference runs
// through PCL's SACSegmentation, ExtractIndices and ConvexHull.
//
// One call extracts planes one after another from the points still
// unclaimed (the reference's loop, while more than 15 % remain):
//   RANSAC   sample slots in batches of 64: one thread per slot draws three
//            positions in the remaining list (SplitMix64 of seed, round,
//            slot) and forms the plane (float); every thread of the grid
//            then tests its points against the 64 planes (the planes in
//            shared memory, counts per block, one atomic per slot and block);
//            the host walks the slots in order with the adaptive stop rule
//            (99 % confidence, at most max_iterations valid samples);
//   refit    one 1024-thread block sums the best plane's inliers in FP64,
//            thread t over positions t, t + 1024, ... in order, then a
//            pairwise tree in shared memory (a fixed order, the oracle's);
//            the host solves the 3x3 eigenproblem (planes_host.cpp);
//   select   the refitted plane's inliers (float test) flagged and scanned;
//   hull     the inliers projected onto the plane (float); the 8 points
//            extreme along u, v, u+v and u-v bound an octagon, and a point
//            strictly inside it (exact double orientation tests) cannot be
//            a hull vertex and is dropped; the rest are sorted by (u, v)
//            with two stable radix passes and one thread runs Andrew's
//            monotone chain (exact orientation tests); the host measures
//            the hull's area and perimeter;
//   remove   the inliers leave the remaining list (stable compaction).
// Everything that decides which points are inliers is computed exactly as
// in the CPU oracle (oracle/planes.c), so planes, inlier sets and hulls are
// bit-identical to it.
#include <math.h>
#include <string.h>

#include <vector>

#include "grid.cuh"
#include "planes_host.h"
#include "scan.cuh"

namespace rtr {

constexpr int PL_SLOTS = 64;        // RANSAC samples scored per batch
constexpr int PL_PARTIALS = 1024;   // strided FP64 partial sums of the refit

__device__ __forceinline__ uint64_t pl_mix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ int pl_pick(uint64_t seed, int round, int slot, int k, int m) {
  const uint64_t key = seed ^ ((uint64_t)round << 48) ^ ((uint64_t)slot << 16) ^ (uint64_t)k;
  return (int)(pl_mix(key) % (uint64_t)m);
}

__device__ __forceinline__ bool pl_within(float4 c, float4 p, float thr) {
  const float s = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(c.x, p.x), __fmul_rn(c.y, p.y)), __fmul_rn(c.z, p.z)), c.w);
  return fabsf(s) <= thr;
}

__device__ __forceinline__ bool finite3(float4 p) { return isfinite(p.x) && isfinite(p.y) && isfinite(p.z); }

__global__ void k_pl_finite(const float4* __restrict__ pts, int n, uint32_t* __restrict__ flags) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    flags[i] = finite3(pts[i]) ? 1u : 0u;
}

// out[pos[i]] = i (or src[i]) where flags[i] (== want)
__global__ void k_pl_compact(const uint32_t* __restrict__ flags, const uint32_t* __restrict__ pos,
                             const int* __restrict__ src, int n, uint32_t want, int* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (flags[i] == want) out[pos[i]] = src ? src[i] : i;
}

// one thread per slot of the batch: three positions and their plane
__global__ void k_pl_slots(const float4* __restrict__ pts, const int* __restrict__ rem, int m, uint64_t seed,
                           int round, int slot0, int n_slots, float4* __restrict__ coef, int* __restrict__ valid) {
  const int s = threadIdx.x;
  if (s >= n_slots) return;
  const int gs = slot0 + s;
  const int i0 = pl_pick(seed, round, gs, 0, m), i1 = pl_pick(seed, round, gs, 1, m), i2 = pl_pick(seed, round, gs, 2, m);
  int ok = i0 != i1 && i0 != i2 && i1 != i2;
  float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
  if (ok) {
    const float4 p0 = pts[rem[i0]], p1 = pts[rem[i1]], p2 = pts[rem[i2]];
    const float ax = __fsub_rn(p1.x, p0.x), ay = __fsub_rn(p1.y, p0.y), az = __fsub_rn(p1.z, p0.z);
    const float bx = __fsub_rn(p2.x, p0.x), by = __fsub_rn(p2.y, p0.y), bz = __fsub_rn(p2.z, p0.z);
    float nx = __fsub_rn(__fmul_rn(ay, bz), __fmul_rn(az, by));
    float ny = __fsub_rn(__fmul_rn(az, bx), __fmul_rn(ax, bz));
    float nz = __fsub_rn(__fmul_rn(ax, by), __fmul_rn(ay, bx));
    const float l2 = __fadd_rn(__fadd_rn(__fmul_rn(nx, nx), __fmul_rn(ny, ny)), __fmul_rn(nz, nz));
    ok = (l2 > 0.f) && (l2 < __int_as_float(0x7f800000));
    if (ok) {
      const float L = __fsqrt_rn(l2);
      nx = __fdiv_rn(nx, L);
      ny = __fdiv_rn(ny, L);
      nz = __fdiv_rn(nz, L);
      c = make_float4(nx, ny, nz,
                      -__fadd_rn(__fadd_rn(__fmul_rn(nx, p0.x), __fmul_rn(ny, p0.y)), __fmul_rn(nz, p0.z)));
    }
  }
  coef[s] = c;
  valid[s] = ok;
}

// inlier counts of the batch's planes over the remaining points
__global__ void __launch_bounds__(256) k_pl_count(const float4* __restrict__ pts, const int* __restrict__ rem, int m,
                                                  const float4* __restrict__ coef, const int* __restrict__ valid,
                                                  int n_slots, float thr, int* __restrict__ count) {
  __shared__ float4 sc[PL_SLOTS];
  __shared__ int sv[PL_SLOTS], cnt[PL_SLOTS];
  for (int s = threadIdx.x; s < PL_SLOTS; s += blockDim.x) {
    sc[s] = s < n_slots ? coef[s] : make_float4(0.f, 0.f, 0.f, 0.f);
    sv[s] = s < n_slots ? valid[s] : 0;
    cnt[s] = 0;
  }
  __syncthreads();
  // a thread holds up to 4 points and walks the planes; per plane one
  // warp-aggregated add into the block's counter
  for (int base = blockIdx.x * blockDim.x * 4; base < m; base += gridDim.x * blockDim.x * 4) {
    float4 p[4];
    bool live[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int j = base + r * blockDim.x + threadIdx.x;
      live[r] = j < m;
      p[r] = live[r] ? pts[rem[j]] : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int s = 0; s < n_slots; ++s) {
      if (!sv[s]) continue;
      const float4 c = sc[s];
      int h = 0;
#pragma unroll
      for (int r = 0; r < 4; ++r) h += (live[r] && pl_within(c, p[r], thr)) ? 1 : 0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) h += __shfl_xor_sync(0xffffffffu, h, o);
      if ((threadIdx.x & 31) == 0 && h) atomicAdd(&cnt[s], h);
    }
  }
  __syncthreads();
  for (int s = threadIdx.x; s < n_slots; s += blockDim.x)
    if (cnt[s]) atomicAdd(&count[s], cnt[s]);
}

// FP64 sums of the inliers of plane c in the oracle's fixed order
__global__ void __launch_bounds__(PL_PARTIALS) k_pl_refit(const float4* __restrict__ pts, const int* __restrict__ rem,
                                                           int m, float4 c, float thr, double* __restrict__ sums,
                                                           int* __restrict__ n_out) {
  extern __shared__ double part[];  // [PL_PARTIALS][9]
  __shared__ int cnt[PL_PARTIALS];
  const int t = threadIdx.x;
  double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  int n = 0;
  for (int j = t; j < m; j += PL_PARTIALS) {
    const float4 p = pts[rem[j]];
    if (!pl_within(c, p, thr)) continue;
    const double x = p.x, y = p.y, z = p.z;
    a[0] = __dadd_rn(a[0], x);
    a[1] = __dadd_rn(a[1], y);
    a[2] = __dadd_rn(a[2], z);
    a[3] = __dadd_rn(a[3], __dmul_rn(x, x));
    a[4] = __dadd_rn(a[4], __dmul_rn(x, y));
    a[5] = __dadd_rn(a[5], __dmul_rn(x, z));
    a[6] = __dadd_rn(a[6], __dmul_rn(y, y));
    a[7] = __dadd_rn(a[7], __dmul_rn(y, z));
    a[8] = __dadd_rn(a[8], __dmul_rn(z, z));
    ++n;
  }
#pragma unroll
  for (int k = 0; k < 9; ++k) part[t * 9 + k] = a[k];
  cnt[t] = n;
  __syncthreads();
  for (int width = PL_PARTIALS / 2; width >= 1; width >>= 1) {
    if (t < width) {
#pragma unroll
      for (int k = 0; k < 9; ++k) part[t * 9 + k] = __dadd_rn(part[t * 9 + k], part[(t + width) * 9 + k]);
      cnt[t] += cnt[t + width];
    }
    __syncthreads();
  }
  if (t < 9) sums[t] = part[t];
  if (t == 0) *n_out = cnt[0];
}

__global__ void k_pl_select(const float4* __restrict__ pts, const int* __restrict__ rem, int m, float4 c, float thr,
                            uint32_t* __restrict__ in, uint32_t* __restrict__ out) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) {
    const bool w = pl_within(c, pts[rem[j]], thr);
    in[j] = w ? 1u : 0u;
    out[j] = w ? 0u : 1u;
  }
}

// (u, v) of the inliers, in their order; -0 becomes +0 so that the sort
// keys order as the float comparisons do
__global__ void k_pl_project(const float4* __restrict__ pts, const int* __restrict__ rem, int m,
                             const uint32_t* __restrict__ in, const uint32_t* __restrict__ pos, float4 e1, float4 e2,
                             float2* __restrict__ uv) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) {
    if (!in[j]) continue;
    const float4 p = pts[rem[j]];
    float u = __fadd_rn(__fadd_rn(__fmul_rn(p.x, e1.x), __fmul_rn(p.y, e1.y)), __fmul_rn(p.z, e1.z));
    float v = __fadd_rn(__fadd_rn(__fmul_rn(p.x, e2.x), __fmul_rn(p.y, e2.y)), __fmul_rn(p.z, e2.z));
    uv[pos[j]] = make_float2(__fadd_rn(u, 0.f), __fadd_rn(v, 0.f));
  }
}

// the 8 extreme points: keys (ordered value << 32) | ~index, largest wins
// (ties to the lowest index); directions u, u+v, v, v-u, -u, -u-v, -v, u-v
__global__ void k_pl_extremes(const float2* __restrict__ uv, const int* __restrict__ d_n,
                              unsigned long long* __restrict__ ext) {
  const int n = *d_n;
  unsigned long long best[8];
#pragma unroll
  for (int d = 0; d < 8; ++d) best[d] = 0ull;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float u = uv[i].x, v = uv[i].y;
    const float val[8] = {u, __fadd_rn(u, v), v, __fsub_rn(v, u), -u, -__fadd_rn(u, v), -v, __fsub_rn(u, v)};
#pragma unroll
    for (int d = 0; d < 8; ++d) {
      const unsigned long long k = ((unsigned long long)float_to_ordered(val[d]) << 32) | (unsigned)(~(unsigned)i);
      best[d] = k > best[d] ? k : best[d];
    }
  }
#pragma unroll
  for (int d = 0; d < 8; ++d) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long x = __shfl_xor_sync(0xffffffffu, best[d], o);
      best[d] = x > best[d] ? x : best[d];
    }
    if ((threadIdx.x & 31) == 0 && best[d]) atomicMax(ext + d, best[d]);
  }
}

__device__ __forceinline__ double pl_cross(float2 o, float2 a, float2 b) {
  const double ax = __dsub_rn((double)a.x, (double)o.x), ay = __dsub_rn((double)a.y, (double)o.y);
  const double bx = __dsub_rn((double)b.x, (double)o.x), by = __dsub_rn((double)b.y, (double)o.y);
  return __dsub_rn(__dmul_rn(ax, by), __dmul_rn(ay, bx));
}

// keep[i] = 0 when point i is strictly inside the octagon of the extreme
// points (then it is no hull vertex), 1 otherwise
__global__ void k_pl_filter(const float2* __restrict__ uv, const int* __restrict__ d_n,
                            const unsigned long long* __restrict__ ext, uint32_t* __restrict__ keep) {
  const int n = *d_n;
  float2 E[8];
  int ne = 0;
  if (n > 0) {
    for (int d = 0; d < 8; ++d) {
      const float2 p = uv[~(unsigned)(ext[d] & 0xffffffffull)];
      if (ne == 0 || p.x != E[ne - 1].x || p.y != E[ne - 1].y) E[ne++] = p;
    }
    while (ne > 1 && E[ne - 1].x == E[0].x && E[ne - 1].y == E[0].y) --ne;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    bool inside = ne >= 3;
    const float2 p = uv[i];
    for (int e = 0; e < ne && inside; ++e) inside = pl_cross(E[e], E[(e + 1) % ne], p) > 0.0;
    keep[i] = inside ? 0u : 1u;
  }
}

__global__ void k_pl_gather_uv(const float2* __restrict__ uv, const uint32_t* __restrict__ keep,
                               const uint32_t* __restrict__ pos, const int* __restrict__ d_n, float2* __restrict__ out) {
  const int n = *d_n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (keep[i]) out[pos[i]] = uv[i];
}

// radix keys: the survivors' v, then (second pass) their u in that order
__global__ void k_pl_keys_v(const float2* __restrict__ su, const int* __restrict__ d_n, uint32_t* __restrict__ k) {
  const int n = *d_n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) k[i] = float_to_ordered(su[i].y);
}
__global__ void k_pl_keys_u(const float2* __restrict__ su, const uint32_t* __restrict__ order, const int* __restrict__ d_n,
                            uint32_t* __restrict__ k) {
  const int n = *d_n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    k[i] = float_to_ordered(su[order[i]].x);
}

// Andrew's monotone chain over the survivors in (u, v) order (one thread)
__global__ void k_pl_chain(const float2* __restrict__ su, const uint32_t* __restrict__ order, const int* __restrict__ d_n,
                           float2* __restrict__ H, int* __restrict__ h_out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int n = *d_n;
  int h = 0;
  for (int i = 0; i < n; ++i) {
    const float2 p = su[order[i]];
    while (h >= 2 && pl_cross(H[h - 2], H[h - 1], p) <= 0.0) --h;
    H[h++] = p;
  }
  for (int i = n - 2, lo = h + 1; i >= 0; --i) {
    const float2 p = su[order[i]];
    while (h >= lo && pl_cross(H[h - 2], H[h - 1], p) <= 0.0) --h;
    H[h++] = p;
  }
  if (h > 1) --h;
  *h_out = h;
}

// get_Vector3D for each keypoint over the kept surfaces, in list order
__global__ void k_vector3d(const float4* __restrict__ keys, int nk, const rtr_surface* __restrict__ s, int ns,
                           double* __restrict__ v3) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nk; k += gridDim.x * blockDim.x) {
    const float4 p = keys[k];
    double v[3] = {0.16, 0.16, 0.16};
    int vertical = 0, horizontal = 0;
    for (int i = 0; i < ns; ++i) {
      if (!s[i].kept) continue;
      const float* c = s[i].coeffs;
      const double d =
          (double)__fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(c[0], c[0]), __fmul_rn(c[1], c[1])), __fmul_rn(c[2], c[2])));
      const float e = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(c[0], p.x), __fmul_rn(c[1], p.y)), __fmul_rn(c[2], p.z)),
                                c[3]);
      const double dist = __ddiv_rn((double)fabsf(e), d);
      if (s[i].is_vertical == 0 && horizontal == 0 && dist <= 0.05) {
        v[0] = s[i].area;
        ++horizontal;
      } else if (s[i].is_vertical == 1 && vertical <= 1 && dist <= 0.02) {
        v[1 + vertical] = s[i].area;
        ++vertical;
      }
    }
    if (v[1] < v[2]) {
      const double t = v[2];
      v[2] = v[1];
      v[1] = t;
    }
    v3[3 * (size_t)k] = v[0];
    v3[3 * (size_t)k + 1] = v[1];
    v3[3 * (size_t)k + 2] = v[2];
  }
}

static int pl_blocks(int n) {
  int b = (n + 255) / 256;
  if (b > 152 * 8) b = 152 * 8;
  return b < 1 ? 1 : b;
}

static rtr_status pl_read(cudaStream_t st, void* h, const void* d, size_t bytes) {
  RTR_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, st));
  RTR_CUDA(cudaStreamSynchronize(st));
  return RTR_OK;
}

}  // namespace rtr

using namespace rtr;

extern "C" {

void rtr_plane_default_params(rtr_plane_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->max_iterations = 150;
  p->distance = 0.005f;
  p->remain_frac = 0.15;
  p->min_area = 0.16;
  p->seed = 0;
}

rtr_status rtr_plane_segment(rtr_context* ctx, const float* d_pts, int n, const rtr_plane_params* prm,
                             rtr_surface* h_surfaces, int max_surfaces, int* h_n_surfaces, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && prm && n >= 0 && h_n_surfaces && max_surfaces >= 0 && (max_surfaces == 0 || h_surfaces),
                "rtr_plane_segment: bad arguments");
  RTR_CHECK_ARG(prm->max_iterations >= 1 && prm->max_iterations <= 100000 && prm->distance > 0.f &&
                    prm->remain_frac >= 0.0 && prm->remain_frac < 1.0,
                "rtr_plane_segment: parameter out of range");
  RTR_CHECK_ARG(n == 0 || d_pts, "rtr_plane_segment: NULL points");
  *h_n_surfaces = 0;
  if (n == 0) return RTR_OK;
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  const int nc = n + 1;
  ScratchPlan plan;
  const size_t o_f = plan.add<uint32_t>(nc), o_g = plan.add<uint32_t>(nc), o_p = plan.add<uint32_t>(nc),
               o_q = plan.add<uint32_t>(nc), o_t = plan.add<uint32_t>(scan_tiles(nc));
  const size_t o_rem = plan.add<int>(nc), o_rem2 = plan.add<int>(nc);
  const size_t o_coef = plan.add<float4>(PL_SLOTS), o_valid = plan.add<int>(PL_SLOTS), o_cnt = plan.add<int>(PL_SLOTS);
  const size_t o_sums = plan.add<double>(16), o_ints = plan.add<int>(16), o_ext = plan.add<unsigned long long>(8);
  const size_t o_uv = plan.add<float2>(nc), o_su = plan.add<float2>(nc), o_hull = plan.add<float2>(2 * (size_t)nc + 2);
  const size_t o_k0 = plan.add<uint32_t>(nc), o_v0 = plan.add<uint32_t>(nc), o_k1 = plan.add<uint32_t>(nc),
               o_v1 = plan.add<uint32_t>(nc), o_hist = plan.add<uint32_t>(radix_hist_entries(nc));
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  char* B = s.base;
  uint32_t* flags = reinterpret_cast<uint32_t*>(B + o_f);
  uint32_t* flags2 = reinterpret_cast<uint32_t*>(B + o_g);
  uint32_t* pos = reinterpret_cast<uint32_t*>(B + o_p);
  uint32_t* pos2 = reinterpret_cast<uint32_t*>(B + o_q);
  uint32_t* tiles = reinterpret_cast<uint32_t*>(B + o_t);
  int* rem = reinterpret_cast<int*>(B + o_rem);
  int* rem2 = reinterpret_cast<int*>(B + o_rem2);
  float4* coef = reinterpret_cast<float4*>(B + o_coef);
  int* valid = reinterpret_cast<int*>(B + o_valid);
  int* cnt = reinterpret_cast<int*>(B + o_cnt);
  double* sums = reinterpret_cast<double*>(B + o_sums);
  int* ints = reinterpret_cast<int*>(B + o_ints);  // [0] remaining, [1] refit n, [2] inliers, [3] kept out, [4] survivors, [5] hull
  unsigned long long* ext = reinterpret_cast<unsigned long long*>(B + o_ext);
  float2* uv = reinterpret_cast<float2*>(B + o_uv);
  float2* su = reinterpret_cast<float2*>(B + o_su);
  float2* hull = reinterpret_cast<float2*>(B + o_hull);
  uint32_t* k0 = reinterpret_cast<uint32_t*>(B + o_k0);
  uint32_t* v0 = reinterpret_cast<uint32_t*>(B + o_v0);
  uint32_t* k1 = reinterpret_cast<uint32_t*>(B + o_k1);
  uint32_t* v1 = reinterpret_cast<uint32_t*>(B + o_v1);
  uint32_t* hist = reinterpret_cast<uint32_t*>(B + o_hist);
  const float4* pts = reinterpret_cast<const float4*>(d_pts);
  ProfScope ps(ctx, st, "plane_segment");
  // the refit's partial sums take 72 KB of shared memory (set per call: the
  // attribute belongs to the current device)
  RTR_CUDA(cudaFuncSetAttribute(k_pl_refit, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)(PL_PARTIALS * 9 * sizeof(double))));

  // the finite points, in index order
  k_pl_finite<<<pl_blocks(n), 256, 0, st>>>(pts, n, flags);
  scan_exclusive(flags, pos, tiles, nc, n, nullptr, reinterpret_cast<uint32_t*>(ints), st);
  k_pl_compact<<<pl_blocks(n), 256, 0, st>>>(flags, pos, nullptr, n, 1u, rem);
  RTR_LAUNCHED(2);
  int m = 0;
  RTR_TRY(pl_read(st, &m, ints, sizeof(int)));
  const int nr_points = m;
  const int max_slots = 11 * prm->max_iterations;
  int np = 0;
  for (int round = 0; (double)m > prm->remain_frac * (double)nr_points && m >= 3; ++round) {
    // RANSAC, batch by batch until the walk ends
    PlaneWalk w;
    float4 bc = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int base = 0; base < max_slots && !w.done; base += PL_SLOTS) {
      const int ns = max_slots - base < PL_SLOTS ? max_slots - base : PL_SLOTS;
      RTR_CUDA(cudaMemsetAsync(cnt, 0, PL_SLOTS * sizeof(int), st));
      k_pl_slots<<<1, PL_SLOTS, 0, st>>>(pts, rem, m, prm->seed, round, base, ns, coef, valid);
      k_pl_count<<<pl_blocks((m + 3) / 4), 256, 0, st>>>(pts, rem, m, coef, valid, ns, prm->distance, cnt);
      RTR_LAUNCHED(2);
      int hv[PL_SLOTS], hc[PL_SLOTS];
      float4 hcoef[PL_SLOTS];
      RTR_CUDA(cudaMemcpyAsync(hv, valid, ns * sizeof(int), cudaMemcpyDeviceToHost, st));
      RTR_CUDA(cudaMemcpyAsync(hc, cnt, ns * sizeof(int), cudaMemcpyDeviceToHost, st));
      RTR_CUDA(cudaMemcpyAsync(hcoef, coef, ns * sizeof(float4), cudaMemcpyDeviceToHost, st));
      RTR_CUDA(cudaStreamSynchronize(st));
      w.slot = 0;
      w.base = base;
      const int prev_best = w.best;
      plane_ransac_walk(hv, hc, ns, m, prm->max_iterations, &w);
      if (w.best != prev_best && w.best >= base) bc = hcoef[w.best - base];
    }
    if (w.best < 0) break;
    // least-squares refit over the best sample's inliers
    k_pl_refit<<<1, PL_PARTIALS, PL_PARTIALS * 9 * sizeof(double), st>>>(pts, rem, m, bc, prm->distance, sums, ints + 1);
    RTR_LAUNCHED(1);
    double h_sums[9];
    int n_fit = 0;
    RTR_CUDA(cudaMemcpyAsync(h_sums, sums, sizeof(h_sums), cudaMemcpyDeviceToHost, st));
    RTR_CUDA(cudaMemcpyAsync(&n_fit, ints + 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    RTR_CUDA(cudaStreamSynchronize(st));
    float c_in[4] = {bc.x, bc.y, bc.z, bc.w}, c[4];
    int flat = 1;
    plane_refit(h_sums, n_fit, c_in, c, &flat);
    const float4 cf = make_float4(c[0], c[1], c[2], c[3]);
    float e1[3], e2[3];
    plane_basis(c, e1, e2);
    // the refitted plane's inliers, their projections, the rest
    k_pl_select<<<pl_blocks(m), 256, 0, st>>>(pts, rem, m, cf, prm->distance, flags, flags2);
    scan_exclusive(flags, pos, tiles, nc, m, nullptr, reinterpret_cast<uint32_t*>(ints + 2), st);
    scan_exclusive(flags2, pos2, tiles, nc, m, nullptr, reinterpret_cast<uint32_t*>(ints + 3), st);
    k_pl_project<<<pl_blocks(m), 256, 0, st>>>(pts, rem, m, flags, pos, make_float4(e1[0], e1[1], e1[2], 0.f),
                                               make_float4(e2[0], e2[1], e2[2], 0.f), uv);
    // hull: octagon filter, (u, v) sort, monotone chain
    RTR_CUDA(cudaMemsetAsync(ext, 0, 8 * sizeof(unsigned long long), st));
    k_pl_extremes<<<pl_blocks(m), 256, 0, st>>>(uv, ints + 2, ext);
    k_pl_filter<<<pl_blocks(m), 256, 0, st>>>(uv, ints + 2, ext, k0);
    scan_exclusive(k0, k1, tiles, nc, m, ints + 2, reinterpret_cast<uint32_t*>(ints + 4), st);
    k_pl_gather_uv<<<pl_blocks(m), 256, 0, st>>>(uv, k0, k1, ints + 2, su);
    k_pl_keys_v<<<pl_blocks(m), 256, 0, st>>>(su, ints + 4, k0);
    uint32_t *ks, *vs;
    radix_sort_pairs(k0, v0, k1, v1, hist, nc, m, ints + 4, 32, true, st, &ks, &vs);
    // second, stable pass by u over the first pass's order
    uint32_t* ka = ks == k0 ? k1 : k0;
    uint32_t* va = vs == v0 ? v1 : v0;
    k_pl_keys_u<<<pl_blocks(m), 256, 0, st>>>(su, vs, ints + 4, ka);
    RTR_CUDA(cudaMemcpyAsync(va, vs, sizeof(uint32_t) * (size_t)m, cudaMemcpyDeviceToDevice, st));
    uint32_t *ks2, *vs2;
    radix_sort_pairs(ka, va, ka == k0 ? k1 : k0, va == v0 ? v1 : v0, hist, nc, m, ints + 4, 32, false, st, &ks2,
                     &vs2);
    k_pl_chain<<<1, 32, 0, st>>>(su, vs2, ints + 4, hull, ints + 5);
    RTR_LAUNCHED(8);
    int hi[6];
    RTR_CUDA(cudaMemcpyAsync(hi, ints, sizeof(hi), cudaMemcpyDeviceToHost, st));
    RTR_CUDA(cudaStreamSynchronize(st));
    const int ni = hi[2], nk = hi[3], nh = hi[5];
    if (ni == 0) break;
    std::vector<float> hv((size_t)2 * (nh > 0 ? nh : 1));
    if (nh > 0) RTR_TRY(pl_read(st, hv.data(), hull, sizeof(float2) * (size_t)nh));
    double area = 0.0, perim = 0.0;
    hull_measure(hv.data(), nh, &area, &perim);
    if (np < max_surfaces) {
      rtr_surface& S = h_surfaces[np];
      memset(&S, 0, sizeof(S));
      S.area = area;
      S.perimeter = perim;
      memcpy(S.coeffs, c, sizeof(c));
      S.n_inliers = ni;
      S.hull_vertices = nh;
      S.flat = flat;
      S.is_vertical = plane_class(c);
      S.kept = S.is_vertical >= 0 && area >= prm->min_area;
    }
    ++np;
    // the rest stays, in order
    k_pl_compact<<<pl_blocks(m), 256, 0, st>>>(flags2, pos2, rem, m, 1u, rem2);
    RTR_LAUNCHED(1);
    int* t = rem;
    rem = rem2;
    rem2 = t;
    m = nk;
  }
  RTR_CUDA(cudaStreamSynchronize(st));
  *h_n_surfaces = np < max_surfaces ? np : max_surfaces;
  if (np > max_surfaces)
    return fail(RTR_ERR_CAPACITY, "rtr_plane_segment: %d planes extracted, room for %d", np, max_surfaces);
  return RTR_OK;
}

rtr_status rtr_vector3d(rtr_context* ctx, const float* d_keys, int n_keys, const rtr_surface* h_surfaces,
                        int n_surfaces, double* d_v3, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n_keys >= 0 && n_surfaces >= 0 && (n_surfaces == 0 || h_surfaces),
                "rtr_vector3d: bad arguments");
  if (n_keys == 0) return RTR_OK;
  RTR_CHECK_ARG(d_keys && d_v3, "rtr_vector3d: NULL keypoints or output");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  ScratchPlan plan;
  const size_t o_s = plan.add<rtr_surface>(n_surfaces > 0 ? n_surfaces : 1);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  rtr_surface* d_s = reinterpret_cast<rtr_surface*>(s.base + o_s);
  if (n_surfaces > 0)
    RTR_CUDA(cudaMemcpyAsync(d_s, h_surfaces, sizeof(rtr_surface) * (size_t)n_surfaces, cudaMemcpyHostToDevice, st));
  k_vector3d<<<pl_blocks(n_keys), 256, 0, st>>>(reinterpret_cast<const float4*>(d_keys), n_keys, d_s, n_surfaces,
                                                d_v3);
  RTR_LAUNCHED(1);
  RTR_CUDA(cudaGetLastError());
  // the host array may be reused once the call returns
  RTR_CUDA(cudaStreamSynchronize(st));
  return RTR_OK;
}

}  // extern "C"
