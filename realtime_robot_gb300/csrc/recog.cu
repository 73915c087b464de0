// recog.cu — voxel-grid filter, uniform sampling, normals, outward normal
// orientation and the SHOT-style descriptor (stages of the chain driven by
// ModelPoint/ScanPoint::getKeypoint and KeyPoint in the reference:
// model_point.h:99-156, scan_point.h:57-113, key_point.h:112-161, 251-334).
#include <math.h>

#include "eig3.cuh"
#include "recog.cuh"
#include "scan.cuh"
#include "search.cuh"

namespace rtr {

__device__ __forceinline__ int cnt_of(int n_host, const int* d_n) { return d_n ? *d_n : n_host; }

static int blocks_for(int n, int per_block = 256, int cap = 152 * 16) {
  int b = (n + per_block - 1) / per_block;
  if (b < 1) b = 1;
  return b > cap ? cap : b;
}

// ---------------------------------------------------------------------------
// voxel segmentation
// ---------------------------------------------------------------------------
__global__ void k_vox_init(VoxMeta* m) {
  if (threadIdx.x < 3) {
    m->lo[threadIdx.x] = 0x7fffffff;
    m->hi[threadIdx.x] = (int)0x80000000;
  }
  if (threadIdx.x == 0) m->error = 0;
}

__device__ __forceinline__ int vox_coord(float v, float inv, int* err) {
  const float f = floorf(__fmul_rn(v, inv));
  if (!(fabsf(f) < 1.0e9f)) {  // also catches NaN
    *err = 1;
    return 0;
  }
  return (int)f;
}

// Points with a non-finite coordinate get no voxel (PCL's VoxelGrid skips
// them in clouds that are not dense): they take the key VOX_SKIP, sort last
// and belong to no segment.
constexpr uint32_t VOX_SKIP = 0xffffffffu;
__device__ __forceinline__ bool finite3(float4 p) { return isfinite(p.x) && isfinite(p.y) && isfinite(p.z); }

__global__ void __launch_bounds__(256) k_vox_bounds(const float4* __restrict__ pts, int n_host,
                                                    const int* d_n, float inv, VoxMeta* m) {
  const int n = cnt_of(n_host, d_n);
  int lo[3] = {0x7fffffff, 0x7fffffff, 0x7fffffff}, hi[3] = {(int)0x80000000, (int)0x80000000, (int)0x80000000};
  int err = 0;
#pragma unroll 4
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = pts[i];
    if (!finite3(p)) continue;
    const int c[3] = {vox_coord(p.x, inv, &err), vox_coord(p.y, inv, &err), vox_coord(p.z, inv, &err)};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      lo[a] = min(lo[a], c[a]);
      hi[a] = max(hi[a], c[a]);
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[a] = min(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
      hi[a] = max(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
    }
  err = __any_sync(0xffffffffu, err);
  // the block's extremes, then a few atomics per block (not per warp)
  __shared__ int s_lo[3][8], s_hi[3][8], s_err[8];
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      s_lo[a][warp] = lo[a];
      s_hi[a][warp] = hi[a];
    }
    s_err[warp] = err;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    const int a = threadIdx.x;
    int l = s_lo[a][0], h = s_hi[a][0], e = s_err[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      l = min(l, s_lo[a][w]);
      h = max(h, s_hi[a][w]);
      e |= s_err[w];
    }
    atomicMin(&m->lo[a], l);
    atomicMax(&m->hi[a], h);
    if (a == 0 && e) atomicExch(&m->error, 1);
  }
}

__global__ void k_vox_setup(VoxMeta* m, int n_host, const int* d_n) {
  const int n = cnt_of(n_host, d_n);
  m->n = n;
  if (n <= 0) {
    m->dx = m->dy = m->dz = 1;
    return;
  }
  if (m->lo[0] > m->hi[0]) {  // no finite point: every key is VOX_SKIP
    m->lo[0] = m->lo[1] = m->lo[2] = 0;
    m->dx = m->dy = m->dz = 1;
    return;
  }
  const long long dx = (long long)m->hi[0] - m->lo[0] + 1, dy = (long long)m->hi[1] - m->lo[1] + 1,
                  dz = (long long)m->hi[2] - m->lo[2] + 1;
  // one key (VOX_SKIP) stays free for the points without a voxel
  if (dx * dy > 0xffffffffLL || dx * dy * dz >= 0xffffffffLL) m->error = 1;
  m->dx = (unsigned)dx;
  m->dy = (unsigned)dy;
  m->dz = (unsigned)dz;
}

__global__ void __launch_bounds__(256) k_vox_keys(const float4* __restrict__ pts, int n_host,
                                                  const int* d_n, float inv, const VoxMeta* __restrict__ m,
                                                  uint32_t* __restrict__ keys) {
  const int n = cnt_of(n_host, d_n);
  const int ok = !m->error;
  const int l0 = m->lo[0], l1 = m->lo[1], l2 = m->lo[2];
  const unsigned dx = m->dx, dy = m->dy;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = pts[i];
    if (!finite3(p)) {
      keys[i] = VOX_SKIP;
      continue;
    }
    int e = 0;
    const unsigned x = (unsigned)(vox_coord(p.x, inv, &e) - l0), y = (unsigned)(vox_coord(p.y, inv, &e) - l1),
                   z = (unsigned)(vox_coord(p.z, inv, &e) - l2);
    keys[i] = ok ? (z * dy + y) * dx + x : 0u;
  }
}

__global__ void __launch_bounds__(256) k_seg_heads(const uint32_t* __restrict__ k, int n_host,
                                                   const int* d_n, uint32_t* __restrict__ flags) {
  const int n = cnt_of(n_host, d_n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    flags[i] = (k[i] != VOX_SKIP && (i == 0 || k[i] != k[i - 1])) ? 1u : 0u;
}

__global__ void __launch_bounds__(256) k_seg_starts(const uint32_t* __restrict__ k,
                                                    const uint32_t* __restrict__ pos, int n_host,
                                                    const int* d_n, int* __restrict__ start,
                                                    const int* __restrict__ d_nseg) {
  const int n = cnt_of(n_host, d_n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const bool keyed = k[i] != VOX_SKIP;
    if (keyed && (i == 0 || k[i] != k[i - 1])) start[pos[i]] = i;
    // the end of the last segment: past the last keyed point (the skipped
    // points sort after every key)
    if (keyed && (i + 1 == n || k[i + 1] == VOX_SKIP)) start[*d_nseg] = i + 1;
    if (i == 0 && !keyed) start[*d_nseg] = 0;
  }
}

void voxseg_plan(ScratchPlan& p, int n_cap) {
  const int n = n_cap > 0 ? n_cap : 1;
  p.add<VoxMeta>(1);
  for (int i = 0; i < 5; ++i) p.add<uint32_t>(n);
  p.add<uint32_t>(radix_hist_entries(n));
  p.add<uint32_t>(scan_tiles(n));
  p.add<int>(n + 1);
  p.add<int>(4);
}

bool voxseg_take(Scratch& s, int n_cap, VoxSeg* v) {
  const int n = n_cap > 0 ? n_cap : 1;
  v->meta = s.take<VoxMeta>(1);
  v->k0 = s.take<uint32_t>(n);
  v->v0 = s.take<uint32_t>(n);
  v->k1 = s.take<uint32_t>(n);
  v->v1 = s.take<uint32_t>(n);
  v->flags = s.take<uint32_t>(n);
  v->hist = s.take<uint32_t>(radix_hist_entries(n));
  v->tile_sums = s.take<uint32_t>(scan_tiles(n));
  v->seg_start = s.take<int>(n + 1);
  v->d_nseg = s.take<int>(4);
  v->n_cap = n_cap;
  return v->meta && v->k0 && v->v0 && v->k1 && v->v1 && v->flags && v->hist && v->tile_sums &&
         v->seg_start && v->d_nseg;
}

void voxseg_build(VoxSeg& v, const float4* pts, int n_host, const int* d_n, float inv, cudaStream_t st) {
  const int nb = blocks_for(v.n_cap);
  k_vox_init<<<1, 32, 0, st>>>(v.meta);
  k_vox_bounds<<<nb < 152 * 2 ? nb : 152 * 2, 256, 0, st>>>(pts, n_host, d_n, inv, v.meta);  // block-reduced
  k_vox_setup<<<1, 1, 0, st>>>(v.meta, n_host, d_n);
  k_vox_keys<<<nb, 256, 0, st>>>(pts, n_host, d_n, inv, v.meta, v.k0);
  uint32_t *ks, *vs;
  radix_sort_pairs(v.k0, v.v0, v.k1, v.v1, v.hist, v.n_cap, n_host, d_n, 32, true, st, &ks, &vs);
  k_seg_heads<<<nb, 256, 0, st>>>(ks, n_host, d_n, v.flags);
  scan_exclusive(v.flags, v.flags, v.tile_sums, v.n_cap, n_host, d_n, reinterpret_cast<uint32_t*>(v.d_nseg), st);
  k_seg_starts<<<nb, 256, 0, st>>>(ks, v.flags, n_host, d_n, v.seg_start, v.d_nseg);
  RTR_LAUNCHED(6);
  v.keys = ks;
  v.order = vs;
}

// ---------------------------------------------------------------------------
// voxel-grid filter: FP32 centroid, points summed in ascending input index
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_vox_centroid(const float4* __restrict__ pts,
                                                      const uint32_t* __restrict__ order,
                                                      const int* __restrict__ start,
                                                      const int* __restrict__ d_nseg,
                                                      const VoxMeta* __restrict__ m,
                                                      float4* __restrict__ out, int* d_count) {
  const int V = m->error ? 0 : *d_nseg;
  if (blockIdx.x == 0 && threadIdx.x == 0 && d_count) *d_count = m->error ? -1 : V;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int b = start[v], e = start[v + 1];
    float sx = 0.f, sy = 0.f, sz = 0.f;
    for (int i = b; i < e; ++i) {
      const float4 p = pts[order[i]];
      sx = __fadd_rn(sx, p.x);
      sy = __fadd_rn(sy, p.y);
      sz = __fadd_rn(sz, p.z);
    }
    const float c = (float)(e - b);
    out[v] = make_float4(__fdiv_rn(sx, c), __fdiv_rn(sy, c), __fdiv_rn(sz, c), 0.f);
  }
}

// ---------------------------------------------------------------------------
// uniform sampling: per voxel of edge r, the point nearest the voxel centre
// ((ijk + 0.5) * r), ties to the lowest index
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_uniform_pick(const float4* __restrict__ pts,
                                                      const uint32_t* __restrict__ order,
                                                      const int* __restrict__ start,
                                                      const int* __restrict__ d_nseg,
                                                      const VoxMeta* __restrict__ m, float inv, float r,
                                                      int* __restrict__ out, int* d_count) {
  const int V = m->error ? 0 : *d_nseg;
  if (blockIdx.x == 0 && threadIdx.x == 0 && d_count) *d_count = m->error ? -1 : V;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const int b = start[v], e = start[v + 1];
    float bd = __int_as_float(0x7f800000);
    int best = -1;
    for (int i = b; i < e; ++i) {
      const int idx = (int)order[i];
      const float4 p = pts[idx];
      const float cx = __fmul_rn(__fadd_rn((float)(int)floorf(__fmul_rn(p.x, inv)), 0.5f), r);
      const float cy = __fmul_rn(__fadd_rn((float)(int)floorf(__fmul_rn(p.y, inv)), 0.5f), r);
      const float cz = __fmul_rn(__fadd_rn((float)(int)floorf(__fmul_rn(p.z, inv)), 0.5f), r);
      const float d = dist2_exact(p, make_float4(cx, cy, cz, 0.f));
      if (d < bd || (d == bd && idx < best)) {
        bd = d;
        best = idx;
      }
    }
    out[v] = best;
  }
}

// ---------------------------------------------------------------------------
// normals: k nearest (incl. the point), FP32 mean and centred covariance in
// kNN order, exact Jacobi, smallest eigenvector flipped towards vp,
// curvature l0 / (l0 + l1 + l2)
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(128) k_normals(GridDev gd, const float4* __restrict__ pts, int n_host,
                                                 const int* d_n, float vx, float vy, float vz,
                                                 float4* __restrict__ out) {
  const GridView g = load_view(gd);
  const int n = cnt_of(n_host, d_n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = pts[i];
    float bd[K];
    int bi[K];
    grid_knn<K>(g, p, bd, bi);
    int m = 0;
    float mx = 0.f, my = 0.f, mz = 0.f;
#pragma unroll
    for (int s = 0; s < K; ++s) {
      if (bi[s] == INT_MAX) continue;
      const float4 q = pts[bi[s]];
      mx = __fadd_rn(mx, q.x);
      my = __fadd_rn(my, q.y);
      mz = __fadd_rn(mz, q.z);
      ++m;
    }
    const float fm = (float)m;
    mx = __fdiv_rn(mx, fm);
    my = __fdiv_rn(my, fm);
    mz = __fdiv_rn(mz, fm);
    float c00 = 0.f, c01 = 0.f, c02 = 0.f, c11 = 0.f, c12 = 0.f, c22 = 0.f;
#pragma unroll
    for (int s = 0; s < K; ++s) {
      if (bi[s] == INT_MAX) continue;
      const float4 q = pts[bi[s]];
      const float dx = __fsub_rn(q.x, mx), dy = __fsub_rn(q.y, my), dz = __fsub_rn(q.z, mz);
      c00 = __fadd_rn(c00, __fmul_rn(dx, dx));
      c01 = __fadd_rn(c01, __fmul_rn(dx, dy));
      c02 = __fadd_rn(c02, __fmul_rn(dx, dz));
      c11 = __fadd_rn(c11, __fmul_rn(dy, dy));
      c12 = __fadd_rn(c12, __fmul_rn(dy, dz));
      c22 = __fadd_rn(c22, __fmul_rn(dz, dz));
    }
    const float A[9] = {c00, c01, c02, c01, c11, c12, c02, c12, c22};
    float w[3], V[9];
    eig3_exact(A, w, V);
    float nx = V[0], ny = V[3], nz = V[6];
    const float ux = __fsub_rn(vx, p.x), uy = __fsub_rn(vy, p.y), uz = __fsub_rn(vz, p.z);
    const float dotv = __fadd_rn(__fadd_rn(__fmul_rn(ux, nx), __fmul_rn(uy, ny)), __fmul_rn(uz, nz));
    if (dotv < 0.f) {
      nx = -nx;
      ny = -ny;
      nz = -nz;
    }
    const float den = __fadd_rn(__fadd_rn(w[0], w[1]), w[2]);
    out[i] = make_float4(nx, ny, nz, den != 0.f ? __fdiv_rn(w[0], den) : 0.f);
  }
}

// ---------------------------------------------------------------------------
// outward orientation of a full model cloud: flip n towards the side whose
// cylinder (radius rc, axial distance in (gap, len]) holds fewer points
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_orient_outward(const float4* __restrict__ pts,
                                                        float4* __restrict__ nrm, int n_host,
                                                        const int* d_n, float rc2, float gap, float len) {
  const int n = cnt_of(n_host, d_n);
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    const float4 p = pts[i];
    const float4 nv = nrm[i];
    int cp = 0, cm = 0;
    for (int j = lane; j < n; j += 32) {
      const float4 q = pts[j];
      const float dx = __fsub_rn(q.x, p.x), dy = __fsub_rn(q.y, p.y), dz = __fsub_rn(q.z, p.z);
      const float ax = __fadd_rn(__fadd_rn(__fmul_rn(dx, nv.x), __fmul_rn(dy, nv.y)), __fmul_rn(dz, nv.z));
      const float aa = fabsf(ax);
      if (!(aa > gap) || aa > len) continue;
      const float r2 = __fsub_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)),
                                 __fmul_rn(ax, ax));
      if (r2 > rc2) continue;
      if (ax > 0.f) ++cp; else ++cm;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      cp += __shfl_xor_sync(0xffffffffu, cp, o);
      cm += __shfl_xor_sync(0xffffffffu, cm, o);
    }
    if (lane == 0 && cp > cm) nrm[i] = make_float4(-nv.x, -nv.y, -nv.z, nv.w);
  }
}

// ---------------------------------------------------------------------------
// SHOT-style 352-d descriptor, one warp per keypoint.  Conventions (shared
// with the oracle): support = points within R whose oriented normal faces the
// keypoint's (n_j . n_k >= -0.2); LRF = eigenvectors of the (R - d) weighted
// covariance (x largest, z smallest), x signed by the majority rule, z signed
// by sum w (n_j . z) >= 0; 2 radial x 2 elevation x 8 azimuth volumes x 11
// bins of cos(n_j, z), quadrilinear interpolation; L2 normalised.
//
// Bit-exact with the oracle's orc_shot352: every per-point term is a fixed
// sequence of separately rounded IEEE operations, every sum over the support
// is an integer sum of fixed-point terms (so the order in which lanes and
// atomics add them cannot change the result), the angles come from
// shot_atan2 below, and the final norm is summed in one stated order.  No
// FP64: every conversion is a single-precision one.
// ---------------------------------------------------------------------------
constexpr int SHOT_WARPS = 8;
constexpr float SHOT_FACING = -0.2f;
constexpr float SHOT_PI = 0x1.921fb6p+1f;

// Fixed-point scales.  Covariance terms are at most R^3 in magnitude and
// z-sign terms at most R: each is scaled by 2^(30 - e), e the exponent with
// bound < 2^e, so every term converts to an int32 and their sums are int64.
// Histogram votes are at most 1 and a point casts at most one vote per bin,
// so with ns support points and votes scaled by 2^(31 - bitlen(ns)) every
// bin's sum fits a uint32.
__device__ __forceinline__ int shot_exp2_above(float v) {  // e with v < 2^e (v > 0, normal)
  return (int)((__float_as_uint(v) >> 23) & 0xffu) - 126;
}

__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }  // -126 <= e <= 127

// atan2 for the angle bins, the same operations as the oracle's shot_atan2
// (library atan2f differs between the GPU and host C libraries in the last
// bits).  The ratio a = min(|x|,|y|) / max(|x|,|y|) lies in [0, 1]; above
// tan(pi/12) the reduction atan(a) = pi/6 + atan((sqrt(3) a - 1) / (a +
// sqrt(3))) (Cody and Waite, Software Manual for the Elementary Functions,
// 1980, ch. 11) leaves |u| <= tan(pi/12), where the series u - u^3/3 + u^5/5
// - u^7/7 + u^9/9 - u^11/11 is within 3e-9; then the octant and the signs.
// atan2(0, 0) = 0, and -0 counts as positive.
__device__ __forceinline__ float shot_atan2(float y, float x) {
  const float ax = fabsf(x), ay = fabsf(y);
  const float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
  if (!(mx > 0.f)) return 0.f;
  const float a = __fdiv_rn(mn, mx);
  float u = a, base = 0.f;
  if (a > 0x1.126146p-2f) {  // tan(pi/12)
    u = __fdiv_rn(__fsub_rn(__fmul_rn(a, 0x1.bb67aep+0f), 1.f), __fadd_rn(a, 0x1.bb67aep+0f));
    base = 0x1.0c1524p-1f;  // pi/6
  }
  const float z = __fmul_rn(u, u);
  float p = -0x1.745d18p-4f;                          // -1/11
  p = __fadd_rn(__fmul_rn(p, z), 0x1.c71c72p-4f);     // 1/9
  p = __fadd_rn(__fmul_rn(p, z), -0x1.24924ap-3f);    // -1/7
  p = __fadd_rn(__fmul_rn(p, z), 0x1.99999ap-3f);     // 1/5
  p = __fadd_rn(__fmul_rn(p, z), -0x1.555556p-2f);    // -1/3
  p = __fmul_rn(p, z);
  float r = __fadd_rn(base, __fadd_rn(u, __fmul_rn(u, p)));
  if (ay > ax) r = __fsub_rn(0x1.921fb6p+0f, r);  // pi/2 - r
  if (x < 0.f) r = __fsub_rn(SHOT_PI, r);
  return y < 0.f ? -r : r;
}

__device__ __forceinline__ float dot3_exact(float a0, float a1, float a2, float b0, float b1, float b2) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a0, b0), __fmul_rn(a1, b1)), __fmul_rn(a2, b2));
}

__device__ __forceinline__ int to_fixed(float t, float scale) { return __float2int_rn(__fmul_rn(t, scale)); }

__device__ __forceinline__ void shot_bins(float pos, int nb, bool circular, int& b0, float& w0, int& b1, float& w1) {
  const float fl = floorf(pos);
  const int lo = (int)fl;
  const float f = __fsub_rn(pos, fl);
  if (circular) {
    b0 = ((lo % nb) + nb) % nb;
    b1 = (b0 + 1) % nb;
    w0 = __fsub_rn(1.f, f);
    w1 = f;
    return;
  }
  if (lo < 0) {
    b0 = 0; w0 = 1.f; b1 = 0; w1 = 0.f;
  } else if (lo >= nb - 1) {
    b0 = nb - 1; w0 = 1.f; b1 = nb - 1; w1 = 0.f;
  } else {
    b0 = lo; w0 = __fsub_rn(1.f, f); b1 = lo + 1; w1 = f;
  }
}

#define SHOT_FOR_SUPPORT(...)                                                                     \
  for (int z = max(cz - 1, 0); z <= min(cz + 1, g.nz - 1); ++z)                                  \
    for (int y = max(cy - 1, 0); y <= min(cy + 1, g.ny - 1); ++y)                                \
      for (int x = max(cx - 1, 0); x <= min(cx + 1, g.nx - 1); ++x) {                            \
        const uint2 c_ = g.cells[((unsigned)z * (unsigned)g.ny + (unsigned)y) * (unsigned)g.nx + (unsigned)x]; \
        for (unsigned j_ = c_.x + (unsigned)lane; j_ < c_.y; j_ += 32) {                         \
          const float4 q = g.pts[j_];                                                            \
          const int qi = pt_index(q);                                                            \
          const float d2 = dist2_exact(kp, q);                                                   \
          if (!(d2 <= R2)) continue;                                                             \
          const float4 qn = nrm[qi];                                                             \
          const float facing = dot3_exact(qn.x, qn.y, qn.z, nk.x, nk.y, nk.z);                   \
          if (!(facing >= SHOT_FACING)) continue;                                                \
          const float dx = __fsub_rn(q.x, kp.x), dy = __fsub_rn(q.y, kp.y), dz = __fsub_rn(q.z, kp.z); \
          __VA_ARGS__                                                                             \
        }                                                                                        \
      }

// The support is gathered once, in pass 1, into a per-warp list in shared
// memory (SHOT_CAP entries: the offset from the keypoint with its squared
// length, and the normal); passes 2 and 3 read the list.  Cells whose box
// lies beyond R are not walked.  A keypoint with more support points than
// the list holds walks the cells again in passes 2 and 3 (the fixed-point
// sums make the order irrelevant).
constexpr int SHOT_CAP = 176;  // with the histograms: 56 KB a block, four blocks an SM

__device__ __forceinline__ float shot_cell_d2(const GridView& g, float4 q, int x, int y, int z) {
  const float lx = g.ox + (float)x * g.h, ly = g.oy + (float)y * g.h, lz = g.oz + (float)z * g.h;
  const float dx = fmaxf(fmaxf(lx - q.x, q.x - (lx + g.h)), 0.f);
  const float dy = fmaxf(fmaxf(ly - q.y, q.y - (ly + g.h)), 0.f);
  const float dz = fmaxf(fmaxf(lz - q.z, q.z - (lz + g.h)), 0.f);
  return dx * dx + dy * dy + dz * dz;
}

// One support point's contribution to the histogram (16 interpolated bins,
// fixed-point votes, scale hs, added by shared-memory atomics).  (dx, dy,
// dz): offset from the keypoint, d2 its exact squared length (> 0), n the
// point's normal.
__device__ __forceinline__ void shot_add(unsigned* H, float hs, float dx, float dy, float dz, float d2, float4 n,
                                         float R, float X0, float X1, float X2, float Y0, float Y1, float Y2,
                                         float Z0, float Z1, float Z2) {
  const float lx = dot3_exact(dx, dy, dz, X0, X1, X2);
  const float ly = dot3_exact(dx, dy, dz, Y0, Y1, Y2);
  const float lz = dot3_exact(dx, dy, dz, Z0, Z1, Z2);
  const float cs = fminf(fmaxf(dot3_exact(n.x, n.y, n.z, Z0, Z1, Z2), -1.f), 1.f);
  const float d = __fsqrt_rn(d2);
  const float az = shot_atan2(ly, lx);
  const float el = shot_atan2(lz, __fsqrt_rn(__fadd_rn(__fmul_rn(lx, lx), __fmul_rn(ly, ly))));
  int cb[2], ab[2], eb[2], rb[2];
  float cw[2], aw[2], ew[2], rw[2];
  shot_bins(__fsub_rn(__fmul_rn(__fadd_rn(cs, 1.f), 5.5f), 0.5f), 11, false, cb[0], cw[0], cb[1], cw[1]);
  shot_bins(__fsub_rn(__fmul_rn(__fadd_rn(az, SHOT_PI), 0x1.45f306p+0f), 0.5f), 8, true, ab[0], aw[0], ab[1], aw[1]);
  shot_bins(__fsub_rn(__fmul_rn(__fadd_rn(el, 0x1.921fb6p+0f), 0x1.45f306p-1f), 0.5f), 2, false, eb[0], ew[0], eb[1],
            ew[1]);
  shot_bins(__fsub_rn(__fmul_rn(__fdiv_rn(d, R), 2.f), 0.5f), 2, false, rb[0], rw[0], rb[1], rw[1]);
#pragma unroll
  for (int i0 = 0; i0 < 2; ++i0)
#pragma unroll
    for (int i1 = 0; i1 < 2; ++i1)
#pragma unroll
      for (int i2 = 0; i2 < 2; ++i2)
#pragma unroll
        for (int i3 = 0; i3 < 2; ++i3) {
          const float w = __fmul_rn(__fmul_rn(__fmul_rn(rw[i0], ew[i1]), aw[i2]), cw[i3]);
          if (w != 0.f) atomicAdd(&H[((rb[i0] * 2 + eb[i1]) * 8 + ab[i2]) * 11 + cb[i3]], __float2uint_rn(__fmul_rn(w, hs)));
        }
}

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(SHOT_WARPS * 32, 4) k_shot(GridDev gd, const float4* __restrict__ pts,
                                                          const float4* __restrict__ nrm,
                                                          const int* __restrict__ keys, int nk_host,
                                                          const int* d_nk, float R,
                                                          float* __restrict__ desc, float* __restrict__ lrf) {
  __shared__ unsigned hist[SHOT_WARPS][352];
  __shared__ float4 s_off[SHOT_WARPS][SHOT_CAP];  // (dx, dy, dz, d^2)
  __shared__ float4 s_nrm[SHOT_WARPS][SHOT_CAP];  // normal
  const GridView g = load_view(gd);
  const int nk_total = cnt_of(nk_host, d_nk);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const float R2 = __fmul_rn(R, R);
  const float cell_r2 = R2 * 1.0001f + 1e-12f;  // a cell is walked when its box is within R (with a margin)
  const int e_cov = 30 - shot_exp2_above(__fmul_rn(R2, R)), e_z = 30 - shot_exp2_above(R);
  const float cov_scale = pow2f(e_cov), cov_unscale = pow2f(-e_cov), z_scale = pow2f(e_z);
  unsigned* H = hist[wid];
  float4* SO = s_off[wid];
  float4* SN = s_nrm[wid];
  for (int kk = blockIdx.x * SHOT_WARPS + wid; kk < nk_total; kk += gridDim.x * SHOT_WARPS) {
    const int key = keys[kk];
    const float4 kp = pts[key];
    const float4 nk = nrm[key];
    const int cx = min(max(q_cell(kp.x, g.ox, g.inv_h), 0), g.nx - 1);
    const int cy = min(max(q_cell(kp.y, g.oy, g.inv_h), 0), g.ny - 1);
    const int cz = min(max(q_cell(kp.z, g.oz, g.inv_h), 0), g.nz - 1);
    // pass 1: weighted covariance (fixed point), and the support gathered in walk order
    long long m0 = 0, m1 = 0, m2 = 0, m3 = 0, m4 = 0, m5 = 0;
    int ns = 0;
    for (int z = max(cz - 1, 0); z <= min(cz + 1, g.nz - 1); ++z)
      for (int y = max(cy - 1, 0); y <= min(cy + 1, g.ny - 1); ++y)
        for (int x = max(cx - 1, 0); x <= min(cx + 1, g.nx - 1); ++x) {
          if (shot_cell_d2(g, kp, x, y, z) > cell_r2) continue;
          const uint2 c = g.cells[((unsigned)z * (unsigned)g.ny + (unsigned)y) * (unsigned)g.nx + (unsigned)x];
          for (unsigned j0 = c.x; j0 < c.y; j0 += 32) {
            const unsigned j = j0 + (unsigned)lane;
            bool in = false;
            float4 q = kp, qn = nk;
            float d2 = 0.f;
            if (j < c.y) {
              q = g.pts[j];
              d2 = dist2_exact(kp, q);
              if (d2 <= R2) {
                qn = nrm[pt_index(q)];
                in = dot3_exact(qn.x, qn.y, qn.z, nk.x, nk.y, nk.z) >= SHOT_FACING;
              }
            }
            const float dx = __fsub_rn(q.x, kp.x), dy = __fsub_rn(q.y, kp.y), dz = __fsub_rn(q.z, kp.z);
            if (in) {
              const float w = __fsub_rn(R, __fsqrt_rn(d2));
              const float wx = __fmul_rn(w, dx), wy = __fmul_rn(w, dy);
              m0 += to_fixed(__fmul_rn(wx, dx), cov_scale);
              m1 += to_fixed(__fmul_rn(wx, dy), cov_scale);
              m2 += to_fixed(__fmul_rn(wx, dz), cov_scale);
              m3 += to_fixed(__fmul_rn(wy, dy), cov_scale);
              m4 += to_fixed(__fmul_rn(wy, dz), cov_scale);
              m5 += to_fixed(__fmul_rn(__fmul_rn(w, dz), dz), cov_scale);
            }
            const unsigned bal = __ballot_sync(0xffffffffu, in);
            const int slot = ns + __popc(bal & lanemask_lt());
            if (in && slot < SHOT_CAP) {
              SO[slot] = make_float4(dx, dy, dz, d2);
              SN[slot] = qn;
            }
            ns += __popc(bal);
          }
        }
    __syncwarp();
    const bool listed = ns <= SHOT_CAP;
    float M[9];
    M[0] = __fmul_rn(__ll2float_rn(warp_sum_ll(m0)), cov_unscale);
    M[1] = M[3] = __fmul_rn(__ll2float_rn(warp_sum_ll(m1)), cov_unscale);
    M[2] = M[6] = __fmul_rn(__ll2float_rn(warp_sum_ll(m2)), cov_unscale);
    M[4] = __fmul_rn(__ll2float_rn(warp_sum_ll(m3)), cov_unscale);
    M[5] = M[7] = __fmul_rn(__ll2float_rn(warp_sum_ll(m4)), cov_unscale);
    M[8] = __fmul_rn(__ll2float_rn(warp_sum_ll(m5)), cov_unscale);
    float ev[3], V[9];
    eig3_exact(M, ev, V);
    float X0 = V[2], X1 = V[5], X2 = V[8], Z0 = V[0], Z1 = V[3], Z2 = V[6];
    // pass 2: signs (x: majority of offsets; z: sum of w (n . z), fixed point)
    int px = 0, nx = 0;
    long long zn = 0;
    if (listed) {
      for (int i = lane; i < ns; i += 32) {
        const float4 o = SO[i], qn = SN[i];
        if (dot3_exact(o.x, o.y, o.z, X0, X1, X2) >= 0.f) ++px; else ++nx;
        const float w = __fsub_rn(R, __fsqrt_rn(o.w));
        zn += to_fixed(__fmul_rn(w, dot3_exact(qn.x, qn.y, qn.z, Z0, Z1, Z2)), z_scale);
      }
    } else {
      SHOT_FOR_SUPPORT({
        if (dot3_exact(dx, dy, dz, X0, X1, X2) >= 0.f) ++px; else ++nx;
        const float w = __fsub_rn(R, __fsqrt_rn(d2));
        zn += to_fixed(__fmul_rn(w, dot3_exact(qn.x, qn.y, qn.z, Z0, Z1, Z2)), z_scale);
      })
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      px += __shfl_xor_sync(0xffffffffu, px, o);
      nx += __shfl_xor_sync(0xffffffffu, nx, o);
    }
    zn = warp_sum_ll(zn);
    if (px < nx) { X0 = -X0; X1 = -X1; X2 = -X2; }
    if (zn < 0) { Z0 = -Z0; Z1 = -Z1; Z2 = -Z2; }
    const float Y0 = __fsub_rn(__fmul_rn(Z1, X2), __fmul_rn(Z2, X1));
    const float Y1 = __fsub_rn(__fmul_rn(Z2, X0), __fmul_rn(Z0, X2));
    const float Y2 = __fsub_rn(__fmul_rn(Z0, X1), __fmul_rn(Z1, X0));
    if (lrf && lane == 0) {
      float* L = lrf + (size_t)kk * 9;
      L[0] = X0; L[1] = X1; L[2] = X2; L[3] = Y0; L[4] = Y1; L[5] = Y2; L[6] = Z0; L[7] = Z1; L[8] = Z2;
    }
    for (int b = lane; b < 352; b += 32) H[b] = 0u;
    __syncwarp();
    // pass 3: histogram (the keypoint itself, d = 0, does not vote)
    const int e_h = 31 - (32 - __clz(ns));
    const float hs = pow2f(e_h);
    if (listed) {
      for (int i = lane; i < ns; i += 32) {
        const float4 o = SO[i];
        if (o.w > 0.f) shot_add(H, hs, o.x, o.y, o.z, o.w, SN[i], R, X0, X1, X2, Y0, Y1, Y2, Z0, Z1, Z2);
      }
    } else {
      SHOT_FOR_SUPPORT({
        if (d2 > 0.f) shot_add(H, hs, dx, dy, dz, d2, qn, R, X0, X1, X2, Y0, Y1, Y2, Z0, Z1, Z2);
      })
    }
    __syncwarp();
    // L2 norm: lane l sums bins l, l + 32, ..., l + 320 in order, then the
    // xor butterfly (each step adds the same two values in both lanes)
    float hb[11];
    float ss = 0.f;
    const float hu = pow2f(-e_h);
#pragma unroll
    for (int k = 0; k < 11; ++k) {
      hb[k] = __fmul_rn(__uint2float_rn(H[lane + 32 * k]), hu);
      ss = __fadd_rn(ss, __fmul_rn(hb[k], hb[k]));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ss = __fadd_rn(ss, __shfl_xor_sync(0xffffffffu, ss, o));
    const float inv = ss > 0.f ? __fdiv_rn(1.f, __fsqrt_rn(ss)) : 0.f;
    float* D = desc + (size_t)kk * 352;
#pragma unroll
    for (int k = 0; k < 11; ++k) D[lane + 32 * k] = __fmul_rn(hb[k], inv);
    __syncwarp();
  }
}
// ---------------------------------------------------------------------------
// host entry points
// ---------------------------------------------------------------------------
rtr_status voxel_downsample_dev(rtr_context* ctx, Scratch& s, const float4* pts, int n_cap, const int* d_n,
                                float leaf, float4* out, int* d_count, cudaStream_t st) {
  VoxSeg v;
  if (!voxseg_take(s, n_cap, &v)) return fail(RTR_ERR_CAPACITY, "voxel_downsample: scratch");
  const float inv = 1.0f / leaf;
  voxseg_build(v, pts, n_cap, d_n, inv, st);
  k_vox_centroid<<<blocks_for(n_cap), 256, 0, st>>>(pts, v.order, v.seg_start, v.d_nseg, v.meta, out, d_count);
  RTR_LAUNCHED(1);
  return RTR_OK;
}

rtr_status uniform_sample_dev(rtr_context* ctx, Scratch& s, const float4* pts, int n_cap, const int* d_n,
                              float r, int* out, int* d_count, cudaStream_t st) {
  VoxSeg v;
  if (!voxseg_take(s, n_cap, &v)) return fail(RTR_ERR_CAPACITY, "uniform_sample: scratch");
  const float inv = 1.0f / r;
  voxseg_build(v, pts, n_cap, d_n, inv, st);
  k_uniform_pick<<<blocks_for(n_cap), 256, 0, st>>>(pts, v.order, v.seg_start, v.d_nseg, v.meta, inv, r, out, d_count);
  RTR_LAUNCHED(1);
  return RTR_OK;
}

rtr_status normals_dev(rtr_context* ctx, Scratch& s, const float4* pts, int n_cap, const int* d_n, int k,
                       const float vp[3], float cell, float4* out, cudaStream_t st) {
  GridBufs gb;
  const unsigned cap = default_cell_cap(n_cap);
  if (!grid_take(s, n_cap, cap, &gb)) return fail(RTR_ERR_CAPACITY, "normals: scratch");
  grid_build(gb, pts, n_cap, d_n, cell, st);
  const int nb = blocks_for(n_cap, 128);
  if (k <= 8)
    k_normals<8><<<nb, 128, 0, st>>>(grid_dev(gb), pts, n_cap, d_n, vp[0], vp[1], vp[2], out);
  else if (k <= 10)
    k_normals<10><<<nb, 128, 0, st>>>(grid_dev(gb), pts, n_cap, d_n, vp[0], vp[1], vp[2], out);
  else if (k <= 16)
    k_normals<16><<<nb, 128, 0, st>>>(grid_dev(gb), pts, n_cap, d_n, vp[0], vp[1], vp[2], out);
  else
    return fail(RTR_ERR_INVALID_ARG, "normals: k must be 8, 10 or 16");
  RTR_LAUNCHED(1);
  return RTR_OK;
}

// SHOT over a grid of the points already built with cell R (grid_build).
rtr_status shot_on_grid(const GridBufs& gb, const float4* pts, const float4* nrm, const int* keys, int nk_cap,
                        const int* d_nk, float R, float* desc, float* lrf, cudaStream_t st) {
  // the fixed-point scales of k_shot are powers of two derived from R
  if (!(R >= 1e-6f && R <= 1e6f)) return fail(RTR_ERR_INVALID_ARG, "shot: radius outside [1e-6, 1e6]");
  k_shot<<<blocks_for(nk_cap, SHOT_WARPS, 152 * 32), SHOT_WARPS * 32, 0, st>>>(grid_dev(gb), pts, nrm, keys, nk_cap,
                                                                                d_nk, R, desc, lrf);
  RTR_LAUNCHED(1);
  return RTR_OK;
}

rtr_status shot_dev(rtr_context* ctx, Scratch& s, const float4* pts, const float4* nrm, int n_cap, const int* d_n,
                    const int* keys, int nk_cap, const int* d_nk, float R, float* desc, float* lrf,
                    cudaStream_t st) {
  GridBufs gb;
  const unsigned cap = default_cell_cap(n_cap);
  if (!grid_take(s, n_cap, cap, &gb)) return fail(RTR_ERR_CAPACITY, "shot: scratch");
  grid_build(gb, pts, n_cap, d_n, R, st);
  return shot_on_grid(gb, pts, nrm, keys, nk_cap, d_nk, R, desc, lrf, st);
}

}  // namespace rtr

using namespace rtr;

static size_t vox_plan_bytes(int n) {
  ScratchPlan p;
  voxseg_plan(p, n);
  return p.bytes;
}

extern "C" {

rtr_status rtr_voxel_downsample(rtr_context* ctx, const float* d_pts, int n, float leaf, float* d_out,
                                int* d_count, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n >= 0 && d_count && leaf > 0.f, "rtr_voxel_downsample: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (n == 0) {
    RTR_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int), st));
    return RTR_OK;
  }
  RTR_CHECK_ARG(d_pts && d_out, "rtr_voxel_downsample: NULL points or output");
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, vox_plan_bytes(n), st, &s));
  ProfScope ps(ctx, st, "voxel_downsample");
  return voxel_downsample_dev(ctx, s, reinterpret_cast<const float4*>(d_pts), n, nullptr, leaf,
                              reinterpret_cast<float4*>(d_out), d_count, st);
}

rtr_status rtr_uniform_sample(rtr_context* ctx, const float* d_pts, int n, float radius, int32_t* d_idx,
                              int* d_count, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n >= 0 && d_count && radius > 0.f, "rtr_uniform_sample: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (n == 0) {
    RTR_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int), st));
    return RTR_OK;
  }
  RTR_CHECK_ARG(d_pts && d_idx, "rtr_uniform_sample: NULL points or output");
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, vox_plan_bytes(n), st, &s));
  ProfScope ps(ctx, st, "uniform_sample");
  return uniform_sample_dev(ctx, s, reinterpret_cast<const float4*>(d_pts), n, nullptr, radius, d_idx, d_count, st);
}

rtr_status rtr_normals(rtr_context* ctx, const float* d_pts, int n, int k, const float* h_vp3, float search_cell,
                       float* d_normals, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n >= 0 && (k == 8 || k == 10 || k == 16), "rtr_normals: k must be 8, 10 or 16");
  if (n == 0) return RTR_OK;
  RTR_CHECK_ARG(d_pts && d_normals, "rtr_normals: NULL points or output");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  ScratchPlan p;
  grid_plan(p, n, default_cell_cap(n));
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, p.bytes, st, &s));
  const float vp[3] = {h_vp3 ? h_vp3[0] : 0.f, h_vp3 ? h_vp3[1] : 0.f, h_vp3 ? h_vp3[2] : 0.f};
  ProfScope ps(ctx, st, "normals");
  return normals_dev(ctx, s, reinterpret_cast<const float4*>(d_pts), n, nullptr, k, vp, search_cell,
                     reinterpret_cast<float4*>(d_normals), st);
}

rtr_status rtr_orient_normals_outward(rtr_context* ctx, const float* d_pts, float* d_normals, int n, float rc,
                                      float gap, float len, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n >= 0 && rc > 0.f && len > gap, "rtr_orient_normals_outward: bad arguments");
  if (n == 0) return RTR_OK;
  RTR_CHECK_ARG(d_pts && d_normals, "rtr_orient_normals_outward: NULL pointer");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  ProfScope ps(ctx, st, "orient_outward");
  const float rc2 = rc * rc;
  k_orient_outward<<<blocks_for(n, 8, 152 * 16), 256, 0, st>>>(reinterpret_cast<const float4*>(d_pts),
                                                                reinterpret_cast<float4*>(d_normals), n, nullptr,
                                                                rc2, gap, len);
  RTR_LAUNCHED(1);
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

rtr_status rtr_shot352(rtr_context* ctx, const float* d_pts, const float* d_normals, int n, const int32_t* d_keys,
                       int nk, float radius, float* d_desc, float* d_lrf, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n >= 0 && nk >= 0 && radius > 0.f, "rtr_shot352: bad arguments");
  if (nk == 0) return RTR_OK;
  RTR_CHECK_ARG(d_pts && d_normals && d_keys && d_desc && n > 0, "rtr_shot352: NULL pointer or empty cloud");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  ScratchPlan p;
  grid_plan(p, n, default_cell_cap(n));
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, p.bytes, st, &s));
  ProfScope ps(ctx, st, "shot352");
  return shot_dev(ctx, s, reinterpret_cast<const float4*>(d_pts), reinterpret_cast<const float4*>(d_normals), n,
                  nullptr, d_keys, nk, nullptr, radius, d_desc, d_lrf, st);
}

}  // extern "C"
