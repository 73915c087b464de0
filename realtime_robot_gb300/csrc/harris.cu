// harris.cu — the reference's keypoint detector: pcl::HarrisKeypoint3D as
// ModelPoint::getKeypoint / ScanPoint::getKeypoint use it (model_point.h:
// 127-136, scan_point.h:85-94: radius 0.05, threshold 0.01, non-maximum
// suppression, refinement at its default).  The operator is the 3-D Harris
// response on surface normals (Sipiran & Bustos 2011):
//   normal   smallest eigenvector of the neighbours' FP32 covariance;
//   M        mean of n n^T over the neighbours' normals;
//   R        det(M) - k tr(M)^2 + k, k = 0.04 (for unit normals tr(M) = 1
//            and R = det(M): 0 on faces and edges, up to 1/27 at a corner
//            of three faces, the scale the reference's 0.01 threshold fits);
//   keypoint R > threshold and no neighbour's R larger;
//   refine   the least-squares intersection of the tangent planes near the
//            keypoint (FP64), up to 10 steps.
// Neighbours are every point within the radius, the point included; every
// sum runs over them in ascending index order, so the results equal the CPU
// oracle's (oracle/harris.c) bit for bit.
//
// Kernels: one warp per point.  The warp walks the 27 grid cells (edge =
// radius) around the point, ballots the points within the radius into a
// shared list, sorts the list by index (bitonic) and lane 0 sums in that
// order.  A list longer than HR_CAP sets an error (RTR_ERR_CAPACITY).
#include <limits.h>
#include <string.h>

#include "eig3.cuh"
#include "grid.cuh"
#include "scan.cuh"
#include "search.cuh"

namespace rtr {

constexpr int HR_WARPS = 8;
constexpr int HR_CAP = 1024;  // neighbours of one point within the radius

struct HrArgs {
  GridDev grid;
  const float4* pts;
  int n;
  float r, r2;
  int* err;
};

// the points within r of q (original indices), ascending; returns the count
// (HR_CAP + 1 on overflow, with *err set)
// The cells that can hold a point within r of q: those of q -+ rr on each
// axis, rr = r with a margin over the rounding of q -+ rr (the cell index is
// monotone in the coordinate).
struct HrBox {
  int x0, x1, y0, y1, z0, z1;
};
__device__ __forceinline__ HrBox hr_box(const GridView& g, float4 q, float r) {
  const float rr = __fadd_rn(__fmul_rn(r, 1.0001f), 1e-6f);
  HrBox b;
  b.x0 = min(max(q_cell(__fsub_rn(q.x, rr), g.ox, g.inv_h), 0), g.nx - 1);
  b.x1 = min(max(q_cell(__fadd_rn(q.x, rr), g.ox, g.inv_h), 0), g.nx - 1);
  b.y0 = min(max(q_cell(__fsub_rn(q.y, rr), g.oy, g.inv_h), 0), g.ny - 1);
  b.y1 = min(max(q_cell(__fadd_rn(q.y, rr), g.oy, g.inv_h), 0), g.ny - 1);
  b.z0 = min(max(q_cell(__fsub_rn(q.z, rr), g.oz, g.inv_h), 0), g.nz - 1);
  b.z1 = min(max(q_cell(__fadd_rn(q.z, rr), g.oz, g.inv_h), 0), g.nz - 1);
  return b;
}

__device__ int hr_gather(const HrArgs& a, const GridView& g, float4 q, int* list, int lane) {
  const HrBox bb = hr_box(g, q, a.r);
  int cnt = 0;
  for (int z = bb.z0; z <= bb.z1; ++z)
    for (int y = bb.y0; y <= bb.y1; ++y)
      for (int x = bb.x0; x <= bb.x1; ++x) {
        const uint2 c = g.cells[((unsigned)z * (unsigned)g.ny + (unsigned)y) * (unsigned)g.nx + (unsigned)x];
        for (unsigned j0 = c.x; j0 < c.y; j0 += 32) {
          const unsigned j = j0 + (unsigned)lane;
          bool in = false;
          int id = 0;
          if (j < c.y) {
            const float4 p = g.pts[j];
            in = dist2_exact(q, p) <= a.r2;
            id = pt_index(p);
          }
          const unsigned b = __ballot_sync(0xffffffffu, in);
          if (in) {
            const int pos = cnt + __popc(b & lanemask_lt());
            if (pos < HR_CAP) list[pos] = id;
          }
          cnt += __popc(b);
        }
      }
  if (cnt > HR_CAP) {
    if (lane == 0) atomicOr(a.err, 1);
    return HR_CAP + 1;
  }
  // ascending index: bitonic sort over the next power of two
  int P = 1;
  while (P < cnt) P <<= 1;
  for (int i = cnt + lane; i < P; i += 32) list[i] = INT_MAX;
  __syncwarp();
  for (int k = 2; k <= P; k <<= 1)
    for (int jj = k >> 1; jj > 0; jj >>= 1) {
      for (int t = lane; t < (P >> 1); t += 32) {
        const int i = ((t & ~(jj - 1)) << 1) | (t & (jj - 1));
        const int l = i | jj;
        const int x = list[i], y = list[l];
        if ((x > y) == ((i & k) == 0)) {
          list[i] = y;
          list[l] = x;
        }
      }
      __syncwarp();
    }
  return cnt;
}

__global__ void __launch_bounds__(HR_WARPS * 32) k_hr_normals(HrArgs a, float4* __restrict__ nrm) {
  __shared__ int s_list[HR_WARPS][HR_CAP + 1];
  const GridView g = load_view(a.grid);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int* list = s_list[w];
  for (int i = blockIdx.x * HR_WARPS + w; i < a.n; i += gridDim.x * HR_WARPS) {
    const float4 q = a.pts[i];
    const int cnt = hr_gather(a, g, q, list, lane);
    if (lane == 0) {
      float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
      if (cnt <= HR_CAP) {
        float mx = 0.f, my = 0.f, mz = 0.f;
        for (int k = 0; k < cnt; ++k) {
          const float4 p = a.pts[list[k]];
          mx = __fadd_rn(mx, p.x);
          my = __fadd_rn(my, p.y);
          mz = __fadd_rn(mz, p.z);
        }
        const float c = (float)cnt;
        mx = __fdiv_rn(mx, c);
        my = __fdiv_rn(my, c);
        mz = __fdiv_rn(mz, c);
        float C[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int k = 0; k < cnt; ++k) {
          const float4 p = a.pts[list[k]];
          const float dx = __fsub_rn(p.x, mx), dy = __fsub_rn(p.y, my), dz = __fsub_rn(p.z, mz);
          C[0] = __fadd_rn(C[0], __fmul_rn(dx, dx));
          C[1] = __fadd_rn(C[1], __fmul_rn(dx, dy));
          C[2] = __fadd_rn(C[2], __fmul_rn(dx, dz));
          C[3] = __fadd_rn(C[3], __fmul_rn(dy, dy));
          C[4] = __fadd_rn(C[4], __fmul_rn(dy, dz));
          C[5] = __fadd_rn(C[5], __fmul_rn(dz, dz));
        }
        const float A[9] = {C[0], C[1], C[2], C[1], C[3], C[4], C[2], C[4], C[5]};
        float ev[3], V[9];
        eig3_exact(A, ev, V);
        out = make_float4(V[0], V[3], V[6], 0.f);
      }
      nrm[i] = out;
    }
    __syncwarp();
  }
}

__device__ __forceinline__ float hr_det3(const float* m) {
  const float a = __fsub_rn(__fmul_rn(m[3], m[5]), __fmul_rn(m[4], m[4]));
  const float b = __fsub_rn(__fmul_rn(m[1], m[5]), __fmul_rn(m[4], m[2]));
  const float c = __fsub_rn(__fmul_rn(m[1], m[4]), __fmul_rn(m[3], m[2]));
  return __fadd_rn(__fsub_rn(__fmul_rn(m[0], a), __fmul_rn(m[1], b)), __fmul_rn(m[2], c));
}

__global__ void __launch_bounds__(HR_WARPS * 32) k_hr_response(HrArgs a, const float4* __restrict__ nrm,
                                                                float* __restrict__ R) {
  __shared__ int s_list[HR_WARPS][HR_CAP + 1];
  const GridView g = load_view(a.grid);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int* list = s_list[w];
  for (int i = blockIdx.x * HR_WARPS + w; i < a.n; i += gridDim.x * HR_WARPS) {
    const int cnt = hr_gather(a, g, a.pts[i], list, lane);
    if (lane == 0) {
      float r = 0.f;
      if (cnt <= HR_CAP) {
        float M[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        for (int k = 0; k < cnt; ++k) {
          const float4 v = nrm[list[k]];
          M[0] = __fadd_rn(M[0], __fmul_rn(v.x, v.x));
          M[1] = __fadd_rn(M[1], __fmul_rn(v.x, v.y));
          M[2] = __fadd_rn(M[2], __fmul_rn(v.x, v.z));
          M[3] = __fadd_rn(M[3], __fmul_rn(v.y, v.y));
          M[4] = __fadd_rn(M[4], __fmul_rn(v.y, v.z));
          M[5] = __fadd_rn(M[5], __fmul_rn(v.z, v.z));
        }
        const float c = (float)cnt;
#pragma unroll
        for (int e = 0; e < 6; ++e) M[e] = __fdiv_rn(M[e], c);
        const float tr = __fadd_rn(__fadd_rn(M[0], M[3]), M[5]);
        r = __fadd_rn(__fsub_rn(hr_det3(M), __fmul_rn(0.04f, __fmul_rn(tr, tr))), 0.04f);
      }
      R[i] = r;
    }
    __syncwarp();
  }
}

// keypoint flags: R over the threshold and (non_max) no neighbour larger
__global__ void __launch_bounds__(HR_WARPS * 32) k_hr_select(HrArgs a, const float* __restrict__ R, float thr,
                                                              int non_max, uint32_t* __restrict__ flag) {
  const GridView g = load_view(a.grid);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = blockIdx.x * HR_WARPS + w; i < a.n; i += gridDim.x * HR_WARPS) {
    const float ri = R[i];
    bool ok = ri > thr;
    if (ok && non_max) {
      const float4 q = a.pts[i];
      const HrBox bb = hr_box(g, q, a.r);
      for (int z = bb.z0; z <= bb.z1 && ok; ++z)
        for (int y = bb.y0; y <= bb.y1 && ok; ++y)
          for (int x = bb.x0; x <= bb.x1 && ok; ++x) {
            const uint2 c = g.cells[((unsigned)z * (unsigned)g.ny + (unsigned)y) * (unsigned)g.nx + (unsigned)x];
            bool larger = false;
            for (unsigned j = c.x + (unsigned)lane; j < c.y; j += 32) {
              const float4 p = g.pts[j];
              if (dist2_exact(q, p) <= a.r2 && ri < R[pt_index(p)]) larger = true;
            }
            ok = !__any_sync(0xffffffffu, larger);
          }
    }
    if (lane == 0) flag[i] = ok ? 1u : 0u;
  }
}

// refinement and output of the keypoints (ascending source index)
__global__ void __launch_bounds__(HR_WARPS * 32) k_hr_refine(HrArgs a, const float4* __restrict__ nrm,
                                                              const float* __restrict__ R,
                                                              const uint32_t* __restrict__ flag,
                                                              const uint32_t* __restrict__ pos, int refine,
                                                              float4* __restrict__ keys, int* __restrict__ src) {
  __shared__ int s_list[HR_WARPS][HR_CAP + 1];
  const GridView g = load_view(a.grid);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int* list = s_list[w];
  for (int i = blockIdx.x * HR_WARPS + w; i < a.n; i += gridDim.x * HR_WARPS) {
    if (!flag[i]) continue;  // uniform in the warp
    const float4 p0 = a.pts[i];
    float4 x = make_float4(p0.x, p0.y, p0.z, 0.f);
    if (refine) {
      for (int it = 0; it < 10; ++it) {
        const int cnt = hr_gather(a, g, x, list, lane);
        int stop = 0;
        float4 y = x;
        if (lane == 0) {
          if (cnt > HR_CAP) {
            stop = 1;
          } else {
            double A[6] = {0, 0, 0, 0, 0, 0}, b[3] = {0, 0, 0};
            for (int k = 0; k < cnt; ++k) {
              const float4 v = nrm[list[k]];
              const float4 p = a.pts[list[k]];
              const double nx = v.x, ny = v.y, nz = v.z;
              const double d = __dadd_rn(__dadd_rn(__dmul_rn(nx, (double)p.x), __dmul_rn(ny, (double)p.y)),
                                         __dmul_rn(nz, (double)p.z));
              A[0] = __dadd_rn(A[0], __dmul_rn(nx, nx));
              A[1] = __dadd_rn(A[1], __dmul_rn(nx, ny));
              A[2] = __dadd_rn(A[2], __dmul_rn(nx, nz));
              A[3] = __dadd_rn(A[3], __dmul_rn(ny, ny));
              A[4] = __dadd_rn(A[4], __dmul_rn(ny, nz));
              A[5] = __dadd_rn(A[5], __dmul_rn(nz, nz));
              b[0] = __dadd_rn(b[0], __dmul_rn(nx, d));
              b[1] = __dadd_rn(b[1], __dmul_rn(ny, d));
              b[2] = __dadd_rn(b[2], __dmul_rn(nz, d));
            }
            const double c00 = __dsub_rn(__dmul_rn(A[3], A[5]), __dmul_rn(A[4], A[4]));
            const double c01 = __dsub_rn(__dmul_rn(A[2], A[4]), __dmul_rn(A[1], A[5]));
            const double c02 = __dsub_rn(__dmul_rn(A[1], A[4]), __dmul_rn(A[2], A[3]));
            const double det = __dadd_rn(__dadd_rn(__dmul_rn(A[0], c00), __dmul_rn(A[1], c01)), __dmul_rn(A[2], c02));
            const double tr = __dadd_rn(__dadd_rn(A[0], A[3]), A[5]);
            if (!(det > __dmul_rn(__dmul_rn(__dmul_rn(1e-12, tr), tr), tr))) {
              stop = 1;
            } else {
              const double c11 = __dsub_rn(__dmul_rn(A[0], A[5]), __dmul_rn(A[2], A[2]));
              const double c12 = __dsub_rn(__dmul_rn(A[1], A[2]), __dmul_rn(A[0], A[4]));
              const double c22 = __dsub_rn(__dmul_rn(A[0], A[3]), __dmul_rn(A[1], A[1]));
              const double px = __ddiv_rn(__dadd_rn(__dadd_rn(__dmul_rn(c00, b[0]), __dmul_rn(c01, b[1])),
                                                    __dmul_rn(c02, b[2])), det);
              const double py = __ddiv_rn(__dadd_rn(__dadd_rn(__dmul_rn(c01, b[0]), __dmul_rn(c11, b[1])),
                                                    __dmul_rn(c12, b[2])), det);
              const double pz = __ddiv_rn(__dadd_rn(__dadd_rn(__dmul_rn(c02, b[0]), __dmul_rn(c12, b[1])),
                                                    __dmul_rn(c22, b[2])), det);
              y = make_float4((float)px, (float)py, (float)pz, 0.f);
              if (!(dist2_exact(y, p0) <= a.r2)) {
                stop = 1;
              } else {
                const float mv = dist2_exact(y, x);
                if (mv < 1e-12f) stop = 2;  // moved, then done
              }
            }
          }
        }
        stop = __shfl_sync(0xffffffffu, stop, 0);
        y.x = __shfl_sync(0xffffffffu, y.x, 0);
        y.y = __shfl_sync(0xffffffffu, y.y, 0);
        y.z = __shfl_sync(0xffffffffu, y.z, 0);
        if (stop == 1) break;
        x = y;
        if (stop == 2) break;
        __syncwarp();
      }
    }
    if (lane == 0) {
      const unsigned k = pos[i];
      keys[k] = make_float4(x.x, x.y, x.z, R[i]);
      if (src) src[k] = i;
    }
    __syncwarp();
  }
}

static int hr_blocks(int n) {
  int b = (n + HR_WARPS - 1) / HR_WARPS;
  if (b > 152 * 16) b = 152 * 16;
  return b < 1 ? 1 : b;
}

}  // namespace rtr

using namespace rtr;

extern "C" {

void rtr_harris_default_params(rtr_harris_params* p) {
  if (!p) return;
  memset(p, 0, sizeof(*p));
  p->radius = 0.05f;
  p->threshold = 0.01f;
  p->non_max = 1;
  p->refine = 1;
}

rtr_status rtr_harris3d(rtr_context* ctx, const float* d_pts, int n, const rtr_harris_params* prm, float* d_keys,
                        int32_t* d_src, int* d_count, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && prm && n >= 0 && d_count, "rtr_harris3d: bad arguments");
  RTR_CHECK_ARG(prm->radius > 0.f && isfinite(prm->radius), "rtr_harris3d: radius must be positive");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (n == 0) {
    RTR_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int), st));
    return RTR_OK;
  }
  RTR_CHECK_ARG(d_pts && d_keys, "rtr_harris3d: NULL points or output");
  const unsigned cap = default_cell_cap(n);
  ScratchPlan plan;
  grid_plan(plan, n, cap);
  const size_t o_n = plan.add<float4>(n), o_r = plan.add<float>(n), o_f = plan.add<uint32_t>(n + 1),
               o_p = plan.add<uint32_t>(n + 1), o_t = plan.add<uint32_t>(scan_tiles(n + 1)), o_e = plan.add<int>(4);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  GridBufs gb;
  if (!grid_take(s, n, cap, &gb)) return fail(RTR_ERR_CAPACITY, "rtr_harris3d: scratch carve");
  // the plan's own entries follow the grid's in the arena
  float4* nrm = reinterpret_cast<float4*>(s.base + o_n);
  float* R = reinterpret_cast<float*>(s.base + o_r);
  uint32_t* flag = reinterpret_cast<uint32_t*>(s.base + o_f);
  uint32_t* pos = reinterpret_cast<uint32_t*>(s.base + o_p);
  uint32_t* tiles = reinterpret_cast<uint32_t*>(s.base + o_t);
  int* err = reinterpret_cast<int*>(s.base + o_e);
  ProfScope ps(ctx, st, "harris3d");
  const float4* pts = reinterpret_cast<const float4*>(d_pts);
  grid_build(gb, pts, n, nullptr, prm->radius, st);
  RTR_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
  HrArgs a{grid_dev(gb), pts, n, prm->radius, prm->radius * prm->radius, err};
  const int nb = hr_blocks(n);
  k_hr_normals<<<nb, HR_WARPS * 32, 0, st>>>(a, nrm);
  k_hr_response<<<nb, HR_WARPS * 32, 0, st>>>(a, nrm, R);
  k_hr_select<<<nb, HR_WARPS * 32, 0, st>>>(a, R, prm->threshold, prm->non_max, flag);
  scan_exclusive(flag, pos, tiles, n + 1, n, nullptr, reinterpret_cast<uint32_t*>(d_count), st);
  k_hr_refine<<<nb, HR_WARPS * 32, 0, st>>>(a, nrm, R, flag, pos, prm->refine, reinterpret_cast<float4*>(d_keys),
                                            d_src);
  RTR_LAUNCHED(4);
  RTR_CUDA(cudaGetLastError());
  int h_err = 0;
  RTR_CUDA(cudaMemcpyAsync(&h_err, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  RTR_CUDA(cudaStreamSynchronize(st));
  if (h_err)
    return fail(RTR_ERR_CAPACITY, "rtr_harris3d: a point has more than %d neighbours within the radius", HR_CAP);
  return RTR_OK;
}

}  // extern "C"
