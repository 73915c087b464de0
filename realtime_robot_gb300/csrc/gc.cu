// gc.cu — geometric-consistency grouping (Chen & Bhanu 2007; PCL
// GeometricConsistencyGrouping), which takes the place of the reference's
// pair-consensus loop (Ransac, function.h:35-109).
//
// Semantics (shared with the oracle): correspondences sorted by descriptor
// distance (ties: input order); each not-yet-taken correspondence, in that
// order, seeds a consensus set that admits, in the same order, every
// not-taken correspondence whose model-side and scene-side distances to EVERY
// member differ by at most gc_size; a set of >= gc_thresh members becomes a
// cluster and its members are taken.
//
// GPU form.  The sequential loop is O(C^2) but its parallel part, each
// seed's set, is only needed for the seeds the walk reaches before it stops
// (at max_clusters, often a few hundred seeds into a cluttered scene).  One
// cooperative launch alternates two phases: all warps compute the sets of a
// window of upcoming seeds under the current taken state, then one warp walks
// the seeds in order and commits.  A stored set stays exact while none of its
// members is taken (removing rejected candidates never changes a greedy
// walk); the walk stops at the first seed whose set lost a member and the
// next window starts there.  No host round trip inside the grouping.
#include "common.cuh"
#include "pose.cuh"
#include "grid.cuh"

namespace rtr {

constexpr int GC_WARPS = 8;
constexpr int GC_TILE = 256;
constexpr int GC_MAXS = 128;  // members per consensus set (larger sets: RTR_ERR_CAPACITY)

struct GcDev {
  const float4* pm;        // model keypoint of sorted correspondence a
  const float4* ps;        // scene keypoint of sorted correspondence a
  int C;
  float gc;
  unsigned* taken;         // bitset over sorted positions
  int* set_size;           // [C]
  int* set_mem;            // [C][GC_MAXS] sorted positions
};

__device__ __forceinline__ bool gc_consistent(float4 am, float4 as, float4 bm, float4 bs, float gc) {
  const float dm = __fsqrt_rn(dist2_exact(am, bm));
  const float ds = __fsqrt_rn(dist2_exact(as, bs));
  return !(fabsf(__fsub_rn(dm, ds)) > gc);
}

// Device-side control block of the grouping walk.
struct GcCoop {
  int* ctl;            // [0] walk position, [1] clusters, [2] done, [3] error status, [4] rounds
  unsigned* arrive;    // grid barrier counter (zero at launch)
  int* computed;       // [C] 1 once the seed's set has been computed
  int* cl_members;     // [max_clusters][GC_MAXS] sorted positions
  int* cl_sizes;       // [max_clusters]
  int thresh, max_clusters;
  long long budget;    // clock64 cycles per barrier wait
  int* status;         // context status word
};

__device__ __forceinline__ bool sbit(const unsigned* s, int i) { return (s[i >> 5] >> (i & 31)) & 1u; }

// Grid barrier (all blocks co-resident: cooperative launch).  Bounded: a
// block that waits longer than the budget records RTR_ERR_TIMEOUT and
// returns false.
__device__ __forceinline__ bool gc_barrier(const GcCoop& c, unsigned target, int* s_ok) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(c.arrive, 1u);
    const long long t0 = clock64();
    int ok = 1;
    while (ld_acquire_gpu(c.arrive) < target) {
      if (clock64() - t0 > c.budget) {
        atomicExch(c.status, (int)RTR_ERR_TIMEOUT);
        atomicExch(c.ctl + 3, (int)RTR_ERR_TIMEOUT);
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

// The whole grouping in one cooperative launch.  Rounds of two phases:
//  A. every warp takes one seed of the window [pos, pos + warps) and, unless
//     the seed is taken or its stored set is still exact (no member taken
//     since it was computed), computes its consensus set under the current
//     taken state: candidates streamed through shared memory in tiles;
//  B. warp 0 of block 0 walks the seeds in order from pos: taken seeds are
//     skipped, a seed whose set lost a member to a commit of this walk ends
//     the round (it is recomputed by the next phase A), a set of >= thresh
//     members commits.  The walk also ends at the window's end, at the last
//     seed, or at max_clusters.
// Every round advances the walk by at least one seed (the seed at pos is
// exact when phase B starts), so the loop ends.
__global__ void __launch_bounds__(GC_WARPS * 32) k_gc_coop(GcDev g, GcCoop c) {
  extern __shared__ unsigned s_taken[];  // copy of the taken bitset
  __shared__ float4 tm[GC_TILE], ts[GC_TILE];
  __shared__ float4 mem_m[GC_WARPS][GC_MAXS], mem_s[GC_WARPS][GC_MAXS];
  __shared__ int s_pos, s_done, s_ok;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nwords = (g.C + 31) >> 5;
  const int W = gridDim.x * GC_WARPS;
  if (threadIdx.x == 0) {
    s_pos = 0;
    s_done = 0;
  }
  unsigned target = 0;
  for (int round = 0;; ++round) {
    __syncthreads();
    for (int i = threadIdx.x; i < nwords; i += blockDim.x) s_taken[i] = __ldcg(g.taken + i);
    __syncthreads();
    const int pos = s_pos;
    // ---- phase A
    const int a = pos + blockIdx.x * GC_WARPS + wid;
    bool need = false;
    if (a < g.C && !sbit(s_taken, a)) {
      if (!__ldcg(c.computed + a)) {
        need = true;
      } else {
        const int n = min(__ldcg(g.set_size + a), GC_MAXS);
        bool st = false;
        for (int k = lane; k < n; k += 32) st |= sbit(s_taken, __ldcg(g.set_mem + (size_t)a * GC_MAXS + k));
        need = __any_sync(0xffffffffu, st);
      }
    }
    if (__syncthreads_or(need ? 1 : 0)) {
      float4 am = make_float4(0, 0, 0, 0), as = am;
      if (need) {
        am = __ldg(g.pm + a);
        as = __ldg(g.ps + a);
        if (lane == 0) {
          mem_m[wid][0] = am;
          mem_s[wid][0] = as;
        }
      }
      int cnt = 1;  // the seed itself is member 0
      __syncwarp();
      for (int t0 = 0; t0 < g.C; t0 += GC_TILE) {
        __syncthreads();
        for (int i = threadIdx.x; i < GC_TILE; i += blockDim.x) {
          const int b = t0 + i;
          if (b < g.C) {
            tm[i] = __ldg(g.pm + b);
            ts[i] = __ldg(g.ps + b);
          }
        }
        __syncthreads();
        if (!need) continue;
        const int tn = min(GC_TILE, g.C - t0);
        for (int c0 = 0; c0 < tn; c0 += 32) {
          const int b = t0 + c0 + lane;
          bool cand = false;
          if (c0 + lane < tn && b != a && !sbit(s_taken, b))
            cand = gc_consistent(am, as, tm[c0 + lane], ts[c0 + lane], g.gc);
          unsigned bal = __ballot_sync(0xffffffffu, cand);
          while (bal) {  // ascending candidate order
            const int src = __ffs(bal) - 1;
            bal &= bal - 1;
            const float4 cm = tm[c0 + src], cs = ts[c0 + src];
            // consistency with members 1..cnt-1 (member 0, the seed, already checked)
            bool ok = true;
            const int stored = min(cnt, GC_MAXS);
            for (int m0 = 1; m0 < stored; m0 += 32) {
              const int m = m0 + lane;
              const bool bad = m < stored && !gc_consistent(mem_m[wid][m], mem_s[wid][m], cm, cs, g.gc);
              if (__any_sync(0xffffffffu, bad)) {
                ok = false;
                break;
              }
            }
            if (ok) {
              if (cnt >= GC_MAXS) {  // longer than supported: reported by the walk
                ++cnt;
                continue;
              }
              if (lane == 0) {
                mem_m[wid][cnt] = cm;
                mem_s[wid][cnt] = cs;
                g.set_mem[(size_t)a * GC_MAXS + cnt] = t0 + c0 + src;
              }
              ++cnt;
              __syncwarp();
            }
          }
        }
      }
      if (need && lane == 0) {
        g.set_mem[(size_t)a * GC_MAXS] = a;
        g.set_size[a] = cnt;
        c.computed[a] = 1;
      }
    }
    target += gridDim.x;
    if (!gc_barrier(c, target, &s_ok)) return;
    // ---- phase B
    if (blockIdx.x == 0 && wid == 0) {
      int ncl = __ldcg(c.ctl + 1), err = 0;
      bool done = false;
      int p = pos;
      const int wend = min(pos + W, g.C);
      while (p < wend) {
        if (sbit(s_taken, p)) {
          ++p;
          continue;
        }
        const int n = __ldcg(g.set_size + p);
        const int ns = min(n, GC_MAXS);
        int mb[GC_MAXS / 32];
        bool st = false;
#pragma unroll
        for (int q = 0; q < GC_MAXS / 32; ++q) {
          const int k = lane + 32 * q;
          mb[q] = k < ns ? __ldcg(g.set_mem + (size_t)p * GC_MAXS + k) : -1;
          if (mb[q] >= 0 && sbit(s_taken, mb[q])) st = true;
        }
        if (__any_sync(0xffffffffu, st)) break;  // lost a member: recompute from p
        if (n >= c.thresh) {
          if (n > GC_MAXS) {
            err = (int)RTR_ERR_CAPACITY;
            done = true;
            break;
          }
#pragma unroll
          for (int q = 0; q < GC_MAXS / 32; ++q)
            if (mb[q] >= 0) {
              atomicOr(&s_taken[mb[q] >> 5], 1u << (mb[q] & 31));
              c.cl_members[(size_t)ncl * GC_MAXS + lane + 32 * q] = mb[q];
            }
          if (lane == 0) c.cl_sizes[ncl] = n;
          __syncwarp();
          ++ncl;
          if (ncl >= c.max_clusters) {
            done = true;
            ++p;
            break;
          }
        }
        ++p;
      }
      if (p >= g.C) done = true;
      __syncwarp();
      for (int i = lane; i < nwords; i += 32) g.taken[i] = s_taken[i];
      if (lane == 0) {
        c.ctl[0] = p;
        c.ctl[1] = ncl;
        c.ctl[2] = done ? 1 : 0;
        if (err) c.ctl[3] = err;
        c.ctl[4] = round + 1;
      }
      __syncwarp();
    }
    target += gridDim.x;
    if (!gc_barrier(c, target, &s_ok)) return;
    if (threadIdx.x == 0) {
      s_pos = __ldcg(c.ctl + 0);
      s_done = __ldcg(c.ctl + 2) || __ldcg(c.ctl + 3);
    }
    __syncthreads();
    if (s_done) break;
  }
}

// Members as original correspondence indices.
__global__ void k_gc_members_out(const int* __restrict__ mem, const int* __restrict__ sizes,
                                 const uint32_t* __restrict__ order, int ncl, int stride, int max_members,
                                 int* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ncl * max_members; i += gridDim.x * blockDim.x) {
    const int c = i / max_members, k = i - c * max_members;
    out[i] = k < sizes[c] ? (int)order[mem[(size_t)c * stride + k]] : -1;
  }
}

// Gather the sorted correspondence endpoints.
__global__ void k_gc_gather(const float4* __restrict__ mk, const float4* __restrict__ sk, const int* __restrict__ cm,
                            const int* __restrict__ cs, const uint32_t* __restrict__ order, int C,
                            float4* __restrict__ pm, float4* __restrict__ ps) {
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < C; a += gridDim.x * blockDim.x) {
    const int i = (int)order[a];
    pm[a] = mk[cm[i]];
    ps[a] = sk[cs[i]];
  }
}

// Per-cluster least-squares pose model -> scene in FP64 (one warp per cluster).
__global__ void k_gc_poses(const float4* __restrict__ pm, const float4* __restrict__ ps,
                           const int* __restrict__ members, const int* __restrict__ sizes, int ncl,
                           int max_members, double* __restrict__ poses) {
  const int lane = threadIdx.x & 31;
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (c >= ncl) return;
  const int n = min(sizes[c], max_members);
  double s[15];
#pragma unroll
  for (int k = 0; k < 15; ++k) s[k] = 0.0;
  // means first (two-pass, as the oracle)
  for (int k = lane; k < n; k += 32) {
    const int b = members[(size_t)c * max_members + k];
    const float4 p = pm[b], q = ps[b];
    s[0] += p.x; s[1] += p.y; s[2] += p.z; s[3] += q.x; s[4] += q.y; s[5] += q.z;
  }
#pragma unroll
  for (int k = 0; k < 6; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s[k] += __shfl_xor_sync(0xffffffffu, s[k], o);
  const double inv = 1.0 / (double)n;
  const double mp[3] = {s[0] * inv, s[1] * inv, s[2] * inv}, mq[3] = {s[3] * inv, s[4] * inv, s[5] * inv};
  double H[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) H[k] = 0.0;
  for (int k = lane; k < n; k += 32) {
    const int b = members[(size_t)c * max_members + k];
    const float4 p = pm[b], q = ps[b];
    const double dp[3] = {p.x - mp[0], p.y - mp[1], p.z - mp[2]};
    const double dq[3] = {q.x - mq[0], q.y - mq[1], q.z - mq[2]};
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) H[r * 3 + cc] += dp[r] * dq[cc];
  }
#pragma unroll
  for (int k = 0; k < 9; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) H[k] += __shfl_xor_sync(0xffffffffu, H[k], o);
  if (lane == 0) {
    double R[9];
    umeyama_rotation_fast(H, R);
    double* T = poses + (size_t)c * 16;
    for (int r = 0; r < 3; ++r) {
      for (int cc = 0; cc < 3; ++cc) T[r * 4 + cc] = R[r * 3 + cc];
      T[r * 4 + 3] = mq[r] - (R[r * 3] * mp[0] + R[r * 3 + 1] * mp[1] + R[r * 3 + 2] * mp[2]);
    }
    T[12] = T[13] = T[14] = 0.0;
    T[15] = 1.0;
  }
}

// Sort keys: non-negative float bits order like the floats.
__global__ void k_gc_keys(const float* __restrict__ d, int C, uint32_t* __restrict__ keys) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < C; i += gridDim.x * blockDim.x) {
    const float v = d[i];
    keys[i] = v > 0.f ? __float_as_uint(v) : 0u;
  }
}

struct GcBufs {
  uint32_t *k0, *v0, *k1, *v1, *hist;
  float4 *pm, *ps;
  unsigned* taken;
  int *set_size, *set_mem, *computed, *misc;
  unsigned* arrive;
  int *members, *sizes;
  double* poses;
};

static void gc_plan(ScratchPlan& p, int C, int max_clusters, int max_members) {
  const int n = C > 0 ? C : 1;
  for (int i = 0; i < 4; ++i) p.add<uint32_t>(n);
  p.add<uint32_t>(radix_hist_entries(n));
  p.add<float4>(n);
  p.add<float4>(n);
  p.add<unsigned>((n + 31) / 32);
  p.add<int>(n);
  p.add<int>((size_t)n * GC_MAXS);
  p.add<int>(n);
  p.add<int>(16);
  p.add<unsigned>(1);
  p.add<int>((size_t)max_clusters * max_members);
  p.add<int>(max_clusters);
  p.add<double>((size_t)max_clusters * 16);
}

static bool gc_take(Scratch& s, int C, int max_clusters, int max_members, GcBufs* b) {
  const int n = C > 0 ? C : 1;
  b->k0 = s.take<uint32_t>(n);
  b->v0 = s.take<uint32_t>(n);
  b->k1 = s.take<uint32_t>(n);
  b->v1 = s.take<uint32_t>(n);
  b->hist = s.take<uint32_t>(radix_hist_entries(n));
  b->pm = s.take<float4>(n);
  b->ps = s.take<float4>(n);
  b->taken = s.take<unsigned>((n + 31) / 32);
  b->set_size = s.take<int>(n);
  b->set_mem = s.take<int>((size_t)n * GC_MAXS);
  b->computed = s.take<int>(n);
  b->misc = s.take<int>(16);
  b->arrive = s.take<unsigned>(1);
  b->members = s.take<int>((size_t)max_clusters * max_members);
  b->sizes = s.take<int>(max_clusters);
  b->poses = s.take<double>((size_t)max_clusters * 16);
  return b->poses != nullptr;
}

// Shared memory of k_gc_coop beyond its static part: the taken bitset.
constexpr size_t GC_MAX_DYN_SMEM = 180 * 1024;

}  // namespace rtr

using namespace rtr;

namespace rtr {

size_t gc_scratch_bytes(int C, int max_clusters) {
  ScratchPlan plan;
  gc_plan(plan, C, max_clusters, GC_MAXS);
  return plan.bytes;
}

rtr_status gc_group_dev(rtr_context* ctx, Scratch& s, const float* d_model_kp, const float* d_scene_kp,
                        const int32_t* d_corr_m, const int32_t* d_corr_s, const float* d_corr_d, int n_corr,
                        float gc_size, int gc_thresh, int max_clusters, int max_members, int32_t* d_members,
                        int32_t* d_sizes, double* d_poses, int* h_n_clusters, cudaStream_t st) {
  *h_n_clusters = 0;
  if (n_corr == 0) return RTR_OK;
  const int C = n_corr;
  GcBufs b;
  if (!gc_take(s, C, max_clusters, GC_MAXS, &b)) return fail(RTR_ERR_CAPACITY, "rtr_gc_group: scratch");
  const int nb = (C + 255) / 256 > 152 * 8 ? 152 * 8 : (C + 255) / 256;
  k_gc_keys<<<nb, 256, 0, st>>>(d_corr_d, C, b.k0);
  uint32_t *ks, *vs;
  radix_sort_pairs(b.k0, b.v0, b.k1, b.v1, b.hist, C, C, nullptr, 32, true, st, &ks, &vs);
  k_gc_gather<<<nb, 256, 0, st>>>(reinterpret_cast<const float4*>(d_model_kp),
                                  reinterpret_cast<const float4*>(d_scene_kp), d_corr_m, d_corr_s, vs, C, b.pm, b.ps);
  const size_t dyn = sizeof(unsigned) * (size_t)((C + 31) / 32);
  if (dyn > GC_MAX_DYN_SMEM)
    return fail(RTR_ERR_CAPACITY, "rtr_gc_group: %d correspondences exceed the supported %d", C,
                (int)(GC_MAX_DYN_SMEM * 8));
  RTR_CUDA(cudaMemsetAsync(b.taken, 0, dyn, st));
  RTR_CUDA(cudaMemsetAsync(b.computed, 0, sizeof(int) * C, st));
  RTR_CUDA(cudaMemsetAsync(b.misc, 0, sizeof(int) * 16, st));
  RTR_CUDA(cudaMemsetAsync(b.arrive, 0, sizeof(unsigned), st));
  GcDev g{b.pm, b.ps, C, gc_size, b.taken, b.set_size, b.set_mem};
  GcCoop c{b.misc, b.arrive, b.computed, b.members, b.sizes, gc_thresh, max_clusters,
           ctx->wait_budget_cycles, ctx->d_status};
  RTR_CUDA(cudaFuncSetAttribute(k_gc_coop, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  int per_sm = 0;
  RTR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gc_coop, GC_WARPS * 32, dyn));
  if (per_sm < 1) return fail(RTR_ERR_CAPACITY, "rtr_gc_group: grouping kernel does not fit an SM");
  const int blocks = (per_sm < 2 ? per_sm : 2) * ctx->num_sms;
  {
    ProfScope pw(ctx, st, "gc_walk");
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(blocks);
    cfg.blockDim = dim3(GC_WARPS * 32);
    cfg.dynamicSmemBytes = dyn;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    RTR_CUDA(cudaLaunchKernelEx(&cfg, k_gc_coop, g, c));
  }
  RTR_LAUNCHED(3);
  int* h = ctx->h_pin;
  RTR_CUDA(cudaMemcpyAsync(h, b.misc, 5 * sizeof(int), cudaMemcpyDeviceToHost, st));
  RTR_CUDA(cudaStreamSynchronize(st));
  const int ncl = h[1];
  if (h[3] == (int)RTR_ERR_CAPACITY)
    return fail(RTR_ERR_CAPACITY, "rtr_gc_group: a consensus set exceeds %d members", GC_MAXS);
  if (h[3] == (int)RTR_ERR_TIMEOUT)
    return fail(RTR_ERR_TIMEOUT, "rtr_gc_group: a grid barrier wait exceeded the budget");
  ctx->gc_rounds = h[4];
  if (ncl > 0) {
    k_gc_poses<<<(ncl + 3) / 4, 128, 0, st>>>(b.pm, b.ps, b.members, b.sizes, ncl, GC_MAXS, b.poses);
    RTR_LAUNCHED(1);
    if (d_poses) RTR_CUDA(cudaMemcpyAsync(d_poses, b.poses, sizeof(double) * 16 * ncl, cudaMemcpyDeviceToDevice, st));
    if (d_sizes) RTR_CUDA(cudaMemcpyAsync(d_sizes, b.sizes, sizeof(int) * ncl, cudaMemcpyDeviceToDevice, st));
    if (d_members) {
      k_gc_members_out<<<(ncl * max_members + 255) / 256, 256, 0, st>>>(b.members, b.sizes, vs, ncl, GC_MAXS,
                                                                         max_members, d_members);
      RTR_LAUNCHED(1);
    }
  }
  *h_n_clusters = ncl;
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

}  // namespace rtr

extern "C" rtr_status rtr_gc_group(rtr_context* ctx, const float* d_model_kp, const float* d_scene_kp,
                                   const int32_t* d_corr_m, const int32_t* d_corr_s, const float* d_corr_d,
                                   int n_corr, float gc_size, int gc_thresh, int max_clusters,
                                   int max_members, int32_t* d_members, int32_t* d_sizes, double* d_poses,
                                   int* h_n_clusters, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n_corr >= 0 && gc_size >= 0.f && gc_thresh >= 1 && max_clusters >= 1 && h_n_clusters,
                "rtr_gc_group: bad arguments");
  RTR_CHECK_ARG(max_members >= 1, "rtr_gc_group: max_members must be >= 1");
  *h_n_clusters = 0;
  if (n_corr == 0) return RTR_OK;
  RTR_CHECK_ARG(d_model_kp && d_scene_kp && d_corr_m && d_corr_s && d_corr_d, "rtr_gc_group: NULL input");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, gc_scratch_bytes(n_corr, max_clusters), st, &s));
  ProfScope ps(ctx, st, "gc_group");
  return gc_group_dev(ctx, s, d_model_kp, d_scene_kp, d_corr_m, d_corr_s, d_corr_d, n_corr, gc_size, gc_thresh,
                      max_clusters, max_members, d_members, d_sizes, d_poses, h_n_clusters, st);
}
