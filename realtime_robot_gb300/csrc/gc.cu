// gc.cu — geometric-consistency grouping (Chen & Bhanu 2007; PCL
// GeometricConsistencyGrouping), the spec stand-in for the reference's
// pair-consensus loop (Ransac, function.h:35-109).
//
// Semantics (shared with the oracle): correspondences sorted by descriptor
// distance (ties: input order); each not-yet-taken correspondence, in that
// order, seeds a consensus set that admits, in the same order, every
// not-taken correspondence whose model-side and scene-side distances to EVERY
// member differ by at most gc_size; a set of >= gc_thresh members becomes a
// cluster and its members are taken.
//
// GPU form.  The sequential loop is O(C^2); its parallel part is computing
// every seed's set.  Pass 1 computes all sets speculatively (no correspondence
// taken), warp per seed, candidates streamed through shared memory in tiles.
// The commit loop then walks seeds in order: a seed whose stored set does not
// intersect anything taken since it was computed is exact (removing rejected
// candidates never changes a greedy walk); the first exact seed with a large
// set commits; seeds whose set intersects the commit are marked stale and are
// recomputed, in parallel, when the walk reaches them.
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
  const unsigned* taken;   // bitset over sorted positions
  int* set_size;           // [C]
  int* set_mem;            // [C][GC_MAXS] sorted positions
  int* stale;              // [C]
};

__device__ __forceinline__ bool gc_consistent(float4 am, float4 as, float4 bm, float4 bs, float gc) {
  const float dm = __fsqrt_rn(dist2_exact(am, bm));
  const float ds = __fsqrt_rn(dist2_exact(as, bs));
  return !(fabsf(__fsub_rn(dm, ds)) > gc);
}

__device__ __forceinline__ bool bit(const unsigned* b, int i) { return (b[i >> 5] >> (i & 31)) & 1u; }

// Pass over seeds listed in `seeds` (or all seeds 0..C-1 when seeds == NULL).
__global__ void __launch_bounds__(GC_WARPS * 32) k_gc_sets(GcDev g, const int* __restrict__ seeds,
                                                           const int* __restrict__ n_seeds) {
  __shared__ float4 tm[GC_TILE], ts[GC_TILE];
  __shared__ float4 mem_m[GC_WARPS][GC_MAXS], mem_s[GC_WARPS][GC_MAXS];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int ns = seeds ? *n_seeds : g.C;
  for (int base = blockIdx.x * GC_WARPS; base < ns; base += gridDim.x * GC_WARPS) {
    const int si = base + wid;
    const int a = si < ns ? (seeds ? seeds[si] : si) : -1;
    const bool active = a >= 0 && !bit(g.taken, a);
    float4 am = make_float4(0, 0, 0, 0), as = am;
    if (a >= 0) {
      am = g.pm[a];
      as = g.ps[a];
    }
    int cnt = 1;  // the seed itself is member 0
    if (lane == 0) {
      mem_m[wid][0] = am;
      mem_s[wid][0] = as;
    }
    __syncwarp();
    for (int t0 = 0; t0 < g.C; t0 += GC_TILE) {
      __syncthreads();
      for (int i = threadIdx.x; i < GC_TILE; i += blockDim.x) {
        const int b = t0 + i;
        if (b < g.C) {
          tm[i] = g.pm[b];
          ts[i] = g.ps[b];
        }
      }
      __syncthreads();
      if (!active) continue;
      const int tn = min(GC_TILE, g.C - t0);
      for (int c0 = 0; c0 < tn; c0 += 32) {
        const int b = t0 + c0 + lane;
        bool cand = false;
        if (c0 + lane < tn && b != a && !bit(g.taken, b))
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
            if (cnt >= GC_MAXS) {  // set longer than supported: reported by the caller
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
    if (a >= 0 && lane == 0) {
      if (active) g.set_mem[(size_t)a * GC_MAXS] = a;
      g.set_size[a] = active ? cnt : 0;
      g.stale[a] = 0;
    }
  }
}

// First seed >= pos that is not taken and either stale or large.
__global__ void k_gc_find(GcDev g, int pos, int thresh, int* out) {
  int best = 0x7fffffff;
  for (int a = pos + blockIdx.x * blockDim.x + threadIdx.x; a < g.C; a += gridDim.x * blockDim.x) {
    if (bit(g.taken, a)) continue;
    if (g.stale[a] == 1 || g.set_size[a] >= thresh) {
      best = a;
      break;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0 && best != 0x7fffffff) atomicMin(out, best);
}

// Copy the found seed's state next to it for one host read.
__global__ void k_gc_peek(GcDev g, int* misc) {
  const int a = misc[0];
  misc[1] = a < g.C ? g.stale[a] : 0;
  misc[2] = a < g.C ? g.set_size[a] : 0;
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

// Commit seed a: take its members (recomputed exactly when the set was too
// long to store: then the walk is redone here by one warp).
__global__ void k_gc_commit(GcDev g, int a, unsigned* taken, int* newly, int* cluster_members,
                            int* cluster_size, int cid, int max_members) {
  const int n = g.set_size[a];
  const int stored = min(n, GC_MAXS);
  for (int k = threadIdx.x; k < stored; k += blockDim.x) {
    const int b = g.set_mem[(size_t)a * GC_MAXS + k];
    atomicOr(&taken[b >> 5], 1u << (b & 31));
    newly[b] = 1;
    if (k < max_members) cluster_members[(size_t)cid * max_members + k] = b;
  }
  if (threadIdx.x == 0) cluster_size[cid] = stored;
}

// Seeds after `a` whose stored set touches the commit become stale.
__global__ void k_gc_invalidate(GcDev g, int a, const int* __restrict__ newly) {
  for (int s = a + 1 + blockIdx.x * blockDim.x + threadIdx.x; s < g.C; s += gridDim.x * blockDim.x) {
    if (bit(g.taken, s) || g.stale[s]) continue;
    const int n = min(g.set_size[s], GC_MAXS);
    for (int k = 0; k < n; ++k)
      if (newly[g.set_mem[(size_t)s * GC_MAXS + k]]) {
        g.stale[s] = 1;
        break;
      }
  }
}

__global__ void k_gc_clear_newly(int* newly, const int* __restrict__ cluster_members, const int* cluster_size,
                                 int cid, int max_members) {
  const int n = cluster_size[cid];
  for (int k = threadIdx.x; k < n && k < max_members; k += blockDim.x) newly[cluster_members[(size_t)cid * max_members + k]] = 0;
}

// Stale seeds in [pos, C) -> compact list (ascending).
__global__ void k_gc_stale_list(GcDev g, int pos, int* list, int* n) {
  for (int a = pos + blockIdx.x * blockDim.x + threadIdx.x; a < g.C; a += gridDim.x * blockDim.x)
    if (g.stale[a] && !bit(g.taken, a)) list[atomicAdd(n, 1)] = a;
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
  int *set_size, *set_mem, *stale, *newly, *list, *misc;
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
  p.add<int>(n);
  p.add<int>(n);
  p.add<int>(16);
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
  b->stale = s.take<int>(n);
  b->newly = s.take<int>(n);
  b->list = s.take<int>(n);
  b->misc = s.take<int>(16);
  b->members = s.take<int>((size_t)max_clusters * max_members);
  b->sizes = s.take<int>(max_clusters);
  b->poses = s.take<double>((size_t)max_clusters * 16);
  return b->poses != nullptr;
}

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
  ProfScope ps(ctx, st, "gc_group");
  const int nb = (C + 255) / 256 > 152 * 8 ? 152 * 8 : (C + 255) / 256;
  k_gc_keys<<<nb, 256, 0, st>>>(d_corr_d, C, b.k0);
  uint32_t *ks, *vs;
  radix_sort_pairs(b.k0, b.v0, b.k1, b.v1, b.hist, C, C, nullptr, 32, true, st, &ks, &vs);
  k_gc_gather<<<nb, 256, 0, st>>>(reinterpret_cast<const float4*>(d_model_kp),
                                  reinterpret_cast<const float4*>(d_scene_kp), d_corr_m, d_corr_s, vs, C, b.pm, b.ps);
  RTR_CUDA(cudaMemsetAsync(b.taken, 0, sizeof(unsigned) * ((C + 31) / 32), st));
  RTR_CUDA(cudaMemsetAsync(b.stale, 0, sizeof(int) * C, st));
  RTR_CUDA(cudaMemsetAsync(b.newly, 0, sizeof(int) * C, st));
  GcDev g{b.pm, b.ps, C, gc_size, b.taken, b.set_size, b.set_mem, b.stale};
  int sb = (C + GC_WARPS - 1) / GC_WARPS;
  if (sb > 152 * 4) sb = 152 * 4;
  k_gc_sets<<<sb, GC_WARPS * 32, 0, st>>>(g, nullptr, nullptr);
  RTR_LAUNCHED(5);
  int pos = 0, ncl = 0;
  int* h = ctx->h_pin;
  for (int guard = 0; guard < 4 * C + 16 && ncl < max_clusters; ++guard) {
    RTR_CUDA(cudaMemsetAsync(b.misc, 0x7f, sizeof(int), st));
    k_gc_find<<<nb, 256, 0, st>>>(g, pos, gc_thresh, b.misc);
    k_gc_peek<<<1, 1, 0, st>>>(g, b.misc);
    RTR_LAUNCHED(2);
    RTR_CUDA(cudaMemcpyAsync(h, b.misc, 3 * sizeof(int), cudaMemcpyDeviceToHost, st));
    RTR_CUDA(cudaStreamSynchronize(st));
    const int a = h[0];
    if (a >= C || a < 0) break;
    if (h[2] > GC_MAXS)
      return fail(RTR_ERR_CAPACITY, "rtr_gc_group: a consensus set exceeds %d members", GC_MAXS);
    if (h[1] == 1) {
      // recompute every stale seed from a on, under the current taken state
      RTR_CUDA(cudaMemsetAsync(b.misc + 4, 0, sizeof(int), st));
      k_gc_stale_list<<<nb, 256, 0, st>>>(g, a, b.list, b.misc + 4);
      k_gc_sets<<<sb, GC_WARPS * 32, 0, st>>>(g, b.list, b.misc + 4);
      RTR_LAUNCHED(2);
      pos = a;
      continue;
    }
    // exact seed with a large set: commit
    k_gc_commit<<<1, 128, 0, st>>>(g, a, b.taken, b.newly, b.members, b.sizes, ncl, GC_MAXS);
    k_gc_invalidate<<<nb, 256, 0, st>>>(g, a, b.newly);
    k_gc_clear_newly<<<1, 128, 0, st>>>(b.newly, b.members, b.sizes, ncl, GC_MAXS);
    RTR_LAUNCHED(3);
    ++ncl;
    pos = a + 1;
  }
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
  return gc_group_dev(ctx, s, d_model_kp, d_scene_kp, d_corr_m, d_corr_s, d_corr_d, n_corr, gc_size, gc_thresh,
                      max_clusters, max_members, d_members, d_sizes, d_poses, h_n_clusters, st);
}
