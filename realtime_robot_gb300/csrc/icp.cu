// icp.cu — persistent point-to-point ICP (replaces the PCL
// IterativeClosestPoint used by keyPointICP, function.h:111-148).
//
// One cooperative launch runs every iteration.  Per iteration each thread
// transforms its source points with the FP32 pose, finds the exact 1-NN in the
// target grid within max_corr_dist (rejection), and accumulates the centred
// sums (dp, dq, dp dq^T, d^2) in FP32 Kahan–Babuška accumulators; warps and
// the block combine them with TwoSum-compensated shuffles into one (hi, lo)
// pair per value per block.  The last block to arrive reduces the block pairs
// in FP64 (fixed order), solves the pose in FP64 (pose.cuh) and releases the
// others through a generation word.  Every wait is bounded by a clock64
// budget; a block that runs out writes RTR_ERR_TIMEOUT and leaves.
#include <math.h>
#include <atomic>
#include <string.h>

#include "grid.cuh"
#include "icp.cuh"
#include "pose.cuh"
#include "search.cuh"

namespace rtr {

constexpr int ICP_THREADS = 256;
constexpr int ICP_WARPS = ICP_THREADS / 32;
constexpr int ICP_NV = 16;  // dp(3) dq(3) dp*dq^T(9) d^2(1)


__device__ __forceinline__ unsigned long long icp_timer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ float centre_of(const GridMeta* m, int a) {
  return 0.5f * (ordered_to_float(m->bmin[a]) + ordered_to_float(m->bmax[a]));
}

// One launch serves many problems: block b works on problem blk2prob[b]
// together with that problem's other nblk - 1 blocks; problems never wait on
// one another.
template <int G>  // lanes cooperating on one source point's 1-NN search
__global__ void __launch_bounds__(ICP_THREADS) k_icp(const IcpDev* __restrict__ probs,
                                                     const int* __restrict__ blk2prob) {
  const IcpDev& a = probs[blk2prob[blockIdx.x]];
  const int lb = (int)blockIdx.x - a.blk0;
  __shared__ float s_red[ICP_WARPS][ICP_NV][2];
  __shared__ int s_cnt[ICP_WARPS];
  __shared__ double s_sum[ICP_NV];
  __shared__ double s_P[16], s_D[16], s_H[9];
  __shared__ long long s_n;
  __shared__ int s_last, s_stop;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (a.d_active && a.slot >= *a.d_active) {  // a capacity slot left unused: every block of it leaves
    if (lb == 0 && tid == 0) {
      a.result->iterations = 0;
      a.result->converged = 0;
      a.result->n_corr = 0;
      a.result->fitness = 0.0;
      a.result->status = RTR_OK;
    }
    return;
  }
  const int B = a.nblk;
  const GridView g = load_view(a.grid);
  const bool near27 = grid_near27_ok(g, a.r2max);  // every match within the 27 cells around a query
  // Centring: target terms about the target box centre c, source terms about
  // the source box centre moved by the current pose (cp), so the FP32 products
  // stay small even while the clouds are far apart.
  const float c[3] = {centre_of(a.grid.meta, 0), centre_of(a.grid.meta, 1), centre_of(a.grid.meta, 2)};
  const float4 cs = make_float4(centre_of(a.src_meta, 0), centre_of(a.src_meta, 1), centre_of(a.src_meta, 2), 0.f);
  constexpr int QPB = ICP_THREADS / G;  // source points per block per pass
  constexpr int NVL = ICP_NV / G;        // sums kept per lane
  const unsigned stride = (unsigned)B * QPB;
  const int lg = lane & (G - 1);
  const unsigned gmask = ((1u << G) - 1u) << (lane & ~(G - 1));

  const bool prof0 = a.prof != nullptr && lb == 0 && tid == 0;
  unsigned long long t_it = 0, t_arr = 0;
  for (int it = 0; it < a.max_it; ++it) {
    if (prof0) t_it = icp_timer();
    float T[12];
    if (it == 0) {
#pragma unroll
      for (int k = 0; k < 12; ++k) T[k] = __double2float_rn(a.init[k]);
    } else {
#pragma unroll
      for (int k = 0; k < 12; ++k) T[k] = __ldcg(a.posef + k);
    }
    const float4 cp = xform_exact(T, cs);
    // The G lanes of a group share the 16 sums of their points: lane lg keeps
    // values lg*NVL .. lg*NVL+NVL-1 (dp 0-2, dq 3-5, dp dq^T 6-14, d^2 15),
    // each over the group's points in order, as one lane holding all 16 would.
    KSum acc[NVL];
#pragma unroll
    for (int k = 0; k < NVL; ++k) acc[k].init();
    int cnt = 0;
    for (unsigned i = (unsigned)lb * QPB + tid / G; i < (unsigned)a.n_src; i += stride) {
      const float4 p = xform_exact(T, a.src[i]);
      float d2;
      int j, pos;
      if (near27)  // the group agrees on (d2, j, pos)
        grid_nn1_near<G>(g, p, a.r2max, lg, gmask, d2, j, pos);
      else
        grid_nn1_group<G, true>(g, p, a.r2max, lg, gmask, d2, j, pos);
      if (j >= 0) {
        const float4 q = g.pts[pos];
        const float dp[3] = {__fsub_rn(p.x, cp.x), __fsub_rn(p.y, cp.y), __fsub_rn(p.z, cp.z)};
        const float dq[3] = {__fsub_rn(q.x, c[0]), __fsub_rn(q.y, c[1]), __fsub_rn(q.z, c[2])};
#pragma unroll
        for (int k = 0; k < NVL; ++k) {
          const int v = lg * NVL + k;
          float x;
          if (v < 3)
            x = v == 0 ? dp[0] : (v == 1 ? dp[1] : dp[2]);
          else if (v < 6)
            x = v == 3 ? dq[0] : (v == 4 ? dq[1] : dq[2]);
          else if (v < 15) {
            const int r = (v - 6) / 3, kk = (v - 6) % 3;
            x = __fmul_rn(r == 0 ? dp[0] : (r == 1 ? dp[1] : dp[2]), kk == 0 ? dq[0] : (kk == 1 ? dq[1] : dq[2]));
          } else
            x = d2;
          acc[k].add(x);
        }
        ++cnt;
      }
      if (a.trace_corr && lg == 0)
        a.trace_corr[(size_t)it * (size_t)a.n_src + (size_t)(a.src_idx ? a.src_idx[i] : (int)i)] = j;
    }
    // block partial: compensated sums over the warp's groups (offsets >= G,
    // the same tree a single lane per group would meet), then across warps
#pragma unroll
    for (int k = 0; k < NVL; ++k) {
      float s = acc[k].s, cc = acc[k].c;
#pragma unroll
      for (int off = 16; off >= G; off >>= 1) {
        const float s2 = __shfl_down_sync(0xffffffffu, s, off);
        const float c2 = __shfl_down_sync(0xffffffffu, cc, off);
        float t, e;
        two_sum(s, s2, t, e);
        s = t;
        cc = __fadd_rn(__fadd_rn(cc, c2), e);
      }
      if (lane < G) {
        s_red[warp][lane * NVL + k][0] = s;
        s_red[warp][lane * NVL + k][1] = cc;
      }
    }
    cnt = lg == 0 ? cnt : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if (lane == 0) s_cnt[warp] = cnt;
    __syncthreads();
    if (tid < ICP_NV) {
      float s = s_red[0][tid][0], cc = s_red[0][tid][1];
      for (int w = 1; w < ICP_WARPS; ++w) {
        float t, e;
        two_sum(s, s_red[w][tid][0], t, e);
        s = t;
        cc = __fadd_rn(__fadd_rn(cc, s_red[w][tid][1]), e);
      }
      a.partial[lb * 32 + tid] = s;
      a.partial[lb * 32 + 16 + tid] = cc;
    }
    if (tid == 0) {
      int tot = 0;
      for (int w = 0; w < ICP_WARPS; ++w) tot += s_cnt[w];
      a.pcount[lb] = tot;
    }
    __syncthreads();
    if (tid == 0) {
      if (prof0) {
        t_arr = icp_timer();
        atomicAdd(a.prof + 0, t_arr - t_it);
      }
      __threadfence();
      const unsigned t = atomicAdd(a.arrive, 1u);
      s_last = (t == (unsigned)(it + 1) * (unsigned)B - 1u) ? 1 : 0;
    }
    __syncthreads();
    if (s_last) {
      const unsigned long long t_s0 = a.prof && tid == 0 ? icp_timer() : 0ull;
      __threadfence();
      // current pose (FP64) fetched early, used after the solve
      if (tid < 16) {
        const double pk = it == 0 ? a.init[tid] : __ldcg(a.pose64 + tid);
        s_P[tid] = pk;
        if (it == 0 && a.trace_pose) a.trace_pose[tid] = pk;
      }
      // Cross-block reduction.  GB300 issues one FP64 warp-instruction per ~16
      // SM cycles, so the tree runs on compensated FP32 pairs (TwoSum, ~48-bit
      // significand) and FP64 closes it: one (double)hi + (double)lo per value.
      // Warp w reduces values 2w and 2w + 1 (lanes stride over the blocks in
      // a fixed order), so no thread holds all sixteen pairs.
      static_assert(ICP_WARPS * 2 == ICP_NV, "two values per warp");
      {
        float hs0 = 0.f, ls0 = 0.f, hs1 = 0.f, ls1 = 0.f;
        int nloc = 0;
        const int v0 = 2 * warp;
        for (int b = lane; b < B; b += 32) {
          const float2 h = __ldcg(reinterpret_cast<const float2*>(a.partial + b * 32 + v0));
          const float2 l = __ldcg(reinterpret_cast<const float2*>(a.partial + b * 32 + 16 + v0));
          if (warp == 0) nloc += __ldcg(a.pcount + b);
          float t, e;
          two_sum(hs0, h.x, t, e);
          hs0 = t;
          ls0 = __fadd_rn(__fadd_rn(ls0, l.x), e);
          two_sum(hs1, h.y, t, e);
          hs1 = t;
          ls1 = __fadd_rn(__fadd_rn(ls1, l.y), e);
        }
        warp_ksum(hs0, ls0);
        warp_ksum(hs1, ls1);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nloc += __shfl_down_sync(0xffffffffu, nloc, o);
        if (lane == 0) {
          s_sum[v0] = (double)hs0 + (double)ls0;
          s_sum[v0 + 1] = (double)hs1 + (double)ls1;
          if (warp == 0) s_n = nloc;
        }
      }
      __syncthreads();
      if (a.prof && tid == 0) atomicAdd(a.prof + 4, icp_timer() - t_s0);
      // centred cross-covariance, one element per lane
      if (tid < 9 && s_n >= 3) {
        const double inv = 1.0 / (double)s_n;
        const int r = tid / 3, k = tid % 3;
        s_H[tid] = s_sum[6 + tid] - (double)s_n * (s_sum[r] * inv) * (s_sum[3 + k] * inv);
      }
      __syncthreads();
      if (warp == 0) {  // the pose solve: warp 0, FP64 products spread over its lanes
        const long long n = s_n;
        int stop = 0, converged = 1;
        double fitness = 0.0;
        double D[12] = {1.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 1.0, 0.0};
        if (n < 3) {
          stop = 1;
          converged = 0;
        } else {
          const double inv = 1.0 / (double)n;
          double mdp[3], mdq[3], H[9], R[9];
          for (int k = 0; k < 3; ++k) {
            mdp[k] = s_sum[k] * inv;
            mdq[k] = s_sum[3 + k] * inv;
          }
#pragma unroll
          for (int k = 0; k < 9; ++k) H[k] = s_H[k];
          umeyama_rotation_warp(H, R);
          double mp[3], mq[3], t[3];
          for (int k = 0; k < 3; ++k) {
            mp[k] = mdp[k] + (double)(k == 0 ? cp.x : (k == 1 ? cp.y : cp.z));
            mq[k] = mdq[k] + (double)c[k];
          }
          for (int r = 0; r < 3; ++r) t[r] = mq[r] - (R[r * 3 + 0] * mp[0] + R[r * 3 + 1] * mp[1] + R[r * 3 + 2] * mp[2]);
#pragma unroll
          for (int r = 0; r < 3; ++r) {
#pragma unroll
            for (int k = 0; k < 3; ++k) D[r * 4 + k] = R[r * 3 + k];
            D[r * 4 + 3] = t[r];
          }
          fitness = s_sum[15] * inv;
          const double cosang = 0.5 * (R[0] + R[4] + R[8] - 1.0);
          const double tsq = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
          if (a.eps_t > 0.0 && tsq < a.eps_t && (a.eps_r <= 0.0 || cosang > a.eps_r)) stop = 1;
        }
        if (it + 1 >= a.max_it) stop = 1;
        if (lane == 0) {
#pragma unroll
          for (int k = 0; k < 16; ++k) s_D[k] = k < 12 ? D[k] : (k == 15 ? 1.0 : 0.0);
          a.result->fitness = fitness;
          a.result->iterations = it + 1;
          a.result->converged = converged;
          a.result->n_corr = (int)n;
          a.result->status = RTR_OK;
          s_stop = stop;
          if (a.prof) atomicAdd(a.prof + 5, icp_timer() - t_s0);
        }
      }
      __syncthreads();
      // pose <- dT * pose, one element per thread
      if (tid < 16) {
        const int r = tid >> 2, cidx = tid & 3;
        const double pk = s_D[r * 4 + 0] * s_P[0 * 4 + cidx] + s_D[r * 4 + 1] * s_P[1 * 4 + cidx] +
                          s_D[r * 4 + 2] * s_P[2 * 4 + cidx] + s_D[r * 4 + 3] * s_P[3 * 4 + cidx];
        a.pose64[tid] = pk;
        if (tid < 12) a.posef[tid] = __double2float_rn(pk);
        if (a.trace_pose) a.trace_pose[(size_t)(it + 1) * 16 + tid] = pk;
        a.result->pose[tid] = pk;
      }
      __syncthreads();
      if (tid == 0) {
        __threadfence();
        st_release_gpu(a.gen, (unsigned)(it + 1) | (s_stop ? 0x80000000u : 0u));
        if (a.prof) {
          atomicAdd(a.prof + 1, icp_timer() - t_s0);
          atomicAdd(a.prof + 3, 1ull);
        }
      }
      __syncthreads();
    } else {
      if (tid == 0) {
        const long long t0 = clock64();
        unsigned gv;
        for (;;) {
          gv = ld_acquire_gpu(a.gen);
          if ((gv & 0x7fffffffu) >= (unsigned)(it + 1)) break;
          if (clock64() - t0 > a.budget) {
            atomicExch(a.status, (int)RTR_ERR_TIMEOUT);
            a.result->status = RTR_ERR_TIMEOUT;
            a.result->converged = 0;
            gv = 0x80000000u;
            break;
          }
          __nanosleep(64);
        }
        s_stop = (gv >> 31) ? 1 : 0;
        if (prof0) atomicAdd(a.prof + 2, icp_timer() - t_arr);
      }
      __syncthreads();
    }
    if (s_stop) break;
  }
}

// Sort keys of the source under the initial pose, in the target grid.
__global__ void __launch_bounds__(256) k_src_keys(const float4* __restrict__ src, int n,
                                                  IcpDev a, uint32_t* __restrict__ keys) {
  const GridMeta* m = a.grid.meta;
  float T[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) T[k] = __double2float_rn(a.init[k]);
  const float ox = m->ox, oy = m->oy, oz = m->oz, ih = m->inv_h;
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float4 p = xform_exact(T, src[i]);
    int cx = min(max(q_cell(p.x, ox, ih), 0), nx - 1);
    int cy = min(max(q_cell(p.y, oy, ih), 0), ny - 1);
    int cz = min(max(q_cell(p.z, oz, ih), 0), nz - 1);
    keys[i] = ((uint32_t)cz * (uint32_t)ny + (uint32_t)cy) * (uint32_t)nx + (uint32_t)cx;
  }
}

__global__ void __launch_bounds__(256) k_gather_pts(const float4* __restrict__ pts,
                                                    const uint32_t* __restrict__ order, int n,
                                                    float4* __restrict__ out, int* __restrict__ idx) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint32_t o = order[i];
    out[i] = pts[o];
    idx[i] = (int)o;
  }
}

// Co-resident blocks of the ICP kernel (the smallest over the group sizes,
// so a plan made for one group size fits every variant).
int icp_max_blocks(rtr_context* ctx) {
  static std::atomic<int> cached[64];  // per device; 0 = not yet known
  const int dev = ctx->device;
  if (dev >= 0 && dev < 64) {
    const int v = cached[dev].load(std::memory_order_relaxed);
    if (v > 0) return v;
  }
  int a = 0, b = 0, c = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_icp<2>, ICP_THREADS, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_icp<4>, ICP_THREADS, 0);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&c, k_icp<8>, ICP_THREADS, 0);
  int per_sm = a < b ? a : b;
  per_sm = per_sm < c ? per_sm : c;
  const int v = per_sm * ctx->num_sms;
  if (dev >= 0 && dev < 64) cached[dev].store(v, std::memory_order_relaxed);
  return v;
}

// Lanes per source point: the tuning override when set, else the most lanes
// (8, 4, 2) with which the launch needs at most four passes over its points
// (measured on GB300: a 20k-point ICP on the ring search is fastest at 8, two
// passes; sixteen 9.2k-point refinements on the 27-cell search at 2, 3.8
// passes: 1.40 ms against 1.48 at 4 and 1.75 at 8).
int icp_pick_group(const rtr_context* ctx, long long total_pts, int blocks) {
  const int t = ctx->tune_icp_group;
  if (t == 2 || t == 4 || t == 8) return t;
  const long long lanes = (long long)blocks * ICP_THREADS;
  if (total_pts * 8 <= 4 * lanes) return 8;
  return total_pts * 4 <= 4 * lanes ? 4 : 2;
}

static rtr_status launch_icp(int G, const IcpDev* d_probs, const int* d_blk2prob, int blocks, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(ICP_THREADS);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (G == 2)
    RTR_CUDA(cudaLaunchKernelEx(&cfg, k_icp<2>, d_probs, d_blk2prob));
  else if (G == 4)
    RTR_CUDA(cudaLaunchKernelEx(&cfg, k_icp<4>, d_probs, d_blk2prob));
  else
    RTR_CUDA(cudaLaunchKernelEx(&cfg, k_icp<8>, d_probs, d_blk2prob));
  RTR_LAUNCHED(1);
  return RTR_OK;
}

// Problem descriptors reach device memory through kernel parameters (so a
// stream capture records them by value).  init_dev (optional) overrides the
// parameter's initial pose with a pose already on the device.
constexpr int ICP_SETUP_BATCH = 16;
struct IcpSetup {
  IcpDev p[ICP_SETUP_BATCH];
  const double* init_dev[ICP_SETUP_BATCH];
  int n, first;
};

__global__ void k_icp_setup(IcpSetup s, IcpDev* __restrict__ probs, int* __restrict__ blk2prob) {
  const int k = blockIdx.x;
  if (k >= s.n) return;
  const int pid = s.first + k;
  const IcpDev& a = s.p[k];
  for (int b = threadIdx.x; b < a.nblk; b += blockDim.x) blk2prob[a.blk0 + b] = pid;
  if (threadIdx.x == 0) {
    IcpDev d = a;
    if (s.init_dev[k])
      for (int i = 0; i < 16; ++i) d.init[i] = s.init_dev[k][i];
    probs[pid] = d;
    d.arrive[0] = 0u;
    d.gen[0] = 0u;
  }
}

void icp_multi_plan(ScratchPlan& p, int n_probs, int max_blocks) {
  p.add<IcpDev>(n_probs);
  p.add<int>(max_blocks);
  p.add<double>((size_t)n_probs * 16);
  p.add<float>((size_t)n_probs * 16);
  p.add<float>((size_t)max_blocks * 32);
  p.add<int>(max_blocks);
  p.add<unsigned>((size_t)n_probs * 2);
}

rtr_status icp_multi(rtr_context* ctx, Scratch& s, std::vector<IcpSpec>& specs, cudaStream_t st) {
  const int M = (int)specs.size();
  if (M == 0) return RTR_OK;
  const int maxb = icp_max_blocks(ctx);
  if (M > maxb) return fail(RTR_ERR_CAPACITY, "icp: %d problems exceed the %d co-resident blocks", M, maxb);
  // a share of the GPU when several contexts run cooperative kernels at once
  int budget = maxb / (ctx->coop_div > 0 ? ctx->coop_div : 1);
  if (budget < M) budget = M;
  IcpDev* d_probs = s.take<IcpDev>(M);
  int* d_b2p = s.take<int>(maxb);
  double* pose64 = s.take<double>((size_t)M * 16);
  float* posef = s.take<float>((size_t)M * 16);
  float* partial = s.take<float>((size_t)maxb * 32);
  int* pcount = s.take<int>(maxb);
  unsigned* sync = s.take<unsigned>((size_t)M * 2);
  if (!sync) return fail(RTR_ERR_CAPACITY, "icp: scratch carve");
  // apportion blocks: want_i = ceil(n_i * G / threads), scaled to fit
  long long want_total = 0;
  std::vector<long long> want(M);
  for (int i = 0; i < M; ++i) {
    want[i] = ((long long)specs[i].dev.n_src * 8 + ICP_THREADS - 1) / ICP_THREADS;
    if (want[i] < 1) want[i] = 1;
    want_total += want[i];
  }
  std::vector<int> nblk(M);
  int used = 0;
  for (int i = 0; i < M; ++i) {
    long long b = want_total <= budget ? want[i] : (want[i] * (budget - M)) / want_total + 1;
    nblk[i] = (int)(b < 1 ? 1 : b);
    used += nblk[i];
  }
  int blk = 0;
  for (int i = 0; i < M; ++i) {
    IcpDev& d = specs[i].dev;
    d.blk0 = blk;
    d.nblk = nblk[i];
    d.pose64 = pose64 + 16 * i;
    d.posef = posef + 16 * i;
    d.partial = partial + (size_t)blk * 32;
    d.pcount = pcount + blk;
    d.arrive = sync + 2 * i;
    d.gen = sync + 2 * i + 1;
    d.status = ctx->d_status;
    d.budget = ctx->wait_budget_cycles;
    d.prof = i == 0 ? reinterpret_cast<unsigned long long*>(ctx->d_status + 32) : nullptr;
    blk += nblk[i];
  }
  RTR_CUDA(cudaMemsetAsync(ctx->d_status + 32, 0, 6 * sizeof(unsigned long long), st));
  for (int f = 0; f < M; f += ICP_SETUP_BATCH) {
    IcpSetup su;
    memset(&su, 0, sizeof(su));
    su.first = f;
    su.n = M - f < ICP_SETUP_BATCH ? M - f : ICP_SETUP_BATCH;
    for (int k = 0; k < su.n; ++k) {
      su.p[k] = specs[f + k].dev;
      su.init_dev[k] = specs[f + k].init_dev;
    }
    k_icp_setup<<<su.n, 128, 0, st>>>(su, d_probs, d_b2p);
    RTR_LAUNCHED(1);
  }
  RTR_CUDA(cudaGetLastError());
  long long total = 0;
  for (int i = 0; i < M; ++i) total += specs[i].dev.n_src;
  return launch_icp(icp_pick_group(ctx, total, used), d_probs, d_b2p, used, st);
}

}  // namespace rtr

using namespace rtr;

extern "C" {

void rtr_icp_default_params(rtr_icp_params* p) {
  if (!p) return;
  p->max_iterations = 10;
  p->max_corr_dist = 0.f;
  p->transformation_epsilon = 0.0;
  p->rotation_epsilon = 0.0;
  p->cell_size = 0.f;
  p->record_trace = 0;
}

rtr_status rtr_icp(rtr_context* ctx, const float* d_src, int n_src, const float* d_tgt, int n_tgt,
                   const rtr_icp_params* params, const double* h_init_pose,
                   rtr_icp_result* d_result, double* d_trace_pose, int32_t* d_trace_corr,
                   rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && params && d_result, "rtr_icp: ctx, params and d_result are required");
  RTR_CHECK_ARG(n_src > 0 && n_tgt > 0 && d_src && d_tgt, "rtr_icp: empty source or target");
  RTR_CHECK_ARG(params->max_iterations > 0, "rtr_icp: max_iterations must be > 0");
  RTR_CHECK_ARG(((uintptr_t)d_src & 15) == 0 && ((uintptr_t)d_tgt & 15) == 0,
                "rtr_icp: point arrays must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));

  const unsigned cell_cap = default_cell_cap(n_tgt);
  const int maxb = icp_max_blocks(ctx);
  int blocks = (int)(((long long)n_src * 8 + ICP_THREADS - 1) / ICP_THREADS);
  if (blocks > maxb) blocks = maxb;
  if (blocks < 1) blocks = 1;

  ScratchPlan plan;
  grid_plan(plan, n_tgt, cell_cap);
  plan.add<float4>(n_src);
  plan.add<int>(n_src);
  for (int i = 0; i < 4; ++i) plan.add<uint32_t>(n_src);
  plan.add<uint32_t>(radix_hist_entries(n_src));
  plan.add<GridMeta>(1);
  icp_multi_plan(plan, 1, maxb);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  GridBufs gb;
  if (!grid_take(s, n_tgt, cell_cap, &gb)) return fail(RTR_ERR_CAPACITY, "rtr_icp: scratch carve");
  float4* src_sorted = s.take<float4>(n_src);
  int* src_idx = s.take<int>(n_src);
  uint32_t* k0 = s.take<uint32_t>(n_src);
  uint32_t* v0 = s.take<uint32_t>(n_src);
  uint32_t* k1 = s.take<uint32_t>(n_src);
  uint32_t* v1 = s.take<uint32_t>(n_src);
  uint32_t* hist = s.take<uint32_t>(radix_hist_entries(n_src));
  GridMeta* src_meta = s.take<GridMeta>(1);
  if (!src_meta) return fail(RTR_ERR_CAPACITY, "rtr_icp: scratch carve");

  float h = params->cell_size;
  if (!(h > 0.f)) h = params->max_corr_dist > 0.f ? 0.5f * params->max_corr_dist : -1.f;
  {
    ProfScope ps(ctx, st, "grid_build");
    grid_build(gb, reinterpret_cast<const float4*>(d_tgt), n_tgt, nullptr, h, st);
  }

  IcpDev a;
  memset(&a, 0, sizeof(a));
  a.grid = grid_dev(gb);
  a.src_meta = src_meta;
  bbox_build(src_meta, reinterpret_cast<const float4*>(d_src), n_src, st);
  a.src = src_sorted;
  a.src_idx = src_idx;
  a.n_src = n_src;
  a.max_it = params->max_iterations;
  const float r = params->max_corr_dist;
  a.r2max = (r > 0.f && r < 1e18f) ? r * r : __builtin_inff();
  a.eps_t = params->transformation_epsilon;
  a.eps_r = params->rotation_epsilon;
  for (int k = 0; k < 16; ++k) a.init[k] = h_init_pose ? h_init_pose[k] : ((k % 5) == 0 ? 1.0 : 0.0);
  a.result = d_result;
  a.trace_pose = params->record_trace ? d_trace_pose : nullptr;
  a.trace_corr = params->record_trace ? d_trace_corr : nullptr;

  int nb = (n_src + 255) / 256;
  if (nb > 152 * 8) nb = 152 * 8;
  ProfScope ps_sort(ctx, st, "src_sort");
  k_src_keys<<<nb, 256, 0, st>>>(reinterpret_cast<const float4*>(d_src), n_src, a, k0);
  int bits = 1;
  while (bits < 32 && (1ull << bits) < (unsigned long long)cell_cap) ++bits;
  uint32_t *ks, *vs;
  radix_sort_pairs(k0, v0, k1, v1, hist, n_src, n_src, nullptr, bits, true, st, &ks, &vs);
  k_gather_pts<<<nb, 256, 0, st>>>(reinterpret_cast<const float4*>(d_src), vs, n_src, src_sorted,
                                   src_idx);
  RTR_LAUNCHED(2);
  RTR_CUDA(cudaGetLastError());
  ps_sort.end();
  ProfScope ps(ctx, st, "icp_kernel");
  std::vector<IcpSpec> specs(1);
  specs[0].dev = a;
  specs[0].init_dev = nullptr;
  return icp_multi(ctx, s, specs, st);
}

rtr_status rtr_icp_multi(rtr_context* ctx, const float* d_src, int n_src, const float* d_tgt, int n_tgt,
                         const rtr_icp_params* params, const double* d_init_poses, int n_problems,
                         rtr_icp_result* d_results, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && params && d_results, "rtr_icp_multi: ctx, params and d_results are required");
  RTR_CHECK_ARG(n_src > 0 && n_tgt > 0 && d_src && d_tgt, "rtr_icp_multi: empty source or target");
  RTR_CHECK_ARG(params->max_iterations > 0, "rtr_icp_multi: max_iterations must be > 0");
  RTR_CHECK_ARG(((uintptr_t)d_src & 15) == 0 && ((uintptr_t)d_tgt & 15) == 0,
                "rtr_icp_multi: point arrays must be 16-byte aligned");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  const int maxb = icp_max_blocks(ctx);
  RTR_CHECK_ARG(n_problems >= 1 && n_problems <= maxb, "rtr_icp_multi: n_problems must be in [1, %d]", maxb);
  const unsigned cell_cap = default_cell_cap(n_tgt);
  ScratchPlan plan;
  grid_plan(plan, n_tgt, cell_cap);
  plan.add<GridMeta>(1);
  icp_multi_plan(plan, n_problems, maxb);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  GridBufs gb;
  if (!grid_take(s, n_tgt, cell_cap, &gb)) return fail(RTR_ERR_CAPACITY, "rtr_icp_multi: scratch carve");
  GridMeta* src_meta = s.take<GridMeta>(1);
  if (!src_meta) return fail(RTR_ERR_CAPACITY, "rtr_icp_multi: scratch carve");
  float h = params->cell_size;
  if (!(h > 0.f)) h = params->max_corr_dist > 0.f ? 0.5f * params->max_corr_dist : -1.f;
  ProfScope ps(ctx, st, "icp_multi");
  grid_build(gb, reinterpret_cast<const float4*>(d_tgt), n_tgt, nullptr, h, st);
  bbox_build(src_meta, reinterpret_cast<const float4*>(d_src), n_src, st);
  std::vector<IcpSpec> specs((size_t)n_problems);
  const float r = params->max_corr_dist;
  for (int k = 0; k < n_problems; ++k) {
    IcpDev& a = specs[(size_t)k].dev;
    memset(&a, 0, sizeof(a));
    a.grid = grid_dev(gb);
    a.src_meta = src_meta;
    a.src = reinterpret_cast<const float4*>(d_src);
    a.src_idx = nullptr;
    a.n_src = n_src;
    a.max_it = params->max_iterations;
    a.r2max = (r > 0.f && r < 1e18f) ? r * r : __builtin_inff();
    a.eps_t = params->transformation_epsilon;
    a.eps_r = params->rotation_epsilon;
    for (int e = 0; e < 16; ++e) a.init[e] = (e % 5) == 0 ? 1.0 : 0.0;
    a.result = d_results + k;
    specs[(size_t)k].init_dev = d_init_poses ? d_init_poses + 16 * (size_t)k : nullptr;
  }
  return icp_multi(ctx, s, specs, st);
}

rtr_status rtr_icp_host(rtr_context* ctx, const float* h_src, int n_src, const float* h_tgt,
                        int n_tgt, const rtr_icp_params* params, const double* h_init_pose,
                        rtr_icp_result* h_result) {
  RTR_CHECK_ARG(ctx && h_src && h_tgt && params && h_result && n_src > 0 && n_tgt > 0,
                "rtr_icp_host: bad arguments");
  RTR_CUDA(cudaSetDevice(ctx->device));
  const size_t bs = (size_t)n_src * 16, bt = (size_t)n_tgt * 16;
  const size_t need = ((bs + 255) & ~size_t(255)) + ((bt + 255) & ~size_t(255)) + 256;
  RTR_TRY(ensure_io(ctx, need));
  char* io = static_cast<char*>(ctx->io);
  float* d_src = reinterpret_cast<float*>(io);
  float* d_tgt = reinterpret_cast<float*>(io + ((bs + 255) & ~size_t(255)));
  rtr_icp_result* d_res =
      reinterpret_cast<rtr_icp_result*>(io + ((bs + 255) & ~size_t(255)) + ((bt + 255) & ~size_t(255)));
  cudaStream_t st = ctx->host_stream;
  RTR_CUDA(cudaMemcpyAsync(d_src, h_src, bs, cudaMemcpyHostToDevice, st));
  RTR_CUDA(cudaMemcpyAsync(d_tgt, h_tgt, bt, cudaMemcpyHostToDevice, st));
  RTR_TRY(rtr_icp(ctx, d_src, n_src, d_tgt, n_tgt, params, h_init_pose, d_res, nullptr, nullptr, st));
  RTR_CUDA(cudaMemcpyAsync(h_result, d_res, sizeof(rtr_icp_result), cudaMemcpyDeviceToHost, st));
  return rtr_context_check(ctx, st);
}

}  // extern "C"

extern "C" rtr_status rtr_icp_stats(rtr_context* ctx, long long* h_stats6) {
  RTR_CHECK_ARG(ctx && h_stats6, "rtr_icp_stats: bad arguments");
  RTR_CUDA(cudaSetDevice(ctx->device));
  RTR_CUDA(cudaDeviceSynchronize());
  RTR_CUDA(cudaMemcpy(h_stats6, ctx->d_status + 32, 6 * sizeof(long long), cudaMemcpyDeviceToHost));
  return RTR_OK;
}
