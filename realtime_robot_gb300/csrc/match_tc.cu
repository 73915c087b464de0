// match_tc.cu — descriptor 1-NN on the 5th-generation tensor cores.
//
// d^2(q, b) = |q|^2 + |b|^2 - 2 q.b with the dot product as a BF16 GEMM with
// FP32 accumulation in tensor memory.  Each FP32 descriptor is split into
// hi = bf16(x) and lo = bf16(x - hi); the accumulator sums hi.hi + hi.lo +
// lo.hi (three tcgen05.mma per K step), which leaves |err(q.b)| of order
// 1e-4 |q| |b| (dropped lo.lo, the split's rounding, FP32 accumulation); the
// certification uses TC_ERR * max(|q|, max |b|)^2, which covers that and the
// FP32 norms with margin (unit-norm SHOT vectors: 1e-3).  Inf or NaN values
// make a query uncertified.  Per query the epilogue keeps the 8
// smallest approximate distances; an exact FP32 re-rank (sequential sums, as
// the oracle) picks the winner, and a query is certified when its 8th
// approximate distance minus the error bound is still above the exact winner,
// so no unseen descriptor can beat or tie it.  Uncertified queries (near-ties)
// take a band pass: the same GEMM over them lists every row whose d~ is
// within twice the bound of the exact winner (every row that could tie or beat
// it), and exact distances to those rows decide; a band over TC_BAND rows
// falls back to an exact scan of the whole database.  The result is
// bit-identical to the exact matcher.
//
// Kernel layout (one CTA per 128 queries, 6 warps): warp 4 issues TMA loads of
// the K-blocks (32 bf16 = one 64-byte swizzle row) of Q_hi, Q_lo, B_hi, B_lo
// into a 4-stage ring; warp 5 issues tcgen05.mma (M=128, N=256, K=16) into one
// of two TMEM accumulators (2 x 256 columns); warps 0-3 drain the finished
// accumulator with tcgen05.ld (thread = query row) and update the top-8.
// Every mbarrier wait is bounded; on timeout the CTA records RTR_ERR_TIMEOUT,
// stops issuing, waits (bounded) for its in-flight work and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <string.h>

#include "common.cuh"

namespace rtr {

constexpr int TC_DIM = 352;
constexpr int TC_KPAD = 384;              // 6 K-blocks of 64
// K-blocks of 32 bf16 (one 64-byte swizzle row): 48 KB stages, four of
// them in flight (two 96 KB stages of 64-wide K-blocks ran 3 % slower).
constexpr int TC_KB = 32;
constexpr int TC_NKB = TC_KPAD / TC_KB;
constexpr int TC_SW = TC_KB * 2;          // swizzle row bytes (64)
constexpr int TC_BM = 128;
constexpr int TC_BN = 256;
constexpr int TC_STAGES = 4;
constexpr int TC_TOP = 8;
constexpr int TC_BAND = 256;      // band pass: rows listed per uncertified query
constexpr int TC_BAND_Q = 16384;  // band pass: uncertified queries it takes (the rest: full scan)
constexpr int TC_A_BYTES = TC_BM * TC_KB * 2;   // 8 KB
constexpr int TC_B_BYTES = TC_BN * TC_KB * 2;   // 16 KB
constexpr int TC_STAGE_BYTES = 2 * TC_A_BYTES + 2 * TC_B_BYTES;  // 48 KB
constexpr int TC_THREADS = 192;
constexpr float TC_ERR = 1.0e-3f;  // conservative bound on |d~ - d| (see top)
constexpr long long TC_SPIN_LIMIT = 1LL << 26;

// ---------------------------------------------------------------------------
// PTX helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait (`limit` tries, from the context's wait budget); returns false
// (and raises the CTA abort flag) on timeout or when another role aborted
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* abort, long long limit) {
  for (long long i = 0; i < limit; ++i) {
    if (mbar_try(b, parity)) return true;
    if (*abort) return false;
  }
  *abort = 1;
  return false;
}
// the drain after an abort: wait for work already issued, up to the fixed
// TC_SPIN_LIMIT tries whatever the budget (a copy or MMA in flight ends by
// itself; this only bounds the wait if the hardware stopped answering)
__device__ __forceinline__ void mbar_drain(uint64_t* b, uint32_t parity) {
  for (long long i = 0; i < TC_SPIN_LIMIT; ++i)
    if (mbar_try(b, parity)) return;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}
// UMMA shared-memory descriptor: K-major, TC_SW-byte swizzle rows, 8-row
// atoms of 8 * TC_SW bytes (SBO), start address in 16-byte units, descriptor
// version 1; layout type 4 = 64-byte swizzle, 2 = 128-byte swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);       // start address
  d |= (uint64_t)1 << 16;                         // LBO (unused for swizzled K-major)
  d |= (uint64_t)((8 * TC_SW) >> 4) << 32;        // SBO
  d |= (uint64_t)1 << 46;                         // version
  d |= (uint64_t)(TC_SW == 128 ? 2 : 4) << 61;    // swizzle mode
  return d;
}
// Instruction descriptor, kind::f16: D = F32, A = B = BF16, K-major, N, M.
__device__ __forceinline__ uint32_t umma_idesc() {
  uint32_t d = 0;
  d |= 1u << 4;                          // D format F32
  d |= 1u << 7;                          // A BF16
  d |= 1u << 10;                         // B BF16
  d |= (uint32_t)(TC_BN >> 3) << 17;     // N
  d |= (uint32_t)(TC_BM >> 4) << 24;     // M
  return d;
}
__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
          tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(accum)
      : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---------------------------------------------------------------------------
// FP32 descriptors -> padded (hi, lo) BF16 rows + FP32 squared norms
// ---------------------------------------------------------------------------
// hi/lo split of each row, padded to TC_KPAD.  Column TC_DIM carries the
// norm term so that the GEMM yields q.b - |b|^2 / 2 directly: 1 in query
// rows, -|b|^2 / 2 (itself split) in database rows.
__global__ void k_split_bf16(const float* __restrict__ x, int n_host, const int* d_n, int n_cap,
                             __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
                             float* __restrict__ norm2, unsigned* __restrict__ max_bits, bool is_db,
                             unsigned char* __restrict__ zero_row) {
  static_assert(TC_DIM % 4 == 0 && TC_KPAD == 96 * 4, "a row is 96 groups of four columns");
  const int n = d_n ? min(*d_n, n_cap) : n_host;
  const int lane = threadIdx.x & 31;
  const bool v4 = (reinterpret_cast<uintptr_t>(x) & 15u) == 0;
  for (int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n_cap; r += gridDim.x * (blockDim.x >> 5)) {
    // lane takes column groups lane, lane + 32, lane + 64: four columns each,
    // one 16-byte load and two 8-byte stores
    float ss = 0.f;
    bool nz = false;
    float4 vv[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int c4 = lane + 32 * k;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r < n && c4 < TC_DIM / 4) {
        const float* src = x + (size_t)r * TC_DIM + 4 * c4;
        v = v4 ? __ldg(reinterpret_cast<const float4*>(src)) : make_float4(src[0], src[1], src[2], src[3]);
      }
      vv[k] = v;
      nz |= v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f;
      ss += v.x * v.x + v.y * v.y + v.z * v.z + v.w * v.w;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
    nz = __any_sync(0xffffffffu, nz);
    // column TC_DIM carries the norm term: 1 in query rows, -|b|^2 / 2 in
    // database rows (zero in padding rows)
    const float tv = r < n ? (is_db ? -0.5f * ss : 1.f) : 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int c4 = lane + 32 * k;
      float4 v = vv[k];
      if (c4 == TC_DIM / 4) v.x = tv;
      const float e[4] = {v.x, v.y, v.z, v.w};
      __nv_bfloat16 h[4], l[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        h[j] = __float2bfloat16_rn(e[j]);
        l[j] = __float2bfloat16_rn(e[j] - __bfloat162float(h[j]));
      }
      uint2 hp, lp;
      hp.x = (unsigned)__bfloat16_as_ushort(h[0]) | ((unsigned)__bfloat16_as_ushort(h[1]) << 16);
      hp.y = (unsigned)__bfloat16_as_ushort(h[2]) | ((unsigned)__bfloat16_as_ushort(h[3]) << 16);
      lp.x = (unsigned)__bfloat16_as_ushort(l[0]) | ((unsigned)__bfloat16_as_ushort(l[1]) << 16);
      lp.y = (unsigned)__bfloat16_as_ushort(l[2]) | ((unsigned)__bfloat16_as_ushort(l[3]) << 16);
      reinterpret_cast<uint2*>(hi + (size_t)r * TC_KPAD)[c4] = hp;
      reinterpret_cast<uint2*>(lo + (size_t)r * TC_KPAD)[c4] = lp;
    }
    if (lane == 0) {
      norm2[r] = ss;
      if (max_bits && r < n) atomicMax(max_bits, __float_as_uint(ss));  // ss >= 0 (or NaN: stays largest)
      if (zero_row) zero_row[r] = (r < n && !nz) ? 1 : 0;
    }
  }
}

// ---------------------------------------------------------------------------
// GEMM + top-8
// ---------------------------------------------------------------------------
struct TcArgs {
  int nq_host;
  const int* d_nq;
  int nq_cap;
  int ndb;
  const float* qn;   // [nq_cap] |q|^2
  int* cand_idx;     // [nq_cap][8]; band pass: [nq_cap][TC_BAND] rows within the threshold
  float* cand_d;     // [nq_cap][8]
  int* status;
  const float* thr;  // band pass: [nq_cap] largest d~ a row may have and still tie the winner
  int* band_n;       // band pass: [nq_cap] rows listed (over TC_BAND: overflowed)
  long long spin_limit;  // tries per mbarrier wait (the context's wait budget)
};

// BAND = false: per query the 8 smallest d~ (the first pass).  BAND = true:
// per query every row with d~ <= thr[q] (the band pass over uncertified
// queries), the first TC_BAND of them listed in band_n[q] (zeroed by the
// caller; a count over TC_BAND means the band overflowed and the row stops
// counting); its grid splits the database into gridDim.y ranges so that a
// few uncertified queries still fill the GPU.
template <bool BAND>
__global__ void __launch_bounds__(TC_THREADS, 1) k_match_tc(const __grid_constant__ CUtensorMap mq_hi,
                                                            const __grid_constant__ CUtensorMap mq_lo,
                                                            const __grid_constant__ CUtensorMap mb_hi,
                                                            const __grid_constant__ CUtensorMap mb_lo, TcArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t full_bar[TC_STAGES], empty_bar[TC_STAGES], acc_full[2], acc_empty[2], drain_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nq = a.d_nq ? min(*a.d_nq, a.nq_cap) : a.nq_host;
  const int q0 = blockIdx.x * TC_BM;
  if (q0 >= nq) return;  // uniform per CTA, before any barrier or TMEM use
  // database tiles of this CTA: all of them, or (band pass, gridDim.y > 1)
  // one of gridDim.y contiguous ranges
  const int n_all = (a.ndb + TC_BN - 1) / TC_BN;
  const int t_lo = (int)((long long)blockIdx.y * n_all / gridDim.y);
  const int t_hi = (int)((long long)(blockIdx.y + 1) * n_all / gridDim.y);

  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < TC_STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 128);
    }
    mbar_init(&drain_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 5) {  // allocate 512 TMEM columns (two 128 x 256 FP32 accumulators)
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  volatile int* abort = &abort_flag;
  const long long lim = a.spin_limit;
  int issued = 0;  // producer: stage loads issued

  if (warp == 4) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int it = 0;
      for (int t = t_lo; t < t_hi && !*abort; ++t) {
        for (int kb = 0; kb < TC_NKB && !*abort; ++kb, ++it) {
          const int s = it % TC_STAGES;
          const uint32_t ph = (uint32_t)(it / TC_STAGES) & 1u;
          if (it >= TC_STAGES && !mbar_wait(&empty_bar[s], ph ^ 1u, abort, lim)) break;
          uint8_t* st = smem + s * TC_STAGE_BYTES;
          mbar_expect_tx(&full_bar[s], TC_STAGE_BYTES);
          tma_load_2d(st, &mq_hi, &full_bar[s], kb * TC_KB, q0);
          tma_load_2d(st + TC_A_BYTES, &mq_lo, &full_bar[s], kb * TC_KB, q0);
          tma_load_2d(st + 2 * TC_A_BYTES, &mb_hi, &full_bar[s], kb * TC_KB, t * TC_BN);
          tma_load_2d(st + 2 * TC_A_BYTES + TC_B_BYTES, &mb_lo, &full_bar[s], kb * TC_KB, t * TC_BN);
        }
      }
      issued = it;
    }
  } else if (warp == 5) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t idesc = umma_idesc();
      int it = 0;
      for (int t = t_lo; t < t_hi && !*abort; ++t) {
        const int buf = (t - t_lo) & 1;
        const uint32_t use = (uint32_t)((t - t_lo) >> 1);
        if (t - t_lo >= 2 && !mbar_wait(&acc_empty[buf], (use - 1) & 1u, abort, lim)) break;
        tc_fence_after();
        const uint32_t dcol = tmem + (uint32_t)buf * TC_BN;
        for (int kb = 0; kb < TC_NKB; ++kb, ++it) {
          const int s = it % TC_STAGES;
          const uint32_t ph = (uint32_t)(it / TC_STAGES) & 1u;
          if (!mbar_wait(&full_bar[s], ph, abort, lim)) break;
          tc_fence_after();
          const uint32_t base = smem_u32(smem + s * TC_STAGE_BYTES);
          const uint32_t ah = base, al = base + TC_A_BYTES, bh = base + 2 * TC_A_BYTES,
                         bl = base + 2 * TC_A_BYTES + TC_B_BYTES;
#pragma unroll
          for (int k = 0; k < TC_KB / 16; ++k) {
            const uint32_t off = (uint32_t)k * 32;  // 16 bf16 along K inside the swizzle row
            const uint32_t acc0 = (kb > 0 || k > 0) ? 1u : 0u;
            umma_f16(dcol, umma_desc(ah + off), umma_desc(bh + off), idesc, acc0);
            umma_f16(dcol, umma_desc(ah + off), umma_desc(bl + off), idesc, 1u);
            umma_f16(dcol, umma_desc(al + off), umma_desc(bh + off), idesc, 1u);
          }
          umma_commit(&empty_bar[s]);  // stage free once these MMAs have read it
        }
        umma_commit(&acc_full[buf]);  // accumulator ready
      }
    }
  } else {
    // ---------------- epilogue: warps 0-3, thread = query row ----------------
    // The accumulator holds q.b - |b|^2 / 2, so the nearest rows are the
    // largest values: one compare per element, d~ = |q|^2 - 2 acc at the end.
    const int row = warp * 32 + lane;
    const int q = q0 + row;
    const float qn = q < nq ? a.qn[q] : 0.f;
    if (BAND) {
      // rows past the live queries (stale scratch, any bits) list nothing
      const bool live = q < nq;
      const float thr = live ? a.thr[q] : 0.f;
      int* list = a.cand_idx + (size_t)(live ? q : 0) * TC_BAND;
      bool over = false;  // this row's band already past TC_BAND: count no further
      for (int t = t_lo; t < t_hi; ++t) {
        const int buf = (t - t_lo) & 1;
        const uint32_t use = (uint32_t)((t - t_lo) >> 1);
        if (!mbar_wait(&acc_full[buf], use & 1u, abort, lim)) break;
        tc_fence_after();
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)buf * TC_BN;
        const int valid = min(TC_BN, a.ndb - t * TC_BN);
        for (int c0 = 0; c0 < TC_BN; c0 += 32) {
          float v[32];
          tmem_ld32(taddr + (uint32_t)c0, v);
          const int jb = t * TC_BN + c0;
          const int lim = valid - c0;
          // d~ exactly as the first pass forms it for its candidates
          uint32_t hit = 0;
#pragma unroll
          for (int i = 0; i < 32; ++i) hit |= (i < lim && qn - 2.f * v[i] <= thr) ? (1u << i) : 0u;
          if (live && hit && !over) {
            // one atomic per chunk (CTAs of other database ranges list into the same row)
            int pos = atomicAdd(a.band_n + q, __popc(hit));
            over = pos + __popc(hit) > TC_BAND;
            while (hit && pos < TC_BAND) {
              list[pos++] = jb + __ffs(hit) - 1;
              hit &= hit - 1;
            }
          }
        }
        tc_fence_before();
        mbar_arrive(&acc_empty[buf]);
      }
    } else {
    float ba[TC_TOP];
    int bi[TC_TOP];
#pragma unroll
    for (int s = 0; s < TC_TOP; ++s) {
      ba[s] = -__int_as_float(0x7f800000);
      bi[s] = 0x7fffffff;
    }
    for (int t = t_lo; t < t_hi; ++t) {
      const int buf = (t - t_lo) & 1;
      const uint32_t use = (uint32_t)((t - t_lo) >> 1);
      if (!mbar_wait(&acc_full[buf], use & 1u, abort, lim)) break;
      tc_fence_after();
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)buf * TC_BN;
      const int valid = min(TC_BN, a.ndb - t * TC_BN);  // rows past the database read as zero
      for (int c0 = 0; c0 < TC_BN; c0 += 32) {
        float v[32];
        tmem_ld32(taddr + (uint32_t)c0, v);
        const int jb = t * TC_BN + c0;
        const int lim = valid - c0;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          if (v[i] > ba[TC_TOP - 1] && i < lim) {
            ba[TC_TOP - 1] = v[i];
            bi[TC_TOP - 1] = jb + i;
#pragma unroll
            for (int s = TC_TOP - 1; s > 0; --s) {
              const bool gt = ba[s] > ba[s - 1];
              const float x0 = ba[s], x1 = ba[s - 1];
              const int y0 = bi[s], y1 = bi[s - 1];
              ba[s] = gt ? x1 : x0;
              ba[s - 1] = gt ? x0 : x1;
              bi[s] = gt ? y1 : y0;
              bi[s - 1] = gt ? y0 : y1;
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&acc_empty[buf]);
    }
    if (q < nq) {
#pragma unroll
      for (int s = 0; s < TC_TOP; ++s) {
        a.cand_idx[(size_t)q * TC_TOP + s] = bi[s] == 0x7fffffff ? -1 : bi[s];
        a.cand_d[(size_t)q * TC_TOP + s] = bi[s] == 0x7fffffff ? __int_as_float(0x7f800000) : qn - 2.f * ba[s];
      }
    }
    }
  }
  // after an abort nothing of this CTA may still be in flight when it frees
  // its TMEM and exits: the MMA issuer waits for every MMA it issued, the
  // producer for the stage loads not yet seen complete (the last ones; each
  // earlier load of a stage completed before the stage was reused)
  __syncthreads();
  if (abort_flag) {
    if (warp == 5 && lane == 0) {
      umma_commit(&drain_bar);
      mbar_drain(&drain_bar, 0u);
    }
    if (warp == 4 && lane == 0)
      for (int i = issued > TC_STAGES ? issued - TC_STAGES : 0; i < issued; ++i)
        mbar_drain(&full_bar[i % TC_STAGES], (uint32_t)(i / TC_STAGES) & 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (abort_flag && threadIdx.x == 0) atomicExch(a.status, (int)RTR_ERR_TIMEOUT);
  if (warp == 5) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
  }
}

// Exact d^2 of one 352-float row pair: sequential sum in k order, each
// operation rounded (the oracle's order).  V4: both rows 16-byte aligned.
template <bool V4>
__device__ __forceinline__ float exact_d2(const float* __restrict__ x, const float* __restrict__ y) {
  float acc = 0.f;
  if (V4) {
    const float4* x4 = reinterpret_cast<const float4*>(x);
    const float4* y4 = reinterpret_cast<const float4*>(y);
#pragma unroll 4
    for (int k = 0; k < TC_DIM / 4; ++k) {
      const float4 a = __ldg(x4 + k), b = __ldg(y4 + k);
      float t = __fsub_rn(a.x, b.x);
      acc = __fadd_rn(acc, __fmul_rn(t, t));
      t = __fsub_rn(a.y, b.y);
      acc = __fadd_rn(acc, __fmul_rn(t, t));
      t = __fsub_rn(a.z, b.z);
      acc = __fadd_rn(acc, __fmul_rn(t, t));
      t = __fsub_rn(a.w, b.w);
      acc = __fadd_rn(acc, __fmul_rn(t, t));
    }
  } else {
    for (int k = 0; k < TC_DIM; ++k) {
      const float t = __fsub_rn(x[k], y[k]);
      acc = __fadd_rn(acc, __fmul_rn(t, t));
    }
  }
  return acc;
}

// Exact FP32 re-rank of the candidates that can still win and
// certification; four queries per warp, one lane per candidate.  Uncertified
// queries go to the redo list with their running minimum reset.
template <bool V4>
__global__ void __launch_bounds__(256) k_rerank(const float* __restrict__ q, int nq_host, const int* d_nq, int nq_cap,
                                                const float* __restrict__ db, int ndb,
                                                const int* __restrict__ cand_idx, const float* __restrict__ cand_d,
                                                int* __restrict__ out_idx, float* __restrict__ out_d2,
                                                int* __restrict__ redo, int* __restrict__ n_redo,
                                                unsigned long long* __restrict__ redo_best,
                                                float* __restrict__ redo_thr,
                                                const float* __restrict__ qn, const float* __restrict__ db_max,
                                                const unsigned long long* __restrict__ zero_best,
                                                const unsigned char* __restrict__ qzero) {
  const int nq = d_nq ? min(*d_nq, nq_cap) : nq_host;
  const int lane = threadIdx.x & 31, sub = lane >> 3, l8 = lane & 7;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int base = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * 4; base < nq; base += warps * 4) {
    const int i = base + sub;
    const bool valid = i < nq;
    const bool zq = valid && qzero[i] != 0;  // (no early exit: the shuffles below need every lane)
    int c = valid && !zq ? cand_idx[(size_t)i * TC_TOP + l8] : -1;
    if (c >= ndb) c = -1;  // never read past the database, whatever the first pass left
    // |d~ - d| <= err: a candidate whose d~ exceeds the smallest d~ (the
    // first, the list is ascending) by more than 2 err has an exact distance
    // above that candidate's, so it can neither win nor tie: its exact
    // distance is not computed
    const float err_q = valid ? TC_ERR * fmaxf(qn[i], *db_max) : 0.f;
    const bool need = c >= 0 && cand_d[(size_t)i * TC_TOP + l8] <= cand_d[(size_t)i * TC_TOP] + 2.f * err_q;
    float d = __int_as_float(0x7f800000);
    if (need) d = exact_d2<V4>(q + (size_t)i * TC_DIM, db + (size_t)c * TC_DIM);
    int bi = need ? c : 0x7fffffff;
    float bd = d;
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {  // within the aligned group of 8 lanes
      const float od = __shfl_xor_sync(0xffffffffu, bd, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (od < bd || (od == bd && oi < bi)) {
        bd = od;
        bi = oi;
      }
    }
    if (zq && l8 == 0) {
      // an all-zero query ties (up to rounding) with every unit-norm row: its
      // answer is the database's, the row of least exact sequential |b|^2
      // (lowest index on ties), found when the database was split
      const unsigned long long key = *zero_best;
      out_idx[i] = key == ~0ull ? -1 : (int)(unsigned)(key & 0xffffffffull);
      if (out_d2) out_d2[i] = key == ~0ull ? __int_as_float(0x7f800000) : __uint_as_float((unsigned)(key >> 32));
    } else if (valid && l8 == 0) {
      const float worst = cand_d[(size_t)i * TC_TOP + TC_TOP - 1];
      const int nvalid = ndb < TC_TOP ? ndb : TC_TOP;
      const bool all_seen = nvalid < TC_TOP;  // every descriptor was a candidate
      // the bound scales with the norms: |err| <= TC_ERR * max(|q|, |b|max)^2
      const float err = TC_ERR * fmaxf(qn[i], *db_max);
      const bool certified = all_seen || (worst - err > bd);
      if (certified) {
        out_idx[i] = bi == 0x7fffffff ? -1 : bi;
        if (out_d2) out_d2[i] = bd;
      } else {
        const int p = atomicAdd(n_redo, 1);
        redo[p] = i;
        redo_best[p] = ~0ull;
        // a row that ties or beats the exact winner has d~ <= bd + err; the
        // band pass lists rows up to twice that margin
        redo_thr[p] = bd + 2.f * err;
      }
    }
  }
}

// The answer for an all-zero query: min over rows of the exact sequential
// sum of (0 - b_k)^2 = b_k^2 (each operation rounded, as exact_d2 with a
// zero row), packed (d^2 bits, index) so that atomicMin keeps the lowest
// index on ties.  Rows with an infinite or NaN sum never win.  It depends on
// the database only: computed when the database is split.
__global__ void k_zero_best(const float* __restrict__ db, int ndb, unsigned long long* __restrict__ best) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < ndb; j += gridDim.x * blockDim.x) {
    const float* y = db + (size_t)j * TC_DIM;
    float acc = 0.f;
    for (int k = 0; k < TC_DIM; ++k) {
      const float t = __fsub_rn(0.f, y[k]);
      acc = __fadd_rn(acc, __fmul_rn(t, t));
    }
    if (acc < __int_as_float(0x7f800000))
      atomicMin(best, ((unsigned long long)__float_as_uint(acc) << 32) | (unsigned)j);
  }
}

__global__ void k_band_gather(const uint4* __restrict__ qhi, const uint4* __restrict__ qlo,
                              const float* __restrict__ qn, const int* __restrict__ redo,
                              const int* __restrict__ n_redo, int cap, uint4* __restrict__ hi2, uint4* __restrict__ lo2,
                              float* __restrict__ qn2) {
  const int n = min(*n_redo, cap);
  constexpr int V = TC_KPAD * 2 / 16;  // uint4 per row
  const int lane = threadIdx.x & 31;
  for (int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < n; w += gridDim.x * (blockDim.x >> 5)) {
    const int i = redo[w];
    for (int k = lane; k < V; k += 32) {
      hi2[(size_t)w * V + k] = qhi[(size_t)i * V + k];
      lo2[(size_t)w * V + k] = qlo[(size_t)i * V + k];
    }
    if (lane == 0) qn2[w] = qn[i];
  }
}

// Band pass, step 3: exact FP32 distances to the listed rows, a block per
// query and a thread per row (a band holds at most TC_BAND = 256 rows).  The
// band holds every row that can tie or beat the exact winner, so its exact
// minimum (lowest index on ties) is the scan's.  Queries past TC_BAND_Q,
// with a band over TC_BAND rows, or with a non-finite threshold (Inf or NaN
// values) go to the full scan list.
template <bool V4>
__global__ void __launch_bounds__(256) k_band_rerank(const float* __restrict__ q, const float* __restrict__ db,
                                                     const int* __restrict__ redo, const int* __restrict__ n_redo,
                                                     const float* __restrict__ thr, const int* __restrict__ band_idx,
                                                     const int* __restrict__ band_n, int cap, int ndb,
                                                     unsigned long long* __restrict__ redo_best,
                                                     int* __restrict__ full, int* __restrict__ n_full) {
  static_assert(TC_BAND <= 256, "a thread per band row");
  __shared__ unsigned long long s_min[8];
  const int n = *n_redo;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int w = blockIdx.x; w < n; w += gridDim.x) {  // uniform per block
    const int cnt = w < cap ? band_n[w] : TC_BAND + 1;
    if (cnt > TC_BAND || !isfinite(w < cap ? thr[w] : 0.f)) {
      if (threadIdx.x == 0) full[atomicAdd(n_full, 1)] = w;
      continue;
    }
    const int i = redo[w];
    unsigned long long key = ~0ull;
    const int m = threadIdx.x;
    if (m < cnt) {
      const int j = band_idx[(size_t)w * TC_BAND + m];
      if ((unsigned)j < (unsigned)ndb) {  // (out of range only after a timed-out band pass, status set)
        const float d = exact_d2<V4>(q + (size_t)i * TC_DIM, db + (size_t)j * TC_DIM);
        if (d < __int_as_float(0x7f800000)) key = ((unsigned long long)__float_as_uint(d) << 32) | (unsigned)j;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, o);
      key = ok < key ? ok : key;
    }
    if (lane == 0) s_min[warp] = key;
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long b = s_min[0];
#pragma unroll
      for (int k = 1; k < 8; ++k) b = s_min[k] < b ? s_min[k] : b;
      redo_best[w] = b;
    }
    __syncthreads();  // s_min is reused by the next query
  }
}

// Exact scan for the queries the band pass could not settle: one CTA per
// (query, 256 database rows), thread per row; the winner is the minimum of
// (d^2 bits, index) packed in 64 bits (d^2 >= 0, so its bits order like the
// value).  A row wins only with d^2 < +inf, as in the sequential scan.
template <bool V4>
__global__ void __launch_bounds__(256) k_match_redo(const float* __restrict__ q, const float* __restrict__ db, int ndb,
                                                    const int* __restrict__ redo, const int* __restrict__ full,
                                                    const int* __restrict__ n_full,
                                                    unsigned long long* __restrict__ redo_best) {
  const int n = *n_full;
  const int rblocks = (ndb + 255) >> 8;
  const int lane = threadIdx.x & 31;
  for (long long item = blockIdx.x; item < (long long)n * rblocks; item += gridDim.x) {
    const int w = full[(int)(item / rblocks)], rb = (int)(item % rblocks);
    const int i = redo[w];
    const int j = rb * 256 + threadIdx.x;
    unsigned long long key = ~0ull;
    if (j < ndb) {
      const float d = exact_d2<V4>(q + (size_t)i * TC_DIM, db + (size_t)j * TC_DIM);
      if (d < __int_as_float(0x7f800000)) key = ((unsigned long long)__float_as_uint(d) << 32) | (unsigned)j;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ok = __shfl_xor_sync(0xffffffffu, key, o);
      key = ok < key ? ok : key;
    }
    if (lane == 0 && key != ~0ull) atomicMin(redo_best + w, key);
  }
}

__global__ void k_match_redo_out(const int* __restrict__ redo, const int* __restrict__ n_redo,
                                 const unsigned long long* __restrict__ redo_best, int* __restrict__ out_idx,
                                 float* __restrict__ out_d2) {
  const int n = *n_redo;
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < n; w += gridDim.x * blockDim.x) {
    const int i = redo[w];
    const unsigned long long key = redo_best[w];
    out_idx[i] = key == ~0ull ? -1 : (int)(unsigned)(key & 0xffffffffull);
    if (out_d2) out_d2[i] = key == ~0ull ? __int_as_float(0x7f800000) : __uint_as_float((unsigned)(key >> 32));
  }
}

// ---------------------------------------------------------------------------
// host: tensor maps through the driver entry point (no libcuda link)
// ---------------------------------------------------------------------------
typedef CUresult (*PFN_encodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static PFN_encodeTiled get_encode() {
  // resolved once (thread-safe static initialisation)
  static const PFN_encodeTiled fn = []() -> PFN_encodeTiled {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      return reinterpret_cast<PFN_encodeTiled>(p);
    return nullptr;
  }();
  return fn;
}

static bool make_map(CUtensorMap* m, const void* base, int rows, int box_rows) {
  PFN_encodeTiled enc = get_encode();
  if (!enc) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)TC_KPAD, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)TC_KPAD * 2};
  const cuuint32_t box[2] = {(cuuint32_t)TC_KB, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, TC_SW == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
             CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

size_t match_tc_bf16_bytes(int rows) { return (size_t)rows * TC_KPAD * 2; }

// rows of the band pass (a multiple of TC_BM)
static int band_rows(int nqp) { return nqp < TC_BAND_Q ? nqp : TC_BAND_Q; }

// mbarrier tries per wait for the context's wait budget (a try is a few
// dozen cycles; the default 2 s budget gives about 2^26 tries)
static long long tc_spin_limit(const rtr_context* ctx) {
  const long long t = ctx->wait_budget_cycles / 64;
  return t < 1 ? 1 : t;
}

void match_tc_plan(ScratchPlan& p, int nq_cap, bool with_db, int ndb) {
  const int nqp = ((nq_cap + TC_BM - 1) / TC_BM) * TC_BM;
  p.add<__nv_bfloat16>((size_t)nqp * TC_KPAD);
  p.add<__nv_bfloat16>((size_t)nqp * TC_KPAD);
  p.add<float>(nqp);
  if (with_db) {
    p.add<__nv_bfloat16>((size_t)ndb * TC_KPAD);
    p.add<__nv_bfloat16>((size_t)ndb * TC_KPAD);
    p.add<float>(db_norm_floats(ndb));
  }
  p.add<int>((size_t)nqp * TC_TOP);
  p.add<float>((size_t)nqp * TC_TOP);
  p.add<int>(nqp);
  p.add<unsigned long long>(nqp);
  p.add<int>(4);
  // band pass
  const int bq = band_rows(nqp);
  p.add<float>(nqp);
  p.add<int>(nqp);
  p.add<__nv_bfloat16>((size_t)bq * TC_KPAD);
  p.add<__nv_bfloat16>((size_t)bq * TC_KPAD);
  p.add<float>(bq);
  p.add<int>((size_t)bq * TC_BAND);
  p.add<int>(bq);
  p.add<unsigned char>(nqp);
}

// Splits a descriptor database once (the model side keeps the result).
rtr_status match_tc_prepare_db(const float* db, int ndb, __nv_bfloat16* hi, __nv_bfloat16* lo, float* norm2,
                               cudaStream_t st) {
  int blocks = (ndb + 7) / 8;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (blocks < 1) blocks = 1;
  // norm2[ndb] receives the largest squared norm (scales the error bound),
  // db_zero_key the answer for an all-zero query
  RTR_CUDA(cudaMemsetAsync(norm2 + ndb, 0, sizeof(float), st));
  RTR_CUDA(cudaMemsetAsync(db_zero_key(norm2, ndb), 0xff, sizeof(unsigned long long), st));
  k_split_bf16<<<blocks, 256, 0, st>>>(db, ndb, nullptr, ndb, hi, lo, norm2, reinterpret_cast<unsigned*>(norm2 + ndb),
                                       true, nullptr);
  const int zb = (ndb + 255) / 256 < 152 * 4 ? (ndb + 255) / 256 : 152 * 4;
  k_zero_best<<<zb > 0 ? zb : 1, 256, 0, st>>>(db, ndb, db_zero_key(norm2, ndb));
  RTR_LAUNCHED(2);
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

rtr_status match_tc_dev(rtr_context* ctx, Scratch& s, const float* q, int nq_cap, const int* d_nq, const float* db,
                        int ndb, const __nv_bfloat16* db_hi, const __nv_bfloat16* db_lo, const float* db_n2,
                        int* out_idx, float* out_d2, cudaStream_t st) {
  const int nqp = ((nq_cap + TC_BM - 1) / TC_BM) * TC_BM;
  __nv_bfloat16* qhi = s.take<__nv_bfloat16>((size_t)nqp * TC_KPAD);
  __nv_bfloat16* qlo = s.take<__nv_bfloat16>((size_t)nqp * TC_KPAD);
  float* qn = s.take<float>(nqp);
  if (!db_hi) {
    __nv_bfloat16* h = s.take<__nv_bfloat16>((size_t)ndb * TC_KPAD);
    __nv_bfloat16* l = s.take<__nv_bfloat16>((size_t)ndb * TC_KPAD);
    float* n2 = s.take<float>(db_norm_floats(ndb));
    if (!n2) return fail(RTR_ERR_CAPACITY, "match_tc: scratch");
    RTR_TRY(match_tc_prepare_db(db, ndb, h, l, n2, st));
    db_hi = h;
    db_lo = l;
    db_n2 = n2;
  }
  int* cidx = s.take<int>((size_t)nqp * TC_TOP);
  float* cd = s.take<float>((size_t)nqp * TC_TOP);
  int* redo = s.take<int>(nqp);
  unsigned long long* redo_best = s.take<unsigned long long>(nqp);
  int* nredo = s.take<int>(4);  // [0] uncertified, [1] left to the full scan
  const int bq = band_rows(nqp);
  float* redo_thr = s.take<float>(nqp);
  int* full = s.take<int>(nqp);
  __nv_bfloat16* hi2 = s.take<__nv_bfloat16>((size_t)bq * TC_KPAD);
  __nv_bfloat16* lo2 = s.take<__nv_bfloat16>((size_t)bq * TC_KPAD);
  float* qn2 = s.take<float>(bq);
  int* band_idx = s.take<int>((size_t)bq * TC_BAND);
  int* band_n = s.take<int>(bq);
  unsigned char* qzero = s.take<unsigned char>(nqp);
  if (!qzero) return fail(RTR_ERR_CAPACITY, "match_tc: scratch");
  int sb = (nqp + 7) / 8;
  if (sb > 152 * 16) sb = 152 * 16;
  {
    ProfScope pp(ctx, st, "match_split");
    k_split_bf16<<<sb, 256, 0, st>>>(q, nq_cap, d_nq, nqp, qhi, qlo, qn, nullptr, false, qzero);
  }
  CUtensorMap m_qh, m_ql, m_bh, m_bl, m_qh2, m_ql2;
  if (!make_map(&m_qh, qhi, nqp, TC_BM) || !make_map(&m_ql, qlo, nqp, TC_BM) || !make_map(&m_bh, db_hi, ndb, TC_BN) ||
      !make_map(&m_bl, db_lo, ndb, TC_BN) || !make_map(&m_qh2, hi2, bq, TC_BM) || !make_map(&m_ql2, lo2, bq, TC_BM))
    return fail(RTR_ERR_CUDA, "match_tc: cuTensorMapEncodeTiled failed");
  const size_t smem = (size_t)TC_STAGES * TC_STAGE_BYTES + 1024;
  // per call: the attribute is per device, and calls may come from several threads
  RTR_CUDA(cudaFuncSetAttribute(k_match_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  RTR_CUDA(cudaFuncSetAttribute(k_match_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  TcArgs a{nq_cap, d_nq, nq_cap, ndb, qn, cidx, cd, ctx->d_status, nullptr, nullptr, tc_spin_limit(ctx)};
  {
    ProfScope pg(ctx, st, "match_gemm");
    k_match_tc<false><<<nqp / TC_BM, TC_THREADS, smem, st>>>(m_qh, m_ql, m_bh, m_bl, a);
  }
  RTR_CUDA(cudaMemsetAsync(nredo, 0, 2 * sizeof(int), st));
  int rb = (nq_cap + 31) / 32;
  if (rb > 152 * 16) rb = 152 * 16;
  // block per uncertified query (grid-stride over the device-side count)
  const int wb = band_rows(nqp) < 152 * 8 ? band_rows(nqp) : 152 * 8;
  const bool v4 = ((reinterpret_cast<uintptr_t>(q) | reinterpret_cast<uintptr_t>(db)) & 15u) == 0;
  // band pass over the uncertified queries: the GEMM again, listing every
  // row within the tie margin, then exact distances to those rows only
  TcArgs ab{bq, nredo, bq, ndb, qn2, band_idx, nullptr, ctx->d_status, redo_thr, band_n, tc_spin_limit(ctx)};
  ProfScope pr(ctx, st, "match_rerank");
  if (v4)
    k_rerank<true><<<rb, 256, 0, st>>>(q, nq_cap, d_nq, nq_cap, db, ndb, cidx, cd, out_idx, out_d2, redo, nredo,
                                       redo_best, redo_thr, qn, db_n2 + ndb, db_zero_key(db_n2, ndb), qzero);
  else
    k_rerank<false><<<rb, 256, 0, st>>>(q, nq_cap, d_nq, nq_cap, db, ndb, cidx, cd, out_idx, out_d2, redo, nredo,
                                        redo_best, redo_thr, qn, db_n2 + ndb, db_zero_key(db_n2, ndb), qzero);
  pr.end();
  ProfScope pu(ctx, st, "match_uncertified");
  k_band_gather<<<(bq + 7) / 8 < 152 * 2 ? (bq + 7) / 8 : 152 * 2, 256, 0, st>>>(reinterpret_cast<const uint4*>(qhi), reinterpret_cast<const uint4*>(qlo),
                                              qn, redo, nredo, bq, reinterpret_cast<uint4*>(hi2),
                                              reinterpret_cast<uint4*>(lo2), qn2);
  RTR_CUDA(cudaMemsetAsync(band_n, 0, sizeof(int) * bq, st));
  {
    ProfScope pb(ctx, st, "match_band");
    const int n_tiles = (ndb + TC_BN - 1) / TC_BN;
    const dim3 grid(bq / TC_BM, n_tiles < 8 ? n_tiles : 8);
    k_match_tc<true><<<grid, TC_THREADS, smem, st>>>(m_qh2, m_ql2, m_bh, m_bl, ab);
  }
  if (v4) {
    k_band_rerank<true><<<wb, 256, 0, st>>>(q, db, redo, nredo, redo_thr, band_idx, band_n, bq, ndb, redo_best, full,
                                            nredo + 1);
    k_match_redo<true><<<152 * 8, 256, 0, st>>>(q, db, ndb, redo, full, nredo + 1, redo_best);
  } else {
    k_band_rerank<false><<<wb, 256, 0, st>>>(q, db, redo, nredo, redo_thr, band_idx, band_n, bq, ndb, redo_best, full,
                                             nredo + 1);
    k_match_redo<false><<<152 * 8, 256, 0, st>>>(q, db, ndb, redo, full, nredo + 1, redo_best);
  }
  k_match_redo_out<<<4, 256, 0, st>>>(redo, nredo, redo_best, out_idx, out_d2);
  RTR_LAUNCHED(9);
  // keep the number of uncertified queries and of full scans for rtr_match_stats
  RTR_CUDA(cudaMemcpyAsync(ctx->d_status + 8, nredo, 2 * sizeof(int), cudaMemcpyDeviceToDevice, st));
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

// ---------------------------------------------------------------------------
// Keypoint-credibility MLP inference on the tensor cores: 352 -> 128 -> 64
// -> 1 (ReLU, ReLU, sigmoid) with BF16 weights.  Layer 1 is a tcgen05 GEMM:
// each FP32 descriptor is split into three BF16 parts (hi + mid + lo = x up
// to the last part's rounding, 2^-24 of |x|), and the three products with
// the BF16 weights accumulate in FP32 in tensor memory: FP32-level accuracy.
// The epilogue (thread = row) adds the bias, applies the ReLU, runs layer 2
// (64 outputs, FP32 FMAs over the 128 inputs in order), the head and the
// sigmoid, so only the score leaves the CTA.
// ---------------------------------------------------------------------------
constexpr int MLP_TC_IN = 352, MLP_TC_H1 = 128, MLP_TC_H2 = 64;
constexpr int MLP_TC_A_BYTES = TC_BM * TC_KB * 2;     // 8 KB: one part's K-block
constexpr int MLP_TC_B_BYTES = MLP_TC_H1 * TC_KB * 2;  // 8 KB: W1's K-block
constexpr int MLP_TC_STAGE_BYTES = 3 * MLP_TC_A_BYTES + MLP_TC_B_BYTES;  // 32 KB
constexpr int MLP_TC_STAGES = 4;
constexpr int MLP_TC_SMEM = MLP_TC_STAGES * MLP_TC_STAGE_BYTES + 1024;

// hi / mid / lo BF16 parts of each row, padded to TC_KPAD (zero past 352 and
// in padding rows); a warp per row, four columns per lane and 16-byte loads.
__global__ void k_split3_bf16(const float* __restrict__ x, int n_cap_rows, const int* d_n, int n_pad,
                              __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ mid,
                              __nv_bfloat16* __restrict__ lo) {
  const int n = d_n ? min(*d_n, n_cap_rows) : n_cap_rows;
  const int lane = threadIdx.x & 31;
  for (int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < n_pad; r += gridDim.x * (blockDim.x >> 5)) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int c4 = lane + 32 * k;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (r < n && c4 < MLP_TC_IN / 4) v = __ldg(reinterpret_cast<const float4*>(x + (size_t)r * MLP_TC_IN) + c4);
      const float e[4] = {v.x, v.y, v.z, v.w};
      unsigned short h[4], m[4], l[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const __nv_bfloat16 bh = __float2bfloat16_rn(e[j]);
        const float r1 = e[j] - __bfloat162float(bh);
        const __nv_bfloat16 bm = __float2bfloat16_rn(r1);
        const __nv_bfloat16 bl = __float2bfloat16_rn(r1 - __bfloat162float(bm));
        h[j] = __bfloat16_as_ushort(bh);
        m[j] = __bfloat16_as_ushort(bm);
        l[j] = __bfloat16_as_ushort(bl);
      }
      const size_t o = (size_t)r * (TC_KPAD / 4) + c4;
      reinterpret_cast<uint2*>(hi)[o] = make_uint2(h[0] | ((unsigned)h[1] << 16), h[2] | ((unsigned)h[3] << 16));
      reinterpret_cast<uint2*>(mid)[o] = make_uint2(m[0] | ((unsigned)m[1] << 16), m[2] | ((unsigned)m[3] << 16));
      reinterpret_cast<uint2*>(lo)[o] = make_uint2(l[0] | ((unsigned)l[1] << 16), l[2] | ((unsigned)l[3] << 16));
    }
  }
}

__device__ __forceinline__ uint32_t umma_idesc_n(int n) {
  uint32_t d = 0;
  d |= 1u << 4;                        // D format F32
  d |= 1u << 7;                        // A BF16
  d |= 1u << 10;                       // B BF16
  d |= (uint32_t)(n >> 3) << 17;       // N
  d |= (uint32_t)(TC_BM >> 4) << 24;   // M
  return d;
}

struct MlpTcArgs {
  int n_cap;
  const int* d_n;
  const float* b1;         // [128]
  const __nv_bfloat16* w2;  // [64][128]
  const float* b2;         // [64]
  const __nv_bfloat16* w3;  // [64]
  const float* b3;         // [1]
  float* score;            // [n]
  int* status;
  long long spin_limit;
};

__global__ void __launch_bounds__(TC_THREADS, 1) k_mlp_tc(const __grid_constant__ CUtensorMap m_hi,
                                                          const __grid_constant__ CUtensorMap m_mid,
                                                          const __grid_constant__ CUtensorMap m_lo,
                                                          const __grid_constant__ CUtensorMap m_w1, MlpTcArgs a) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ uint64_t full_bar[MLP_TC_STAGES], empty_bar[MLP_TC_STAGES], acc_full, drain_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  __shared__ float s_w2[MLP_TC_H1][MLP_TC_H2];  // [input c][output j]
  __shared__ float s_b1[MLP_TC_H1], s_b2[MLP_TC_H2], s_w3[MLP_TC_H2];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = a.d_n ? min(*a.d_n, a.n_cap) : a.n_cap;
  const int q0 = blockIdx.x * TC_BM;
  if (q0 >= n) return;  // uniform per CTA, before any barrier or TMEM use

  for (int i = threadIdx.x; i < MLP_TC_H1 * MLP_TC_H2; i += blockDim.x) {
    const int j = i / MLP_TC_H1, c = i - j * MLP_TC_H1;  // w2 row-major [j][c]
    s_w2[c][j] = __bfloat162float(a.w2[i]);
  }
  for (int i = threadIdx.x; i < MLP_TC_H1; i += blockDim.x) s_b1[i] = a.b1[i];
  for (int i = threadIdx.x; i < MLP_TC_H2; i += blockDim.x) {
    s_b2[i] = a.b2[i];
    s_w3[i] = __bfloat162float(a.w3[i]);
  }
  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < MLP_TC_STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], 1);
    }
    mbar_init(&acc_full, 1);
    mbar_init(&drain_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 5) {  // 128 TMEM columns: one 128 x 128 FP32 accumulator
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(smem_u32(&tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  volatile int* abort = &abort_flag;
  const long long lim = a.spin_limit;
  int issued = 0;

  if (warp == 4) {
    // ---------------- TMA producer ----------------
    if (lane == 0) {
      int kb = 0;
      for (; kb < TC_NKB && !*abort; ++kb) {
        const int s = kb % MLP_TC_STAGES;
        const uint32_t ph = (uint32_t)(kb / MLP_TC_STAGES) & 1u;
        if (kb >= MLP_TC_STAGES && !mbar_wait(&empty_bar[s], ph ^ 1u, abort, lim)) break;
        uint8_t* st = smem + s * MLP_TC_STAGE_BYTES;
        mbar_expect_tx(&full_bar[s], MLP_TC_STAGE_BYTES);
        tma_load_2d(st, &m_hi, &full_bar[s], kb * TC_KB, q0);
        tma_load_2d(st + MLP_TC_A_BYTES, &m_mid, &full_bar[s], kb * TC_KB, q0);
        tma_load_2d(st + 2 * MLP_TC_A_BYTES, &m_lo, &full_bar[s], kb * TC_KB, q0);
        tma_load_2d(st + 3 * MLP_TC_A_BYTES, &m_w1, &full_bar[s], kb * TC_KB, 0);
      }
      issued = kb;
    }
  } else if (warp == 5) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {
      const uint32_t idesc = umma_idesc_n(MLP_TC_H1);
      bool ok = true;
      for (int kb = 0; kb < TC_NKB; ++kb) {
        const int s = kb % MLP_TC_STAGES;
        const uint32_t ph = (uint32_t)(kb / MLP_TC_STAGES) & 1u;
        if (!mbar_wait(&full_bar[s], ph, abort, lim)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t base = smem_u32(smem + s * MLP_TC_STAGE_BYTES);
        const uint32_t ah = base, am = base + MLP_TC_A_BYTES, al = base + 2 * MLP_TC_A_BYTES,
                       bw = base + 3 * MLP_TC_A_BYTES;
#pragma unroll
        for (int k = 0; k < TC_KB / 16; ++k) {
          const uint32_t off = (uint32_t)k * 32;  // 16 bf16 along K inside the swizzle row
          const uint32_t acc0 = (kb > 0 || k > 0) ? 1u : 0u;
          umma_f16(tmem, umma_desc(ah + off), umma_desc(bw + off), idesc, acc0);
          umma_f16(tmem, umma_desc(am + off), umma_desc(bw + off), idesc, 1u);
          umma_f16(tmem, umma_desc(al + off), umma_desc(bw + off), idesc, 1u);
        }
        umma_commit(&empty_bar[s]);
      }
      if (ok) umma_commit(&acc_full);
    }
  } else {
    // ---------------- epilogue: warps 0-3, thread = row ----------------
    const int row = warp * 32 + lane;
    const int q = q0 + row;
    if (mbar_wait(&acc_full, 0u, abort, lim)) {
      tc_fence_after();
      float h2[MLP_TC_H2];
#pragma unroll
      for (int j = 0; j < MLP_TC_H2; ++j) h2[j] = 0.f;
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
      for (int c0 = 0; c0 < MLP_TC_H1; c0 += 32) {
        float v[32];
        tmem_ld32(taddr + (uint32_t)c0, v);
#pragma unroll 4
        for (int i = 0; i < 32; ++i) {
          const float h = fmaxf(v[i] + s_b1[c0 + i], 0.f);
#pragma unroll
          for (int j = 0; j < MLP_TC_H2; ++j) h2[j] = fmaf(h, s_w2[c0 + i][j], h2[j]);
        }
      }
      float z = 0.f;
#pragma unroll
      for (int j = 0; j < MLP_TC_H2; ++j) z = fmaf(fmaxf(h2[j] + s_b2[j], 0.f), s_w3[j], z);
      z += *a.b3;
      if (q < n) a.score[q] = 1.f / (1.f + __expf(-z));
    }
  }
  __syncthreads();
  if (abort_flag) {
    if (warp == 5 && lane == 0) {
      umma_commit(&drain_bar);
      mbar_drain(&drain_bar, 0u);
    }
    if (warp == 4 && lane == 0)
      for (int i = issued > MLP_TC_STAGES ? issued - MLP_TC_STAGES : 0; i < issued; ++i)
        mbar_drain(&full_bar[i % MLP_TC_STAGES], (uint32_t)(i / MLP_TC_STAGES) & 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (abort_flag && threadIdx.x == 0) atomicExch(a.status, (int)RTR_ERR_TIMEOUT);
  if (warp == 5) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem));
  }
}

size_t mlp_tc_bytes(int n_cap) {
  const size_t nqp = (size_t)(((n_cap > 0 ? n_cap : 1) + TC_BM - 1) / TC_BM) * TC_BM;
  ScratchPlan p;
  for (int i = 0; i < 3; ++i) p.add<__nv_bfloat16>(nqp * TC_KPAD);
  return p.bytes;
}

// Scores of rows X[0 .. *d_n) (n_cap rows of capacity).  w1pad: W1 as BF16
// [128][TC_KPAD] with zero columns past 352; theta_b1/b2/b3: the FP32 biases.
rtr_status mlp_tc_score(rtr_context* ctx, Scratch& s, const float* X, int n_cap, const int* d_n,
                        const __nv_bfloat16* w1pad, const float* b1, const __nv_bfloat16* w2, const float* b2,
                        const __nv_bfloat16* w3, const float* b3, float* score, cudaStream_t st) {
  if (n_cap <= 0) return RTR_OK;
  const int nqp = ((n_cap + TC_BM - 1) / TC_BM) * TC_BM;
  __nv_bfloat16* hi = s.take<__nv_bfloat16>((size_t)nqp * TC_KPAD);
  __nv_bfloat16* mid = s.take<__nv_bfloat16>((size_t)nqp * TC_KPAD);
  __nv_bfloat16* lo = s.take<__nv_bfloat16>((size_t)nqp * TC_KPAD);
  if (!lo) return fail(RTR_ERR_CAPACITY, "mlp_tc: scratch");
  int sb = (nqp + 7) / 8;
  if (sb > 152 * 16) sb = 152 * 16;
  k_split3_bf16<<<sb, 256, 0, st>>>(X, n_cap, d_n, nqp, hi, mid, lo);
  CUtensorMap mh, mm, ml, mw;
  if (!make_map(&mh, hi, nqp, TC_BM) || !make_map(&mm, mid, nqp, TC_BM) || !make_map(&ml, lo, nqp, TC_BM) ||
      !make_map(&mw, w1pad, MLP_TC_H1, MLP_TC_H1))
    return fail(RTR_ERR_CUDA, "mlp_tc: cuTensorMapEncodeTiled failed");
  RTR_CUDA(cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, MLP_TC_SMEM));
  MlpTcArgs a{n_cap, d_n, b1, w2, b2, w3, b3, score, ctx->d_status, tc_spin_limit(ctx)};
  k_mlp_tc<<<nqp / TC_BM, TC_THREADS, MLP_TC_SMEM, st>>>(mh, mm, ml, mw, a);
  RTR_LAUNCHED(2);
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

}  // namespace rtr

using namespace rtr;

extern "C" rtr_status rtr_match_stats(rtr_context* ctx, int* h_uncertified) {
  RTR_CHECK_ARG(ctx && h_uncertified, "rtr_match_stats: bad arguments");
  RTR_CUDA(cudaSetDevice(ctx->device));
  RTR_CUDA(cudaDeviceSynchronize());
  RTR_CUDA(cudaMemcpy(h_uncertified, ctx->d_status + 8, sizeof(int), cudaMemcpyDeviceToHost));
  return RTR_OK;
}

extern "C" rtr_status rtr_match_stats_ex(rtr_context* ctx, int* h_uncertified, int* h_full_scans) {
  RTR_CHECK_ARG(ctx && h_uncertified && h_full_scans, "rtr_match_stats_ex: bad arguments");
  RTR_CUDA(cudaSetDevice(ctx->device));
  RTR_CUDA(cudaDeviceSynchronize());
  int h[2];
  RTR_CUDA(cudaMemcpy(h, ctx->d_status + 8, sizeof(h), cudaMemcpyDeviceToHost));
  *h_uncertified = h[0];
  *h_full_scans = h[1];
  return RTR_OK;
}

extern "C" rtr_status rtr_match(rtr_context* ctx, const float* d_query, int n_query, const float* d_db, int n_db,
                                int32_t* d_idx, float* d_d2, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n_query >= 0 && n_db >= 0, "rtr_match: bad arguments");
  if (n_query == 0) return RTR_OK;
  RTR_CHECK_ARG(d_query && d_idx, "rtr_match: NULL query or output");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (n_db == 0) {
    RTR_CUDA(cudaMemsetAsync(d_idx, 0xff, (size_t)n_query * 4, st));
    return RTR_OK;
  }
  RTR_CHECK_ARG(d_db != nullptr, "rtr_match: NULL database");
  ScratchPlan p;
  match_tc_plan(p, n_query, true, n_db);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, p.bytes, st, &s));
  ProfScope ps(ctx, st, "match_tc");
  return match_tc_dev(ctx, s, d_query, n_query, nullptr, d_db, n_db, nullptr, nullptr, nullptr, d_idx, d_d2, st);
}
