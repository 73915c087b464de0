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
constexpr int GC_MAXS = 128;  // members of a set staged in shared memory (the rest are read from set_mem)
// Members stored per consensus set: every member while C rows of C fit in
// GC_SET_BUDGET bytes, else as many as fit, never fewer than GC_MAXS (a set
// beyond the stride: RTR_ERR_CAPACITY).
constexpr size_t GC_SET_BUDGET = (size_t)128 << 20;
inline int gc_set_stride(int C) {
  const long long n = C > 0 ? C : 1;
  const long long by_budget = (long long)(GC_SET_BUDGET / sizeof(int)) / n;
  const long long m = n < by_budget ? n : by_budget;
  return (int)(m > GC_MAXS ? m : GC_MAXS);
}

struct GcDev {
  const float4* pm;        // model keypoint of sorted correspondence a
  const float4* ps;        // scene keypoint of sorted correspondence a
  int C;                   // correspondences (the capacity when d_C is set)
  const int* d_C;          // device count of correspondences, or NULL
  float gc;
  unsigned* taken;         // bitset over sorted positions
  int* set_size;           // [C]
  int* set_mem;            // [C][maxs] sorted positions
  int maxs;                // members stored per set (gc_set_stride)
};

__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// The consistency test of the oracle, !(|sqrt(dm2) - sqrt(ds2)| > gc) with
// IEEE square roots, answered without them when the answer is certain:
//  - ds2 > r2max: the scene distance exceeds the largest model distance plus
//    gc (r2max carries a relative margin far above the rounding of both
//    sides), so the test fails;
//  - |sqrt u - sqrt v| = |u - v| / (sqrt u + sqrt v) >= |u - v| / (2 sqrt(max(u, v))),
//    so (u - v)^2 > 4.004 gc^2 max(u, v) fails the test with a 0.05 % margin
//    on gc; while gc >= 1e-3 sqrt(max(u, v)) that margin is far above the
//    rounding of the roots, their difference and this bound (< 2e-4 gc);
//  - otherwise approximate roots (relative error far below 1e-5) decide
//    unless |a - b| lies within 1e-5 (a + b) + 1e-6 of gc, where the exact
//    form runs.  NaN differences fall through to the exact form.
__device__ __forceinline__ bool gc_consistent(float4 am, float4 as, float4 bm, float4 bs, float gc, float r2max) {
  const float v = dist2_exact(as, bs);
  if (v > r2max) return false;
  const float u = dist2_exact(am, bm);
  const float duv = u - v, m = fmaxf(u, v), gc2 = gc * gc;
  if (gc2 >= 1.0e-6f * m && duv * duv > 4.004f * gc2 * m) return false;
  const float a = sqrt_approx(u), b = sqrt_approx(v);
  const float diff = fabsf(a - b);
  const float tol = 1.0e-5f * (a + b) + 1.0e-6f;
  if (diff > gc + tol) return false;
  if (diff < gc - tol) return true;
  return !(fabsf(__fsub_rn(__fsqrt_rn(u), __fsqrt_rn(v))) > gc);
}

// Spatial pruning of the seed tests.  A candidate b passes seed a only if
// |d_model(a, b) - d_scene(a, b)| <= gc, and d_model(a, b) is at most F_a,
// the distance from a's model endpoint to the farthest corner of the model
// endpoints' box; so every passing b has its scene endpoint within
// R_a = F_a + gc of a's.  The candidates are sorted by a coarse cell of
// their scene endpoint, cut into chunks of 32 and each chunk given the exact
// box of its endpoints; a seed skips every chunk whose box lies farther than
// R_a (plus a slack far above the rounding of every quantity involved) and
// tests the others' candidates as before, so the pass bits are the same as
// testing every candidate.  A chunk holding a point with a non-finite
// coordinate is never skipped.
struct GcGrid {
  GridMeta m;     // box of the scene endpoints, origin, cell edge, dims, ncells
  float mlo[3], mhi[3];  // box of the model endpoints
  float slack;    // metres added to every reach
};
constexpr unsigned GC_GRID_CELLS = 1u << 15;

__device__ __forceinline__ int gcg_cell(float v, float o, float inv_h, int n) {
  float f = __fmul_rn(__fsub_rn(v, o), inv_h);
  f = fminf(fmaxf(f, -1.0e8f), 1.0e8f);
  const int c = (int)floorf(f);
  return c < 0 ? 0 : (c > n - 1 ? n - 1 : c);
}

// Cell edge an eighth of the largest reach (model box diagonal + gc), grown
// until the scene endpoints' box needs at most GC_GRID_CELLS cells.
__global__ void k_gcg_setup(GcGrid* gg, const GridMeta* __restrict__ mbox, float gc, int C_host, const int* d_C) {
  if (threadIdx.x != 0) return;
  const int n = d_C ? min(*d_C, C_host) : C_host;
  GridMeta& m = gg->m;
  float lo[3], hi[3];
  double diag2 = 0.0, mag = 0.0;
  for (int a = 0; a < 3; ++a) {
    lo[a] = n > 0 ? ordered_to_float(m.bmin[a]) : 0.f;
    hi[a] = n > 0 ? ordered_to_float(m.bmax[a]) : 0.f;
    if (!isfinite(lo[a]) || !isfinite(hi[a]) || !(hi[a] >= lo[a])) {
      lo[a] = isfinite(lo[a]) ? lo[a] : (isfinite(hi[a]) ? hi[a] : 0.f);
      hi[a] = isfinite(hi[a]) && hi[a] >= lo[a] ? hi[a] : lo[a];
    }
    const float ml = n > 0 ? ordered_to_float(mbox->bmin[a]) : 0.f;
    const float mh = n > 0 ? ordered_to_float(mbox->bmax[a]) : 0.f;
    gg->mlo[a] = ml;
    gg->mhi[a] = mh;
    const double e = (double)mh - (double)ml;
    diag2 += e * e;
    mag = fmax(mag, fmax(fmax(fabs((double)lo[a]), fabs((double)hi[a])), fmax(fabs((double)ml), fabs((double)mh))));
  }
  const double R = sqrt(diag2) + (double)gc;
  double h = R / 8.0;
  if (!(h > 1.0e-4) || !(h < 1.0e15)) h = !(h < 1.0e15) ? 1.0e15 : 1.0e-4;
  int dims[3] = {1, 1, 1};
  bool fits = false;
  for (int tries = 0; tries < 64 && !fits; ++tries) {
    double cells = 1.0;
    for (int a = 0; a < 3; ++a) {
      double e = floor(((double)hi[a] - (double)lo[a]) / h) + 1.0;
      if (e > 2.0e9) e = 2.0e9;
      dims[a] = (int)e;
      cells *= e;
    }
    if (cells <= (double)GC_GRID_CELLS) fits = true;
    else h = h * cbrt(cells / (double)GC_GRID_CELLS) * 1.001;
  }
  if (!fits) {  // one cell: the order is the sorted order, boxes stay exact
    dims[0] = dims[1] = dims[2] = 1;
    h = 1.0e15;
  }
  const float hf = (float)h;
  m.ox = lo[0];
  m.oy = lo[1];
  m.oz = lo[2];
  m.h = hf;
  m.inv_h = 1.0f / hf;
  m.nx = dims[0];
  m.ny = dims[1];
  m.nz = dims[2];
  m.n = n;
  m.ncells = (unsigned)dims[0] * (unsigned)dims[1] * (unsigned)dims[2];
  const double slack = 1.0e-4 + 1.0e-5 * (R + mag);
  gg->slack = (float)(slack < 1.0e30 ? slack : 1.0e30);
}

__global__ void __launch_bounds__(256) k_gcg_keys(const float4* __restrict__ ps, int C_host, const int* d_C,
                                                  const GcGrid* __restrict__ gg, uint32_t* __restrict__ keys) {
  const int n = d_C ? min(*d_C, C_host) : C_host;
  const GridMeta& m = gg->m;
  const float ox = m.ox, oy = m.oy, oz = m.oz, ih = m.inv_h;
  const int nx = m.nx, ny = m.ny, nz = m.nz;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = ps[i];
    if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) {
      keys[i] = m.ncells;
      continue;
    }
    const int cx = gcg_cell(p.x, ox, ih, nx), cy = gcg_cell(p.y, oy, ih, ny), cz = gcg_cell(p.z, oz, ih, nz);
    keys[i] = ((uint32_t)cz * (uint32_t)ny + (uint32_t)cy) * (uint32_t)nx + (uint32_t)cx;
  }
}

// Candidates in cell order (w = sorted position) and, per chunk of 32, the
// box of their scene endpoints (lo.w = 1 when the chunk holds a non-finite
// point).  Block size a multiple of 32: each warp covers whole chunks.
__global__ void __launch_bounds__(256) k_gcg_gather(const float4* __restrict__ ps, const float4* __restrict__ pm,
                                                    const uint32_t* __restrict__ order, int C_host, const int* d_C,
                                                    float4* __restrict__ cpts, float4* __restrict__ cpm,
                                                    float4* __restrict__ cbox) {
  const int n = d_C ? min(*d_C, C_host) : C_host;
  const int lane = threadIdx.x & 31;
  const int stride = gridDim.x * blockDim.x;
  for (int i0 = blockIdx.x * blockDim.x + (threadIdx.x & ~31); i0 < n; i0 += stride) {
    const int i = i0 + lane;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    int nf = 0;
    if (i < n) {
      const uint32_t o = order[i];
      float4 p = ps[o];
      if (isfinite(p.x) && isfinite(p.y) && isfinite(p.z)) {
        lo[0] = hi[0] = p.x;
        lo[1] = hi[1] = p.y;
        lo[2] = hi[2] = p.z;
      } else {
        nf = 1;
      }
      p.w = __int_as_float((int)o);
      cpts[i] = p;
      cpm[i] = pm[o];
    }
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], off));
        hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], off));
      }
    nf = __any_sync(0xffffffffu, nf);
    if (lane == 0) {
      cbox[2 * (i0 >> 5)] = make_float4(lo[0], lo[1], lo[2], nf ? 1.f : 0.f);
      cbox[2 * (i0 >> 5) + 1] = make_float4(hi[0], hi[1], hi[2], 0.f);
    }
  }
}

// Device-side control block of the grouping walk.
struct GcCoop {
  int* ctl;            // [0] walk position, [1] clusters, [2] done, [3] error status, [4] rounds,
                       // [5] sets computed, [6] seeds needing a set this round,
                       // [7] candidates that passed a seed test (summed over sets),
                       // [8..11] microseconds in phases P, A1, A2, B (block 0's view),
                       // [12] the next round's window (0: the first window),
                       // [13] pass-list pool entries handed out
  unsigned* arrive;    // grid barrier counter (zero at launch)
  int* computed;       // [C] 1 once the seed's set has been computed
  int* cl_members;     // [max_clusters][maxs] sorted positions
  int* cl_sizes;       // [max_clusters]
  int thresh, max_clusters;
  long long budget;    // clock64 cycles per barrier wait
  int* status;         // context status word
  const GridMeta* mbox;  // bounding box of the model endpoints
  int* need;           // [win] seeds whose set is computed this round
  unsigned* mask;      // [win][nwp] seed-test pass bits, one row per needed seed
  int win;             // seeds in the first window
  int win_max;         // seeds a window may grow to (the need/mask capacity)
  int nwp;             // words per mask row (C/32 rounded up to a multiple of 4)
  const GcGrid* sg;    // pruning constants (model box, slack)
  const float4* cpts;  // scene endpoints sorted by coarse cell; w = sorted position (int bits)
  const float4* cpm;   // model endpoints in the same order
  const float4* cbox;  // [chunks][2] box of each chunk of 32 cpts (lo.w = 1: holds a non-finite point)
  float4* seed_s;      // [win_max] listed seed's scene endpoint, w = its reach (+inf: unbounded)
  float4* seed_m;      // [win_max] listed seed's model endpoint
  int* pcnt;           // [win_max] seed-test passes of each listed seed
  int* plist_off;      // [C] start of the seed's pass list in pool (-1: none kept)
  int* plist_cnt;      // [C] length of the seed's pass list
  float4* pool_m;      // pass lists in ascending sorted position: model endpoint (w = position bits)
  float4* pool_s;      // ... and scene endpoint
  int pool_cap;        // entries (0: no lists kept)
  int inline_max;      // sets the walk recomputes in place per round before it ends the round
};

__device__ __forceinline__ bool sbit(const unsigned* s, int i) { return (s[i >> 5] >> (i & 31)) & 1u; }
__device__ __forceinline__ uint32_t smem_u32_gc(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

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

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ float4 shfl4(float4 v, int src) {
  return make_float4(__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src),
                     __shfl_sync(0xffffffffu, v.z, src), __shfl_sync(0xffffffffu, v.w, src));
}

constexpr int GC_PEND = 64;  // candidates staged per warp before admission
constexpr int GC_PREF = 7;   // mask loads in flight per lane during admission

// Greedy admission of the n (<= 32) staged candidates, in slot order, into
// the warp's set (members in mem_m/mem_s; member 0 is the seed, which every
// staged candidate already passed).  Lane k tests candidate k against the
// members so far in parallel; then, lowest lane first, the next passing
// candidate is admitted and every later candidate is also tested against
// it.  Same result as admitting one candidate at a time.
template <bool LONG>
__device__ __forceinline__ void gc_admit(const GcDev& g, int a, const int* slot, int n, float4* mem_m,
                                         float4* mem_s, int& cnt, float r2max, int* n_tested, float4* list_m,
                                         float4* list_s, int list_len) {
  const int lane = threadIdx.x & 31;
  const int pj = lane < n ? slot[lane] : -1;
  float4 cm = make_float4(0, 0, 0, 0), cs = cm;
  if (pj >= 0) {
    cm = __ldg(g.pm + pj);
    cs = __ldg(g.ps + pj);
    if (list_m && *n_tested + lane < list_len) {  // the pass list entry: endpoints, position in w
      list_m[*n_tested + lane] = make_float4(cm.x, cm.y, cm.z, __int_as_float(pj));
      list_s[*n_tested + lane] = cs;
    }
  }
  *n_tested += n;
  bool pass = pj >= 0;
  const int maxs = LONG ? g.maxs : GC_MAXS;
  const int stored = min(cnt, maxs);
  const int staged = min(stored, GC_MAXS);
  for (int m = 1; m < staged; ++m) {
    if (pass) pass = gc_consistent(mem_m[m], mem_s[m], cm, cs, g.gc, r2max);
    if ((m & 3) == 0 && !__any_sync(0xffffffffu, pass)) break;
  }
  // members past the shared-memory stage, read through set_mem
  if (LONG)
    for (int m = GC_MAXS; m < stored && __any_sync(0xffffffffu, pass); ++m) {
      const int pb = __ldcg(g.set_mem + (size_t)a * maxs + m);
      if (pass) pass = gc_consistent(__ldg(g.pm + pb), __ldg(g.ps + pb), cm, cs, g.gc, r2max);
    }
  unsigned bal = __ballot_sync(0xffffffffu, pass);
  while (bal) {
    const int f = __ffs(bal) - 1;
    const float4 fm = shfl4(cm, f), fs = shfl4(cs, f);
    if (lane == f && cnt < maxs) {
      if (cnt < GC_MAXS) {
        mem_m[cnt] = cm;
        mem_s[cnt] = cs;
      }
      g.set_mem[(size_t)a * maxs + cnt] = pj;
    }
    ++cnt;  // counted beyond the stride too: reported by the walk
    if (lane > f && pass) pass = gc_consistent(fm, fs, cm, cs, g.gc, r2max);
    if (lane <= f) pass = false;
    bal = __ballot_sync(0xffffffffu, pass);
  }
  __syncwarp();
}

// The consensus set of seed a under the current taken bits, from a's pass
// list (entries in ascending sorted position that passed a's seed test when
// it was computed; a superset of the ones not taken now): greedy admission in
// list order, candidates taken since skipped, each candidate tested against
// every member so far (member 0 is the seed).  Members go to rec[]
// (positions) and mem_m/mem_s.  Returns the member count, or -1 when the set
// would exceed cap (the caller falls back to a recompute in the next round).
__device__ __forceinline__ int gc_inline_set(const GcDev& g, int a, const float4* lm, const float4* ls, int nl,
                                             const unsigned* taken, float4* mem_m, float4* mem_s, int* rec, int cap,
                                             float r2max) {
  const int lane = threadIdx.x & 31;
  if (lane == 0) {
    mem_m[0] = __ldg(g.pm + a);
    mem_s[0] = __ldg(g.ps + a);
    rec[0] = a;
  }
  __syncwarp();
  int cnt = 1;
  float4 nm = make_float4(0.f, 0.f, 0.f, 0.f), ns = nm;
  if (lane < nl) {
    nm = __ldcg(lm + lane);
    ns = __ldcg(ls + lane);
  }
  for (int i0 = 0; i0 < nl; i0 += 32) {
    const bool have = i0 + lane < nl;
    const float4 cm = nm, cs = ns;
    if (i0 + 32 + lane < nl) {  // the next chunk's entries in flight during this one
      nm = __ldcg(lm + i0 + 32 + lane);
      ns = __ldcg(ls + i0 + 32 + lane);
    }
    const int b = have ? __float_as_int(cm.w) : -1;
    bool pass = have && !sbit(taken, b);
    // the member tests are independent: no early exit, so they overlap
#pragma unroll 4
    for (int m = 1; m < cnt; ++m) pass &= gc_consistent(mem_m[m], mem_s[m], cm, cs, g.gc, r2max);
    unsigned bal = __ballot_sync(0xffffffffu, pass);
    while (bal) {
      const int f = __ffs(bal) - 1;
      if (cnt >= cap) return -1;
      const float4 fm = shfl4(cm, f), fs = shfl4(cs, f);
      if (lane == f) {
        mem_m[cnt] = cm;
        mem_s[cnt] = cs;
        rec[cnt] = b;
      }
      ++cnt;
      if (lane > f && pass) pass = gc_consistent(fm, fs, cm, cs, g.gc, r2max);
      if (lane <= f) pass = false;
      bal = __ballot_sync(0xffffffffu, pass);
    }
    __syncwarp();
  }
  return cnt;
}

// The whole grouping in one cooperative launch.  Each round:
//  P. warps check the seeds of the window [pos, pos + win): a seed that is
//     not taken and has no set yet, or whose set lost a member to a commit,
//     joins this round's list;
//  A1. seed tests of every listed seed against every candidate, spread over
//     all warps (a warp stages 32 candidates once and tests them against
//     its group's 32 seeds, one seed per lane); the results are pass
//     bitmasks in candidate order;
//  A2. one warp per listed seed admits the passing candidates in ascending
//     order, greedily, against the members so far;
//  B.  warp 0 of block 0 walks the seeds in order from pos: taken seeds are
//     skipped, a seed whose set lost a member ends the round (recomputed in
//     the next one), a set of >= thresh members commits.  The walk also ends
//     at the window's end, at the last seed, or at max_clusters.
// A stored set stays exact while none of its members is taken (removing
// rejected candidates never changes a greedy walk).  Every round advances the
// walk by at least one seed (the seed at pos is exact when B starts).
// LONG: sets may be stored past GC_MAXS members (g.maxs > GC_MAXS); false
// compiles the fixed GC_MAXS stride.
template <bool LONG>
__global__ void __launch_bounds__(GC_WARPS * 32, 2) k_gc_coop(GcDev g, GcCoop c) {
  const int maxs = LONG ? g.maxs : GC_MAXS;
  extern __shared__ unsigned s_taken[];  // copy of the taken bitset
  __shared__ float4 mem_m[GC_WARPS][GC_MAXS], mem_s[GC_WARPS][GC_MAXS];
  __shared__ int s_slot[GC_WARPS][GC_PEND];
  __shared__ int s_rec[GC_MAXS];  // walk: members of a set recomputed in place
  __shared__ int s_pf[3][32][9];  // walk: sizes and first 8 members of the next batches (cp.async ring)
  __shared__ int s_pos, s_done, s_ok, s_win;
  __shared__ float s_r2max;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (g.d_C) g.C = min(max(*g.d_C, 0), g.C);  // counted on the device
  const int nwords = (g.C + 31) >> 5;
  const int nwp = (nwords + 3) & ~3;  // live width of a mask row (rows are c.nwp apart)
  const int gw = blockIdx.x * GC_WARPS + wid, nwarps = gridDim.x * GC_WARPS;
  if (threadIdx.x == 0) {
    s_pos = 0;
    s_win = c.win;
    s_done = 0;
    // largest model-side distance: the diagonal of the endpoints' box
    float d2 = 0.f;
    for (int k = 0; k < 3; ++k) {
      const float e = ordered_to_float(c.mbox->bmax[k]) - ordered_to_float(c.mbox->bmin[k]);
      d2 += e * e;
    }
    const float R = (sqrtf(d2) + g.gc) * 1.0001f + 1.0e-5f;
    const float r2 = R * R * 1.0001f;
    s_r2max = r2 < 3.0e38f ? r2 : __int_as_float(0x7f800000);
  }
  __syncthreads();
  const float r2max = s_r2max;
  unsigned target = 0;
  unsigned long long ph[4] = {0, 0, 0, 0}, tp = 0;
  const bool timer = blockIdx.x == 0 && threadIdx.x == 0;
  if (timer) tp = gtimer();
#define GC_PHASE(k)                            \
  if (timer) {                                 \
    const unsigned long long tn_ = gtimer();   \
    ph[k] += tn_ - tp;                         \
    tp = tn_;                                  \
  }
  for (int round = 0;; ++round) {
    __syncthreads();
    for (int i = threadIdx.x; i < nwords; i += blockDim.x) s_taken[i] = __ldcg(g.taken + i);
    __syncthreads();
    const int pos = s_pos;
    // ---- P: seeds that need a set this round
    const int win = s_win;
    for (int t = gw; t < win; t += nwarps) {
      const int a = pos + t;
      bool need = false;
      if (a < g.C && !sbit(s_taken, a)) {
        if (!__ldcg(c.computed + a)) {
          need = true;
        } else {
          const int n = min(__ldcg(g.set_size + a), maxs);
          bool st = false;
          for (int k = lane; k < n; k += 32) st |= sbit(s_taken, __ldcg(g.set_mem + (size_t)a * maxs + k));
          need = __any_sync(0xffffffffu, st);
        }
      }
      int slot = 0;
      if (need && lane == 0) {
        slot = atomicAdd(c.ctl + 6, 1);
        c.need[slot] = a;
        c.pcnt[slot] = 0;
        // reach: farthest corner of the model box from a's model endpoint, plus gc
        const float4 am = __ldg(g.pm + a), as = __ldg(g.ps + a);
        const float fx = fmaxf(fabsf(am.x - c.sg->mlo[0]), fabsf(c.sg->mhi[0] - am.x));
        const float fy = fmaxf(fabsf(am.y - c.sg->mlo[1]), fabsf(c.sg->mhi[1] - am.y));
        const float fz = fmaxf(fabsf(am.z - c.sg->mlo[2]), fabsf(c.sg->mhi[2] - am.z));
        float R = sqrtf(fx * fx + fy * fy + fz * fz) * 1.00001f + g.gc + c.sg->slack;
        R = R < 1.0e18f ? R * R : __int_as_float(0x7f800000);  // NaN reach: unbounded
        c.seed_s[slot] = make_float4(as.x, as.y, as.z, R);
        c.seed_m[slot] = am;
      }
      // the seed tests only set bits: its mask row starts clear
      slot = __shfl_sync(0xffffffffu, slot, 0);
      if (need) {
        uint4* row = reinterpret_cast<uint4*>(c.mask + (size_t)slot * c.nwp);
        for (int v = lane; v < (nwp >> 2); v += 32) row[v] = make_uint4(0u, 0u, 0u, 0u);
      }
    }
    target += gridDim.x;
    if (!gc_barrier(c, target, &s_ok)) return;
    GC_PHASE(0)
    const int nneed = __ldcg(c.ctl + 6);
    // ---- A1: seed tests -> pass bitmasks.  Items are (chunk of 32
    // candidates in cell order, group of 32 listed seeds), spread over all
    // warps (a chunk near many seeds is shared by as many warps as it has
    // seed groups).  Lane k holds candidate k of the chunk and seed k of the
    // group; the group's seeds whose reach meets the chunk's box are taken in
    // turn, and every lane tests its candidate against each, setting its pass
    // bit in the seed's row.
    if (nneed > 0) {
      const int nchunks = (g.C + 31) >> 5;
      const int ngroups = (nneed + 31) >> 5;
      const long long items = (long long)nchunks * ngroups;
      for (long long it = gw; it < items; it += nwarps) {
        const int ch = (int)(it / ngroups);
        const int s0 = (int)(it - (long long)ch * ngroups) * 32;
        const int i = ch * 32 + lane, k = s0 + lane;
        float4 q = make_float4(0.f, 0.f, 0.f, 0.f), bm = q, sa = q, sm = q;
        int sa_i = -1;
        if (i < g.C) {
          q = __ldg(c.cpts + i);
          bm = __ldg(c.cpm + i);
        }
        if (k < nneed) {
          sa = __ldcg(c.seed_s + k);
          sm = __ldcg(c.seed_m + k);
          sa_i = __ldcg(c.need + k);
        }
        const float4 blo = __ldg(c.cbox + 2 * ch), bhi = __ldg(c.cbox + 2 * ch + 1);
        const int b = i < g.C ? __float_as_int(q.w) : -1;
        const bool ok = b >= 0 && !sbit(s_taken, b);
        if (!__any_sync(0xffffffffu, ok)) continue;
        bool hit = false;
        if (k < nneed) {
          const float dx = fmaxf(fmaxf(blo.x - sa.x, sa.x - bhi.x), 0.f);
          const float dy = fmaxf(fmaxf(blo.y - sa.y, sa.y - bhi.y), 0.f);
          const float dz = fmaxf(fmaxf(blo.z - sa.z, sa.z - bhi.z), 0.f);
          hit = blo.w != 0.f || !(dx * dx + dy * dy + dz * dz > sa.w);  // NaN distance: not skipped
        }
        const unsigned bit = 1u << (b & 31);
        const int word = b >> 5;
        unsigned hits = __ballot_sync(0xffffffffu, hit);
        while (hits) {
          const int f = __ffs(hits) - 1;
          hits &= hits - 1;
          const float4 fa = shfl4(sa, f), fm = shfl4(sm, f);
          const int a = __shfl_sync(0xffffffffu, sa_i, f);
          const bool pass = ok && b != a && gc_consistent(fm, fa, bm, q, g.gc, r2max);
          const unsigned pb = __ballot_sync(0xffffffffu, pass);
          if (pass) atomicOr(c.mask + (size_t)(s0 + f) * c.nwp + word, bit);
          if (lane == 0 && pb) atomicAdd(c.pcnt + s0 + f, __popc(pb));
        }
      }
    }
    target += gridDim.x;
    if (!gc_barrier(c, target, &s_ok)) return;
    GC_PHASE(1)
    // ---- A2: ordered admission, warp per listed seed
    for (int slot = gw; slot < nneed; slot += nwarps) {
      const int a = __ldcg(c.need + slot);
      if (lane == 0) {
        mem_m[wid][0] = __ldg(g.pm + a);
        mem_s[wid][0] = __ldg(g.ps + a);
        g.set_mem[(size_t)a * maxs] = a;
      }
      __syncwarp();
      int cnt = 1, npend = 0, ntest = 0;
      // the seed's pass list (ascending) is kept for the walk, which
      // recomputes a set that lost a member from it
      int n_list = 0, off = -1;
      if (lane == 0) {
        n_list = __ldcg(c.pcnt + slot);
        off = atomicAdd(c.ctl + 13, n_list);
        if (off < 0 || (long long)off + n_list > (long long)c.pool_cap) off = -1;
      }
      n_list = __shfl_sync(0xffffffffu, n_list, 0);
      off = __shfl_sync(0xffffffffu, off, 0);
      int nemit = 0;
      float4* lmp = off >= 0 ? c.pool_m + off : nullptr;
      float4* lsp = off >= 0 ? c.pool_s + off : nullptr;
      const uint4* row = reinterpret_cast<const uint4*>(c.mask + (size_t)slot * c.nwp);
      const int nv = nwp >> 2;
      for (int v0 = 0; v0 < nv; v0 += 32 * GC_PREF) {
        uint4 buf[GC_PREF];
#pragma unroll
        for (int j = 0; j < GC_PREF; ++j) {
          const int idx = v0 + j * 32 + lane;
          buf[j] = idx < nv ? __ldcg(row + idx) : make_uint4(0u, 0u, 0u, 0u);
        }
#pragma unroll
        for (int j = 0; j < GC_PREF; ++j) {
          const int w0 = (v0 + j * 32) * 4;  // first word of this 128-word block
          unsigned wv[4] = {buf[j].x, buf[j].y, buf[j].z, buf[j].w};
          int rc = __popc(wv[0]) + __popc(wv[1]) + __popc(wv[2]) + __popc(wv[3]);
          while (__any_sync(0xffffffffu, rc > 0)) {
            int incl = rc;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
              const int y = __shfl_up_sync(0xffffffffu, incl, o);
              if (lane >= o) incl += y;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            const int ex = incl - rc;
            const int room = GC_PEND - npend;
            // lanes whose lower neighbours all fit emit their first candidates
            int take = min(max(room - ex, 0), rc);
            int dst = npend + ex;
            for (int q = 0; q < 4 && take > 0; ++q) {
              while (wv[q] && take > 0) {
                const int bit = __ffs(wv[q]) - 1;
                wv[q] &= wv[q] - 1;
                s_slot[wid][dst++] = (w0 + lane * 4 + q) * 32 + bit;
                --take;
                --rc;
              }
            }
            nemit += min(total, room);
            npend += min(total, room);
            __syncwarp();
            while (npend >= 32) {
              gc_admit<LONG>(g, a, s_slot[wid], 32, mem_m[wid], mem_s[wid], cnt, r2max, &ntest, lmp, lsp, n_list);
              const int rest = npend - 32;
              const int mv = lane < rest ? s_slot[wid][32 + lane] : 0;
              __syncwarp();
              if (lane < rest) s_slot[wid][lane] = mv;
              npend = rest;
              __syncwarp();
            }
          }
        }
      }
      if (npend > 0) gc_admit<LONG>(g, a, s_slot[wid], npend, mem_m[wid], mem_s[wid], cnt, r2max, &ntest, lmp, lsp, n_list);
      if (lane == 0) {
        c.plist_off[a] = (nemit == n_list && ntest == n_list) ? off : -1;
        c.plist_cnt[a] = n_list;
        g.set_size[a] = cnt;
        c.computed[a] = 1;
        atomicAdd(c.ctl + 5, 1);
        atomicAdd(c.ctl + 7, ntest);
      }
      __syncwarp();
    }
    target += gridDim.x;
    if (!gc_barrier(c, target, &s_ok)) return;
    GC_PHASE(2)
    // ---- B: the ordered walk, 32 seeds per batch.  Lane l evaluates seed
    // p + l (taken? lost a member?) in parallel; only events (a commit or a
    // stale set) are handled in order, and after a commit the later lanes
    // evaluate again.
    if (blockIdx.x == 0 && wid == 0) {
      int ncl = __ldcg(c.ctl + 1), err = 0, n_inline = 0;
      bool done = false, stop = false;
      int p = pos;
      const int wend = min(pos + win, g.C);
      // each lane's seed size and first 8 members are copied two batches
      // ahead into a 3-slot shared-memory ring with cp.async (a slot past the
      // set holds a stale member, which the size masks): they do not change
      // during the walk (only the taken bits do), and the walk goes on to
      // the next batch of 32 only as a whole
      auto prefetch = [&](int pb, int slot) {
        if (pb + lane < wend) {
          const int* src = g.set_mem + (size_t)(pb + lane) * maxs;
#pragma unroll
          for (int k = 0; k < 8; ++k)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32_gc(&s_pf[slot][lane][k])),
                         "l"(src + k)
                         : "memory");
          asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32_gc(&s_pf[slot][lane][8])),
                       "l"(g.set_size + pb + lane)
                       : "memory");
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
      };
      int ring = 0;
      prefetch(p, 0);
      prefetch(p + 32, 1);
      while (p < wend && !stop) {
        const int nb = min(32, wend - p);
        const int my = p + lane;
        prefetch(p + 64, (ring + 2) % 3);
        asm volatile("cp.async.wait_group 2;" ::: "memory");  // this batch's copies are in
        __syncwarp();
        const bool have = lane < nb;
        const int n_l = have ? s_pf[ring][lane][8] : 0;
        int m_cur[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) m_cur[k] = s_pf[ring][lane][k];
        ring = ring == 2 ? 0 : ring + 1;
        const int ns_l = min(n_l, maxs);
        int cursor = 0;
        for (;;) {
          bool taken_l = true, stale_l = false;
          if (lane >= cursor && lane < nb) {
            taken_l = sbit(s_taken, my);
            if (!taken_l) {
              // the first 8 members' taken bits in one round of independent
              // shared-memory loads (a slot past the set reads the seed's own
              // bit: clear)
              unsigned acc = 0u;
#pragma unroll
              for (int k = 0; k < 8; ++k) {
                const int mb = k < ns_l ? m_cur[k] : my;
                acc |= s_taken[mb >> 5] >> (mb & 31);
              }
              stale_l = (acc & 1u) != 0u;
              // a longer set: its other members eight independent loads at a time
              for (int k0 = 8; k0 < ns_l && !stale_l; k0 += 8) {
                int mbk[8];
#pragma unroll
                for (int j = 0; j < 8; ++j)
                  mbk[j] = k0 + j < ns_l ? __ldcg(g.set_mem + (size_t)my * maxs + k0 + j) : my;
                unsigned a2 = 0u;
#pragma unroll
                for (int j = 0; j < 8; ++j) a2 |= s_taken[mbk[j] >> 5] >> (mbk[j] & 31);
                stale_l = (a2 & 1u) != 0u;
              }
            }
          }
          const unsigned ev = __ballot_sync(0xffffffffu, !taken_l && (stale_l || n_l >= c.thresh));
          if (!ev) {
            p += nb;
            break;
          }
          const int f = __ffs(ev) - 1;
          const bool f_stale = __shfl_sync(0xffffffffu, stale_l, f);
          const int nf = __shfl_sync(0xffffffffu, n_l, f);
          if (f_stale) {
            // lost a member: recompute in place from the pass list, or
            // (no list kept, or too many members) end the round here
            const int sa = p + f;
            const int off = n_inline < c.inline_max ? __ldcg(c.plist_off + sa) : -1;
            const int ns = off < 0 ? -1
                                   : gc_inline_set(g, sa, c.pool_m + off, c.pool_s + off, __ldcg(c.plist_cnt + sa),
                                                   s_taken, mem_m[0], mem_s[0], s_rec, min(GC_MAXS, maxs), r2max);
            ++n_inline;
            if (ns < 0) {
              p += f;
              stop = true;
              break;
            }
            if (lane == 0) atomicAdd(c.ctl + 5, 1);
            if (ns >= c.thresh) {
              for (int k = lane; k < ns; k += 32) {
                const int mb = s_rec[k];
                atomicOr(&s_taken[mb >> 5], 1u << (mb & 31));
                c.cl_members[(size_t)ncl * maxs + k] = mb;
              }
              if (lane == 0) c.cl_sizes[ncl] = ns;
              __syncwarp();
              ++ncl;
              if (ncl >= c.max_clusters) {
                done = stop = true;
                p += f + 1;
                break;
              }
            }
            cursor = f + 1;
            continue;
          }
          if (nf > maxs) {
            err = (int)RTR_ERR_CAPACITY;
            done = stop = true;
            p += f;
            break;
          }
          // the committing seed's first 8 members from lane f's registers
          int mine = 0;
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const int v = __shfl_sync(0xffffffffu, m_cur[k], f);
            if (lane == k) mine = v;
          }
          for (int k = lane; k < nf; k += 32) {
            const int mb = k < 8 ? mine : __ldcg(g.set_mem + (size_t)(p + f) * maxs + k);
            atomicOr(&s_taken[mb >> 5], 1u << (mb & 31));
            c.cl_members[(size_t)ncl * maxs + k] = mb;
          }
          if (lane == 0) c.cl_sizes[ncl] = nf;
          __syncwarp();
          ++ncl;
          if (ncl >= c.max_clusters) {
            done = stop = true;
            p += f + 1;
            break;
          }
          cursor = f + 1;
        }
        __syncwarp();
      }
      asm volatile("cp.async.wait_all;" ::: "memory");  // no copy left in flight into the ring
      if (p >= g.C) done = true;
      __syncwarp();
      for (int i = lane; i < nwords; i += 32) g.taken[i] = s_taken[i];
      if (lane == 0) {
        // a walk that used its whole window (no stale set, no cap) doubles
        // the next window: scenes whose walk runs far (few clusters) take
        // fewer rounds; a stale stop goes back to the first window
        c.ctl[12] = (!stop && p >= wend) ? min(2 * win, c.win_max) : c.win;
        c.ctl[0] = p;
        c.ctl[1] = ncl;
        c.ctl[2] = done ? 1 : 0;
        if (err) c.ctl[3] = err;
        c.ctl[4] = round + 1;
        c.ctl[6] = 0;
      }
      __syncwarp();
    }
    target += gridDim.x;
    if (!gc_barrier(c, target, &s_ok)) return;
    GC_PHASE(3)
    if (threadIdx.x == 0) {
      s_pos = __ldcg(c.ctl + 0);
      s_done = __ldcg(c.ctl + 2) || __ldcg(c.ctl + 3);
      s_win = __ldcg(c.ctl + 12);
    }
    __syncthreads();
    if (s_done) break;
  }
#undef GC_PHASE
  if (timer)
    for (int k = 0; k < 4; ++k) c.ctl[8 + k] = (int)(ph[k] / 1000ull);
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
                            const int* __restrict__ cs, const uint32_t* __restrict__ order, int C, const int* d_C,
                            float4* __restrict__ pm, float4* __restrict__ ps) {
  if (d_C) C = min(*d_C, C);
  for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < C; a += gridDim.x * blockDim.x) {
    const int i = (int)order[a];
    pm[a] = mk[cm[i]];
    ps[a] = sk[cs[i]];
  }
}

// Per-cluster least-squares pose model -> scene in FP64 (one warp per cluster).
__global__ void k_gc_poses(const float4* __restrict__ pm, const float4* __restrict__ ps,
                           const int* __restrict__ members, const int* __restrict__ sizes, int ncl,
                           const int* d_ncl, int max_members, double* __restrict__ poses) {
  const int lane = threadIdx.x & 31;
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (d_ncl) ncl = min(*d_ncl, ncl);
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
  // the whole warp solves the rotation, on lane 0's sums (the butterfly
  // leaves every lane a total, not necessarily the same bits)
#pragma unroll
  for (int k = 0; k < 9; ++k) H[k] = __shfl_sync(0xffffffffu, H[k], 0);
  double R[9];
  umeyama_rotation_warp(H, R);
  if (lane == 0) {
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
__global__ void k_gc_keys(const float* __restrict__ d, int C, const int* d_C, uint32_t* __restrict__ keys) {
  if (d_C) C = min(*d_C, C);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < C; i += gridDim.x * blockDim.x) {
    const float v = d[i];
    keys[i] = v > 0.f ? __float_as_uint(v) : 0u;
  }
}

// After the walk: the cluster count for the next stages, the error (if any)
// into the context status word, and the walk's statistics beside it.
__global__ void k_gc_post(const int* __restrict__ ctl, int max_clusters, int* d_ncl, int* status, int* stats) {
  if (threadIdx.x != 0) return;
  const int err = ctl[3];
  if (d_ncl) *d_ncl = err ? 0 : min(ctl[1], max_clusters);
  if (err) atomicCAS(status, 0, err);
  for (int k = 0; k < 12; ++k) stats[k] = ctl[k];
}

struct GcBufs {
  uint32_t *k0, *v0, *k1, *v1, *hist;
  float4 *pm, *ps;
  unsigned* taken;
  int *set_size, *set_mem, *computed, *misc;
  unsigned* arrive;
  int *members, *sizes;
  double* poses;
  GridMeta* mbox;
  int* need;
  unsigned* mask;
  GcGrid* sg;
  uint32_t *gk0, *gv0, *gk1, *gv1;
  float4 *cpts, *cpm;
  float4* cbox;
  float4 *seed_s, *seed_m;
  int *pcnt, *plist_off, *plist_cnt;
  float4 *pool_m, *pool_s;
};

// Window of the walk and the width of a pass-mask row.
constexpr int GC_WIN = 512;      // first window (room scene: 1.21 ms at 512, 1.27 at 256, 1.25 at 128); results identical
constexpr int GC_WIN_MAX = 2048;  // a window grows to this while the walk keeps using whole windows
static int gc_nwp(int C) { return (((C > 0 ? C : 1) + 31) / 32 + 3) & ~3; }
static int gc_win(int C, int want = 0) {
  const size_t row = (size_t)gc_nwp(C) * 4;
  size_t w = (size_t(256) << 20) / row;  // masks within 256 MB
  const size_t cap = want > 0 ? (size_t)want : (size_t)GC_WIN;
  if (w > cap) w = cap;
  if (w < 32) w = 32;
  return (int)w;
}

// Pass-list pool: 64 entries (32 bytes each) per correspondence, between
// 256K and 4M (a seed whose list does not fit keeps none: its set is
// recomputed by a round).
static int gc_pool_cap(int C) {
  const long long want = (long long)(C > 0 ? C : 1) * 64;
  return (int)(want < (1 << 18) ? (1 << 18) : (want > (4 << 20) ? (4 << 20) : want));
}
// Sets the walk recomputes in place per round (measured on the room scene).
constexpr int GC_INLINE_MAX = 16;

static void gc_plan(ScratchPlan& p, int C, int max_clusters, int max_members) {
  const int n = C > 0 ? C : 1;
  for (int i = 0; i < 4; ++i) p.add<uint32_t>(n);
  p.add<uint32_t>(radix_hist_entries(n));
  p.add<float4>(n);
  p.add<float4>(n);
  p.add<unsigned>((n + 31) / 32);
  p.add<int>(n);
  p.add<int>((size_t)n * gc_set_stride(C));
  p.add<int>(n);
  p.add<int>(16);
  p.add<unsigned>(1);
  p.add<int>((size_t)max_clusters * max_members);
  p.add<int>(max_clusters);
  p.add<double>((size_t)max_clusters * 16);
  p.add<GridMeta>(1);
  p.add<int>(gc_win(C, GC_WIN_MAX));
  p.add<unsigned>((size_t)gc_win(C, GC_WIN_MAX) * gc_nwp(C));
  p.add<GcGrid>(1);
  for (int i = 0; i < 4; ++i) p.add<uint32_t>(n);
  p.add<float4>(n);
  p.add<float4>(n);
  p.add<float4>((size_t)2 * ((n + 31) / 32));
  p.add<float4>(gc_win(C, GC_WIN_MAX));
  p.add<float4>(gc_win(C, GC_WIN_MAX));
  p.add<int>(gc_win(C, GC_WIN_MAX));
  p.add<int>(n);
  p.add<int>(n);
  p.add<float4>(gc_pool_cap(C));
  p.add<float4>(gc_pool_cap(C));
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
  b->set_mem = s.take<int>((size_t)n * gc_set_stride(C));
  b->computed = s.take<int>(n);
  b->misc = s.take<int>(16);
  b->arrive = s.take<unsigned>(1);
  b->members = s.take<int>((size_t)max_clusters * max_members);
  b->sizes = s.take<int>(max_clusters);
  b->poses = s.take<double>((size_t)max_clusters * 16);
  b->mbox = s.take<GridMeta>(1);
  b->need = s.take<int>(gc_win(C, GC_WIN_MAX));
  b->mask = s.take<unsigned>((size_t)gc_win(C, GC_WIN_MAX) * gc_nwp(C));
  b->sg = s.take<GcGrid>(1);
  b->gk0 = s.take<uint32_t>(n);
  b->gv0 = s.take<uint32_t>(n);
  b->gk1 = s.take<uint32_t>(n);
  b->gv1 = s.take<uint32_t>(n);
  b->cpts = s.take<float4>(n);
  b->cpm = s.take<float4>(n);
  b->cbox = s.take<float4>((size_t)2 * ((n + 31) / 32));
  b->seed_s = s.take<float4>(gc_win(C, GC_WIN_MAX));
  b->seed_m = s.take<float4>(gc_win(C, GC_WIN_MAX));
  b->pcnt = s.take<int>(gc_win(C, GC_WIN_MAX));
  b->plist_off = s.take<int>(n);
  b->plist_cnt = s.take<int>(n);
  b->pool_m = s.take<float4>(gc_pool_cap(C));
  b->pool_s = s.take<float4>(gc_pool_cap(C));
  return b->pool_s != nullptr;
}

// Shared memory of k_gc_coop beyond its static part (the taken bitset).  The
// kernel's dynamic-shared-memory limit is always set to this one value, so
// calls from several threads (the batch driver) never lower it under each
// other's launches.
constexpr size_t GC_MAX_DYN_SMEM = 176 * 1024;

}  // namespace rtr

using namespace rtr;

namespace rtr {

size_t gc_scratch_bytes(int C, int max_clusters) {
  ScratchPlan plan;
  gc_plan(plan, C, max_clusters, gc_set_stride(C));
  return plan.bytes;
}

// The grouping up to the walk's end, without a host round trip.  C_cap
// bounds the correspondences; with d_C the live count is read on the device.
static rtr_status gc_launch(rtr_context* ctx, Scratch& s, const float* d_model_kp, const float* d_scene_kp,
                            const int32_t* d_corr_m, const int32_t* d_corr_s, const float* d_corr_d, int C_cap,
                            const int* d_C, float gc_size, int gc_thresh, int max_clusters, cudaStream_t st,
                            GcBufs* bo, uint32_t** order) {
  const int C = C_cap;
  GcBufs& b = *bo;
  if (!gc_take(s, C, max_clusters, gc_set_stride(C), &b)) return fail(RTR_ERR_CAPACITY, "rtr_gc_group: scratch");
  const size_t dyn = sizeof(unsigned) * (size_t)((C + 31) / 32);
  if (dyn > GC_MAX_DYN_SMEM)
    return fail(RTR_ERR_CAPACITY, "rtr_gc_group: %d correspondences exceed the supported %d", C,
                (int)(GC_MAX_DYN_SMEM * 8));
  const int nb = (C + 255) / 256 > 152 * 8 ? 152 * 8 : (C + 255) / 256;
  ProfScope pso(ctx, st, "gc_sort");
  k_gc_keys<<<nb, 256, 0, st>>>(d_corr_d, C, d_C, b.k0);
  uint32_t *ks, *vs;
  radix_sort_pairs(b.k0, b.v0, b.k1, b.v1, b.hist, C, C, d_C, 32, true, st, &ks, &vs);
  k_gc_gather<<<nb, 256, 0, st>>>(reinterpret_cast<const float4*>(d_model_kp),
                                  reinterpret_cast<const float4*>(d_scene_kp), d_corr_m, d_corr_s, vs, C, d_C, b.pm,
                                  b.ps);
  RTR_CUDA(cudaMemsetAsync(b.taken, 0, dyn, st));
  RTR_CUDA(cudaMemsetAsync(b.computed, 0, sizeof(int) * C, st));
  RTR_CUDA(cudaMemsetAsync(b.misc, 0, sizeof(int) * 16, st));
  RTR_CUDA(cudaMemsetAsync(b.arrive, 0, sizeof(unsigned), st));
  GcDev g{b.pm, b.ps, C, d_C, gc_size, b.taken, b.set_size, b.set_mem, gc_set_stride(C)};
  bbox_build(b.mbox, b.pm, C, d_C, st);
  pso.end();
  // the coarse grid over the scene endpoints (seed-test pruning)
  ProfScope pgr(ctx, st, "gc_grid");
  bbox_build(&b.sg->m, b.ps, C, d_C, st);
  k_gcg_setup<<<1, 32, 0, st>>>(b.sg, b.mbox, gc_size, C, d_C);
  k_gcg_keys<<<nb, 256, 0, st>>>(b.ps, C, d_C, b.sg, b.gk0);
  uint32_t *gks, *gvs;  // gks unused: the cell order is all the seed tests need
  radix_sort_pairs(b.gk0, b.gv0, b.gk1, b.gv1, b.hist, C, C, d_C, 16, true, st, &gks, &gvs);
  k_gcg_gather<<<nb, 256, 0, st>>>(b.ps, b.pm, gvs, C, d_C, b.cpts, b.cpm, b.cbox);
  RTR_LAUNCHED(3);
  pgr.end();
  GcCoop c{b.misc, b.arrive, b.computed, b.members, b.sizes, gc_thresh, max_clusters,
           ctx->wait_budget_cycles, ctx->d_status, b.mbox, b.need, b.mask,
           gc_win(C, ctx->tune_gc_window > 0 ? ctx->tune_gc_window : 0), gc_win(C, GC_WIN_MAX), gc_nwp(C),
           b.sg, b.cpts, b.cpm, b.cbox, b.seed_s, b.seed_m, b.pcnt, b.plist_off, b.plist_cnt, b.pool_m, b.pool_s,
           ctx->tune_gc_no_lists ? 0 : gc_pool_cap(C),
           ctx->tune_gc_inline > 0 ? ctx->tune_gc_inline : GC_INLINE_MAX};
  const bool long_sets = gc_set_stride(C) > GC_MAXS;
  auto kern = long_sets ? k_gc_coop<true> : k_gc_coop<false>;
  RTR_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GC_MAX_DYN_SMEM));
  int per_sm = 0;
  RTR_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, GC_WARPS * 32, dyn));
  if (per_sm < 1) return fail(RTR_ERR_CAPACITY, "rtr_gc_group: grouping kernel does not fit an SM");
  // enough warps for the work (a few thousand correspondences need a few
  // blocks), and a share of the GPU when several contexts run at once
  int blocks = (per_sm < 2 ? per_sm : 2) * ctx->num_sms;
  const int div = ctx->coop_div > 0 ? ctx->coop_div : 1;
  blocks = blocks / div > 0 ? blocks / div : 1;
  const int by_work = (C + 255) / 256;
  if (by_work < blocks) blocks = by_work > 4 ? by_work : 4;
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
    RTR_CUDA(cudaLaunchKernelEx(&cfg, kern, g, c));
  }
  RTR_LAUNCHED(3);
  *order = vs;
  return RTR_OK;
}

// Grouping with every count on the device (no host round trip; the
// pipeline's form).  Writes the cluster count to *d_ncl, the first
// max_clusters sizes and poses; an error goes to the context status word.
rtr_status gc_group_async(rtr_context* ctx, Scratch& s, const float* d_model_kp, const float* d_scene_kp,
                          const int32_t* d_corr_m, const int32_t* d_corr_s, const float* d_corr_d, int C_cap,
                          const int* d_C, float gc_size, int gc_thresh, int max_clusters, int32_t* d_sizes,
                          double* d_poses, int* d_ncl, cudaStream_t st) {
  GcBufs b;
  uint32_t* order = nullptr;
  RTR_TRY(gc_launch(ctx, s, d_model_kp, d_scene_kp, d_corr_m, d_corr_s, d_corr_d, C_cap > 0 ? C_cap : 1, d_C,
                    gc_size, gc_thresh, max_clusters, st, &b, &order));
  ProfScope pp(ctx, st, "gc_poses");
  k_gc_post<<<1, 32, 0, st>>>(b.misc, max_clusters, d_ncl, ctx->d_status, ctx->d_status + 16);
  k_gc_poses<<<(max_clusters + 3) / 4, 128, 0, st>>>(b.pm, b.ps, b.members, b.sizes, max_clusters, d_ncl,
                                                      gc_set_stride(C_cap > 0 ? C_cap : 1), b.poses);
  RTR_LAUNCHED(2);
  if (d_poses)
    RTR_CUDA(cudaMemcpyAsync(d_poses, b.poses, sizeof(double) * 16 * max_clusters, cudaMemcpyDeviceToDevice, st));
  if (d_sizes) RTR_CUDA(cudaMemcpyAsync(d_sizes, b.sizes, sizeof(int) * max_clusters, cudaMemcpyDeviceToDevice, st));
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

rtr_status gc_group_dev(rtr_context* ctx, Scratch& s, const float* d_model_kp, const float* d_scene_kp,
                        const int32_t* d_corr_m, const int32_t* d_corr_s, const float* d_corr_d, int n_corr,
                        float gc_size, int gc_thresh, int max_clusters, int max_members, int32_t* d_members,
                        int32_t* d_sizes, double* d_poses, int* h_n_clusters, cudaStream_t st) {
  *h_n_clusters = 0;
  if (n_corr == 0) return RTR_OK;
  GcBufs b;
  uint32_t* vs = nullptr;
  RTR_TRY(gc_launch(ctx, s, d_model_kp, d_scene_kp, d_corr_m, d_corr_s, d_corr_d, n_corr, nullptr, gc_size,
                    gc_thresh, max_clusters, st, &b, &vs));
  // errors come back as this call's status, so they go to a spare status slot
  k_gc_post<<<1, 32, 0, st>>>(b.misc, max_clusters, nullptr, ctx->d_status + 15, ctx->d_status + 16);
  RTR_LAUNCHED(1);
  int* h = ctx->h_pin;
  RTR_CUDA(cudaMemcpyAsync(h, b.misc, 12 * sizeof(int), cudaMemcpyDeviceToHost, st));
  RTR_CUDA(cudaStreamSynchronize(st));
  const int ncl = h[1];
  if (h[3] == (int)RTR_ERR_CAPACITY)
    return fail(RTR_ERR_CAPACITY, "rtr_gc_group: a consensus set exceeds %d members", gc_set_stride(n_corr));
  if (h[3] == (int)RTR_ERR_TIMEOUT)
    return fail(RTR_ERR_TIMEOUT, "rtr_gc_group: a grid barrier wait exceeded the budget");
  if (ncl > 0) {
    k_gc_poses<<<(ncl + 3) / 4, 128, 0, st>>>(b.pm, b.ps, b.members, b.sizes, ncl, nullptr, gc_set_stride(n_corr),
                                               b.poses);
    RTR_LAUNCHED(1);
    if (d_poses) RTR_CUDA(cudaMemcpyAsync(d_poses, b.poses, sizeof(double) * 16 * ncl, cudaMemcpyDeviceToDevice, st));
    if (d_sizes) RTR_CUDA(cudaMemcpyAsync(d_sizes, b.sizes, sizeof(int) * ncl, cudaMemcpyDeviceToDevice, st));
    if (d_members) {
      k_gc_members_out<<<(ncl * max_members + 255) / 256, 256, 0, st>>>(b.members, b.sizes, vs, ncl,
                                                                         gc_set_stride(n_corr), max_members,
                                                                         d_members);
      RTR_LAUNCHED(1);
    }
  }
  *h_n_clusters = ncl;
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

}  // namespace rtr

extern "C" rtr_status rtr_gc_stats(rtr_context* ctx, int* h_stats8) {
  RTR_CHECK_ARG(ctx && h_stats8, "rtr_gc_stats: bad arguments");
  RTR_CUDA(cudaSetDevice(ctx->device));
  RTR_CUDA(cudaDeviceSynchronize());
  int h[12];
  RTR_CUDA(cudaMemcpy(h, ctx->d_status + 16, sizeof(h), cudaMemcpyDeviceToHost));
  h_stats8[0] = h[4];  // rounds
  h_stats8[1] = h[0];  // walk end
  h_stats8[2] = h[5];  // sets computed
  for (int k = 0; k < 4; ++k) h_stats8[3 + k] = h[8 + k];
  h_stats8[7] = h[7];  // candidates
  return RTR_OK;
}

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
