// refmatch.cu — the reference's own descriptor route on the GPU:
//
//   KeyPoint::getOccupiedGrid  key_point.h:112-161  -> rtr_ref_occupancy
//   KeyPoint::get_TSDF         key_point.h:251-334  -> rtr_ref_tdf
//   get_Distance               matching.h:122-222   -> rtr_ref_distance
//   the all-pairs loop + match_by_* gates
//                              RealTimeRobot.cpp:70-102, function.h:158-178
//                                                   -> rtr_ref_correspond
//   Ransac                     function.h:35-109    -> rtr_ref_ransac
//
// The reference runs each of these through PCL 1.8.0 octrees built per call
// (per keypoint, per pair and per rotation).  Here nothing is a tree: an
// octree with a defined bounding box is a cube of 2^depth leaves, so a leaf
// is its integer key, the leaves' depth-first order is the Morton order of
// the keys (x the high bit of each level), and the tree's growth when a point
// lands outside is a rule on the cube's corner and depth.  The octree rules
// restated (the same in the CPU oracle):
//   define: depth = fewest levels covering ceil((hi - lo - FLT_EPSILON)/res)
//     leaves on the widest axis (at least 2); each axis padded equally on
//     both sides to the cube edge 2^depth * res (when the pad exceeds
//     FLT_EPSILON);
//   growth: a point with p < min or p >= max on some axis adds a level: on
//     every axis where the point is not above, min -= old edge; then
//     max = min + new edge - FLT_EPSILON; repeated until the point fits;
//     points are inserted in ascending order of their cloud index;
//   key = (unsigned)((p - min) / res) in double against the final cube;
//   centre = (float)((key + 0.5) * res + min).
// All double and float arithmetic that has to agree with the oracle uses the
// _rn intrinsics, so nothing is contracted into an FMA.
//
// Kernels (one CTA per keypoint or per pair; the work is gather- and
// latency-bound, the pair kernel's inner loop runs from registers and a
// 4 KB shared bitmap):
//   k_ref_occ        box search over the cloud, occupied-leaf count (Number),
//                    ordered append of the box's point indices;
//   k_ref_tdf_cells  the keypoint's occupied leaves in the +-half_tdf cube,
//                    first leaf dropped, as integer voxels -> k_tdf (tdf.cu);
//   k_ref_distance   36 yaw steps of the translated occupancy cloud, leaves
//                    deduplicated in a 32^3 bitmap around the cloud, the
//                    field read per leaf, the leaves sorted into tree order
//                    and their squared values added in float one by one
//                    (the reference's running score), pair transform;
//   k_ref_gates / k_ref_scatter   the kept pairs in loop order;
//   k_ref_ransac / k_ref_argmax   inliers of every kept pair's transform.
#include <math.h>
#include <string.h>

#include "common.cuh"
#include "scan.cuh"

namespace rtr {

constexpr int REF_DIM = 30;
constexpr int REF_VOL = REF_DIM * REF_DIM * REF_DIM;
constexpr int REF_MAX_DEPTH = 21;
constexpr int REF_PPT = 8;        // cloud points per thread in k_ref_distance
constexpr int REF_WIN = 32;       // leaves per axis of the distance kernel's bitmap window
constexpr int REF_OCC_DEPTH = 5;  // cube depth the occupancy and field kernels hold in a bitmap
constexpr double REF_FLT_EPS = 1.1920928955078125e-07;  // FLT_EPSILON

// error bits of the status word
constexpr int REF_ERR_WINDOW = 1;  // a rotated occupancy cloud spans more than REF_WIN leaves
constexpr int REF_ERR_DEPTH = 2;   // an occupancy or field cube deeper than REF_OCC_DEPTH
constexpr int REF_ERR_GROW = 4;    // the occupancy cloud left the field's cube (occupancy box wider)

struct RefRot {
  float c1, s1;          // cosf / sinf of theta = (float)(pi / 18)
  float c2[36], s2[36];  // (float)cos((double)(i * theta)), likewise sin
};

struct OctBox {
  double mn[3], mx[3];
  int depth;
};

__device__ __forceinline__ void oct_define(OctBox& b, const float lo[3], const float hi[3], double res) {
  unsigned mv = 2;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double ext = __dsub_rn((double)hi[a], (double)lo[a]);
    const double k = ceil(__ddiv_rn(__dsub_rn(ext, REF_FLT_EPS), res));
    if (k > (double)mv) mv = (unsigned)k;
  }
  int d = 0;
  while (d < 31 && (1u << d) < mv) ++d;
  const double side = __dmul_rn((double)(1u << d), res);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    b.mn[a] = (double)lo[a];
    b.mx[a] = (double)hi[a];
    const double over = __ddiv_rn(__dsub_rn(side, __dsub_rn((double)hi[a], (double)lo[a])), 2.0);
    if (over > REF_FLT_EPS) {
      b.mn[a] = __dsub_rn(b.mn[a], over);
      b.mx[a] = __dadd_rn(b.mx[a], over);
    }
  }
  b.depth = d;
}

__device__ __forceinline__ bool oct_outside(const OctBox& b, float x, float y, float z) {
  return (double)x < b.mn[0] || (double)y < b.mn[1] || (double)z < b.mn[2] || (double)x >= b.mx[0] ||
         (double)y >= b.mx[1] || (double)z >= b.mx[2];
}

// Grow until (x, y, z) fits; false past REF_MAX_DEPTH levels.
__device__ bool oct_fit(OctBox& b, float x, float y, float z, double res) {
  const float p[3] = {x, y, z};
  for (int guard = 0; guard <= REF_MAX_DEPTH + 1; ++guard) {
    bool up[3], out = false;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      up[a] = (double)p[a] >= b.mx[a];
      out = out || up[a] || (double)p[a] < b.mn[a];
    }
    if (!out) return true;
    if (b.depth >= REF_MAX_DEPTH) return false;
    const double side = __dmul_rn((double)(1u << b.depth), res);
#pragma unroll
    for (int a = 0; a < 3; ++a)
      if (!up[a]) b.mn[a] = __dsub_rn(b.mn[a], side);
    b.depth++;
    const double edge = __dsub_rn(__dmul_rn((double)(1u << b.depth), res), REF_FLT_EPS);
#pragma unroll
    for (int a = 0; a < 3; ++a) b.mx[a] = __dadd_rn(b.mn[a], edge);
  }
  return false;
}

__device__ __forceinline__ unsigned oct_key1(const OctBox& b, float p, int a, double res) {
  const unsigned top = (1u << b.depth) - 1u;
  const unsigned v = __double2uint_rz(__ddiv_rn(__dsub_rn((double)p, b.mn[a]), res));
  return v > top ? top : v;
}

// The cube's float view.  For a float p and a double bound c, p < c exactly
// when p < (c rounded up to float), and p >= c exactly when p >= (c rounded
// up): no float lies strictly between c and its upward rounding.  So the
// inside test needs no double arithmetic.
struct OctBoxF {
  float mn_up[3], mx_up[3], mn_f[3];
};

__device__ __forceinline__ void oct_float(const OctBox& b, OctBoxF& f) {
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    f.mn_up[a] = __double2float_ru(b.mn[a]);
    f.mx_up[a] = __double2float_ru(b.mx[a]);
    f.mn_f[a] = __double2float_rn(b.mn[a]);
  }
}

__device__ __forceinline__ bool oct_outside_f(const OctBoxF& f, float x, float y, float z) {
  return x < f.mn_up[0] || y < f.mn_up[1] || z < f.mn_up[2] || x >= f.mx_up[0] || y >= f.mx_up[1] ||
         z >= f.mx_up[2];
}

// oct_key1 with a float estimate first: y = (p - min) * (1/res) in float is
// within (|min|/res + 3|y|) * 2^-24 of the exact quotient t, so when y is
// farther than four times that from every integer, floor(y) = floor(t) =
// the double-precision key.  Otherwise (a few keys in 10^5) the double path.
__device__ __forceinline__ unsigned oct_key_f(const OctBox& b, const OctBoxF& f, float p, int a, double res,
                                              float inv) {
  const float y = __fmul_rn(__fsub_rn(p, f.mn_f[a]), inv);
  const float fl = floorf(y);
  const float gap = fminf(__fsub_rn(y, fl), __fsub_rn(__fadd_rn(fl, 1.f), y));
  const float margin = __fmul_rn(__fadd_rn(__fadd_rn(__fmul_rn(fabsf(f.mn_f[a]), inv), __fmul_rn(4.f, fabsf(y))), 4.f),
                                 2.4e-7f);
  if (gap > margin && fl >= 0.f && fl < 4194304.f) {
    const unsigned top = (1u << b.depth) - 1u;
    const unsigned v = (unsigned)fl;
    return v > top ? top : v;
  }
  return oct_key1(b, p, a, res);
}

// Morton code of a key (each coordinate < 2^21): the bits of x, y, z
// interleaved with x the high bit of each triple, so ascending codes list the
// leaves depth-first in child order (x << 2 | y << 1 | z) at any depth.
__device__ __forceinline__ unsigned long long spread3(unsigned v) {
  unsigned long long x = v & 0x1fffffu;
  x = (x | x << 32) & 0x1f00000000ffffull;
  x = (x | x << 16) & 0x1f0000ff0000ffull;
  x = (x | x << 8) & 0x100f00f00f00f00full;
  x = (x | x << 4) & 0x10c30c30c30c30c3ull;
  x = (x | x << 2) & 0x1249249249249249ull;
  return x;
}

__device__ __forceinline__ unsigned compact3(unsigned long long x) {
  x &= 0x1249249249249249ull;
  x = (x ^ (x >> 2)) & 0x10c30c30c30c30c3ull;
  x = (x ^ (x >> 4)) & 0x100f00f00f00f00full;
  x = (x ^ (x >> 8)) & 0x1f0000ff0000ffull;
  x = (x ^ (x >> 16)) & 0x1f00000000ffffull;
  x = (x ^ (x >> 32)) & 0x1fffffull;
  return (unsigned)x;
}

__device__ __forceinline__ unsigned long long morton3(unsigned kx, unsigned ky, unsigned kz, int /*depth*/) {
  return (spread3(kx) << 2) | (spread3(ky) << 1) | spread3(kz);
}

__device__ __forceinline__ void demorton3(unsigned long long m, int /*depth*/, unsigned& kx, unsigned& ky,
                                          unsigned& kz) {
  kx = compact3(m >> 2);
  ky = compact3(m >> 1);
  kz = compact3(m);
}

__device__ __forceinline__ float oct_centre(const OctBox& b, unsigned key, int a, double res) {
  return __double2float_rn(__dadd_rn(__dmul_rn(__dadd_rn((double)key, 0.5), res), b.mn[a]));
}

// ((m0*x + m1*y) + m2*z) + m3 per row, each operation rounded.
__device__ __forceinline__ void xf3(const float* M, float& x, float& y, float& z) {
  const float ox = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(M[0], x), __fmul_rn(M[1], y)), __fmul_rn(M[2], z)), M[3]);
  const float oy = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(M[4], x), __fmul_rn(M[5], y)), __fmul_rn(M[6], z)), M[7]);
  const float oz =
      __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(M[8], x), __fmul_rn(M[9], y)), __fmul_rn(M[10], z)), M[11]);
  x = ox, y = oy, z = oz;
}

// C = A B (4x4 row-major float), the four terms summed in index order.
__device__ void mm4(const float* A, const float* B, float* C) {
  float T[16];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      float s = __fmul_rn(A[4 * r], B[c]);
      s = __fadd_rn(s, __fmul_rn(A[4 * r + 1], B[4 + c]));
      s = __fadd_rn(s, __fmul_rn(A[4 * r + 2], B[8 + c]));
      s = __fadd_rn(s, __fmul_rn(A[4 * r + 3], B[12 + c]));
      T[4 * r + c] = s;
    }
  for (int i = 0; i < 16; ++i) C[i] = T[i];
}

__device__ __forceinline__ void eye4(float* M) {
  for (int i = 0; i < 16; ++i) M[i] = (i % 5) == 0 ? 1.f : 0.f;
}

__device__ __forceinline__ bool in_box(float4 p, const float lo[3], const float hi[3]) {
  return p.x >= lo[0] && p.y >= lo[1] && p.z >= lo[2] && p.x <= hi[0] && p.y <= hi[1] && p.z <= hi[2];
}

// ---------------------------------------------------------------------------
// getOccupiedGrid: one CTA per keypoint.  fill == false: count[k] and
// number[k]; fill == true: indices from offsets[k], ascending.
// ---------------------------------------------------------------------------
constexpr int OCC_NT = 256;

__global__ void __launch_bounds__(OCC_NT) k_ref_occ(const float4* __restrict__ cloud, int n,
                                                    const float4* __restrict__ keys, float res, float half,
                                                    bool fill, int* __restrict__ count, int* __restrict__ number,
                                                    const int* __restrict__ offsets, int* __restrict__ indices,
                                                    int* __restrict__ err) {
  __shared__ unsigned s_bm[1024];
  __shared__ int s_wsum[OCC_NT / 32];
  const int k = blockIdx.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const float4 kp = keys[k];
  const float lo[3] = {__fsub_rn(kp.x, half), __fsub_rn(kp.y, half), __fsub_rn(kp.z, half)};
  const float hi[3] = {__fadd_rn(kp.x, half), __fadd_rn(kp.y, half), __fadd_rn(kp.z, half)};
  if (!fill) {
    OctBox b;
    oct_define(b, lo, hi, (double)res);
    const bool deep = b.depth > REF_OCC_DEPTH;
    if (deep && tid == 0) atomicOr(err, REF_ERR_DEPTH);
    for (int i = tid; i < 1024; i += OCC_NT) s_bm[i] = 0u;
    __syncthreads();
    int c = 0;
    for (int i = tid; i < n; i += OCC_NT) {
      const float4 p = cloud[i];
      if (!in_box(p, lo, hi)) continue;
      ++c;
      if (deep) continue;
      const unsigned long long m = morton3(oct_key1(b, p.x, 0, (double)res), oct_key1(b, p.y, 1, (double)res),
                                           oct_key1(b, p.z, 2, (double)res), b.depth);
      atomicOr(&s_bm[(unsigned)(m >> 5)], 1u << (unsigned)(m & 31ull));
    }
    __syncthreads();
    int u = 0;
    for (int i = tid; i < 1024; i += OCC_NT) u += __popc(s_bm[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      c += __shfl_xor_sync(0xffffffffu, c, o);
      u += __shfl_xor_sync(0xffffffffu, u, o);
    }
    __shared__ int s_c[OCC_NT / 32], s_u[OCC_NT / 32];
    if (lane == 0) s_c[w] = c, s_u[w] = u;
    __syncthreads();
    if (tid == 0) {
      int tc = 0, tu = 0;
      for (int i = 0; i < OCC_NT / 32; ++i) tc += s_c[i], tu += s_u[i];
      count[k] = tc;
      number[k] = tu;
    }
    return;
  }
  int base = offsets[k];
  for (int c0 = 0; c0 < n; c0 += OCC_NT) {
    const int i = c0 + tid;
    const bool f = i < n && in_box(cloud[i], lo, hi);
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    if (lane == 0) s_wsum[w] = __popc(bal);
    __syncthreads();
    int before = 0, tot = 0;
    for (int j = 0; j < OCC_NT / 32; ++j) {
      before += j < w ? s_wsum[j] : 0;
      tot += s_wsum[j];
    }
    if (f) indices[base + before + __popc(bal & lanemask_lt())] = i;
    base += tot;
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// get_TSDF's occupied voxels: one CTA per keypoint.  fill == false:
// cnt[k] = leaves - 1 (0 without leaves); fill == true: the integer voxels of
// every leaf but the first, in leaf order, from cell_off[k].
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(OCC_NT) k_ref_tdf_cells(const float4* __restrict__ cloud,
                                                          const float4* __restrict__ keys,
                                                          const int* __restrict__ offsets,
                                                          const int* __restrict__ indices, float res, float half,
                                                          bool fill, int* __restrict__ cnt,
                                                          const int* __restrict__ cell_off, int* __restrict__ occ,
                                                          int* __restrict__ err) {
  __shared__ unsigned s_bm[1024];
  __shared__ int s_ws[OCC_NT / 32];
  const int k = blockIdx.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const float4 kp = keys[k];
  const float lo[3] = {__fsub_rn(kp.x, half), __fsub_rn(kp.y, half), __fsub_rn(kp.z, half)};
  const float hi[3] = {__fadd_rn(kp.x, half), __fadd_rn(kp.y, half), __fadd_rn(kp.z, half)};
  OctBox b;
  oct_define(b, lo, hi, (double)res);
  if (b.depth > REF_OCC_DEPTH) {
    if (tid == 0) {
      atomicOr(err, REF_ERR_DEPTH);
      if (!fill) cnt[k] = 0;
    }
    return;
  }
  for (int i = tid; i < 1024; i += OCC_NT) s_bm[i] = 0u;
  __syncthreads();
  const int beg = offsets[k], end = offsets[k + 1];
  bool grew = false;
  for (int j = beg + tid; j < end; j += OCC_NT) {
    const float4 p = cloud[indices[j]];
    if (oct_outside(b, p.x, p.y, p.z)) {
      grew = true;
      continue;
    }
    const unsigned long long m = morton3(oct_key1(b, p.x, 0, (double)res), oct_key1(b, p.y, 1, (double)res),
                                         oct_key1(b, p.z, 2, (double)res), b.depth);
    atomicOr(&s_bm[(unsigned)(m >> 5)], 1u << (unsigned)(m & 31ull));
  }
  if (grew) atomicOr(err, REF_ERR_GROW);
  __syncthreads();
  // each thread owns 4 consecutive words (1024 = 4 * OCC_NT)
  unsigned wd[4];
  int mine = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    wd[q] = s_bm[4 * tid + q];
    mine += __popc(wd[q]);
  }
  int incl = mine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) s_ws[w] = incl;
  __syncthreads();
  int before = incl - mine, total = 0;
  for (int j = 0; j < OCC_NT / 32; ++j) {
    before += j < w ? s_ws[j] : 0;
    total += s_ws[j];
  }
  if (!fill) {
    if (tid == 0) cnt[k] = total > 0 ? total - 1 : 0;
    return;
  }
  int rank = before;
  const int out0 = cell_off[k];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    unsigned bits = wd[q];
    while (bits) {
      const int bit = __ffs(bits) - 1;
      bits &= bits - 1u;
      if (rank > 0) {
        const unsigned long long m = (unsigned long long)(4 * tid + q) * 32ull + (unsigned long long)bit;
        unsigned kx, ky, kz;
        demorton3(m, b.depth, kx, ky, kz);
        const unsigned kk[3] = {kx, ky, kz};
        int* o = occ + 3 * (size_t)(out0 + rank - 1);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const float c = oct_centre(b, kk[a], a, (double)res);
          o[a] = __double2int_rz(__ddiv_rn(__dsub_rn((double)c, (double)lo[a]), (double)res));
        }
      }
      ++rank;
    }
  }
}

// ---------------------------------------------------------------------------
// get_Distance: one CTA per pair.
// ---------------------------------------------------------------------------
template <int NT>
struct RefShared {
  unsigned bm[REF_WIN * REF_WIN * REF_WIN / 32];
  int first[NT / 32];
  unsigned long long mmin[NT / 32];
  unsigned kmin[NT / 32][3], kmax[NT / 32][3];
  int u;  // distinct leaves of the current rotation
  float px, py, pz;
};

// get_Distance adds the squared field values of a rotation's leaves (all but
// the first) in float, one by one in the octree's depth-first order, into a
// running score that no rotation resets (matching.h:141,179-189).  Float
// addition does not reassociate, so the leaves are first put in that order:
// a bitonic sort of (Morton code, field value) pairs in shared memory (codes
// are distinct; padding keys are ~0), then one thread adds them in sequence.
// P is a power of two >= 2; `t` / `nt` this thread's index and the number of
// threads sorting; `sync` orders the stages (__syncwarp or __syncthreads).
template <class Sync>
__device__ __forceinline__ void leaf_sort(unsigned long long* key, float* val, int P, int t, int nt, Sync sync) {
  for (int k = 2; k <= P; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int q = t; q < (P >> 1); q += nt) {
        const int i = ((q & ~(j - 1)) << 1) | (q & (j - 1));  // bit j of i clear
        const int l = i | j;
        const unsigned long long a = key[i], b = key[l];
        if ((a > b) == ((i & k) == 0)) {
          key[i] = b;
          key[l] = a;
          const float x = val[i];
          val[i] = val[l];
          val[l] = x;
        }
      }
      sync();
    }
}

// The running score's update for one rotation from its sorted leaves:
// score = (score + v_1^2 + ... + v_{u-1}^2) / (u - 1), each operation a
// float operation rounded to nearest; (size_t)(u - 1) is 2^64 for u = 0.
__device__ __forceinline__ float leaf_running_score(float dtf, const float* val, int u) {
  for (int i = 1; i < u; ++i) dtf = __fadd_rn(dtf, __fmul_rn(val[i], val[i]));
  const float div = u == 0 ? 18446744073709551616.f : (float)(u - 1);
  return __fdiv_rn(dtf, div);
}

struct WarpSync {
  __device__ void operator()() const { __syncwarp(); }
};
struct BlockSync {
  __device__ void operator()() const { __syncthreads(); }
};

__device__ __forceinline__ float field_at(const float* __restrict__ grid, const OctBox& b, unsigned kx, unsigned ky,
                                          unsigned kz, const float lo[3], float res) {
  const unsigned kk[3] = {kx, ky, kz};
  long long ix[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float c = oct_centre(b, kk[a], a, (double)res);
    const float q = __fdiv_rn(__fsub_rn(c, lo[a]), res);
    if (!(q > -2147483648.f && q < 2147483648.f)) return 900.f;
    ix[a] = (long long)__float2int_rz(q);
  }
  const long long idx = ix[1] * REF_DIM + ix[2] * (REF_DIM * REF_DIM) + ix[0];
  return (idx >= 0 && idx < REF_VOL) ? __ldg(grid + idx) : 900.f;
}

template <int NT>
__global__ void __launch_bounds__(NT) k_ref_distance(const float4* __restrict__ mcloud,
                                                     const float4* __restrict__ mkeys,
                                                     const int* __restrict__ moff, const int* __restrict__ midx,
                                                     const float* __restrict__ mtdf,
                                                     const float4* __restrict__ skeys, int ns,
                                                     const int* __restrict__ pair_m,
                                                     const int* __restrict__ pair_s, float res, float half,
                                                     RefRot rot, float* __restrict__ score, float* __restrict__ Tout,
                                                     int* __restrict__ err) {
  constexpr int NW = NT / 32;
  constexpr int CAP = NT * REF_PPT;  // distinct leaves <= points
  __shared__ RefShared<NT> sh;
  extern __shared__ unsigned long long s_leaf_key[];  // [CAP] keys, then [CAP] floats
  float* s_leaf_val = reinterpret_cast<float*>(s_leaf_key + CAP);
  const long long p = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int m = pair_m ? pair_m[p] : (int)(p / ns);
  const int s = pair_s ? pair_s[p] : (int)(p % ns);
  const float4 km = mkeys[m], ks = skeys[s];
  float* To = Tout + 16 * p;
  if (!(isfinite(km.x) && isfinite(km.y) && isfinite(km.z) && isfinite(ks.x) && isfinite(ks.y) &&
        isfinite(ks.z))) {
    if (tid == 0) {
      score[p] = __int_as_float(0x7fc00000);
      eye4(To);
    }
    return;
  }
  const int beg = moff[m], n = moff[m + 1] - beg;
  const float* grid = mtdf + (size_t)m * REF_VOL;
  const double dres = (double)res;
  const float inv = __fdiv_rn(1.f, res);
  const float lo[3] = {__fsub_rn(km.x, half), __fsub_rn(km.y, half), __fsub_rn(km.z, half)};
  const float hi[3] = {__fadd_rn(km.x, half), __fadd_rn(km.y, half), __fadd_rn(km.z, half)};
  float Tm[16], T1[16], T3[16], M[16];
  eye4(Tm);
  Tm[3] = __fsub_rn(km.x, ks.x), Tm[7] = __fsub_rn(km.y, ks.y), Tm[11] = __fsub_rn(km.z, ks.z);
  eye4(T1);
  T1[3] = -km.x, T1[7] = -km.y;
  eye4(T3);
  T3[3] = km.x, T3[7] = km.y;
  {
    float Rs[16];
    eye4(Rs);
    Rs[0] = rot.c1, Rs[4] = rot.s1, Rs[1] = -rot.s1, Rs[5] = rot.c1;
    mm4(T3, Rs, M);
    mm4(M, T1, M);
  }
  float px[REF_PPT], py[REF_PPT], pz[REF_PPT];
#pragma unroll
  for (int q = 0; q < REF_PPT; ++q) {
    const int j = tid + q * NT;
    px[q] = py[q] = pz[q] = 0.f;
    if (j < n) {
      const float4 c = mcloud[midx[beg + j]];
      px[q] = c.x, py[q] = c.y, pz[q] = c.z;
      xf3(Tm, px[q], py[q], pz[q]);
    }
  }
  OctBox b0;
  oct_define(b0, lo, hi, dres);
  float dtf = 0.f, bestf = 100000000.f;
  int best_i = 0;
  bool bad = false;
  for (int it = 0; it < 36 && !bad; ++it) {
    if (it != 0) {
#pragma unroll
      for (int q = 0; q < REF_PPT; ++q)
        if (tid + q * NT < n) xf3(M, px[q], py[q], pz[q]);
    }
    // the tree's growth, point by point in index order: every thread keeps
    // the same cube, grown by the first point outside it until none is
    OctBox b = b0;
    OctBoxF bf;
    oct_float(b, bf);
    for (int round = 0; round < 4 * REF_MAX_DEPTH + 4; ++round) {
      int first = 0x7fffffff;
#pragma unroll
      for (int q = 0; q < REF_PPT; ++q) {
        const int j = tid + q * NT;
        if (j < n && first == 0x7fffffff && oct_outside_f(bf, px[q], py[q], pz[q])) first = j;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
      if (lane == 0) sh.first[w] = first;
      __syncthreads();
      first = 0x7fffffff;
#pragma unroll
      for (int i = 0; i < NW; ++i) first = min(first, sh.first[i]);
      if (first == 0x7fffffff) break;
      if (first % NT == tid) {
        const int q = first / NT;
#pragma unroll
        for (int qq = 0; qq < REF_PPT; ++qq)
          if (qq == q) sh.px = px[qq], sh.py = py[qq], sh.pz = pz[qq];
      }
      __syncthreads();
      if (!oct_fit(b, sh.px, sh.py, sh.pz, dres)) bad = true;
      oct_float(b, bf);
      __syncthreads();
      if (bad) break;
    }
    if (bad) break;
    // leaf keys (as Morton codes), the first leaf, the keys' bounding window
    unsigned long long mc[REF_PPT];
    unsigned long long mmin = ~0ull;
    unsigned kmin[3] = {~0u, ~0u, ~0u}, kmax[3] = {0u, 0u, 0u};
#pragma unroll
    for (int q = 0; q < REF_PPT; ++q) {
      mc[q] = ~0ull;
      if (tid + q * NT < n) {
        const unsigned kx = oct_key_f(b, bf, px[q], 0, dres, inv), ky = oct_key_f(b, bf, py[q], 1, dres, inv),
                       kz = oct_key_f(b, bf, pz[q], 2, dres, inv);
        mc[q] = morton3(kx, ky, kz, b.depth);
        mmin = min(mmin, mc[q]);
        kmin[0] = min(kmin[0], kx), kmin[1] = min(kmin[1], ky), kmin[2] = min(kmin[2], kz);
        kmax[0] = max(kmax[0], kx), kmax[1] = max(kmax[1], ky), kmax[2] = max(kmax[2], kz);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      mmin = min(mmin, __shfl_xor_sync(0xffffffffu, mmin, o));
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        kmin[a] = min(kmin[a], __shfl_xor_sync(0xffffffffu, kmin[a], o));
        kmax[a] = max(kmax[a], __shfl_xor_sync(0xffffffffu, kmax[a], o));
      }
    }
    if (lane == 0) {
      sh.mmin[w] = mmin;
#pragma unroll
      for (int a = 0; a < 3; ++a) sh.kmin[w][a] = kmin[a], sh.kmax[w][a] = kmax[a];
    }
    for (int i = tid; i < REF_WIN * REF_WIN * REF_WIN / 32; i += NT) sh.bm[i] = 0u;
    if (tid == 0) sh.u = 0;
    __syncthreads();
    for (int i = 0; i < NW; ++i) {
      mmin = min(mmin, sh.mmin[i]);
#pragma unroll
      for (int a = 0; a < 3; ++a) kmin[a] = min(kmin[a], sh.kmin[i][a]), kmax[a] = max(kmax[a], sh.kmax[i][a]);
    }
    const bool window_ok = n == 0 || (kmax[0] - kmin[0] < (unsigned)REF_WIN && kmax[1] - kmin[1] < (unsigned)REF_WIN &&
                                      kmax[2] - kmin[2] < (unsigned)REF_WIN);
    if (!window_ok && tid == 0) atomicOr(err, REF_ERR_WINDOW);
    // distinct leaves: the thread that sets a leaf's bit reads its field and
    // lists (Morton code, value); the first leaf's value is never added
    if (window_ok) {
#pragma unroll
      for (int q = 0; q < REF_PPT; ++q) {
        if (mc[q] == ~0ull) continue;
        unsigned kx, ky, kz;
        demorton3(mc[q], b.depth, kx, ky, kz);
        const unsigned l = (kx - kmin[0]) + REF_WIN * ((ky - kmin[1]) + REF_WIN * (kz - kmin[2]));
        const unsigned bit = 1u << (l & 31u);
        const unsigned old = atomicOr(&sh.bm[l >> 5], bit);
        if (old & bit) continue;
        const float v = mc[q] == mmin ? 0.f : field_at(grid, b, kx, ky, kz, lo, res);
        const int slot = atomicAdd(&sh.u, 1);
        s_leaf_key[slot] = mc[q];
        s_leaf_val[slot] = v;
      }
    }
    __syncthreads();
    const int u = sh.u;
    int P = 2;
    while (P < u) P <<= 1;
    for (int i = u + tid; i < P; i += NT) s_leaf_key[i] = ~0ull;
    __syncthreads();
    leaf_sort(s_leaf_key, s_leaf_val, P, tid, NT, BlockSync());
    if (tid == 0) {
      dtf = leaf_running_score(dtf, s_leaf_val, u);
      if (dtf < bestf) {
        bestf = dtf;
        best_i = it;
      }
    }
    __syncthreads();
  }
  if (tid != 0) return;
  if (bad) {
    score[p] = __int_as_float(0x7fc00000);
    eye4(To);
    return;
  }
  score[p] = bestf;
  float S[16], R2[16], A[16];
  eye4(S);
  const float cs = __fdiv_rn(km.z, ks.z);
  S[0] = S[5] = S[10] = cs;
  eye4(R2);
  R2[0] = rot.c2[best_i], R2[4] = rot.s2[best_i], R2[1] = -rot.s2[best_i], R2[5] = rot.c2[best_i];
  mm4(S, T3, A);
  mm4(A, R2, A);
  mm4(A, T1, A);
  mm4(A, Tm, A);
  for (int i = 0; i < 16; ++i) To[i] = A[i];
}

// get_Distance, one warp per pair, for occupancy clouds of up to 256 points
// (8 per lane): the same steps as k_ref_distance with every reduction a
// shuffle, the growth's point broadcast by shuffle, and the warp's own 4 KB
// bitmap cleared by the points that set it.
constexpr int REFW_PPT = 8;
constexpr int REFW_WARPS = 4;

__global__ void __launch_bounds__(32 * REFW_WARPS, 4)
    k_ref_distance_warp(const float4* __restrict__ mcloud, const float4* __restrict__ mkeys,
                        const int* __restrict__ moff, const int* __restrict__ midx, const float* __restrict__ mtdf,
                        const float4* __restrict__ skeys, int ns, const int* __restrict__ pair_m,
                        const int* __restrict__ pair_s, long long n_pairs, float res, float half, RefRot rot,
                        float* __restrict__ score, float* __restrict__ Tout, int* __restrict__ err) {
  __shared__ unsigned s_bm[REFW_WARPS][REF_WIN * REF_WIN * REF_WIN / 32];
  __shared__ long long s_ix[REFW_WARPS][3][REF_WIN];
  __shared__ unsigned long long s_key[REFW_WARPS][REFW_PPT * 32];
  __shared__ float s_val[REFW_WARPS][REFW_PPT * 32];
  __shared__ int s_u[REFW_WARPS];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned* bm = s_bm[w];
  const float inv = __fdiv_rn(1.f, res);
  for (int i = lane; i < REF_WIN * REF_WIN * REF_WIN / 32; i += 32) bm[i] = 0u;
  __syncwarp();
  const double dres = (double)res;
  for (long long p = (long long)blockIdx.x * REFW_WARPS + w; p < n_pairs; p += (long long)gridDim.x * REFW_WARPS) {
    const int m = pair_m ? pair_m[p] : (int)(p / ns);
    const int s = pair_s ? pair_s[p] : (int)(p % ns);
    const float4 km = mkeys[m], ks = skeys[s];
    float* To = Tout + 16 * p;
    if (!(isfinite(km.x) && isfinite(km.y) && isfinite(km.z) && isfinite(ks.x) && isfinite(ks.y) &&
          isfinite(ks.z))) {
      if (lane == 0) {
        score[p] = __int_as_float(0x7fc00000);
        eye4(To);
      }
      continue;
    }
    const int beg = moff[m], n = moff[m + 1] - beg;
    const float* grid = mtdf + (size_t)m * REF_VOL;
    const float lo[3] = {__fsub_rn(km.x, half), __fsub_rn(km.y, half), __fsub_rn(km.z, half)};
    const float hi[3] = {__fadd_rn(km.x, half), __fadd_rn(km.y, half), __fadd_rn(km.z, half)};
    float Tm[16], T1[16], T3[16], M[16];
    eye4(Tm);
    Tm[3] = __fsub_rn(km.x, ks.x), Tm[7] = __fsub_rn(km.y, ks.y), Tm[11] = __fsub_rn(km.z, ks.z);
    eye4(T1);
    T1[3] = -km.x, T1[7] = -km.y;
    eye4(T3);
    T3[3] = km.x, T3[7] = km.y;
    {
      float Rs[16];
      eye4(Rs);
      Rs[0] = rot.c1, Rs[4] = rot.s1, Rs[1] = -rot.s1, Rs[5] = rot.c1;
      mm4(T3, Rs, M);
      mm4(M, T1, M);
    }
    float px[REFW_PPT], py[REFW_PPT], pz[REFW_PPT];
#pragma unroll
    for (int q = 0; q < REFW_PPT; ++q) {
      const int j = lane + 32 * q;
      px[q] = py[q] = pz[q] = 0.f;
      if (j < n) {
        const float4 c = mcloud[midx[beg + j]];
        px[q] = c.x, py[q] = c.y, pz[q] = c.z;
        xf3(Tm, px[q], py[q], pz[q]);
      }
    }
    OctBox b0;
    oct_define(b0, lo, hi, dres);
    OctBoxF bf0;
    oct_float(b0, bf0);
    float dtf = 0.f, bestf = 100000000.f;
    int best_i = 0;
    bool bad = false;
    for (int it = 0; it < 36 && !bad; ++it) {
      if (it != 0) {
#pragma unroll
        for (int q = 0; q < REFW_PPT; ++q)
          if (lane + 32 * q < n) xf3(M, px[q], py[q], pz[q]);
      }
      OctBox b = b0;
      OctBoxF bf = bf0;
      for (int round = 0; round < 4 * REF_MAX_DEPTH + 4; ++round) {
        int first = 0x7fffffff;
#pragma unroll
        for (int q = 0; q < REFW_PPT; ++q) {
          const int j = lane + 32 * q;
          if (j < n && first == 0x7fffffff && oct_outside_f(bf, px[q], py[q], pz[q])) first = j;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) first = min(first, __shfl_xor_sync(0xffffffffu, first, o));
        if (first == 0x7fffffff) break;
        const int q0 = first >> 5, src = first & 31;
        float sx = 0.f, sy = 0.f, sz = 0.f;
#pragma unroll
        for (int q = 0; q < REFW_PPT; ++q)
          if (q == q0) sx = px[q], sy = py[q], sz = pz[q];
        sx = __shfl_sync(0xffffffffu, sx, src);
        sy = __shfl_sync(0xffffffffu, sy, src);
        sz = __shfl_sync(0xffffffffu, sz, src);
        if (!oct_fit(b, sx, sy, sz, dres)) {
          bad = true;
          break;
        }
        oct_float(b, bf);
      }
      if (bad) break;
      // keys packed 21 bits per axis; the Morton code only for the first leaf
      unsigned long long pk[REFW_PPT];
      unsigned long long mmin = ~0ull;
      unsigned kmin[3] = {~0u, ~0u, ~0u}, kmax[3] = {0u, 0u, 0u};
#pragma unroll
      for (int q = 0; q < REFW_PPT; ++q) {
        pk[q] = ~0ull;
        if (lane + 32 * q < n) {
          const unsigned kx = oct_key_f(b, bf, px[q], 0, dres, inv), ky = oct_key_f(b, bf, py[q], 1, dres, inv),
                         kz = oct_key_f(b, bf, pz[q], 2, dres, inv);
          pk[q] = (unsigned long long)kx | ((unsigned long long)ky << 21) | ((unsigned long long)kz << 42);
          mmin = min(mmin, morton3(kx, ky, kz, b.depth));
          kmin[0] = min(kmin[0], kx), kmin[1] = min(kmin[1], ky), kmin[2] = min(kmin[2], kz);
          kmax[0] = max(kmax[0], kx), kmax[1] = max(kmax[1], ky), kmax[2] = max(kmax[2], kz);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        mmin = min(mmin, __shfl_xor_sync(0xffffffffu, mmin, o));
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          kmin[a] = min(kmin[a], __shfl_xor_sync(0xffffffffu, kmin[a], o));
          kmax[a] = max(kmax[a], __shfl_xor_sync(0xffffffffu, kmax[a], o));
        }
      }
      const bool window_ok = n == 0 || (kmax[0] - kmin[0] < (unsigned)REF_WIN &&
                                        kmax[1] - kmin[1] < (unsigned)REF_WIN && kmax[2] - kmin[2] < (unsigned)REF_WIN);
      if (!window_ok && lane == 0) atomicOr(err, REF_ERR_WINDOW);
      // the field's integer coordinate of every leaf column of the window,
      // one per lane and axis (a huge negative value where get_Distance's
      // float quotient leaves the int range: the index is then out of range)
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float c = oct_centre(b, kmin[a] + (unsigned)lane, a, dres);
        const float qv = __fdiv_rn(__fsub_rn(c, lo[a]), res);
        s_ix[w][a][lane] = (qv > -2147483648.f && qv < 2147483648.f) ? (long long)__float2int_rz(qv)
                                                                      : -(1ll << 50);
      }
      unsigned long long pk_first;
      {
        unsigned fx, fy, fz;
        demorton3(mmin, b.depth, fx, fy, fz);
        pk_first = (unsigned long long)fx | ((unsigned long long)fy << 21) | ((unsigned long long)fz << 42);
      }
      if (lane == 0) s_u[w] = 0;
      __syncwarp();
      // distinct leaves: the lane that sets a leaf's bit reads its field and
      // lists (Morton code, value); the first leaf's value is never added
      unsigned lw[REFW_PPT];
#pragma unroll
      for (int q = 0; q < REFW_PPT; ++q) {
        lw[q] = 0xffffffffu;
        if (!window_ok || pk[q] == ~0ull) continue;
        const unsigned kx = (unsigned)(pk[q] & 0x1fffffull), ky = (unsigned)((pk[q] >> 21) & 0x1fffffull),
                       kz = (unsigned)(pk[q] >> 42);
        const unsigned lx = kx - kmin[0], ly = ky - kmin[1], lz = kz - kmin[2];
        const unsigned l = lx + REF_WIN * (ly + REF_WIN * lz);
        lw[q] = l >> 5;
        const unsigned bit = 1u << (l & 31u);
        const unsigned old = atomicOr(&bm[l >> 5], bit);
        if (old & bit) continue;
        float v = 0.f;
        if (pk[q] != pk_first) {
          const long long idx = s_ix[w][1][ly] * REF_DIM + s_ix[w][2][lz] * (REF_DIM * REF_DIM) + s_ix[w][0][lx];
          v = (idx >= 0 && idx < REF_VOL) ? __ldg(grid + idx) : 900.f;
        }
        const int slot = atomicAdd(&s_u[w], 1);
        s_key[w][slot] = morton3(kx, ky, kz, b.depth);
        s_val[w][slot] = v;
      }
      __syncwarp();
      const int u = s_u[w];
      int P = 2;
      while (P < u) P <<= 1;
      for (int i = u + lane; i < P; i += 32) s_key[w][i] = ~0ull;
      __syncwarp();
      leaf_sort(s_key[w], s_val[w], P, lane, 32, WarpSync());
      if (lane == 0) {
        dtf = leaf_running_score(dtf, s_val[w], u);
        if (dtf < bestf) {
          bestf = dtf;
          best_i = it;
        }
      }
      __syncwarp();
#pragma unroll
      for (int q = 0; q < REFW_PPT; ++q)
        if (lw[q] != 0xffffffffu) bm[lw[q]] = 0u;
      __syncwarp();
    }
    if (lane != 0) continue;
    if (bad) {
      score[p] = __int_as_float(0x7fc00000);
      eye4(To);
      continue;
    }
    score[p] = bestf;
    float S[16], R2[16], A[16];
    eye4(S);
    const float cs = __fdiv_rn(km.z, ks.z);
    S[0] = S[5] = S[10] = cs;
    eye4(R2);
    R2[0] = rot.c2[best_i], R2[4] = rot.s2[best_i], R2[1] = -rot.s2[best_i], R2[5] = rot.c2[best_i];
    mm4(S, T3, A);
    mm4(A, R2, A);
    mm4(A, T1, A);
    mm4(A, Tm, A);
    for (int i = 0; i < 16; ++i) To[i] = A[i];
  }
}

__global__ void k_ref_sum_counts(const uint32_t* __restrict__ cnt, int n, unsigned long long* __restrict__ out) {
  unsigned long long v = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v += cnt[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(out, v);
}

__global__ void k_ref_max_count(const int* __restrict__ off, int n, int* __restrict__ out) {
  int v = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    v = max(v, off[i + 1] - off[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, v);
}

// ---------------------------------------------------------------------------
// the all-pairs loop's gates (function.h:158-178, as written)
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool ref_gates(float4 km, int mnum, const double* mv3, float4 ks, int snum,
                                          const double* sv3) {
  const float h = __fdiv_rn(km.z, ks.z);
  if (!(h >= 0.f || h <= 1.5f)) return false;
  for (int a = 0; a < 3; ++a) {
    const double r = __ddiv_rn(mv3 ? mv3[a] : 0.16, sv3 ? sv3[a] : 0.16);
    if (r > 3.0 || r < 0.0) return false;
  }
  if (snum == 0) return false;
  const float q = (float)(mnum / snum);
  return !(q > 2.f || q < 0.5f);
}

__global__ void k_ref_gates(const float4* __restrict__ mkeys, const int* __restrict__ mnum,
                            const double* __restrict__ mv3, const float4* __restrict__ skeys,
                            const int* __restrict__ snum, const double* __restrict__ sv3, int ns, long long np,
                            const float* __restrict__ score, float max_score, uint32_t* __restrict__ flags) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x) {
    const int m = (int)(p / ns), s = (int)(p % ns);
    flags[p] = (score[p] < max_score &&
                ref_gates(mkeys[m], mnum[m], mv3 ? mv3 + 3 * (size_t)m : nullptr, skeys[s], snum[s],
                          sv3 ? sv3 + 3 * (size_t)s : nullptr))
                   ? 1u
                   : 0u;
  }
}

__global__ void k_ref_scatter(const uint32_t* __restrict__ flags, const uint32_t* __restrict__ pos, long long np,
                              int cap, int* __restrict__ out) {
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x)
    if (flags[p] && pos[p] < (uint32_t)cap) out[pos[p]] = (int)p;
}

// ---------------------------------------------------------------------------
// Ransac (function.h:35-109): inliers of every kept pair's transform
// ---------------------------------------------------------------------------
constexpr int RANSAC_NT = 256;

__global__ void __launch_bounds__(RANSAC_NT) k_ref_ransac(const float4* __restrict__ mkeys,
                                                          const float4* __restrict__ skeys, int ns,
                                                          const int* __restrict__ pair_idx, int np,
                                                          const float* __restrict__ score,
                                                          const float* __restrict__ T_all, float inlier,
                                                          float max_des, int* __restrict__ cnt) {
  __shared__ int s_c[RANSAC_NT / 32];
  const int i = blockIdx.x, tid = threadIdx.x;
  float Ti[12];
  const float* src = T_all + 16 * (size_t)pair_idx[i];
#pragma unroll
  for (int e = 0; e < 12; ++e) Ti[e] = src[e];
  int c = 0;
  for (int j = tid; j < np; j += RANSAC_NT) {
    const long long p = pair_idx[j];
    const int m = (int)(p / ns), s = (int)(p % ns);
    const float4 sk = skeys[s], k = mkeys[m];
    float x = sk.x, y = sk.y, z = sk.z;
    xf3(Ti, x, y, z);
    const float dx = __fsub_rn(k.x, x), dy = __fsub_rn(k.y, y), dz = __fsub_rn(k.z, z);
    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
    const float dis = __fsqrt_rn(d2);
    if ((double)dis < (double)inlier && score[p] < max_des) ++c;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((tid & 31) == 0) s_c[tid >> 5] = c;
  __syncthreads();
  if (tid == 0) {
    int t = 0;
    for (int w = 0; w < RANSAC_NT / 32; ++w) t += s_c[w];
    cnt[i] = t;
  }
}

// First position with the most inliers (> 0): out[0] = position or -1, out[1] = inliers.
__global__ void k_ref_argmax(const int* __restrict__ cnt, int np, int* __restrict__ out) {
  __shared__ int s_v[32], s_i[32];
  int bv = 0, bi = -1;
  for (int i = threadIdx.x; i < np; i += blockDim.x)
    if (cnt[i] > bv) bv = cnt[i], bi = i;  // ascending i per thread: first max kept
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const int ov = __shfl_xor_sync(0xffffffffu, bv, o), oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ov > bv || (ov == bv && ov > 0 && oi < bi)) bv = ov, bi = oi;
  }
  if ((threadIdx.x & 31) == 0) s_v[threadIdx.x >> 5] = bv, s_i[threadIdx.x >> 5] = bi;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
      if (s_v[w] > bv || (s_v[w] == bv && bv > 0 && s_i[w] < bi)) bv = s_v[w], bi = s_i[w];
    out[0] = bv > 0 ? bi : -1;
    out[1] = bv;
  }
}

static RefRot ref_rot_tables() {
  RefRot r;
  const float theta = (float)(3.14159265358979323846 / 18);  // M_PI / 18 rounded to float
  r.c1 = cosf(theta);
  r.s1 = sinf(theta);
  for (int i = 0; i < 36; ++i) {
    const float th = (float)i * theta;
    r.c2[i] = (float)cos((double)th);
    r.s2[i] = (float)sin((double)th);
  }
  return r;
}

static rtr_status ref_read_ints(rtr_context* ctx, const int* d, int n, cudaStream_t st, int* h) {
  if (!ctx->h_pin || n > 64) return fail(RTR_ERR_CUDA, "rtr_ref: pinned staging missing");
  RTR_CUDA(cudaMemcpyAsync(ctx->h_pin, d, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, st));
  RTR_CUDA(cudaStreamSynchronize(st));
  memcpy(h, ctx->h_pin, sizeof(int) * (size_t)n);
  return RTR_OK;
}

static rtr_status ref_check_err(int e, const char* who) {
  if (e & REF_ERR_DEPTH)
    return fail(RTR_ERR_INVALID_ARG, "%s: the box spans more than %d octree levels (half / res too large)", who,
                REF_OCC_DEPTH);
  if (e & REF_ERR_GROW)
    return fail(RTR_ERR_INVALID_ARG, "%s: occupancy points outside the field's box (occupancy box wider)", who);
  if (e & REF_ERR_WINDOW)
    return fail(RTR_ERR_INVALID_ARG, "%s: a rotated occupancy cloud spans more than %d leaves (occupancy box too "
                "wide for this resolution)", who, REF_WIN);
  return RTR_OK;
}

}  // namespace rtr

using namespace rtr;

extern "C" {

rtr_status rtr_ref_occupancy(rtr_context* ctx, const float* d_cloud, int n, const float* d_keys, int n_keys,
                             float resolution, float half_box, int32_t* d_number, int32_t* d_offsets,
                             int32_t* d_indices, long long cap_indices, long long* h_total, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n >= 0 && n_keys >= 0 && h_total, "rtr_ref_occupancy: bad arguments");
  RTR_CHECK_ARG(resolution > 0.f && half_box > 0.f && isfinite(resolution) && isfinite(half_box),
                "rtr_ref_occupancy: resolution and half_box must be positive");
  RTR_CHECK_ARG(2.0 * half_box / resolution <= 30.0, "rtr_ref_occupancy: half_box / resolution above 15");
  *h_total = 0;
  RTR_CHECK_ARG(d_offsets, "rtr_ref_occupancy: NULL offsets");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (n_keys == 0) {
    RTR_CUDA(cudaMemsetAsync(d_offsets, 0, sizeof(int32_t), st));
    RTR_CUDA(cudaStreamSynchronize(st));
    return RTR_OK;
  }
  RTR_CHECK_ARG(d_keys && d_number && (n == 0 || d_cloud), "rtr_ref_occupancy: NULL input");
  ScratchPlan plan;
  const size_t o_cnt = plan.add<uint32_t>((size_t)n_keys + 1);
  const size_t o_tiles = plan.add<uint32_t>((size_t)scan_tiles(n_keys + 1));
  const size_t o_err = plan.add<int>(4);
  const size_t o_tot = plan.add<unsigned long long>(1);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  uint32_t* cnt = reinterpret_cast<uint32_t*>(s.base + o_cnt);
  uint32_t* tiles = reinterpret_cast<uint32_t*>(s.base + o_tiles);
  int* err = reinterpret_cast<int*>(s.base + o_err);
  unsigned long long* tot64 = reinterpret_cast<unsigned long long*>(s.base + o_tot);
  ProfScope ps(ctx, st, "ref_occupancy");
  RTR_CUDA(cudaMemsetAsync(err, 0, 4 * sizeof(int), st));
  RTR_CUDA(cudaMemsetAsync(tot64, 0, sizeof(unsigned long long), st));
  RTR_CUDA(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * ((size_t)n_keys + 1), st));
  const float4* cloud = reinterpret_cast<const float4*>(d_cloud);
  const float4* keys = reinterpret_cast<const float4*>(d_keys);
  k_ref_occ<<<n_keys, OCC_NT, 0, st>>>(cloud, n, keys, resolution, half_box, false, reinterpret_cast<int*>(cnt),
                                       d_number, nullptr, nullptr, err);
  // offsets = exclusive scan over n_keys + 1 counts (the last is 0): offsets[n_keys] = total
  scan_exclusive(cnt, reinterpret_cast<uint32_t*>(d_offsets), tiles, n_keys + 1, n_keys + 1, nullptr, nullptr, st);
  k_ref_sum_counts<<<(n_keys + 255) / 256 < 1024 ? (n_keys + 255) / 256 : 1024, 256, 0, st>>>(cnt, n_keys, tot64);
  RTR_LAUNCHED(3);
  int h[4];
  RTR_TRY(ref_read_ints(ctx, err, 4, st, h));
  RTR_TRY(ref_check_err(h[0], "rtr_ref_occupancy"));
  int h2[2];
  RTR_TRY(ref_read_ints(ctx, reinterpret_cast<const int*>(tot64), 2, st, h2));
  unsigned long long total64 = 0;
  memcpy(&total64, h2, sizeof(total64));
  const long long total = (long long)total64;
  *h_total = total;
  if (total > 0x7fffffffLL)
    return fail(RTR_ERR_CAPACITY, "rtr_ref_occupancy: %lld indices (offsets are 32-bit: at most 2^31 - 1)", total);
  if (total > cap_indices) return fail(RTR_ERR_CAPACITY, "rtr_ref_occupancy: %lld indices, capacity %lld", total,
                                       cap_indices);
  if (total > 0) {
    RTR_CHECK_ARG(d_indices, "rtr_ref_occupancy: NULL indices");
    k_ref_occ<<<n_keys, OCC_NT, 0, st>>>(cloud, n, keys, resolution, half_box, true, nullptr, nullptr, d_offsets,
                                         d_indices, err);
    RTR_LAUNCHED(1);
  }
  RTR_CUDA(cudaGetLastError());
  RTR_CUDA(cudaStreamSynchronize(st));
  return RTR_OK;
}

rtr_status rtr_ref_tdf(rtr_context* ctx, const float* d_cloud, const float* d_keys, int n_keys,
                       const int32_t* d_offsets, const int32_t* d_indices, float resolution, float half_tdf,
                       float* d_tdf, int* h_dim, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n_keys >= 0, "rtr_ref_tdf: bad arguments");
  RTR_CHECK_ARG(resolution > 0.f && half_tdf > 0.f && isfinite(resolution) && isfinite(half_tdf),
                "rtr_ref_tdf: resolution and half_tdf must be positive");
  const int dim = (int)(half_tdf / resolution * 2);  // key_point.h:313, in float
  RTR_CHECK_ARG(dim >= 1 && dim <= REF_DIM && 2.0 * half_tdf / resolution <= 31.0,
                "rtr_ref_tdf: dim %d outside [1, 30]", dim);
  if (h_dim) *h_dim = dim;
  if (n_keys == 0) return RTR_OK;
  RTR_CHECK_ARG(d_cloud && d_keys && d_offsets && d_tdf, "rtr_ref_tdf: NULL input or output");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  int h_last = 0;
  RTR_TRY(ref_read_ints(ctx, d_offsets + n_keys, 1, st, &h_last));
  RTR_CHECK_ARG(h_last >= 0, "rtr_ref_tdf: bad offsets");
  RTR_CHECK_ARG(h_last == 0 || d_indices, "rtr_ref_tdf: NULL indices");
  ScratchPlan plan;
  const size_t o_cnt = plan.add<uint32_t>((size_t)n_keys + 1);
  const size_t o_off = plan.add<uint32_t>((size_t)n_keys + 1);
  const size_t o_tiles = plan.add<uint32_t>((size_t)scan_tiles(n_keys + 1));
  const size_t o_err = plan.add<int>(4);
  const size_t o_occ = plan.add<int>(3 * (size_t)(h_last > 0 ? h_last : 1));
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  uint32_t* cnt = reinterpret_cast<uint32_t*>(s.base + o_cnt);
  uint32_t* coff = reinterpret_cast<uint32_t*>(s.base + o_off);
  uint32_t* tiles = reinterpret_cast<uint32_t*>(s.base + o_tiles);
  int* err = reinterpret_cast<int*>(s.base + o_err);
  int* occ = reinterpret_cast<int*>(s.base + o_occ);
  ProfScope ps(ctx, st, "ref_tdf");
  RTR_CUDA(cudaMemsetAsync(err, 0, 4 * sizeof(int), st));
  RTR_CUDA(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * ((size_t)n_keys + 1), st));
  const float4* cloud = reinterpret_cast<const float4*>(d_cloud);
  const float4* keys = reinterpret_cast<const float4*>(d_keys);
  k_ref_tdf_cells<<<n_keys, OCC_NT, 0, st>>>(cloud, keys, d_offsets, d_indices, resolution, half_tdf, false,
                                             reinterpret_cast<int*>(cnt), nullptr, nullptr, err);
  scan_exclusive(cnt, coff, tiles, n_keys + 1, n_keys + 1, nullptr, nullptr, st);
  k_ref_tdf_cells<<<n_keys, OCC_NT, 0, st>>>(cloud, keys, d_offsets, d_indices, resolution, half_tdf, true,
                                             nullptr, reinterpret_cast<const int*>(coff), occ, err);
  RTR_LAUNCHED(3);
  int h[4];
  RTR_TRY(ref_read_ints(ctx, err, 4, st, h));
  RTR_TRY(ref_check_err(h[0], "rtr_ref_tdf"));
  RTR_TRY(rtr_tdf_batch(ctx, occ, reinterpret_cast<const int*>(coff), n_keys, dim, d_tdf, stream));
  RTR_CUDA(cudaStreamSynchronize(st));
  return RTR_OK;
}

}  // extern "C"

// Dynamic shared memory of k_ref_distance<NT>: the sort list of a rotation's
// distinct leaves, 8-byte codes and 4-byte values, one per cloud point.
static size_t ref_leaf_smem(int nt) { return (size_t)nt * REF_PPT * (sizeof(unsigned long long) + sizeof(float)); }

template <int NT>
static rtr_status ref_distance_smem() {
  // the attribute is per function and device; setting it again is harmless
  RTR_CUDA(cudaFuncSetAttribute(k_ref_distance<NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)ref_leaf_smem(NT)));
  return RTR_OK;
}

extern "C" {

rtr_status rtr_ref_distance(rtr_context* ctx, const float* d_mcloud, const float* d_mkeys, int n_model,
                            const int32_t* d_moffsets, const int32_t* d_mindices, const float* d_mtdf,
                            const float* d_skeys, int n_scan, const int32_t* d_pair_m, const int32_t* d_pair_s,
                            long long n_pairs, float resolution, float half_tdf, float* d_score, float* d_T,
                            rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n_model >= 0 && n_scan >= 0, "rtr_ref_distance: bad arguments");
  RTR_CHECK_ARG(resolution > 0.f && half_tdf > 0.f && isfinite(resolution) && isfinite(half_tdf),
                "rtr_ref_distance: resolution and half_tdf must be positive");
  RTR_CHECK_ARG((int)(half_tdf / resolution * 2) == REF_DIM,
                "rtr_ref_distance: the field must be 30^3 voxels (get_Distance reads it as 30^3)");
  const bool all = d_pair_m == nullptr;
  RTR_CHECK_ARG(all == (d_pair_s == nullptr), "rtr_ref_distance: pair_m and pair_s both or neither");
  if (all) n_pairs = (long long)n_model * n_scan;
  RTR_CHECK_ARG(n_pairs >= 0 && n_pairs <= 0x7fffffffLL, "rtr_ref_distance: %lld pairs (at most 2^31 - 1)",
                n_pairs);
  if (n_pairs == 0) return RTR_OK;
  RTR_CHECK_ARG(n_model > 0 && n_scan > 0 && d_mcloud && d_mkeys && d_moffsets && d_mtdf && d_skeys && d_score &&
                    d_T,
                "rtr_ref_distance: NULL input or output");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  ScratchPlan plan;
  const size_t o_err = plan.add<int>(4);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  int* err = reinterpret_cast<int*>(s.base + o_err);
  RTR_CUDA(cudaMemsetAsync(err, 0, 4 * sizeof(int), st));
  k_ref_max_count<<<(n_model + 255) / 256, 256, 0, st>>>(d_moffsets, n_model, err + 1);
  RTR_LAUNCHED(1);
  int h[4];
  RTR_TRY(ref_read_ints(ctx, err, 4, st, h));
  const int nmax = h[1];
  if (nmax > 0) RTR_CHECK_ARG(d_mindices, "rtr_ref_distance: NULL indices");
  if (nmax > REF_PPT * 1024)
    return fail(RTR_ERR_CAPACITY, "rtr_ref_distance: an occupancy cloud of %d points (at most %d)", nmax,
                REF_PPT * 1024);
  if (!all) {
    // every pair index inside [0, n_model) x [0, n_scan): checked on the host
    std::vector<int32_t> pm((size_t)n_pairs), ps_((size_t)n_pairs);
    RTR_CUDA(cudaMemcpyAsync(pm.data(), d_pair_m, sizeof(int32_t) * (size_t)n_pairs, cudaMemcpyDeviceToHost, st));
    RTR_CUDA(cudaMemcpyAsync(ps_.data(), d_pair_s, sizeof(int32_t) * (size_t)n_pairs, cudaMemcpyDeviceToHost, st));
    RTR_CUDA(cudaStreamSynchronize(st));
    for (long long i = 0; i < n_pairs; ++i)
      RTR_CHECK_ARG(pm[(size_t)i] >= 0 && pm[(size_t)i] < n_model && ps_[(size_t)i] >= 0 && ps_[(size_t)i] < n_scan,
                    "rtr_ref_distance: pair %lld = (%d, %d) out of range", i, pm[(size_t)i], ps_[(size_t)i]);
  }
  const RefRot rot = ref_rot_tables();
  ProfScope ps(ctx, st, "ref_distance");
  const float4* mc = reinterpret_cast<const float4*>(d_mcloud);
  const float4* mk = reinterpret_cast<const float4*>(d_mkeys);
  const float4* sk = reinterpret_cast<const float4*>(d_skeys);
  const unsigned nb = (unsigned)n_pairs;
  if (nmax <= REFW_PPT * 32) {
    const long long nbw = (n_pairs + REFW_WARPS - 1) / REFW_WARPS;
    k_ref_distance_warp<<<(unsigned)nbw, 32 * REFW_WARPS, 0, st>>>(mc, mk, d_moffsets, d_mindices, d_mtdf, sk, n_scan,
                                                                   d_pair_m, d_pair_s, n_pairs, resolution, half_tdf,
                                                                   rot, d_score, d_T, err);
  } else if (nmax <= REF_PPT * 256) {
    RTR_TRY(ref_distance_smem<256>());
    k_ref_distance<256><<<nb, 256, ref_leaf_smem(256), st>>>(mc, mk, d_moffsets, d_mindices, d_mtdf, sk, n_scan,
                                                             d_pair_m, d_pair_s, resolution, half_tdf, rot, d_score,
                                                             d_T, err);
  } else if (nmax <= REF_PPT * 512) {
    RTR_TRY(ref_distance_smem<512>());
    k_ref_distance<512><<<nb, 512, ref_leaf_smem(512), st>>>(mc, mk, d_moffsets, d_mindices, d_mtdf, sk, n_scan,
                                                             d_pair_m, d_pair_s, resolution, half_tdf, rot, d_score,
                                                             d_T, err);
  } else {
    RTR_TRY(ref_distance_smem<1024>());
    k_ref_distance<1024><<<nb, 1024, ref_leaf_smem(1024), st>>>(mc, mk, d_moffsets, d_mindices, d_mtdf, sk, n_scan,
                                                                d_pair_m, d_pair_s, resolution, half_tdf, rot, d_score,
                                                                d_T, err);
  }
  RTR_LAUNCHED(1);
  RTR_CUDA(cudaGetLastError());
  RTR_TRY(ref_read_ints(ctx, err, 4, st, h));
  return ref_check_err(h[0], "rtr_ref_distance");
}

rtr_status rtr_ref_correspond(rtr_context* ctx, const float* d_mkeys, const int32_t* d_mnumber, const double* d_mv3,
                              int n_model, const float* d_skeys, const int32_t* d_snumber, const double* d_sv3,
                              int n_scan, const float* d_score_all, float max_score, int32_t* d_pair_idx, int cap,
                              int* h_n_pairs, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n_model >= 0 && n_scan >= 0 && cap >= 0 && h_n_pairs, "rtr_ref_correspond: bad arguments");
  *h_n_pairs = 0;
  const long long np = (long long)n_model * n_scan;
  RTR_CHECK_ARG(np <= (1LL << 30), "rtr_ref_correspond: %lld pairs (at most 2^30)", np);
  if (np == 0) return RTR_OK;
  RTR_CHECK_ARG(d_mkeys && d_mnumber && d_skeys && d_snumber && d_score_all, "rtr_ref_correspond: NULL input");
  RTR_CHECK_ARG(cap == 0 || d_pair_idx, "rtr_ref_correspond: NULL output");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  ScratchPlan plan;
  const size_t o_f = plan.add<uint32_t>((size_t)np + 1);
  const size_t o_p = plan.add<uint32_t>((size_t)np + 1);
  const size_t o_tiles = plan.add<uint32_t>((size_t)scan_tiles((int)np + 1));
  const size_t o_tot = plan.add<uint32_t>(4);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  uint32_t* flags = reinterpret_cast<uint32_t*>(s.base + o_f);
  uint32_t* pos = reinterpret_cast<uint32_t*>(s.base + o_p);
  uint32_t* tiles = reinterpret_cast<uint32_t*>(s.base + o_tiles);
  uint32_t* tot = reinterpret_cast<uint32_t*>(s.base + o_tot);
  ProfScope ps(ctx, st, "ref_correspond");
  RTR_CUDA(cudaMemsetAsync(flags + np, 0, sizeof(uint32_t), st));
  const int nb = (int)((np + 255) / 256 < 65535 ? (np + 255) / 256 : 65535);
  k_ref_gates<<<nb, 256, 0, st>>>(reinterpret_cast<const float4*>(d_mkeys), d_mnumber, d_mv3,
                                  reinterpret_cast<const float4*>(d_skeys), d_snumber, d_sv3, n_scan, np, d_score_all,
                                  max_score, flags);
  scan_exclusive(flags, pos, tiles, (int)np + 1, (int)np + 1, nullptr, tot, st);
  k_ref_scatter<<<nb, 256, 0, st>>>(flags, pos, np, cap, d_pair_idx);
  RTR_LAUNCHED(3);
  RTR_CUDA(cudaGetLastError());
  int h[1];
  RTR_TRY(ref_read_ints(ctx, reinterpret_cast<const int*>(tot), 1, st, h));
  *h_n_pairs = h[0];
  if (h[0] > cap) return fail(RTR_ERR_CAPACITY, "rtr_ref_correspond: %d pairs, capacity %d", h[0], cap);
  return RTR_OK;
}

rtr_status rtr_ref_ransac(rtr_context* ctx, const float* d_mkeys, int n_model, const float* d_skeys, int n_scan,
                          const int32_t* d_pair_idx, int n_pairs, const float* d_score_all, const float* d_T_all,
                          float inlier_dist, float max_des, float* h_T, int* h_inliers, int* h_best,
                          rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && n_model > 0 && n_scan > 0 && n_pairs >= 0 && h_T && h_inliers && h_best,
                "rtr_ref_ransac: bad arguments");
  for (int i = 0; i < 16; ++i) h_T[i] = (i % 5) == 0 ? 1.f : 0.f;
  *h_inliers = 0;
  *h_best = -1;
  if (n_pairs == 0) return RTR_OK;
  RTR_CHECK_ARG(d_mkeys && d_skeys && d_pair_idx && d_score_all && d_T_all, "rtr_ref_ransac: NULL input");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  {
    // every pair index inside the n_model x n_scan table: checked on the host
    std::vector<int32_t> pi((size_t)n_pairs);
    RTR_CUDA(cudaMemcpyAsync(pi.data(), d_pair_idx, sizeof(int32_t) * (size_t)n_pairs, cudaMemcpyDeviceToHost, st));
    RTR_CUDA(cudaStreamSynchronize(st));
    const long long np_all = (long long)n_model * n_scan;
    for (int i = 0; i < n_pairs; ++i)
      RTR_CHECK_ARG(pi[(size_t)i] >= 0 && pi[(size_t)i] < np_all, "rtr_ref_ransac: pair index %d = %d out of range", i,
                    pi[(size_t)i]);
  }
  ScratchPlan plan;
  const size_t o_c = plan.add<int>((size_t)n_pairs);
  const size_t o_o = plan.add<int>(4);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  int* cnt = reinterpret_cast<int*>(s.base + o_c);
  int* out = reinterpret_cast<int*>(s.base + o_o);
  ProfScope ps(ctx, st, "ref_ransac");
  k_ref_ransac<<<n_pairs, RANSAC_NT, 0, st>>>(reinterpret_cast<const float4*>(d_mkeys),
                                              reinterpret_cast<const float4*>(d_skeys), n_scan, d_pair_idx, n_pairs,
                                              d_score_all, d_T_all, inlier_dist, max_des, cnt);
  k_ref_argmax<<<1, 1024, 0, st>>>(cnt, n_pairs, out);
  RTR_LAUNCHED(2);
  RTR_CUDA(cudaGetLastError());
  int h[2];
  RTR_TRY(ref_read_ints(ctx, out, 2, st, h));
  *h_best = h[0];
  *h_inliers = h[1];
  if (h[0] >= 0) {
    int pidx = 0;
    RTR_CUDA(cudaMemcpyAsync(ctx->h_pin, d_pair_idx + h[0], sizeof(int), cudaMemcpyDeviceToHost, st));
    RTR_CUDA(cudaStreamSynchronize(st));
    pidx = ctx->h_pin[0];
    RTR_CUDA(cudaMemcpyAsync(h_T, d_T_all + 16 * (size_t)pidx, 16 * sizeof(float), cudaMemcpyDeviceToHost, st));
    RTR_CUDA(cudaStreamSynchronize(st));
  }
  return RTR_OK;
}

}  // extern "C"
