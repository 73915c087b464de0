// common.cuh — shared device helpers, context internals and error plumbing for
// the rtr_* C ABI (include/rtr.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string>

#include "../../include/rtr.h"

#define RTR_VERSION_STRING "0.1.0"

// ---------------------------------------------------------------------------
// error plumbing (host)
// ---------------------------------------------------------------------------
namespace rtr {

void set_error(const char* fmt, ...);
rtr_status fail(rtr_status st, const char* fmt, ...);
rtr_status cuda_fail(cudaError_t e, const char* what, const char* file, int line);

}  // namespace rtr

#define RTR_CUDA(call)                                                        \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) return rtr::cuda_fail(e_, #call, __FILE__, __LINE__); \
  } while (0)

#define RTR_TRY(call)                   \
  do {                                  \
    rtr_status s_ = (call);             \
    if (s_ != RTR_OK) return s_;        \
  } while (0)

#define RTR_CHECK_ARG(cond, ...)                                   \
  do {                                                             \
    if (!(cond)) return rtr::fail(RTR_ERR_INVALID_ARG, __VA_ARGS__); \
  } while (0)

// ---------------------------------------------------------------------------
// context (host) + scratch arena
// ---------------------------------------------------------------------------
#include <atomic>
#include <vector>

namespace rtr {
extern std::atomic<uint64_t> g_launches;
// A number no other model or network of this process has had (never 0).
uint64_t next_uid();
}
// Count kernel launches issued by the library (rtr_launch_count).
#define RTR_LAUNCHED(n) (rtr::g_launches.fetch_add((n), std::memory_order_relaxed))

struct rtr_prof_rec {
  const char* name;
  cudaEvent_t a, b;
};

// The last recognition enqueued on a context and, once the same call has been
// made twice in a row, its launches captured as a CUDA graph (pipeline.cu).
// The key holds everything the enqueued work depends on: the inputs' device
// addresses, the parameters, the model's and network's identities, the
// arena's generation and the context's configuration generation.
struct RecogGraphSlot {
  const void* model = nullptr;
  uint64_t model_uid = 0;
  const void* mlp = nullptr;
  uint64_t mlp_uid = 0;
  float keep = 0.f;
  const float* scene = nullptr;
  int n = 0;
  void* result = nullptr;
  rtr_recog_params params{};
  unsigned scratch_gen = 0, cfg_gen = 0;
  bool armed = false;   // this key ran once directly (the arena is sized for it)
  bool failed = false;  // its capture failed: it stays direct
  cudaGraphExec_t exec = nullptr;
  uint64_t launches = 0;  // kernels in the graph
};

struct rtr_context {
  int device = 0;
  int num_sms = 0;
  int max_smem_optin = 0;
  void* arena = nullptr;        // scratch arena (device)
  unsigned scratch_gen = 0;     // times the arena was (re)allocated: a captured graph is valid only for one
  size_t arena_bytes = 0;
  int* d_status = nullptr;      // device status word written by persistent kernels
  unsigned* d_sync = nullptr;   // 64 words of barrier counters for persistent kernels
  double wait_budget_ms = 2000.0;
  long long wait_budget_cycles = 0;
  int clock_khz = 0;
  void* io = nullptr;           // device staging for the host-pointer entry points
  size_t io_bytes = 0;
  cudaStream_t host_stream = nullptr;  // stream of the host-pointer entry points
  int* h_pin = nullptr;                // 64 pinned ints for small device->host reads
  int tune_icp_group = 0;              // lanes per ICP source point (0: automatic)
  size_t scratch_limit = 0;            // largest scratch arena this context may hold (0: no limit)
  int tune_batch_workers = 0;          // workers of rtr_recognize_batch (0: automatic)
  int coop_div = 1;                    // cooperative grids use 1/coop_div of the GPU
  int tune_gc_window = 0;              // seeds per grouping window (0: automatic)
  int tune_gc_no_lists = 0;            // 1: the grouping keeps no pass lists (every stale set ends a round)
  int tune_gc_inline = 0;              // sets the grouping walk recomputes in place per round (0: automatic)
  int tune_scene_grid_mm = 0;          // cell edge of the recognition's scene grid (0: 1.5 ICP distances)
  int tune_normals_grid_mm = 0;        // cell edge of the scene normals' k-NN grid (0: 5 voxel leaves)
  std::vector<rtr_context*> workers;   // child contexts of the batch driver
  cudaEvent_t ev_fork = nullptr;       // fork/join event of the batch driver
  int gc_stats[8] = {};                // last grouping: rounds, walk end, sets, phase us, candidates
  bool profiling = false;
  std::vector<rtr_prof_rec> prof;      // recorded stages (in order)
  std::vector<cudaEvent_t> event_pool; // reusable events
  int auto_graph = 1;                  // replay repeated recognitions from a CUDA graph
  unsigned cfg_gen = 0;                // bumped by every tuning or wait-budget change
  cudaStream_t cap_stream = nullptr;   // private stream that graphs are captured on
  RecogGraphSlot rgraph;
  cudaStream_t side_stream = nullptr;  // second stream of a recognition's independent stages
  cudaEvent_t ev_side[3] = {};         // its fork and join events
};

namespace rtr {

// Bump allocator over the context arena.  A top-level call first sums what it
// needs (ScratchPlan), ensures the arena holds it, then carves pointers.
struct ScratchPlan {
  size_t bytes = 0;
  template <class T>
  size_t add(size_t n) {
    size_t off = (bytes + 255) & ~size_t(255);
    bytes = off + n * sizeof(T);
    return off;
  }
};

struct Scratch {
  char* base = nullptr;
  size_t off = 0, cap = 0;
  template <class T>
  T* take(size_t n) {
    size_t o = (off + 255) & ~size_t(255);
    if (o + n * sizeof(T) > cap) return nullptr;
    off = o + n * sizeof(T);
    return reinterpret_cast<T*>(base + o);
  }
};

// Ensure the arena holds `bytes`; grows (synchronising) unless `stream` is
// being captured, in which case RTR_ERR_CAPACITY is returned.
rtr_status ensure_scratch(rtr_context* ctx, size_t bytes, cudaStream_t stream, Scratch* out);

bool stream_is_capturing(cudaStream_t s);

// Create the context's side stream and its events on first use.
rtr_status side_stream_ready(rtr_context* ctx);

// Worker contexts of a batch (batch.cu): make sure `n` exist and share the
// GPU's co-resident blocks; how many a call of `n_items` uses; and their
// status words after a synchronised batch.
rtr_status batch_ensure_workers(rtr_context* ctx, int n);
int batch_worker_count(const rtr_context* ctx, int n_items);
rtr_status batch_check_workers(rtr_context* ctx, int nw);

// Grow the host-entry staging buffer (synchronises when it grows).
rtr_status ensure_io(rtr_context* ctx, size_t bytes);

// Records a named event pair around a stage when ctx->profiling is on.
struct ProfScope {
  rtr_context* ctx;
  cudaStream_t st;
  int slot = -1;
  ProfScope(rtr_context* c, cudaStream_t s, const char* name);
  void end();
  ~ProfScope() { end(); }
};

// A prepared descriptor database's FP32 side: the squared norms [ndb], their
// maximum, then (8-byte aligned) the packed answer for an all-zero query.
inline int db_norm_floats(int ndb) { return ((ndb + 2) & ~1) + 2; }
__host__ __device__ inline unsigned long long* db_zero_key(float* n2, int ndb) {
  return reinterpret_cast<unsigned long long*>(n2 + ((ndb + 2) & ~1));
}
__host__ __device__ inline const unsigned long long* db_zero_key(const float* n2, int ndb) {
  return reinterpret_cast<const unsigned long long*>(n2 + ((ndb + 2) & ~1));
}

}  // namespace rtr

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
#ifdef __CUDACC__

// Squared distance with every operation rounded separately:
// ((dx*dx + dy*dy) + dz*dz), dx = q.x - p.x.  The CPU oracle uses the same
// expression with floating-point contraction disabled.
__device__ __forceinline__ float dist2_exact(float4 q, float4 p) {
  float dx = __fsub_rn(q.x, p.x), dy = __fsub_rn(q.y, p.y), dz = __fsub_rn(q.z, p.z);
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// y = R p + t with R, t in FP32, each row evaluated as ((r0*x + r1*y) + r2*z) + t.
__device__ __forceinline__ float4 xform_exact(const float* T12, float4 p) {
  float4 o;
  o.x = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T12[0], p.x), __fmul_rn(T12[1], p.y)), __fmul_rn(T12[2], p.z)), T12[3]);
  o.y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T12[4], p.x), __fmul_rn(T12[5], p.y)), __fmul_rn(T12[6], p.z)), T12[7]);
  o.z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T12[8], p.x), __fmul_rn(T12[9], p.y)), __fmul_rn(T12[10], p.z)), T12[11]);
  o.w = 0.f;
  return o;
}

// Knuth TwoSum: s + e == a + b exactly.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  float bp = __fsub_rn(s, a);
  float ap = __fsub_rn(s, bp);
  e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
}

// Kahan–Babuška (Neumaier) accumulator.
struct KSum {
  float s, c;
  __device__ __forceinline__ void init() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    float t, e;
    two_sum(s, x, t, e);
    s = t;
    c = __fadd_rn(c, e);
  }
};

// Warp-level compensated reduction of (s, c) pairs; lane 0 holds the result.
__device__ __forceinline__ void warp_ksum(float& s, float& c) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    float s2 = __shfl_down_sync(0xffffffffu, s, off);
    float c2 = __shfl_down_sync(0xffffffffu, c, off);
    float t, e;
    two_sum(s, s2, t, e);
    s = t;
    c = __fadd_rn(__fadd_rn(c, c2), e);
  }
}

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Float <-> order-preserving unsigned (for atomicMin/Max on floats).
__device__ __forceinline__ unsigned float_to_ordered(float f) {
  unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ordered_to_float(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

#endif  // __CUDACC__
