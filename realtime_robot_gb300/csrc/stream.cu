// stream.cu — the streaming workload: depth frames, back-projection and the
// voxel-hash fusion map.
//
// Depth frames are organised (W x H) float32 images of z in metres (0 = no
// return), pinhole (fx, fy, cx, cy); poses map camera coordinates (x right,
// y down, z forward) to world coordinates.
//
// Fusion map: an open-addressing hash table of 5 mm voxels (linear probing,
// 64-bit keys claimed with atomicCAS, at most MAP_MAX_PROBE slots looked at
// per insert: a point that finds no slot within them sets the table's full
// flag and is dropped, so a table run past its capacity stays fast and is
// reported instead of degrading into scans of the whole table).  Each voxel keeps its point count and
// the sum of its points' offsets from the voxel's lower corner in fixed point
// (units of 2^-40 m, unsigned 64-bit atomics).  Integer sums do not depend on
// the order of the adds, so the map's contents (count and mean per voxel)
// are the same on every run whatever the thread schedule; only the slot a
// voxel lands in depends on it.
#include <math.h>

#include "common.cuh"
#include "scan.cuh"

struct rtr_map {
  int device = 0;
  float voxel = 0.005f;
  int cap = 0;                          // slots (power of two)
  unsigned long long* keys = nullptr;   // [cap], ~0 = empty
  unsigned long long* sums = nullptr;   // [cap][3] fixed-point offset sums
  unsigned* counts = nullptr;           // [cap]
  int* d_full = nullptr;                // set when an insert found no free slot
};

namespace rtr {

constexpr unsigned long long MAP_EMPTY = ~0ull;
constexpr double MAP_FIX = 1099511627776.0;  // 2^40 fixed-point units per metre
// With splitmix keys at load <= 1/2 a probe run of 256 has probability far
// below 1e-30; a run this long means the table is (nearly) full.
constexpr int MAP_MAX_PROBE = 256;

__device__ __forceinline__ unsigned long long splitmix(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// ---------------------------------------------------------------------------
// ray-cast depth frames of the room (floor z = 0, walls x = -2.5 and y = 2.5,
// furniture boxes)
// ---------------------------------------------------------------------------
struct BoxDev {
  float c, s, x, y;     // instance yaw (cos, sin) and position
  float lo[3], hi[3];   // box in the object frame
  float shape, inst;
};

__device__ float ray_box_obj(const float o[3], const float d[3], const float lo[3], const float hi[3]) {
  float t0 = -1e30f, t1 = 1e30f;
  for (int a = 0; a < 3; ++a) {
    if (fabsf(d[a]) < 1e-12f) {
      if (o[a] < lo[a] || o[a] > hi[a]) return -1.f;
      continue;
    }
    float ta = (lo[a] - o[a]) / d[a], tb = (hi[a] - o[a]) / d[a];
    if (ta > tb) {
      const float t = ta;
      ta = tb;
      tb = t;
    }
    t0 = fmaxf(t0, ta);
    t1 = fminf(t1, tb);
    if (t0 > t1) return -1.f;
  }
  if (t1 < 1e-6f) return -1.f;
  return t0 > 1e-6f ? t0 : -1.f;
}

// One thread per pixel of one frame.  The ray direction is R (u', v', 1), so
// its parameter t is the depth z directly.  Noise: N(0, (k z^2)^2) from a
// counter-based hash of (seed, frame, pixel).
__global__ void k_raycast_depth(const BoxDev* __restrict__ boxes, int nbox, const float* __restrict__ poses12,
                                int W, int H, float fx, float fy, float cx, float cy, float noise_k,
                                unsigned long long seed, float max_depth, float* __restrict__ depth) {
  const int f = blockIdx.y;
  const float* T = poses12 + 12 * f;
  for (int px = blockIdx.x * blockDim.x + threadIdx.x; px < W * H; px += gridDim.x * blockDim.x) {
    const int u = px % W, v = px / W;
    const float a = ((float)u - cx) / fx, b = ((float)v - cy) / fy;
    float d[3], o[3];
    for (int k = 0; k < 3; ++k) {
      d[k] = T[4 * k + 0] * a + T[4 * k + 1] * b + T[4 * k + 2];
      o[k] = T[4 * k + 3];
    }
    float best = 1e30f;
    if (d[2] < -1e-9f) {  // floor
      const float t = -o[2] / d[2];
      const float x = o[0] + t * d[0], y = o[1] + t * d[1];
      if (fabsf(x) <= 2.5f && fabsf(y) <= 2.5f && t > 0.f) best = fminf(best, t);
    }
    if (d[1] > 1e-9f) {  // back wall
      const float t = (2.5f - o[1]) / d[1];
      const float x = o[0] + t * d[0], z = o[2] + t * d[2];
      if (fabsf(x) <= 2.5f && z >= 0.f && z <= 3.f && t > 0.f) best = fminf(best, t);
    }
    if (d[0] < -1e-9f) {  // left wall
      const float t = (-2.5f - o[0]) / d[0];
      const float y = o[1] + t * d[1], z = o[2] + t * d[2];
      if (fabsf(y) <= 2.5f && z >= 0.f && z <= 3.f && t > 0.f) best = fminf(best, t);
    }
    for (int i = 0; i < nbox; ++i) {
      const BoxDev B = boxes[i];
      const float ow0 = o[0] - B.x, ow1 = o[1] - B.y;
      const float oo[3] = {B.c * ow0 + B.s * ow1, -B.s * ow0 + B.c * ow1, o[2]};
      const float dd[3] = {B.c * d[0] + B.s * d[1], -B.s * d[0] + B.c * d[1], d[2]};
      const float t = ray_box_obj(oo, dd, B.lo, B.hi);
      if (t > 0.f && t < best) best = t;
    }
    float z = 0.f;
    if (best < max_depth) {
      const unsigned long long h = splitmix(seed ^ ((unsigned long long)f << 40) ^ (unsigned long long)px);
      const float u1 = ((float)((h >> 40) + 1ull)) * (1.0f / 16777217.0f);          // (0, 1]
      const float u2 = (float)((h >> 16) & 0xFFFFFFull) * (1.0f / 16777216.0f);     // [0, 1)
      const float g = sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
      z = best + noise_k * best * best * g;
    }
    depth[(size_t)f * W * H + px] = z;
  }
}

// ---------------------------------------------------------------------------
// back-projection: p_cam = ((u - cx) z / fx, (v - cy) z / fy, z), then the
// pose (each operation rounded, no FMA: the oracle's arithmetic)
// ---------------------------------------------------------------------------
__global__ void k_depth_flags(const float* __restrict__ depth, int n, float min_z, float max_z,
                              uint32_t* __restrict__ flags) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float z = depth[i];
    flags[i] = (z > min_z && z < max_z) ? 1u : 0u;
  }
}

__global__ void k_backproject(const float* __restrict__ depth, int W, int H, float fx, float fy, float cx, float cy,
                              const float* __restrict__ T12, const uint32_t* __restrict__ flags,
                              const uint32_t* __restrict__ pos, float4* __restrict__ out) {
  __shared__ float sT[12];
  if (threadIdx.x < 12) sT[threadIdx.x] = T12[threadIdx.x];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < W * H; i += gridDim.x * blockDim.x) {
    if (!flags[i]) continue;
    const float z = depth[i];
    const int u = i % W, v = i / W;
    const float x = __fdiv_rn(__fmul_rn(__fsub_rn((float)u, cx), z), fx);
    const float y = __fdiv_rn(__fmul_rn(__fsub_rn((float)v, cy), z), fy);
    out[pos[i]] = xform_exact(sT, make_float4(x, y, z, 0.f));
  }
}

// ---------------------------------------------------------------------------
// fusion map
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long map_key(int kx, int ky, int kz) {
  return ((unsigned long long)(kx + (1 << 20)) & 0x1FFFFFull) |
         (((unsigned long long)(ky + (1 << 20)) & 0x1FFFFFull) << 21) |
         (((unsigned long long)(kz + (1 << 20)) & 0x1FFFFFull) << 42);
}

__global__ void k_map_integrate(const float4* __restrict__ pts, int n_cap, const int* d_n, float voxel, float inv,
                                int cap, unsigned long long* __restrict__ keys, unsigned long long* __restrict__ sums,
                                unsigned* __restrict__ counts, int* __restrict__ full) {
  const int n = d_n ? min(*d_n, n_cap) : n_cap;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 p = pts[i];
    const float fxk = floorf(__fmul_rn(p.x, inv)), fyk = floorf(__fmul_rn(p.y, inv)), fzk = floorf(__fmul_rn(p.z, inv));
    if (!(fabsf(fxk) < 1048000.f && fabsf(fyk) < 1048000.f && fabsf(fzk) < 1048000.f)) continue;  // also NaN
    const int kx = (int)fxk, ky = (int)fyk, kz = (int)fzk;
    const unsigned long long key = map_key(kx, ky, kz);
    unsigned slot = (unsigned)splitmix(key) & (unsigned)(cap - 1);
    bool placed = false;
    const int max_probe = cap < MAP_MAX_PROBE ? cap : MAP_MAX_PROBE;
    for (int probe = 0; probe < max_probe; ++probe) {
      const unsigned long long prev = atomicCAS(keys + slot, MAP_EMPTY, key);
      if (prev == MAP_EMPTY || prev == key) {
        placed = true;
        break;
      }
      slot = (slot + 1) & (unsigned)(cap - 1);
    }
    if (!placed) {
      atomicExch(full, 1);
      continue;
    }
    // offsets from the voxel's lower corner, in [0, voxel) up to rounding
    const double ox = (double)p.x - (double)kx * (double)voxel;
    const double oy = (double)p.y - (double)ky * (double)voxel;
    const double oz = (double)p.z - (double)kz * (double)voxel;
    const double lim = 2.0 * (double)voxel;
    atomicAdd(sums + 3 * (size_t)slot + 0, (unsigned long long)llrint(fmin(fmax(ox, 0.0), lim) * MAP_FIX));
    atomicAdd(sums + 3 * (size_t)slot + 1, (unsigned long long)llrint(fmin(fmax(oy, 0.0), lim) * MAP_FIX));
    atomicAdd(sums + 3 * (size_t)slot + 2, (unsigned long long)llrint(fmin(fmax(oz, 0.0), lim) * MAP_FIX));
    atomicAdd(counts + slot, 1u);
  }
}

__global__ void k_map_flags(const unsigned long long* __restrict__ keys, int cap, uint32_t* __restrict__ flags) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x)
    flags[i] = keys[i] != MAP_EMPTY ? 1u : 0u;
}

__global__ void k_map_extract(const unsigned long long* __restrict__ keys, const unsigned long long* __restrict__ sums,
                              const unsigned* __restrict__ counts, int cap, float voxel,
                              const uint32_t* __restrict__ flags, const uint32_t* __restrict__ pos,
                              float4* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cap; i += gridDim.x * blockDim.x) {
    if (!flags[i]) continue;
    const unsigned long long k = keys[i];
    const int kx = (int)(k & 0x1FFFFFull) - (1 << 20), ky = (int)((k >> 21) & 0x1FFFFFull) - (1 << 20),
              kz = (int)((k >> 42) & 0x1FFFFFull) - (1 << 20);
    const double c = (double)counts[i];
    float4 o;
    o.x = (float)((double)kx * (double)voxel + (double)sums[3 * (size_t)i + 0] / MAP_FIX / c);
    o.y = (float)((double)ky * (double)voxel + (double)sums[3 * (size_t)i + 1] / MAP_FIX / c);
    o.z = (float)((double)kz * (double)voxel + (double)sums[3 * (size_t)i + 2] / MAP_FIX / c);
    o.w = __int_as_float((int)counts[i]);
    out[pos[i]] = o;
  }
}

static int blocks_of(long long n, int per = 256) {
  long long b = (n + per - 1) / per;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b < 1 ? 1 : b);
}

}  // namespace rtr

using namespace rtr;

extern "C" {

rtr_status rtr_synth_depth_frames(rtr_context* ctx, const float* h_boxes12, int n_boxes, const double* h_poses16,
                                  int n_frames, int width, int height, float fx, float fy, float cx, float cy,
                                  float noise_k, uint64_t seed, float* d_depth, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && d_depth && h_poses16 && n_frames > 0 && width > 0 && height > 0 && n_boxes >= 0 &&
                    (n_boxes == 0 || h_boxes12),
                "rtr_synth_depth_frames: bad arguments");
  RTR_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = (cudaStream_t)stream;
  std::vector<float> poses((size_t)n_frames * 12);
  for (int f = 0; f < n_frames; ++f)
    for (int k = 0; k < 12; ++k) poses[(size_t)f * 12 + k] = (float)h_poses16[(size_t)f * 16 + k];
  ScratchPlan plan;
  plan.add<BoxDev>(n_boxes > 0 ? n_boxes : 1);
  plan.add<float>(poses.size());
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  BoxDev* db = s.take<BoxDev>(n_boxes > 0 ? n_boxes : 1);
  float* dp = s.take<float>(poses.size());
  static_assert(sizeof(BoxDev) == 12 * sizeof(float), "box layout");
  if (n_boxes > 0) RTR_CUDA(cudaMemcpyAsync(db, h_boxes12, sizeof(BoxDev) * n_boxes, cudaMemcpyHostToDevice, st));
  RTR_CUDA(cudaMemcpyAsync(dp, poses.data(), sizeof(float) * poses.size(), cudaMemcpyHostToDevice, st));
  const dim3 grid((unsigned)((width * height + 255) / 256 < 1024 ? (width * height + 255) / 256 : 1024),
                  (unsigned)n_frames);
  k_raycast_depth<<<grid, 256, 0, st>>>(db, n_boxes, dp, width, height, fx, fy, cx, cy, noise_k, seed, 8.f, d_depth);
  RTR_LAUNCHED(1);
  RTR_CUDA(cudaGetLastError());
  RTR_CUDA(cudaStreamSynchronize(st));  // the staged boxes and poses live in scratch
  return RTR_OK;
}

rtr_status rtr_depth_to_points(rtr_context* ctx, const float* d_depth, int width, int height, float fx, float fy,
                               float cx, float cy, const double* h_pose16, float min_z, float max_z, float* d_points,
                               int* d_count, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && d_depth && d_points && d_count && width > 0 && height > 0,
                "rtr_depth_to_points: bad arguments");
  RTR_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = (cudaStream_t)stream;
  const int n = width * height;
  ScratchPlan plan;
  plan.add<uint32_t>(n);
  plan.add<uint32_t>(n);
  plan.add<uint32_t>(scan_tiles(n));
  plan.add<float>(12);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  uint32_t* flags = s.take<uint32_t>(n);
  uint32_t* pos = s.take<uint32_t>(n);
  uint32_t* tiles = s.take<uint32_t>(scan_tiles(n));
  float* T = s.take<float>(12);
  float hT[12];
  for (int k = 0; k < 12; ++k) hT[k] = h_pose16 ? (float)h_pose16[k] : ((k % 5) == 0 ? 1.f : 0.f);
  // kernel parameter copy: no host buffer has to outlive the call
  RTR_CUDA(cudaMemcpyAsync(T, hT, sizeof(hT), cudaMemcpyHostToDevice, st));
  k_depth_flags<<<blocks_of(n), 256, 0, st>>>(d_depth, n, min_z, max_z, flags);
  scan_exclusive(flags, pos, tiles, n, n, nullptr, reinterpret_cast<uint32_t*>(d_count), st);
  k_backproject<<<blocks_of(n), 256, 0, st>>>(d_depth, width, height, fx, fy, cx, cy, T, flags, pos,
                                              reinterpret_cast<float4*>(d_points));
  RTR_LAUNCHED(2);
  RTR_CUDA(cudaGetLastError());
  RTR_CUDA(cudaStreamSynchronize(st));  // the pose was staged from the host
  return RTR_OK;
}

rtr_status rtr_map_create(rtr_context* ctx, int capacity, float voxel, rtr_map** out) {
  RTR_CHECK_ARG(ctx && out && capacity > 0 && voxel > 0.f, "rtr_map_create: bad arguments");
  *out = nullptr;
  int cap = 1;
  while (cap < capacity && cap < (1 << 30)) cap <<= 1;
  RTR_CUDA(cudaSetDevice(ctx->device));
  rtr_map* m = new rtr_map();
  m->device = ctx->device;
  m->voxel = voxel;
  m->cap = cap;
  if (cudaMalloc(&m->keys, sizeof(unsigned long long) * cap) != cudaSuccess ||
      cudaMalloc(&m->sums, sizeof(unsigned long long) * 3 * (size_t)cap) != cudaSuccess ||
      cudaMalloc(&m->counts, sizeof(unsigned) * cap) != cudaSuccess || cudaMalloc(&m->d_full, sizeof(int)) != cudaSuccess) {
    (void)cudaGetLastError();
    rtr_map_destroy(m);
    return fail(RTR_ERR_OOM, "rtr_map_create: %d slots", cap);
  }
  rtr_status r = rtr_map_clear(m, nullptr);
  if (r != RTR_OK) {
    rtr_map_destroy(m);
    return r;
  }
  RTR_CUDA(cudaDeviceSynchronize());
  *out = m;
  return RTR_OK;
}

rtr_status rtr_map_clear(rtr_map* m, rtr_stream_t stream) {
  RTR_CHECK_ARG(m, "rtr_map_clear: NULL map");
  RTR_CUDA(cudaSetDevice(m->device));
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaMemsetAsync(m->keys, 0xff, sizeof(unsigned long long) * m->cap, st));
  RTR_CUDA(cudaMemsetAsync(m->sums, 0, sizeof(unsigned long long) * 3 * (size_t)m->cap, st));
  RTR_CUDA(cudaMemsetAsync(m->counts, 0, sizeof(unsigned) * m->cap, st));
  RTR_CUDA(cudaMemsetAsync(m->d_full, 0, sizeof(int), st));
  return RTR_OK;
}

rtr_status rtr_map_destroy(rtr_map* m) {
  if (!m) return RTR_OK;
  cudaSetDevice(m->device);
  cudaFree(m->keys);
  cudaFree(m->sums);
  cudaFree(m->counts);
  cudaFree(m->d_full);
  delete m;
  return RTR_OK;
}

rtr_status rtr_map_integrate(rtr_map* m, const float* d_points, int n_cap, const int* d_n, rtr_stream_t stream) {
  RTR_CHECK_ARG(m && n_cap >= 0 && (n_cap == 0 || d_points), "rtr_map_integrate: bad arguments");
  if (n_cap == 0) return RTR_OK;
  RTR_CUDA(cudaSetDevice(m->device));
  k_map_integrate<<<blocks_of(n_cap), 256, 0, (cudaStream_t)stream>>>(
      reinterpret_cast<const float4*>(d_points), n_cap, d_n, m->voxel, 1.f / m->voxel, m->cap, m->keys, m->sums,
      m->counts, m->d_full);
  RTR_LAUNCHED(1);
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

rtr_status rtr_map_extract(rtr_context* ctx, rtr_map* m, float* d_out, int max_out, int* h_count) {
  RTR_CHECK_ARG(ctx && m && h_count && (max_out == 0 || d_out), "rtr_map_extract: bad arguments");
  RTR_CUDA(cudaSetDevice(m->device));
  cudaStream_t st = ctx->host_stream;
  RTR_CUDA(cudaDeviceSynchronize());
  int full = 0;
  RTR_CUDA(cudaMemcpy(&full, m->d_full, sizeof(int), cudaMemcpyDeviceToHost));
  if (full) return fail(RTR_ERR_CAPACITY, "rtr_map: the table (%d slots) filled up", m->cap);
  ScratchPlan plan;
  plan.add<uint32_t>(m->cap);
  plan.add<uint32_t>(m->cap);
  plan.add<uint32_t>(scan_tiles(m->cap));
  plan.add<uint32_t>(1);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  uint32_t* flags = s.take<uint32_t>(m->cap);
  uint32_t* pos = s.take<uint32_t>(m->cap);
  uint32_t* tiles = s.take<uint32_t>(scan_tiles(m->cap));
  uint32_t* total = s.take<uint32_t>(1);
  k_map_flags<<<blocks_of(m->cap), 256, 0, st>>>(m->keys, m->cap, flags);
  scan_exclusive(flags, pos, tiles, m->cap, m->cap, nullptr, total, st);
  RTR_LAUNCHED(1);
  uint32_t nv = 0;
  RTR_CUDA(cudaMemcpyAsync(&nv, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
  RTR_CUDA(cudaStreamSynchronize(st));
  *h_count = (int)nv;
  if ((int)nv > max_out) return RTR_OK;  // count only
  k_map_extract<<<blocks_of(m->cap), 256, 0, st>>>(m->keys, m->sums, m->counts, m->cap, m->voxel, flags, pos,
                                                   reinterpret_cast<float4*>(d_out));
  RTR_LAUNCHED(1);
  RTR_CUDA(cudaStreamSynchronize(st));
  return RTR_OK;
}

}  // extern "C"
