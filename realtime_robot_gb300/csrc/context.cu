// context.cu — rtr_context lifecycle, scratch arena and error reporting.
#include <stdarg.h>
#include <string.h>

#include "common.cuh"

namespace rtr {

std::atomic<uint64_t> g_launches{0};
static std::atomic<uint64_t> g_uid{0};
uint64_t next_uid() { return g_uid.fetch_add(1, std::memory_order_relaxed) + 1; }
static thread_local char g_last_error[512] = "";

static cudaEvent_t pool_event(rtr_context* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

ProfScope::ProfScope(rtr_context* c, cudaStream_t s, const char* name) : ctx(c), st(s) {
  if (!ctx || !ctx->profiling || stream_is_capturing(s)) return;
  rtr_prof_rec r{name, pool_event(ctx), pool_event(ctx)};
  cudaEventRecord(r.a, st);
  ctx->prof.push_back(r);
  slot = (int)ctx->prof.size() - 1;
}

void ProfScope::end() {
  if (slot >= 0) cudaEventRecord(ctx->prof[slot].b, st);
  slot = -1;
}

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

rtr_status fail(rtr_status st, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return st;
}

rtr_status cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  const char* base = strrchr(file, '/');
  set_error("%s failed: %s (%s:%d)", what, cudaGetErrorString(e), base ? base + 1 : file, line);
  return e == cudaErrorMemoryAllocation ? RTR_ERR_OOM : RTR_ERR_CUDA;
}

bool stream_is_capturing(cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &st) != cudaSuccess) return false;
  return st != cudaStreamCaptureStatusNone;
}

rtr_status side_stream_ready(rtr_context* ctx) {
  if (!ctx->side_stream) RTR_CUDA(cudaStreamCreateWithFlags(&ctx->side_stream, cudaStreamNonBlocking));
  for (cudaEvent_t& e : ctx->ev_side)
    if (!e) RTR_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  return RTR_OK;
}

rtr_status ensure_scratch(rtr_context* ctx, size_t bytes, cudaStream_t stream, Scratch* out) {
  if (bytes > ctx->arena_bytes) {
    if (stream_is_capturing(stream))
      return fail(RTR_ERR_CAPACITY,
                  "scratch arena holds %zu bytes but %zu are needed while the stream is "
                  "being captured; call rtr_context_reserve first",
                  ctx->arena_bytes, bytes);
    size_t grow = bytes + bytes / 4 + (1u << 20);
    if (ctx->scratch_limit) {
      // a memory budget set by the caller: refused exactly as a failed
      // cudaMalloc would be, with the arena held so far kept
      if (bytes > ctx->scratch_limit)
        return fail(RTR_ERR_OOM, "scratch arena: %zu bytes needed, the context's limit is %zu", bytes,
                    ctx->scratch_limit);
      if (grow > ctx->scratch_limit) grow = ctx->scratch_limit;
    }
    RTR_CUDA(cudaDeviceSynchronize());
    ++ctx->scratch_gen;  // from here on the old arena is gone, whatever the allocation below does
    if (ctx->arena) RTR_CUDA(cudaFree(ctx->arena));
    ctx->arena = nullptr;
    ctx->arena_bytes = 0;
    cudaError_t e = cudaMalloc(&ctx->arena, grow);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(RTR_ERR_OOM, "scratch arena: cudaMalloc(%zu) failed: %s", grow,
                  cudaGetErrorString(e));
    }
    ctx->arena_bytes = grow;
  }
  out->base = static_cast<char*>(ctx->arena);
  out->off = 0;
  out->cap = ctx->arena_bytes;
  return RTR_OK;
}

rtr_status ensure_io(rtr_context* ctx, size_t bytes) {
  if (bytes <= ctx->io_bytes) return RTR_OK;
  RTR_CUDA(cudaDeviceSynchronize());
  if (ctx->io) RTR_CUDA(cudaFree(ctx->io));
  ctx->io = nullptr;
  ctx->io_bytes = 0;
  size_t grow = bytes + bytes / 4 + (1u << 16);
  if (cudaMalloc(&ctx->io, grow) != cudaSuccess) {
    cudaGetLastError();
    return fail(RTR_ERR_OOM, "host-entry staging: cudaMalloc(%zu) failed", grow);
  }
  ctx->io_bytes = grow;
  return RTR_OK;
}

}  // namespace rtr

extern "C" {

const char* rtr_status_string(int status) {
  switch (status) {
    case RTR_OK: return "RTR_OK";
    case RTR_ERR_INVALID_ARG: return "RTR_ERR_INVALID_ARG";
    case RTR_ERR_OOM: return "RTR_ERR_OOM";
    case RTR_ERR_TIMEOUT: return "RTR_ERR_TIMEOUT";
    case RTR_ERR_NOT_FOUND: return "RTR_ERR_NOT_FOUND";
    case RTR_ERR_CUDA: return "RTR_ERR_CUDA";
    case RTR_ERR_CAPACITY: return "RTR_ERR_CAPACITY";
    case RTR_ERR_NO_DEVICE: return "RTR_ERR_NO_DEVICE";
    default: return "RTR_ERR_UNKNOWN";
  }
}

const char* rtr_last_error(void) { return rtr::g_last_error; }

const char* rtr_version(void) { return RTR_VERSION_STRING; }

rtr_status rtr_context_create(int device, rtr_context** out) {
  if (!out) return rtr::fail(RTR_ERR_INVALID_ARG, "rtr_context_create: out is NULL");
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev <= device || device < 0) {
    cudaGetLastError();
    return rtr::fail(RTR_ERR_NO_DEVICE, "no CUDA device %d (%d visible): %s", device, ndev,
                     cudaGetErrorString(e));
  }
  cudaDeviceProp prop;
  RTR_CUDA(cudaGetDeviceProperties(&prop, device));
  if (prop.major != 10 || prop.minor != 3)
    return rtr::fail(RTR_ERR_NO_DEVICE,
                     "device %d is sm_%d%d; this library is built for sm_103a only", device,
                     prop.major, prop.minor);
  RTR_CUDA(cudaSetDevice(device));
  rtr_context* ctx = new rtr_context();
  ctx->device = device;
  ctx->num_sms = prop.multiProcessorCount;
  ctx->max_smem_optin = (int)prop.sharedMemPerBlockOptin;
  int khz = 0;
  cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, device);
  ctx->clock_khz = khz > 0 ? khz : 2070000;
  ctx->wait_budget_cycles = (long long)(ctx->wait_budget_ms * 1e-3 * ctx->clock_khz * 1e3);
  if (cudaMalloc(&ctx->d_status, 64 * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&ctx->d_sync, 64 * sizeof(unsigned)) != cudaSuccess) {
    cudaGetLastError();
    if (ctx->d_status) cudaFree(ctx->d_status);
    delete ctx;
    return rtr::fail(RTR_ERR_OOM, "rtr_context_create: status words");
  }
  cudaStreamCreateWithFlags(&ctx->host_stream, cudaStreamNonBlocking);
  if (cudaMallocHost(&ctx->h_pin, 64 * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    ctx->h_pin = nullptr;
  }
  cudaMemset(ctx->d_status, 0, 64 * sizeof(int));
  cudaMemset(ctx->d_sync, 0, 64 * sizeof(unsigned));
  RTR_CUDA(cudaDeviceSynchronize());
  *out = ctx;
  return RTR_OK;
}

rtr_status rtr_context_set_profiling(rtr_context* ctx, int enabled) {
  if (!ctx) return rtr::fail(RTR_ERR_INVALID_ARG, "rtr_context_set_profiling: ctx is NULL");
  ctx->profiling = enabled != 0;
  return RTR_OK;
}

int rtr_context_profile_count(rtr_context* ctx) { return ctx ? (int)ctx->prof.size() : 0; }

rtr_status rtr_context_profile_get(rtr_context* ctx, int i, const char** name, float* ms) {
  if (!ctx || i < 0 || i >= (int)ctx->prof.size())
    return rtr::fail(RTR_ERR_INVALID_ARG, "rtr_context_profile_get: index out of range");
  const rtr_prof_rec& r = ctx->prof[i];
  if (name) *name = r.name;
  if (ms) {
    RTR_CUDA(cudaEventSynchronize(r.b));
    RTR_CUDA(cudaEventElapsedTime(ms, r.a, r.b));
  }
  return RTR_OK;
}

void rtr_context_profile_clear(rtr_context* ctx) {
  if (!ctx) return;
  for (auto& r : ctx->prof) {
    ctx->event_pool.push_back(r.a);
    ctx->event_pool.push_back(r.b);
  }
  ctx->prof.clear();
}

uint64_t rtr_launch_count(void) { return rtr::g_launches.load(); }

rtr_status rtr_context_destroy(rtr_context* ctx) {
  if (!ctx) return RTR_OK;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  for (rtr_context* w : ctx->workers) rtr_context_destroy(w);
  ctx->workers.clear();
  cudaSetDevice(ctx->device);
  rtr_context_profile_clear(ctx);
  for (cudaEvent_t e : ctx->event_pool) cudaEventDestroy(e);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  if (ctx->rgraph.exec) cudaGraphExecDestroy(ctx->rgraph.exec);
  for (cudaEvent_t e : ctx->ev_side)
    if (e) cudaEventDestroy(e);
  if (ctx->side_stream) cudaStreamDestroy(ctx->side_stream);
  if (ctx->cap_stream) cudaStreamDestroy(ctx->cap_stream);
  if (ctx->arena) cudaFree(ctx->arena);
  if (ctx->io) cudaFree(ctx->io);
  if (ctx->host_stream) cudaStreamDestroy(ctx->host_stream);
  if (ctx->h_pin) cudaFreeHost(ctx->h_pin);
  if (ctx->d_status) cudaFree(ctx->d_status);
  if (ctx->d_sync) cudaFree(ctx->d_sync);
  delete ctx;
  return RTR_OK;
}

rtr_status rtr_context_reserve(rtr_context* ctx, size_t bytes) {
  if (!ctx) return rtr::fail(RTR_ERR_INVALID_ARG, "rtr_context_reserve: ctx is NULL");
  RTR_CUDA(cudaSetDevice(ctx->device));
  rtr::Scratch s;
  return rtr::ensure_scratch(ctx, bytes, 0, &s);
}

size_t rtr_context_scratch_bytes(const rtr_context* ctx) { return ctx ? ctx->arena_bytes : 0; }

rtr_status rtr_context_set_wait_budget_ms(rtr_context* ctx, double ms) {
  if (!ctx || !(ms > 0)) return rtr::fail(RTR_ERR_INVALID_ARG, "wait budget must be > 0 ms");
  ctx->wait_budget_ms = ms;
  ctx->wait_budget_cycles = (long long)(ms * 1e-3 * ctx->clock_khz * 1e3);
  ++ctx->cfg_gen;
  return RTR_OK;
}

static rtr_status set_tuning(rtr_context* ctx, const char* key, int value);

rtr_status rtr_context_set_tuning(rtr_context* ctx, const char* key, int value) {
  if (!ctx || !key) return rtr::fail(RTR_ERR_INVALID_ARG, "rtr_context_set_tuning: NULL argument");
  const rtr_status r = set_tuning(ctx, key, value);
  if (r == RTR_OK) ++ctx->cfg_gen;  // a captured recognition no longer matches
  return r;
}

static rtr_status set_tuning(rtr_context* ctx, const char* key, int value) {
  if (strcmp(key, "auto_graph") == 0) {
    if (value < 0 || value > 1) return rtr::fail(RTR_ERR_INVALID_ARG, "auto_graph must be 0 or 1 (got %d)", value);
    ctx->auto_graph = value;
    return RTR_OK;
  }
  if (strcmp(key, "batch_workers") == 0) {
    if (value < 0 || value > 16)
      return rtr::fail(RTR_ERR_INVALID_ARG, "batch_workers must be 0..16 (got %d)", value);
    ctx->tune_batch_workers = value;
    return RTR_OK;
  }
  if (strcmp(key, "gc_window") == 0) {
    if (value < 0 || value > 1024)
      return rtr::fail(RTR_ERR_INVALID_ARG, "gc_window must be 0..1024 (got %d)", value);
    ctx->tune_gc_window = value;
    return RTR_OK;
  }
  if (strcmp(key, "gc_pass_lists") == 0) {
    if (value < 0 || value > 1)
      return rtr::fail(RTR_ERR_INVALID_ARG, "gc_pass_lists must be 0 or 1 (got %d)", value);
    ctx->tune_gc_no_lists = value;
    return RTR_OK;
  }
  if (strcmp(key, "gc_inline") == 0) {
    if (value < 0 || value > 4096)
      return rtr::fail(RTR_ERR_INVALID_ARG, "gc_inline must be 0..4096 (got %d)", value);
    ctx->tune_gc_inline = value;
    return RTR_OK;
  }
  if (strcmp(key, "scene_grid_mm") == 0 || strcmp(key, "normals_grid_mm") == 0) {
    if (value < 0 || value > 1000)
      return rtr::fail(RTR_ERR_INVALID_ARG, "%s must be 0..1000 (got %d)", key, value);
    (key[0] == 's' ? ctx->tune_scene_grid_mm : ctx->tune_normals_grid_mm) = value;
    return RTR_OK;
  }
  if (strcmp(key, "scratch_limit_mb") == 0) {
    if (value < 0) return rtr::fail(RTR_ERR_INVALID_ARG, "scratch_limit_mb must be >= 0 (got %d)", value);
    ctx->scratch_limit = (size_t)value << 20;
    return RTR_OK;
  }
  if (strcmp(key, "icp_group") == 0) {
    if (value != 0 && value != 2 && value != 4 && value != 8)
      return rtr::fail(RTR_ERR_INVALID_ARG, "icp_group must be 0, 2, 4 or 8 (got %d)", value);
    ctx->tune_icp_group = value;
    return RTR_OK;
  }
  return rtr::fail(RTR_ERR_INVALID_ARG, "rtr_context_set_tuning: unknown key '%s'", key);
}

rtr_status rtr_context_get_tuning(const rtr_context* ctx, const char* key, int* value) {
  if (!ctx || !key || !value) return rtr::fail(RTR_ERR_INVALID_ARG, "rtr_context_get_tuning: NULL argument");
  if (strcmp(key, "auto_graph") == 0) *value = ctx->auto_graph;
  else if (strcmp(key, "batch_workers") == 0) *value = ctx->tune_batch_workers;
  else if (strcmp(key, "gc_window") == 0) *value = ctx->tune_gc_window;
  else if (strcmp(key, "gc_pass_lists") == 0) *value = ctx->tune_gc_no_lists;
  else if (strcmp(key, "gc_inline") == 0) *value = ctx->tune_gc_inline;
  else if (strcmp(key, "scene_grid_mm") == 0) *value = ctx->tune_scene_grid_mm;
  else if (strcmp(key, "normals_grid_mm") == 0) *value = ctx->tune_normals_grid_mm;
  else if (strcmp(key, "icp_group") == 0) *value = ctx->tune_icp_group;
  else if (strcmp(key, "scratch_limit_mb") == 0) *value = (int)(ctx->scratch_limit >> 20);
  else return rtr::fail(RTR_ERR_INVALID_ARG, "rtr_context_get_tuning: unknown key '%s'", key);
  return RTR_OK;
}

rtr_status rtr_context_check(rtr_context* ctx, rtr_stream_t stream) {
  if (!ctx) return rtr::fail(RTR_ERR_INVALID_ARG, "rtr_context_check: ctx is NULL");
  int st = 0;
  RTR_CUDA(cudaMemcpyAsync(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, stream));
  RTR_CUDA(cudaStreamSynchronize(stream));
  if (st != 0) {
    RTR_CUDA(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), stream));
    RTR_CUDA(cudaStreamSynchronize(stream));
    return rtr::fail((rtr_status)st, "device status word: %s", rtr_status_string(st));
  }
  return RTR_OK;
}

}  // extern "C"
