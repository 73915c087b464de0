// batch.cu — batched registration: many model x segment pairs at once.
//
// One pair (2k-60k points) fills a small part of a GB300.  The recognition
// chain keeps every count on the device (no host round trip), so one host
// thread can spread a batch over several streams: each worker is a child
// context (scratch arena, stream, status words), the pairs are dealt out
// round-robin in largest-first order, and the worker streams are forked from
// and joined back to the caller's stream with events.  The same enqueue
// sequence can be captured once into a CUDA graph (rtr_batch_graph_*) and
// replayed, which removes the per-launch host cost of the ~130 kernels of
// every pair.
//
// Each worker's cooperative kernels (grouping, ICP) take 1/workers of the
// co-resident blocks so they run side by side.  A pair's result is the
// single-call result up to the FP32 rounding of ICP block sums over a
// different block count.  rtr_batch_autotune picks the worker count and the
// ICP lanes per point by timing the caller's batch.
#include <algorithm>
#include <chrono>
#include <vector>

#include "common.cuh"

struct rtr_batch_graph {
  rtr_context* ctx = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // scratch generations of the context and of each worker at capture: the
  // graph holds their arena addresses, so it may run only while none of the
  // arenas has been reallocated since
  std::vector<unsigned> gens;
};

namespace rtr {

rtr_status batch_ensure_workers(rtr_context* ctx, int n) {
  while ((int)ctx->workers.size() < n) {
    rtr_context* w = nullptr;
    RTR_TRY(rtr_context_create(ctx->device, &w));
    ctx->workers.push_back(w);
  }
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (!ctx->ev_fork) RTR_CUDA(cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming));
  for (rtr_context* w : ctx->workers) {
    if (!w->ev_fork) RTR_CUDA(cudaEventCreateWithFlags(&w->ev_fork, cudaEventDisableTiming));
    w->coop_div = n;  // cooperative kernels of the n workers fit the GPU side by side
    w->auto_graph = 0;  // a worker's consecutive pairs differ; whole batches are graphed instead
    w->wait_budget_ms = ctx->wait_budget_ms;
    w->wait_budget_cycles = ctx->wait_budget_cycles;
    w->tune_icp_group = ctx->tune_icp_group;
    w->tune_scene_grid_mm = ctx->tune_scene_grid_mm;
    w->tune_normals_grid_mm = ctx->tune_normals_grid_mm;
    w->scratch_limit = ctx->scratch_limit;
  }
  return RTR_OK;
}

int batch_worker_count(const rtr_context* ctx, int n_pairs) {
  int w = ctx->tune_batch_workers > 0 ? ctx->tune_batch_workers : 4;
  return w < n_pairs ? w : n_pairs;
}

// Enqueue the batch on `origin` (forked to the workers' streams and joined
// back); returns without synchronising.
static rtr_status enqueue_batch(rtr_context* ctx, const rtr_batch_pair* pairs, int n_pairs, const rtr_recog_params* p,
                                const rtr_mlp* mlp, float keep, int nw, rtr_recog_result* d_results,
                                cudaStream_t origin) {
  RTR_TRY(batch_ensure_workers(ctx, nw));
  std::vector<int> order((size_t)n_pairs);
  for (int i = 0; i < n_pairs; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return pairs[a].n > pairs[b].n; });
  RTR_CUDA(cudaEventRecord(ctx->ev_fork, origin));
  for (int wi = 0; wi < nw; ++wi) RTR_CUDA(cudaStreamWaitEvent(ctx->workers[wi]->host_stream, ctx->ev_fork, 0));
  for (int k = 0; k < n_pairs; ++k) {
    rtr_context* w = ctx->workers[k % nw];
    const int i = order[k];
    const rtr_batch_pair& q = pairs[i];
    const rtr_status r = mlp ? rtr_recognize_learned(w, q.model, mlp, keep, q.d_scene, q.n, p, d_results + i,
                                                     w->host_stream)
                             : rtr_recognize(w, q.model, q.d_scene, q.n, p, d_results + i, w->host_stream);
    if (r != RTR_OK) return fail(r, "rtr_recognize_batch: pair %d: %s", i, rtr_last_error());
  }
  for (int wi = 0; wi < nw; ++wi) {
    rtr_context* w = ctx->workers[wi];
    RTR_CUDA(cudaEventRecord(w->ev_fork, w->host_stream));
    RTR_CUDA(cudaStreamWaitEvent(origin, w->ev_fork, 0));
  }
  RTR_CUDA(cudaSetDevice(ctx->device));
  return RTR_OK;
}

// Device status words of the workers (timeouts, capacity) after a batch.
rtr_status batch_check_workers(rtr_context* ctx, int nw) {
  for (int wi = 0; wi < nw; ++wi) RTR_TRY(rtr_context_check(ctx->workers[wi], ctx->workers[wi]->host_stream));
  RTR_CUDA(cudaSetDevice(ctx->device));
  return RTR_OK;
}

static rtr_status check_args(rtr_context* ctx, const rtr_batch_pair* h_pairs, int n_pairs, const rtr_recog_params* p,
                             const rtr_mlp* mlp, float keep, const rtr_recog_result* d_results) {
  RTR_CHECK_ARG(ctx && p && n_pairs >= 0 && (n_pairs == 0 || (h_pairs && d_results)),
                "rtr_recognize_batch: bad arguments");
  RTR_CHECK_ARG(!mlp || (keep > 0.f && keep <= 1.f), "rtr_recognize_batch: keep must be in (0, 1]");
  for (int i = 0; i < n_pairs; ++i)
    RTR_CHECK_ARG(h_pairs[i].model && h_pairs[i].n >= 0 && (h_pairs[i].n == 0 || h_pairs[i].d_scene),
                  "rtr_recognize_batch: pair %d is incomplete", i);
  return RTR_OK;
}

}  // namespace rtr

using namespace rtr;

extern "C" {

rtr_status rtr_recognize_batch(rtr_context* ctx, const rtr_batch_pair* h_pairs, int n_pairs,
                               const rtr_recog_params* p, const rtr_mlp* mlp, float keep,
                               rtr_recog_result* d_results) {
  RTR_TRY(check_args(ctx, h_pairs, n_pairs, p, mlp, keep, d_results));
  if (n_pairs == 0) return RTR_OK;
  RTR_CUDA(cudaSetDevice(ctx->device));
  RTR_CUDA(cudaDeviceSynchronize());  // inputs written on other streams are complete
  const int nw = batch_worker_count(ctx, n_pairs);
  RTR_TRY(enqueue_batch(ctx, h_pairs, n_pairs, p, mlp, keep, nw, d_results, ctx->host_stream));
  RTR_CUDA(cudaStreamSynchronize(ctx->host_stream));
  return batch_check_workers(ctx, nw);
}

rtr_status rtr_batch_graph_create(rtr_context* ctx, const rtr_batch_pair* h_pairs, int n_pairs,
                                  const rtr_recog_params* p, const rtr_mlp* mlp, float keep,
                                  rtr_recog_result* d_results, rtr_batch_graph** out) {
  RTR_CHECK_ARG(out, "rtr_batch_graph_create: out is NULL");
  *out = nullptr;
  RTR_TRY(check_args(ctx, h_pairs, n_pairs, p, mlp, keep, d_results));
  RTR_CHECK_ARG(n_pairs > 0, "rtr_batch_graph_create: empty batch");
  // one plain run sizes every worker's scratch for its pairs
  RTR_TRY(rtr_recognize_batch(ctx, h_pairs, n_pairs, p, mlp, keep, d_results));
  const int nw = batch_worker_count(ctx, n_pairs);
  for (int wi = 0; wi < nw; ++wi)
    RTR_CHECK_ARG(!ctx->workers[wi]->profiling, "rtr_batch_graph_create: profiling is on");
  cudaStream_t origin = ctx->host_stream;
  RTR_CUDA(cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal));
  const rtr_status r = enqueue_batch(ctx, h_pairs, n_pairs, p, mlp, keep, nw, d_results, origin);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(origin, &g);
  if (r != RTR_OK) {
    if (g) cudaGraphDestroy(g);
    return r;
  }
  if (e != cudaSuccess) return fail(RTR_ERR_CUDA, "rtr_batch_graph_create: capture failed: %s", cudaGetErrorString(e));
  cudaGraphExec_t x = nullptr;
  const cudaError_t ei = cudaGraphInstantiate(&x, g, 0);
  if (ei != cudaSuccess) {
    cudaGraphDestroy(g);
    return fail(RTR_ERR_CUDA, "rtr_batch_graph_create: instantiate failed: %s", cudaGetErrorString(ei));
  }
  rtr_batch_graph* bg = new rtr_batch_graph();
  bg->ctx = ctx;
  bg->graph = g;
  bg->exec = x;
  bg->gens.push_back(ctx->scratch_gen);
  for (int wi = 0; wi < nw; ++wi) bg->gens.push_back(ctx->workers[wi]->scratch_gen);
  *out = bg;
  return RTR_OK;
}

rtr_status rtr_batch_graph_launch(rtr_batch_graph* bg, rtr_stream_t stream) {
  RTR_CHECK_ARG(bg && bg->exec, "rtr_batch_graph_launch: bad graph");
  bool same = !bg->gens.empty() && bg->gens[0] == bg->ctx->scratch_gen &&
              bg->gens.size() <= bg->ctx->workers.size() + 1;
  for (size_t k = 1; same && k < bg->gens.size(); ++k) same = bg->gens[k] == bg->ctx->workers[k - 1]->scratch_gen;
  RTR_CHECK_ARG(same,
                "rtr_batch_graph_launch: a call on this context grew its scratch after the graph was made (its "
                "buffers moved); destroy and recreate the graph, or reserve scratch before creating it");
  RTR_CUDA(cudaSetDevice(bg->ctx->device));
  RTR_CUDA(cudaGraphLaunch(bg->exec, (cudaStream_t)stream));
  return RTR_OK;
}

rtr_status rtr_batch_graph_destroy(rtr_batch_graph* bg) {
  if (!bg) return RTR_OK;
  cudaSetDevice(bg->ctx->device);
  if (bg->exec) cudaGraphExecDestroy(bg->exec);
  if (bg->graph) cudaGraphDestroy(bg->graph);
  delete bg;
  return RTR_OK;
}

rtr_status rtr_batch_autotune(rtr_context* ctx, const rtr_batch_pair* h_pairs, int n_pairs,
                              const rtr_recog_params* p, const rtr_mlp* mlp, float keep,
                              rtr_recog_result* d_results, int* h_workers, int* h_icp_group) {
  RTR_CHECK_ARG(ctx && p && h_pairs && d_results && n_pairs > 0, "rtr_batch_autotune: bad arguments");
  RTR_CUDA(cudaSetDevice(ctx->device));
  const int saved[4] = {ctx->tune_batch_workers, ctx->tune_icp_group, ctx->tune_scene_grid_mm,
                        ctx->tune_normals_grid_mm};
  int* knob[4] = {&ctx->tune_batch_workers, &ctx->tune_icp_group, &ctx->tune_scene_grid_mm,
                  &ctx->tune_normals_grid_mm};
  // one untimed pass (scratch growth), then one timed pass
  auto run = [&](double* dt) -> rtr_status {
    rtr_status r = rtr_recognize_batch(ctx, h_pairs, n_pairs, p, mlp, keep, d_results);
    const auto t0 = std::chrono::steady_clock::now();
    if (r == RTR_OK) r = rtr_recognize_batch(ctx, h_pairs, n_pairs, p, mlp, keep, d_results);
    *dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return r;
  };
  auto restore = [&]() {
    for (int k = 0; k < 4; ++k) *knob[k] = saved[k];
  };
  // stage 1: workers (pairs per stream, "warps per pair" of the shared GPU)
  // x lanes per ICP source point; stages 2 and 3, with those fixed: the
  // scene grid's cell (verification and refinement searches) and the
  // normals' k-NN grid cell, in mm (0 = the automatic choice)
  static const int kWorkers[] = {1, 2, 4, 8};
  static const int kGroups[] = {2, 4, 8};
  static const int kSceneMm[] = {0, 20, 40, 60};
  static const int kNormalsMm[] = {0, 20, 30, 80};
  double best = 1e300;
  int bw = 4, bg = 0;
  for (int g : kGroups)
    for (int w : kWorkers) {
      if (w > n_pairs && w != 1) continue;
      ctx->tune_batch_workers = w;
      ctx->tune_icp_group = g;
      double dt = 0;
      const rtr_status r = run(&dt);
      if (r != RTR_OK) {
        restore();
        return r;
      }
      if (dt < best) {
        best = dt;
        bw = w;
        bg = g;
      }
    }
  ctx->tune_batch_workers = bw;
  ctx->tune_icp_group = bg;
  for (int stage = 2; stage <= 3; ++stage) {
    const int* cand = stage == 2 ? kSceneMm : kNormalsMm;
    int* k = stage == 2 ? &ctx->tune_scene_grid_mm : &ctx->tune_normals_grid_mm;
    int bestv = *k;
    for (int i = 0; i < 4; ++i) {
      *k = cand[i];
      double dt = 0;
      const rtr_status r = run(&dt);
      if (r != RTR_OK) {
        restore();
        return r;
      }
      if (dt < best) {
        best = dt;
        bestv = cand[i];
      }
    }
    *k = bestv;
  }
  if (h_workers) *h_workers = bw;
  if (h_icp_group) *h_icp_group = bg;
  return RTR_OK;
}

}  // extern "C"
