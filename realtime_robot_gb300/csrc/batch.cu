// batch.cu — batched registration: many model x segment pairs at once.
//
// One pair (2k-60k points) fills a small part of a GB300: its stages are a
// few hundred thousand threads each, and the pipeline synchronises twice
// (correspondence count, cluster count).  The batch driver therefore runs
// the pairs concurrently: a pool of worker threads, each with its own child
// context (scratch arena, stream, status words), takes pairs largest first
// (LPT order by point count) and runs the full recognition chain on its own
// stream.  Concurrent streams overlap one pair's host round trips and small
// kernels with the other pairs' work.  Every pair's result is identical to
// a single rtr_recognize / rtr_recognize_learned call.
//
// The worker count (and the ICP lanes per point) can be chosen by
// rtr_batch_autotune, which times the candidates on the caller's batch.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "common.cuh"

namespace rtr {

static rtr_status ensure_workers(rtr_context* ctx, int n) {
  while ((int)ctx->workers.size() < n) {
    rtr_context* w = nullptr;
    RTR_TRY(rtr_context_create(ctx->device, &w));
    ctx->workers.push_back(w);
  }
  for (rtr_context* w : ctx->workers) {
    w->wait_budget_ms = ctx->wait_budget_ms;
    w->wait_budget_cycles = ctx->wait_budget_cycles;
    w->tune_icp_group = ctx->tune_icp_group;
  }
  return RTR_OK;
}

static int batch_workers(const rtr_context* ctx, int n_pairs) {
  int w = ctx->tune_batch_workers > 0 ? ctx->tune_batch_workers : 4;
  return w < n_pairs ? w : n_pairs;
}

static rtr_status run_batch(rtr_context* ctx, const rtr_batch_pair* pairs, int n_pairs, const rtr_recog_params* p,
                            const rtr_mlp* mlp, float keep, int nw, rtr_recog_result* d_results) {
  RTR_TRY(ensure_workers(ctx, nw));
  // largest pairs first, so the last ones to finish are short
  std::vector<int> order((size_t)n_pairs);
  for (int i = 0; i < n_pairs; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return pairs[a].n > pairs[b].n; });
  std::atomic<int> next{0};
  std::mutex mu;
  rtr_status first = RTR_OK;
  std::string first_msg;
  auto work = [&](int wi) {
    rtr_context* w = ctx->workers[wi];
    cudaStream_t st = w->host_stream;
    for (;;) {
      const int k = next.fetch_add(1);
      if (k >= n_pairs) break;
      const int i = order[k];
      const rtr_batch_pair& q = pairs[i];
      rtr_status r = mlp ? rtr_recognize_learned(w, q.model, mlp, keep, q.d_scene, q.n, p, d_results + i, st)
                         : rtr_recognize(w, q.model, q.d_scene, q.n, p, d_results + i, st);
      if (r == RTR_OK) r = rtr_context_check(w, st);
      if (r != RTR_OK) {
        std::lock_guard<std::mutex> lk(mu);
        if (first == RTR_OK) {
          first = r;
          first_msg = std::string("pair ") + std::to_string(i) + ": " + rtr_last_error();
        }
        break;
      }
    }
    cudaStreamSynchronize(st);
  };
  std::vector<std::thread> threads;
  for (int wi = 1; wi < nw; ++wi) threads.emplace_back(work, wi);
  work(0);
  for (auto& t : threads) t.join();
  RTR_CUDA(cudaSetDevice(ctx->device));
  if (first != RTR_OK) return fail(first, "rtr_recognize_batch: %s", first_msg.c_str());
  return RTR_OK;
}

}  // namespace rtr

using namespace rtr;

extern "C" {

rtr_status rtr_recognize_batch(rtr_context* ctx, const rtr_batch_pair* h_pairs, int n_pairs,
                               const rtr_recog_params* p, const rtr_mlp* mlp, float keep,
                               rtr_recog_result* d_results) {
  RTR_CHECK_ARG(ctx && p && n_pairs >= 0 && (n_pairs == 0 || (h_pairs && d_results)),
                "rtr_recognize_batch: bad arguments");
  RTR_CHECK_ARG(!mlp || (keep > 0.f && keep <= 1.f), "rtr_recognize_batch: keep must be in (0, 1]");
  for (int i = 0; i < n_pairs; ++i)
    RTR_CHECK_ARG(h_pairs[i].model && h_pairs[i].n >= 0 && (h_pairs[i].n == 0 || h_pairs[i].d_scene),
                  "rtr_recognize_batch: pair %d is incomplete", i);
  if (n_pairs == 0) return RTR_OK;
  RTR_CUDA(cudaSetDevice(ctx->device));
  RTR_CUDA(cudaDeviceSynchronize());  // inputs written on other streams are complete
  return run_batch(ctx, h_pairs, n_pairs, p, mlp, keep, batch_workers(ctx, n_pairs), d_results);
}

rtr_status rtr_batch_autotune(rtr_context* ctx, const rtr_batch_pair* h_pairs, int n_pairs,
                              const rtr_recog_params* p, const rtr_mlp* mlp, float keep,
                              rtr_recog_result* d_results, int* h_workers, int* h_icp_group) {
  RTR_CHECK_ARG(ctx && p && h_pairs && d_results && n_pairs > 0, "rtr_batch_autotune: bad arguments");
  RTR_CUDA(cudaSetDevice(ctx->device));
  static const int kWorkers[] = {1, 2, 4, 8};
  static const int kGroups[] = {4, 8};
  double best = 1e300;
  int bw = 4, bg = 0;
  const int saved_w = ctx->tune_batch_workers, saved_g = ctx->tune_icp_group;
  for (int g : kGroups) {
    for (int w : kWorkers) {
      if (w > n_pairs && w != 1) continue;
      ctx->tune_batch_workers = w;
      ctx->tune_icp_group = g;
      // one untimed pass (scratch growth, module load), then one timed pass
      rtr_status r = rtr_recognize_batch(ctx, h_pairs, n_pairs, p, mlp, keep, d_results);
      if (r != RTR_OK) {
        ctx->tune_batch_workers = saved_w;
        ctx->tune_icp_group = saved_g;
        return r;
      }
      const auto t0 = std::chrono::steady_clock::now();
      r = rtr_recognize_batch(ctx, h_pairs, n_pairs, p, mlp, keep, d_results);
      const double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      if (r != RTR_OK) {
        ctx->tune_batch_workers = saved_w;
        ctx->tune_icp_group = saved_g;
        return r;
      }
      if (dt < best) {
        best = dt;
        bw = w;
        bg = g;
      }
    }
  }
  ctx->tune_batch_workers = bw;
  ctx->tune_icp_group = bg;
  if (h_workers) *h_workers = bw;
  if (h_icp_group) *h_icp_group = bg;
  return RTR_OK;
}

}  // extern "C"
