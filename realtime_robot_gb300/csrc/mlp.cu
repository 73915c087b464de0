// mlp.cu — the keypoint-credibility MLP: inference, gradients and Adam.
//
// 352 -> 128 -> 64 -> 1 (ReLU, ReLU, sigmoid) over SHOT-352 descriptors.
// Parameters live on the device as FP32 master weights plus BF16 copies of
// the three weight matrices; every forward pass multiplies by the BF16
// copies and accumulates in FP32.  Training is minibatch Adam on the mean
// binary cross-entropy of the logit; gradients flow to the master weights
// with the BF16 rounding treated as the identity.
//
// At these shapes (a 4096-row batch is 0.37 GFLOP forward) every product is
// a small GEMM; they share one tiled SIMT kernel (64 x 64 tiles, K steps of
// 16, 4 x 4 outputs per thread) whose operand strides express the
// transposes, and whose epilogue fuses the bias, the ReLU and the ReLU mask
// of the backward pass.  Reductions are fixed-order, so results repeat run
// to run.
#include <cuda_bf16.h>
#include <string.h>

#include <vector>

#include "common.cuh"

struct rtr_mlp {
  int device = 0;
  float* theta = nullptr;          // [RTR_MLP_PARAMS] FP32 master weights
  __nv_bfloat16* wbf = nullptr;    // BF16 W1 | W2 | w3
  __nv_bfloat16* w1pad = nullptr;  // BF16 W1 as [128][384], zero past column 352 (tensor-core inference)
  float* m = nullptr;              // Adam first moment
  float* v = nullptr;              // Adam second moment
  int step = 0;                    // Adam steps taken
  uint64_t uid = 0;                // identity for captured recognitions (rtr::next_uid)
};

uint64_t rtr_mlp_uid(const rtr_mlp* m) { return m ? m->uid : 0; }

namespace rtr {

constexpr int MLP_IN = 352, MLP_H1 = 128, MLP_H2 = 64;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + MLP_H1 * MLP_IN, OFF_W2 = OFF_B1 + MLP_H1,
              OFF_B2 = OFF_W2 + MLP_H2 * MLP_H1, OFF_W3 = OFF_B2 + MLP_H2, OFF_B3 = OFF_W3 + MLP_H2,
              N_PARAMS = OFF_B3 + 1;
static_assert(N_PARAMS == RTR_MLP_PARAMS, "parameter layout");
constexpr int BF_W1 = 0, BF_W2 = MLP_H1 * MLP_IN, BF_W3 = BF_W2 + MLP_H2 * MLP_H1, BF_N = BF_W3 + MLP_H2;

// ---------------------------------------------------------------------------
// tiled SIMT GEMM: C[m][n] = sum_k A(m, k) B(n, k), then the epilogue
//   A(m, k) = A[m * sam + k * sak], B(n, k) = B[n * sbn + k * sbk]
// EPI 0: store; 1: + bias[n], ReLU; 2: * (mask[m * ldc + n] > 0)
// ---------------------------------------------------------------------------
constexpr int GT = 64, GK = 16;

template <typename TB>
__device__ __forceinline__ float ldB(const TB* p);
template <>
__device__ __forceinline__ float ldB<float>(const float* p) {
  return *p;
}
template <>
__device__ __forceinline__ float ldB<__nv_bfloat16>(const __nv_bfloat16* p) {
  return __bfloat162float(*p);
}

template <typename TB, int EPI>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float* __restrict__ A, long long sam,
                                              long long sak, const TB* __restrict__ B, long long sbn, long long sbk,
                                              float* __restrict__ Cm, int ldc, const float* __restrict__ bias,
                                              const float* __restrict__ mask, const int* __restrict__ dM) {
  __shared__ float As[GK][GT + 4], Bs[GK][GT + 4];
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int m0 = blockIdx.y * GT, n0 = blockIdx.x * GT;
  if (dM) M = min(*dM, M);  // rows counted on the device (grid sized for the capacity)
  if (m0 >= M) return;      // uniform per block, before any barrier
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  const bool a_mfast = sam == 1, b_nfast = sbn == 1;
  for (int k0 = 0; k0 < K; k0 += GK) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int e = tid + 256 * r;  // element of the 64 x 16 tile
      int mm, kk;
      if (a_mfast) {
        mm = e & 63;
        kk = e >> 6;
      } else {
        kk = e & 15;
        mm = e >> 4;
      }
      const int gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? A[(long long)gm * sam + (long long)gk * sak] : 0.f;
      int nn, kb;
      if (b_nfast) {
        nn = e & 63;
        kb = e >> 6;
      } else {
        kb = e & 15;
        nn = e >> 4;
      }
      const int gn = n0 + nn, gkb = k0 + kb;
      Bs[kb][nn] = (gn < N && gkb < K) ? ldB<TB>(B + (long long)gn * sbn + (long long)gkb * sbk) : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int gm = m0 + ty + 16 * i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int gn = n0 + tx + 16 * j;
      if (gn >= N) continue;
      float c = acc[i][j];
      if (EPI == 1) c = fmaxf(c + bias[gn], 0.f);
      if (EPI == 2) c = mask[(long long)gm * ldc + gn] > 0.f ? c : 0.f;
      Cm[(long long)gm * ldc + gn] = c;
    }
  }
}

template <typename TB, int EPI>
static void gemm(int M, int N, int K, const float* A, long long sam, long long sak, const TB* B, long long sbn,
                 long long sbk, float* C, int ldc, const float* bias, const float* mask, cudaStream_t st,
                 const int* dM = nullptr) {
  const dim3 grid((N + GT - 1) / GT, (M + GT - 1) / GT);
  k_gemm<TB, EPI><<<grid, 256, 0, st>>>(M, N, K, A, sam, sak, B, sbn, sbk, C, ldc, bias, mask, dM);
  RTR_LAUNCHED(1);
}

// ---------------------------------------------------------------------------
// head: z = h2 . w3 + b3 per row; score = sigmoid(z); with labels also the
// loss terms, dz = (sigmoid(z) - y) / n and dh2 = dz w3 (h2 > 0)
// ---------------------------------------------------------------------------
__global__ void k_head(const float* __restrict__ h2, int n, const __nv_bfloat16* __restrict__ w3bf,
                       const float* __restrict__ theta, const float* __restrict__ y, float* __restrict__ score,
                       float* __restrict__ dz, float* __restrict__ dh2, float* __restrict__ loss_terms,
                       const int* __restrict__ d_n) {
  if (d_n) n = min(*d_n, n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float* h = h2 + (size_t)i * MLP_H2;
    float z = 0.f;
#pragma unroll 8
    for (int j = 0; j < MLP_H2; ++j) z = fmaf(h[j], __bfloat162float(w3bf[j]), z);
    z += theta[OFF_B3];
    const float s = 1.f / (1.f + __expf(-z));
    if (score) score[i] = s;
    if (y) {
      const float yi = y[i];
      loss_terms[i] = fmaxf(z, 0.f) - yi * z + log1pf(__expf(-fabsf(z)));
      const float d = (s - yi) / (float)n;
      dz[i] = d;
      for (int j = 0; j < MLP_H2; ++j) dh2[(size_t)i * MLP_H2 + j] = h[j] > 0.f ? d * __bfloat162float(w3bf[j]) : 0.f;
    }
  }
}

// Column sums of an n x cols row-major matrix (fixed order: per thread a
// strided partial, then a tree over the block): out[c] = sum_i X[i][c].
__global__ void k_colsum(const float* __restrict__ X, int n, int cols, float* __restrict__ out) {
  __shared__ float s[256];
  const int c = blockIdx.x;
  float a = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) a += X[(size_t)i * cols + c];
  s[threadIdx.x] = a;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[c] = s[0];
}

constexpr int W1PAD_K = 384;
__global__ void k_to_bf16(const float* __restrict__ theta, __nv_bfloat16* __restrict__ wbf,
                          __nv_bfloat16* __restrict__ w1pad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < BF_N; i += gridDim.x * blockDim.x) {
    const int src = i < BF_W2 ? OFF_W1 + i : (i < BF_W3 ? OFF_W2 + (i - BF_W2) : OFF_W3 + (i - BF_W3));
    wbf[i] = __float2bfloat16_rn(theta[src]);
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < MLP_H1 * W1PAD_K; i += gridDim.x * blockDim.x) {
    const int r = i / W1PAD_K, k = i - r * W1PAD_K;
    w1pad[i] = __float2bfloat16_rn(k < MLP_IN ? theta[OFF_W1 + r * MLP_IN + k] : 0.f);
  }
}

__global__ void k_adam(float* __restrict__ theta, const float* __restrict__ g, float* __restrict__ m,
                       float* __restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    theta[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void k_sum(const float* __restrict__ x, int n, float* __restrict__ out) {
  __shared__ float s[256];
  float a = 0.f;
  for (int i = threadIdx.x; i < n; i += blockDim.x) a += x[i];
  s[threadIdx.x] = a;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0] / (float)(n > 0 ? n : 1);
}

__global__ void k_accum(float* __restrict__ acc, const float* __restrict__ x, float w) { *acc += w * *x; }

__global__ void k_gather_rows(const float* __restrict__ X, const float* __restrict__ y, const int* __restrict__ idx,
                              int n, float* __restrict__ Xo, float* __restrict__ yo) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)n * MLP_IN;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / MLP_IN), c = (int)(e - (long long)r * MLP_IN);
    Xo[e] = X[(size_t)idx[r] * MLP_IN + c];
    if (c == 0) yo[r] = y[idx[r]];
  }
}

// Scratch of one forward/backward over n rows.
struct MlpWork {
  float *h1, *h2, *dz, *dh2, *dh1, *loss_terms, *grad;
};

static void mlp_plan(ScratchPlan& p, int n) {
  p.add<float>((size_t)n * MLP_H1);
  p.add<float>((size_t)n * MLP_H2);
  p.add<float>(n);
  p.add<float>((size_t)n * MLP_H2);
  p.add<float>((size_t)n * MLP_H1);
  p.add<float>(n);
  p.add<float>(N_PARAMS);
}

static bool mlp_take(Scratch& s, int n, MlpWork* w) {
  w->h1 = s.take<float>((size_t)n * MLP_H1);
  w->h2 = s.take<float>((size_t)n * MLP_H2);
  w->dz = s.take<float>(n);
  w->dh2 = s.take<float>((size_t)n * MLP_H2);
  w->dh1 = s.take<float>((size_t)n * MLP_H1);
  w->loss_terms = s.take<float>(n);
  w->grad = s.take<float>(N_PARAMS);
  return w->grad != nullptr;
}

// Forward over n rows of X; with y also the loss (mean, into *d_loss) and
// the gradient (into w.grad).
static void mlp_pass(const rtr_mlp* m, const float* X, const float* y, int n, float* score, const MlpWork& w,
                     float* d_loss, cudaStream_t st) {
  const float* th = m->theta;
  // h1 = relu(X W1^T + b1), h2 = relu(h1 W2^T + b2)
  gemm<__nv_bfloat16, 1>(n, MLP_H1, MLP_IN, X, MLP_IN, 1, m->wbf + BF_W1, MLP_IN, 1, w.h1, MLP_H1, th + OFF_B1,
                         nullptr, st);
  gemm<__nv_bfloat16, 1>(n, MLP_H2, MLP_H1, w.h1, MLP_H1, 1, m->wbf + BF_W2, MLP_H1, 1, w.h2, MLP_H2, th + OFF_B2,
                         nullptr, st);
  int hb = (n + 255) / 256;
  if (hb > 152 * 8) hb = 152 * 8;
  if (hb < 1) hb = 1;
  k_head<<<hb, 256, 0, st>>>(w.h2, n, m->wbf + BF_W3, th, y, score, w.dz, w.dh2, w.loss_terms, nullptr);
  RTR_LAUNCHED(1);
  if (!y) return;
  float* g = w.grad;
  // dw3[j] = sum_i dz_i h2[i][j]; db3 = sum_i dz_i
  gemm<float, 0>(1, MLP_H2, n, w.dz, 0, 1, w.h2, 1, MLP_H2, g + OFF_W3, MLP_H2, nullptr, nullptr, st);
  k_colsum<<<1, 256, 0, st>>>(w.dz, n, 1, g + OFF_B3);
  // dW2[j][k] = sum_i dh2[i][j] h1[i][k]; db2 = column sums of dh2
  gemm<float, 0>(MLP_H2, MLP_H1, n, w.dh2, 1, MLP_H2, w.h1, 1, MLP_H1, g + OFF_W2, MLP_H1, nullptr, nullptr, st);
  k_colsum<<<MLP_H2, 256, 0, st>>>(w.dh2, n, MLP_H2, g + OFF_B2);
  // dh1 = (dh2 W2) * (h1 > 0): C[i][k] = sum_j dh2[i][j] W2[j][k]
  gemm<__nv_bfloat16, 2>(n, MLP_H1, MLP_H2, w.dh2, MLP_H2, 1, m->wbf + BF_W2, 1, MLP_H1, w.dh1, MLP_H1, nullptr,
                         w.h1, st);
  // dW1[j][k] = sum_i dh1[i][j] X[i][k]; db1 = column sums of dh1
  gemm<float, 0>(MLP_H1, MLP_IN, n, w.dh1, 1, MLP_H1, X, 1, MLP_IN, g + OFF_W1, MLP_IN, nullptr, nullptr, st);
  k_colsum<<<MLP_H1, 256, 0, st>>>(w.dh1, n, MLP_H1, g + OFF_B1);
  k_sum<<<1, 256, 0, st>>>(w.loss_terms, n, d_loss);
  RTR_LAUNCHED(4);
}

static void mlp_refresh_bf16(rtr_mlp* m, cudaStream_t st) {
  k_to_bf16<<<(BF_N + 255) / 256, 256, 0, st>>>(m->theta, m->wbf, m->w1pad);
  RTR_LAUNCHED(1);
}

static void mlp_adam(rtr_mlp* m, const float* grad, float lr, cudaStream_t st) {
  m->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)m->step), c2 = 1.f - powf(b2, (float)m->step);
  k_adam<<<(N_PARAMS + 255) / 256, 256, 0, st>>>(m->theta, grad, m->m, m->v, N_PARAMS, lr, b1, b2, 1e-8f, c1, c2);
  RTR_LAUNCHED(1);
  mlp_refresh_bf16(m, st);
}

// He-uniform initialisation on the host (SplitMix64 stream, bound
// sqrt(6 / fan_in)), zero biases.
static void mlp_host_init(uint64_t seed, float* out) {
  uint64_t s = seed;
  auto next = [&s]() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  auto uni = [&next](float bound) { return (float)((double)(next() >> 11) * 0x1.0p-53 * 2.0 - 1.0) * bound; };
  memset(out, 0, sizeof(float) * N_PARAMS);
  const float bw1 = sqrtf(6.f / MLP_IN), bw2 = sqrtf(6.f / MLP_H1), bw3 = sqrtf(6.f / MLP_H2);
  for (int i = 0; i < MLP_H1 * MLP_IN; ++i) out[OFF_W1 + i] = uni(bw1);
  for (int i = 0; i < MLP_H2 * MLP_H1; ++i) out[OFF_W2 + i] = uni(bw2);
  for (int i = 0; i < MLP_H2; ++i) out[OFF_W3 + i] = uni(bw3);
}

size_t mlp_tc_bytes(int n_cap);
rtr_status mlp_tc_score(rtr_context* ctx, Scratch& s, const float* X, int n_cap, const int* d_n,
                        const __nv_bfloat16* w1pad, const float* b1, const __nv_bfloat16* w2, const float* b2,
                        const __nv_bfloat16* w3, const float* b3, float* score, cudaStream_t st);

// Inference on the tensor cores (match_tc.cu: layer 1 as a tcgen05 GEMM of
// three BF16 parts of X, layers 2 and 3 in its epilogue) when X is 16-byte
// aligned; the SIMT passes otherwise.
static bool mlp_tc_ok(const float* X) { return (reinterpret_cast<uintptr_t>(X) & 15u) == 0; }
static rtr_status mlp_tc(rtr_context* ctx, Scratch& s, const rtr_mlp* m, const float* X, int n_cap, const int* d_n,
                         float* score, cudaStream_t st) {
  const float* th = m->theta;
  return mlp_tc_score(ctx, s, X, n_cap, d_n, m->w1pad, th + OFF_B1, m->wbf + BF_W2, th + OFF_B2, m->wbf + BF_W3,
                      th + OFF_B3, score, st);
}

rtr_status mlp_score_dev(rtr_context* ctx, Scratch& s, const rtr_mlp* m, const float* X, int n, float* score,
                         cudaStream_t st) {
  if (n <= 0) return RTR_OK;
  if (mlp_tc_ok(X)) return mlp_tc(ctx, s, m, X, n, nullptr, score, st);
  MlpWork w;
  if (!mlp_take(s, n, &w)) return fail(RTR_ERR_CAPACITY, "mlp: scratch");
  (void)ctx;
  mlp_pass(m, X, nullptr, n, score, w, nullptr, st);
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

// Scores of the first *d_n (<= n_cap) rows of X, for callers whose row count
// lives on the device; needs mlp_infer_bytes(n_cap) of scratch.
size_t mlp_infer_bytes(int n_cap) {
  ScratchPlan p;
  p.add<float>((size_t)(n_cap > 0 ? n_cap : 1) * MLP_H1);
  p.add<float>((size_t)(n_cap > 0 ? n_cap : 1) * MLP_H2);
  const size_t tc = mlp_tc_bytes(n_cap);
  return p.bytes > tc ? p.bytes : tc;
}

rtr_status mlp_score_rows(rtr_context* ctx, Scratch& s, const rtr_mlp* m, const float* X, int n_cap, const int* d_n,
                          float* score, cudaStream_t st) {
  if (n_cap <= 0) return RTR_OK;
  if (mlp_tc_ok(X)) return mlp_tc(ctx, s, m, X, n_cap, d_n, score, st);
  float* h1 = s.take<float>((size_t)n_cap * MLP_H1);
  float* h2 = s.take<float>((size_t)n_cap * MLP_H2);
  if (!h2) return fail(RTR_ERR_CAPACITY, "mlp: scratch");
  const float* th = m->theta;
  gemm<__nv_bfloat16, 1>(n_cap, MLP_H1, MLP_IN, X, MLP_IN, 1, m->wbf + BF_W1, MLP_IN, 1, h1, MLP_H1, th + OFF_B1,
                         nullptr, st, d_n);
  gemm<__nv_bfloat16, 1>(n_cap, MLP_H2, MLP_H1, h1, MLP_H1, 1, m->wbf + BF_W2, MLP_H1, 1, h2, MLP_H2, th + OFF_B2,
                         nullptr, st, d_n);
  int hb = (n_cap + 255) / 256;
  if (hb > 152 * 8) hb = 152 * 8;
  k_head<<<hb, 256, 0, st>>>(h2, n_cap, m->wbf + BF_W3, th, nullptr, score, nullptr, nullptr, nullptr, d_n);
  RTR_LAUNCHED(1);
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

size_t mlp_scratch_bytes(int n) {
  ScratchPlan p;
  mlp_plan(p, n > 0 ? n : 1);
  return p.bytes;
}

}  // namespace rtr

using namespace rtr;

extern "C" {

rtr_status rtr_mlp_create(rtr_context* ctx, const float* h_params, uint64_t seed, rtr_mlp** out) {
  RTR_CHECK_ARG(ctx && out, "rtr_mlp_create: bad arguments");
  *out = nullptr;
  RTR_CUDA(cudaSetDevice(ctx->device));
  std::vector<float> init;
  if (!h_params) {
    init.resize(N_PARAMS);
    mlp_host_init(seed, init.data());
    h_params = init.data();
  }
  rtr_mlp* m = new rtr_mlp();
  m->device = ctx->device;
  m->uid = next_uid();
  if (cudaMalloc(&m->theta, sizeof(float) * N_PARAMS) != cudaSuccess ||
      cudaMalloc(&m->wbf, sizeof(__nv_bfloat16) * BF_N) != cudaSuccess ||
      cudaMalloc(&m->w1pad, sizeof(__nv_bfloat16) * MLP_H1 * W1PAD_K) != cudaSuccess ||
      cudaMalloc(&m->m, sizeof(float) * N_PARAMS) != cudaSuccess ||
      cudaMalloc(&m->v, sizeof(float) * N_PARAMS) != cudaSuccess) {
    cudaFree(m->theta);
    cudaFree(m->wbf);
    cudaFree(m->w1pad);
    cudaFree(m->m);
    cudaFree(m->v);
    delete m;
    (void)cudaGetLastError();
    return fail(RTR_ERR_OOM, "rtr_mlp_create: device allocation failed");
  }
  RTR_CUDA(cudaMemcpy(m->theta, h_params, sizeof(float) * N_PARAMS, cudaMemcpyHostToDevice));
  RTR_CUDA(cudaMemset(m->m, 0, sizeof(float) * N_PARAMS));
  RTR_CUDA(cudaMemset(m->v, 0, sizeof(float) * N_PARAMS));
  mlp_refresh_bf16(m, 0);
  RTR_CUDA(cudaDeviceSynchronize());
  *out = m;
  return RTR_OK;
}

rtr_status rtr_mlp_destroy(rtr_mlp* m) {
  if (!m) return RTR_OK;
  cudaSetDevice(m->device);
  cudaFree(m->theta);
  cudaFree(m->wbf);
  cudaFree(m->w1pad);
  cudaFree(m->m);
  cudaFree(m->v);
  delete m;
  return RTR_OK;
}

rtr_status rtr_mlp_get_params(const rtr_mlp* m, float* h_params) {
  RTR_CHECK_ARG(m && h_params, "rtr_mlp_get_params: bad arguments");
  RTR_CUDA(cudaSetDevice(m->device));
  RTR_CUDA(cudaDeviceSynchronize());
  RTR_CUDA(cudaMemcpy(h_params, m->theta, sizeof(float) * N_PARAMS, cudaMemcpyDeviceToHost));
  return RTR_OK;
}

rtr_status rtr_mlp_set_params(rtr_mlp* m, const float* h_params) {
  RTR_CHECK_ARG(m && h_params, "rtr_mlp_set_params: bad arguments");
  RTR_CUDA(cudaSetDevice(m->device));
  RTR_CUDA(cudaDeviceSynchronize());
  RTR_CUDA(cudaMemcpy(m->theta, h_params, sizeof(float) * N_PARAMS, cudaMemcpyHostToDevice));
  RTR_CUDA(cudaMemset(m->m, 0, sizeof(float) * N_PARAMS));
  RTR_CUDA(cudaMemset(m->v, 0, sizeof(float) * N_PARAMS));
  m->step = 0;
  mlp_refresh_bf16(m, 0);
  RTR_CUDA(cudaDeviceSynchronize());
  return RTR_OK;
}

rtr_status rtr_mlp_score(rtr_context* ctx, const rtr_mlp* m, const float* d_x, int n, float* d_score,
                         rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && m && n >= 0, "rtr_mlp_score: bad arguments");
  if (n == 0) return RTR_OK;
  RTR_CHECK_ARG(d_x && d_score, "rtr_mlp_score: NULL input or output");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  Scratch s;
  const size_t need = mlp_scratch_bytes(n) > mlp_tc_bytes(n) ? mlp_scratch_bytes(n) : mlp_tc_bytes(n);
  RTR_TRY(ensure_scratch(ctx, need, st, &s));
  ProfScope ps(ctx, st, "mlp_score");
  return mlp_score_dev(ctx, s, m, d_x, n, d_score, st);
}

rtr_status rtr_mlp_loss_grad(rtr_context* ctx, const rtr_mlp* m, const float* d_x, const float* d_y, int n,
                             float* d_grad, float* d_loss, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && m && n > 0 && d_x && d_y && d_grad && d_loss, "rtr_mlp_loss_grad: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, mlp_scratch_bytes(n), st, &s));
  MlpWork w;
  if (!mlp_take(s, n, &w)) return fail(RTR_ERR_CAPACITY, "mlp: scratch");
  mlp_pass(m, d_x, d_y, n, nullptr, w, d_loss, st);
  RTR_CUDA(cudaMemcpyAsync(d_grad, w.grad, sizeof(float) * N_PARAMS, cudaMemcpyDeviceToDevice, st));
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

rtr_status rtr_mlp_train_step(rtr_context* ctx, rtr_mlp* m, const float* d_x, const float* d_y, int n, float lr,
                              float* d_loss, rtr_stream_t stream) {
  RTR_CHECK_ARG(ctx && m && n > 0 && d_x && d_y && d_loss && lr > 0.f, "rtr_mlp_train_step: bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  RTR_CUDA(cudaSetDevice(ctx->device));
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, mlp_scratch_bytes(n), st, &s));
  MlpWork w;
  if (!mlp_take(s, n, &w)) return fail(RTR_ERR_CAPACITY, "mlp: scratch");
  mlp_pass(m, d_x, d_y, n, nullptr, w, d_loss, st);
  mlp_adam(m, w.grad, lr, st);
  RTR_CUDA(cudaGetLastError());
  return RTR_OK;
}

rtr_status rtr_mlp_train(rtr_context* ctx, rtr_mlp* m, const float* d_x, const float* d_y, int n, int batch,
                         int epochs, float lr, uint64_t seed, float* h_epoch_loss) {
  RTR_CHECK_ARG(ctx && m && d_x && d_y && n > 0 && batch > 0 && epochs > 0 && lr > 0.f,
                "rtr_mlp_train: bad arguments");
  RTR_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = ctx->host_stream;
  const int b = batch < n ? batch : n;
  ScratchPlan plan;
  mlp_plan(plan, b);
  plan.add<float>((size_t)b * MLP_IN);
  plan.add<float>(b);
  plan.add<int>(n);
  plan.add<float>(epochs * 2 + 2);
  Scratch s;
  RTR_TRY(ensure_scratch(ctx, plan.bytes, st, &s));
  MlpWork w;
  if (!mlp_take(s, b, &w)) return fail(RTR_ERR_CAPACITY, "mlp: scratch");
  float* xb = s.take<float>((size_t)b * MLP_IN);
  float* yb = s.take<float>(b);
  int* perm = s.take<int>(n);
  float* losses = s.take<float>(epochs * 2 + 2);
  if (!losses) return fail(RTR_ERR_CAPACITY, "mlp: scratch");
  // the epoch order: a seeded Fisher-Yates shuffle on the host, one copy per epoch
  std::vector<int> order((size_t)n);
  for (int i = 0; i < n; ++i) order[i] = i;
  uint64_t rs = seed;
  auto next = [&rs]() {
    uint64_t z = (rs += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  };
  const int nb = (n + b - 1) / b;
  for (int e = 0; e < epochs; ++e) {
    for (int i = n - 1; i > 0; --i) {
      const int j = (int)(next() % (uint64_t)(i + 1));
      const int t = order[i];
      order[i] = order[j];
      order[j] = t;
    }
    RTR_CUDA(cudaMemcpyAsync(perm, order.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, st));
    RTR_CUDA(cudaMemsetAsync(losses + 2 * e, 0, sizeof(float), st));
    for (int k = 0; k < nb; ++k) {
      const int r0 = k * b, rn = (r0 + b <= n) ? b : n - r0;
      k_gather_rows<<<152 * 4, 256, 0, st>>>(d_x, d_y, perm + r0, rn, xb, yb);
      RTR_LAUNCHED(1);
      mlp_pass(m, xb, yb, rn, nullptr, w, losses + 2 * e + 1, st);
      mlp_adam(m, w.grad, lr, st);
      k_accum<<<1, 1, 0, st>>>(losses + 2 * e, losses + 2 * e + 1, (float)rn / (float)n);
      RTR_LAUNCHED(1);
    }
    RTR_CUDA(cudaGetLastError());
  }
  std::vector<float> h((size_t)epochs * 2);
  RTR_CUDA(cudaMemcpyAsync(h.data(), losses, sizeof(float) * h.size(), cudaMemcpyDeviceToHost, st));
  RTR_CUDA(cudaStreamSynchronize(st));
  if (h_epoch_loss)
    for (int e = 0; e < epochs; ++e) h_epoch_loss[e] = h[(size_t)2 * e];
  return RTR_OK;
}

}  // extern "C"
