// Piecewise-quadratic coupling transform of the normalizing-flow importance
// sampler (Mueller, McWilliams, Rousselle, Gross, Novak, "Neural Importance
// Sampling", ACM TOG 38 (2019) 145, section 3.3): per transformed dimension,
// K bin widths W = softmax(W~) and K+1 vertex heights V = exp(V~)/norm with
// norm = sum_k (exp V~_k + exp V~_{k+1})/2 W_k, a piecewise-linear density on
// [0,1] and its piecewise-quadratic CDF.
//
// Layouts: x, y [N][nb] (the transformed dimensions of one coupling layer),
// params [N][nb][2K+1] (W~ then V~, the conditioner network's output),
// logdet [N] = sum over the nb dimensions of log(pdf).  One thread per event.
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/madflow_gb300.h"

namespace {
constexpr int KMAX = 64;

struct Bins {
  float W[KMAX], V[KMAX + 1], E[KMAX + 1], C[KMAX + 1];  // widths, heights, edges, CDF at edges
};

__device__ __forceinline__ void make_bins(const float* __restrict__ p, int K, Bins& b) {
  float m = p[0];
  for (int k = 1; k < K; ++k) m = fmaxf(m, p[k]);
  float s = 0.f;
  for (int k = 0; k < K; ++k) {
    b.W[k] = __expf(p[k] - m);
    s += b.W[k];
  }
  float inv = 1.f / s;
  for (int k = 0; k < K; ++k) b.W[k] *= inv;
  float mv = p[K];
  for (int k = 1; k <= K; ++k) mv = fmaxf(mv, p[K + k]);
  for (int k = 0; k <= K; ++k) b.V[k] = __expf(p[K + k] - mv);
  float norm = 0.f;
  for (int k = 0; k < K; ++k) norm += 0.5f * (b.V[k] + b.V[k + 1]) * b.W[k];
  float in = 1.f / norm;
  for (int k = 0; k <= K; ++k) b.V[k] *= in;
  b.E[0] = 0.f;
  b.C[0] = 0.f;
  for (int k = 0; k < K; ++k) {
    b.E[k + 1] = b.E[k] + b.W[k];
    b.C[k + 1] = b.C[k] + 0.5f * (b.V[k] + b.V[k + 1]) * b.W[k];
  }
}

__device__ __forceinline__ int find_bin(const float* edges, int K, float x) {
  int b = 0;
  for (int k = 1; k < K; ++k) b += (x >= edges[k]) ? 1 : 0;
  return b;
}

// y = CDF(x), logdet = sum log pdf(x)
__global__ void pq_forward_kernel(const float* __restrict__ x, const float* __restrict__ params, int64_t N, int nb,
                                  int K, float* __restrict__ y, float* __restrict__ logdet) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= N) return;
  Bins b;
  float ld = 0.f;
  for (int d = 0; d < nb; ++d) {
    make_bins(params + ((int64_t)e * nb + d) * (2 * K + 1), K, b);
    float xv = fminf(fmaxf(x[e * nb + d], 0.f), 1.f);
    int k = find_bin(b.E, K, xv);
    float t = xv - b.E[k];
    float D = b.V[k + 1] - b.V[k];
    float pdf = b.V[k] + t / b.W[k] * D;
    y[e * nb + d] = fminf(b.C[k] + t * b.V[k] + 0.5f * t * t / b.W[k] * D, 1.f);
    ld += __logf(pdf);
  }
  logdet[e] = ld;
}

// x = CDF^-1(u), logdet = sum log pdf(x)
__global__ void pq_inverse_kernel(const float* __restrict__ u, const float* __restrict__ params, int64_t N, int nb,
                                  int K, float* __restrict__ x, float* __restrict__ logdet) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= N) return;
  Bins b;
  float ld = 0.f;
  for (int d = 0; d < nb; ++d) {
    make_bins(params + ((int64_t)e * nb + d) * (2 * K + 1), K, b);
    float uv = fminf(fmaxf(u[e * nb + d], 0.f), 1.f);
    int k = find_bin(b.C, K, uv);
    float r = fmaxf(uv - b.C[k], 0.f);
    float D = b.V[k + 1] - b.V[k];
    float a = 0.5f * b.W[k] * D, bq = b.W[k] * b.V[k];
    // alpha solving a alpha^2 + bq alpha = r, in the cancellation-free form
    float alpha = 2.f * r / (bq + sqrtf(fmaxf(bq * bq + 4.f * a * r, 0.f)));
    alpha = fminf(fmaxf(alpha, 0.f), 1.f);
    x[e * nb + d] = fminf(b.E[k] + alpha * b.W[k], 1.f);
    ld += __logf(b.V[k] + alpha * D);
  }
  logdet[e] = ld;
}

// Backward of pq_forward: gy [N][nb] = dL/dy, gld [N] = dL/dlogdet ->
// gx [N][nb], gparams [N][nb][2K+1].
__global__ void pq_backward_kernel(const float* __restrict__ x, const float* __restrict__ params,
                                   const float* __restrict__ gy, const float* __restrict__ gld, int64_t N, int nb,
                                   int K, float* __restrict__ gx, float* __restrict__ gparams) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= N) return;
  Bins b;
  float gW[KMAX], gV[KMAX + 1];
  float gl = gld ? gld[e] : 0.f;
  for (int d = 0; d < nb; ++d) {
    const float* p = params + ((int64_t)e * nb + d) * (2 * K + 1);
    make_bins(p, K, b);
    float xv = fminf(fmaxf(x[e * nb + d], 0.f), 1.f);
    float g = gy ? gy[e * nb + d] : 0.f;
    int k = find_bin(b.E, K, xv);
    float t = xv - b.E[k];
    float Wb = b.W[k];
    float D = b.V[k + 1] - b.V[k];
    float pdf = b.V[k] + t / Wb * D;
    float glp = gl / pdf;  // dL/dpdf
    gx[e * nb + d] = g * pdf + glp * D / Wb;
    for (int j = 0; j < K; ++j) gW[j] = 0.f;
    for (int j = 0; j <= K; ++j) gV[j] = 0.f;
    // y = c_k + t V_k + t^2/(2 W_k) D ; pdf = V_k + t/W_k D ; t = x - e_k
    for (int j = 0; j < k; ++j) {
      gW[j] += g * (0.5f * (b.V[j] + b.V[j + 1]) - pdf) + glp * (-D / Wb);
      gV[j] += g * 0.5f * b.W[j];
      gV[j + 1] += g * 0.5f * b.W[j];
    }
    gW[k] += g * (-0.5f * t * t * D / (Wb * Wb)) + glp * (-t * D / (Wb * Wb));
    gV[k] += g * (t - 0.5f * t * t / Wb) + glp * (1.f - t / Wb);
    gV[k + 1] += g * (0.5f * t * t / Wb) + glp * (t / Wb);
    // chain through V = exp(V~)/norm(W, V~) and W = softmax(W~)
    float S = 0.f;
    for (int j = 0; j <= K; ++j) S += gV[j] * b.V[j];
    float geff[KMAX];
    float sw = 0.f;
    for (int j = 0; j < K; ++j) {
      geff[j] = gW[j] - S * 0.5f * (b.V[j] + b.V[j + 1]);
      sw += geff[j] * b.W[j];
    }
    float* gp = gparams + ((int64_t)e * nb + d) * (2 * K + 1);
    for (int j = 0; j < K; ++j) gp[j] = b.W[j] * (geff[j] - sw);
    for (int j = 0; j <= K; ++j) {
      float wl = j > 0 ? b.W[j - 1] : 0.f, wr = j < K ? b.W[j] : 0.f;
      gp[K + j] = b.V[j] * (gV[j] - S * 0.5f * (wl + wr));
    }
  }
}

int launch_check() { return cudaPeekAtLastError() == cudaSuccess ? MF_OK : MF_ERR_CUDA; }
}  // namespace

extern "C" {

int mf_pq_forward(const float* x, const float* params, int64_t n, int nb, int K, float* y, float* logdet,
                  void* stream) {
  if (n < 0 || nb <= 0 || K < 2 || K > KMAX || (n > 0 && (!x || !params || !y || !logdet))) return MF_ERR_ARG;
  if (n == 0) return MF_OK;
  pq_forward_kernel<<<(int)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(x, params, n, nb, K, y, logdet);
  return launch_check();
}

int mf_pq_inverse(const float* u, const float* params, int64_t n, int nb, int K, float* x, float* logdet,
                  void* stream) {
  if (n < 0 || nb <= 0 || K < 2 || K > KMAX || (n > 0 && (!u || !params || !x || !logdet))) return MF_ERR_ARG;
  if (n == 0) return MF_OK;
  pq_inverse_kernel<<<(int)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(u, params, n, nb, K, x, logdet);
  return launch_check();
}

int mf_pq_backward(const float* x, const float* params, const float* gy, const float* glogdet, int64_t n, int nb,
                   int K, float* gx, float* gparams, void* stream) {
  if (n < 0 || nb <= 0 || K < 2 || K > KMAX || (n > 0 && (!x || !params || !gx || !gparams))) return MF_ERR_ARG;
  if (n == 0) return MF_OK;
  pq_backward_kernel<<<(int)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(x, params, gy, glogdet, n, nb, K, gx,
                                                                              gparams);
  return launch_check();
}

int mf_flow_fwd(const float* x, const float* params, int64_t n, int nb, int K, float* y, float* logdet,
                void* stream) {
  return mf_pq_forward(x, params, n, nb, K, y, logdet, stream);
}
int mf_flow_inv(const float* u, const float* params, int64_t n, int nb, int K, float* x, float* logdet,
                void* stream) {
  return mf_pq_inverse(u, params, n, nb, K, x, logdet, stream);
}
int mf_flow_grad(const float* x, const float* params, const float* gy, const float* glogdet, int64_t n, int nb, int K,
                 float* gx, float* gparams, void* stream) {
  return mf_pq_backward(x, params, gy, glogdet, n, nb, K, gx, gparams, stream);
}

}  // extern "C"
