// Piecewise-quadratic coupling transform of the normalizing-flow importance
// sampler (Mueller, McWilliams, Rousselle, Gross, Novak, "Neural Importance
// Sampling", ACM TOG 38 (2019) 145, section 3.3), per transformed dimension:
// K bin widths W = softmax(W~) and K+1 vertex heights V = exp(V~)/norm with
// norm = sum_k (exp V~_k + exp V~_{k+1})/2 W_k, a piecewise-linear density on
// [0,1] and its piecewise-quadratic CDF.  Device functions shared by the
// stand-alone transform kernels (mf_flow.cu) and the whole-layer kernels
// (mf_flow_train.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mfpq {
constexpr int KMAX = 64;

struct Bins {
  float W[KMAX], V[KMAX + 1], E[KMAX + 1], C[KMAX + 1];  // widths, heights, edges, CDF at edges
};

// the bins of one dimension from its 2K+1 raw parameters p (W~ then V~)
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

// y = CDF(x) of one dimension; pdf(x) in *pdf
__device__ __forceinline__ float pq_fwd1(const Bins& b, int K, float x, float* pdf) {
  float xv = fminf(fmaxf(x, 0.f), 1.f);
  int k = find_bin(b.E, K, xv);
  float t = xv - b.E[k];
  float D = b.V[k + 1] - b.V[k];
  *pdf = b.V[k] + t / b.W[k] * D;
  return fminf(b.C[k] + t * b.V[k] + 0.5f * t * t / b.W[k] * D, 1.f);
}

// x = CDF^-1(u) of one dimension; pdf(x) in *pdf
__device__ __forceinline__ float pq_inv1(const Bins& b, int K, float u, float* pdf) {
  float uv = fminf(fmaxf(u, 0.f), 1.f);
  int k = find_bin(b.C, K, uv);
  float r = fmaxf(uv - b.C[k], 0.f);
  float D = b.V[k + 1] - b.V[k];
  float a = 0.5f * b.W[k] * D, bq = b.W[k] * b.V[k];
  // alpha solving a alpha^2 + bq alpha = r, in the cancellation-free form
  float alpha = 2.f * r / (bq + sqrtf(fmaxf(bq * bq + 4.f * a * r, 0.f)));
  alpha = fminf(fmaxf(alpha, 0.f), 1.f);
  *pdf = b.V[k] + alpha * D;
  return fminf(b.E[k] + alpha * b.W[k], 1.f);
}

// Backward of pq_fwd1 for one dimension: g = dL/dy, gl = dL/dlogdet (log
// pdf enters the log-determinant); returns dL/dx and writes dL/dp to gp
// [2K+1].  The raw parameters p are read before gp is written, so gp may
// be p itself.
__device__ __forceinline__ float pq_bwd1(const float* p, int K, float x, float g, float gl, float* gp) {
  Bins b;
  make_bins(p, K, b);
  float gW[KMAX], gV[KMAX + 1];
  float xv = fminf(fmaxf(x, 0.f), 1.f);
  int k = find_bin(b.E, K, xv);
  float t = xv - b.E[k];
  float Wb = b.W[k];
  float D = b.V[k + 1] - b.V[k];
  float pdf = b.V[k] + t / Wb * D;
  float glp = gl / pdf;  // dL/dpdf
  const float gx = g * pdf + glp * D / Wb;
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
  for (int j = 0; j < K; ++j) gp[j] = b.W[j] * (geff[j] - sw);
  for (int j = 0; j <= K; ++j) {
    float wl = j > 0 ? b.W[j - 1] : 0.f, wr = j < K ? b.W[j] : 0.f;
    gp[K + j] = b.V[j] * (gV[j] - S * 0.5f * (wl + wr));
  }
  return gx;
}
}  // namespace mfpq
