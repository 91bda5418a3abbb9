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
#include "mf_pq.cuh"

namespace {
using mfpq::Bins;
using mfpq::KMAX;
using mfpq::make_bins;

// y = CDF(x), logdet = sum log pdf(x)
__global__ void pq_forward_kernel(const float* __restrict__ x, const float* __restrict__ params, int64_t N, int nb,
                                  int K, float* __restrict__ y, float* __restrict__ logdet) {
  int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= N) return;
  Bins b;
  float ld = 0.f;
  for (int d = 0; d < nb; ++d) {
    make_bins(params + ((int64_t)e * nb + d) * (2 * K + 1), K, b);
    float pdf;
    y[e * nb + d] = mfpq::pq_fwd1(b, K, x[e * nb + d], &pdf);
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
    float pdf;
    x[e * nb + d] = mfpq::pq_inv1(b, K, u[e * nb + d], &pdf);
    ld += __logf(pdf);
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
  float gl = gld ? gld[e] : 0.f;
  for (int d = 0; d < nb; ++d) {
    const int64_t o = ((int64_t)e * nb + d) * (2 * K + 1);
    gx[e * nb + d] = mfpq::pq_bwd1(params + o, K, x[e * nb + d], gy ? gy[e * nb + d] : 0.f, gl, gparams + o);
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
