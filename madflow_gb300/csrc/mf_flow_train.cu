// Whole coupling layers of the normalizing-flow sampler in hand-written
// kernels: the conditioner MLP na -> 64 -> 64 -> nb (2K+1) (ReLU) and the
// piecewise-quadratic transform of mf_pq.cuh, for training (density
// direction and its gradient) and for sampling at any size the tensor-core
// sampling layer does not take.  FP32 throughout.
//
//   flow_layer_kernel<K, INV>   one thread per point: the MLP from the
//                               conditioning dimensions ia (read as 2z - 1),
//                               then the transform (INV = false: density,
//                               y = CDF(x); INV = true: sampling, x =
//                               CDF^-1(u)) of the dimensions ib; logq +=
//                               sum of log pdf
//   flow_grad_kernel<K>         tiles of 32 points, 256 threads: the MLP
//                               forward again (H1, H2, P as tiles in shared
//                               memory), the transform's backward per (point,
//                               dimension), then the MLP backward as small
//                               GEMMs over the tile: dL/dW, dL/db into this
//                               block's partial sums, dL/dz to g_in
//   flow_grad_reduce_kernel     the partial sums of all blocks in a fixed
//                               order: the weight gradients
//
// Weights in torch.nn.Linear layout (out x in).  In shared memory the rows of
// W2 and W3 are padded to 65 floats and those of W1 to an odd length, so a
// warp reading a column (threads along the rows) or a row (threads along the
// columns) hits 32 different banks either way.  Every gradient element is
// summed by one thread in a fixed order, so a gradient is reproducible for a
// given grid (one block per SM).
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/madflow_gb300.h"
#include "mf_pq.cuh"

namespace {
constexpr int FH = 64;        // hidden units of the conditioner
constexpr int FH_P = FH + 1;  // padded row of W2 and W3 in shared memory
constexpr int FA_MAX = 16;    // conditioning dimensions
constexpr int FB_MAX = 16;    // transformed dimensions
constexpr int FO_MAX = 320;   // MLP outputs nb (2K+1)
constexpr int FT = 32;        // points per tile of the gradient kernel
constexpr int FNT = 256;      // threads of the gradient kernel

struct MlpW {
  const float *W1, *b1, *W2, *b2, *W3, *b3;
};
struct MlpG {
  float *W1, *b1, *W2, *b2, *W3, *b3;
};

__host__ __device__ inline int odd_up(int n) { return n | 1; }

// floats of the weights in shared memory
__host__ __device__ inline int weights_floats(int na, int no) {
  return FH * odd_up(na) + FH + FH * FH_P + FH + no * FH_P + no;
}
// floats of one block's partial gradient sums
__host__ __device__ inline int grad_floats(int na, int no) { return FH * na + FH + FH * FH + FH + no * FH + no; }

struct SmemW {
  float *W1, *b1, *W2, *b2, *W3, *b3;
  int w1s;  // row stride of W1
};

__device__ SmemW load_weights(float* sh, const MlpW& w, int na, int no, int tid, int nt) {
  SmemW s;
  s.w1s = odd_up(na);
  s.W1 = sh;
  s.b1 = s.W1 + FH * s.w1s;
  s.W2 = s.b1 + FH;
  s.b2 = s.W2 + FH * FH_P;
  s.W3 = s.b2 + FH;
  s.b3 = s.W3 + no * FH_P;
  for (int i = tid; i < FH * na; i += nt) s.W1[(i / na) * s.w1s + i % na] = w.W1[i];
  for (int i = tid; i < FH * FH; i += nt) s.W2[(i / FH) * FH_P + i % FH] = w.W2[i];
  for (int i = tid; i < no * FH; i += nt) s.W3[(i / FH) * FH_P + i % FH] = w.W3[i];
  for (int i = tid; i < FH; i += nt) {
    s.b1[i] = w.b1[i];
    s.b2[i] = w.b2[i];
  }
  for (int i = tid; i < no; i += nt) s.b3[i] = w.b3[i];
  return s;
}

// The layer's dimension indices in shared memory, clamped to [0, dim) so
// that no caller index reads outside a point's row.
__device__ void load_dims(int* sia, int* sib, const int* __restrict__ ia, int na, const int* __restrict__ ib, int nb,
                          int dim, int tid, int nt) {
  for (int i = tid; i < na; i += nt) sia[i] = min(max(ia[i], 0), dim - 1);
  for (int i = tid; i < nb; i += nt) sib[i] = min(max(ib[i], 0), dim - 1);
}

// One coupling layer, one thread per point.  z_in, z_out [N][dim] (may be
// the same array); logq [N] accumulates the log-determinant.
template <int K, bool INV>
__global__ void __launch_bounds__(128) flow_layer_kernel(const float* z_in, float* z_out, int64_t N,
                                                         int dim, const int* __restrict__ ia, int na,
                                                         const int* __restrict__ ib, int nb, MlpW w,
                                                         float* __restrict__ logq) {
  constexpr int NP = 2 * K + 1;
  extern __shared__ __align__(16) float flow_sh[];
  const int no = nb * NP;
  __shared__ int sia[FA_MAX], sib[FB_MAX];
  const SmemW s = load_weights(flow_sh, w, na, no, threadIdx.x, blockDim.x);
  load_dims(sia, sib, ia, na, ib, nb, dim, threadIdx.x, blockDim.x);
  __syncthreads();
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    const float* zi = z_in + e * dim;
    float a[FA_MAX];
#pragma unroll
    for (int i = 0; i < FA_MAX; ++i) a[i] = i < na ? 2.f * zi[sia[i]] - 1.f : 0.f;
    float h1[FH], h2[FH];
#pragma unroll
    for (int j = 0; j < FH; ++j) {
      float t = s.b1[j];
#pragma unroll
      for (int i = 0; i < FA_MAX; ++i)
        if (i < na) t = fmaf(s.W1[j * s.w1s + i], a[i], t);
      h1[j] = fmaxf(t, 0.f);
    }
#pragma unroll
    for (int j = 0; j < FH; ++j) {
      float t = s.b2[j];
#pragma unroll
      for (int k = 0; k < FH; ++k) t = fmaf(s.W2[j * FH_P + k], h1[k], t);
      h2[j] = fmaxf(t, 0.f);
    }
    float xb[FB_MAX];
#pragma unroll
    for (int d = 0; d < FB_MAX; ++d) xb[d] = d < nb ? zi[sib[d]] : 0.f;
    float* zo = z_out + e * dim;
    if (zo != zi)
      for (int d = 0; d < dim; ++d) zo[d] = zi[d];
    float ld = 0.f;
    for (int d = 0; d < nb; ++d) {
      float p[NP];
#pragma unroll
      for (int o = 0; o < NP; ++o) {
        const int r = d * NP + o;
        float t = s.b3[r];
#pragma unroll
        for (int j = 0; j < FH; ++j) t = fmaf(s.W3[r * FH_P + j], h2[j], t);
        p[o] = t;
      }
      mfpq::Bins b;
      mfpq::make_bins(p, K, b);
      float pdf;
      zo[sib[d]] = INV ? mfpq::pq_inv1(b, K, xb[d], &pdf) : mfpq::pq_fwd1(b, K, xb[d], &pdf);
      ld += __logf(pdf);
    }
    logq[e] += ld;
  }
}

// C(m, n) = sum_k A(m, k) B(k, n) over shared-memory operands with strides
// (A(m, k) at A[m sam + k sak], B(k, n) at B[k sbk + n sbn]), each thread
// one TM x TN block held in registers: rows m0 .. m0 + TM - 1, columns n,
// n + NB, .. (NB = ceil(N / TN) column groups, so the threads of a warp read
// neighbouring columns of B and the same rows of A).  Out-of-range rows and
// columns read a valid element and their results are dropped; epi(m, n, c)
// receives every result in range.
template <int TM, int TN, class Epi>
__device__ __forceinline__ void tile_gemm(int M, int N, int K, const float* __restrict__ A, int sam, int sak,
                                          const float* __restrict__ B, int sbk, int sbn, int tid, int nt, Epi epi) {
  const int nbk = (N + TN - 1) / TN, nblk = (M + TM - 1) / TM * nbk;
  for (int blk = tid; blk < nblk; blk += nt) {
    const int m0 = (blk / nbk) * TM, n0 = blk % nbk;
    int am[TM], bn[TN];
#pragma unroll
    for (int i = 0; i < TM; ++i) am[i] = min(m0 + i, M - 1) * sam;
#pragma unroll
    for (int j = 0; j < TN; ++j) bn[j] = min(n0 + j * nbk, N - 1) * sbn;
    float acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) acc[i][j] = 0.f;
#pragma unroll 4
    for (int k = 0; k < K; ++k) {
      float a[TM], b[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = A[am[i] + k * sak];
#pragma unroll
      for (int j = 0; j < TN; ++j) b[j] = B[k * sbk + bn[j]];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) {
        const int m = m0 + i, n = n0 + j * nbk;
        if (m < M && n < N) epi(m, n, acc[i][j]);
      }
  }
}

// Gradient of one coupling layer in the density direction.  z_in [N][dim]
// the layer's input, g_out [N][dim] = dL/d(layer output), gl [N] = dL/d(log
// pdf sum) -> g_in [N][dim] = dL/d(layer input); part [gridDim][grad_floats]
// the block's partial sums of the weight gradients (overwritten).
template <int K>
__global__ void __launch_bounds__(FNT, 1) flow_grad_kernel(const float* __restrict__ z_in,
                                                           const float* __restrict__ g_out, float* __restrict__ g_in,
                                                           int64_t N, int dim, const int* __restrict__ ia, int na,
                                                           const int* __restrict__ ib, int nb, MlpW w,
                                                           const float* __restrict__ gl, float* __restrict__ part) {
  constexpr int NP = 2 * K + 1;
  extern __shared__ __align__(16) float flow_sh[];
  const int tid = threadIdx.x;
  const int no = nb * NP;
  __shared__ int sia[FA_MAX], sib[FB_MAX];
  const SmemW s = load_weights(flow_sh, w, na, no, tid, FNT);
  load_dims(sia, sib, ia, na, ib, nb, dim, tid, FNT);
  float* A = flow_sh + weights_floats(na, no);  // [FT][FA_MAX]
  float* H1 = A + FT * FA_MAX;                  // [FT][FH]
  float* H2 = H1 + FT * FH;
  float* G2 = H2 + FT * FH;
  float* G1 = G2 + FT * FH;
  float* P = G1 + FT * FH;  // [FT][no]: the MLP outputs, then their gradients
  // this block's partial sums
  const int T = grad_floats(na, no);
  float* pW1 = part + (int64_t)blockIdx.x * T;
  float* pb1 = pW1 + FH * na;
  float* pW2 = pb1 + FH;
  float* pb2 = pW2 + FH * FH;
  float* pW3 = pb2 + FH;
  float* pb3 = pW3 + no * FH;
  for (int i = tid; i < T; i += FNT) pW1[i] = 0.f;
  __syncthreads();
  for (int64_t t0 = (int64_t)blockIdx.x * FT; t0 < N; t0 += (int64_t)gridDim.x * FT) {
    const int np = (int)min((int64_t)FT, N - t0);
    // the tile's conditioning inputs, and dL/dz_in = dL/dz_out to start with
    for (int i = tid; i < FT * na; i += FNT) {
      const int p = i / na, c = i % na;
      A[p * FA_MAX + c] = p < np ? 2.f * z_in[(t0 + p) * dim + sia[c]] - 1.f : 0.f;
    }
    for (int i = tid; i < np * dim; i += FNT) g_in[t0 * dim + i] = g_out[t0 * dim + i];
    __syncthreads();
    // H1 = relu(A W1^T + b1), H2 = relu(H1 W2^T + b2), P = H2 W3^T + b3
    tile_gemm<4, 2>(FT, FH, na, A, FA_MAX, 1, s.W1, 1, s.w1s, tid, FNT,
                    [&](int p, int j, float c) { H1[p * FH + j] = fmaxf(c + s.b1[j], 0.f); });
    __syncthreads();
    tile_gemm<4, 2>(FT, FH, FH, H1, FH, 1, s.W2, 1, FH_P, tid, FNT,
                    [&](int p, int j, float c) { H2[p * FH + j] = fmaxf(c + s.b2[j], 0.f); });
    __syncthreads();
    tile_gemm<4, 4>(FT, no, FH, H2, FH, 1, s.W3, 1, FH_P, tid, FNT,
                    [&](int p, int o, float c) { P[p * no + o] = c + s.b3[o]; });
    __syncthreads();
    // the transform's backward per (point, dimension): dL/dx to g_in, the
    // parameters' gradient over the parameters (0 for points past the end)
    for (int i = tid; i < FT * nb; i += FNT) {
      const int p = i / nb, d = i % nb;
      float* pp = P + p * no + d * NP;
      if (p < np) {
        const int64_t o = (t0 + p) * dim + sib[d];
        g_in[o] = mfpq::pq_bwd1(pp, K, z_in[o], g_out[o], gl[t0 + p], pp);
      } else {
        for (int q = 0; q < NP; ++q) pp[q] = 0.f;
      }
    }
    __syncthreads();
    // G2 = (GP W3) * [H2 > 0]; dW3 += GP^T H2, db3 += sum GP
    tile_gemm<4, 2>(FT, FH, no, P, no, 1, s.W3, FH_P, 1, tid, FNT,
                    [&](int p, int j, float c) { G2[p * FH + j] = H2[p * FH + j] > 0.f ? c : 0.f; });
    tile_gemm<4, 4>(no, FH, FT, P, 1, no, H2, FH, 1, tid, FNT,
                    [&](int o, int j, float c) { pW3[o * FH + j] += c; });
    for (int o = tid; o < no; o += FNT) {
      float t = 0.f;
      for (int p = 0; p < FT; ++p) t += P[p * no + o];
      pb3[o] += t;
    }
    __syncthreads();
    // G1 = (G2 W2) * [H1 > 0]; dW2 += G2^T H1, db2 += sum G2
    tile_gemm<4, 2>(FT, FH, FH, G2, FH, 1, s.W2, FH_P, 1, tid, FNT,
                    [&](int p, int k, float c) { G1[p * FH + k] = H1[p * FH + k] > 0.f ? c : 0.f; });
    tile_gemm<4, 4>(FH, FH, FT, G2, 1, FH, H1, FH, 1, tid, FNT,
                    [&](int j, int k, float c) { pW2[j * FH + k] += c; });
    for (int j = tid; j < FH; j += FNT) {
      float t = 0.f;
      for (int p = 0; p < FT; ++p) t += G2[p * FH + j];
      pb2[j] += t;
    }
    __syncthreads();
    // dL/dz_in += 2 G1 W1 on the conditioning dimensions; dW1 += G1^T A, db1 += sum G1
    for (int i = tid; i < np * na; i += FNT) {
      const int p = i / na, c = i % na;
      float t = 0.f;
      for (int j = 0; j < FH; ++j) t = fmaf(G1[p * FH + j], s.W1[j * s.w1s + c], t);
      const int64_t o = (t0 + p) * dim + sia[c];
      g_in[o] = g_out[o] + 2.f * t;
    }
    for (int i = tid; i < FH * na; i += FNT) {
      const int j = i / na, c = i % na;
      float t = 0.f;
      for (int p = 0; p < FT; ++p) t = fmaf(G1[p * FH + j], A[p * FA_MAX + c], t);
      pW1[i] += t;
    }
    for (int j = tid; j < FH; j += FNT) {
      float t = 0.f;
      for (int p = 0; p < FT; ++p) t += G1[p * FH + j];
      pb1[j] += t;
    }
    __syncthreads();
  }
}

// grads = sum over the nblocks partial rows, in block order
__global__ void flow_grad_reduce_kernel(const float* __restrict__ part, int nblocks, int na, int no, MlpG g) {
  const int T = grad_floats(na, no);
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= T) return;
  float t = 0.f;
  for (int b = 0; b < nblocks; ++b) t += part[(int64_t)b * T + i];
  int r = i;
  if (r < FH * na) { g.W1[r] = t; return; }
  r -= FH * na;
  if (r < FH) { g.b1[r] = t; return; }
  r -= FH;
  if (r < FH * FH) { g.W2[r] = t; return; }
  r -= FH * FH;
  if (r < FH) { g.b2[r] = t; return; }
  r -= FH;
  if (r < no * FH) { g.W3[r] = t; return; }
  g.b3[r - no * FH] = t;
}

inline size_t grad_smem_bytes(int na, int no) {
  return sizeof(float) * (size_t)(weights_floats(na, no) + FT * FA_MAX + 4 * FT * FH + FT * no);
}
inline size_t layer_smem_bytes(int na, int no) { return sizeof(float) * (size_t)weights_floats(na, no); }

int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

// raise the dynamic shared-memory limit of every instantiation once per device
std::mutex g_attr_mu;
bool g_attr_done[64] = {false};
template <int K> int set_attrs() {
  int st = cudaFuncSetAttribute(flow_grad_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)grad_smem_bytes(FA_MAX, FO_MAX));
  if (!st) st = cudaFuncSetAttribute(flow_layer_kernel<K, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)layer_smem_bytes(FA_MAX, FO_MAX));
  if (!st) st = cudaFuncSetAttribute(flow_layer_kernel<K, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)layer_smem_bytes(FA_MAX, FO_MAX));
  return st;
}
int ensure_attrs() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return MF_ERR_CUDA;
  if (dev < 0 || dev >= 64) return MF_ERR_CAPACITY;
  std::lock_guard<std::mutex> lk(g_attr_mu);
  if (g_attr_done[dev]) return MF_OK;
  int st = set_attrs<4>();
  if (!st) st = set_attrs<8>();
  if (!st) st = set_attrs<16>();
  if (st) return MF_ERR_CUDA;
  g_attr_done[dev] = true;
  return MF_OK;
}

int check_shape(int64_t n, int dim, const int* ia, int na, const int* ib, int nb, int K) {
  if (n < 0 || dim <= 0 || !ia || !ib || na < 1 || na > FA_MAX || nb < 1 || nb > FB_MAX || na + nb > dim)
    return MF_ERR_ARG;
  if (K != 4 && K != 8 && K != 16) return MF_ERR_UNSUPPORTED;
  if (nb * (2 * K + 1) > FO_MAX) return MF_ERR_CAPACITY;
  return MF_OK;
}

template <int K>
int launch_layer(bool inv, const float* z_in, float* z_out, int64_t n, int dim, const int* ia, int na, const int* ib,
                 int nb, const MlpW& w, float* logq, cudaStream_t st) {
  const int no = nb * (2 * K + 1);
  int64_t blocks = (n + 127) / 128, cap = (int64_t)sm_count() * 4;
  if (blocks > cap) blocks = cap;
  if (inv)
    flow_layer_kernel<K, true><<<(int)blocks, 128, layer_smem_bytes(na, no), st>>>(z_in, z_out, n, dim, ia, na, ib,
                                                                                   nb, w, logq);
  else
    flow_layer_kernel<K, false><<<(int)blocks, 128, layer_smem_bytes(na, no), st>>>(z_in, z_out, n, dim, ia, na, ib,
                                                                                    nb, w, logq);
  return cudaPeekAtLastError() == cudaSuccess ? MF_OK : MF_ERR_CUDA;
}

int layer_common(bool inv, const float* z_in, float* z_out, int64_t n, int dim, const int* ia, int na, const int* ib,
                 int nb, int K, const float* W1, const float* b1, const float* W2, const float* b2, const float* W3,
                 const float* b3, float* logq, void* stream) {
  int st = check_shape(n, dim, ia, na, ib, nb, K);
  if (st) return st;
  if (n > 0 && (!z_in || !z_out || !W1 || !b1 || !W2 || !b2 || !W3 || !b3 || !logq)) return MF_ERR_ARG;
  if (n == 0) return MF_OK;
  st = ensure_attrs();
  if (st) return st;
  const MlpW w = {W1, b1, W2, b2, W3, b3};
  cudaStream_t s = (cudaStream_t)stream;
  if (K == 4) return launch_layer<4>(inv, z_in, z_out, n, dim, ia, na, ib, nb, w, logq, s);
  if (K == 8) return launch_layer<8>(inv, z_in, z_out, n, dim, ia, na, ib, nb, w, logq, s);
  return launch_layer<16>(inv, z_in, z_out, n, dim, ia, na, ib, nb, w, logq, s);
}
}  // namespace

extern "C" {

int mf_flow_layer_density(const float* z_in, float* z_out, int64_t n, int dim, const int* ia, int na, const int* ib,
                          int nb, int K, const float* W1, const float* b1, const float* W2, const float* b2,
                          const float* W3, const float* b3, float* logq, void* stream) {
  return layer_common(false, z_in, z_out, n, dim, ia, na, ib, nb, K, W1, b1, W2, b2, W3, b3, logq, stream);
}

int mf_flow_layer_sample(const float* z_in, float* z_out, int64_t n, int dim, const int* ia, int na, const int* ib,
                         int nb, int K, const float* W1, const float* b1, const float* W2, const float* b2,
                         const float* W3, const float* b3, float* logq, void* stream) {
  return layer_common(true, z_in, z_out, n, dim, ia, na, ib, nb, K, W1, b1, W2, b2, W3, b3, logq, stream);
}

int mf_flow_layer_grad_workspace(int na, int nb, int K, int64_t* bytes) {
  if (!bytes || na < 1 || na > FA_MAX || nb < 1 || nb > FB_MAX || K < 2) return MF_ERR_ARG;
  const int no = nb * (2 * K + 1);
  if (no > FO_MAX) return MF_ERR_CAPACITY;
  *bytes = (int64_t)sizeof(float) * grad_floats(na, no) * sm_count();
  return MF_OK;
}

int mf_flow_layer_grad(const float* z_in, const float* g_out, float* g_in, int64_t n, int dim, const int* ia, int na,
                       const int* ib, int nb, int K, const float* W1, const float* b1, const float* W2,
                       const float* b2, const float* W3, const float* b3, const float* glogdet, float* gW1, float* gb1,
                       float* gW2, float* gb2, float* gW3, float* gb3, float* workspace, int64_t workspace_bytes,
                       void* stream) {
  int st = check_shape(n, dim, ia, na, ib, nb, K);
  if (st) return st;
  if (!W1 || !b1 || !W2 || !b2 || !W3 || !b3 || !gW1 || !gb1 || !gW2 || !gb2 || !gW3 || !gb3 || !workspace)
    return MF_ERR_ARG;
  if (n > 0 && (!z_in || !g_out || !g_in || !glogdet)) return MF_ERR_ARG;
  if (z_in == g_in || g_out == g_in) return MF_ERR_ARG;
  const int no = nb * (2 * K + 1);
  int64_t need = 0;
  st = mf_flow_layer_grad_workspace(na, nb, K, &need);
  if (st) return st;
  if (workspace_bytes < need) return MF_ERR_CAPACITY;
  st = ensure_attrs();
  if (st) return st;
  const MlpW w = {W1, b1, W2, b2, W3, b3};
  const MlpG g = {gW1, gb1, gW2, gb2, gW3, gb3};
  cudaStream_t s = (cudaStream_t)stream;
  // blocks: at most one per SM (the workspace holds that many partial rows)
  // and one per tile; n = 0 still runs one block so the gradients come out 0
  int64_t tiles = (n + FT - 1) / FT;
  int blocks = (int)(tiles < 1 ? 1 : (tiles < sm_count() ? tiles : sm_count()));
  const size_t smem = grad_smem_bytes(na, no);
  if (K == 4)
    flow_grad_kernel<4><<<blocks, FNT, smem, s>>>(z_in, g_out, g_in, n, dim, ia, na, ib, nb, w, glogdet, workspace);
  else if (K == 8)
    flow_grad_kernel<8><<<blocks, FNT, smem, s>>>(z_in, g_out, g_in, n, dim, ia, na, ib, nb, w, glogdet, workspace);
  else
    flow_grad_kernel<16><<<blocks, FNT, smem, s>>>(z_in, g_out, g_in, n, dim, ia, na, ib, nb, w, glogdet, workspace);
  const int T = grad_floats(na, no);
  flow_grad_reduce_kernel<<<(T + 255) / 256, 256, 0, s>>>(workspace, blocks, na, no, g);
  return cudaPeekAtLastError() == cudaSuccess ? MF_OK : MF_ERR_CUDA;
}

}  // extern "C"
