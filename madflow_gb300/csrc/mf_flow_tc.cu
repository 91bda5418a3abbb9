// One coupling layer of the normalizing-flow sampler in the sampling
// direction, fused in one kernel on the 5th-generation tensor cores: the
// conditioner MLP (na -> 64 -> 64 -> nb (2K+1), ReLU) as three tcgen05 GEMMs
// (kind::tf32 on TF32 operands, or kind::f16 on BF16 operands) with FP32
// accumulators in tensor memory, and the inverse
// piecewise-quadratic transform (Mueller et al., ACM TOG 38 (2019) 145) of
// the nb transformed dimensions in the epilogue.  The activations of a tile of
// 128 points stay on chip (tensor memory and shared memory); z is read and
// written once.
//
// Block: 128 threads, thread r owns point r of the tile (tensor-memory lane
// r).  Shared memory: the three weight matrices as B operands (K-major, no
// swizzle, 8-row x 16-byte core matrices: 4 TF32 or 8 BF16 elements of K per
// row; LBO 128 bytes along K, SBO (K / elements per row) x 128 bytes between
// 8-row groups; one MMA covers 32 bytes of K), loaded once per block; the A
// operands (the conditioning inputs 2z - 1, padded to K = 16, and the hidden
// activations, K = 64); the biases.  Tensor memory: 256 columns (D1 at 0,
// D2 at 64, D3 at 0 once D1 and D2 have been read).  A layer with more than
// 256 MLP outputs runs the third GEMM in two column chunks of whole
// dimensions (each at most 256 columns, the second after the first one's
// epilogue has read its accumulator), with the rows of W3 stored in the
// two chunks' padded blocks.  Every wait on the MMA
// completion is bounded (1000 tries of <= 1 ms); one that runs out sets *err,
// the block stops and frees its tensor memory.
#include <cstdint>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/madflow_gb300.h"
#include "mf_tcgen05.cuh"

namespace {

constexpr int FH = 64;        // hidden units
constexpr int FTILE = 128;    // points per tile (MMA M)
constexpr int FK1 = 16;       // padded conditioning inputs (GEMM1 K)
constexpr int FTMEM = 256;    // tensor-memory columns per block
constexpr int FMAXN3 = 256;   // one chunk of the third GEMM: at most 256 columns

__host__ __device__ inline int pad16(int n) { return (n + 15) / 16 * 16; }
// The column chunks of the third GEMM for nb dimensions of np = 2K+1
// parameters: da dimensions in the first, nb - da in the second, padded to
// n3ap and n3bp columns (n3bp = 0: one chunk).  false: more than two chunks.
__host__ __device__ inline bool flow_tc_chunks(int nb, int np, int& da, int& n3ap, int& n3bp) {
  da = nb < FMAXN3 / np ? nb : FMAXN3 / np;
  n3ap = pad16(da * np);
  n3bp = pad16((nb - da) * np);
  return n3bp <= FMAXN3;
}

// The operand element type: TF32 (4 bytes, kind::tf32, K = 8 per MMA) or
// BF16 (2 bytes, kind::f16, K = 16 per MMA).  Values are rounded to BF16 to
// nearest even; TF32 operands are stored as FP32 and truncated by the MMA.
template <bool BF> struct FlowOp {
  static constexpr int ESZ = BF ? 2 : 4;    // bytes per element
  static constexpr int EPR = 16 / ESZ;      // elements per 16-byte core-matrix row
  static constexpr int KSTEP = 32 / ESZ;    // K of one MMA (32 bytes of K)
  // byte offset of element (r, k) in a K-major canonical operand with kdim
  // columns
  __host__ __device__ static int off(int r, int k, int kdim) {
    return (r >> 3) * (kdim / EPR) * 128 + (k / EPR) * 128 + (r & 7) * 16 + (k % EPR) * ESZ;
  }
  static constexpr uint32_t sbo(int kdim) { return (uint32_t)(kdim / EPR) * 128u; }
  static constexpr uint32_t idesc(int m, int n) { return BF ? tc_idesc_bf16(m, n) : tc_idesc_tf32(m, n); }
#if MF_TCGEN05
  static __device__ __forceinline__ void put(unsigned char* base, int r, int k, int kdim, float v) {
    if constexpr (BF)
      *reinterpret_cast<unsigned short*>(base + off(r, k, kdim)) = __bfloat16_as_ushort(__float2bfloat16_rn(v));
    else
      *reinterpret_cast<float*>(base + off(r, k, kdim)) = v;
  }
  // the EPR consecutive elements k .. k + EPR - 1 (k a multiple of EPR) of
  // row r: one 16-byte store
  static __device__ __forceinline__ void put_row(unsigned char* base, int r, int k, int kdim, const float* v) {
    uint4 w;
    if constexpr (BF) {
      uint32_t h[4];
#pragma unroll
      for (int j = 0; j < 4; ++j)
        h[j] = (uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v[2 * j])) |
               ((uint32_t)__bfloat16_as_ushort(__float2bfloat16_rn(v[2 * j + 1])) << 16);
      w = make_uint4(h[0], h[1], h[2], h[3]);
    } else {
      w = make_uint4(__float_as_uint(v[0]), __float_as_uint(v[1]), __float_as_uint(v[2]), __float_as_uint(v[3]));
    }
    *reinterpret_cast<uint4*>(base + off(r, k, kdim)) = w;
  }
  static __device__ __forceinline__ void mma(uint32_t d, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
    if constexpr (BF)
      tc_mma_f16(d, a, b, id, acc);
    else
      tc_mma_tf32(d, a, b, id, acc);
  }
#endif
};

struct FlowTcSmem {
  unsigned char* B1;  // [64][16]
  unsigned char* B2;  // [64][64]
  unsigned char* B3;  // [n3ap + n3bp][64]: the chunks' rows of W3, each block padded
  unsigned char* A1;  // [128][16]
  unsigned char* A2;  // [128][64]
  float* bias;  // b1[64] b2[64] b3[n3ap + n3bp] (b3 by output column)
  int* idx;     // ia[16] ib[16]
  unsigned long long* mbar;
  uint32_t* tmem;
  int* bad;
};

__host__ __device__ inline size_t flow_tc_smem_bytes(int n3p, int esz) {
  size_t ops = (size_t)FH * FK1 + FH * FH + (size_t)n3p * FH + FTILE * FK1 + FTILE * FH;
  size_t b = ops * esz + (2 * FH + n3p) * 4 + 32 * 4 + 64;
  b = (b + 1023) / 1024 * 1024 + 1024;  // alignment slack
  // at least 80 KB, so that at most two blocks (2 x 256 tensor-memory
  // columns) share an SM
  return b < 80 * 1024 ? 80 * 1024 : b;
}

#if MF_TCGEN05
MF_DO void tc_ld_x1(uint32_t taddr, float& v) {
  uint32_t r;
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(r) : "r"(taddr) : "memory");
  v = __uint_as_float(r);
}

// bounded wait for the MMA group committed to bar (all threads of the block
// call it with the same parity; the result is block-uniform)
MF_DO bool flow_tc_wait(unsigned long long* bar, uint32_t parity, int* bad) {
  bool done = false;
  for (uint32_t spin = 0; spin < 1000u && !done; ++spin) done = tc_mbar_try_wait(bar, parity, 1000000u);
  if (!done) atomicExch(bad, 1);
  __syncthreads();
  return *(volatile int*)bad == 0;
}

// inverse piecewise-quadratic transform of one dimension from its 2K+1 raw
// parameters (softmax widths, exp heights normalised to unit area)
template <int K> MF_DO float pq_inverse_one(const float* p, float u, float& logpdf) {
  float W[K], V[K + 1];
  float m = p[0];
#pragma unroll
  for (int k = 1; k < K; ++k) m = fmaxf(m, p[k]);
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    W[k] = __expf(p[k] - m);
    s += W[k];
  }
  const float inv = 1.f / s;
#pragma unroll
  for (int k = 0; k < K; ++k) W[k] *= inv;
  float mv = p[K];
#pragma unroll
  for (int k = 1; k <= K; ++k) mv = fmaxf(mv, p[K + k]);
#pragma unroll
  for (int k = 0; k <= K; ++k) V[k] = __expf(p[K + k] - mv);
  float norm = 0.f;
#pragma unroll
  for (int k = 0; k < K; ++k) norm += 0.5f * (V[k] + V[k + 1]) * W[k];
  const float in = 1.f / norm;
#pragma unroll
  for (int k = 0; k <= K; ++k) V[k] *= in;
  // the bin of u: the last edge whose CDF is <= u (CDF at the left edges)
  u = fminf(fmaxf(u, 0.f), 1.f);
  float Eb = 0.f, Cb = 0.f, Wb = W[0], Vb = V[0], Vn = V[1];
  float E = 0.f, C = 0.f;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    if (k > 0 && u >= C) {
      Eb = E;
      Cb = C;
      Wb = W[k];
      Vb = V[k];
      Vn = V[k + 1];
    }
    E += W[k];
    C += 0.5f * (V[k] + V[k + 1]) * W[k];
  }
  const float r = fmaxf(u - Cb, 0.f);
  const float D = Vn - Vb;
  const float a = 0.5f * Wb * D, bq = Wb * Vb;
  float alpha = 2.f * r / (bq + sqrtf(fmaxf(bq * bq + 4.f * a * r, 0.f)));
  alpha = fminf(fmaxf(alpha, 0.f), 1.f);
  logpdf = __logf(Vb + alpha * D);
  return fminf(Eb + alpha * Wb, 1.f);
}
#endif

template <int K, bool BF>
__global__ void __launch_bounds__(FTILE) flow_inv_layer_tc_kernel(float* __restrict__ z, int64_t n, int dim,
                                                                  const int* __restrict__ ia, int na,
                                                                  const int* __restrict__ ib, int nb,
                                                                  const float* __restrict__ W1,
                                                                  const float* __restrict__ b1,
                                                                  const float* __restrict__ W2,
                                                                  const float* __restrict__ b2,
                                                                  const float* __restrict__ W3,
                                                                  const float* __restrict__ b3,
                                                                  float* __restrict__ logq, int* __restrict__ err) {
#if MF_TCGEN05
  using Op = FlowOp<BF>;
  constexpr int ESZ = Op::ESZ;
  constexpr int NP = 2 * K + 1;
  const int n3 = nb * NP;
  int da, n3ap, n3bp;
  flow_tc_chunks(nb, NP, da, n3ap, n3bp);
  const int n3a = da * NP, n3b = n3 - n3a;
  extern __shared__ __align__(1024) unsigned char fsm[];
  uintptr_t base = (reinterpret_cast<uintptr_t>(fsm) + 1023) & ~(uintptr_t)1023;
  FlowTcSmem S;
  S.B1 = reinterpret_cast<unsigned char*>(base);
  S.B2 = S.B1 + FH * FK1 * ESZ;
  S.B3 = S.B2 + FH * FH * ESZ;
  S.A1 = S.B3 + (n3ap + n3bp) * FH * ESZ;
  S.A2 = S.A1 + FTILE * FK1 * ESZ;
  S.bias = reinterpret_cast<float*>(S.A2 + FTILE * FH * ESZ);
  S.idx = reinterpret_cast<int*>(S.bias + 2 * FH + n3ap + n3bp);
  S.mbar = reinterpret_cast<unsigned long long*>(S.idx + 32);
  S.tmem = reinterpret_cast<uint32_t*>(S.mbar + 1);
  S.bad = reinterpret_cast<int*>(S.tmem + 1);
  const int tid = threadIdx.x, warp = tid >> 5;

  // weights into the canonical B layouts (zero padding), biases, indices
  for (int i = tid; i < FH * FK1; i += FTILE) {
    const int r = i / FK1, k = i % FK1;
    Op::put(S.B1, r, k, FK1, k < na ? W1[r * na + k] : 0.f);
  }
  for (int i = tid; i < FH * FH; i += FTILE) Op::put(S.B2, i / FH, i % FH, FH, W2[i]);
  for (int i = tid; i < (n3ap + n3bp) * FH; i += FTILE) {
    const int r = i / FH, k = i % FH;
    // row r of the chunk blocks: output column src of W3 (-1: padding)
    const int src = r < n3ap ? (r < n3a ? r : -1) : (r - n3ap < n3b ? n3a + r - n3ap : -1);
    Op::put(S.B3, r, k, FH, src >= 0 ? W3[src * FH + k] : 0.f);
  }
  for (int i = tid; i < FH; i += FTILE) {
    S.bias[i] = b1[i];
    S.bias[FH + i] = b2[i];
  }
  for (int i = tid; i < n3ap + n3bp; i += FTILE) S.bias[2 * FH + i] = i < n3 ? b3[i] : 0.f;
  if (tid < 16) {
    // caller indices, clamped to the point's dim columns
    S.idx[tid] = tid < na ? min(max(ia[tid], 0), dim - 1) : 0;
    S.idx[16 + tid] = tid < nb ? min(max(ib[tid], 0), dim - 1) : 0;
  }
  if (warp == 0) tc_tmem_alloc(S.tmem, FTMEM);
  if (tid == 0) {
    tc_mbar_init(S.mbar, 1);
    *S.bad = 0;
  }
  tc_fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tm = *S.tmem;
  const uint32_t lane_base = tm + ((uint32_t)(32 * warp) << 16);
  const uint32_t a1 = tc_smem_u32(S.A1), a2 = tc_smem_u32(S.A2);
  const uint32_t w1 = tc_smem_u32(S.B1), w2 = tc_smem_u32(S.B2), w3 = tc_smem_u32(S.B3);
  constexpr uint32_t L = 128, SB1 = Op::sbo(FK1), SB2 = Op::sbo(FH);
  const uint32_t id64 = Op::idesc(FTILE, FH), id3a = Op::idesc(FTILE, n3ap);
  const uint32_t id3b = Op::idesc(FTILE, n3bp > 0 ? n3bp : 16);
  // the second chunk's rows start n3ap rows (n3ap / 8 core-matrix groups) in
  const uint32_t w3b = w3 + (uint32_t)n3ap * FH * ESZ;
  uint32_t phase = 0;
  const int64_t ntiles = (n + FTILE - 1) / FTILE;

  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const int64_t e = t * FTILE + tid;
    const bool valid = e < n;
    float* zr = z + (valid ? e : 0) * dim;
    // A1: the conditioning inputs 2 z - 1 (zero beyond na and n)
#pragma unroll
    for (int k = 0; k < FK1; k += Op::EPR) {
      float v[Op::EPR];
#pragma unroll
      for (int j = 0; j < Op::EPR; ++j) v[j] = (valid && k + j < na) ? 2.f * zr[S.idx[k + j]] - 1.f : 0.f;
      Op::put_row(S.A1, tid, k, FK1, v);
    }
    tc_fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    // GEMM1: D1 [128][64] = A1 [128][16] B1^T
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int s = 0; s < FK1 / Op::KSTEP; ++s)
        Op::mma(tm, tc_smem_desc(a1 + 256 * s, L, SB1), tc_smem_desc(w1 + 256 * s, L, SB1), id64, s > 0);
      tc_commit(S.mbar);
    }
    if (!flow_tc_wait(S.mbar, phase, S.bad)) break;
    phase ^= 1u;
    tc_fence_after();
    // hidden layer 1 -> A2
#pragma unroll
    for (int c = 0; c < FH; c += 16) {
      float d[16];
      tc_ld_x16(lane_base + c, d);
      tc_wait_ld();
#pragma unroll
      for (int j = 0; j < 16; ++j) d[j] = fmaxf(d[j] + S.bias[c + j], 0.f);
#pragma unroll
      for (int j = 0; j < 16; j += Op::EPR) Op::put_row(S.A2, tid, c + j, FH, d + j);
    }
    tc_fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    // GEMM2: D2 [128][64] (columns 64..127) = A2 B2^T
    if (tid == 0) {
      tc_fence_after();
#pragma unroll
      for (int s = 0; s < FH / Op::KSTEP; ++s)
        Op::mma(tm + FH, tc_smem_desc(a2 + 256 * s, L, SB2), tc_smem_desc(w2 + 256 * s, L, SB2), id64, s > 0);
      tc_commit(S.mbar);
    }
    if (!flow_tc_wait(S.mbar, phase, S.bad)) break;
    phase ^= 1u;
    tc_fence_after();
    // hidden layer 2 -> A2 (GEMM2 has read it)
#pragma unroll
    for (int c = 0; c < FH; c += 16) {
      float d[16];
      tc_ld_x16(lane_base + FH + c, d);
      tc_wait_ld();
#pragma unroll
      for (int j = 0; j < 16; ++j) d[j] = fmaxf(d[j] + S.bias[FH + c + j], 0.f);
#pragma unroll
      for (int j = 0; j < 16; j += Op::EPR) Op::put_row(S.A2, tid, c + j, FH, d + j);
    }
    tc_fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    // GEMM3 by column chunks: D3 [128][n3ap] (columns 0..) = A2 B3a^T, its
    // epilogue, then the same for the second chunk (if any) into the same
    // columns; the epilogue is the inverse transform of each dimension
    float ld = 0.f;
    bool stop = false;
    for (int ch = 0; ch < 2; ++ch) {
      const int d0 = ch ? da : 0, d1 = ch ? nb : da;
      if (d0 >= d1) break;
      if (ch) {
        // the first chunk's accumulator has been read by every thread
        tc_fence_before();
        __syncthreads();
      }
      if (tid == 0) {
        tc_fence_after();
        const uint32_t wb = ch ? w3b : w3;
        const uint32_t id3 = ch ? id3b : id3a;
#pragma unroll
        for (int s = 0; s < FH / Op::KSTEP; ++s)
          Op::mma(tm, tc_smem_desc(a2 + 256 * s, L, SB2), tc_smem_desc(wb + 256 * s, L, SB2), id3, s > 0);
        tc_commit(S.mbar);
      }
      if (!flow_tc_wait(S.mbar, phase, S.bad)) {
        stop = true;
        break;
      }
      phase ^= 1u;
      tc_fence_after();
      for (int d = d0; d < d1; ++d) {
        float p[NP];
#pragma unroll
        for (int j = 0; j < NP; ++j) tc_ld_x1(lane_base + (d - d0) * NP + j, p[j]);
        tc_wait_ld();
#pragma unroll
        for (int j = 0; j < NP; ++j) p[j] += S.bias[2 * FH + d * NP + j];
        const int col = S.idx[16 + d];
        float lp;
        const float x = pq_inverse_one<K>(p, valid ? zr[col] : 0.5f, lp);
        if (valid) zr[col] = x;
        ld += lp;
      }
    }
    if (stop) break;
    if (valid) logq[e] += ld;
    tc_fence_before();
    __syncthreads();
  }
  // a timed-out wait: let the MMA in flight finish (bounded) before the
  // tensor memory is freed
  if (*(volatile int*)S.bad) {
    if (tid == 0) atomicExch(err, 1);
    bool done = false;
    for (uint32_t spin = 0; spin < 1000u && !done; ++spin) done = tc_mbar_try_wait(S.mbar, phase, 1000000u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tc_tmem_dealloc(tm, FTMEM);
  }
#else
  if (threadIdx.x == 0 && blockIdx.x == 0 && err) atomicExch(err, 2);
#endif
}

template <int K, bool BF>
int launch_flow_tc(float* z, int64_t n, int dim, const int* ia, int na, const int* ib, int nb, const float* W1,
                   const float* b1, const float* W2, const float* b2, const float* W3, const float* b3, float* logq,
                   int* err, cudaStream_t st) {
  int da, n3ap, n3bp;
  flow_tc_chunks(nb, 2 * K + 1, da, n3ap, n3bp);
  const size_t smem = flow_tc_smem_bytes(n3ap + n3bp, FlowOp<BF>::ESZ);
  auto fn = flow_inv_layer_tc_kernel<K, BF>;
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return MF_ERR_CUDA;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t tiles = (n + FTILE - 1) / FTILE, grid = (int64_t)(sms > 0 ? sms : 152) * 2;
  if (grid > tiles) grid = tiles;
  fn<<<(int)grid, FTILE, smem, st>>>(z, n, dim, ia, na, ib, nb, W1, b1, W2, b2, W3, b3, logq, err);
  return cudaPeekAtLastError() == cudaSuccess ? MF_OK : MF_ERR_CUDA;
}

template <bool BF>
int flow_inv_layer_tc(float* z, int64_t n, int dim, const int* ia, int na, const int* ib, int nb, int K,
                      const float* W1, const float* b1, const float* W2, const float* b2, const float* W3,
                      const float* b3, float* logq, int* err, void* stream) {
  if (n < 0 || dim <= 0 || na < 1 || na > 16 || nb < 1 || nb > 16 || na + nb > dim) return MF_ERR_ARG;
  int da, n3ap, n3bp;
  if (!(K == 4 || K == 8 || K == 16) || !flow_tc_chunks(nb, 2 * K + 1, da, n3ap, n3bp)) return MF_ERR_ARG;
  if (n == 0) return MF_OK;
  if (!z || !ia || !ib || !W1 || !b1 || !W2 || !b2 || !W3 || !b3 || !logq || !err) return MF_ERR_ARG;
  cudaStream_t st = (cudaStream_t)stream;
  switch (K) {
    case 4: return launch_flow_tc<4, BF>(z, n, dim, ia, na, ib, nb, W1, b1, W2, b2, W3, b3, logq, err, st);
    case 8: return launch_flow_tc<8, BF>(z, n, dim, ia, na, ib, nb, W1, b1, W2, b2, W3, b3, logq, err, st);
    default: return launch_flow_tc<16, BF>(z, n, dim, ia, na, ib, nb, W1, b1, W2, b2, W3, b3, logq, err, st);
  }
}

}  // namespace

extern "C" int mf_flow_inv_layer_tc(float* z, int64_t n, int dim, const int* ia, int na, const int* ib, int nb, int K,
                                    const float* W1, const float* b1, const float* W2, const float* b2,
                                    const float* W3, const float* b3, float* logq, int* err, void* stream) {
  return flow_inv_layer_tc<false>(z, n, dim, ia, na, ib, nb, K, W1, b1, W2, b2, W3, b3, logq, err, stream);
}

extern "C" int mf_flow_inv_layer_tc_bf16(float* z, int64_t n, int dim, const int* ia, int na, const int* ib, int nb,
                                         int K, const float* W1, const float* b1, const float* W2, const float* b2,
                                         const float* W3, const float* b3, float* logq, int* err, void* stream) {
  return flow_inv_layer_tc<true>(z, n, dim, ia, na, ib, nb, K, W1, b1, W2, b2, W3, b3, logq, err, stream);
}
