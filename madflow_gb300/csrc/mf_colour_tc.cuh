// Colour contraction of one event on the 5th-generation tensor cores
// (tcgen05.mma, kind::tf32, FP32 accumulator in tensor memory).
//
// The amplitudes of an event form a real matrix A [2 NC][NPERM]: row c holds
// Re A(sigma, c), row NC + c holds Im A(sigma, c) for the NC helicity
// combinations.  With C the (symmetric, integer) colour numerators,
//   sum_c A_c^dagger C A_c = sum_m sum_tau D[m][tau] A[m][tau],  D = A C,
// so one M = 2 NC = 128, N = NPERM (padded to 32), K = NPERM MMA per event
// gives every colour sum.  A enters split in two TF32 terms: A_hi is A with
// the 13 low mantissa bits cleared (exact in TF32), A_lo = A - A_hi (exact in
// FP32, rounded to TF32 by the MMA, so its error is 2^-11 of A_lo); C is
// exact in TF32.  D = A_hi C + A_lo C thus carries about the error of an
// FP32 product.
//
// Operands sit in shared memory in the no-swizzle K-major canonical layout:
// core matrices of 8 rows x 16 bytes stored contiguously, neighbours along K
// LBO = 128 bytes apart, neighbouring 8-row groups SBO = NPERM/4 x 128 bytes
// apart.  The B operand (C^T, zero rows up to TC_N) is emitted in that layout
// by the process generator (colour_tc_b).  One elected thread issues the
// MMAs and commits them to an mbarrier; warps 0-3 wait on it (bounded), read
// their 32 accumulator lanes with tcgen05.ld and finish the sums.
#pragma once
#include <cstdint>

#include "mf_tcgen05.cuh"

// Per-process constants of the tensor-core colour operand (enabled by
// MF_DEFINE_TC for processes whose generated header carries colour_tc_b).
template <int K> struct TcTraits {
  static constexpr bool enabled = false;
};
#define MF_DEFINE_TC(KK)                                                      \
  template <> struct TcTraits<KK> {                                           \
    static constexpr bool enabled = true;                                     \
    static constexpr int N = ttng##KK::TC_N, LBO = ttng##KK::TC_LBO;          \
    static constexpr int SBO = ttng##KK::TC_SBO;                              \
    MF_DO static const float* b() { return ttng##KK::colour_tc_b; }           \
  };

// Bytes of shared memory the operands of one event take: B, A_hi, A_lo.
template <int K> MF_HD constexpr int tc_operand_bytes() {
  return TcTraits<K>::enabled
             ? (TcTraits<K>::N + 2 * 2 * (1 << (K + 2))) * RecTraits<K>::NPERM * (int)sizeof(float)
             : 0;
}


// Operands of one event into shared memory (all threads): the B operand
// copied from the generated table, A_hi and A_lo from the amplitudes.
// region: 128-byte aligned, tc_operand_bytes<K>() long.
template <int K> MF_DO void tc_fill(const RecWS<float, K>& ws, float* region, int tid, int nt) {
  using R = RecTraits<K>;
  using TT = TcTraits<K>;
  constexpr int NP = R::NPERM, NC = 1 << (K + 2);
  constexpr int SBOF = TT::SBO / 4, LBOF = TT::LBO / 4;
  const int4* src = reinterpret_cast<const int4*>(TT::b());
  int4* dB = reinterpret_cast<int4*>(region);
  for (int i = tid; i < TT::N * NP / 4; i += nt) dB[i] = src[i];
  float* hi = region + TT::N * NP;
  float* lo = hi + 2 * NC * NP;
  for (int it = tid; it < NC * (NP / 4); it += nt) {
    const int c = it % NC, k4 = it / NC;
    float rh[4], rl[4], ih[4], il[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      cx<float> a = ws.A[(4 * k4 + j) * NC + c];
      rh[j] = tc_hi(a.re);
      rl[j] = a.re - rh[j];
      ih[j] = tc_hi(a.im);
      il[j] = a.im - ih[j];
    }
    const int ore = (c / 8) * SBOF + k4 * LBOF + (c % 8) * 4;
    const int oim = ((c + NC) / 8) * SBOF + k4 * LBOF + ((c + NC) % 8) * 4;
    *reinterpret_cast<float4*>(hi + ore) = make_float4(rh[0], rh[1], rh[2], rh[3]);
    *reinterpret_cast<float4*>(lo + ore) = make_float4(rl[0], rl[1], rl[2], rl[3]);
    *reinterpret_cast<float4*>(hi + oim) = make_float4(ih[0], ih[1], ih[2], ih[3]);
    *reinterpret_cast<float4*>(lo + oim) = make_float4(il[0], il[1], il[2], il[3]);
  }
}
