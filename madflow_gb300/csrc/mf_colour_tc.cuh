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

#if defined(__CUDA_ARCH__) && (defined(__CUDA_ARCH_FEAT_SM103_ALL) || defined(__CUDA_ARCH_FEAT_SM100_ALL))
#define MF_TCGEN05 1
#else
#define MF_TCGEN05 0
#endif

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

// Shared-memory matrix descriptor of tcgen05 (no swizzle): start address,
// leading and stride byte offsets (all >> 4), descriptor version 1 at bit 46.
MF_HD uint64_t tc_smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::tf32: D FP32 (bits 4-5 = 1), A and B TF32
// (bits 7-9 and 10-12 = 2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
MF_HD constexpr uint32_t tc_idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// TF32 split: hi = x with the 13 low mantissa bits cleared
MF_HD float tc_hi(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  u &= 0xFFFFE000u;
  float h;
  memcpy(&h, &u, 4);
  return h;
}

// Bytes of shared memory the operands of one event take: B, A_hi, A_lo.
template <int K> MF_HD constexpr int tc_operand_bytes() {
  return TcTraits<K>::enabled
             ? (TcTraits<K>::N + 2 * 2 * (1 << (K + 2))) * RecTraits<K>::NPERM * (int)sizeof(float)
             : 0;
}

#if MF_TCGEN05
MF_DO uint32_t tc_smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
// one full warp
MF_DO void tc_tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tc_smem_u32(dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
// one full warp
MF_DO void tc_tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
MF_DO void tc_mbar_init(unsigned long long* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(tc_smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Waits for the phase of the given parity to complete, suspending the thread
// for up to about `ns` nanoseconds (woken early when the phase completes).
MF_DO bool tc_mbar_try_wait(unsigned long long* bar, uint32_t parity, uint32_t ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(tc_smem_u32(bar)), "r"(parity), "r"(ns)
      : "memory");
  return ok != 0;
}
MF_DO void tc_fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
MF_DO void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
MF_DO void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
MF_DO void tc_mma_tf32(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
MF_DO void tc_commit(unsigned long long* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   tc_smem_u32(bar))
               : "memory");
}
// 32 lanes x 16 consecutive 32-bit columns (thread i of the warp: lane i)
MF_DO void tc_ld_x16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
MF_DO void tc_ld_x8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
MF_DO void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
#endif

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
