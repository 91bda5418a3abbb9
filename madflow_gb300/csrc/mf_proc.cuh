// Instantiation of the kernels of one process; included by mf_proc_k<K>.cu
// after the generated header of that process.
#pragma once
#include "mf_launch.h"
#include "mf_me.cuh"

template <int K, class T> static int rec_smem_bytes() { return (int)sizeof(RecSmem<T, K>); }
// whether the block-per-event workspace of a process fits in shared memory
template <int K, class T> constexpr bool rec_in_smem() { return sizeof(RecSmem<T, K>) <= 200 * 1024; }
// blocks of the global-workspace kernel per SM (its workspaces are allocated per block)
constexpr int MF_GWS_PER_SM = 1;
// resident blocks per SM of the record-writing kernels (ps_iter_kernel,
// prep_kernel): each thread builds its 1.5 KB record in local memory, and
// with more blocks the local working set spills out of L1 and L2 (measured:
// 2 blocks of 128 threads per SM 10.6 ms, 3 or more 11.8 ms, 1 15.1 ms per
// 10^7 gg > tt~gg events)
#ifndef MF_PS_BLOCKS_PER_SM
#define MF_PS_BLOCKS_PER_SM 2
#endif
#ifndef MF_PREP_BLOCKS_PER_SM
#define MF_PREP_BLOCKS_PER_SM 2
#endif

static int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

#define MF_DEFINE_PROCESS(KK)                                                                                  \
  MF_DEFINE_REC(KK)                                                                                            \
  void mf_host_tables_k##KK(int* nperm, int* ncomb, double* den, double* cden, const float** cn,              \
                            const signed char** hh) {                                                          \
    *nperm = ttng##KK::NPERM;                                                                                  \
    *ncomb = ttng##KK::NCOMB;                                                                                  \
    *den = ttng##KK::DENOMINATOR;                                                                              \
    *cden = ttng##KK::COLOUR_DEN;                                                                              \
    *cn = ttng##KK::colour_num_h;                                                                              \
    *hh = &ttng##KK::hel_h[0][0];                                                                              \
  }                                                                                                            \
  template <class T, int COLOUR>                                                                               \
  static int me_rec_launch_k##KK(const int4* prep, int64_t N, const double* skip, double* out, double* hel_out, \
                                 int* err, int waves, uint32_t tries, cudaStream_t st) {                                       \
    if constexpr (one_warp_per_event<KK>()) {                                                                  \
      /* one warp per event (few helicities and colour flows) */                                              \
      constexpr int WPB = MF_REC_NT / 32;                                                                      \
      const void* fm = (const void*)me_rec_warp_kernel<KK, T>;                                                 \
      int mb = (int)sizeof(RecSmem<T, KK>) * WPB;                                                              \
      cudaFuncSetAttribute(fm, cudaFuncAttributeMaxDynamicSharedMemorySize, mb);                               \
      int pm = 0;                                                                                              \
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pm, fm, MF_REC_NT, mb);                                   \
      if (pm < 1) pm = 1;                                                                                      \
      int64_t gm = (int64_t)sm_count() * pm * (waves > 0 ? waves : 1);                                         \
      int64_t need = (N + WPB - 1) / WPB;                                                                      \
      if (gm > need) gm = need;                                                                                \
      if (gm < 1) gm = 1;                                                                                      \
      me_rec_warp_kernel<KK, T><<<(int)gm, MF_REC_NT, mb, st>>>(prep, N, skip, out, hel_out);                 \
      return cudaPeekAtLastError() == cudaSuccess ? 0 : 2;                                                     \
    } else {                                                                                                   \
      const void* fn = (const void*)me_rec_kernel<KK, T, COLOUR>;                                              \
      const void* fn0 = (const void*)me_rec_kernel<KK, T, 0>;                                                  \
      int bytes = rec_smem_bytes<KK, T>();                                                                     \
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);                            \
      cudaFuncSetAttribute(fn0, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);                           \
      /* resident blocks per SM from the SIMT variant: the same registers and  */                              \
      /* shared memory (the occupancy query reports 1 for kernels that         */                              \
      /* allocate tensor memory, although 4 blocks x 32 columns fit)           */                              \
      int per = 0;                                                                                             \
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn0, MF_REC_NT, bytes);                              \
      if (per < 1) per = 1;                                                                                    \
      int64_t g = (int64_t)sm_count() * per * (waves > 0 ? waves : 1);                                         \
      if (g > N) g = N;                                                                                        \
      if (g < 1) g = 1;                                                                                        \
      me_rec_kernel<KK, T, COLOUR><<<(int)g, MF_REC_NT, bytes, st>>>(prep, N, skip, out, hel_out, err, tries); \
      return cudaPeekAtLastError() == cudaSuccess ? 0 : 2;                                                     \
    }                                                                                                          \
  }                                                                                                            \
  int64_t mf_prep_bytes_k##KK(int prec) {                                                                      \
    return prec == 0 ? (int64_t)sizeof(PrepRec<double, KK>) : (int64_t)sizeof(PrepRec<float, KK>);           \
  }                                                                                                            \
  bool mf_colour_tc_k##KK() { return TcTraits<KK>::enabled; }                                                  \
  template <class T, int COLOUR>                                                                               \
  static int me_gws_launch_k##KK(const int4* prep, int64_t N, const double* skip, double* out, double* hel_out,  \
                                 int* err, void* ws, uint32_t tries, cudaStream_t st) {                        \
    if (!ws) return 3;                                                                                         \
    const void* fn = (const void*)me_gws_kernel<KK, T, COLOUR>;                                                \
    int bytes = gws_smem_bytes<T, KK>(COLOUR);                                                                 \
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);                              \
    int64_t g = (int64_t)sm_count() * MF_GWS_PER_SM;                                                           \
    me_gws_kernel<KK, T, COLOUR><<<(int)g, MF_GWS_NT, bytes, st>>>(prep, N, skip, out, hel_out,                \
                                                                   reinterpret_cast<RecWS<T, KK>*>(ws), err,   \
                                                                   tries);                                     \
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 2;                                                       \
  }                                                                                                            \
  int64_t mf_ws_bytes_k##KK(int prec) {                                                                        \
    if (prec == 0) return rec_in_smem<KK, double>() ? 0 : (int64_t)sizeof(RecWS<double, KK>) * sm_count() * MF_GWS_PER_SM; \
    return rec_in_smem<KK, float>() ? 0 : (int64_t)sizeof(RecWS<float, KK>) * sm_count() * MF_GWS_PER_SM;      \
  }                                                                                                            \
  int mf_launch_me_k##KK(int prec, const int4* prep, int64_t N, const double* skip, double* out,               \
                         double* hel_out, int* err, MeTune t, void* ws, cudaStream_t st) {                     \
    if (prec == 0) {                                                                                           \
      if constexpr (rec_in_smem<KK, double>())                                                                 \
        return me_rec_launch_k##KK<double, 0>(prep, N, skip, out, hel_out, err, t.waves, (uint32_t)t.wait_tries, st);                 \
      else                                                                                                     \
        return me_gws_launch_k##KK<double, 0>(prep, N, skip, out, hel_out, err, ws, (uint32_t)t.wait_tries, st);                       \
    }                                                                                                          \
    if constexpr (!rec_in_smem<KK, float>()) {                                                                 \
      if constexpr (TcTraits<KK>::enabled)                                                                     \
        if (t.colour == 1) return me_gws_launch_k##KK<float, 1>(prep, N, skip, out, hel_out, err, ws, (uint32_t)t.wait_tries, st);     \
      return me_gws_launch_k##KK<float, 0>(prep, N, skip, out, hel_out, err, ws, (uint32_t)t.wait_tries, st);                          \
    } else {                                                                                                   \
      if constexpr (TcTraits<KK>::enabled)                                                                     \
        if (t.colour == 1) return me_rec_launch_k##KK<float, 1>(prep, N, skip, out, hel_out, err, t.waves, (uint32_t)t.wait_tries, st); \
      return me_rec_launch_k##KK<float, 0>(prep, N, skip, out, hel_out, err, t.waves, (uint32_t)t.wait_tries, st);                    \
    }                                                                                                          \
  }                                                                                                            \
  int mf_launch_prep_k##KK(int prec, const double* ps, int64_t N, double mt, double wt, const double* coup,    \
                           int64_t cstride, int4* prep, cudaStream_t st) {                                     \
    int64_t b = (N + 127) / 128, cap = (int64_t)sm_count() * MF_PREP_BLOCKS_PER_SM;                            \
    if (b > cap) b = cap;                                                                                      \
    if (b < 1) b = 1;                                                                                          \
    if (prec == 0) prep_kernel<KK, double><<<(int)b, 128, 0, st>>>(ps, N, mt, wt, coup, cstride, prep);       \
    else prep_kernel<KK, float><<<(int)b, 128, 0, st>>>(ps, N, mt, wt, coup, cstride, prep);                  \
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 2;                                                       \
  }                                                                                                            \
  int mf_launch_ps_k##KK(int prec, const IterArgs& A, cudaStream_t st) {                                       \
    int64_t b = (A.N + 127) / 128;                                                                             \
    int64_t cap = (int64_t)sm_count() * MF_PS_BLOCKS_PER_SM;                                                   \
    if (b > cap) b = cap;                                                                                      \
    if (b < 1) b = 1;                                                                                          \
    /* the dynamical scale is a separate instantiation: the fixed-scale kernel */ \
    /* keeps its registers */                                                      \
    if (prec == 0 && A.dyn) ps_iter_kernel<KK, double, true><<<(int)b, 128, 0, st>>>(A);                      \
    else if (prec == 0) ps_iter_kernel<KK, double, false><<<(int)b, 128, 0, st>>>(A);                         \
    else if (A.dyn) ps_iter_kernel<KK, float, true><<<(int)b, 128, 0, st>>>(A);                               \
    else ps_iter_kernel<KK, float, false><<<(int)b, 128, 0, st>>>(A);                                         \
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 2;                                                       \
  }                                                                                                            \
  int64_t mf_state_words_k##KK() { return ps_state_words<KK>(); }                                               \
  int mf_launch_seed_k##KK(int prec, const IterArgs& A, int* kmin, int batch_rule, cudaStream_t st) {          \
    int64_t blocks = (A.N + 255) / 256;                                                                        \
    int64_t cap = (int64_t)sm_count() * 8;                                                                     \
    if (blocks > cap) blocks = cap;                                                                            \
    if (blocks < 1) blocks = 1;                                                                                \
    size_t grid_words = A.x_in ? 0 : (size_t)A.ndim * (A.nb + 1);                                              \
    if (prec == 0)                                                                                             \
      ps_seed_kernel<KK, double><<<(int)blocks, 256, grid_words * sizeof(double), st>>>(A, kmin, batch_rule);   \
    else                                                                                                       \
      ps_seed_kernel<KK, float><<<(int)blocks, 256, grid_words * sizeof(float), st>>>(A, kmin, batch_rule);     \
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 2;                                                       \
  }
