// Instantiation of the matrix-element kernels for one process; included by
// mf_proc_k<K>.cu after the generated header of that process.
#pragma once
#include "mf_me.cuh"
#include "mf_launch.h"

#define MF_DEFINE_PROCESS(KK)                                                                                    \
  template <> struct ProcTraits<KK> {                                                                            \
    static constexpr int NPERM = ttng##KK::NPERM;                                                                \
    static constexpr int NCOMB = ttng##KK::NCOMB;                                                                \
    static constexpr double DENOMINATOR = ttng##KK::DENOMINATOR;                                                 \
    static constexpr double COLOUR_DEN = ttng##KK::COLOUR_DEN;                                                   \
    MF_DO static const signed char* helicity(int h) { return ttng##KK::hel[h]; }                                  \
    MF_DO static float colour(int i) { return ttng##KK::colour_num[i]; }                                         \
    template <class T>                                                                                           \
    MF_D static void amps(const EvData<T, KK>& ev, const W4<T>* g, const W4<T>& wt, const W4<T>& wtb, cx<T>* A) { \
      ttng##KK##_amps<T>(ev, g, wt, wtb, A);                                                                     \
    }                                                                                                            \
  };                                                                                                             \
  template <class T> static int grid_for(const void* fn, size_t dyn, int64_t work_units) {                       \
    int dev = 0, sms = 0, per = 0;                                                                               \
    cudaGetDevice(&dev);                                                                                         \
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);                                           \
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, 32 * MF_WARPS, dyn);                                 \
    if (per < 1) per = 1;                                                                                        \
    int64_t g = (int64_t)sms * per;                                                                              \
    if (work_units < g) g = work_units;                                                                          \
    return (int)(g < 1 ? 1 : g);                                                                                 \
  }                                                                                                              \
  void mf_host_tables_k##KK(int* nperm, int* ncomb, double* den, double* cden, const float** cn,                \
                             const signed char** hh) {                                                           \
    *nperm = ttng##KK::NPERM;                                                                                    \
    *ncomb = ttng##KK::NCOMB;                                                                                    \
    *den = ttng##KK::DENOMINATOR;                                                                                \
    *cden = ttng##KK::COLOUR_DEN;                                                                                \
    *cn = ttng##KK::colour_num_h;                                                                                \
    *hh = &ttng##KK::hel_h[0][0];                                                                                \
  }                                                                                                              \
  int mf_launch_smatrix_k##KK(int prec, const double* ps, int64_t N, double mt, double wt, const double* coup,    \
                              int64_t cstride, double* out, double* hel_out, cudaStream_t st) {                  \
    using G = Geom<ttng##KK::NCOMB>;                                                                             \
    int64_t units = (N + MF_WARPS * G::EPW - 1) / (MF_WARPS * G::EPW);                                           \
    if (prec == 0) {                                                                                             \
      int g = grid_for<double>((const void*)smatrix_kernel<KK, double>, 0, units);                              \
      smatrix_kernel<KK, double><<<g, 32 * MF_WARPS, 0, st>>>(ps, N, mt, wt, coup, cstride, out, hel_out);      \
    } else {                                                                                                     \
      int g = grid_for<float>((const void*)smatrix_kernel<KK, float>, 0, units);                                \
      smatrix_kernel<KK, float><<<g, 32 * MF_WARPS, 0, st>>>(ps, N, mt, wt, coup, cstride, out, hel_out);       \
    }                                                                                                            \
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 2;                                                         \
  }                                                                                                              \
  int mf_iteration_grid_k##KK(int prec, int ndim, int nb, int64_t N) {                                           \
    size_t dyn = (size_t)MF_WARPS * ndim * nb * sizeof(double);                                                  \
    int64_t units = (N + MF_WARPS * 32 - 1) / (MF_WARPS * 32);                                                   \
    const void* fn = prec == 0 ? (const void*)iteration_kernel<KK, double> : (const void*)iteration_kernel<KK, float>; \
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);                             \
    return grid_for<double>(fn, dyn, units);                                                                     \
  }                                                                                                              \
  int mf_launch_iteration_k##KK(int prec, const IterArgs& A, int grid, cudaStream_t st) {                        \
    size_t dyn = (size_t)MF_WARPS * A.ndim * A.nb * sizeof(double);                                              \
    if (prec == 0) iteration_kernel<KK, double><<<grid, 32 * MF_WARPS, dyn, st>>>(A);                           \
    else iteration_kernel<KK, float><<<grid, 32 * MF_WARPS, dyn, st>>>(A);                                      \
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 2;                                                         \
  }                                                                                                              \
  int mf_launch_newton_k##KK(const IterArgs& A, int* kmin, cudaStream_t st) {                                    \
    int dev = 0, sms = 0;                                                                                        \
    cudaGetDevice(&dev);                                                                                         \
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);                                           \
    int64_t blocks = (A.N + 255) / 256;                                                                          \
    if (blocks > 8 * sms) blocks = 8 * sms;                                                                      \
    if (blocks < 1) blocks = 1;                                                                                  \
    newton_pass_kernel<KK><<<(int)blocks, 256, 0, st>>>(A, kmin);                                               \
    return cudaPeekAtLastError() == cudaSuccess ? 0 : 2;                                                         \
  }
