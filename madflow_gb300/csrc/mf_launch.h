// Host-side launchers of the per-process kernels (one translation unit per
// process), called by the C ABI in mf_core.cu.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
struct IterArgs;
#define MF_DECLARE_PROCESS(KK)                                                                                \
  void mf_host_tables_k##KK(int* nperm, int* ncomb, double* den, double* cden, const float** cn,               \
                            const signed char** hh);                                                          \
  int mf_launch_smatrix_k##KK(int prec, const double* ps, int64_t N, double mt, double wt, const double* coup, \
                              int64_t cstride, double* out, double* hel_out, cudaStream_t st);               \
  int mf_iteration_grid_k##KK(int prec, int ndim, int nb, int64_t N);                                         \
  int mf_launch_iteration_k##KK(int prec, const IterArgs& A, int grid, cudaStream_t st);                      \
  int mf_launch_newton_k##KK(const IterArgs& A, int* kmin, cudaStream_t st);
MF_DECLARE_PROCESS(2)
MF_DECLARE_PROCESS(3)
MF_DECLARE_PROCESS(4)

inline void mf_host_tables(int k, int* nperm, int* ncomb, double* den, double* cden, const float** cn,
                           const signed char** hh) {
  switch (k) {
    case 2: mf_host_tables_k2(nperm, ncomb, den, cden, cn, hh); break;
    case 3: mf_host_tables_k3(nperm, ncomb, den, cden, cn, hh); break;
    default: mf_host_tables_k4(nperm, ncomb, den, cden, cn, hh); break;
  }
}
