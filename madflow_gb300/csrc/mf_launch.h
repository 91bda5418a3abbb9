// Host-side launchers of the per-process kernels (one translation unit per
// process), called by the C ABI in mf_core.cu.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
struct IterArgs;
// Launch configuration of the matrix-element kernel (chosen by the
// autotuner): colour sum on the SIMT lanes (0) or the tensor cores (1), and
// the grid as `waves` x (SMs x resident blocks per SM).
// wait_tries: ~1 ms tries of each bounded wait on the tensor cores before a
// block gives up (its events then get NaN and error bit 0 is raised).
constexpr int MF_TC_WAIT_TRIES = 1000;
struct MeTune {
  int colour;
  int waves;
  int wait_tries;
};
// Work list of one multi-process launch: n processes, process j with k[j]
// gluons, records prep[j], its events at list positions [off[j], off[j+1]),
// results out[j].
constexpr int MF_MULTI_MAX = 4;
struct MultiMe {
  int n;
  int k[MF_MULTI_MAX];
  const int4* prep[MF_MULTI_MAX];
  int64_t off[MF_MULTI_MAX + 1];
  double* out[MF_MULTI_MAX];
};
int mf_launch_me_multi(int prec, const MultiMe& M, unsigned long long* counter, cudaStream_t st);
#define MF_DECLARE_PROCESS(KK)                                                                              \
  void mf_host_tables_k##KK(int* nperm, int* ncomb, double* den, double* cden, const float** cn,             \
                            const signed char** hh);                                                        \
  int64_t mf_prep_bytes_k##KK(int prec);                                                                     \
  int mf_launch_me_k##KK(int prec, const int4* prep, int64_t N, const double* skip, double* out,             \
                         double* hel_out, int* err, MeTune t, void* ws, cudaStream_t st);                   \
  int64_t mf_ws_bytes_k##KK(int prec);                                                                       \
  bool mf_colour_tc_k##KK();                                                                                 \
  int mf_launch_prep_k##KK(int prec, const double* ps, int64_t N, double mt, double wt, const double* coup,  \
                           int64_t cstride, int4* prep, cudaStream_t st);                                   \
  int mf_launch_ps_k##KK(int prec, const IterArgs& A, cudaStream_t st);                                     \
  int64_t mf_state_words_k##KK();                                                                            \
  int mf_launch_seed_k##KK(int prec, const IterArgs& A, int* kmin, int batch_rule, cudaStream_t st);
MF_DECLARE_PROCESS(2)
MF_DECLARE_PROCESS(3)
MF_DECLARE_PROCESS(4)
MF_DECLARE_PROCESS(5)

inline void mf_host_tables(int k, int* nperm, int* ncomb, double* den, double* cden, const float** cn,
                           const signed char** hh) {
  switch (k) {
    case 2: mf_host_tables_k2(nperm, ncomb, den, cden, cn, hh); break;
    case 3: mf_host_tables_k3(nperm, ncomb, den, cden, cn, hh); break;
    case 4: mf_host_tables_k4(nperm, ncomb, den, cden, cn, hh); break;
    default: mf_host_tables_k5(nperm, ncomb, den, cden, cn, hh); break;
  }
}
inline int64_t mf_prep_bytes(int k, int prec) {
  switch (k) {
    case 2: return mf_prep_bytes_k2(prec);
    case 3: return mf_prep_bytes_k3(prec);
    case 4: return mf_prep_bytes_k4(prec);
    default: return mf_prep_bytes_k5(prec);
  }
}
inline int mf_launch_me(int k, int prec, const int4* prep, int64_t N, const double* skip, double* out,
                        double* hel_out, int* err, MeTune t, void* ws, cudaStream_t st) {
  switch (k) {
    case 2: return mf_launch_me_k2(prec, prep, N, skip, out, hel_out, err, t, ws, st);
    case 3: return mf_launch_me_k3(prec, prep, N, skip, out, hel_out, err, t, ws, st);
    case 4: return mf_launch_me_k4(prec, prep, N, skip, out, hel_out, err, t, ws, st);
    case 5: return mf_launch_me_k5(prec, prep, N, skip, out, hel_out, err, t, ws, st);
  }
  return 3;
}
// bytes of global workspace the matrix-element launch of a process needs (0: shared memory only)
inline int64_t mf_ws_bytes(int k, int prec) {
  switch (k) {
    case 2: return mf_ws_bytes_k2(prec);
    case 3: return mf_ws_bytes_k3(prec);
    case 4: return mf_ws_bytes_k4(prec);
    default: return mf_ws_bytes_k5(prec);
  }
}
// whether the process has a tensor-core colour variant (FP32)
inline bool mf_colour_tc(int k) {
  switch (k) {
    case 2: return mf_colour_tc_k2();
    case 3: return mf_colour_tc_k3();
    case 4: return mf_colour_tc_k4();
    default: return mf_colour_tc_k5();
  }
}
inline int mf_launch_prep(int k, int prec, const double* ps, int64_t N, double mt, double wt, const double* coup,
                          int64_t cstride, int4* prep, cudaStream_t st) {
  switch (k) {
    case 2: return mf_launch_prep_k2(prec, ps, N, mt, wt, coup, cstride, prep, st);
    case 3: return mf_launch_prep_k3(prec, ps, N, mt, wt, coup, cstride, prep, st);
    case 4: return mf_launch_prep_k4(prec, ps, N, mt, wt, coup, cstride, prep, st);
    case 5: return mf_launch_prep_k5(prec, ps, N, mt, wt, coup, cstride, prep, st);
  }
  return 3;
}
inline int mf_launch_ps(int k, int prec, const IterArgs& A, cudaStream_t st) {
  switch (k) {
    case 2: return mf_launch_ps_k2(prec, A, st);
    case 3: return mf_launch_ps_k3(prec, A, st);
    case 4: return mf_launch_ps_k4(prec, A, st);
    case 5: return mf_launch_ps_k5(prec, A, st);
  }
  return 3;
}
inline int64_t mf_state_words(int k) {
  switch (k) {
    case 2: return mf_state_words_k2();
    case 3: return mf_state_words_k3();
    case 4: return mf_state_words_k4();
    default: return mf_state_words_k5();
  }
}
inline int mf_launch_seed(int k, int prec, const IterArgs& A, int* kmin, int batch_rule, cudaStream_t st) {
  switch (k) {
    case 2: return mf_launch_seed_k2(prec, A, kmin, batch_rule, st);
    case 3: return mf_launch_seed_k3(prec, A, kmin, batch_rule, st);
    case 4: return mf_launch_seed_k4(prec, A, kmin, batch_rule, st);
    case 5: return mf_launch_seed_k5(prec, A, kmin, batch_rule, st);
  }
  return 3;
}
