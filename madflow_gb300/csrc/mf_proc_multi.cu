// Several processes in one persistent launch: the events of up to
// MF_MULTI_MAX processes (g g > t t~ + 0, 1 or 2 gluons, uneven costs) form
// one work list, ordered by cost (the process with the most colour flows
// first); every block takes the next event from a global counter, so the
// blocks stay busy until the list is empty whatever the mix.
#include "mf_me.cuh"
#include "generated/ttng2.cuh"
#include "generated/ttng3.cuh"
#include "generated/ttng4.cuh"
#include "mf_launch.h"

MF_DEFINE_REC(2)
MF_DEFINE_REC(3)
MF_DEFINE_REC(4)

template <class T> constexpr size_t multi_smem_bytes() {
  size_t a = sizeof(RecSmem<T, 2>), b = sizeof(RecSmem<T, 3>), c = sizeof(RecSmem<T, 4>);
  size_t m = a > b ? a : b;
  return m > c ? m : c;
}

template <class T>
__global__ void __launch_bounds__(MF_REC_NT, sizeof(T) == 4 ? 4 : 2)
    me_multi_kernel(MultiMe M, unsigned long long* __restrict__ counter) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  __shared__ unsigned long long item;
  const int tid = threadIdx.x;
  constexpr int nt = MF_REC_NT;  // launched with MF_REC_NT threads
  const unsigned long long total = (unsigned long long)M.off[M.n];
  for (;;) {
    if (tid == 0) item = atomicAdd(counter, 1ull);
    __syncthreads();
    const unsigned long long it = item;
    __syncthreads();
    if (it >= total) break;
    int j = 0;
    while (j + 1 < M.n && it >= (unsigned long long)M.off[j + 1]) ++j;
    const int64_t e = (int64_t)(it - (unsigned long long)M.off[j]);
    double r = 0.0;
    switch (M.k[j]) {
      case 2:
        r = me_rec_event<T, 2, nt>(*reinterpret_cast<RecSmem<T, 2>*>(smem_raw), M.prep[j] + e * prep_words<T, 2>(), tid);
        break;
      case 3:
        r = me_rec_event<T, 3, nt>(*reinterpret_cast<RecSmem<T, 3>*>(smem_raw), M.prep[j] + e * prep_words<T, 3>(), tid);
        break;
      default:
        r = me_rec_event<T, 4, nt>(*reinterpret_cast<RecSmem<T, 4>*>(smem_raw), M.prep[j] + e * prep_words<T, 4>(), tid);
        break;
    }
    if (tid == 0) M.out[j][e] = r;
  }
}

int mf_launch_me_multi(int prec, const MultiMe& M, unsigned long long* counter, cudaStream_t st) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st) != cudaSuccess) return 2;
  const void* fn = prec == 0 ? (const void*)me_multi_kernel<double> : (const void*)me_multi_kernel<float>;
  int bytes = prec == 0 ? (int)multi_smem_bytes<double>() : (int)multi_smem_bytes<float>();
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, MF_REC_NT, bytes);
  if (per < 1) per = 1;
  int64_t g = (int64_t)sms * per;
  if (g > M.off[M.n]) g = M.off[M.n];
  if (g < 1) g = 1;
  if (prec == 0)
    me_multi_kernel<double><<<(int)g, MF_REC_NT, bytes, st>>>(M, counter);
  else
    me_multi_kernel<float><<<(int)g, MF_REC_NT, bytes, st>>>(M, counter);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : 2;
}
