// Common device types for the madflow GB300 kernels: complex numbers, the
// four-component HELAS spinor/polarisation, Philox4x32-10 and the constants
// madflow carries with float32 rounding.
#pragma once
#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

#define MF_HD __host__ __device__ __forceinline__
#define MF_D __host__ __device__ __forceinline__
#define MF_DO __device__ __forceinline__

template <class T> struct cx {
  T re, im;
};
template <class T> MF_HD cx<T> operator+(cx<T> a, cx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <class T> MF_HD cx<T> operator-(cx<T> a, cx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <class T> MF_HD cx<T> operator-(cx<T> a) { return {-a.re, -a.im}; }
template <class T> MF_HD cx<T> operator*(cx<T> a, cx<T> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <class T> MF_HD cx<T> operator*(T s, cx<T> a) { return {s * a.re, s * a.im}; }
template <class T> MF_HD cx<T>& operator+=(cx<T>& a, cx<T> b) { a.re += b.re; a.im += b.im; return a; }
template <class T> MF_HD cx<T>& operator-=(cx<T>& a, cx<T> b) { a.re -= b.re; a.im -= b.im; return a; }
template <class T> MF_HD cx<T> conjg(cx<T> a) { return {a.re, -a.im}; }
template <class T> MF_HD cx<T> mul_i(cx<T> a) { return {-a.im, a.re}; }
template <class T> MF_HD cx<T> mul_mi(cx<T> a) { return {a.im, -a.re}; }
template <class T> MF_HD cx<T> cdiv(cx<T> a, cx<T> b) {
  T d = b.re * b.re + b.im * b.im;
  return {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}
template <class T, class S> MF_HD cx<T> ccast(cx<S> a) { return {(T)a.re, (T)a.im}; }

// Slots 2-5 of a HELAS wavefunction (the momentum flow of slots 0-1 is kept
// per subset of external legs instead).
template <class T> struct alignas(16) W4 {
  cx<T> v[4];
};
template <class T> MF_HD W4<T> w4zero() {
  W4<T> z;
#pragma unroll
  for (int i = 0; i < 4; ++i) z.v[i] = cx<T>{T(0), T(0)};
  return z;
}
template <class T> MF_HD W4<T> neg(const W4<T>& a) {
  W4<T> z;
#pragma unroll
  for (int i = 0; i < 4; ++i) z.v[i] = -a.v[i];
  return z;
}

// madflow turns Python floats into float64 tensors through float32
// (float_me = tf.cast), so these reference constants carry float32 rounding.
struct MfConsts {
  double pi, acc, sqh, gev2pb;
};
MF_HD MfConsts mf_consts(bool f32_quirks) {
  if (f32_quirks) return {3.1415927410125732, 1.0000000133514320e-10, 0.70710676908493042, 389379360.0};
  return {3.141592653589793, 1e-10, 0.70710678118654752, 389379365.6};
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11).
// ---------------------------------------------------------------------------
MF_HD void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
    uint32_t hi0 = __umulhi(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
#else
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0], p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0, hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
#endif
    uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0; c[1] = lo1; c[2] = n2; c[3] = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
}
// 53-bit uniform in (0, 1)
MF_HD double u53(uint32_t hi, uint32_t lo) {
  uint64_t m = (((uint64_t)hi << 32) | lo) >> 11;
  return ((double)m + 0.5) * (1.0 / 9007199254740992.0);
}
// Two uniforms (dimensions 2j, 2j+1) of `event` in `iteration` of `stream`.
MF_HD void philox_pair(uint64_t seed, uint32_t stream, uint32_t iteration, uint64_t event, uint32_t j, double& u0,
                       double& u1) {
  uint32_t c[4] = {(uint32_t)event, (uint32_t)(event >> 32), j, iteration};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32) ^ stream);
  u0 = u53(c[0], c[1]);
  u1 = u53(c[2], c[3]);
}
