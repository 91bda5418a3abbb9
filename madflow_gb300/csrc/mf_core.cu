// C ABI of madflow_gb300 (declared in include/madflow_gb300.h): process
// handles, phase space, wavefunctions, ALOHA routines, VEGAS and the fused
// integrand/iteration drivers.  Per-process matrix-element kernels live in
// mf_proc_k<K>.cu.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/madflow_gb300.h"
#include "mf_launch.h"
#include "mf_me.cuh"

namespace {
thread_local std::string g_cuda_err;

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return MF_OK;
  g_cuda_err = cudaGetErrorString(e);
  return MF_ERR_CUDA;
}
int last_launch() { return cuda_status(cudaPeekAtLastError()); }
cudaStream_t S(void* s) { return (cudaStream_t)s; }
int blocks_for(int64_t n, int threads = 256) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 65535LL * 64) b = 65535LL * 64;
  return (int)(b < 1 ? 1 : b);
}

// The accumulation kernels keep the histogram of every dimension in dynamic
// shared memory: up to kAccumMaxBins bins in all plus 3 doubles per thread.
// Their attribute is raised once per device to that largest size (a
// process-wide setting, so it is never lowered by a later, smaller call).
constexpr int kAccumMaxBins = 8192;
constexpr int kAccumSmemMax = (kAccumMaxBins + 3 * 256) * (int)sizeof(double);
std::mutex g_attr_mu;
int smem_attr_once(const void* fn, bool* done_per_dev) {
  int dev = 0;
  int st = cuda_status(cudaGetDevice(&dev));
  if (st) return st;
  if (dev < 0 || dev >= 64) return MF_ERR_CAPACITY;
  std::lock_guard<std::mutex> lk(g_attr_mu);
  if (!done_per_dev[dev]) {
    st = cuda_status(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kAccumSmemMax));
    if (st) return st;
    done_per_dev[dev] = true;
  }
  return MF_OK;
}

// ---- synthetic PDF tables, one copy per device -----------------------------
// The gluon of the configurations, x g = A x^-0.2 (1-x)^5 with int x g = 1/2,
// and synthetic quarks for p p > t t~ (x f independent of Q):
//   valence  x u_v = A x^0.5 (1-x)^3 (int u_v = 2), x d_v = A x^0.5 (1-x)^4
//            (int d_v = 1);
//   sea      x qbar = A x^-0.2 (1-x)^7 with int x qbar = 0.03 (ubar, dbar),
//            0.015 (s = sbar), 0.005 (c = cbar);  u = u_v + ubar, d = d_v + dbar.
// Tables [MF_PDF_NF][kNQ][kNX] in the flavour order of pdf_flavour_index.
constexpr int kNX = 100, kNQ = 50;
struct PdfHost {
  std::vector<double> tab;
  double lx0, dlx, lq0, dlq;
};
double beta_fn(double a, double b) { return std::exp(std::lgamma(a) + std::lgamma(b) - std::lgamma(a + b)); }
double synth_xfx(int pdg, double x) {
  if (x >= 1.0) return 0.0;
  if (pdg == 21) return 0.5 / beta_fn(0.8, 6.0) * std::pow(x, -0.2) * std::pow(1.0 - x, 5.0);
  const int a = pdg < 0 ? -pdg : pdg;
  const double frac = a <= 2 ? 0.03 : (a == 3 ? 0.015 : 0.005);
  double v = frac / beta_fn(0.8, 8.0) * std::pow(x, -0.2) * std::pow(1.0 - x, 7.0);
  if (pdg == 2) v += 2.0 / beta_fn(0.5, 4.0) * std::pow(x, 0.5) * std::pow(1.0 - x, 3.0);
  if (pdg == 1) v += 1.0 / beta_fn(0.5, 5.0) * std::pow(x, 0.5) * std::pow(1.0 - x, 4.0);
  return v;
}
const PdfHost& pdf_host() {
  static PdfHost P = [] {
    PdfHost h;
    h.lx0 = std::log(1e-6);
    h.dlx = (0.0 - h.lx0) / (kNX - 1);
    h.lq0 = std::log(1.0);
    h.dlq = (std::log(1e10) - h.lq0) / (kNQ - 1);
    h.tab.resize((size_t)MF_PDF_NF * kNX * kNQ);
    for (int f = 0; f < MF_PDF_NF; ++f)
      for (int iq = 0; iq < kNQ; ++iq)
        for (int ix = 0; ix < kNX; ++ix) {
          double x = std::exp(h.lx0 + ix * h.dlx);
          if (ix == kNX - 1) x = 1.0;
          h.tab[((size_t)f * kNQ + iq) * kNX + ix] = synth_xfx(pdf_flavour_pdg(f), x);
        }
    return h;
  }();
  return P;
}
std::mutex g_pdf_mu;
double* g_pdf_dev[64] = {nullptr};
int pdf_device_table(PdfTable& T) {
  int dev = 0;
  int st = cuda_status(cudaGetDevice(&dev));
  if (st) return st;
  if (dev < 0 || dev >= 64) return MF_ERR_CAPACITY;
  const PdfHost& H = pdf_host();
  {
    std::lock_guard<std::mutex> lk(g_pdf_mu);
    if (!g_pdf_dev[dev]) {
      double* d = nullptr;
      const size_t bytes = sizeof(double) * H.tab.size();
      st = cuda_status(cudaMalloc(&d, bytes));
      if (!st) st = cuda_status(cudaMemcpy(d, H.tab.data(), bytes, cudaMemcpyHostToDevice));
      if (st) {
        cudaFree(d);
        return st;
      }
      g_pdf_dev[dev] = d;
    }
  }
  T.tab = g_pdf_dev[dev];
  T.nx = kNX;
  T.nq = kNQ;
  T.lx0 = H.lx0;
  T.dlx = H.dlx;
  T.lq0 = H.lq0;
  T.dlq = H.dlq;
  return MF_OK;
}

struct Masses {
  double m[MF_MAX_OUT];
};

__global__ void set_int_kernel(int* p, int v) { *p = v; }

// ---- phase space kernels ----------------------------------------------------
// pass 1 of the batch Newton rule for rambo / ramboflow
__global__ void rambo_conv_kernel(const double* __restrict__ x, int64_t N, int n, const double* __restrict__ sqrts,
                                  int64_t sstride, Masses M, int flow, double com_s, double shat_min, int* kmin) {
  int local = 11;
  MfConsts K = mf_consts(true);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    double xe[4 * MF_MAX_OUT + 2];
    int nd = flow ? 4 * n + 2 : 4 * n;
    for (int d = 0; d < nd; ++d) xe[d] = x[(int64_t)d * N + e];
    double roots;
    const double* xr = xe;
    if (flow) {
      double shat, w, x1, x2;
      get_x1x2(xe[0], xe[1], shat_min, com_s, shat, w, x1, x2);
      roots = sqrt(shat);
      xr = xe + 2;
    } else {
      roots = sqrts[e * sstride];
    }
    double p[MF_MAX_OUT][4];
    rambo_massless(xr, n, roots, K.pi, p);
    // a non-finite event takes no part in the batch minimum (its f0 > ACC
    // test is false at once and would stop the iteration for every event)
    double chk = roots;
    for (int i = 0; i < n; ++i) chk += p[i][0];
    if (isfinite(chk)) local = min(local, newton_conv_iter(n, M.m, p, roots, K.acc));
  }
  for (int o = 16; o > 0; o >>= 1) local = min(local, __shfl_xor_sync(0xffffffffu, local, o));
  if ((threadIdx.x & 31) == 0) atomicMin(kmin, local);
}

// rambo (flow = 0, n outgoing particles in p[n][4][N]) or ramboflow (flow = 1,
// p[n+2][4][N] with the two incoming partons first).
__global__ void rambo_kernel(const double* __restrict__ x, int64_t N, int n, const double* __restrict__ sqrts,
                             int64_t sstride, Masses M, int massive, int flow, double com_s, double shat_min,
                             const int* __restrict__ kmin, int per_event, double* __restrict__ p,
                             double* __restrict__ w, double* __restrict__ x1o, double* __restrict__ x2o) {
  MfConsts K = mf_consts(true);
  int iters = per_event ? 0 : min(*kmin, 10);
  int npo = flow ? n + 2 : n;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    double xe[4 * MF_MAX_OUT + 2];
    int nd = flow ? 4 * n + 2 : 4 * n;
    for (int d = 0; d < nd; ++d) xe[d] = x[(int64_t)d * N + e];
    double roots, shat = 0, wgt = 1.0, x1 = 1, x2 = 1;
    const double* xr = xe;
    if (flow) {
      get_x1x2(xe[0], xe[1], shat_min, com_s, shat, wgt, x1, x2);
      roots = sqrt(shat);
      xr = xe + 2;
    } else {
      roots = sqrts[e * sstride];
    }
    double q[MF_MAX_OUT + 2][4];
    double(*po)[4] = flow ? q + 2 : q;
    double logw = rambo_massless(xr, n, roots, K.pi, po);
    double wps;
    if (massive) logw = rambo_massive(n, M.m, po, roots, logw, K.acc, iters);
    wps = exp(logw) / pow(2.0 * K.pi, (double)(3 * n - 4));
    if (flow) {
      double ein = roots / 2.0;
      q[0][0] = ein; q[0][1] = 0; q[0][2] = 0; q[0][3] = ein;
      q[1][0] = ein; q[1][1] = 0; q[1][2] = 0; q[1][3] = -ein;
      wgt = wgt * wps;
      wgt = wgt * K.gev2pb;
      wgt = wgt / (2.0 * shat);
      x1o[e] = x1;
      x2o[e] = x2;
    } else {
      wgt = wps;
    }
    w[e] = wgt;
    for (int i = 0; i < npo; ++i)
      for (int c = 0; c < 4; ++c) p[((int64_t)i * 4 + c) * N + e] = q[i][c];
  }
}

__global__ void boost_kernel(double* __restrict__ p, int64_t N, int n, const double* __restrict__ x1,
                             const double* __restrict__ x2) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x)
    for (int i = 0; i < n; ++i) {
      double q[4];
      for (int c = 0; c < 4; ++c) q[c] = p[((int64_t)i * 4 + c) * N + e];
      boost_lab(q, x1[e], x2[e]);
      p[((int64_t)i * 4 + 0) * N + e] = q[0];
      p[((int64_t)i * 4 + 3) * N + e] = q[3];
    }
}

// ---- wavefunction / ALOHA kernels (reference slot layout [6][2][N]) --------
__device__ __forceinline__ void load_p(const double* p, int64_t N, int64_t e, double* q) {
  for (int c = 0; c < 4; ++c) q[c] = p[(int64_t)c * N + e];
}
__device__ __forceinline__ void store_slot(double* out, int64_t N, int64_t e, int s, cx<double> v) {
  out[((int64_t)s * 2 + 0) * N + e] = v.re;
  out[((int64_t)s * 2 + 1) * N + e] = v.im;
}
__device__ __forceinline__ cx<double> load_slot(const double* in, int64_t N, int64_t e, int s) {
  return {in[((int64_t)s * 2 + 0) * N + e], in[((int64_t)s * 2 + 1) * N + e]};
}
__device__ __forceinline__ W4<double> load_w4(const double* in, int64_t N, int64_t e) {
  W4<double> w;
  for (int k = 0; k < 4; ++k) w.v[k] = load_slot(in, N, e, 2 + k);
  return w;
}
__device__ __forceinline__ void slot_mom(const double* in, int64_t N, int64_t e, double* P) {
  cx<double> s0 = load_slot(in, N, e, 0), s1 = load_slot(in, N, e, 1);
  P[0] = s0.re; P[1] = s1.re; P[2] = s1.im; P[3] = s0.im;
}

__global__ void wf_kernel(int which, const double* __restrict__ p, int64_t N, double m, double nhel, double ns,
                          double* __restrict__ out) {
  const double sqh = mf_consts(true).sqh;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    double q[4];
    load_p(p, N, e, q);
    W4<double> f;
    double sg = ns;
    if (which == 0) { f = ixxxxx<double>(q, m, nhel, ns); sg = -ns; }
    else if (which == 1) f = oxxxxx<double>(q, m, nhel, ns);
    else if (which == 2) f = vxxxxx<double>(q, m, nhel, ns, sqh);
    if (which == 3) {
      store_slot(out, N, e, 0, {q[0] * ns, q[3] * ns});
      store_slot(out, N, e, 1, {q[1] * ns, q[2] * ns});
      store_slot(out, N, e, 2, {1.0, 0.0});
      continue;
    }
    store_slot(out, N, e, 0, {q[0] * sg, q[3] * sg});
    store_slot(out, N, e, 1, {q[1] * sg, q[2] * sg});
    for (int k = 0; k < 4; ++k) store_slot(out, N, e, 2 + k, f.v[k]);
  }
}

// y += S(V)^T F
__device__ __forceinline__ void svt_add(const W4<double>& V, const W4<double>& F, W4<double>& y) {
  cx<double> p03 = V.v[0] + V.v[3], m03 = V.v[0] - V.v[3];
  cx<double> p12 = V.v[1] + mul_i(V.v[2]), m12 = V.v[1] - mul_i(V.v[2]);
  y.v[0] += m03 * F.v[2] - m12 * F.v[3];
  y.v[1] += -(p12 * F.v[2]) + p03 * F.v[3];
  y.v[2] += p03 * F.v[0] + m12 * F.v[1];
  y.v[3] += p12 * F.v[0] + m03 * F.v[1];
}

// which: 0 FFV1_0, 1 FFV1_1, 2 FFV1_2, 3 VVV1P0_1
__global__ void aloha_kernel(int which, const double* __restrict__ A, const double* __restrict__ B,
                             const double* __restrict__ Cw, cx<double> coup, double M, double W, int64_t N,
                             double* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    if (which == 0) {
      cx<double> t = sandwich<double>(load_w4(A, N, e), load_w4(Cw, N, e), load_w4(B, N, e));
      cx<double> a = coup * mul_mi(t);
      out[e] = a.re;
      out[N + e] = a.im;
      continue;
    }
    double Pa[4], Pb[4], Q[4];
    slot_mom(A, N, e, Pa);
    slot_mom(B, N, e, Pb);
    for (int c = 0; c < 4; ++c) Q[c] = Pa[c] + Pb[c];
    double q2 = Q[0] * Q[0] - Q[1] * Q[1] - Q[2] * Q[2] - Q[3] * Q[3];
    cx<double> cf = cdiv(mul_i(coup), cx<double>{q2 - M * M, M * W});
    W4<double> r;
    if (which == 1) {
      W4<double> y = w4zero<double>();
      sv_add<double>(load_w4(B, N, e), load_w4(A, N, e), y);
      r = topprop<double>(Q, M, cf, y);
    } else if (which == 2) {
      W4<double> y = w4zero<double>(), z = w4zero<double>();
      svt_add(load_w4(B, N, e), load_w4(A, N, e), y);
      W4<double> mq;  // S(P)^T with P = -Q
      for (int c = 0; c < 4; ++c) mq.v[c] = {-Q[c], 0.0};
      svt_add(mq, y, z);
      for (int c = 0; c < 4; ++c) r.v[c] = cf * (z.v[c] + M * y.v[c]);
    } else {
      W4<double> acc = w4zero<double>();
      vvv_add<double>(load_w4(A, N, e), Pa, load_w4(B, N, e), Pb, acc);
      for (int c = 0; c < 4; ++c) r.v[c] = cf * acc.v[c];
    }
    cx<double> a0 = load_slot(A, N, e, 0), b0 = load_slot(B, N, e, 0);
    cx<double> a1 = load_slot(A, N, e, 1), b1 = load_slot(B, N, e, 1);
    store_slot(out, N, e, 0, a0 + b0);
    store_slot(out, N, e, 1, a1 + b1);
    for (int c = 0; c < 4; ++c) store_slot(out, N, e, 2 + c, r.v[c]);
  }
}

// ---- VEGAS ------------------------------------------------------------------
__global__ void vegas_sample_kernel(const double* __restrict__ div, int ndim, int nb, const double* __restrict__ u,
                                    int64_t N, double* __restrict__ x, double* __restrict__ jac,
                                    int32_t* __restrict__ bins) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    double j = 1.0;
    for (int d = 0; d < ndim; ++d) {
      double xn = u[(int64_t)d * N + e] * (double)nb;
      int i = (int)xn;
      // caller uniforms outside [0, 1) (or NaN) fall in the edge bins
      if (!(xn >= 0.0)) i = 0;
      if (i > nb - 1) i = nb - 1;
      double frac = xn - (double)i;
      double lo = div[d * (nb + 1) + i];
      double w = div[d * (nb + 1) + i + 1] - lo;
      x[(int64_t)d * N + e] = fma(w, frac, lo);
      j *= w * (double)nb;
      bins[(int64_t)d * N + e] = i;
    }
    jac[e] = j;
  }
}

// Lepage refinement, one thread per dimension (smoothing with neighbours,
// damping ((r-1)/ln r)^alpha, equal-share redistribution of the bin edges).
__global__ void vegas_refine_kernel(double* __restrict__ div, const double* __restrict__ hist, int ndim, int nb,
                                    double alpha) {
  int dim = blockIdx.x * blockDim.x + threadIdx.x;
  if (dim >= ndim) return;
  constexpr int NBMAX = 256;
  double d[NBMAX], r[NBMAX], nd[NBMAX + 1];
  const double* h = hist + dim * nb;
  double* g = div + dim * (nb + 1);
  d[0] = (h[0] + h[1]) / 2.0;
  for (int i = 1; i < nb - 1; ++i) d[i] = (h[i - 1] + h[i] + h[i + 1]) / 3.0;
  d[nb - 1] = (h[nb - 2] + h[nb - 1]) / 2.0;
  double tot = 0.0;
  for (int i = 0; i < nb; ++i) tot += d[i];
  if (!(tot > 0.0)) return;
  double rsum = 0.0;
  for (int i = 0; i < nb; ++i) {
    double q = d[i] / tot;
    r[i] = (q > 0.0) ? pow((q - 1.0) / log(q), alpha) : 0.0;
    rsum += r[i];
  }
  if (!(rsum > 0.0)) return;
  double per = rsum / (double)nb;
  nd[0] = g[0];
  nd[nb] = g[nb];
  int i = 0;
  double accum = 0.0;
  for (int j = 1; j < nb; ++j) {
    double target = per * (double)j;
    while (i < nb && accum + r[i] < target) { accum += r[i]; ++i; }
    if (i >= nb) { nd[j] = g[nb]; continue; }
    double frac = (target - accum) / r[i];
    nd[j] = g[i] + frac * (g[i + 1] - g[i]);
  }
  for (int j = 0; j <= nb; ++j) g[j] = nd[j];
}

// Fixed-order sum of the per-block partials: out[i] = sum_b partials[b][i]
// (add: out[i] += that sum, for the later slices of an iteration).
__global__ void reduce_partials_kernel(const double* __restrict__ partials, int nblocks, int width,
                                       double* __restrict__ out, int add = 0) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= width) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += partials[(int64_t)b * width + i];
  out[i] = add ? out[i] + s : s;
}

// Deterministic VEGAS accumulation for integrands evaluated outside the fused
// kernel: block b owns a contiguous slice of events; sums are tree-reduced in
// a fixed order and each histogram dimension is summed by one thread in event
// order.
__global__ void vegas_accum_kernel(const double* __restrict__ f, const double* __restrict__ jac,
                                   const int32_t* __restrict__ bins, int64_t N, int ndim, int nb, double inv_n,
                                   double* __restrict__ partials) {
  extern __shared__ double sh[];  // [ndim*nb] + [2*blockDim] + [blockDim]
  double* hist = sh;
  double* red = sh + ndim * nb;
  int width = 2 + ndim * nb;
  int64_t per = (N + gridDim.x - 1) / gridDim.x;
  int64_t e0 = (int64_t)blockIdx.x * per, e1 = min(N, e0 + per);
  for (int i = threadIdx.x; i < ndim * nb; i += blockDim.x) hist[i] = 0.0;
  double a = 0.0, b = 0.0;
  for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    double w = f[e] * jac[e] * inv_n;
    a += w;
    b += w * w;
  }
  red[threadIdx.x] = a;
  red[blockDim.x + threadIdx.x] = b;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      red[threadIdx.x] += red[threadIdx.x + s];
      red[blockDim.x + threadIdx.x] += red[blockDim.x + threadIdx.x + s];
    }
    __syncthreads();
  }
  // per-bin sums of w^2 in event order, one thread per dimension; w^2 of a
  // chunk of blockDim events is formed once by all threads
  double* w2 = red + 2 * blockDim.x;
  for (int64_t c0 = e0; c0 < e1; c0 += blockDim.x) {
    const int64_t e = c0 + threadIdx.x;
    if (e < e1) {
      const double w = f[e] * jac[e] * inv_n;
      w2[threadIdx.x] = w * w;
    }
    __syncthreads();
    const int cn = (int)min((int64_t)blockDim.x, e1 - c0);
    for (int d = threadIdx.x; d < ndim; d += blockDim.x) {
      const int32_t* bd = bins + (int64_t)d * N + c0;
      double* hd = hist + d * nb;
      // bins come from the caller: an index outside [0, nb) is not added
      for (int j = 0; j < cn; ++j) {
        const int32_t b = bd[j];
        if ((uint32_t)b < (uint32_t)nb) hd[b] += w2[j];
      }
    }
    __syncthreads();
  }
  double* out = partials + (int64_t)blockIdx.x * width;
  if (threadIdx.x == 0) { out[0] = red[0]; out[1] = red[blockDim.x]; }
  for (int i = threadIdx.x; i < ndim * nb; i += blockDim.x) out[2 + i] = hist[i];
}

__global__ void philox_kernel(uint64_t seed, uint32_t stream, uint32_t it, uint64_t e0, int64_t N, int ndim,
                              double* __restrict__ u) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x)
    for (int d = 0; d < ndim; d += 2) {
      double a, b;
      philox_pair(seed, stream, it, e0 + (uint64_t)e, d / 2, a, b);
      u[(int64_t)d * N + e] = a;
      if (d + 1 < ndim) u[(int64_t)(d + 1) * N + e] = b;
    }
}

__global__ void pdf_kernel(PdfTable P, const double* __restrict__ x, int64_t N, double q2, double* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = pdf_xfx(P, x[e], q2);
}
__global__ void pdf_flavour_kernel(PdfTable P, int f, const double* __restrict__ x, int64_t N, double q2,
                                   double* __restrict__ out) {
  const double v = pdf_qcoord(P, q2);
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = pdf_xfx_fv(P, f, x[e], v);
}

// q q~ > t t~, one thread per event: ps [4][4][N] (q, q~, t, t~), couplings
// [N or 1][3] complex (GC_11 used)
__global__ void qq_ttx_kernel(int prec, const double* __restrict__ ps, int64_t N, double mt,
                              const double* __restrict__ coup, int64_t cstride, double* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    double p[4][4];
    for (int i = 0; i < 4; ++i)
      for (int c = 0; c < 4; ++c) p[i][c] = ps[((int64_t)i * 4 + c) * N + e];
    const double* cp = coup + 6 * cstride * e;
    const double g11sq = cp[2] * cp[2] + cp[3] * cp[3];
    out[e] = prec == MF_PREC_FP64 ? uux_ttx_me<double>(p, mt, g11sq) : uux_ttx_me<float>(p, mt, g11sq);
  }
}
template <class T>
__global__ void __launch_bounds__(128) gg2_smatrix_kernel(const double* __restrict__ ps, int64_t N, double mt,
                                                          double wt, const double* __restrict__ coup, int64_t cstride,
                                                          double* __restrict__ out, double* __restrict__ hel_out) {
  const T sqh = (T)mf_consts(true).sqh;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    double p[4][4];
    for (int i = 0; i < 4; ++i)
      for (int c = 0; c < 4; ++c) p[i][c] = ps[((int64_t)i * 4 + c) * N + e];
    const double* cp = coup + 6 * cstride * e;
    out[e] = gg2_me<T>(p, mt, wt, {cp[0], cp[1]}, {cp[2], cp[3]}, sqh, hel_out ? hel_out + e : nullptr, N);
  }
}

template <class T>
__global__ void __launch_bounds__(128) qq3_smatrix_kernel(int channel, const double* __restrict__ ps, int64_t N,
                                                          double mt, double wt, const double* __restrict__ coup,
                                                          int64_t cstride, double* __restrict__ out) {
  // a group of four lanes per event (mfqq3)
  const int lane = threadIdx.x & 3, base = (threadIdx.x & 31) & ~3;
  const unsigned mask = 0xFu << base;
  const T sqh = (T)mf_consts(true).sqh;
  const int64_t stride = (int64_t)gridDim.x * (blockDim.x >> 2);
  for (int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2; e < N; e += stride) {
    double p[5][4];
    for (int i = 0; i < 5; ++i)
      for (int c = 0; c < 4; ++c) p[i][c] = ps[((int64_t)i * 4 + c) * N + e];
    const double* cp = coup + 6 * cstride * e;
    const cx<double> gc10{cp[0], cp[1]}, gc11{cp[2], cp[3]};
    // the evaluation of the channel in qq3_weighted_sum's order (q q~, q~ q, q g, q~ g, ...)
    double w[6] = {0, 0, 0, 0, 0, 0};
    w[channel == 0 ? 0 : channel + 1] = 1.0;
    const double r = qq3_weighted_sum<T>(p, w, mt, wt, gc10, gc11, sqh, mask, lane, base);
    if (lane == 0) out[e] = r;
  }
}
}  // namespace

// ---------------------------------------------------------------------------
// per-event pipeline buffers of one slice of a call
struct SliceBuf {
  int4* prep = nullptr;
  double* state = nullptr;
  double* pref = nullptr;
  double* me = nullptr;
  unsigned char* bins = nullptr;
  double* extra = nullptr;
  double* qqin = nullptr;
  int* kmin = nullptr;
  int64_t cap = 0, extra_cap = 0, qqin_cap = 0;
  void release() {
    for (void* q : {(void*)prep, (void*)state, (void*)pref, (void*)me, (void*)bins, (void*)extra, (void*)qqin,
                    (void*)kmin})
      if (q) cudaFree(q);
    *this = SliceBuf();
  }
};

struct mf_process {
  int k, prec;
  int ncomb, nperm, ndiags;
  double denominator;
  std::vector<double> hel, colour;
  int device;
  // scratch owned by the handle (grown on demand): the Newton counter, the
  // block partials and the per-event pipeline buffers of an iteration
  int* d_kmin = nullptr;
  double* d_partials = nullptr;
  size_t partial_cap = 0;
  int* d_zero_iter = nullptr;
  int* d_event_iter = nullptr;  // iteration index of mf_vegas_events
  unsigned long long* d_counter = nullptr;  // work counter of multi-process launches
  void* d_ws = nullptr;     // global matrix-element workspace (processes too large for shared memory)
  int4* d_prep = nullptr;   // [cap] per-event matrix-element records
  double* d_state = nullptr; // [state words][cap] first-pass phase-space state
  double* d_pref = nullptr; // [cap]
  double* d_me = nullptr;   // [cap]
  double* d_extra = nullptr;  // [extra_cap] weights of further channels (p p > t t~ (j))
  int64_t extra_cap = 0;
  double* d_qqin = nullptr;   // [26][qqin_cap] inputs of the light-quark channels of p p > t t~ j
  int64_t qqin_cap = 0;
  unsigned char* d_bins = nullptr;  // [MF_MAX_DIM][cap]
  int64_t event_cap = 0;
  // the second buffer set of a call in slices (the odd slices), the side
  // stream their phase-space passes run on and the events that order the
  // two streams
  SliceBuf alt;
  cudaStream_t side = nullptr;
  cudaEvent_t ev_start = nullptr, ev_ps[2] = {nullptr, nullptr}, ev_acc[2] = {nullptr, nullptr};
  int* d_err = nullptr;     // device error flags of the kernels (bit 0: a tensor-core wait ran out,
                            // bit 1: non-finite weights were zeroed)
  unsigned long long* d_nonfinite = nullptr;  // count of the zeroed non-finite weights
  // matrix-element launch configuration and the autotuner's record
  MeTune tune = {1, 8, MF_TC_WAIT_TRIES};
  bool tuned = false;
  float tune_ms[MF_TUNE_VARIANTS] = {};
  // optional stage timing of the fused iteration (events on the caller's stream)
  int timing = 0;
  bool timed_last = false;
  cudaEvent_t tev[MF_STAGES + 1] = {};
};

static const int kDiagrams[6] = {0, 0, 3, 16, 123, 1240};

extern "C" {
static int ensure_events(mf_process* p, int64_t N);
static bool autotune_wanted(const mf_process* p, int64_t N, void* stream);
static int autotune_me(mf_process* p, const int4* prep, int64_t N, const double* skip, double* out, void* stream);

const char* mf_version(void) { return "madflow_gb300 0.1 (sm_103a)"; }

const char* mf_status_string(int s) {
  switch (s) {
    case MF_OK: return "ok";
    case MF_ERR_ARG: return "invalid argument";
    case MF_ERR_CUDA: return "CUDA error";
    case MF_ERR_UNSUPPORTED: return "unsupported process or precision";
    case MF_ERR_CAPACITY: return "request exceeds the supported maximum";
    case MF_ERR_NONFINITE: return "non-finite weights produced";
    case MF_ERR_STATE: return "no result of that kind yet";
  }
  return "unknown status";
}

const char* mf_last_cuda_error(void) { return g_cuda_err.c_str(); }

int mf_process_create(int n_gluons, int precision, mf_process** out) {
  if (!out) return MF_ERR_ARG;
  *out = nullptr;
  if (n_gluons < 2 || n_gluons > 5) return MF_ERR_UNSUPPORTED;
  if (precision != MF_PREC_FP64 && precision != MF_PREC_MIXED) return MF_ERR_ARG;
  auto* p = new mf_process();
  p->k = n_gluons;
  p->prec = precision;
  const float* cn = nullptr;
  const signed char* hh = nullptr;
  double cden = 1.0;
  mf_host_tables(n_gluons, &p->nperm, &p->ncomb, &p->denominator, &cden, &cn, &hh);
  p->ndiags = kDiagrams[n_gluons];
  p->colour.resize((size_t)p->nperm * p->nperm);
  for (size_t i = 0; i < p->colour.size(); ++i) p->colour[i] = (double)cn[i] / cden;
  int npart = n_gluons + 2;
  p->hel.resize((size_t)p->ncomb * npart);
  for (size_t i = 0; i < p->hel.size(); ++i) p->hel[i] = (double)hh[i];
  p->device = -1;
  *out = p;
  return MF_OK;
}

int mf_process_destroy(mf_process* p) {
  if (!p) return MF_ERR_ARG;
  if (p->d_kmin) cudaFree(p->d_kmin);
  if (p->d_partials) cudaFree(p->d_partials);
  if (p->d_zero_iter) cudaFree(p->d_zero_iter);
  if (p->d_event_iter) cudaFree(p->d_event_iter);
  if (p->d_counter) cudaFree(p->d_counter);
  if (p->d_ws) cudaFree(p->d_ws);
  if (p->d_prep) cudaFree(p->d_prep);
  if (p->d_state) cudaFree(p->d_state);
  if (p->d_pref) cudaFree(p->d_pref);
  if (p->d_me) cudaFree(p->d_me);
  if (p->d_bins) cudaFree(p->d_bins);
  if (p->d_err) cudaFree(p->d_err);
  if (p->d_nonfinite) cudaFree(p->d_nonfinite);
  if (p->d_extra) cudaFree(p->d_extra);
  if (p->d_qqin) cudaFree(p->d_qqin);
  p->alt.release();
  if (p->side) cudaStreamDestroy(p->side);
  for (cudaEvent_t e : {p->ev_start, p->ev_ps[0], p->ev_ps[1], p->ev_acc[0], p->ev_acc[1]})
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : p->tev)
    if (e) cudaEventDestroy(e);
  delete p;
  return MF_OK;
}

int mf_process_info(const mf_process* p, int* nexternal, int* ncomb, int* ncolor, int* ndiags, double* den) {
  if (!p) return MF_ERR_ARG;
  if (nexternal) *nexternal = p->k + 2;
  if (ncomb) *ncomb = p->ncomb;
  if (ncolor) *ncolor = p->nperm;
  if (ndiags) *ndiags = p->ndiags;
  if (den) *den = p->denominator;
  return MF_OK;
}

int mf_process_helicities(const mf_process* p, double* out) {
  if (!p || !out) return MF_ERR_ARG;
  std::memcpy(out, p->hel.data(), sizeof(double) * p->hel.size());
  return MF_OK;
}

int mf_process_colour_matrix(const mf_process* p, double* out) {
  if (!p || !out) return MF_ERR_ARG;
  std::memcpy(out, p->colour.data(), sizeof(double) * p->colour.size());
  return MF_OK;
}

int mf_smatrix(const mf_process* p, const double* ps, int64_t N, double mt, double wt, const double* coup,
               int64_t cstride, double* out, double* hel_out, void* stream) {
  if (!p || (N > 0 && (!ps || !coup || !out)) || N < 0 || (cstride != 0 && cstride != 1)) return MF_ERR_ARG;
  if (N == 0) return MF_OK;
  mf_process* pm = const_cast<mf_process*>(p);
  if (p->k == 2) {
    // g g > t t~: one thread per event straight from the momenta
    if (p->prec == MF_PREC_FP64)
      gg2_smatrix_kernel<double><<<blocks_for(N, 128), 128, 0, S(stream)>>>(ps, N, mt, wt, coup, cstride, out,
                                                                             hel_out);
    else
      gg2_smatrix_kernel<float><<<blocks_for(N, 128), 128, 0, S(stream)>>>(ps, N, mt, wt, coup, cstride, out,
                                                                            hel_out);
    return last_launch();
  }
  int st = ensure_events(pm, N);
  if (st) return st;
  if (mf_launch_prep(p->k, p->prec, ps, N, mt, wt, coup, cstride, pm->d_prep, S(stream))) return last_launch();
  if (autotune_wanted(pm, N, stream)) {
    st = autotune_me(pm, pm->d_prep, N, nullptr, out, stream);
    if (st) return st;
  }
  st = mf_launch_me(p->k, p->prec, pm->d_prep, N, nullptr, out, hel_out, pm->d_err, pm->tune, pm->d_ws, S(stream));
  if (st == 3) return MF_ERR_UNSUPPORTED;
  return st ? last_launch() : MF_OK;
}

int mf_smatrix_multi(mf_process* const* procs, int nproc, const double* const* ps, const int64_t* n, double mt,
                     double wt, const double* coup, double* const* out, void* stream) {
  if (!procs || nproc < 1 || nproc > MF_MULTI_MAX || !ps || !n || !coup || !out) return MF_ERR_ARG;
  int prec = -1;
  for (int j = 0; j < nproc; ++j) {
    if (!procs[j] || n[j] < 0 || (n[j] > 0 && (!ps[j] || !out[j]))) return MF_ERR_ARG;
    if (procs[j]->k > 4) return MF_ERR_UNSUPPORTED;  // the shared-memory evaluation only
    if (prec >= 0 && procs[j]->prec != prec) return MF_ERR_ARG;
    prec = procs[j]->prec;
    for (int i = 0; i < j; ++i)
      if (procs[i] == procs[j]) return MF_ERR_ARG;  // each handle holds one batch of records
  }
  // records of every batch (one thread per event each)
  for (int j = 0; j < nproc; ++j) {
    if (n[j] == 0) continue;
    int st = ensure_events(procs[j], n[j]);
    if (st) return st;
    if (mf_launch_prep(procs[j]->k, prec, ps[j], n[j], mt, wt, coup, 0, procs[j]->d_prep, S(stream)))
      return last_launch();
  }
  // the work list, most colour flows first
  int order[MF_MULTI_MAX];
  for (int j = 0; j < nproc; ++j) order[j] = j;
  for (int a = 0; a < nproc; ++a)
    for (int b = a + 1; b < nproc; ++b)
      if (procs[order[b]]->k > procs[order[a]]->k) std::swap(order[a], order[b]);
  MultiMe M;
  std::memset(&M, 0, sizeof(M));
  M.n = 0;
  M.off[0] = 0;
  for (int a = 0; a < nproc; ++a) {
    int j = order[a];
    if (n[j] == 0) continue;
    M.k[M.n] = procs[j]->k;
    M.prep[M.n] = procs[j]->d_prep;
    M.out[M.n] = out[j];
    M.off[M.n + 1] = M.off[M.n] + n[j];
    ++M.n;
  }
  if (M.n == 0) return MF_OK;
  mf_process* p0 = procs[order[0]];
  if (!p0->d_counter) {
    int st = cuda_status(cudaMalloc(&p0->d_counter, sizeof(unsigned long long)));
    if (st) return st;
  }
  if (mf_launch_me_multi(prec, M, p0->d_counter, S(stream))) return last_launch();
  return MF_OK;
}

// ---- phase space --------------------------------------------------------------
static int fill_masses(const double* masses, int n, Masses& M, bool& massive) {
  massive = false;
  for (int i = 0; i < MF_MAX_OUT; ++i) M.m[i] = 0.0;
  if (!masses) return MF_OK;
  for (int i = 0; i < n; ++i) {
    // madflow holds the masses list as float_me(masses): float32-rounded
    M.m[i] = (double)(float)masses[i];
    if (masses[i] != 0.0) massive = true;
  }
  return MF_OK;
}

// scratch int for the Newton rule: one per host thread and device, freed
// when the thread exits
struct NewtonScratch {
  int* ptr[64] = {nullptr};
  ~NewtonScratch() {
    for (int* p : ptr)
      if (p) cudaFree(p);
  }
};
static int newton_scratch(int** out) {
  static thread_local NewtonScratch S;
  int dev = 0;
  int st = cuda_status(cudaGetDevice(&dev));
  if (st) return st;
  if (dev < 0 || dev >= 64) return MF_ERR_CAPACITY;
  if (!S.ptr[dev]) {
    st = cuda_status(cudaMalloc(&S.ptr[dev], sizeof(int)));
    if (st) return st;
  }
  *out = S.ptr[dev];
  return MF_OK;
}

static int rambo_common(const double* x, int64_t N, int n, const double* sqrts, int64_t sstride,
                        const double* masses, int rule, int flow, double com_sqrts, double* p, double* w, double* x1,
                        double* x2, void* stream) {
  if (N < 0 || n < 2 || n > MF_MAX_OUT || (N > 0 && (!x || !p || !w))) return MF_ERR_ARG;
  if (!flow && N > 0 && !sqrts) return MF_ERR_ARG;
  if (flow && N > 0 && (!x1 || !x2)) return MF_ERR_ARG;
  if (rule != MF_NEWTON_BATCH && rule != MF_NEWTON_PER_EVENT) return MF_ERR_ARG;
  if (N == 0) return MF_OK;
  Masses M;
  bool massive;
  fill_masses(masses, n, M, massive);
  double msum = 0.0;
  if (masses)
    for (int i = 0; i < n; ++i) msum += masses[i];
  double shat_min = msum * msum, com_s = com_sqrts * com_sqrts;
  int* kmin = nullptr;
  int st = newton_scratch(&kmin);
  if (st) return st;
  int per_event = rule == MF_NEWTON_PER_EVENT;
  set_int_kernel<<<1, 1, 0, S(stream)>>>(kmin, 11);
  if (massive && !per_event)
    rambo_conv_kernel<<<blocks_for(N), 256, 0, S(stream)>>>(x, N, n, sqrts, sstride, M, flow, com_s, shat_min, kmin);
  rambo_kernel<<<blocks_for(N), 256, 0, S(stream)>>>(x, N, n, sqrts, sstride, M, massive ? 1 : 0, flow, com_s,
                                                      shat_min, kmin, per_event, p, w, x1, x2);
  return last_launch();
}

int mf_rambo(const double* x, int64_t N, int n, const double* sqrts, int64_t sstride, const double* masses, int rule,
             double* p, double* w, void* stream) {
  return rambo_common(x, N, n, sqrts, sstride, masses, rule, 0, 0.0, p, w, nullptr, nullptr, stream);
}

int mf_ramboflow(const double* x, int64_t N, int npart, double com_sqrts, const double* masses, int rule, double* p,
                 double* w, double* x1, double* x2, void* stream) {
  if (npart < 4) return MF_ERR_UNSUPPORTED;
  return rambo_common(x, N, npart - 2, nullptr, 0, masses, rule, 1, com_sqrts, p, w, x1, x2, stream);
}

int mf_boost_to_lab(double* p, int64_t N, int n, const double* x1, const double* x2, void* stream) {
  if (N < 0 || (N > 0 && (!p || !x1 || !x2))) return MF_ERR_ARG;
  if (N == 0) return MF_OK;
  boost_kernel<<<blocks_for(N), 256, 0, S(stream)>>>(p, N, n, x1, x2);
  return last_launch();
}

// ---- wavefunctions / ALOHA ------------------------------------------------------
static int wf_launch(int which, const double* p, int64_t N, double m, double nhel, double ns, double* out,
                     void* stream) {
  if (N < 0 || (N > 0 && (!p || !out))) return MF_ERR_ARG;
  if (N == 0) return MF_OK;
  wf_kernel<<<blocks_for(N), 256, 0, S(stream)>>>(which, p, N, m, nhel, ns, out);
  return last_launch();
}
int mf_ixxxxx(const double* p, int64_t n, double fm, double nhel, double nsf, double* out, void* s) {
  return wf_launch(0, p, n, fm, nhel, nsf, out, s);
}
int mf_oxxxxx(const double* p, int64_t n, double fm, double nhel, double nsf, double* out, void* s) {
  return wf_launch(1, p, n, fm, nhel, nsf, out, s);
}
int mf_vxxxxx(const double* p, int64_t n, double vm, double nhel, double nsv, double* out, void* s) {
  return wf_launch(2, p, n, vm, nhel, nsv, out, s);
}
int mf_sxxxxx(const double* p, int64_t n, double nss, double* out, void* s) {
  return wf_launch(3, p, n, 0.0, 0.0, nss, out, s);
}
static int aloha_launch(int which, const double* A, const double* B, const double* C, const double* coup, double M,
                        double W, int64_t N, double* out, void* stream) {
  if (N < 0 || !coup || (N > 0 && (!A || !B || !out || (which == 0 && !C)))) return MF_ERR_ARG;
  if (N == 0) return MF_OK;
  aloha_kernel<<<blocks_for(N), 256, 0, S(stream)>>>(which, A, B, C, cx<double>{coup[0], coup[1]}, M, W, N, out);
  return last_launch();
}
int mf_FFV1_0(const double* F1, const double* F2, const double* V3, const double* coup, int64_t n, double* out,
              void* s) {
  return aloha_launch(0, F1, F2, V3, coup, 0.0, 0.0, n, out, s);
}
int mf_FFV1_1(const double* F2, const double* V3, const double* coup, double M1, double W1, int64_t n, double* out,
              void* s) {
  return aloha_launch(1, F2, V3, nullptr, coup, M1, W1, n, out, s);
}
int mf_FFV1_2(const double* F1, const double* V3, const double* coup, double M2, double W2, int64_t n, double* out,
              void* s) {
  return aloha_launch(2, F1, V3, nullptr, coup, M2, W2, n, out, s);
}
int mf_VVV1P0_1(const double* V2, const double* V3, const double* coup, double M1, double W1, int64_t n, double* out,
                void* s) {
  return aloha_launch(3, V2, V3, nullptr, coup, M1, W1, n, out, s);
}

// ---- integrand / VEGAS ----------------------------------------------------------
int mf_integrand_ndim(const mf_process* p, const mf_integrand_config* c, int* ndim) {
  if (!p || !c || !ndim) return MF_ERR_ARG;
  if (c->kind == 0) {
    if (p->k != 2) return MF_ERR_UNSUPPORTED;
    *ndim = 8;
  } else if (c->kind == 1) {
    *ndim = 4 * p->k + 2;
  } else {
    return MF_ERR_ARG;
  }
  return MF_OK;
}

static int ensure_partials(mf_process* p, size_t n) {
  if (p->partial_cap >= n) return MF_OK;
  if (p->d_partials) cudaFree(p->d_partials);
  p->d_partials = nullptr;
  p->partial_cap = 0;
  int st = cuda_status(cudaMalloc(&p->d_partials, n * sizeof(double)));
  if (st) return st;
  p->partial_cap = n;
  return MF_OK;
}

static int fill_iter_args(const mf_process* p, const mf_integrand_config* c, IterArgs& A) {
  std::memset(&A, 0, sizeof(A));
  if (c->initial_states != MF_INITIAL_GG && c->initial_states != MF_INITIAL_PP) return MF_ERR_ARG;
  if (c->initial_states == MF_INITIAL_PP && (c->kind != 1 || (p->k != 2 && p->k != 3))) return MF_ERR_UNSUPPORTED;
  A.qq = c->initial_states == MF_INITIAL_PP;
  A.kind = c->kind;
  A.sqrts = c->sqrts;
  A.mt = c->mt;
  A.wt = c->wt;
  double g = 2.0 * std::sqrt(M_PI * c->alpha_s);
  A.gc10 = {-g, 0.0};
  A.gc11 = {0.0, g};
  A.gc12 = {0.0, g * g};
  for (int i = 0; i < MF_MAX_OUT; ++i) A.masses[i] = 0.0;
  A.masses[0] = (double)(float)c->mt;
  A.masses[1] = (double)(float)c->mt;
  A.shat_min = (2.0 * c->mt) * (2.0 * c->mt);
  A.ptmin = c->ptmin;
  A.etamax = c->etamax;
  A.drmin = c->drmin;
  if (c->ptmin_all > 0.0 && c->kind != 1) return MF_ERR_ARG;
  A.ptmin_all = c->ptmin_all > 0.0 ? (double)(float)c->ptmin_all : 0.0;
  if (c->ncuts < 0 || c->ncuts > MF_MAX_CUTS || (c->ncuts > 0 && c->kind != 1)) return MF_ERR_ARG;
  A.ncuts = c->ncuts;
  for (int i = 0; i < c->ncuts; ++i) {
    mf_cut C = c->cuts[i];
    if (C.variable < MF_CUT_PT || C.variable > MF_CUT_ETA || C.particle < 0 || C.particle >= p->k + 2) return MF_ERR_ARG;
    C.has_min = C.has_min != 0;
    C.has_max = C.has_max != 0;
    // float_me(min_val), float_me(max_val): the reference's float32 thresholds
    C.min_val = C.has_min ? (double)(float)C.min_val : 0.0;
    C.max_val = C.has_max ? (double)(float)C.max_val : 0.0;
    A.cuts[i] = C;
  }
  A.q2 = c->q2;
  if (c->q2 < 0.0) {
    // dynamical scale: hadronic collisions only, alpha_s is alpha_s(M_Z^2)
    if (c->kind != 1 || !(c->alpha_s > 0.0)) return MF_ERR_ARG;
    A.dyn = 1;
    A.alpha0 = c->alpha_s;
  } else if (c->kind == 1 && !(c->q2 > 0.0)) {
    return MF_ERR_ARG;  // log Q^2 of the densities
  }
  A.f32q = 1;
  return pdf_device_table(A.pdf);
}

// ---- autotuner of the matrix-element launch ----------------------------------
// On the first uncaptured call with at least kTuneMinEvents events the
// matrix-element kernel is timed (CUDA events, the caller's stream, the
// call's own records, up to kTuneEvents of them) in every variant: colour sum
// on the SIMT lanes or the tensor cores x grid of 1, 2, 4 or 8 waves of
// resident blocks; the fastest becomes the handle's configuration.
// MF_AUTOTUNE=0 in the environment keeps the defaults (tensor cores, 8 waves).
static const int kTuneWaves[4] = {1, 2, 4, 8};
static const int64_t kTuneMinEvents = 262144, kTuneEvents = 1 << 20;
// processes with a global workspace (five gluons): 2^14 events, 16 times the cost each
static const int64_t kTuneMinEventsGws = 16384, kTuneEventsGws = 1 << 14;

static bool autotune_wanted(const mf_process* p, int64_t N, void* stream) {
  const bool gws = mf_ws_bytes(p->k, p->prec) > 0;  // fixed grid: only the colour method is tuned
  if (p->tuned || N < (gws ? kTuneMinEventsGws : kTuneMinEvents)) return false;
  if (gws && (p->prec == MF_PREC_FP64 || !mf_colour_tc(p->k))) return false;
  const char* env = getenv("MF_AUTOTUNE");
  if (env && env[0] == '0') return false;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(S(stream), &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return false;
  return true;
}

static int autotune_me(mf_process* p, const int4* prep, int64_t N, const double* skip, double* out, void* stream) {
  const bool gws = mf_ws_bytes(p->k, p->prec) > 0;
  const int64_t cap = gws ? kTuneEventsGws : kTuneEvents;
  int64_t n = N < cap ? N : cap;
  cudaEvent_t a = nullptr, b = nullptr;
  int st = cuda_status(cudaEventCreate(&a));
  if (!st) st = cuda_status(cudaEventCreate(&b));
  float best = 0.0f;
  MeTune pick = p->tune;
  bool have = false;
  for (int c = 0; c < 2 && !st; ++c) {
    if (c == 1 && (p->prec == MF_PREC_FP64 || !mf_colour_tc(p->k))) {
      for (int w = 0; w < 4; ++w) p->tune_ms[4 * c + w] = -1.0f;
      continue;
    }
    for (int w = 0; w < 4 && !st; ++w) {
      if (gws && w != 3) {  // the grid does not depend on the waves
        p->tune_ms[4 * c + w] = -1.0f;
        continue;
      }
      MeTune t = {c, kTuneWaves[w], p->tune.wait_tries};
      float ms = 0.0f;
      for (int rep = 0; rep < 2 && !st; ++rep) {  // the first launch of a variant is a warm-up
        st = cuda_status(cudaEventRecord(a, S(stream)));
        if (!st && mf_launch_me(p->k, p->prec, prep, n, skip, out, nullptr, p->d_err, t, p->d_ws, S(stream)))
          st = last_launch();
        if (!st) st = cuda_status(cudaEventRecord(b, S(stream)));
        if (!st) st = cuda_status(cudaEventSynchronize(b));
        if (!st) st = cuda_status(cudaEventElapsedTime(&ms, a, b));
      }
      if (st) break;
      p->tune_ms[4 * c + w] = ms;
      if (!have || ms < best) {
        best = ms;
        pick = t;
        have = true;
      }
    }
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (st) return st;
  p->tune = pick;
  p->tuned = true;
  return MF_OK;
}

static int ensure_events(mf_process* p, int64_t N) {
  if (!p->d_err) {
    int st = cuda_status(cudaMalloc(&p->d_err, sizeof(int)));
    if (!st) st = cuda_status(cudaMemset(p->d_err, 0, sizeof(int)));
    if (st) return st;
  }
  if (!p->d_nonfinite) {
    int st = cuda_status(cudaMalloc(&p->d_nonfinite, sizeof(unsigned long long)));
    if (!st) st = cuda_status(cudaMemset(p->d_nonfinite, 0, sizeof(unsigned long long)));
    if (st) return st;
  }
  const int64_t wsb = mf_ws_bytes(p->k, p->prec);
  if (wsb > 0 && !p->d_ws) {
    int st = cuda_status(cudaMalloc(&p->d_ws, (size_t)wsb));
    if (st) return st;
  }
  if (p->event_cap >= N) return MF_OK;
  cudaFree(p->d_prep);
  cudaFree(p->d_state);
  cudaFree(p->d_pref);
  cudaFree(p->d_me);
  cudaFree(p->d_bins);
  p->d_prep = nullptr;
  p->d_state = nullptr;
  p->d_pref = p->d_me = nullptr;
  p->d_bins = nullptr;
  p->event_cap = 0;
  int st = cuda_status(cudaMalloc(&p->d_prep, (size_t)mf_prep_bytes(p->k, p->prec) * N));
  if (!st) st = cuda_status(cudaMalloc(&p->d_state, sizeof(double) * (size_t)mf_state_words(p->k) * N));
  if (!st) st = cuda_status(cudaMalloc(&p->d_pref, sizeof(double) * (size_t)N));
  if (!st) st = cuda_status(cudaMalloc(&p->d_me, sizeof(double) * (size_t)N));
  if (!st) st = cuda_status(cudaMalloc(&p->d_bins, (size_t)MF_MAX_DIM * N));
  if (st) return st;
  p->event_cap = N;
  return MF_OK;
}

// The buffers of one slice (grown to n events, as ensure_events does for
// the handle's own set)
static int ensure_slicebuf(const mf_process* p, SliceBuf& b, int64_t n, bool qq) {
  if (b.cap < n) {
    for (void** q : {(void**)&b.prep, (void**)&b.state, (void**)&b.pref, (void**)&b.me, (void**)&b.bins}) {
      cudaFree(*q);
      *q = nullptr;
    }
    b.cap = 0;
    int st = cuda_status(cudaMalloc(&b.prep, (size_t)mf_prep_bytes(p->k, p->prec) * n));
    if (!st) st = cuda_status(cudaMalloc(&b.state, sizeof(double) * (size_t)mf_state_words(p->k) * n));
    if (!st) st = cuda_status(cudaMalloc(&b.pref, sizeof(double) * (size_t)n));
    if (!st) st = cuda_status(cudaMalloc(&b.me, sizeof(double) * (size_t)n));
    if (!st) st = cuda_status(cudaMalloc(&b.bins, (size_t)MF_MAX_DIM * n));
    if (st) return st;
    b.cap = n;
  }
  if (qq && b.extra_cap < n) {
    cudaFree(b.extra);
    b.extra = nullptr;
    b.extra_cap = 0;
    int st = cuda_status(cudaMalloc(&b.extra, sizeof(double) * (size_t)n));
    if (st) return st;
    b.extra_cap = n;
  }
  if (qq && p->k == 3 && b.qqin_cap < n) {
    cudaFree(b.qqin);
    b.qqin = nullptr;
    b.qqin_cap = 0;
    int st = cuda_status(cudaMalloc(&b.qqin, sizeof(double) * 26 * (size_t)n));
    if (st) return st;
    b.qqin_cap = n;
  }
  if (!b.kmin) {
    int st = cuda_status(cudaMalloc(&b.kmin, sizeof(int)));
    if (st) return st;
  }
  return MF_OK;
}

// the handle's own buffer set as a SliceBuf view
static SliceBuf main_buffers(mf_process* p) {
  SliceBuf b;
  b.prep = p->d_prep;
  b.state = p->d_state;
  b.pref = p->d_pref;
  b.me = p->d_me;
  b.bins = p->d_bins;
  b.extra = p->d_extra;
  b.qqin = p->d_qqin;
  b.kmin = p->d_kmin;
  return b;
}

static void bind_slice(IterArgs& A, const mf_process* p, const SliceBuf& b, int64_t n) {
  A.N = n;
  A.prep = b.prep;
  A.state = b.state;
  A.pref = b.pref;
  A.me = b.me;
  A.extra = A.qq ? b.extra : nullptr;
  A.qqin = A.qq && p->k == 3 ? b.qqin : nullptr;
  A.bins = A.x_in ? nullptr : b.bins;
  A.newton_iters = b.kmin;
}

// The phase-space half of a slice (A bound to its buffers): the first pass
// with the batch Newton minimum of the slice, the second pass with the
// records, and the light-quark channels of p p > t t~ j.
static int slice_phase_space(mf_process* p, IterArgs& A, const mf_integrand_config* c, const SliceBuf& b,
                             bool timed, cudaStream_t st_) {
  const bool per_event = c->newton_rule == MF_NEWTON_PER_EVENT;
  if (timed) cudaEventRecord(p->tev[0], st_);
  set_int_kernel<<<1, 1, 0, st_>>>(b.kmin, per_event ? 0 : 11);
  if (mf_launch_seed(p->k, p->prec, A, b.kmin, per_event ? 0 : 1, st_)) return last_launch();
  if (timed) cudaEventRecord(p->tev[1], st_);
  if (mf_launch_ps(p->k, p->prec, A, st_)) return last_launch();
  if (A.qqin) {
    const int grid = blocks_for(4 * A.N, 128);  // four lanes per event
    if (p->prec == MF_PREC_FP64)
      qq3_channels_kernel<double><<<grid, 128, 0, st_>>>(A);
    else
      qq3_channels_kernel<float><<<grid, 128, 0, st_>>>(A);
  }
  if (timed) cudaEventRecord(p->tev[2], st_);
  return last_launch();
}

// The matrix-element half of a slice: |M|^2 and the accumulation.  results
// (optional) [2 + ndim*nb] (add_results: added to, for the later slices);
// f_out (optional) [n].
static int slice_matrix_element(mf_process* p, IterArgs& A, double* results, int add_results, double* f_out,
                                bool timed, void* stream) {
  const int64_t n = A.N;
  int accum_grid = 8 * 152;
  {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    accum_grid = 8 * (sms > 0 ? sms : 152);
    if (accum_grid > n) accum_grid = (int)n;
  }
  const int width = 2 + A.ndim * A.nb;
  int st = ensure_partials(p, (size_t)accum_grid * width);
  if (st) return st;
  // g g > t t~: |M|^2 came with the phase space (ps_iter_kernel)
  if (p->k != 2) {
    if (autotune_wanted(p, n, stream)) {
      st = autotune_me(p, A.prep, n, A.pref, A.me, stream);
      if (st) return st;
    }
    if (mf_launch_me(p->k, p->prec, A.prep, n, A.pref, A.me, nullptr, p->d_err, p->tune, p->d_ws, S(stream)))
      return last_launch();
  }
  if (timed) cudaEventRecord(p->tev[3], S(stream));
  size_t shm = (size_t)(A.ndim * A.nb + 3 * 256) * sizeof(double);
  static bool attr_done[64] = {false};
  st = smem_attr_once((const void*)accum_kernel, attr_done);
  if (st) return st;
  accum_kernel<<<accum_grid, 256, shm, S(stream)>>>(A.pref, A.me, A.qq ? A.extra : nullptr, A.bins, n, A.ndim,
                                                     A.nb, A.inv_n, f_out,
                                                     results ? p->d_partials : nullptr, p->d_err, p->d_nonfinite);
  if (results)
    reduce_partials_kernel<<<(width + 127) / 128, 128, 0, S(stream)>>>(p->d_partials, accum_grid, width, results,
                                                                       add_results);
  if (timed) cudaEventRecord(p->tev[4], S(stream));
  return last_launch();
}

static int ensure_pipeline(mf_process* p) {
  if (!p->side) {
    int st = cuda_status(cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking));
    if (st) return st;
  }
  for (cudaEvent_t* e : {&p->ev_start, &p->ev_ps[0], &p->ev_ps[1], &p->ev_acc[0], &p->ev_acc[1]})
    if (!*e) {
      int st = cuda_status(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
      if (st) return st;
    }
  return MF_OK;
}

// The pipeline over the A.N events of a call, in consecutive slices of at
// most c->events_limit events (0: one slice), as the reference's integrator
// hands its integrand one slice of events_limit events per call
// (scripts/madflow_exec.py:474-487): the batch Newton rule runs per slice,
// the slices' sums add up in results (in slice order).  The Philox event
// index, x_in, u_out, f_out and ps_out run over the whole call.
// With several slices, two buffer sets alternate: the phase-space passes of
// slice i + 1 run on the handle's side stream while slice i's matrix element
// runs on the caller's stream (events order the two: a slice's matrix
// element waits for its phase space, a buffer's next phase space for the
// accumulation of the slice before).  The scratch then holds two slices.
static int run_fused(mf_process* p, IterArgs& A, const mf_integrand_config* c, double* results, double* f_out,
                     void* stream) {
  if (c->events_limit < 0) return MF_ERR_ARG;
  const int64_t total = A.N;
  const int64_t slice = (c->events_limit > 0 && c->events_limit < total) ? c->events_limit : total;
  const bool piped = slice < total;
  int st = ensure_events(p, slice);
  if (st) return st;
  if (A.qq && p->extra_cap < slice) {
    cudaFree(p->d_extra);
    p->d_extra = nullptr;
    p->extra_cap = 0;
    st = cuda_status(cudaMalloc(&p->d_extra, sizeof(double) * (size_t)slice));
    if (st) return st;
    p->extra_cap = slice;
  }
  if (A.qq && p->k == 3 && p->qqin_cap < slice) {
    cudaFree(p->d_qqin);
    p->d_qqin = nullptr;
    p->qqin_cap = 0;
    st = cuda_status(cudaMalloc(&p->d_qqin, sizeof(double) * 26 * (size_t)slice));
    if (st) return st;
    p->qqin_cap = slice;
  }
  if (!p->d_kmin) {
    st = cuda_status(cudaMalloc(&p->d_kmin, sizeof(int)));
    if (st) return st;
  }
  if (piped) {
    st = ensure_slicebuf(p, p->alt, slice, A.qq != 0);
    if (!st) st = ensure_pipeline(p);
    if (st) return st;
  }
  // stage timing: one slice, and not while the stream is being captured into a graph
  bool timed = false;
  if (p->timing && !piped) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(S(stream), &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone) {
      timed = true;
      for (cudaEvent_t& e : p->tev)
        if (!e && cudaEventCreate(&e) != cudaSuccess) timed = false;
    }
  }
  p->timed_last = timed;
  A.ld = total;
  const int npart = p->k + 2;
  double* ps_out = A.ps_out;
  const SliceBuf bufs[2] = {main_buffers(p), p->alt};
  if (piped) {
    // the side stream starts after the caller's earlier work
    cudaEventRecord(p->ev_start, S(stream));
    cudaStreamWaitEvent(p->side, p->ev_start, 0);
  }
  int i = 0;
  for (int64_t off = 0; off < total; off += slice, ++i) {
    const int64_t n = total - off < slice ? total - off : slice;
    const int b = piped ? (i & 1) : 0;
    IterArgs As = A;
    As.e0 = off;
    As.ps_out = ps_out ? ps_out + off * npart * 4 : nullptr;
    bind_slice(As, p, bufs[b], n);
    if (piped) {
      if (i >= 2) cudaStreamWaitEvent(p->side, p->ev_acc[b], 0);
      st = slice_phase_space(p, As, c, bufs[b], false, p->side);
      if (st) return st;
      cudaEventRecord(p->ev_ps[b], p->side);
      cudaStreamWaitEvent(S(stream), p->ev_ps[b], 0);
      st = slice_matrix_element(p, As, results, off > 0, f_out ? f_out + off : nullptr, false, stream);
      if (st) return st;
      cudaEventRecord(p->ev_acc[b], S(stream));
    } else {
      st = slice_phase_space(p, As, c, bufs[b], timed, S(stream));
      if (!st) st = slice_matrix_element(p, As, results, off > 0, f_out ? f_out + off : nullptr, timed, stream);
      if (st) return st;
    }
  }
  return last_launch();
}

int mf_process_tuning(const mf_process* p, int* colour, int* waves, int* tuned, float* ms) {
  if (!p) return MF_ERR_ARG;
  if (colour) *colour = p->tune.colour;
  if (waves) *waves = p->tune.waves;
  if (tuned) *tuned = p->tuned ? 1 : 0;
  if (ms)
    for (int i = 0; i < MF_TUNE_VARIANTS; ++i) ms[i] = p->tune_ms[i];
  return MF_OK;
}

int mf_process_set_tuning(mf_process* p, int colour, int waves) {
  if (!p || (colour != 0 && colour != 1) || (waves != 1 && waves != 2 && waves != 4 && waves != 8)) return MF_ERR_ARG;
  if (colour == 1 && (p->prec == MF_PREC_FP64 || !mf_colour_tc(p->k))) return MF_ERR_UNSUPPORTED;
  p->tune = {colour, waves, p->tune.wait_tries};
  p->tuned = true;
  return MF_OK;
}

int mf_process_set_wait_limit(mf_process* p, int tries) {
  if (!p || tries < 0 || tries > 100000) return MF_ERR_ARG;
  p->tune.wait_tries = tries;
  return MF_OK;
}

int mf_process_error_flags(mf_process* p, int* flags, int clear) {
  if (!p || !flags) return MF_ERR_ARG;
  *flags = 0;
  if (!p->d_err) return MF_OK;
  int st = cuda_status(cudaMemcpy(flags, p->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (!st && clear) st = cuda_status(cudaMemset(p->d_err, 0, sizeof(int)));
  return st;
}

int mf_process_nonfinite(mf_process* p, int64_t* count, int clear) {
  if (!p || !count) return MF_ERR_ARG;
  *count = 0;
  if (!p->d_nonfinite) return MF_OK;
  unsigned long long c = 0;
  int st = cuda_status(cudaMemcpy(&c, p->d_nonfinite, sizeof(c), cudaMemcpyDeviceToHost));
  if (!st && clear) st = cuda_status(cudaMemset(p->d_nonfinite, 0, sizeof(c)));
  if (st) return st;
  *count = (int64_t)c;
  return c ? MF_ERR_NONFINITE : MF_OK;
}

int mf_process_set_timing(mf_process* p, int enable) {
  if (!p) return MF_ERR_ARG;
  p->timing = enable != 0;
  return MF_OK;
}

int mf_process_stage_ms(const mf_process* p, float* ms) {
  if (!p || !ms) return MF_ERR_ARG;
  if (!p->timed_last) return MF_ERR_STATE;
  for (int i = 0; i < MF_STAGES; ++i) {
    int st = cuda_status(cudaEventElapsedTime(&ms[i], p->tev[i], p->tev[i + 1]));
    if (st) return st;
  }
  return MF_OK;
}

int mf_process_scratch_bytes(const mf_process* p, int64_t* bytes) {
  if (!p || !bytes) return MF_ERR_ARG;
  const int64_t per_event = mf_prep_bytes(p->k, p->prec) + (int64_t)sizeof(double) * (mf_state_words(p->k) + 2) +
                            MF_MAX_DIM;
  int64_t b = p->event_cap * per_event + p->extra_cap * (int64_t)sizeof(double) +
              p->qqin_cap * 26 * (int64_t)sizeof(double) +
              (int64_t)p->partial_cap * (int64_t)sizeof(double);
  if (p->d_ws) b += mf_ws_bytes(p->k, p->prec);
  b += p->alt.cap * per_event + p->alt.extra_cap * (int64_t)sizeof(double) +
       p->alt.qqin_cap * 26 * (int64_t)sizeof(double);
  *bytes = b;
  return MF_OK;
}

int mf_integrand(const mf_process* pc, const mf_integrand_config* c, const double* x, int64_t N, double* f,
                 void* stream) {
  mf_process* p = const_cast<mf_process*>(pc);
  int ndim = 0;
  if (!p || !c || N < 0 || (N > 0 && (!x || !f))) return MF_ERR_ARG;
  int st = mf_integrand_ndim(p, c, &ndim);
  if (st) return st;
  if (N == 0) return MF_OK;
  IterArgs A;
  st = fill_iter_args(p, c, A);
  if (st) return st;
  if (!p->d_zero_iter) {
    st = cuda_status(cudaMalloc(&p->d_zero_iter, sizeof(int)));
    if (st) return st;
    st = cuda_status(cudaMemset(p->d_zero_iter, 0, sizeof(int)));
    if (st) return st;
  }
  A.div = nullptr;
  A.ndim = ndim;
  A.nb = 1;
  A.iteration = p->d_zero_iter;
  A.N = N;
  A.inv_n = 1.0;
  A.x_in = x;
  return run_fused(p, A, c, nullptr, f, stream);
}

// The device address of a caller's buffer: device or managed memory as it
// is, page-locked host memory through its mapping (the kernels then read or
// write it over the host link, zero-copy); other host memory: MF_ERR_ARG.
static int device_view(const void* ptr, void** out) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
    cudaGetLastError();
    return MF_ERR_ARG;
  }
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) {
    *out = const_cast<void*>(ptr);
    return MF_OK;
  }
  if (at.type == cudaMemoryTypeHost) {
    if (at.devicePointer) {
      *out = at.devicePointer;
      return MF_OK;
    }
    return cuda_status(cudaHostGetDevicePointer(out, const_cast<void*>(ptr), 0));
  }
  return MF_ERR_ARG;
}

int mf_integrand_rows(const mf_process* pc, const mf_integrand_config* c, const double* x, int64_t N, double* f,
                      void* stream) {
  mf_process* p = const_cast<mf_process*>(pc);
  int ndim = 0;
  if (!p || !c || N < 0 || (N > 0 && (!x || !f))) return MF_ERR_ARG;
  int st = mf_integrand_ndim(p, c, &ndim);
  if (st) return st;
  if (N == 0) return MF_OK;
  void *xd = nullptr, *fd = nullptr;
  st = device_view(x, &xd);
  if (!st) st = device_view(f, &fd);
  if (st) return st;
  IterArgs A;
  st = fill_iter_args(p, c, A);
  if (st) return st;
  if (!p->d_zero_iter) {
    st = cuda_status(cudaMalloc(&p->d_zero_iter, sizeof(int)));
    if (st) return st;
    st = cuda_status(cudaMemset(p->d_zero_iter, 0, sizeof(int)));
    if (st) return st;
  }
  A.div = nullptr;
  A.ndim = ndim;
  A.nb = 1;
  A.iteration = p->d_zero_iter;
  A.N = N;
  A.inv_n = 1.0;
  A.x_in = static_cast<const double*>(xd);
  A.x_rows = 1;
  return run_fused(p, A, c, nullptr, static_cast<double*>(fd), stream);
}

int mf_vegas_iteration(const mf_process* pc, const mf_integrand_config* c, const double* grid, int nb, uint64_t seed,
                       uint32_t stream_id, const int* iteration, int64_t N, double* results, double* f_out,
                       float* u_out, void* stream) {
  mf_process* p = const_cast<mf_process*>(pc);
  int ndim = 0;
  if (!p || !c || !grid || !iteration || !results || N <= 0 || nb < 2 || nb > 255) return MF_ERR_ARG;
  int st = mf_integrand_ndim(p, c, &ndim);
  if (st) return st;
  if (ndim > MF_MAX_DIM) return MF_ERR_CAPACITY;
  IterArgs A;
  st = fill_iter_args(p, c, A);
  if (st) return st;
  A.div = grid;
  A.ndim = ndim;
  A.nb = nb;
  A.seed = seed;
  A.stream = stream_id;
  A.iteration = iteration;
  A.N = N;
  A.inv_n = 1.0 / (double)N;
  A.u_out = u_out;
  return run_fused(p, A, c, results, f_out, stream);
}

int mf_vegas_events(const mf_process* pc, const mf_integrand_config* c, const double* grid, int nb, uint64_t seed,
                    uint32_t stream_id, int iteration, int64_t N, double* f_out, double* ps_out, void* stream) {
  mf_process* p = const_cast<mf_process*>(pc);
  int ndim = 0;
  if (!p || !c || !grid || !f_out || !ps_out || N <= 0 || nb < 2 || nb > 255 || iteration < 0) return MF_ERR_ARG;
  // an event record names its initial-state flavours: one channel only
  if (c->initial_states != MF_INITIAL_GG) return MF_ERR_UNSUPPORTED;
  int st = mf_integrand_ndim(p, c, &ndim);
  if (st) return st;
  if (ndim > MF_MAX_DIM) return MF_ERR_CAPACITY;
  IterArgs A;
  st = fill_iter_args(p, c, A);
  if (st) return st;
  if (!p->d_event_iter) {
    st = cuda_status(cudaMalloc(&p->d_event_iter, sizeof(int)));
    if (st) return st;
  }
  set_int_kernel<<<1, 1, 0, S(stream)>>>(p->d_event_iter, iteration);
  A.div = grid;
  A.ndim = ndim;
  A.nb = nb;
  A.seed = seed;
  A.stream = stream_id;
  A.iteration = p->d_event_iter;
  A.N = N;
  A.inv_n = 1.0 / (double)N;
  A.ps_out = ps_out;
  return run_fused(p, A, c, nullptr, f_out, stream);
}

// Unweighting (hit or miss): event e is kept when u_e * w_max < |w_e|, u_e a
// Philox uniform of (seed, stream, event).
__global__ void unweight_kernel(const double* __restrict__ w, int64_t N, double wmax, uint64_t seed, uint32_t stream,
                                unsigned char* __restrict__ keep) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    double u0, u1;
    philox_pair(seed, stream, 0xFFFFFFFFu, (uint64_t)e, 0, u0, u1);
    keep[e] = (u0 * wmax < fabs(w[e])) ? 1 : 0;
  }
}

int mf_unweight(const double* w, int64_t N, double w_max, uint64_t seed, uint32_t stream_id, unsigned char* keep,
                void* stream) {
  if (N < 0 || (N > 0 && (!w || !keep)) || !(w_max > 0.0)) return MF_ERR_ARG;
  if (N == 0) return MF_OK;
  int64_t blocks = (N + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  unweight_kernel<<<(int)blocks, 256, 0, S(stream)>>>(w, N, w_max, seed, stream_id, keep);
  return last_launch();
}

// Block partials of mf_vegas_accumulate: one buffer per host thread and
// device (calls of different threads never share one), freed when the thread
// exits.
struct AccumPartials {
  double* part[64] = {nullptr};
  size_t cap[64] = {0};
  ~AccumPartials() {
    for (double* p : part)
      if (p) cudaFree(p);
  }
};

int mf_vegas_accumulate(const double* f, const double* jac, const int32_t* bins, int64_t N, int ndim, int nb,
                        double inv_n, double* results, void* stream) {
  if (!f || !jac || !bins || !results || N <= 0 || ndim <= 0 || nb < 2 || (int64_t)ndim * nb > kAccumMaxBins)
    return MF_ERR_ARG;
  static thread_local AccumPartials P;
  int dev = 0;
  int st = cuda_status(cudaGetDevice(&dev));
  if (st) return st;
  if (dev < 0 || dev >= 64) return MF_ERR_CAPACITY;
  int blocks = 256;
  int width = 2 + ndim * nb;
  size_t need = (size_t)blocks * width;
  if (P.cap[dev] < need) {
    if (P.part[dev]) cudaFree(P.part[dev]);
    P.part[dev] = nullptr;
    P.cap[dev] = 0;
    st = cuda_status(cudaMalloc(&P.part[dev], need * sizeof(double)));
    if (st) return st;
    P.cap[dev] = need;
  }
  static bool attr_done[64] = {false};
  st = smem_attr_once((const void*)vegas_accum_kernel, attr_done);
  if (st) return st;
  size_t shm = (size_t)(ndim * nb + 3 * 256) * sizeof(double);
  vegas_accum_kernel<<<blocks, 256, shm, S(stream)>>>(f, jac, bins, N, ndim, nb, inv_n, P.part[dev]);
  reduce_partials_kernel<<<(width + 127) / 128, 128, 0, S(stream)>>>(P.part[dev], blocks, width, results);
  return last_launch();
}

}  // extern "C"

// ---- VEGAS accumulation without allocation ----------------------------------
// For callers that must not allocate device memory (allocation is banned
// inside their timed or captured region, or their memory is owned by a pool
// manager), the block partials of the accumulation live in this file-scope
// array instead of a cudaMalloc'd buffer.  Every GPU that loads the library
// holds it (MF_NOALLOC_BLOCKS x (2 + MF_NOALLOC_MAX_BINS) doubles, 4.2 MB)
// until the process exits.
constexpr int MF_NOALLOC_BLOCKS = 256;  // same block count as mf_vegas_accumulate
constexpr int MF_NOALLOC_MAX_BINS = 2048;
static __device__ __align__(256) double g_noalloc_partials[MF_NOALLOC_BLOCKS * (2 + MF_NOALLOC_MAX_BINS)];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[64] = {nullptr};
// Device address of the array for the current device.  Host code cannot use
// the symbol itself: on the host, g_noalloc_partials names a host-side
// stand-in, so it is resolved once per device with that device current.
int noalloc_scratch(double** out) {
  int dev = 0;
  int st = cuda_status(cudaGetDevice(&dev));
  if (st) return st;
  if (dev < 0 || dev >= 64) return MF_ERR_CAPACITY;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    st = cuda_status(cudaGetSymbolAddress(&p, g_noalloc_partials));
    if (st) return st;
    g_noalloc_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return MF_OK;
}
}  // namespace

extern "C" {

int mf_vegas_accumulate_noalloc(const double* f, const double* jac, const int32_t* bins, int64_t N, int ndim, int nb,
                                double inv_n, double* results, void* stream) {
  if (!f || !jac || !bins || !results || N <= 0 || ndim <= 0 || nb < 2) return MF_ERR_ARG;
  if ((int64_t)ndim * nb > MF_NOALLOC_MAX_BINS) return MF_ERR_CAPACITY;
  double* part = nullptr;
  int st = noalloc_scratch(&part);
  if (st) return st;
  const int blocks = MF_NOALLOC_BLOCKS;
  const int width = 2 + ndim * nb;
  // every block writes all `width` entries of its row, so the partials left
  // by an earlier call never need clearing
  static bool attr_done[64] = {false};
  st = smem_attr_once((const void*)vegas_accum_kernel, attr_done);
  if (st) return st;
  size_t shm = (size_t)(ndim * nb + 3 * 256) * sizeof(double);
  vegas_accum_kernel<<<blocks, 256, shm, S(stream)>>>(f, jac, bins, N, ndim, nb, inv_n, part);
  reduce_partials_kernel<<<(width + 127) / 128, 128, 0, S(stream)>>>(part, blocks, width, results);
  return last_launch();
}

int mf_vegas_refine(double* grid, const double* hist, int ndim, int nb, double alpha, void* stream) {
  if (!grid || !hist || ndim <= 0 || nb < 2 || nb > 256) return MF_ERR_ARG;
  vegas_refine_kernel<<<(ndim + 31) / 32, 32, 0, S(stream)>>>(grid, hist, ndim, nb, alpha);
  return last_launch();
}

int mf_vegas_sample(const double* grid, int ndim, int nb, const double* u, int64_t N, double* x, double* jac,
                    int32_t* bins, void* stream) {
  if (!grid || ndim <= 0 || nb < 1 || N < 0 || (N > 0 && (!u || !x || !jac || !bins))) return MF_ERR_ARG;
  if (N == 0) return MF_OK;
  vegas_sample_kernel<<<blocks_for(N), 256, 0, S(stream)>>>(grid, ndim, nb, u, N, x, jac, bins);
  return last_launch();
}

int mf_philox_uniforms(uint64_t seed, uint32_t stream_id, uint32_t it, uint64_t e0, int64_t N, int ndim, double* u,
                       void* stream) {
  if (N < 0 || ndim <= 0 || (N > 0 && !u)) return MF_ERR_ARG;
  if (N == 0) return MF_OK;
  philox_kernel<<<blocks_for(N), 256, 0, S(stream)>>>(seed, stream_id, it, e0, N, ndim, u);
  return last_launch();
}

int mf_pdf_xfx_flavour(int pdg, const double* x, int64_t N, double q2, double* out, void* stream) {
  const int f = pdf_flavour_index(pdg);
  if (f < 0 || N < 0 || (N > 0 && (!x || !out))) return MF_ERR_ARG;
  if (N == 0) return MF_OK;
  PdfTable P;
  int st = pdf_device_table(P);
  if (st) return st;
  pdf_flavour_kernel<<<blocks_for(N), 256, 0, S(stream)>>>(P, f, x, N, q2, out);
  return last_launch();
}

int mf_smatrix_qq_ttx(int precision, const double* ps, int64_t N, double mt, double wt, const double* coup,
                      int64_t cstride, double* out, void* stream) {
  (void)wt;  // the s-channel gluon carries no width; kept for the exporter's parameter order
  if ((precision != MF_PREC_FP64 && precision != MF_PREC_MIXED) || N < 0 || (N > 0 && (!ps || !coup || !out)) ||
      (cstride != 0 && cstride != 1))
    return MF_ERR_ARG;
  if (N == 0) return MF_OK;
  qq_ttx_kernel<<<blocks_for(N, 128), 128, 0, S(stream)>>>(precision, ps, N, mt, coup, cstride, out);
  return last_launch();
}

int mf_smatrix_qq_ttxj(int precision, int channel, const double* ps, int64_t N, double mt, double wt,
                       const double* coup, int64_t cstride, double* out, void* stream) {
  if ((precision != MF_PREC_FP64 && precision != MF_PREC_MIXED) || channel < 0 || channel > 2 || N < 0 ||
      (N > 0 && (!ps || !coup || !out)) || (cstride != 0 && cstride != 1))
    return MF_ERR_ARG;
  if (N == 0) return MF_OK;
  if (precision == MF_PREC_FP64)
    qq3_smatrix_kernel<double><<<blocks_for(4 * N, 128), 128, 0, S(stream)>>>(channel, ps, N, mt, wt, coup, cstride,
                                                                               out);
  else
    qq3_smatrix_kernel<float><<<blocks_for(4 * N, 128), 128, 0, S(stream)>>>(channel, ps, N, mt, wt, coup, cstride,
                                                                              out);
  return last_launch();
}

int mf_pdf_xfx(const double* x, int64_t N, double q2, double* out, void* stream) {
  if (N < 0 || (N > 0 && (!x || !out))) return MF_ERR_ARG;
  if (N == 0) return MF_OK;
  PdfTable P;
  int st = pdf_device_table(P);
  if (st) return st;
  pdf_kernel<<<blocks_for(N), 256, 0, S(stream)>>>(P, x, N, q2, out);
  return last_launch();
}

}  // extern "C"
