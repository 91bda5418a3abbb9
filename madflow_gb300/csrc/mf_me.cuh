// Matrix-element kernels for g g > t t~ + (K-2) g, templated on the number of
// gluons K and on the arithmetic type T of the helicity work (double: the
// plain FP64 path; float: the mixed path, whose per-event momenta, propagator
// denominators and sums stay in FP64).
//
// Mapping: one warp per tile of events, the lanes of an event spread over its
// helicities (LPE = min(32, ncomb) lanes per event, ncomb/LPE helicities per
// lane), helicity sum by warp shuffles.  The per-event data every helicity
// needs (subset momenta, propagators) is computed once per event by the lanes
// of that event and kept in shared memory, as is the colour matrix.
#pragma once
#include "mf_helas.cuh"
#include "mf_phasespace.cuh"
#include "mf_vertex.cuh"

constexpr int MF_WARPS = 4;  // warps per block of the matrix-element kernels

template <int K> struct ProcTraits;

// Lane-group geometry for ncomb helicities.
template <int NCOMB> struct Geom {
  static constexpr int LPE = NCOMB < 32 ? NCOMB : 32;  // lanes per event
  static constexpr int EPW = 32 / LPE;                 // events per warp step
  static constexpr int HPL = NCOMB / LPE;              // helicities per lane
};

// Sum over this lane's helicities of the colour-summed |M|^2 (without the
// coupling factor |GC_11|^2 of the amplitudes and without the average).
template <int K, class T>
MF_DO double me_lane(const EvData<T, K>& ev, const T* __restrict__ cm, int lane_in_ev, double* hel_vals) {
  using P = ProcTraits<K>;
  constexpr int NP = P::NPERM;
  using G = Geom<P::NCOMB>;
  const T sqh = (T)0.70710676908493042;  // madflow's float32-rounded sqrt(1/2)
  double acc = 0.0;
#pragma unroll 1
  for (int j = 0; j < G::HPL; ++j) {
    int h = lane_in_ev + G::LPE * j;
    const signed char* hv = P::helicity(h);
    W4<T> g[K];
#pragma unroll
    for (int q = 0; q < K; ++q) {
      int part = gluon_particle<K>(q);
      g[q] = vxxxxx<T>(ev.pext[part], T(0), (T)hv[part], part < 2 ? T(-1) : T(1), sqh);
    }
    W4<T> wt = oxxxxx<T>(ev.pext[2], ev.mt, (T)hv[2], T(1));
    W4<T> wtb = ixxxxx<T>(ev.pext[3], ev.mt, (T)hv[3], T(-1));
    cx<T> A[NP];
    P::template amps<T>(ev, g, wt, wtb, A);
    // colour sum: sum_ij C_ij Re(A_i A_j^*), C symmetric
    T s = T(0);
#pragma unroll 1
    for (int a = 0; a < NP; ++a) {
      cx<T> z = {T(0), T(0)};
      for (int b = a + 1; b < NP; ++b) z += cm[a * NP + b] * A[b];
      T diag = cm[a * NP + a] * (A[a].re * A[a].re + A[a].im * A[a].im);
      s += diag + T(2) * (A[a].re * z.re + A[a].im * z.im);
    }
    double v = (double)s;
    if (hel_vals) hel_vals[j] = v;
    acc += v;
  }
  return acc;
}

// Fill EvData of one event from FP64 momenta pd[npart][4]; the `lanes` lanes
// of the event share the subsets.
template <int K, class T>
MF_DO void evdata_fill(EvData<T, K>& ev, const double (*pd)[4], int lane_in_ev, int lanes, double mt, double wt,
                      cx<double> gc10, cx<double> gc11, cx<double> gc12) {
  for (int s = lane_in_ev; s < (1 << K); s += lanes) evdata_subset<T, K>(ev, s, pd, mt, wt, gc10, gc11, gc12);
  for (int i = lane_in_ev; i < 4 * (K + 2); i += lanes) ev.pext[i / 4][i % 4] = (T)pd[i / 4][i % 4];
  if (lane_in_ev == 0) ev.mt = (T)mt;
}

template <class T> MF_DO T group_sum(T v, int lpe) {
  for (int o = lpe / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Stage the colour matrix (numerators) into shared memory.
template <int K, class T> MF_DO void stage_colour(T* cm) {
  using P = ProcTraits<K>;
  for (int i = threadIdx.x; i < P::NPERM * P::NPERM; i += blockDim.x) cm[i] = (T)P::colour(i);
}

// |M|^2 factor common to all helicities: |amplitude coupling|^2 / (colour denominator x average)
template <int K> MF_DO double me_scale(cx<double> gc11) {
  using P = ProcTraits<K>;
  return (gc11.re * gc11.re + gc11.im * gc11.im) / (P::COLOUR_DEN * P::DENOMINATOR);
}

// Matrix_<proc>.smatrix: ps [npart][4][N] (SoA), couplings [3] complex per
// event (stride 1) or shared (stride 0), out [N]; hel_out [ncomb][N] optional
// (per-helicity |M|^2 before the average, as Matrix_<proc>.matrix returns).
template <int K, class T>
__global__ void __launch_bounds__(32 * MF_WARPS) smatrix_kernel(const double* __restrict__ ps, int64_t N, double mt,
                                                                 double wt, const double* __restrict__ coup,
                                                                 int64_t cstride, double* __restrict__ out,
                                                                 double* __restrict__ hel_out) {
  using P = ProcTraits<K>;
  using G = Geom<P::NCOMB>;
  constexpr int NPART = K + 2;
  __shared__ T cm[P::NPERM * P::NPERM];
  __shared__ EvData<T, K> evs[MF_WARPS][G::EPW];
  __shared__ double pds[MF_WARPS][G::EPW][NPART][4];
  stage_colour<K, T>(cm);
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int grp = lane / G::LPE, lig = lane % G::LPE;
  const int64_t stride = (int64_t)gridDim.x * MF_WARPS * G::EPW;
  for (int64_t base = ((int64_t)blockIdx.x * MF_WARPS + warp) * G::EPW; base < N; base += stride) {
    int64_t e = base + grp;
    bool valid = e < N;
    if (valid)
      for (int i = lig; i < 4 * NPART; i += G::LPE) pds[warp][grp][i / 4][i % 4] = ps[(int64_t)i * N + e];
    __syncwarp();
    cx<double> c10 = {0, 0}, c11 = {0, 0}, c12 = {0, 0};
    if (valid) {
      const double* cp = coup + 6 * cstride * e;
      c10 = {cp[0], cp[1]}; c11 = {cp[2], cp[3]}; c12 = {cp[4], cp[5]};
      evdata_fill<K, T>(evs[warp][grp], pds[warp][grp], lig, G::LPE, mt, wt, c10, c11, c12);
    }
    __syncwarp();
    double hv[G::HPL];
    double part = valid ? me_lane<K, T>(evs[warp][grp], cm, lig, hv) : 0.0;
    double tot = group_sum(part, G::LPE);
    if (valid) {
      double sc = me_scale<K>(c11);
      if (hel_out)
        for (int j = 0; j < G::HPL; ++j)
          hel_out[(int64_t)(lig + G::LPE * j) * N + e] = hv[j] * sc * P::DENOMINATOR;
      if (lig == 0) out[e] = tot * sc;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// One VEGAS iteration, fused: Philox uniforms -> VEGAS map -> phase space ->
// cuts -> PDF luminosity -> |M|^2 -> weight -> per-block sums and bin
// histograms.  The block partials are reduced in a fixed order afterwards, so
// an iteration is bit-reproducible.
// ---------------------------------------------------------------------------
struct IterArgs {
  const double* div;  // VEGAS grid [ndim][nb+1]
  int ndim, nb;
  uint64_t seed;
  uint32_t stream;
  const int* iteration;  // device counter (so a captured graph can be replayed)
  int64_t N;
  double inv_n;
  int kind;  // 0: gg->tt~ at fixed sqrt(s-hat); 1: hadronic ramboflow + PDF + cuts
  double sqrts, mt, wt;
  cx<double> gc10, gc11, gc12;
  double masses[MF_MAX_OUT];
  double shat_min;
  double ptmin, etamax, drmin;
  PdfTable pdf;
  double q2;
  const int* newton_iters;  // device: iterations of the batch Newton rule (<= 0: per event)
  int f32q;
  const double* x_in;  // optional [ndim][N] points (integrand API): no Philox / VEGAS map, jac = 1
  double* f_out;       // optional [N]: jac * f (the integrand times the VEGAS Jacobian)
  double* partials;    // [gridDim][2 + ndim*nb]
  float* u_out;        // optional [ndim][N] uniforms (flow training), unused when null
};

constexpr int MF_MAX_DIM = 32;

// Phase-space part of one event; returns false when it fails the cuts.
// p: [npart][4] FP64 momenta in the partonic c.o.m. frame.
MF_D bool event_phase_space(const IterArgs& A, int npart, const double* x, int newton_iters, double (*p)[4],
                            double& wgt_lum) {
  MfConsts KC = mf_consts(A.f32q != 0);
  int nout = npart - 2;
  double shat, wgt, x1 = 1.0, x2 = 1.0;
  const double* xr = x;
  if (A.kind == 0) {
    shat = A.sqrts * A.sqrts;
    wgt = 1.0;
  } else {
    get_x1x2(x[0], x[1], A.shat_min, A.sqrts * A.sqrts, shat, wgt, x1, x2);
    xr = x + 2;
  }
  double roots = (A.kind == 0) ? A.sqrts : sqrt(shat);
  double logw = rambo_massless(xr, nout, roots, KC.pi, p + 2);
  logw = rambo_massive(nout, A.masses, p + 2, roots, logw, KC.acc, newton_iters);
  double wps = exp(logw) / pow(2.0 * KC.pi, (double)(3 * nout - 4));
  double ein = roots / 2.0;
  p[0][0] = ein; p[0][1] = 0.0; p[0][2] = 0.0; p[0][3] = ein;
  p[1][0] = ein; p[1][1] = 0.0; p[1][2] = 0.0; p[1][3] = -ein;
  if (A.kind == 0) {
    wgt_lum = wps * (KC.gev2pb / (2.0 * shat));
    return true;
  }
  wgt = wgt * wps;
  wgt = wgt * KC.gev2pb;
  wgt = wgt / (2.0 * shat);
  bool ok = true;
  if (A.ptmin > 0.0 || A.etamax > 0.0 || A.drmin > 0.0) {
    double plab[MF_MAX_OUT + 2][4];
    for (int i = 0; i < npart; ++i) {
      for (int c = 0; c < 4; ++c) plab[i][c] = p[i][c];
      boost_lab(plab[i], x1, x2);
    }
    ok = pass_gluon_cuts(plab, npart, A.ptmin, A.etamax, A.drmin);
  }
  double lum = pdf_xfx(A.pdf, x1, A.q2) * pdf_xfx(A.pdf, x2, A.q2) / x1 / x2;
  wgt_lum = wgt * lum;
  return ok;
}

// VEGAS map of one event: x = lo + w*frac (fma), jac = prod w*nb.
MF_D double vegas_map(const double* __restrict__ div, int ndim, int nb, const double* u, double* x,
                      unsigned char* bins) {
  double jac = 1.0;
  for (int d = 0; d < ndim; ++d) {
    double xn = u[d] * (double)nb;
    int i = (int)xn;
    if (i > nb - 1) i = nb - 1;
    double frac = xn - (double)i;
    double lo = div[d * (nb + 1) + i];
    double w = div[d * (nb + 1) + i + 1] - lo;
    x[d] = fma(w, frac, lo);
    jac *= w * (double)nb;
    bins[d] = (unsigned char)i;
  }
  return jac;
}

// Batch Newton rule, first pass: the iteration at which the first event of the
// batch converges (atomicMin into *kmin).
template <int K>
__global__ void __launch_bounds__(256) newton_pass_kernel(IterArgs A, int* kmin) {
  constexpr int NPART = K + 2;
  int local = 11;
  const int it = *A.iteration;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < A.N; e += (int64_t)gridDim.x * blockDim.x) {
    double u[MF_MAX_DIM], x[MF_MAX_DIM];
    unsigned char bins[MF_MAX_DIM];
    if (A.x_in) {
      for (int d = 0; d < A.ndim; ++d) x[d] = A.x_in[(int64_t)d * A.N + e];
    } else {
      for (int d = 0; d < A.ndim; d += 2) philox_pair(A.seed, A.stream, (uint32_t)it, (uint64_t)e, d / 2, u[d], u[d + 1]);
      vegas_map(A.div, A.ndim, A.nb, u, x, bins);
    }
    MfConsts KC = mf_consts(A.f32q != 0);
    double shat, wgt, x1, x2;
    const double* xr = x;
    if (A.kind == 0) shat = A.sqrts * A.sqrts;
    else { get_x1x2(x[0], x[1], A.shat_min, A.sqrts * A.sqrts, shat, wgt, x1, x2); xr = x + 2; }
    double roots = (A.kind == 0) ? A.sqrts : sqrt(shat);
    double p[NPART][4];
    rambo_massless(xr, NPART - 2, roots, KC.pi, p);
    int c = newton_conv_iter(NPART - 2, A.masses, p, roots, KC.acc);
    local = min(local, c);
  }
  for (int o = 16; o > 0; o >>= 1) local = min(local, __shfl_xor_sync(0xffffffffu, local, o));
  if ((threadIdx.x & 31) == 0) atomicMin(kmin, local);
}

template <int K, class T>
__global__ void __launch_bounds__(32 * MF_WARPS) iteration_kernel(IterArgs A) {
  using P = ProcTraits<K>;
  using G = Geom<P::NCOMB>;
  constexpr int NPART = K + 2;
  __shared__ T cm[P::NPERM * P::NPERM];
  __shared__ EvData<T, K> evs[MF_WARPS][G::EPW];
  __shared__ double pds[MF_WARPS][32][NPART][4];
  __shared__ double pref[MF_WARPS][32];
  __shared__ double mes[MF_WARPS][32];
  __shared__ unsigned char bins_s[MF_WARPS][32][MF_MAX_DIM];
  __shared__ unsigned char pass_s[MF_WARPS][32];
  extern __shared__ double hist[];  // [MF_WARPS][ndim*nb]
  stage_colour<K, T>(cm);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nh = A.ndim * A.nb;
  for (int i = threadIdx.x; i < MF_WARPS * nh; i += blockDim.x) hist[i] = 0.0;
  __syncthreads();
  const int it = *A.iteration;
  // the batch rule runs at most 10 iterations (11 = no event converged)
  const int niter_newton = min(*A.newton_iters, 10);
  const double sc = me_scale<K>(A.gc11);
  double s1 = 0.0, s2 = 0.0;
  double* wh = hist + warp * nh;
  const int64_t tstride = (int64_t)gridDim.x * MF_WARPS * 32;
  for (int64_t tile = ((int64_t)blockIdx.x * MF_WARPS + warp) * 32; tile < A.N; tile += tstride) {
    // phase 1: lane <-> event
    {
      int64_t e = tile + lane;
      bool ok = false;
      double pl = 0.0;
      if (e < A.N) {
        double u[MF_MAX_DIM], x[MF_MAX_DIM];
        double jac = 1.0;
        if (A.x_in) {
          for (int d = 0; d < A.ndim; ++d) { x[d] = A.x_in[(int64_t)d * A.N + e]; bins_s[warp][lane][d] = 0; }
        } else {
          for (int d = 0; d < A.ndim; d += 2)
            philox_pair(A.seed, A.stream, (uint32_t)it, (uint64_t)e, d / 2, u[d], u[d + 1]);
          jac = vegas_map(A.div, A.ndim, A.nb, u, x, bins_s[warp][lane]);
          if (A.u_out)
            for (int d = 0; d < A.ndim; ++d) A.u_out[(int64_t)d * A.N + e] = (float)u[d];
        }
        double wl;
        ok = event_phase_space(A, NPART, x, niter_newton, pds[warp][lane], wl);
        pl = jac * wl;
      }
      pref[warp][lane] = pl;
      pass_s[warp][lane] = ok ? 1 : 0;
      mes[warp][lane] = 0.0;
    }
    __syncwarp();
    // phase 2: the warp's lanes across the helicities of each passing event
    const int grp = lane / G::LPE, lig = lane % G::LPE;
    for (int base = 0; base < 32; base += G::EPW) {
      int slot = base + grp;
      bool go = pass_s[warp][slot] != 0;
      if (go) evdata_fill<K, T>(evs[warp][grp], pds[warp][slot], lig, G::LPE, A.mt, A.wt, A.gc10, A.gc11, A.gc12);
      __syncwarp();
      double part = go ? me_lane<K, T>(evs[warp][grp], cm, lig, nullptr) : 0.0;
      double tot = group_sum(part, G::LPE);
      if (go && lig == 0) mes[warp][slot] = tot * sc;
      __syncwarp();
    }
    // phase 3: lane <-> event: weight, sums, histograms (per-dimension lanes,
    // events in order, so the histogram sums are deterministic)
    {
      int64_t e = tile + lane;
      double fw = (e < A.N) ? pref[warp][lane] * mes[warp][lane] : 0.0;
      if (A.f_out && e < A.N) A.f_out[e] = fw;
      fw *= A.inv_n;
      pref[warp][lane] = fw;
      double a = fw, b = fw * fw;
      for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        b += __shfl_xor_sync(0xffffffffu, b, o);
      }
      s1 += a;
      s2 += b;
    }
    __syncwarp();
    if (!A.x_in)
      for (int d = lane; d < A.ndim; d += 32)
        for (int i = 0; i < 32; ++i) {
          double fw = pref[warp][i];
          wh[d * A.nb + bins_s[warp][i][d]] += fw * fw;
        }
    __syncwarp();
  }
  __syncthreads();
  // block partials in fixed order
  double* out = A.partials + (int64_t)blockIdx.x * (2 + nh);
  __shared__ double ws[MF_WARPS][2];
  if (lane == 0) { ws[warp][0] = s1; ws[warp][1] = s2; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t1 = 0.0, t2 = 0.0;
    for (int w = 0; w < MF_WARPS; ++w) { t1 += ws[w][0]; t2 += ws[w][1]; }
    out[0] = t1;
    out[1] = t2;
  }
  for (int i = threadIdx.x; i < nh; i += blockDim.x) {
    double t = 0.0;
    for (int w = 0; w < MF_WARPS; ++w) t += hist[w * nh + i];
    out[2 + i] = t;
  }
}
