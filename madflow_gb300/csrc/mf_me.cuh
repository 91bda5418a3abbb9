// One VEGAS iteration of the g g > t t~ + (K-2) g integrand as a pipeline of
// persistent kernels over all N events of the iteration:
//
//   ps_seed_kernel      one thread per event, FP64: Philox uniforms -> VEGAS
//                       grid map (bin indices) -> x1, x2 -> massless rambo;
//                       stores that state and takes the first pass of
//                       madflow's batch Newton rule (the batch minimum of
//                       the iteration at which an event converges)
//   ps_iter_kernel      one thread per event, FP64: massive rambo correction
//                       with the batch iteration count -> lab boost -> cuts
//                       -> PDF; writes the prefactor jac * weight *
//                       luminosity (0 for events failing the cuts) and the
//                       matrix-element record of every passing event
//   me_rec_kernel       one thread block per passing event: |M|^2 summed over
//                       helicities and colours (mf_me_rec.cuh)
//   accum_kernel        w = prefactor * |M|^2 / N; fixed-order block sums of
//                       w, w^2 and the per-bin w^2
//   reduce_partials     fixed-order sum of the block partials
//
// so that an iteration is bit-reproducible.
#pragma once
#include "../../include/madflow_gb300.h"
#include "mf_me_rec.cuh"
#include "mf_qq.cuh"
#include "mf_qq3.cuh"
#include "mf_gg2.cuh"

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
  double ptmin_all;  // > 0: p_T > ptmin_all for every outgoing particle (madflow's --pt_cut)
  int ncuts;         // registered cuts (mf_cut), thresholds already held through float32
  mf_cut cuts[MF_MAX_CUTS];
  PdfTable pdf;
  double q2;
  int dyn;        // dynamical scale: mu_F = mu_R = sum of the outgoing m_T / 2 per event
  double alpha0;  // with dyn: alpha_s(M_Z^2), the start of the running
  const int* newton_iters;  // device: iterations of the batch Newton rule (<= 0: per event)
  int f32q;
  const double* x_in;  // optional points (integrand API): no Philox / VEGAS map, jac = 1;
                       // [ndim][ld], or [ld][ndim] (rows, madflow's xrand) with x_rows
  int x_rows;
  float* u_out;        // optional [ndim][ld] uniforms
  int64_t e0, ld;      // the slice's first event in the call (Philox event index, x_in / u_out column)
                       // and the call's event count (x_in / u_out row length)
  double* ps_out;      // optional [N][K+2][4] lab-frame momenta of the passing events (event output)
  int qq;              // p p > t t~ (K = 2) or p p > t t~ j (K = 3): add the light-quark channels
  double* extra;       // [N] with qq: their weight, jac x weight x luminosity x |M|^2 summed
  double* qqin;        // [26][N] with qq and K = 3: the event's momenta [5][4] (partonic frame) and
                       // its weight times each channel evaluation's luminosity (qq3_weighted_sum's
                       // order; all 0: the event failed the cuts)
  // pipeline buffers (scratch)
  double* state;            // [4K+16][N] first-pass state (ps_state_words)
  int4* prep;              // [N] per-event records (PrepRec), passing events only
  double* pref;            // [N]
  unsigned char* bins;     // [ndim][N]
  double* me;              // [N]
};

constexpr int MF_MAX_DIM = 32;

// Per-event state of the first pass, stored SoA [ps_state_words][N]: the
// massless rambo momenta of the K outgoing particles [K][4], its log-weight,
// s-hat, the x1 x2 weight, x1, x2, the VEGAS jacobian and (batch Newton
// rule) the Newton iterates x_0 .. x_9.
template <int K> MF_HD constexpr int ps_state_words() { return 4 * K + 16; }

// Uniforms of dimensions 2j, 2j+1 of an event: 53-bit in FP64, 24-bit in
// FP32 (the high words of the same Philox4x32-10 block, so an FP32 uniform
// is the FP64 one rounded down to 24 bits, plus half an FP32 step).
MF_HD float u24(uint32_t hi) { return ((float)(hi >> 8) + 0.5f) * (1.0f / 16777216.0f); }
template <class P> MF_HD void uniform_pair(uint64_t seed, uint32_t stream, uint32_t it, uint64_t e, uint32_t j, P& u0,
                                           P& u1);
template <> MF_HD void uniform_pair<double>(uint64_t seed, uint32_t stream, uint32_t it, uint64_t e, uint32_t j,
                                            double& u0, double& u1) {
  philox_pair(seed, stream, it, e, j, u0, u1);
}
template <> MF_HD void uniform_pair<float>(uint64_t seed, uint32_t stream, uint32_t it, uint64_t e, uint32_t j,
                                           float& u0, float& u1) {
  uint32_t c[4] = {(uint32_t)e, (uint32_t)(e >> 32), j, it};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32) ^ stream);
  u0 = u24(c[0]);
  u1 = u24(c[2]);
}

// VEGAS map of one event: x = lo + w*frac (fma), jac = prod w*nb; div is
// the grid [ndim][nb+1] in P.
template <class P>
MF_DO P vegas_map(const P* __restrict__ div, int ndim, int nb, const P* u, P* x, unsigned char* bins, int64_t N) {
  P jac = P(1);
  for (int d = 0; d < ndim; ++d) {
    P xn = u[d] * (P)nb;
    int i = (int)xn;
    if (i > nb - 1) i = nb - 1;
    P frac = xn - (P)i;
    P lo = div[d * (nb + 1) + i];
    P w = div[d * (nb + 1) + i + 1] - lo;
    x[d] = fma(w, frac, lo);
    jac *= w * (P)nb;
    if (bins) bins[(int64_t)d * N] = (unsigned char)i;
  }
  return jac;
}

// The point of event e of the slice: the caller's x (integrand API, jac = 1) or Philox
// uniforms through the VEGAS grid (sdiv: the grid in P).
template <class P>
MF_DO void event_point(const IterArgs& A, int64_t e, int it, const P* sdiv, P* x, P& jac, bool store) {
  const int64_t g = A.e0 + e;  // the event's index in the call
  if (A.x_in) {
    if (A.x_rows)
      for (int d = 0; d < A.ndim; ++d) x[d] = (P)A.x_in[g * A.ndim + d];
    else
      for (int d = 0; d < A.ndim; ++d) x[d] = (P)A.x_in[(int64_t)d * A.ld + g];
    jac = P(1);
    return;
  }
  P u[MF_MAX_DIM];
  for (int d = 0; d < A.ndim; d += 2) uniform_pair<P>(A.seed, A.stream, (uint32_t)it, (uint64_t)g, d / 2, u[d], u[d + 1]);
  jac = vegas_map<P>(sdiv, A.ndim, A.nb, u, x, store ? A.bins + e : nullptr, A.N);
  if (store && A.u_out)
    for (int d = 0; d < A.ndim; ++d) A.u_out[(int64_t)d * A.ld + g] = (float)u[d];
}

// First part of the phase space of one event (phasespace.py:257-300 up to
// the massive correction).  p: [npart][4]; w0 = rambo_w0(npart - 2, pi).
template <class P>
MF_DO void event_massless(const IterArgs& A, int npart, const P* x, double w0, double (*p)[4], double& logw,
                          double& shat, double& wgt, double& x1, double& x2) {
  MfConsts KC = mf_consts(A.f32q != 0);
  x1 = 1.0;
  x2 = 1.0;
  const P* xr = x;
  if (A.kind == 0) {
    shat = A.sqrts * A.sqrts;
    wgt = 1.0;
  } else {
    // x1, x2, s-hat and the x1 x2 weight in FP64 for either precision: the
    // PDF's (1 - x)^5 falls steeply towards x = 1, where the FP32 rounding
    // of x1 = tau^u1 showed up as 1e-3 of the weight
    get_x1x2<double>((double)x[0], (double)x[1], A.shat_min, A.sqrts * A.sqrts, shat, wgt, x1, x2);
    xr = x + 2;
  }
  double roots = (A.kind == 0) ? A.sqrts : sqrt(shat);
  double q[MF_MAX_OUT][4];
  rambo_generate<P>(xr, npart - 2, (P)KC.pi, q);
  logw = rambo_conformal<sizeof(P) == 4>(q, npart - 2, roots, w0, p + 2);
}

// Rest of the phase space of one event: massive correction with
// newton_iters iterations (<= 0: per event), incoming momenta, flux, lab
// boost, cuts and luminosity.  v: the PDF table coordinate of Q^2 (DYN: set
// to the event's own); pw: (2 pi)^(3 nout - 4).  Returns false when the
// event fails the cuts.
// The event weight (the exponentiated log-weight, flux, luminosity) is FP64
// for either precision P: exp of an FP32 log-weight of 30 to 50 alone erred
// by 2e-6; the cuts are decided in P.
template <class P, bool DYN = false>
MF_DO bool event_finish(const IterArgs& A, int npart, int newton_iters, double (*p)[4], double logw, double shat,
                        double wgt, double x1, double x2, double& v, double pw, double& wgt_lum,
                        double x_start = -1.0, double* wgt_ps = nullptr, double* as_ratio = nullptr) {
  MfConsts KC = mf_consts(A.f32q != 0);
  int nout = npart - 2;
  double roots = (A.kind == 0) ? A.sqrts : sqrt(shat);
  logw = rambo_massive<P>(nout, A.masses, p + 2, roots, logw, KC.acc, newton_iters, x_start);
  double wps = exp(logw) / pw;
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
  if (wgt_ps) *wgt_ps = wgt;  // the weight before the luminosity
  bool ok = true;
  if (A.ptmin_all > 0.0) {
    // madflow's --pt_cut on every outgoing particle, decided in FP64 on the
    // partonic-frame momenta, as PhaseSpaceGenerator cuts before its boost
    // (p_x, p_y are the lab frame's)
    for (int i = 2; i < npart; ++i) ok = ok && sqrt(p[i][1] * p[i][1] + p[i][2] * p[i][2]) > A.ptmin_all;
  }
  if (ok && (A.ptmin > 0.0 || A.etamax > 0.0 || A.drmin > 0.0)) {
    P plab[MF_MAX_OUT + 2][4];
    for (int i = 0; i < npart; ++i) {
      for (int c = 0; c < 4; ++c) plab[i][c] = (P)p[i][c];
      boost_lab<P>(plab[i], (P)x1, (P)x2);
    }
    ok = pass_gluon_cuts<P>(plab, npart, (P)A.ptmin, (P)A.etamax, (P)A.drmin);
  }
  if constexpr (DYN) {
    // madflow's default scale (scripts/madflow_exec.py:428-431): mu^2 =
    // (sum over the outgoing particles of m_T / 2)^2, m_T^2 = p.p + p_T^2
    // (phasespace.py:406-415; invariant under the boost to the lab frame);
    // the densities at mu^2 and alpha_s(mu^2) / alpha_s(M_Z^2) from one-loop
    // running with five flavours
    double smt = 0.0;
    for (int i = 2; i < npart; ++i) {
      const double m2 = p[i][0] * p[i][0] - p[i][1] * p[i][1] - p[i][2] * p[i][2] - p[i][3] * p[i][3];
      const double pt = sqrt(p[i][1] * p[i][1] + p[i][2] * p[i][2]);
      smt += sqrt(m2 + pt * pt);
    }
    const double q2e = (smt / 2.0) * (smt / 2.0);
    v = pdf_qcoord(A.pdf, q2e);
    if (as_ratio) *as_ratio = alphas_running_ratio(A.alpha0, q2e);
  }
  const double lum = pdf_xfx_v(A.pdf, x1, v) * pdf_xfx_v(A.pdf, x2, v) / x1 / x2;
  wgt_lum = wgt * lum;
  return ok;
}

// The registered cuts (mf_cut), in FP64 on the partonic-frame momenta
// p [NPART][4] (madflow's PhaseSpaceGenerator cuts before its boost,
// phasespace.py:458-466), in the reference's operation order (_fourdot; mt2 =
// p.p + pt^2 with pt a square root).  Compile-time indices throughout, so
// the cut table and the momenta stay out of local memory.
template <int NPART> MF_DO bool pass_cut_table(const IterArgs& A, const double (*p)[4]) {
#pragma unroll
  for (int c = 0; c < MF_MAX_CUTS; ++c) {
    if (c >= A.ncuts) break;
    const mf_cut C = A.cuts[c];
    double q[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int i = 0; i < NPART; ++i)
      if (i == C.particle) {
#pragma unroll
        for (int j = 0; j < 4; ++j) q[j] = p[i][j];
      }
    const double pt = sqrt(q[1] * q[1] + q[2] * q[2]);
    double val = pt;
    if (C.variable == MF_CUT_MT || C.variable == MF_CUT_MT2) {
      const double mt2 = (q[0] * q[0] - ((q[1] * q[1] + q[2] * q[2]) + q[3] * q[3])) + pt * pt;
      val = C.variable == MF_CUT_MT ? sqrt(mt2) : mt2;
    } else if (C.variable == MF_CUT_ETA) {
      const double pabs = sqrt((q[1] * q[1] + q[2] * q[2]) + q[3] * q[3]);
      val = 0.5 * log((pabs + q[3]) / (pabs - q[3]));
    }
    if (C.has_min && !(val > C.min_val)) return false;
    if (C.has_max && !(val < C.max_val)) return false;
  }
  return true;
}

// First pass: the phase-space state of every event and, when batch_rule is
// set, the batch minimum of the Newton convergence iteration (atomicMin into
// *kmin, which starts at 11).  An event only needs to be followed up to the
// smallest iteration seen so far, read from *kmin as it goes.  Dynamic
// shared memory: the VEGAS grid in P.
template <int K, class P> __global__ void __launch_bounds__(256) ps_seed_kernel(IterArgs A, int* kmin, int batch_rule) {
  constexpr int NPART = K + 2;
  extern __shared__ __align__(16) unsigned char seed_smem[];
  P* sdiv = reinterpret_cast<P*>(seed_smem);
  if (!A.x_in)
    for (int i = threadIdx.x; i < A.ndim * (A.nb + 1); i += blockDim.x) sdiv[i] = (P)A.div[i];
  __syncthreads();
  const int it = *A.iteration;
  const int64_t N = A.N;
  const MfConsts KC = mf_consts(A.f32q != 0);
  const double w0 = rambo_w0(K, KC.pi);
  int local = 11;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    P x[MF_MAX_DIM], jacp;
    double p[NPART][4], logw, shat, wgt, x1, x2;
    event_point<P>(A, e, it, sdiv, x, jacp, true);
    event_massless<P>(A, NPART, x, w0, p, logw, shat, wgt, x1, x2);
    double* st = A.state + e;
#pragma unroll
    for (int i = 0; i < K; ++i)
#pragma unroll
      for (int c = 0; c < 4; ++c) st[(int64_t)(4 * i + c) * N] = p[i + 2][c];
    st[(int64_t)(4 * K) * N] = logw;
    st[(int64_t)(4 * K + 1) * N] = shat;
    st[(int64_t)(4 * K + 2) * N] = wgt;
    st[(int64_t)(4 * K + 3) * N] = x1;
    st[(int64_t)(4 * K + 4) * N] = x2;
    st[(int64_t)(4 * K + 5) * N] = (double)jacp;
    // a non-finite event (e.g. from non-finite caller points) takes no part
    // in the batch minimum: its f0 > ACC test is false at once, which would
    // otherwise stop the Newton iteration of the whole batch
    double chk = logw + shat;
#pragma unroll
    for (int i = 0; i < K; ++i) chk += p[i + 2][0];
    if (batch_rule && isfinite(chk)) {
      const int lim = min(local, *(volatile int*)kmin);
      const double roots = (A.kind == 0) ? A.sqrts : sqrt(shat);
      const int c = newton_conv_iter_xs<sizeof(P) == 4>(K, A.masses, p + 2, roots, KC.acc, lim,
                                                         st + (int64_t)(4 * K + 6) * N, N);
      if (c < lim) {
        local = c;
        atomicMin(kmin, c);
      }
    }
  }
}

// Second pass: the rest of the phase space of every event (phase-space
// precision = the matrix-element precision T), and the per-event record of
// the matrix element for the events that pass.
template <int K, class T, bool DYN> __global__ void __launch_bounds__(128) ps_iter_kernel(IterArgs A) {
  constexpr int NPART = K + 2;
  constexpr int NW = prep_words<T, K>();
  const int64_t N = A.N;
  // the batch rule runs at most 10 iterations (11 = no event converged)
  const int niter = min(*A.newton_iters, 10);
  const MfConsts KC = mf_consts(A.f32q != 0);
  const double v = DYN ? 0.0 : pdf_qcoord(A.pdf, A.q2);
  const double pw = pow(2.0 * KC.pi, (double)(3 * K - 4));
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    double p[NPART][4], wl;
    const double* st = A.state + e;
#pragma unroll
    for (int i = 0; i < K; ++i)
#pragma unroll
      for (int c = 0; c < 4; ++c) p[i + 2][c] = st[(int64_t)(4 * i + c) * N];
    const double logw = st[(int64_t)(4 * K) * N], shat = st[(int64_t)(4 * K + 1) * N];
    const double wgt = st[(int64_t)(4 * K + 2) * N], x1 = st[(int64_t)(4 * K + 3) * N];
    const double x2 = st[(int64_t)(4 * K + 4) * N], jac = st[(int64_t)(4 * K + 5) * N];
    // batch rule: one step from the first pass's x_(niter-1) (the steps
    // before it are the ones the first pass took)
    const double xs = niter > 0 ? st[(int64_t)(4 * K + 6 + niter - 1) * N] : -1.0;
    double wps = 0.0, ve = v, asr = 1.0;
    bool ok = event_finish<T, DYN>(A, NPART, niter > 0 ? 1 : niter, p, logw, shat, wgt, x1, x2, ve, pw, wl, xs, &wps,
                                   &asr);
    ok = ok && pass_cut_table<NPART>(A, p);
    // the event's coupling: every tree diagram of these processes (g g > t t~
    // + (K-2) g, and the light-quark channels of p p > t t~ (j)) has K strong
    // vertices, so |M|^2 at alpha_s(mu^2) is |M|^2 at alpha_s(M_Z^2) times
    // (alpha_s(mu^2) / alpha_s(M_Z^2))^K: the per-event couplings of madflow's
    // model.evaluate(alpha_s) (scripts/madflow_exec.py:431, 446) as one factor
    double cs = 1.0;
    if constexpr (DYN)
      for (int j = 0; j < K; ++j) cs *= asr;
    A.pref[e] = ok ? jac * wl * cs : 0.0;
    if constexpr (K == 2) {
      // the light-quark channels of p p > t t~, one thread per event (two
      // orders of magnitude cheaper than the block-per-event gluon channel)
      if (A.qq) {
        double ex = 0.0;
        if (ok) {
          const double g11sq = A.gc11.re * A.gc11.re + A.gc11.im * A.gc11.im;
          ex = jac * wps * pdf_qq_luminosity(A.pdf, x1, x2, ve) * uux_ttx_me<T>(p, A.mt, g11sq) * cs;
        }
        A.extra[e] = ex;
      }
    }
    if constexpr (K == 3) {
      // the light-quark channels of p p > t t~ j: their inputs, for
      // qq3_channels_kernel
      if (A.qq) {
        double* q = A.qqin + e;
#pragma unroll
        for (int i = 0; i < 5; ++i)
#pragma unroll
          for (int c = 0; c < 4; ++c) q[(int64_t)(4 * i + c) * N] = p[i][c];
        double lw[6] = {0, 0, 0, 0, 0, 0};
        if (ok) {
          // the densities at x1 and x2 from one interpolation stencil each
          const PdfStencil s1 = pdf_stencil(A.pdf, x1, ve), s2 = pdf_stencil(A.pdf, x2, ve);
          double qq = 0.0, qbq = 0.0, Q1 = 0.0, Qb1 = 0.0, Q2 = 0.0, Qb2 = 0.0;
          for (int f = 1; f <= 4; ++f) {
            const double a = pdf_xfx_st(A.pdf, f, s1), ab = pdf_xfx_st(A.pdf, f + 4, s1);
            const double b = pdf_xfx_st(A.pdf, f, s2), bb = pdf_xfx_st(A.pdf, f + 4, s2);
            qq += a * bb;
            qbq += ab * b;
            Q1 += a;
            Qb1 += ab;
            Q2 += b;
            Qb2 += bb;
          }
          const double g1 = pdf_xfx_st(A.pdf, 0, s1), g2 = pdf_xfx_st(A.pdf, 0, s2);
          const double c = jac * wps / x1 / x2 * cs;
          // qq3_weighted_sum's order: q q~, q~ q, q g, q~ g, g q, g q~
          lw[0] = c * qq;
          lw[1] = c * qbq;
          lw[2] = c * (Q1 * g2);
          lw[3] = c * (Qb1 * g2);
          lw[4] = c * (g1 * Q2);
          lw[5] = c * (g1 * Qb2);
        }
#pragma unroll
        for (int j = 0; j < 6; ++j) q[(int64_t)(20 + j) * N] = lw[j];
      }
    }
    if (A.ps_out) {
      // madflow's all_ps (com_output=False): lab frame, FP64
      double* q = A.ps_out + (int64_t)e * NPART * 4;
      for (int i = 0; i < NPART; ++i) {
        double t[4] = {p[i][0], p[i][1], p[i][2], p[i][3]};
        if (A.kind != 0) boost_lab<double>(t, x1, x2);
        for (int c = 0; c < 4; ++c) q[4 * i + c] = ok ? t[c] : 0.0;
      }
    }
    if constexpr (K == 2) {
      // g g > t t~: |M|^2 here, one thread per event, instead of a record
      // for a matrix-element kernel
      A.me[e] = ok ? gg2_me<T>(p, A.mt, A.wt, A.gc10, A.gc11, (T)KC.sqh) : 0.0;
    } else if (ok) {
      PrepRec<T, K> r;
      prep_event<T, K>(r, p, A.mt, A.wt, A.gc10, A.gc11, A.gc12);
      const int4* src = reinterpret_cast<const int4*>(&r);
      int4* dst = A.prep + e * NW;
      for (int w = 0; w < NW; ++w) dst[w] = src[w];
    }
  }
}

// The light-quark channels of p p > t t~ j, a group of four lanes per event
// (madflow sums the processes of a run, each over its initial states and
// their mirror images, scripts/madflow_exec.py:444-458, utilities.py:25-39):
//   extra = w / (x1 x2) [ |M|^2(q q~ > t t~ g)(p1, p2) sum_q q(x1) q~(x2)
//                        + |M|^2(q q~ > t t~ g)(p2, p1) sum_q q~(x1) q(x2)
//                        + |M|^2(q g > t t~ q)(p1, p2) Q(x1) g(x2) + mirror
//                        + |M|^2(q~ g > t t~ q~)(p1, p2) Qb(x1) g(x2) + mirror ]
// Q, Qb the sums of x f over q = d u s c and their antiquarks.
template <class T> __global__ void __launch_bounds__(128) qq3_channels_kernel(IterArgs A) {
  const int64_t N = A.N;
  const int lane = threadIdx.x & 3, base = (threadIdx.x & 31) & ~3;
  const unsigned mask = 0xFu << base;
  const T sqh = (T)mf_consts(A.f32q != 0).sqh;
  const int64_t stride = (int64_t)gridDim.x * (blockDim.x >> 2);
  for (int64_t e = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 2; e < N; e += stride) {
    const double* q = A.qqin + e;
    double lw[6];
    bool any = false;
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      lw[j] = q[(int64_t)(20 + j) * N];
      any = any || lw[j] != 0.0;
    }
    double ex = 0.0;
    if (any) {
      double p[5][4];
#pragma unroll
      for (int i = 0; i < 5; ++i)
#pragma unroll
        for (int c = 0; c < 4; ++c) p[i][c] = q[(int64_t)(4 * i + c) * N];
      ex = qq3_weighted_sum<T>(p, lw, A.mt, A.wt, A.gc10, A.gc11, sqh, mask, lane, base);
    }
    if (lane == 0) A.extra[e] = ex;
  }
}

// The weight f = pref * me of an event; a non-finite f (NaN or +-inf from a
// non-finite input point or matrix element) is replaced by 0.
MF_DO double finite_weight(double f) { return isfinite(f) ? f : 0.0; }

// w = (pref * me + extra) * inv_n (extra optional: further channels of the
// same events); block b owns a contiguous slice of events.  f_out
// (optional) = pref * me + extra.  partials [gridDim][2 + ndim*nb].  Non-finite
// weights are counted into *nonfinite (bit 1 of *err set) and enter the sums,
// the histogram and f_out as 0.
static __global__ void __launch_bounds__(256) accum_kernel(const double* __restrict__ pref, const double* __restrict__ me,
                                                    const double* __restrict__ extra,
                                                    const unsigned char* __restrict__ bins, int64_t N, int ndim,
                                                    int nb, double inv_n, double* __restrict__ f_out,
                                                    double* __restrict__ partials, int* __restrict__ err,
                                                    unsigned long long* __restrict__ nonfinite) {
  extern __shared__ double sh[];  // [ndim*nb] + [2*blockDim] + [blockDim]
  double* hist = sh;
  double* red = sh + ndim * nb;
  const int width = 2 + ndim * nb;
  int64_t per = (N + gridDim.x - 1) / gridDim.x;
  int64_t e0 = (int64_t)blockIdx.x * per, e1 = min(N, e0 + per);
  for (int i = threadIdx.x; i < ndim * nb; i += blockDim.x) hist[i] = 0.0;
  double a = 0.0, b = 0.0;
  unsigned int bad = 0;
  for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    const double f0 = pref[e] * me[e] + (extra ? extra[e] : 0.0);
    const double f = finite_weight(f0);
    bad += f0 != f;
    if (f_out) f_out[e] = f;
    double w = f * inv_n;
    a += w;
    b += w * w;
  }
  if (bad) {
    if (nonfinite) atomicAdd(nonfinite, (unsigned long long)bad);
    if (err) atomicOr(err, 2);
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
  if (bins) {
    // per-bin sums of w^2 in event order, one thread per dimension; w^2 of a
    // chunk of blockDim events is formed once by all threads
    double* w2 = red + 2 * blockDim.x;
    for (int64_t c0 = e0; c0 < e1; c0 += blockDim.x) {
      const int64_t e = c0 + threadIdx.x;
      if (e < e1) {
        const double w = finite_weight(pref[e] * me[e] + (extra ? extra[e] : 0.0)) * inv_n;
        w2[threadIdx.x] = w * w;
      }
      __syncthreads();
      const int cn = (int)min((int64_t)blockDim.x, e1 - c0);
      for (int d = threadIdx.x; d < ndim; d += blockDim.x) {
        const unsigned char* bd = bins + (int64_t)d * N + c0;
        double* hd = hist + d * nb;
        for (int j = 0; j < cn; ++j) hd[bd[j]] += w2[j];
      }
      __syncthreads();
    }
  }
  __syncthreads();
  if (partials) {
    double* out = partials + (int64_t)blockIdx.x * width;
    if (threadIdx.x == 0) { out[0] = red[0]; out[1] = red[blockDim.x]; }
    for (int i = threadIdx.x; i < ndim * nb; i += blockDim.x) out[2 + i] = bins ? hist[i] : 0.0;
  }
}
