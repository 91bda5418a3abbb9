// Phase space on the device (madflow phasespace.py), one event per thread,
// in a precision P: FP64 throughout for the FP64 path; for the mixed path
// the uniforms, the massless momentum generation, x1 x2, the lab boost, the
// cuts and the PDF run in FP32, the conformal transformation, the massive
// rescaling and the weights in FP64.  The massive rescaling is split so that madflow's batch-wide Newton
// stopping rule (phasespace.py:84-103) can be reproduced: newton_conv_iter()
// gives the iteration at which an event first meets f0 <= ACC, the batch
// minimum of that is the iteration count every event then runs.
#pragma once
#include "mf_common.cuh"

constexpr int MF_MAX_OUT = 8;

// Elementary functions for a phase-space precision P (float: the
// single-precision library functions).
MF_HD double ps_log(double x) { return log(x); }
MF_HD float ps_log(float x) { return logf(x); }
MF_HD double ps_sqrt(double x) { return sqrt(x); }
MF_HD float ps_sqrt(float x) { return sqrtf(x); }
MF_HD double ps_exp(double x) { return exp(x); }
MF_HD float ps_exp(float x) { return expf(x); }
MF_HD double ps_pow(double x, double y) { return pow(x, y); }
MF_HD float ps_pow(float x, float y) { return powf(x, y); }
MF_HD double ps_atan2(double y, double x) { return atan2(y, x); }
MF_HD float ps_atan2(float y, float x) { return atan2f(y, x); }
MF_HD double ps_cosh(double x) { return cosh(x); }
MF_HD float ps_cosh(float x) { return coshf(x); }
MF_HD double ps_sinh(double x) { return sinh(x); }
MF_HD float ps_sinh(float x) { return sinhf(x); }
MF_HD void ps_sincos(double x, double* s, double* c) { sincos(x, s, c); }
MF_HD void ps_sincos(float x, float* s, float* c) { sincosf(x, s, c); }
MF_HD double ps_fabs(double x) { return fabs(x); }
MF_HD float ps_fabs(float x) { return fabsf(x); }
MF_HD double ps_floor(double x) { return floor(x); }
MF_HD float ps_floor(float x) { return floorf(x); }

// _gen_unconstrained_momenta (phasespace.py:121-142): n massless momenta q
// [n][4] from 4n uniforms, computed in P and returned in FP64.
template <class P> MF_HD void rambo_generate(const P* x, int n, P pi, double (*q)[4]) {
  for (int i = 0; i < n; ++i) {
    const P* xi = x + 4 * i;
    P costh = P(2) * xi[0] - P(1);
    P sinth = ps_sqrt(P(1) - costh * costh);
    P phi = (P(2) * pi) * xi[1];
    P energy = P(-1) * ps_log(xi[2] * xi[3]);
    P sphi, cphi;
    ps_sincos(phi, &sphi, &cphi);
    q[i][0] = energy;
    q[i][1] = energy * sinth * sphi;
    q[i][2] = energy * sinth * cphi;
    q[i][3] = energy * costh;
  }
}

// The constant part of the massless rambo log-weight (phasespace.py:186-192).
MF_HD double rambo_w0(int n, double pi) {
  double wt = log(pi / 2.0) * (double)(n - 1);
  wt -= 2.0 * lgamma((double)(n - 1));
  wt -= log((double)(n - 1));
  return wt;
}

// Conformal transformation and scaling of rambo (phasespace.py:166-192),
// FP64: p [n][4] from q; returns the log-weight before the massive
// correction (w0 = rambo_w0(n, pi)).
// FAST (the mixed-precision path): one reciprocal of the mass instead of
// five divisions.
template <bool FAST = false>
MF_HD double rambo_conformal(const double (*q)[4], int n, double sqrts, double w0, double (*p)[4]) {
  double sum[4] = {0, 0, 0, 0};
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 4; ++k) sum[k] += q[i][k];
  double qmass = sqrt(sum[0] * sum[0] - (sum[1] * sum[1] + sum[2] * sum[2] + sum[3] * sum[3]));
  double xs, b[4];
  if constexpr (FAST) {
    const double iq = 1.0 / qmass;
    xs = sqrts * iq;
    for (int k = 0; k < 4; ++k) b[k] = -sum[k] * iq;
  } else {
    xs = sqrts / qmass;
    for (int k = 0; k < 4; ++k) b[k] = -sum[k] / qmass;
  }
  double gamma = -b[0];
  double a = 1.0 / (1.0 + gamma);
  for (int i = 0; i < n; ++i) {
    double bq = q[i][1] * b[1] + q[i][2] * b[2] + q[i][3] * b[3];
    double tmp = bq * a + q[i][0];
    p[i][1] = (q[i][1] + b[1] * tmp) * xs;
    p[i][2] = (q[i][2] + b[2] * tmp) * xs;
    p[i][3] = (q[i][3] + b[3] * tmp) * xs;
    p[i][0] = (q[i][0] * gamma + bq) * xs;
  }
  return w0 + (double)(2 * n - 4) * log(sqrts);
}

// rambo without the massive correction (FP64): p [n][4]; returns the
// log-weight before the massive correction.
MF_HD double rambo_massless(const double* x, int n, double sqrts, double pi, double (*p)[4]) {
  double q[MF_MAX_OUT][4];
  rambo_generate<double>(x, n, pi, q);
  return rambo_conformal(q, n, sqrts, rambo_w0(n, pi), p);
}

// One Newton step of _massive_xfactor (phasespace.py:77-92).  FAST (the
// mixed-precision path): a massless particle's energy is |E| x and its
// derivative term E^2 / (|E| x) = |E| / x, so the massless particles cost one
// division together and no square root (e: the energies |E|).
template <bool FAST = false>
MF_HD bool newton_step(int n, const double* m2, const double* e2, double sqrts, double acc, double& xf, double* newE,
                       const double* e = nullptr) {
  double x2 = xf * xf;
  double f0 = 0.0, g0 = 0.0;
  if constexpr (FAST) {
    double el = 0.0;
    for (int i = 0; i < n; ++i) {
      if (m2[i] == 0.0) {
        newE[i] = e[i] * xf;
        el += e[i];
      } else {
        newE[i] = sqrt(m2[i] + e2[i] * x2);
        g0 += e2[i] / newE[i];
      }
      f0 += newE[i];
    }
    f0 = f0 - sqrts;
    g0 += el / xf;
  } else {
    for (int i = 0; i < n; ++i) {
      newE[i] = sqrt(m2[i] + e2[i] * x2);
      f0 += newE[i];
    }
    f0 = f0 - sqrts;
    for (int i = 0; i < n; ++i) g0 += e2[i] / newE[i];
  }
  double nx = xf - f0 / (xf * g0);
  bool unconverged = f0 > acc;
  if (unconverged) xf = nx;
  return unconverged;
}

// Iteration (1..10) at which this event's f0 <= ACC first holds; 11 if never.
// With lim <= 10 the search stops before iteration lim and returns lim when
// the event has not converged by then (callers that only need the batch
// minimum pass the smallest value found so far).
MF_HD int newton_conv_iter(int n, const double* masses, const double (*p)[4], double sqrts, double acc,
                           int lim = 11) {
  double m2[MF_MAX_OUT], e2[MF_MAX_OUT], newE[MF_MAX_OUT], tm = 0.0;
  for (int i = 0; i < n; ++i) { m2[i] = masses[i] * masses[i]; e2[i] = p[i][0] * p[i][0]; tm += masses[i]; }
  double r = tm / sqrts;
  double xf = sqrt(1.0 - r * r);
  const int last = lim - 1 < 10 ? lim - 1 : 10;
  for (int it = 1; it <= last; ++it)
    if (!newton_step(n, m2, e2, sqrts, acc, xf, newE)) return it;
  return lim < 11 ? lim : 11;
}

// newton_conv_iter that also keeps the iterates: xs[j * stride] = x after j
// steps (x_0 the starting value), for j = 0 .. min(steps taken, 9).  The
// steps of an event are those of rambo_massive, so the second pass can
// resume from x_(n-1) instead of repeating n-1 steps.
template <bool FAST = false>
MF_HD int newton_conv_iter_xs(int n, const double* masses, const double (*p)[4], double sqrts, double acc, int lim,
                              double* xs, int64_t stride) {
  double m2[MF_MAX_OUT], e2[MF_MAX_OUT], ea[MF_MAX_OUT], newE[MF_MAX_OUT], tm = 0.0;
  for (int i = 0; i < n; ++i) {
    m2[i] = masses[i] * masses[i];
    e2[i] = p[i][0] * p[i][0];
    ea[i] = fabs(p[i][0]);
    tm += masses[i];
  }
  double r = tm / sqrts;
  double xf = sqrt(1.0 - r * r);
  xs[0] = xf;
  const int last = lim - 1 < 10 ? lim - 1 : 10;
  for (int it = 1; it <= last; ++it) {
    if (!newton_step<FAST>(n, m2, e2, sqrts, acc, xf, newE, ea)) return it;
    if (it <= 9) xs[it * stride] = xf;
  }
  return lim < 11 ? lim : 11;
}

// Massive correction of rambo (phasespace.py:194-212) running `iters` Newton
// iterations (iters <= 0: iterate this event to its own convergence) from
// x_start (< 0: the rule's starting value sqrt(1 - (sum m / sqrts)^2)).
// Rescales p in place and returns the final log-weight.
// The weight products run in W (the momenta, the Newton solve and the logs
// stay FP64).  With W = float (the mixed-precision path) the Newton steps are
// FAST ones.
template <class W = double>
MF_HD double rambo_massive(int n, const double* masses, double (*p)[4], double sqrts, double logw, double acc,
                           int iters, double x_start = -1.0) {
  constexpr bool FAST = sizeof(W) == 4;
  double m2[MF_MAX_OUT], e2[MF_MAX_OUT], ea[MF_MAX_OUT], newE[MF_MAX_OUT], tm = 0.0;
  for (int i = 0; i < n; ++i) {
    m2[i] = masses[i] * masses[i];
    e2[i] = p[i][0] * p[i][0];
    ea[i] = fabs(p[i][0]);
    newE[i] = p[i][0];
    tm += masses[i];
  }
  double r = tm / sqrts;
  double xf = x_start >= 0.0 ? x_start : sqrt(1.0 - r * r);
  if (iters > 0) {
    for (int it = 0; it < iters; ++it) newton_step<FAST>(n, m2, e2, sqrts, acc, xf, newE, ea);
  } else {
    for (int it = 0; it < 10; ++it)
      if (!newton_step<FAST>(n, m2, e2, sqrts, acc, xf, newE, ea)) break;
  }
  W wt2 = W(1), wt3 = W(0);
  for (int i = 0; i < n; ++i) {
    double v = p[i][0] * xf;
    const W vw = (W)v, ew = (W)newE[i];
    wt2 = wt2 * (vw / ew);
    wt3 = wt3 + vw * vw / ew;
    p[i][0] = newE[i];
    p[i][1] *= xf;
    p[i][2] *= xf;
    p[i][3] *= xf;
  }
  // the logs in FP64: the log-weight is exponentiated in FP64
  const double a = (double)(2 * n - 3) * log(xf), b = log((double)(wt2 / wt3) * sqrts);
  return logw + a + b;
}

// _get_x1x2 (phasespace.py:215-233)
template <class P>
MF_HD void get_x1x2(P xr0, P xr1, P shat_min, P s_in, P& shat, P& wgt, P& x1, P& x2) {
  P taumin = shat_min / s_in;
  P delta = P(1) - taumin;
  P tau = xr0 * delta + taumin;
  wgt = delta;
  x1 = ps_pow(tau, xr1);
  x2 = tau / x1;
  wgt = wgt * (P(-1) * ps_log(tau));
  shat = x1 * x2 * s_in;
}

// _boost_to_lab (phasespace.py:322-356) of one momentum
template <class P> MF_HD void boost_lab(P* q, P x1, P x2) {
  P eta = P(-0.5) * ps_log(x1 / x2);
  P c = ps_cosh(eta), s = ps_sinh(eta);
  P E = q[0], pz = q[3];
  q[0] = E * c - pz * s;
  q[3] = pz * c - E * s;
}

// Cut decision on the outgoing gluons (particles 4..) in the lab frame: pT,
// |eta| and Delta R between gluon pairs.  A threshold <= 0 disables a cut.
template <class P> MF_HD bool pass_gluon_cuts(const P (*plab)[4], int npart, P ptmin, P etamax, P drmin) {
  int ng = npart - 4;
  P eta[MF_MAX_OUT], phi[MF_MAX_OUT];
  for (int g = 0; g < ng; ++g) {
    const P* q = plab[4 + g];
    P pt = ps_sqrt(q[1] * q[1] + q[2] * q[2]);
    if (ptmin > P(0) && !(pt > ptmin)) return false;
    P pabs = ps_sqrt(pt * pt + q[3] * q[3]);
    eta[g] = P(0.5) * ps_log((pabs + q[3]) / (pabs - q[3]));
    phi[g] = ps_atan2(q[2], q[1]);
    if (etamax > P(0) && !(ps_fabs(eta[g]) < etamax)) return false;
  }
  if (drmin > P(0))
    for (int a = 0; a < ng; ++a)
      for (int b = a + 1; b < ng; ++b) {
        P de = eta[a] - eta[b];
        P dp = phi[a] - phi[b];
        const P pi = P(3.141592653589793);
        while (dp > pi) dp -= P(2) * pi;
        while (dp < -pi) dp += P(2) * pi;
        if (!(ps_sqrt(de * de + dp * dp) > drmin)) return false;
      }
  return true;
}

// Synthetic gluon PDF x g(x) read back from its (log x, log Q^2) table by
// bicubic convolution (Keys 1981, a = -1/2) with clamped edge nodes.
struct PdfTable {
  const double* tab;  // [MF_PDF_NF][nq][nx], the gluon first
  int nx, nq;
  double lx0, dlx, lq0, dlq;
};
template <class P> MF_HD P keys_w(P t) {
  t = ps_fabs(t);
  if (t <= P(1)) return (P(1.5) * t - P(2.5)) * t * t + P(1);
  if (t < P(2)) return ((P(-0.5) * t + P(2.5)) * t - P(4)) * t + P(2);
  return P(0);
}
// Flavours of the tables: 0 gluon, 1..4 d u s c, 5..8 their antiquarks.
constexpr int MF_PDF_NF = 9;
MF_HD int pdf_flavour_pdg(int f) { return f == 0 ? 21 : (f <= 4 ? f : 4 - f); }
// table index of a PDG code (21, +-1..+-4), -1 for others
MF_HD int pdf_flavour_index(int pdg) {
  if (pdg == 21) return 0;
  if (pdg >= 1 && pdg <= 4) return pdg;
  if (pdg <= -1 && pdg >= -4) return 4 - pdg;
  return -1;
}
// table coordinate of log Q^2 (the same for every event of a batch)
MF_HD double pdf_qcoord(const PdfTable& T, double q2) { return (log(q2) - T.lq0) / T.dlq; }
// alpha_s(Q^2) / alpha_s(M_Z^2) at one loop with five flavours,
// 1 / (1 + alpha_s(M_Z^2) b0 ln(Q^2 / M_Z^2)), b0 = (33 - 2 nf) / (12 pi):
// the running coupling of the dynamical scale, standing in for the PDF set's
// alpha_s(Q^2) (pdfflow's alphasQ2), which the synthetic densities lack
MF_HD double alphas_running_ratio(double alpha_mz, double q2) {
  const double mz = 91.1876, b0 = 23.0 / (12.0 * 3.141592653589793);
  return 1.0 / (1.0 + alpha_mz * b0 * log(q2 / (mz * mz)));
}
// x f(x, Q^2) of table flavour f (0 = gluon) with v = pdf_qcoord(T, q2),
// FP64 (the indices are clamped to the table, so any x, NaN included, reads
// inside it)
MF_HD double pdf_xfx_fv(const PdfTable& T, int f, double x, double v) {
  const double* tab = T.tab + (int64_t)f * T.nq * T.nx;
  double u = (log(x) - T.lx0) / T.dlx;
  int iu = (int)floor(u), iv = (int)floor(v);
  double fu = u - iu, fv = v - iv;
  double wu[4];
  for (int b = -1; b <= 2; ++b) wu[b + 1] = keys_w<double>(fu - b);
  double s = 0.0;
  for (int a = -1; a <= 2; ++a) {
    int qi = min(max(iv + a, 0), T.nq - 1);
    double wv = keys_w<double>(fv - a);
    for (int b = -1; b <= 2; ++b) {
      int xi = min(max(iu + b, 0), T.nx - 1);
      s += wv * wu[b + 1] * tab[qi * T.nx + xi];
    }
  }
  return s > 0.0 ? s : 0.0;  // the cubic can overshoot below zero next to x = 1
}
// The same interpolation split in two, for several flavours at one x: the
// stencil of x (clamped nodes, weights) once, then 16 products per flavour
// in pdf_xfx_fv's order (so the values are the same to the bit).
struct PdfStencil {
  int xi[4], qi[4];
  double wu[4], wv[4];
};
MF_HD PdfStencil pdf_stencil(const PdfTable& T, double x, double v) {
  PdfStencil st;
  const double u = (log(x) - T.lx0) / T.dlx;
  const int iu = (int)floor(u), iv = (int)floor(v);
  const double fu = u - iu, fv = v - iv;
  for (int b = -1; b <= 2; ++b) {
    st.wu[b + 1] = keys_w<double>(fu - b);
    st.xi[b + 1] = min(max(iu + b, 0), T.nx - 1);
  }
  for (int a = -1; a <= 2; ++a) {
    st.wv[a + 1] = keys_w<double>(fv - a);
    st.qi[a + 1] = min(max(iv + a, 0), T.nq - 1);
  }
  return st;
}
MF_HD double pdf_xfx_st(const PdfTable& T, int f, const PdfStencil& st) {
  const double* tab = T.tab + (int64_t)f * T.nq * T.nx;
  double s = 0.0;
  for (int a = 0; a < 4; ++a)
    for (int b = 0; b < 4; ++b) s += st.wv[a] * st.wu[b] * tab[st.qi[a] * T.nx + st.xi[b]];
  return s > 0.0 ? s : 0.0;
}
// the gluon
MF_HD double pdf_xfx_v(const PdfTable& T, double x, double v) { return pdf_xfx_fv(T, 0, x, v); }
MF_HD double pdf_xfx(const PdfTable& T, double x, double q2) { return pdf_xfx_v(T, x, pdf_qcoord(T, q2)); }
// Light-quark luminosity of q q~ > t t~ as madflow sums it: the initial
// states (q, q~) and their mirror images (q~, q), q = d u s c, times 1/(x1 x2)
// (scripts/madflow_exec.py:450-455, utilities.py:25-39)
MF_HD double pdf_qq_luminosity(const PdfTable& T, double x1, double x2, double v) {
  double s = 0.0;
  for (int q = 1; q <= 4; ++q)
    s += pdf_xfx_fv(T, q, x1, v) * pdf_xfx_fv(T, q + 4, x2, v) + pdf_xfx_fv(T, q + 4, x1, v) * pdf_xfx_fv(T, q, x2, v);
  return s / x1 / x2;
}
