// Phase space on the device (madflow phasespace.py), FP64, one event per
// thread.  The massive rescaling is split so that madflow's batch-wide Newton
// stopping rule (phasespace.py:84-103) can be reproduced: newton_conv_iter()
// gives the iteration at which an event first meets f0 <= ACC, the batch
// minimum of that is the iteration count every event then runs.
#pragma once
#include "mf_common.cuh"

constexpr int MF_MAX_OUT = 8;

// _gen_unconstrained_momenta (phasespace.py:121-142) + the conformal
// transformation and scaling of rambo (phasespace.py:166-192) for one event.
// p: [n][4]; returns the log-weight before the massive correction.
MF_HD double rambo_massless(const double* x, int n, double sqrts, double pi, double (*p)[4]) {
  double q[MF_MAX_OUT][4];
  double sum[4] = {0, 0, 0, 0};
  for (int i = 0; i < n; ++i) {
    const double* xi = x + 4 * i;
    double costh = 2.0 * xi[0] - 1.0;
    double sinth = sqrt(1.0 - costh * costh);
    double phi = (2.0 * pi) * xi[1];
    double energy = -1.0 * log(xi[2] * xi[3]);
    double sphi, cphi;
    sincos(phi, &sphi, &cphi);
    q[i][0] = energy;
    q[i][1] = energy * sinth * sphi;
    q[i][2] = energy * sinth * cphi;
    q[i][3] = energy * costh;
    for (int k = 0; k < 4; ++k) sum[k] += q[i][k];
  }
  double qmass = sqrt(sum[0] * sum[0] - (sum[1] * sum[1] + sum[2] * sum[2] + sum[3] * sum[3]));
  double xs = sqrts / qmass;
  double b[4];
  for (int k = 0; k < 4; ++k) b[k] = -sum[k] / qmass;
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
  double wt = log(pi / 2.0) * (double)(n - 1);
  wt -= 2.0 * lgamma((double)(n - 1));
  wt -= log((double)(n - 1));
  wt += (double)(2 * n - 4) * log(sqrts);
  return wt;
}

// One Newton step of _massive_xfactor (phasespace.py:77-92).
MF_HD bool newton_step(int n, const double* m2, const double* e2, double sqrts, double acc, double& xf, double* newE) {
  double x2 = xf * xf;
  double f0 = 0.0, g0 = 0.0;
  for (int i = 0; i < n; ++i) {
    newE[i] = sqrt(m2[i] + e2[i] * x2);
    f0 += newE[i];
  }
  f0 = f0 - sqrts;
  for (int i = 0; i < n; ++i) g0 += e2[i] / newE[i];
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

// Massive correction of rambo (phasespace.py:194-212) running `iters` Newton
// iterations (iters <= 0: iterate this event to its own convergence).
// Rescales p in place and returns the final log-weight.
MF_HD double rambo_massive(int n, const double* masses, double (*p)[4], double sqrts, double logw, double acc,
                           int iters) {
  double m2[MF_MAX_OUT], e2[MF_MAX_OUT], newE[MF_MAX_OUT], tm = 0.0;
  for (int i = 0; i < n; ++i) {
    m2[i] = masses[i] * masses[i];
    e2[i] = p[i][0] * p[i][0];
    newE[i] = p[i][0];
    tm += masses[i];
  }
  double r = tm / sqrts;
  double xf = sqrt(1.0 - r * r);
  if (iters > 0) {
    for (int it = 0; it < iters; ++it) newton_step(n, m2, e2, sqrts, acc, xf, newE);
  } else {
    for (int it = 0; it < 10; ++it)
      if (!newton_step(n, m2, e2, sqrts, acc, xf, newE)) break;
  }
  double wt2 = 1.0, wt3 = 0.0;
  for (int i = 0; i < n; ++i) {
    double v = p[i][0] * xf;
    wt2 = wt2 * (v / newE[i]);
    wt3 = wt3 + v * v / newE[i];
    p[i][0] = newE[i];
    p[i][1] *= xf;
    p[i][2] *= xf;
    p[i][3] *= xf;
  }
  return logw + (double)(2 * n - 3) * log(xf) + log(wt2 / wt3 * sqrts);
}

// _get_x1x2 (phasespace.py:215-233)
MF_HD void get_x1x2(double xr0, double xr1, double shat_min, double s_in, double& shat, double& wgt, double& x1,
                    double& x2) {
  double taumin = shat_min / s_in;
  double delta = 1.0 - taumin;
  double tau = xr0 * delta + taumin;
  wgt = delta;
  x1 = pow(tau, xr1);
  x2 = tau / x1;
  wgt = wgt * (-1.0 * log(tau));
  shat = x1 * x2 * s_in;
}

// _boost_to_lab (phasespace.py:322-356) of one momentum
MF_HD void boost_lab(double* q, double x1, double x2) {
  double eta = -0.5 * log(x1 / x2);
  double c = cosh(eta), s = sinh(eta);
  double E = q[0], pz = q[3];
  q[0] = E * c - pz * s;
  q[3] = pz * c - E * s;
}

// Cut decision on the outgoing gluons (particles 4..) in the lab frame: pT,
// |eta| and Delta R between gluon pairs.  A threshold <= 0 disables a cut.
MF_HD bool pass_gluon_cuts(const double (*plab)[4], int npart, double ptmin, double etamax, double drmin) {
  int ng = npart - 4;
  double eta[MF_MAX_OUT], phi[MF_MAX_OUT];
  for (int g = 0; g < ng; ++g) {
    const double* q = plab[4 + g];
    double pt = sqrt(q[1] * q[1] + q[2] * q[2]);
    if (ptmin > 0.0 && !(pt > ptmin)) return false;
    double pabs = sqrt(pt * pt + q[3] * q[3]);
    eta[g] = 0.5 * log((pabs + q[3]) / (pabs - q[3]));
    phi[g] = atan2(q[2], q[1]);
    if (etamax > 0.0 && !(fabs(eta[g]) < etamax)) return false;
  }
  if (drmin > 0.0)
    for (int a = 0; a < ng; ++a)
      for (int b = a + 1; b < ng; ++b) {
        double de = eta[a] - eta[b];
        double dp = phi[a] - phi[b];
        const double pi = 3.141592653589793;
        while (dp > pi) dp -= 2.0 * pi;
        while (dp < -pi) dp += 2.0 * pi;
        if (!(sqrt(de * de + dp * dp) > drmin)) return false;
      }
  return true;
}

// Synthetic gluon PDF x g(x) read back from its (log x, log Q^2) table by
// bicubic convolution (Keys 1981, a = -1/2) with clamped edge nodes.
struct PdfTable {
  const double* tab;  // [nq][nx]
  int nx, nq;
  double lx0, dlx, lq0, dlq;
};
MF_HD double keys_w(double t) {
  t = fabs(t);
  if (t <= 1.0) return (1.5 * t - 2.5) * t * t + 1.0;
  if (t < 2.0) return ((-0.5 * t + 2.5) * t - 4.0) * t + 2.0;
  return 0.0;
}
MF_HD double pdf_xfx(const PdfTable& P, double x, double q2) {
  double u = (log(x) - P.lx0) / P.dlx, v = (log(q2) - P.lq0) / P.dlq;
  int iu = (int)floor(u), iv = (int)floor(v);
  double fu = u - iu, fv = v - iv;
  double s = 0.0;
  for (int a = -1; a <= 2; ++a) {
    int qi = min(max(iv + a, 0), P.nq - 1);
    double wv = keys_w(fv - a);
    for (int b = -1; b <= 2; ++b) {
      int xi = min(max(iu + b, 0), P.nx - 1);
      s += wv * keys_w(fu - b) * P.tab[qi * P.nx + xi];
    }
  }
  return s > 0.0 ? s : 0.0;  // the cubic can overshoot below zero next to x = 1
}
