// CPU oracle for the madflow hot path.  TEST INFRASTRUCTURE ONLY: the CUDA
// library is compared against it (tests, smoke check, and the CPU-baseline
// leg of the benchmark).  Nothing in the product links it.
//
// Every routine restates madflow's algorithm in plain C++ (double precision
// unless a counting scalar is substituted for R), citing the reference file and
// line it follows.  Paths are relative to the madflow source tree.
//
// Parity status: pinned against golden vectors produced by running madflow's
// own phasespace.py / wavefunctions_flow.py / tests/mockup_debug_me.py
// (tests/golden/make_golden.py).  VEGAS (vegasflow, unpinned dependency) and
// the synthetic PDF have no reference implementation here: they follow the
// published algorithms named at each function.
#pragma once
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <vector>

namespace orc {

// ---------------------------------------------------------------------------
// Scalars.  R = double for evaluation; R = Flop for operation counting.
// ---------------------------------------------------------------------------
struct Flop {
  double v;
  static inline unsigned long long count = 0;
  Flop() : v(0) {}
  Flop(double x) : v(x) {}
};
inline Flop operator+(Flop a, Flop b) { ++Flop::count; return Flop(a.v + b.v); }
inline Flop operator-(Flop a, Flop b) { ++Flop::count; return Flop(a.v - b.v); }
inline Flop operator*(Flop a, Flop b) { ++Flop::count; return Flop(a.v * b.v); }
inline Flop operator/(Flop a, Flop b) { ++Flop::count; return Flop(a.v / b.v); }
inline Flop operator-(Flop a) { return Flop(-a.v); }
inline Flop& operator+=(Flop& a, Flop b) { a = a + b; return a; }
inline Flop& operator-=(Flop& a, Flop b) { a = a - b; return a; }
inline Flop& operator*=(Flop& a, Flop b) { a = a * b; return a; }
inline Flop& operator/=(Flop& a, Flop b) { a = a / b; return a; }
inline bool operator==(Flop a, Flop b) { return a.v == b.v; }
inline bool operator!=(Flop a, Flop b) { return a.v != b.v; }
inline bool operator<(Flop a, Flop b) { return a.v < b.v; }
inline bool operator>(Flop a, Flop b) { return a.v > b.v; }
inline bool operator<=(Flop a, Flop b) { return a.v <= b.v; }
inline bool operator>=(Flop a, Flop b) { return a.v >= b.v; }
inline Flop sqrt(Flop a) { ++Flop::count; return Flop(std::sqrt(a.v)); }
inline Flop log(Flop a) { ++Flop::count; return Flop(std::log(a.v)); }
inline Flop exp(Flop a) { ++Flop::count; return Flop(std::exp(a.v)); }
inline Flop sin(Flop a) { ++Flop::count; return Flop(std::sin(a.v)); }
inline Flop cos(Flop a) { ++Flop::count; return Flop(std::cos(a.v)); }
inline Flop fabs(Flop a) { return Flop(std::fabs(a.v)); }
inline double val(double x) { return x; }
inline double val(Flop x) { return x.v; }
using std::sqrt; using std::log; using std::exp; using std::sin; using std::cos; using std::fabs;

template <class R> inline R rmin(R a, R b) { return (b < a) ? b : a; }
template <class R> inline R rmax(R a, R b) { return (a < b) ? b : a; }
// tf.math.sign semantics: sign(0) = 0
template <class R> inline R tfsign(R y) { return (y > R(0)) ? R(1) : ((y < R(0)) ? R(-1) : R(0)); }

template <class R> struct Cx {
  R re, im;
  Cx() : re(0), im(0) {}
  Cx(R r) : re(r), im(0) {}
  Cx(R r, R i) : re(r), im(i) {}
};
template <class R> inline Cx<R> operator+(Cx<R> a, Cx<R> b) { return {a.re + b.re, a.im + b.im}; }
template <class R> inline Cx<R> operator-(Cx<R> a, Cx<R> b) { return {a.re - b.re, a.im - b.im}; }
template <class R> inline Cx<R> operator-(Cx<R> a) { return {-a.re, -a.im}; }
template <class R> inline Cx<R> operator*(Cx<R> a, Cx<R> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <class R> inline Cx<R> operator*(R s, Cx<R> a) { return {s * a.re, s * a.im}; }
template <class R> inline Cx<R> operator/(Cx<R> a, Cx<R> b) {
  R d = b.re * b.re + b.im * b.im;
  return {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}
template <class R> inline Cx<R>& operator+=(Cx<R>& a, Cx<R> b) { a = a + b; return a; }
template <class R> inline Cx<R> conj(Cx<R> a) { return {a.re, -a.im}; }
template <class R> inline Cx<R> mul_i(Cx<R> a) { return {-a.im, a.re}; }    // i*a
template <class R> inline Cx<R> mul_mi(Cx<R> a) { return {a.im, -a.re}; }   // -i*a

// A HELAS wavefunction: slots 0-1 carry the momentum flow
// [E + i pz, px + i py] (times the in/out sign), slots 2-5 the spinor or
// polarisation vector (wavefunctions_flow.py:72-73,105-106,136-137).
template <class R> struct WF { Cx<R> w[6]; };

// ---------------------------------------------------------------------------
// Constants as madflow sees them.  madflow turns Python floats into tensors
// with float_me (= tf.cast(x, float64)), which goes through float32 first, so
// several "double" constants carry float32 rounding (phasespace.py:16-17,
// wavefunctions_flow.py:10, phasespace.py:316).
// ---------------------------------------------------------------------------
struct RefConsts {
  double pi;      // float_me(np.pi)
  double acc;     // float_me(1e-10)
  double sqh;     // float_me(sqrt(0.5)) computed in float32
  double gev2pb;  // float_me(389379365.6)
};
inline RefConsts ref_consts(bool f32_quirks) {
  if (!f32_quirks) return {M_PI, 1e-10, std::sqrt(0.5), 389379365.6};
  return {(double)(float)M_PI, (double)(float)1e-10, (double)std::sqrt(0.5f), (double)(float)389379365.6};
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  Counter-based: the
// uniforms of an event depend only on (seed, iteration, event, dimension).
// ---------------------------------------------------------------------------
inline void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}
// 53-bit uniform in the open interval (0, 1).
inline double u53(uint32_t hi, uint32_t lo) {
  uint64_t m = (((uint64_t)hi << 32) | lo) >> 11;
  return ((double)m + 0.5) * (1.0 / 9007199254740992.0);
}
// Uniform number `dim` of event `event` in pass `iteration` of stream `stream`.
inline void philox_uniforms(uint64_t seed, uint32_t stream, uint32_t iteration, uint64_t event,
                            int ndim, double* u) {
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32) ^ stream};
  for (int j = 0; 2 * j < ndim; ++j) {
    uint32_t ctr[4] = {(uint32_t)event, (uint32_t)(event >> 32), (uint32_t)j, iteration};
    uint32_t r[4];
    philox4x32_10(ctr, key, r);
    u[2 * j] = u53(r[0], r[1]);
    if (2 * j + 1 < ndim) u[2 * j + 1] = u53(r[2], r[3]);
  }
}

// ---------------------------------------------------------------------------
// Phase space: phasespace.py
// ---------------------------------------------------------------------------
// _gen_unconstrained_momenta, phasespace.py:121-142
template <class R> inline void gen_unconstrained(const R x[4], R pi, R q[4]) {
  R costh = R(2.0) * x[0] - R(1.0);
  R sinth = sqrt(R(1.0) - costh * costh);
  R phi = (R(2.0) * pi) * x[1];
  R energy = R(-1.0) * log(x[2] * x[3]);
  q[0] = energy;
  q[1] = energy * sinth * sin(phi);
  q[2] = energy * sinth * cos(phi);
  q[3] = energy * costh;
}

// _conformal_transformation, phasespace.py:109-118
template <class R> inline void conformal(const R q[4], const R b[4], R p[4]) {
  R gamma = -b[0];
  R a = R(1.0) / (R(1.0) + gamma);
  R bq = q[1] * b[1] + q[2] * b[2] + q[3] * b[3];
  R tmp = bq * a + q[0];
  p[1] = q[1] + b[1] * tmp;
  p[2] = q[2] + b[2] * tmp;
  p[3] = q[3] + b[3] * tmp;
  p[0] = q[0] * gamma + bq;
}

inline double lgamma_d(double x) { return std::lgamma(x); }
inline Flop lgamma_d(Flop x) { ++Flop::count; return Flop(std::lgamma(x.v)); }

// How the massive Newton rescaling decides to stop.
//  kNewtonBatch:   madflow's rule (phasespace.py:84-103): the loop runs while
//                  *every* event of the batch still has f0 > ACC, at most 10
//                  times; each event updates only while its own f0 > ACC, and
//                  the returned energies are those of the last iteration's
//                  *pre-update* x.
//  kNewtonPerEvent: each event iterates to its own convergence (max 10).
enum NewtonRule { kNewtonBatch = 0, kNewtonPerEvent = 1 };

// Massless part of rambo (phasespace.py:145-192) for one event: momenta of
// n particles at sqrt(s) and the log-weight before the massive correction.
template <class R>
inline void rambo_massless_event(const R* x, int n, R sqrts, R pi, R* p /*n*4*/, R* logw) {
  R q[8][4];
  R sum[4] = {R(0), R(0), R(0), R(0)};
  for (int i = 0; i < n; ++i) {
    gen_unconstrained<R>(x + 4 * i, pi, q[i]);
    for (int k = 0; k < 4; ++k) sum[k] += q[i][k];
  }
  R qmass = sqrt(sum[0] * sum[0] - (sum[1] * sum[1] + sum[2] * sum[2] + sum[3] * sum[3]));
  R xs = sqrts / qmass;
  R b[4];
  for (int k = 0; k < 4; ++k) b[k] = -sum[k] / qmass;
  for (int i = 0; i < n; ++i) {
    R pp[4];
    conformal<R>(q[i], b, pp);
    for (int k = 0; k < 4; ++k) p[4 * i + k] = pp[k] * xs;
  }
  R wt = log(pi / R(2.0)) * R((double)(n - 1));
  wt -= R(2.0) * lgamma_d(R((double)(n - 1)));
  wt -= log(R((double)(n - 1)));
  wt += R((double)(2 * n - 4)) * log(sqrts);
  *logw = wt;
}

// One Newton step of _massive_xfactor (phasespace.py:77-92) for one event.
template <class R>
inline void newton_step(int n, const R* m2, const R* e2, R sqrts, R acc, R& xf, R* newE, bool& unconverged) {
  R x2 = xf * xf;
  R f0 = R(0), g0 = R(0);
  for (int i = 0; i < n; ++i) {
    newE[i] = sqrt(m2[i] + e2[i] * x2);
    f0 += newE[i];
  }
  f0 = f0 - sqrts;
  for (int i = 0; i < n; ++i) g0 += e2[i] / newE[i];
  R nx = xf - f0 / (xf * g0);
  unconverged = f0 > acc;
  if (unconverged) xf = nx;
}

// rambo (phasespace.py:145-212) over a batch.  x: [N][4n], sqrts: [N],
// masses: [n] (already as the reference holds them), p: [N][n][4], w: [N].
// Returns the number of Newton iterations taken (0 for massless).
template <class R>
inline int rambo_batch(const R* x, int64_t N, int n, const R* sqrts, const R* masses, bool massive,
                       const RefConsts& K, NewtonRule rule, R* p, R* w) {
  R pi = R(K.pi);
  std::vector<R> logw(N);
  for (int64_t e = 0; e < N; ++e) rambo_massless_event<R>(x + 4 * n * e, n, sqrts[e], pi, p + 4 * n * e, &logw[e]);
  // tf.pow(2*PI, 3n-4)
  R twopi_pow = R(std::pow(val(R(2.0) * pi), (double)(3 * n - 4)));
  if (!massive) {
    for (int64_t e = 0; e < N; ++e) w[e] = exp(logw[e]) / twopi_pow;
    return 0;
  }
  R total_mass = R(0);
  std::vector<R> m2(n);
  for (int i = 0; i < n; ++i) { total_mass += masses[i]; m2[i] = masses[i] * masses[i]; }
  std::vector<R> xf(N), newE((size_t)N * n), e2((size_t)N * n);
  for (int64_t e = 0; e < N; ++e) {
    R r = total_mass / sqrts[e];
    xf[e] = sqrt(R(1) - r * r);
    for (int i = 0; i < n; ++i) { R E = p[4 * (n * e + i)]; e2[n * e + i] = E * E; newE[n * e + i] = E; }
  }
  R acc = R(K.acc);
  int iters = 0;
  if (rule == kNewtonBatch) {
    for (int it = 0; it < 10; ++it) {
      bool all_unconv = true;
      for (int64_t e = 0; e < N; ++e) {
        bool u;
        newton_step<R>(n, m2.data(), &e2[n * e], sqrts[e], acc, xf[e], &newE[n * e], u);
        all_unconv = all_unconv && u;
      }
      ++iters;
      if (!all_unconv) break;
    }
  } else {
    for (int64_t e = 0; e < N; ++e) {
      for (int it = 0; it < 10; ++it) {
        bool u;
        newton_step<R>(n, m2.data(), &e2[n * e], sqrts[e], acc, xf[e], &newE[n * e], u);
        if (!u) break;
      }
    }
    iters = -1;
  }
  // rescale (phasespace.py:197-212)
  for (int64_t e = 0; e < N; ++e) {
    R wt2 = R(1), wt3 = R(0);
    for (int i = 0; i < n; ++i) {
      R* pi4 = p + 4 * (n * e + i);
      R v = pi4[0] * xf[e];
      R nE = newE[n * e + i];
      wt2 = wt2 * (v / nE);
      wt3 = wt3 + v * v / nE;
      pi4[0] = nE;
      pi4[1] = pi4[1] * xf[e];
      pi4[2] = pi4[2] * xf[e];
      pi4[3] = pi4[3] * xf[e];
    }
    R lw = logw[e] + R((double)(2 * n - 3)) * log(xf[e]) + log(wt2 / wt3 * sqrts[e]);
    w[e] = exp(lw) / twopi_pow;
  }
  return iters;
}

// _get_x1x2 (phasespace.py:215-233)
template <class R> inline void get_x1x2(const R xr[2], R shat_min, R s_in, R& shat, R& wgt, R& x1, R& x2) {
  R taumin = shat_min / s_in;
  R delta = R(1.0) - taumin;
  R tau = xr[0] * delta + taumin;
  wgt = delta;
  x1 = R(std::pow(val(tau), val(xr[1])));
  x2 = tau / x1;
  wgt = wgt * (R(-1.0) * log(tau));
  shat = x1 * x2 * s_in;
}

// _boost_to_lab (phasespace.py:322-356), in place on [n][4]
template <class R> inline void boost_to_lab(R* p, int n, R x1, R x2) {
  R eta = R(-0.5) * log(x1 / x2);
  R cth = R(std::cosh(val(eta))), sth = R(std::sinh(val(eta)));
  for (int i = 0; i < n; ++i) {
    R E = p[4 * i], pz = p[4 * i + 3];
    p[4 * i] = E * cth - pz * sth;
    p[4 * i + 3] = pz * cth - E * sth;
  }
}

// ---------------------------------------------------------------------------
// External wavefunctions: wavefunctions_flow.py
// ---------------------------------------------------------------------------
// _ox_massive_pp_zero (wavefunctions_flow.py:370-392)
template <class R> inline void ox_massive_pp_zero(R fmass, R nsf, int ip, int im, Cx<R>* v) {
  R s0 = sqrt(fabs(fmass));
  R sqm[2] = {s0, s0 * tfsign(fmass)};
  v[0] = Cx<R>(R((double)im) * sqm[std::abs(im)]);
  v[1] = Cx<R>(R((double)ip) * nsf * sqm[std::abs(im)]);
  v[2] = Cx<R>(R((double)im) * nsf * sqm[std::abs(ip)]);
  v[3] = Cx<R>(R((double)ip) * sqm[std::abs(ip)]);
}
// float floor-division helper: (a) // 2 for the +-1/0 values used here
inline int fdiv2(double a) { return (int)std::floor(a / 2.0); }

// ixxxxx (wavefunctions_flow.py:56-85, 159-330)
template <class R> inline void ixxxxx(const R p[4], R fmass, R nhel, R nsf, WF<R>& f) {
  f.w[0] = Cx<R>(-p[0] * nsf, -p[3] * nsf);
  f.w[1] = Cx<R>(-p[1] * nsf, -p[2] * nsf);
  R nh = nhel * nsf;
  Cx<R>* v = f.w + 2;
  if (fmass != R(0)) {
    R pp = rmin(p[0], sqrt(p[1] * p[1] + p[2] * p[2] + p[3] * p[3]));
    int ip = fdiv2(1 + val(nh)), im = fdiv2(1 - val(nh));
    if (pp == R(0)) { ox_massive_pp_zero<R>(fmass, nsf, im, ip, v); return; }
    R sf0 = (R(1) + nsf + (R(1) - nsf) * nh) * R(0.5);
    R sf1 = (R(1) + nsf - (R(1) - nsf) * nh) * R(0.5);
    R om[2] = {sqrt(p[0] + pp), fmass / sqrt(p[0] + pp)};
    R sfo0 = sf0 * om[ip], sfo1 = sf1 * om[im];
    R pp3 = rmax(pp + p[3], R(0));
    Cx<R> chi1 = (pp3 == R(0)) ? Cx<R>(-nh, R(0))
                               : Cx<R>(nh * p[1] / sqrt(R(2.0) * pp * pp3), p[2] / sqrt(R(2.0) * pp * pp3));
    Cx<R> chi[2] = {Cx<R>(sqrt(pp3 * R(0.5) / pp)), chi1};
    v[0] = sfo0 * chi[im]; v[1] = sfo0 * chi[ip];
    v[2] = sfo1 * chi[im]; v[3] = sfo1 * chi[ip];
    return;
  }
  R sq = sqrt(rmax(p[0] + p[3], R(0))) * nsf;
  Cx<R> chi1 = (sq == R(0)) ? Cx<R>(-nhel * sqrt(R(2.0) * p[0]), R(0)) : Cx<R>(nh * p[1] / sq, p[2] / sq);
  Cx<R> chi0(sq, R(0));
  if (nh == R(1)) { v[0] = Cx<R>(); v[1] = Cx<R>(); v[2] = chi0; v[3] = chi1; }
  else { v[0] = chi1; v[1] = chi0; v[2] = Cx<R>(); v[3] = Cx<R>(); }
}

// oxxxxx (wavefunctions_flow.py:89-116, 336-462)
template <class R> inline void oxxxxx(const R p[4], R fmass, R nhel, R nsf, WF<R>& f) {
  f.w[0] = Cx<R>(p[0] * nsf, p[3] * nsf);
  f.w[1] = Cx<R>(p[1] * nsf, p[2] * nsf);
  R nh = nhel * nsf;
  Cx<R>* v = f.w + 2;
  if (fmass != R(0)) {
    R pp = rmin(p[0], sqrt(p[1] * p[1] + p[2] * p[2] + p[3] * p[3]));
    if (pp == R(0)) {
      int ipz = (int)(-(double)fdiv2(1 - val(nh)) * val(nhel));
      int imz = (int)((double)fdiv2(1 + val(nh)) * val(nhel));
      ox_massive_pp_zero<R>(fmass, nsf, ipz, imz, v);
      return;
    }
    R sf0 = (R(1) + nsf + (R(1) - nsf) * nh) * R(0.5);
    R sf1 = (R(1) + nsf - (R(1) - nsf) * nh) * R(0.5);
    R om[2] = {sqrt(p[0] + pp), fmass / sqrt(p[0] + pp)};
    int ip = fdiv2(1 + val(nh)), im = fdiv2(1 - val(nh));
    R sfo0 = sf0 * om[ip], sfo1 = sf1 * om[im];
    R pp3 = rmax(pp + p[3], R(0));
    Cx<R> chi1 = (pp3 == R(0)) ? Cx<R>(-nh, R(0))
                               : Cx<R>(nh * p[1] / sqrt(R(2.0) * pp * pp3), -p[2] / sqrt(R(2.0) * pp * pp3));
    Cx<R> chi[2] = {Cx<R>(sqrt(pp3 * R(0.5) / pp)), chi1};
    v[0] = sfo1 * chi[im]; v[1] = sfo1 * chi[ip];
    v[2] = sfo0 * chi[im]; v[3] = sfo0 * chi[ip];
    return;
  }
  R sq = sqrt(rmax(p[0] + p[3], R(0))) * nsf;
  Cx<R> chi0 = (sq == R(0)) ? Cx<R>(-nhel * sqrt(R(2.0) * p[0]), R(0)) : Cx<R>(nh * p[1] / sq, -p[2] / sq);
  Cx<R> csq(sq, R(0));
  if (nh == R(1)) { v[0] = csq; v[1] = chi0; v[2] = Cx<R>(); v[3] = Cx<R>(); }
  else { v[0] = Cx<R>(); v[1] = Cx<R>(); v[2] = chi0; v[3] = csq; }
}

// vxxxxx (wavefunctions_flow.py:120-154, 469-747)
template <class R> inline void vxxxxx(const R p[4], R vmass, R nhel, R nsv, R sqh, WF<R>& f) {
  f.w[0] = Cx<R>(p[0] * nsv, p[3] * nsv);
  f.w[1] = Cx<R>(p[1] * nsv, p[2] * nsv);
  Cx<R>* v = f.w + 2;
  R pt2 = p[1] * p[1] + p[2] * p[2];
  R pp = rmin(p[0], sqrt(pt2 + p[3] * p[3]));
  R pt = rmin(pp, sqrt(pt2));
  R hel0 = R(1) - fabs(nhel);
  R nsvahl = nsv * fabs(nhel);
  if (nhel == R(4)) {  // BRST check: polarisation replaced by the momentum
    R d = (vmass == R(0)) ? p[0] : vmass;
    for (int k = 0; k < 4; ++k) v[k] = Cx<R>(p[k] / d);
    return;
  }
  if (vmass != R(0)) {
    if (pp == R(0)) {
      v[0] = Cx<R>(R(1)); v[1] = Cx<R>(-nhel * sqh); v[2] = Cx<R>(R(0), nsvahl * sqh); v[3] = Cx<R>(hel0);
      return;
    }
    R emp = p[0] / (vmass * pp);
    v[0] = Cx<R>(hel0 * pp / vmass);
    v[3] = Cx<R>(hel0 * p[3] * emp + nhel * pt / pp * sqh);
    if (pt != R(0)) {
      R pzpt = p[3] / (pp * pt) * sqh * nhel;
      v[1] = Cx<R>(hel0 * p[1] * emp - p[1] * pzpt, -nsvahl * p[2] / pt * sqh);
      v[2] = Cx<R>(hel0 * p[2] * emp - p[2] * pzpt, nsvahl * p[1] / pt * sqh);
    } else {
      v[1] = Cx<R>(-nhel * sqh);
      v[2] = Cx<R>(R(0), nsvahl * (sqh * tfsign(p[3])));
    }
    return;
  }
  R ppl = p[0];
  R ptl = sqrt(p[1] * p[1] + p[2] * p[2]);
  v[0] = Cx<R>();
  v[3] = Cx<R>(nhel * ptl / ppl * sqh);
  if (ptl != R(0)) {
    R pzpt = p[3] / (ppl * ptl) * sqh * nhel;
    v[1] = Cx<R>(-p[1] * pzpt, -nsv * p[2] / ptl * sqh);
    v[2] = Cx<R>(-p[2] * pzpt, nsv * p[1] / ptl * sqh);
  } else {
    v[1] = Cx<R>(-nhel * sqh);
    v[2] = Cx<R>(R(0), nsv * (sqh * tfsign(p[3])));
  }
}

// sxxxxx (wavefunctions_flow.py:34-51): three slots, the last one = 1
template <class R> inline void sxxxxx(const R p[4], R nss, Cx<R> s[3]) {
  s[0] = Cx<R>(p[0] * nss, p[3] * nss);
  s[1] = Cx<R>(p[1] * nss, p[2] * nss);
  s[2] = Cx<R>(R(1));
}

// ---------------------------------------------------------------------------
// ALOHA routines of tests/mockup_debug_me.py, restated from the Dirac algebra.
// In the HELAS chiral basis the bilinear F1^T S(a) F2 uses
//   S(a) = [[0, a+], [a-, 0]],  a+ = [[a0+a3, a1+i a2], [a1-i a2, a0-a3]],
//                               a- = [[a0-a3, -(a1+i a2)], [-a1+i a2, a0+a3]].
// ---------------------------------------------------------------------------
template <class R> inline void mom_of(const WF<R>& f, R P[4]) {
  P[0] = f.w[0].re; P[1] = f.w[1].re; P[2] = f.w[1].im; P[3] = f.w[0].im;
}
template <class R> inline void blocks(const Cx<R> a[4], Cx<R> ap[2][2], Cx<R> am[2][2]) {
  Cx<R> a12p = a[1] + mul_i(a[2]), a12m = a[1] - mul_i(a[2]);
  ap[0][0] = a[0] + a[3]; ap[0][1] = a12p; ap[1][0] = a12m; ap[1][1] = a[0] - a[3];
  am[0][0] = a[0] - a[3]; am[0][1] = -a12p; am[1][0] = -a12m; am[1][1] = a[0] + a[3];
}
// y = S(a) x  (column action)
template <class R> inline void s_apply(const Cx<R> a[4], const Cx<R> x[4], Cx<R> y[4]) {
  Cx<R> ap[2][2], am[2][2];
  blocks<R>(a, ap, am);
  y[0] = ap[0][0] * x[2] + ap[0][1] * x[3];
  y[1] = ap[1][0] * x[2] + ap[1][1] * x[3];
  y[2] = am[0][0] * x[0] + am[0][1] * x[1];
  y[3] = am[1][0] * x[0] + am[1][1] * x[1];
}
// y = S(a)^T x
template <class R> inline void s_apply_t(const Cx<R> a[4], const Cx<R> x[4], Cx<R> y[4]) {
  Cx<R> ap[2][2], am[2][2];
  blocks<R>(a, ap, am);
  y[0] = am[0][0] * x[2] + am[1][0] * x[3];
  y[1] = am[0][1] * x[2] + am[1][1] * x[3];
  y[2] = ap[0][0] * x[0] + ap[1][0] * x[1];
  y[3] = ap[0][1] * x[0] + ap[1][1] * x[1];
}
template <class R> inline Cx<R> prop_denom(Cx<R> coup, const R P[4], R M, R W) {
  R p2 = P[0] * P[0] - P[1] * P[1] - P[2] * P[2] - P[3] * P[3];
  // P^2 - M (M - i W)
  Cx<R> d(p2 - M * M, M * W);
  return coup / d;
}

// FFV1_0 (mockup_debug_me.py:43-54): COUP * (-i) * F1^T S(V3) F2
template <class R> inline Cx<R> FFV1_0(const WF<R>& F1, const WF<R>& F2, const WF<R>& V3, Cx<R> coup) {
  Cx<R> y[4];
  s_apply<R>(V3.w + 2, F2.w + 2, y);
  Cx<R> t = F1.w[2] * y[0] + F1.w[3] * y[1] + F1.w[4] * y[2] + F1.w[5] * y[3];
  return coup * mul_mi(t);
}
// FFV1_1 (mockup_debug_me.py:67-194): F1 = i*denom*(S(-P1)+M1) S(V3) F2, P1 = -(p_F2 + p_V3)
template <class R> inline void FFV1_1(const WF<R>& F2, const WF<R>& V3, Cx<R> coup, R M1, R W1, WF<R>& F1) {
  F1.w[0] = F2.w[0] + V3.w[0];
  F1.w[1] = F2.w[1] + V3.w[1];
  R P[4];
  mom_of<R>(F1, P);
  for (int k = 0; k < 4; ++k) P[k] = -P[k];
  Cx<R> den = prop_denom<R>(coup, P, M1, W1);
  Cx<R> y[4], z[4], mp[4];
  s_apply<R>(V3.w + 2, F2.w + 2, y);
  for (int k = 0; k < 4; ++k) mp[k] = Cx<R>(-P[k]);
  s_apply<R>(mp, y, z);
  Cx<R> c = mul_i(den);
  for (int k = 0; k < 4; ++k) F1.w[2 + k] = c * (z[k] + M1 * y[k]);
}
// FFV1_2 (mockup_debug_me.py:207-328): F2 = i*denom*(S(P2)+M2)^T S(V3)^T F1, P2 = -(p_F1 + p_V3)
template <class R> inline void FFV1_2(const WF<R>& F1, const WF<R>& V3, Cx<R> coup, R M2, R W2, WF<R>& F2) {
  F2.w[0] = F1.w[0] + V3.w[0];
  F2.w[1] = F1.w[1] + V3.w[1];
  R P[4];
  mom_of<R>(F2, P);
  for (int k = 0; k < 4; ++k) P[k] = -P[k];
  Cx<R> den = prop_denom<R>(coup, P, M2, W2);
  Cx<R> y[4], z[4], pp[4];
  s_apply_t<R>(V3.w + 2, F1.w + 2, y);
  for (int k = 0; k < 4; ++k) pp[k] = Cx<R>(P[k]);
  s_apply_t<R>(pp, y, z);
  Cx<R> c = mul_i(den);
  for (int k = 0; k < 4; ++k) F2.w[2 + k] = c * (z[k] + M2 * y[k]);
}
template <class R> inline Cx<R> mdot(const Cx<R>* a, const Cx<R>* b) {
  return a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
}
template <class R> inline Cx<R> mdotr(const Cx<R>* a, const R* b) {
  return b[0] * a[0] - b[1] * a[1] - b[2] * a[2] - b[3] * a[3];
}
// VVV1P0_1 (mockup_debug_me.py:341-397): off-shell gluon of the triple-gluon
// vertex, V1 = i*denom*[(V2.V3)(P3-P2) + V2 (V3.P2 - V3.P1) + V3 (V2.P1 - V2.P3)]
template <class R> inline void VVV1P0_1(const WF<R>& V2, const WF<R>& V3, Cx<R> coup, R M1, R W1, WF<R>& V1) {
  R P2[4], P3[4], P1[4];
  mom_of<R>(V2, P2);
  mom_of<R>(V3, P3);
  V1.w[0] = V2.w[0] + V3.w[0];
  V1.w[1] = V2.w[1] + V3.w[1];
  mom_of<R>(V1, P1);
  for (int k = 0; k < 4; ++k) P1[k] = -P1[k];
  const Cx<R>* a = V2.w + 2;
  const Cx<R>* b = V3.w + 2;
  Cx<R> v23 = mdot<R>(b, a);
  Cx<R> c2 = mdotr<R>(b, P2) - mdotr<R>(b, P1);
  Cx<R> c3 = mdotr<R>(a, P1) - mdotr<R>(a, P3);
  Cx<R> den = prop_denom<R>(coup, P1, M1, W1);
  Cx<R> c = mul_i(den);
  for (int k = 0; k < 4; ++k) V1.w[2 + k] = c * (v23 * Cx<R>(P3[k] - P2[k]) + a[k] * c2 + b[k] * c3);
}
// Off-shell vector from a fermion pair (the ALOHA routine MadGraph names
// FFV1P0_3; no instance in the reference's mock-up, restated from the same
// Dirac algebra): with c_mu = F1^T S(e_mu) F2, so that F1^T S(V) F2 =
// sum_mu c_mu V^mu, V3^mu = i denom g^{mu mu} c_mu, P3 = -(p_F1 + p_F2).
template <class R> inline void FFV1P0_3(const WF<R>& F1, const WF<R>& F2, Cx<R> coup, R M3, R W3, WF<R>& V3) {
  V3.w[0] = F1.w[0] + F2.w[0];
  V3.w[1] = F1.w[1] + F2.w[1];
  R P3[4];
  mom_of<R>(V3, P3);
  for (int k = 0; k < 4; ++k) P3[k] = -P3[k];
  Cx<R> den = prop_denom<R>(coup, P3, M3, W3);
  Cx<R> c = mul_i(den);
  for (int mu = 0; mu < 4; ++mu) {
    Cx<R> e[4];
    e[mu] = Cx<R>(R(1));
    Cx<R> y[4];
    s_apply<R>(e, F2.w + 2, y);
    Cx<R> cm = F1.w[2] * y[0] + F1.w[3] * y[1] + F1.w[4] * y[2] + F1.w[5] * y[3];
    V3.w[2 + mu] = c * (mu == 0 ? cm : -cm);
  }
}

// Colour-ordered four-gluon contact current (no reference instance exists:
// derived from the QCD Feynman rules).  For the cyclic order (1,2,3,4) the
// colour-ordered vertex is proportional to 2 g13 g24 - g12 g34 - g14 g23, so
// with leg 1 off-shell
//   V1 = i*denom*[2 V3 (V2.V4) - V2 (V3.V4) - V4 (V2.V3)],  P1 = -(p2+p3+p4).
template <class R>
inline void VVVV_ord_1(const WF<R>& V2, const WF<R>& V3, const WF<R>& V4, Cx<R> coup, WF<R>& V1) {
  V1.w[0] = V2.w[0] + V3.w[0] + V4.w[0];
  V1.w[1] = V2.w[1] + V3.w[1] + V4.w[1];
  R P1[4];
  mom_of<R>(V1, P1);
  for (int k = 0; k < 4; ++k) P1[k] = -P1[k];
  const Cx<R>* a = V2.w + 2;
  const Cx<R>* b = V3.w + 2;
  const Cx<R>* d = V4.w + 2;
  Cx<R> ad = mdot<R>(a, d), bd = mdot<R>(b, d), ab = mdot<R>(a, b);
  Cx<R> den = prop_denom<R>(coup, P1, R(0), R(0));
  Cx<R> c = mul_i(den);
  Cx<R> two(R(2.0));
  for (int k = 0; k < 4; ++k) V1.w[2 + k] = c * (two * b[k] * ad - a[k] * bd - d[k] * ab);
}

}  // namespace orc
