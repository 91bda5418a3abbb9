// Vertex algebra of the colour-ordered recursion, restated from the ALOHA
// routines madflow runs (tests/mockup_debug_me.py: FFV1_0 :43, FFV1_1 :67,
// FFV1_2 :207, VVV1P0_1 :341) plus the four-gluon contact term, which has no
// instance in the reference and follows the QCD Feynman rules.
//
// The momentum flow of a current is kept per subset of external legs (the
// "slot" momentum Q: +p for outgoing, -p for incoming), so the propagator
// factor of every subset is computed once per event (the momenta and
// invariants in FP64, or in double-float for the FP32 path) instead of once
// per current and helicity.  In the HELAS chiral basis the vertex bilinear is
// F1^T S(V) F2 with S(a) = [[0, a+], [a-, 0]],
//   a+ = [[a0+a3, a1+i a2], [a1-i a2, a0-a3]],
//   a- = [[a0-a3, -(a1+i a2)], [-a1+i a2, a0+a3]].
#pragma once
#include "mf_common.cuh"

template <class T> MF_D cx<T> mdot(const W4<T>& a, const W4<T>& b) {
  return a.v[0] * b.v[0] - a.v[1] * b.v[1] - a.v[2] * b.v[2] - a.v[3] * b.v[3];
}
template <class T> MF_D cx<T> mdotq(const W4<T>& a, T q0, T q1, T q2, T q3) {
  return cx<T>{q0 * a.v[0].re - q1 * a.v[1].re - q2 * a.v[2].re - q3 * a.v[3].re,
               q0 * a.v[0].im - q1 * a.v[1].im - q2 * a.v[2].im - q3 * a.v[3].im};
}

// Three-gluon colour-ordered current (VVV1P0_1 Lorentz structure), without
// the propagator/coupling factor: with P2 = Qa, P3 = Qb, P1 = -(Qa+Qb),
//   acc += (a.b)(Qb-Qa) + a (b.(2Qa+Qb)) - b (a.(Qa+2Qb)).
template <class T> MF_D void vvv_add(const W4<T>& a, const T* Qa, const W4<T>& b, const T* Qb, W4<T>& acc) {
  cx<T> ab = mdot(a, b);
  cx<T> ca = mdotq(b, T(2) * Qa[0] + Qb[0], T(2) * Qa[1] + Qb[1], T(2) * Qa[2] + Qb[2], T(2) * Qa[3] + Qb[3]);
  cx<T> cb = mdotq(a, Qa[0] + T(2) * Qb[0], Qa[1] + T(2) * Qb[1], Qa[2] + T(2) * Qb[2], Qa[3] + T(2) * Qb[3]);
#pragma unroll
  for (int k = 0; k < 4; ++k) acc.v[k] += (Qb[k] - Qa[k]) * ab + a.v[k] * ca - b.v[k] * cb;
}
// Four-gluon colour-ordered contact term for the order (a, b, d, off-shell):
//   acc += 2 b (a.d) - a (b.d) - d (a.b)
template <class T> MF_D void vvvv_add(const W4<T>& a, const W4<T>& b, const W4<T>& d, W4<T>& acc) {
  cx<T> ad = mdot(a, d), bd = mdot(b, d), ab = mdot(a, b);
  cx<T> ad2 = ad + ad;
#pragma unroll
  for (int k = 0; k < 4; ++k) acc.v[k] += b.v[k] * ad2 - a.v[k] * bd - d.v[k] * ab;
}
template <class T> MF_D W4<T> combine(cx<T> c3, const W4<T>& a3, cx<T> c4, const W4<T>& a4) {
  W4<T> r;
#pragma unroll
  for (int k = 0; k < 4; ++k) r.v[k] = c3 * a3.v[k] + c4 * a4.v[k];
  return r;
}
// y += S(V) F
template <class T> MF_D void sv_add(const W4<T>& V, const W4<T>& F, W4<T>& y) {
  cx<T> p03 = V.v[0] + V.v[3], m03 = V.v[0] - V.v[3];
  cx<T> p12 = V.v[1] + mul_i(V.v[2]), m12 = V.v[1] - mul_i(V.v[2]);
  y.v[0] += p03 * F.v[2] + p12 * F.v[3];
  y.v[1] += m12 * F.v[2] + m03 * F.v[3];
  y.v[2] += m03 * F.v[0] - p12 * F.v[1];
  y.v[3] += -(m12 * F.v[0]) + p03 * F.v[1];
}
// Off-shell top current from y = sum S(V) F: cf * (S(Q) + M) y, with cf the
// propagator/coupling factor i*GC_11/(Q^2 - M^2 + i M W) (FFV1_1, P1 = -Q).
template <class T> MF_D W4<T> topprop(const T* Q, T M, cx<T> cf, const W4<T>& y) {
  T p03 = Q[0] + Q[3], m03 = Q[0] - Q[3];
  cx<T> p12 = {Q[1], Q[2]}, m12 = {Q[1], -Q[2]};
  W4<T> z;
  z.v[0] = p03 * y.v[2] + p12 * y.v[3] + M * y.v[0];
  z.v[1] = m12 * y.v[2] + m03 * y.v[3] + M * y.v[1];
  z.v[2] = m03 * y.v[0] - p12 * y.v[1] + M * y.v[2];
  z.v[3] = -(m12 * y.v[0]) + p03 * y.v[1] + M * y.v[3];
#pragma unroll
  for (int k = 0; k < 4; ++k) z.v[k] = cf * z.v[k];
  return z;
}
// F1^T S(V) F2 (the FFV1_0 bilinear without its coupling -i*GC_11)
template <class T> MF_D cx<T> sandwich(const W4<T>& F1, const W4<T>& V, const W4<T>& F2) {
  W4<T> y = w4zero<T>();
  sv_add(V, F2, y);
  return F1.v[0] * y.v[0] + F1.v[1] * y.v[1] + F1.v[2] * y.v[2] + F1.v[3] * y.v[3];
}

// row vector r = F1^T S(V), so that F1^T S(V) F2 = r . F2
template <class T> MF_D W4<T> sandwich_row(const W4<T>& F1, const W4<T>& V) {
  cx<T> p03 = V.v[0] + V.v[3], m03 = V.v[0] - V.v[3];
  cx<T> p12 = V.v[1] + mul_i(V.v[2]), m12 = V.v[1] - mul_i(V.v[2]);
  W4<T> r;
  r.v[0] = F1.v[2] * m03 - F1.v[3] * m12;
  r.v[1] = F1.v[3] * p03 - F1.v[2] * p12;
  r.v[2] = F1.v[0] * p03 + F1.v[1] * m12;
  r.v[3] = F1.v[0] * p12 + F1.v[1] * m03;
  return r;
}
template <class T> MF_D cx<T> dot4(const W4<T>& a, const W4<T>& b) {
  return a.v[0] * b.v[0] + a.v[1] * b.v[1] + a.v[2] * b.v[2] + a.v[3] * b.v[3];
}
// sandwich_row(F1, e_mu) for the unit vector e_mu (the row of the bilinear
// F1^T S(e_mu) F2 = row . F2): components of F1 permuted, negated or times i
template <class T> MF_D W4<T> unit_row(const W4<T>& F1, int mu) {
  W4<T> r;
  if (mu == 0) {
    r.v[0] = F1.v[2]; r.v[1] = F1.v[3]; r.v[2] = F1.v[0]; r.v[3] = F1.v[1];
  } else if (mu == 1) {
    r.v[0] = -F1.v[3]; r.v[1] = -F1.v[2]; r.v[2] = F1.v[1]; r.v[3] = F1.v[0];
  } else if (mu == 2) {
    r.v[0] = mul_i(F1.v[3]); r.v[1] = mul_mi(F1.v[2]); r.v[2] = mul_mi(F1.v[1]); r.v[3] = mul_i(F1.v[0]);
  } else {
    r.v[0] = -F1.v[2]; r.v[1] = F1.v[3]; r.v[2] = F1.v[0]; r.v[3] = -F1.v[1];
  }
  return r;
}

// Per-event data shared by all helicities of one event: slot momenta of every
// subset of gluons (Qg) and of the top line (Qt = p_t + Qg), and the
// propagator x coupling factors, evaluated in FP64 (double-float for T =
// float) and stored in T.
template <class T, int K> struct EvData {
  T Qg[1 << K][4];
  T Qt[1 << K][4];
  cx<T> gv3[1 << K];   // GC_10 / Qg^2
  cx<T> gv4[1 << K];   // -i GC_12 / Qg^2
  cx<T> tden[1 << K];  // i GC_11 / (Qt^2 - M^2 + i M W)
  T pext[K + 2][4];    // external momenta
  cx<T> M[4][4];       // WTB[q>>1]^T S(e_mu) WT[q&1]: the top-line bilinears
  T mt;
};

// Slot sign of gluon label j: incoming gluons (particles 0, 1) carry -p.
template <int K> MF_D int gluon_particle(int j) { return j < 2 ? j : j + 2; }

// Double-float arithmetic (a value as an unevaluated sum hi + lo of two
// floats, about 48 significant bits), after Dekker (Numer. Math. 18 (1971)
// 224) and Knuth (TAOCP vol. 2, 4.2.2): the error-free two_sum and the
// fma-based two_prod.  GB300 runs FP32 at 64 times its FP64 rate, so the
// subset invariants of the mixed path are formed this way.
struct ffl {
  float hi, lo;
};
MF_HD ffl ff_two_sum(float a, float b) {
  float s = a + b, bb = s - a;
  return {s, (a - (s - bb)) + (b - bb)};
}
MF_HD ffl ff_quick_two_sum(float a, float b) {
  float s = a + b;
  return {s, b - (s - a)};
}
MF_HD ffl ff_from(double x) {
  float h = (float)x;
  return {h, (float)(x - (double)h)};
}
MF_HD ffl ff_add(ffl a, ffl b) {
  ffl s = ff_two_sum(a.hi, b.hi), t = ff_two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = ff_quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return ff_quick_two_sum(s.hi, s.lo);
}
MF_HD ffl ff_neg(ffl a) { return {-a.hi, -a.lo}; }
MF_HD ffl ff_sqr(ffl a) {
  float p = a.hi * a.hi;
  float e = fmaf(a.hi, a.hi, -p) + 2.0f * a.hi * a.lo;
  return ff_quick_two_sum(p, e);
}
MF_HD float ff_float(ffl a) { return a.hi + a.lo; }
// Minkowski square in double-float
MF_HD ffl ff_msq(const ffl* v) {
  ffl r = ff_sqr(v[0]);
  r = ff_add(r, ff_neg(ff_sqr(v[1])));
  r = ff_add(r, ff_neg(ff_sqr(v[2])));
  return ff_add(r, ff_neg(ff_sqr(v[3])));
}

// Every subset of EvData<float> from FP64 external momenta p[K+2][4]: the
// subset momenta, P^2 and the top line's P^2 - M^2 (where the pole cancels)
// in double-float, the divisions in FP32.
template <int K>
MF_D void evdata_all_ff(EvData<float, K>& ev, const double (*p)[4], double mt, double wt, cx<double> gc10,
                        cx<double> gc11, cx<double> gc12) {
  ffl pg[K][4], pt[4];
#pragma unroll
  for (int j = 0; j < K; ++j) {
    const int part = gluon_particle<K>(j);
#pragma unroll
    for (int c = 0; c < 4; ++c) pg[j][c] = ff_from(part < 2 ? -p[part][c] : p[part][c]);
  }
#pragma unroll
  for (int c = 0; c < 4; ++c) pt[c] = ff_from(p[2][c]);
  const ffl mt2 = ff_from(mt * mt);
  const float g10r = (float)gc10.re, g10i = (float)gc10.im, g12r = (float)gc12.re, g12i = (float)gc12.im;
  const cx<float> num = mul_i(ccast<float>(gc11));
  const float mw = (float)(mt * wt);
  for (int s = 0; s < (1 << K); ++s) {
    ffl Q[4] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}}, Qt[4];
    int nbits = 0;
#pragma unroll
    for (int j = 0; j < K; ++j)
      if (s >> j & 1) {
        ++nbits;
#pragma unroll
        for (int c = 0; c < 4; ++c) Q[c] = ff_add(Q[c], pg[j][c]);
      }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      Qt[c] = ff_add(pt[c], Q[c]);
      ev.Qg[s][c] = ff_float(Q[c]);
      ev.Qt[s][c] = ff_float(Qt[c]);
    }
    if (nbits >= 2) {
      const float iq = 1.0f / ff_float(ff_msq(Q));
      ev.gv3[s] = cx<float>{g10r * iq, g10i * iq};
      ev.gv4[s] = cx<float>{g12i * iq, -g12r * iq};
    } else {
      ev.gv3[s] = cx<float>{0.0f, 0.0f};
      ev.gv4[s] = cx<float>{0.0f, 0.0f};
    }
    const cx<float> den = {ff_float(ff_add(ff_msq(Qt), ff_neg(mt2))), mw};
    ev.tden[s] = cdiv(num, den);
  }
}

// Fill subset `s` of EvData from FP64 external momenta p[K+2][4].
template <class T, int K>
MF_D void evdata_subset(EvData<T, K>& ev, int s, const double (*p)[4], double mt, double wt, cx<double> gc10,
                        cx<double> gc11, cx<double> gc12) {
  double Q[4] = {0, 0, 0, 0};
#pragma unroll
  for (int j = 0; j < K; ++j)
    if (s >> j & 1) {
      int part = gluon_particle<K>(j);
      double sg = part < 2 ? -1.0 : 1.0;
#pragma unroll
      for (int c = 0; c < 4; ++c) Q[c] += sg * p[part][c];
    }
  double Qt[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) Qt[c] = p[2][c] + Q[c];
  double q2 = Q[0] * Q[0] - Q[1] * Q[1] - Q[2] * Q[2] - Q[3] * Q[3];
  double t2 = Qt[0] * Qt[0] - Qt[1] * Qt[1] - Qt[2] * Qt[2] - Qt[3] * Qt[3];
#pragma unroll
  for (int c = 0; c < 4; ++c) { ev.Qg[s][c] = (T)Q[c]; ev.Qt[s][c] = (T)Qt[c]; }
  int nbits = 0;
  for (int j = 0; j < K; ++j) nbits += (s >> j) & 1;
  // The sums and the invariants P^2, P^2 - M^2 (where the top pole cancels)
  // are FP64; the divisions then run in T.
  if (nbits >= 2) {
    T iq = T(1) / (T)q2;
    ev.gv3[s] = cx<T>{(T)gc10.re * iq, (T)gc10.im * iq};
    ev.gv4[s] = cx<T>{(T)gc12.im * iq, -(T)gc12.re * iq};
  } else {
    ev.gv3[s] = cx<T>{T(0), T(0)};
    ev.gv4[s] = cx<T>{T(0), T(0)};
  }
  cx<T> den = {(T)(t2 - mt * mt), (T)(mt * wt)};
  ev.tden[s] = cdiv(mul_i(ccast<T>(gc11)), den);
}
