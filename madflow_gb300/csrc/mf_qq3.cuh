// p p > t t~ j at leading order: the channels with one light-quark line,
// q q~ > t t~ g, q g > t t~ q and q~ g > t t~ q~ (MadGraph's u u~ > t t~ g,
// u g > t t~ u and u~ g > t t~ u~ modules of a p p > t t~ j run; no instance
// in the reference's tests).  One thread per event.
//
// Five diagrams per channel with the HELAS wavefunctions of
// wavefunctions_flow.py and the ALOHA vertex algebra of
// tests/mockup_debug_me.py (FFV1_0 :43, FFV1_1 :67, FFV1_2 :207, VVV1P0_1
// :341) plus the fermion-pair current FFV1P0_3.  The light line runs from its
// i-type end I (incoming quark or outgoing antiquark) to its o-type end O
// (outgoing quark or incoming antiquark), the top line from the t~ to the t:
//   a1 gluon on the light line at I    colour (T^b T^a)_{O I} T^b_{t tb}
//   a2 gluon on the light line at O    colour (T^a T^b)_{O I} T^b_{t tb}
//   a3 gluon on the top line at the t  colour T^b_{O I} (T^a T^b)_{t tb}
//   a4 gluon on the top line at the t~ colour T^b_{O I} (T^b T^a)_{t tb}
//   a5 three-gluon vertex             colour f^{bac} T^b_{O I} T^c_{t tb}
// The colour matrix of these tensors has the eigenvectors (1,1,1,1),
// (1,-1,1,-1), (1,1,-1,-1), (1,-1,-1,1) on the first four diagrams (the
// last with eigenvalue 0), which turns the colour sum of one helicity into
//   |S1|^2 + 3/2 |S2 + 2i a5|^2 + 1/6 |S3|^2,
//   S1 = a1+a2+a3+a4, S2 = a1-a2+a3-a4, S3 = a1+a2-a3-a4.
// Averages: 1/36 (q q~), 1/96 (q g, q~ g).
//
// T: the arithmetic of the wavefunctions and amplitudes (FP32 on the mixed
// path); the slot momenta and the propagator denominators are FP64.
#pragma once
#include "mf_helas.cuh"
#include "mf_vertex.cuh"

namespace mfqq3 {

// a wavefunction and its HELAS slot momentum (+p for an outgoing particle,
// -p for an incoming one, as ixxxxx / oxxxxx / vxxxxx store it)
template <class T> struct QW {
  W4<T> w;
  double q[4];
};

// i * coup / (P^2 - M^2 + i M W), the factor of the ALOHA off-shell routines
template <class T> MF_D cx<T> offshell_factor(const double* P, double M, double W, cx<double> coup) {
  const double p2 = P[0] * P[0] - P[1] * P[1] - P[2] * P[2] - P[3] * P[3];
  const double dr = p2 - M * M, di = M * W;
  const double inv = 1.0 / (dr * dr + di * di);
  const double re = (coup.re * dr + coup.im * di) * inv, im = (coup.im * dr - coup.re * di) * inv;
  return cx<T>{(T)(-im), (T)re};
}

template <class T> MF_D void add_q(const QW<T>& a, const QW<T>& b, double* q) {
#pragma unroll
  for (int k = 0; k < 4; ++k) q[k] = a.q[k] + b.q[k];
}

// FFV1_1: the o-type line continued past the vertex with V,
// c (S(Q) + M) S(V) F2 with Q the summed slot momentum
template <class T> MF_D QW<T> ffv1_1(const QW<T>& F2, const QW<T>& V, cx<double> coup, double M, double W) {
  QW<T> r;
  add_q(F2, V, r.q);
  W4<T> y = w4zero<T>();
  sv_add(V.w, F2.w, y);
  const T Q[4] = {(T)r.q[0], (T)r.q[1], (T)r.q[2], (T)r.q[3]};
  r.w = topprop(Q, (T)M, offshell_factor<T>(r.q, M, W, coup), y);
  return r;
}

// FFV1_2: the i-type line continued past the vertex with V,
// c (S(-Q)^T + M) S(V)^T F1
template <class T> MF_D QW<T> ffv1_2(const QW<T>& F1, const QW<T>& V, cx<double> coup, double M, double W) {
  QW<T> r;
  add_q(F1, V, r.q);
  const W4<T> y = sandwich_row(F1.w, V.w);
  W4<T> P;
#pragma unroll
  for (int k = 0; k < 4; ++k) P.v[k] = cx<T>{(T)(-r.q[k]), T(0)};
  const W4<T> z = sandwich_row(y, P);
  const cx<T> c = offshell_factor<T>(r.q, M, W, coup);
#pragma unroll
  for (int k = 0; k < 4; ++k) r.w.v[k] = c * (z.v[k] + (T)M * y.v[k]);
  return r;
}

// F1^T S(e_mu) F2 for mu = 0..3, so that F1^T S(V) F2 = sum_mu c_mu V^mu
template <class T> MF_D W4<T> bilinear(const W4<T>& F1, const W4<T>& F2) {
  W4<T> c;
#pragma unroll
  for (int mu = 0; mu < 4; ++mu) c.v[mu] = dot4(unit_row(F1, mu), F2);
  return c;
}

// FFV1P0_3: the massless gluon current of a fermion pair
template <class T> MF_D QW<T> ffv1p0_3(const QW<T>& F1, const QW<T>& F2, cx<double> coup) {
  QW<T> r;
  add_q(F1, F2, r.q);
  const W4<T> c = bilinear(F1.w, F2.w);
  const cx<T> f = offshell_factor<T>(r.q, 0.0, 0.0, coup);
  r.w.v[0] = f * c.v[0];
#pragma unroll
  for (int mu = 1; mu < 4; ++mu) r.w.v[mu] = -(f * c.v[mu]);
  return r;
}

// VVV1P0_1: the massless gluon of the three-gluon vertex of V2 and V3
template <class T> MF_D QW<T> vvv1p0_1(const QW<T>& V2, const QW<T>& V3, cx<double> coup) {
  QW<T> r;
  add_q(V2, V3, r.q);
  T P1[4], P2[4], P3[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    P1[k] = (T)(-r.q[k]);
    P2[k] = (T)V2.q[k];
    P3[k] = (T)V3.q[k];
  }
  const W4<T>& a = V2.w;
  const W4<T>& b = V3.w;
  const cx<T> v23 = mdot(b, a);
  const cx<T> c2 = mdotq(b, P2[0] - P1[0], P2[1] - P1[1], P2[2] - P1[2], P2[3] - P1[3]);
  const cx<T> c3 = mdotq(a, P1[0] - P3[0], P1[1] - P3[1], P1[2] - P3[2], P1[3] - P3[3]);
  const cx<T> f = offshell_factor<T>(r.q, 0.0, 0.0, coup);
#pragma unroll
  for (int k = 0; k < 4; ++k) r.w.v[k] = f * ((P3[k] - P2[k]) * v23 + a.v[k] * c2 + b.v[k] * c3);
  return r;
}

template <class T> MF_D cx<T> contract(const W4<T>& c, const W4<T>& V) {
  return c.v[0] * V.v[0] + c.v[1] * V.v[1] + c.v[2] * V.v[2] + c.v[3] * V.v[3];
}
template <class T> MF_D T abs2(cx<T> z) { return z.re * z.re + z.im * z.im; }

template <class T> MF_D bool is_zero(const W4<T>& w) {
  bool z = true;
#pragma unroll
  for (int k = 0; k < 4; ++k) z = z && w.v[k].re == T(0) && w.v[k].im == T(0);
  return z;
}

template <class T> MF_D QW<T> external(int kind, const double* p, double m, T h, T sqh) {
  // kind 0: ixxxxx incoming quark, 1: ixxxxx outgoing antiquark, 2: oxxxxx
  // outgoing quark, 3: oxxxxx incoming antiquark, 4: vxxxxx outgoing gluon,
  // 5: vxxxxx incoming gluon
  const T pt[4] = {(T)p[0], (T)p[1], (T)p[2], (T)p[3]};
  // nsf / nsv: +1 for an incoming fermion, an outgoing fermion or an
  // outgoing vector, -1 for antifermions and an incoming vector
  const double ns = (kind == 0 || kind == 2 || kind == 4) ? 1.0 : -1.0;
  const double out = (kind == 1 || kind == 2 || kind == 4) ? 1.0 : -1.0;
  QW<T> r;
  if (kind <= 1) r.w = ixxxxx<T>(pt, (T)m, h, (T)ns);
  else if (kind <= 3) r.w = oxxxxx<T>(pt, (T)m, h, (T)ns);
  else r.w = vxxxxx<T>(pt, (T)m, h, (T)ns, sqh);
#pragma unroll
  for (int k = 0; k < 4; ++k) r.q[k] = out * p[k];
  return r;
}

}  // namespace mfqq3

// ---- four lanes per event --------------------------------------------------
// The 16 helicity configurations of a channel with non-zero amplitudes (the
// massless quark pair has one chirality: its two spinors share nhel * nsf)
// are the products of 4 light-line states (gluon helicity x chirality) and 4
// top-line states (t x t~ helicities).  Lane l of an event's group of four
// builds the light-line currents of light state l and the top-line
// bilinears of top state l; the 16 products are formed after the light
// currents pass round the group by shuffles, so nothing is computed twice.
// The top-line objects depend on the gluon's momentum only, so they serve
// two of an event's six channel evaluations at once.
namespace mfqq3 {

template <class T> struct TopSide {
  W4<T> c;        // Itb^T S(e_mu) Ot: diagrams a1, a2, a5
  W4<T> d3[2];    // Itb^T S(e_mu) FFV1_1(Ot, G): a3, per gluon helicity
  W4<T> d4[2];    // FFV1_2(Itb, G)^T S(e_mu) Ot: a4
};
template <class T> struct LightSide {
  W4<T> vs0, vs1, vs2, vs5;
};

// kG: 4 outgoing gluon, 5 incoming gluon
template <class T>
MF_D TopSide<T> top_side(const double (*p)[4], const double* pG, int kG, int lane, double mt, double wt,
                         cx<double> gc11, T sqh) {
  const QW<T> Ot = external<T>(2, p[2], mt, (lane >> 1) ? T(1) : T(-1), sqh);
  const QW<T> Itb = external<T>(1, p[3], mt, (lane & 1) ? T(1) : T(-1), sqh);
  TopSide<T> t;
  t.c = bilinear(Itb.w, Ot.w);
#pragma unroll
  for (int hg = 0; hg < 2; ++hg) {
    const QW<T> G = external<T>(kG, pG, 0.0, hg ? T(1) : T(-1), sqh);
    t.d3[hg] = bilinear(Itb.w, ffv1_1(Ot, G, gc11, mt, wt).w);
    t.d4[hg] = bilinear(ffv1_2(Itb, G, gc11, mt, wt).w, Ot.w);
  }
  return t;
}

// light state l: gluon helicity l >> 1, chirality nh = +-1 (l & 1) of the
// quark pair, nhel = nh * nsf for each of the two
template <class T>
MF_D LightSide<T> light_side(int kI, const double* pI, int kO, const double* pO, int kG, const double* pG, int lane,
                             cx<double> gc10, cx<double> gc11, T sqh) {
  const T nh = (lane & 1) ? T(1) : T(-1);
  const T nsfI = kI == 0 ? T(1) : T(-1), nsfO = kO == 2 ? T(1) : T(-1);
  const QW<T> G = external<T>(kG, pG, 0.0, (lane >> 1) ? T(1) : T(-1), sqh);
  const QW<T> I = external<T>(kI, pI, 0.0, nh * nsfI, sqh);
  const QW<T> O = external<T>(kO, pO, 0.0, nh * nsfO, sqh);
  LightSide<T> l;
  const QW<T> vs0 = ffv1p0_3(I, O, gc11);
  l.vs0 = vs0.w;
  l.vs1 = ffv1p0_3(ffv1_2(I, G, gc11, 0.0, 0.0), O, gc11).w;
  l.vs2 = ffv1p0_3(I, ffv1_1(O, G, gc11, 0.0, 0.0), gc11).w;
  l.vs5 = vvv1p0_1(vs0, G, gc10).w;
  return l;
}

template <class T> MF_D cx<T> shfl(unsigned mask, cx<T> v, int src) {
  return cx<T>{__shfl_sync(mask, v.re, src), __shfl_sync(mask, v.im, src)};
}
template <class T> MF_D W4<T> shfl(unsigned mask, const W4<T>& v, int src) {
  W4<T> r;
#pragma unroll
  for (int k = 0; k < 4; ++k) r.v[k] = shfl(mask, v.v[k], src);
  return r;
}

// This lane's share of the colour- and helicity-summed |M|^2 (without the
// factor |GC_11|^2 and the average): top state `lane` times the four light
// states of the group.  mask: the group's four lanes; base: its first lane.
template <class T>
MF_D T group_products(const TopSide<T>& t, const LightSide<T>& l, unsigned mask, int base) {
  T tot = T(0);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const W4<T> vs0 = shfl(mask, l.vs0, base + j), vs1 = shfl(mask, l.vs1, base + j);
    const W4<T> vs2 = shfl(mask, l.vs2, base + j), vs5 = shfl(mask, l.vs5, base + j);
    const cx<T> a1 = contract(t.c, vs1), a2 = contract(t.c, vs2), a5 = contract(t.c, vs5);
    const cx<T> a3 = contract(t.d3[j >> 1], vs0), a4 = contract(t.d4[j >> 1], vs0);
    const cx<T> s1 = a1 + a2 + a3 + a4, s3 = a1 + a2 - a3 - a4;
    const cx<T> s2 = a1 - a2 + a3 - a4 + cx<T>{T(-2) * a5.im, T(2) * a5.re};
    tot += abs2(s1) + T(1.5) * abs2(s2) + abs2(s3) * T(1.0 / 6.0);
  }
  return tot;
}

// external kinds and momenta of (I, O, G) of a channel; a, b: the indices
// of the momenta of particles 0 and 1 (1, 0 for the mirrored initial state)
MF_D void channel_legs(int channel, int a, int b, int& kI, int& iI, int& kO, int& iO, int& kG, int& iG) {
  if (channel == 0) {        // q q~ > t t~ g
    kI = 0; iI = a; kO = 3; iO = b; kG = 4; iG = 4;
  } else if (channel == 1) { // q g > t t~ q
    kI = 0; iI = a; kO = 2; iO = 4; kG = 5; iG = b;
  } else {                   // q~ g > t t~ q~
    kI = 1; iI = 4; kO = 3; iO = a; kG = 5; iG = b;
  }
}

template <class T> MF_D T group_sum(T v, unsigned mask) {
  v += __shfl_xor_sync(mask, v, 1);
  v += __shfl_xor_sync(mask, v, 2);
  return v;
}

}  // namespace mfqq3

// |M|^2 of one channel (C ABI mf_smatrix_qq_ttxj), evaluated by a group of
// four lanes; every lane of the group returns the value.  channel 0
// q(p[0]) q~(p[1]) > t(p[2]) t~(p[3]) g(p[4]); 1 q(p[0]) g(p[1]) > t t~
// q(p[4]); 2 q~(p[0]) g(p[1]) > t t~ q~(p[4]); averaged over the initial
// spins and colours.  All four lanes of the group (mask) must call it.
template <class T>
MF_D double qq3_me_group(int channel, const double (*p)[4], double mt, double wt, cx<double> gc10, cx<double> gc11,
                         T sqh, unsigned mask, int lane, int base) {
  using namespace mfqq3;
  int kI, iI, kO, iO, kG, iG;
  channel_legs(channel, 0, 1, kI, iI, kO, iO, kG, iG);
  const TopSide<T> t = top_side<T>(p, p[iG], kG, lane, mt, wt, gc11, sqh);
  const LightSide<T> l = light_side<T>(kI, p[iI], kO, p[iO], kG, p[iG], lane, gc10, gc11, sqh);
  const T tot = group_sum(group_products(t, l, mask, base), mask);
  const double g11sq = gc11.re * gc11.re + gc11.im * gc11.im;  // the FFV1_0 factor -i GC_11
  return (double)tot * g11sq / (channel == 0 ? 36.0 : 96.0);
}

// The six channel evaluations of an event of p p > t t~ j weighted by their
// luminosities lum[6] (q q~, q~ q, q g, g q, q~ g, g q~), summed; the three
// gluon momenta (p[4]; p[1]; p[0]) each serve two evaluations' top lines.
template <class T>
MF_D double qq3_lum_sum(const double (*p)[4], const double* lum, double mt, double wt, cx<double> gc10,
                        cx<double> gc11, T sqh, unsigned mask, int lane, int base) {
  using namespace mfqq3;
  double s = 0.0;
#pragma unroll 1
  for (int g = 0; g < 3; ++g) {
    // g = 0: q q~ and its mirror (gluon p[4]); 1: q g, q~ g (gluon p[1]);
    // 2: g q, g q~ (gluon p[0])
    const int kG = g == 0 ? 4 : 5, iG = g == 0 ? 4 : (g == 1 ? 1 : 0);
    const TopSide<T> t = top_side<T>(p, p[iG], kG, lane, mt, wt, gc11, sqh);
#pragma unroll 1
    for (int u = 0; u < 2; ++u) {
      const int channel = g == 0 ? 0 : 1 + u, m = g == 0 ? u : g - 1;
      int kI, iI, kO, iO, kGc, iGc;
      channel_legs(channel, m, 1 - m, kI, iI, kO, iO, kGc, iGc);
      const LightSide<T> l = light_side<T>(kI, p[iI], kO, p[iO], kGc, p[iGc], lane, gc10, gc11, sqh);
      const int j = g == 0 ? u : (channel == 1 ? 2 + m : 4 + m);
      s += lum[j] / (channel == 0 ? 36.0 : 96.0) * (double)group_products(t, l, mask, base);
    }
  }
  const double g11sq = gc11.re * gc11.re + gc11.im * gc11.im;
  return group_sum(s, mask) * g11sq;
}
