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

// a wavefunction and its HELAS slot momentum in T (+p for an outgoing
// particle, -p for an incoming one, as ixxxxx / oxxxxx / vxxxxx store it)
template <class T> struct QW {
  W4<T> w;
  T q[4];
};

template <class T> MF_D void add_q(const QW<T>& a, const QW<T>& b, T* q) {
#pragma unroll
  for (int k = 0; k < 4; ++k) q[k] = a.q[k] + b.q[k];
}

// The off-shell routines take their factor c = i * coup / (P^2 - M^2 + i M W)
// ready-made (the invariants P^2 are FP64, computed once per event).

// FFV1_1: the o-type line continued past the vertex with V,
// c (S(Q) + M) S(V) F2 with Q the summed slot momentum
template <class T> MF_D QW<T> ffv1_1(const QW<T>& F2, const QW<T>& V, cx<T> c, T M) {
  QW<T> r;
  add_q(F2, V, r.q);
  W4<T> y = w4zero<T>();
  sv_add(V.w, F2.w, y);
  r.w = topprop(r.q, M, c, y);
  return r;
}

// FFV1_2: the i-type line continued past the vertex with V,
// c (S(-Q)^T + M) S(V)^T F1
template <class T> MF_D QW<T> ffv1_2(const QW<T>& F1, const QW<T>& V, cx<T> c, T M) {
  QW<T> r;
  add_q(F1, V, r.q);
  const W4<T> y = sandwich_row(F1.w, V.w);
  W4<T> P;
#pragma unroll
  for (int k = 0; k < 4; ++k) P.v[k] = cx<T>{-r.q[k], T(0)};
  const W4<T> z = sandwich_row(y, P);
#pragma unroll
  for (int k = 0; k < 4; ++k) r.w.v[k] = c * (z.v[k] + M * y.v[k]);
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
template <class T> MF_D QW<T> ffv1p0_3(const QW<T>& F1, const QW<T>& F2, cx<T> c) {
  QW<T> r;
  add_q(F1, F2, r.q);
  const W4<T> b = bilinear(F1.w, F2.w);
  r.w.v[0] = c * b.v[0];
#pragma unroll
  for (int mu = 1; mu < 4; ++mu) r.w.v[mu] = -(c * b.v[mu]);
  return r;
}

// VVV1P0_1: the massless gluon of the three-gluon vertex of V2 and V3
template <class T> MF_D QW<T> vvv1p0_1(const QW<T>& V2, const QW<T>& V3, cx<T> c) {
  QW<T> r;
  add_q(V2, V3, r.q);
  const T* P2 = V2.q;
  const T* P3 = V3.q;
  T P1[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) P1[k] = -r.q[k];
  const W4<T>& a = V2.w;
  const W4<T>& b = V3.w;
  const cx<T> v23 = mdot(b, a);
  const cx<T> c2 = mdotq(b, P2[0] - P1[0], P2[1] - P1[1], P2[2] - P1[2], P2[3] - P1[3]);
  const cx<T> c3 = mdotq(a, P1[0] - P3[0], P1[1] - P3[1], P1[2] - P3[2], P1[3] - P3[3]);
#pragma unroll
  for (int k = 0; k < 4; ++k) r.w.v[k] = c * ((P3[k] - P2[k]) * v23 + a.v[k] * c2 + b.v[k] * c3);
  return r;
}

template <class T> MF_D cx<T> contract(const W4<T>& c, const W4<T>& V) {
  return c.v[0] * V.v[0] + c.v[1] * V.v[1] + c.v[2] * V.v[2] + c.v[3] * V.v[3];
}
template <class T> MF_D T abs2(cx<T> z) { return z.re * z.re + z.im * z.im; }

template <class T> MF_D QW<T> external(int kind, const T* pt, T m, T h, T sqh) {
  // kind 0: ixxxxx incoming quark, 1: ixxxxx outgoing antiquark, 2: oxxxxx
  // outgoing quark, 3: oxxxxx incoming antiquark, 4: vxxxxx outgoing gluon,
  // 5: vxxxxx incoming gluon; pt the momentum in T
  // nsf / nsv: +1 for an incoming fermion, an outgoing fermion or an
  // outgoing vector, -1 for antifermions and an incoming vector
  const T ns = (kind == 0 || kind == 2 || kind == 4) ? T(1) : T(-1);
  const T out = (kind == 1 || kind == 2 || kind == 4) ? T(1) : T(-1);
  QW<T> r;
  if (kind <= 1) r.w = ixxxxx<T>(pt, m, h, ns);
  else if (kind <= 3) r.w = oxxxxx<T>(pt, m, h, ns);
  else r.w = vxxxxx<T>(pt, m, h, ns, sqh);
#pragma unroll
  for (int k = 0; k < 4; ++k) r.q[k] = out * pt[k];
  return r;
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
template <class T> MF_D T group_sum(T v, unsigned mask) {
  v += __shfl_xor_sync(mask, v, 1);
  v += __shfl_xor_sync(mask, v, 2);
  return v;
}

// external kinds and momentum indices of (I, O, G) of a channel; a, b: the
// indices of the momenta of particles 0 and 1 (1, 0 for the mirrored
// initial state)
MF_D void channel_legs(int channel, int a, int b, int& kI, int& iI, int& kO, int& iO, int& kG, int& iG) {
  if (channel == 0) {        // q q~ > t t~ g
    kI = 0; iI = a; kO = 3; iO = b; kG = 4; iG = 4;
  } else if (channel == 1) { // q g > t t~ q
    kI = 0; iI = a; kO = 2; iO = 4; kG = 5; iG = b;
  } else {                   // q~ g > t t~ q~
    kI = 1; iI = 4; kO = 3; iO = a; kG = 5; iG = b;
  }
}
MF_D double out_sign(int kind) { return (kind == 1 || kind == 2 || kind == 4) ? 1.0 : -1.0; }

// ---- the propagator factors of an event ---------------------------------------
// 1 / (P^2 - M^2 + i M W) of the event's 25 off-shell lines, P^2 in FP64
// (massless differences such as (p_q - p_g)^2 cancel in FP32):
//   0        the gluon of the top pair, P = p0 + p1 - p4
//   1 + 2g   the top after the gluon of set g, P = p2 + q_g
//   2 + 2g   the anti-top before it, P = p3 + q_g
//   7 + 3j   evaluation j: the light line at I with the gluon, P = q_I + q_G
//   8 + 3j   at O with the gluon, P = q_O + q_G
//   9 + 3j   the light-line gluon, P = q_I + q_O
// q: slot momenta; gluon sets g = 0 (p4 outgoing), 1 (p1 incoming), 2 (p0
// incoming); evaluations j = 2g + u in the order of qq3_lum_sum.
constexpr int kQQ3Factors = 25;

MF_D void eval_channel(int j, int& channel, int& m) {
  const int g = j >> 1, u = j & 1;
  channel = g == 0 ? 0 : 1 + u;
  m = g == 0 ? u : g - 1;
}

template <class T>
MF_D cx<T> factor(int k, const double (*p)[4], double mt, double wt) {
  double P[4];
  double M = 0.0, W = 0.0;
  if (k == 0) {
    // the light side's momenta, as the off-shell routines sum them (equal to
    // p2 + p3 up to the phase space's energy conservation)
    for (int c = 0; c < 4; ++c) P[c] = p[0][c] + p[1][c] - p[4][c];
  } else if (k < 7) {
    const int g = (k - 1) >> 1, top = (k - 1) & 1;
    const int ig = g == 0 ? 4 : 2 - g;
    const double sg = g == 0 ? 1.0 : -1.0;
    for (int c = 0; c < 4; ++c) P[c] = p[2 + top][c] + sg * p[ig][c];
    M = mt;
    W = wt;
  } else {
    const int j = (k - 7) / 3, r = (k - 7) % 3;
    int channel, m, kI, iI, kO, iO, kG, iG;
    eval_channel(j, channel, m);
    channel_legs(channel, m, 1 - m, kI, iI, kO, iO, kG, iG);
    const double sI = out_sign(kI), sO = out_sign(kO), sG = out_sign(kG);
    for (int c = 0; c < 4; ++c)
      P[c] = r == 0 ? sI * p[iI][c] + sG * p[iG][c]
                    : (r == 1 ? sO * p[iO][c] + sG * p[iG][c] : sI * p[iI][c] + sO * p[iO][c]);
  }
  const double d = P[0] * P[0] - P[1] * P[1] - P[2] * P[2] - P[3] * P[3] - M * M;
  // 1 / (d + i M W) in T
  const T dr = (T)d, di = (T)(M * W);
  const T inv = T(1) / (dr * dr + di * di);
  return cx<T>{dr * inv, -di * inv};
}

// all 25 factors in every lane of the group: lane l computes those with
// index = l (mod 4), the group exchanges them
template <class T> struct Factors {
  cx<T> r[kQQ3Factors];
};
template <class T>
MF_D Factors<T> event_factors(const double (*p)[4], double mt, double wt, unsigned mask, int lane, int base) {
  cx<T> mine[(kQQ3Factors + 3) / 4];
#pragma unroll
  for (int i = 0; i < (kQQ3Factors + 3) / 4; ++i) {
    const int k = 4 * i + lane;
    mine[i] = k < kQQ3Factors ? factor<T>(k, p, mt, wt) : cx<T>{T(0), T(0)};
  }
  Factors<T> f;
#pragma unroll
  for (int k = 0; k < kQQ3Factors; ++k) f.r[k] = shfl(mask, mine[k >> 2], base + (k & 3));
  return f;
}

// i * coup * r
template <class T> MF_D cx<T> ic(cx<double> coup, cx<T> r) {
  const cx<T> c{(T)coup.re, (T)coup.im};
  const cx<T> z = c * r;
  return cx<T>{-z.im, z.re};
}

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
template <class T> struct TopSide {
  W4<T> c;        // Itb^T S(e_mu) Ot: diagrams a1, a2, a5
  W4<T> d3[2];    // Itb^T S(e_mu) FFV1_1(Ot, G): a3, per gluon helicity
  W4<T> d4[2];    // FFV1_2(Itb, G)^T S(e_mu) Ot: a4
};
template <class T> struct LightSide {
  W4<T> vs0, vs1, vs2, vs5;
};

// gluon set g (0: p4 outgoing, 1: p1 incoming, 2: p0 incoming)
template <class T>
MF_D TopSide<T> top_side(const T (*p)[4], int g, int lane, T mt, cx<double> gc11, const Factors<T>& F, T sqh) {
  const QW<T> Ot = external<T>(2, p[2], mt, (lane >> 1) ? T(1) : T(-1), sqh);
  const QW<T> Itb = external<T>(1, p[3], mt, (lane & 1) ? T(1) : T(-1), sqh);
  const int kG = g == 0 ? 4 : 5, iG = g == 0 ? 4 : 2 - g;
  const cx<T> ct = ic<T>(gc11, F.r[1 + 2 * g]), cb = ic<T>(gc11, F.r[2 + 2 * g]);
  TopSide<T> t;
  t.c = bilinear(Itb.w, Ot.w);
#pragma unroll
  for (int hg = 0; hg < 2; ++hg) {
    const QW<T> G = external<T>(kG, p[iG], T(0), hg ? T(1) : T(-1), sqh);
    t.d3[hg] = bilinear(Itb.w, ffv1_1(Ot, G, ct, mt).w);
    t.d4[hg] = bilinear(ffv1_2(Itb, G, cb, mt).w, Ot.w);
  }
  return t;
}

// evaluation j's light state l: gluon helicity l >> 1, chirality nh = +-1
// (l & 1) of the quark pair, nhel = nh * nsf for each of the two
template <class T>
MF_D LightSide<T> light_side(const T (*p)[4], int j, int lane, cx<double> gc10, cx<double> gc11, const Factors<T>& F,
                             T sqh) {
  int channel, m, kI, iI, kO, iO, kG, iG;
  eval_channel(j, channel, m);
  channel_legs(channel, m, 1 - m, kI, iI, kO, iO, kG, iG);
  const T nh = (lane & 1) ? T(1) : T(-1);
  const T nsfI = kI == 0 ? T(1) : T(-1), nsfO = kO == 2 ? T(1) : T(-1);
  const QW<T> G = external<T>(kG, p[iG], T(0), (lane >> 1) ? T(1) : T(-1), sqh);
  const QW<T> I = external<T>(kI, p[iI], T(0), nh * nsfI, sqh);
  const QW<T> O = external<T>(kO, p[iO], T(0), nh * nsfO, sqh);
  const cx<T> cs = ic<T>(gc11, F.r[0]);
  LightSide<T> l;
  const QW<T> vs0 = ffv1p0_3(I, O, ic<T>(gc11, F.r[9 + 3 * j]));
  l.vs0 = vs0.w;
  l.vs1 = ffv1p0_3(ffv1_2(I, G, ic<T>(gc11, F.r[7 + 3 * j]), T(0)), O, cs).w;
  l.vs2 = ffv1p0_3(I, ffv1_1(O, G, ic<T>(gc11, F.r[8 + 3 * j]), T(0)), cs).w;
  l.vs5 = vvv1p0_1(vs0, G, ic<T>(gc10, F.r[0])).w;
  return l;
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

}  // namespace mfqq3

// The six channel evaluations j of an event of p p > t t~ j, |M|^2 averaged
// over the initial spins and colours, in the order q q~, q~ q (mirrored),
// q g, q~ g, g q, g q~; weighted by w[j] and summed (w[j] = 1 for one j
// alone gives that evaluation).  Evaluated by a group of four lanes (mask,
// lane 0..3, base: the group's first lane); every lane of the group must
// call it and every lane returns the sum.  p: [5][4] momenta in FP64.
template <class T>
MF_D double qq3_weighted_sum(const double (*p)[4], const double* w, double mt, double wt, cx<double> gc10,
                             cx<double> gc11, T sqh, unsigned mask, int lane, int base) {
  using namespace mfqq3;
  const Factors<T> F = event_factors<T>(p, mt, wt, mask, lane, base);
  T pt[5][4];
#pragma unroll
  for (int i = 0; i < 5; ++i)
#pragma unroll
    for (int c = 0; c < 4; ++c) pt[i][c] = (T)p[i][c];
  double s = 0.0;
#pragma unroll 1
  for (int g = 0; g < 3; ++g) {
    if (w[2 * g] == 0.0 && w[2 * g + 1] == 0.0) continue;  // uniform across the group
    const TopSide<T> t = top_side<T>(pt, g, lane, (T)mt, gc11, F, sqh);
#pragma unroll 1
    for (int u = 0; u < 2; ++u) {
      const int j = 2 * g + u;
      if (w[j] == 0.0) continue;
      int channel, m;
      eval_channel(j, channel, m);
      const LightSide<T> l = light_side<T>(pt, j, lane, gc10, gc11, F, sqh);
      // the averages over the initial spins and colours: 1/36, 1/96
      s += w[j] * (channel == 0 ? 1.0 / 36.0 : 1.0 / 96.0) * (double)group_products(t, l, mask, base);
    }
  }
  const double g11sq = gc11.re * gc11.re + gc11.im * gc11.im;  // the FFV1_0 factor -i GC_11
  return group_sum(s, mask) * g11sq;
}
