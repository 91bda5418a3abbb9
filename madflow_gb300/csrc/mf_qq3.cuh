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

// |M|^2 averaged over the initial spins and colours of one light-quark
// channel: channel 0 q(p[0]) q~(p[1]) > t(p[2]) t~(p[3]) g(p[4]); 1 q(p[0])
// g(p[1]) > t t~ q(p[4]); 2 q~(p[0]) g(p[1]) > t t~ q~(p[4]).  a, b: the
// indices of the momenta of particles 0 and 1 in p (0, 1, or 1, 0 for the
// mirrored initial state).  gc10, gc11: GC_10, GC_11; sqh: sqrt(1/2) of the
// gluon polarisations.
template <class T>
MF_D double qq3_me(int channel, const double (*p)[4], int a, int b, double mt, double wt, cx<double> gc10,
                   cx<double> gc11, T sqh) {
  using namespace mfqq3;
  // external kinds of (I, O, G) per channel, and their momenta
  const int kI = channel == 2 ? 1 : 0, kO = channel == 0 ? 3 : (channel == 1 ? 2 : 3), kG = channel == 0 ? 4 : 5;
  const double* pI = channel == 2 ? p[4] : p[a];
  const double* pO = channel == 0 ? p[b] : (channel == 1 ? p[4] : p[a]);
  const double* pG = channel == 0 ? p[4] : p[b];
  QW<T> Ot[2], Itb[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    Ot[h] = external<T>(2, p[2], mt, h ? T(1) : T(-1), sqh);
    Itb[h] = external<T>(1, p[3], mt, h ? T(1) : T(-1), sqh);
  }
  T tot = T(0);
  for (int hg = 0; hg < 2; ++hg) {
    const QW<T> G = external<T>(kG, pG, 0.0, hg ? T(1) : T(-1), sqh);
    QW<T> ot3[2], itb4[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      ot3[h] = ffv1_1(Ot[h], G, gc11, mt, wt);
      itb4[h] = ffv1_2(Itb[h], G, gc11, mt, wt);
    }
    for (int hio = 0; hio < 4; ++hio) {
      const QW<T> I = external<T>(kI, pI, 0.0, (hio & 1) ? T(1) : T(-1), sqh);
      const QW<T> O = external<T>(kO, pO, 0.0, (hio & 2) ? T(1) : T(-1), sqh);
      const QW<T> vs0 = ffv1p0_3(I, O, gc11);
      // massless quarks: the pairs of opposite chirality give an exactly
      // zero current (and zero amplitudes)
      if (is_zero(vs0.w)) continue;
      const QW<T> vs1 = ffv1p0_3(ffv1_2(I, G, gc11, 0.0, 0.0), O, gc11);
      const QW<T> vs2 = ffv1p0_3(I, ffv1_1(O, G, gc11, 0.0, 0.0), gc11);
      const QW<T> vs5 = vvv1p0_1(vs0, G, gc10);
#pragma unroll
      for (int ht = 0; ht < 2; ++ht)
#pragma unroll
        for (int hb = 0; hb < 2; ++hb) {
          const W4<T> c = bilinear(Itb[hb].w, Ot[ht].w);
          const cx<T> a1 = contract(c, vs1.w), a2 = contract(c, vs2.w), a5 = contract(c, vs5.w);
          const cx<T> a3 = contract(bilinear(Itb[hb].w, ot3[ht].w), vs0.w);
          const cx<T> a4 = contract(bilinear(itb4[hb].w, Ot[ht].w), vs0.w);
          const cx<T> s1 = a1 + a2 + a3 + a4, s3 = a1 + a2 - a3 - a4;
          const cx<T> s2 = a1 - a2 + a3 - a4 + cx<T>{T(-2) * a5.im, T(2) * a5.re};
          tot += abs2(s1) + T(1.5) * abs2(s2) + abs2(s3) * T(1.0 / 6.0);
        }
    }
  }
  // every amplitude carries the FFV1_0 factor -i GC_11
  const double g11sq = gc11.re * gc11.re + gc11.im * gc11.im;
  return (double)tot * g11sq / (channel == 0 ? 36.0 : 96.0);
}
