// q q~ > t t~ at leading order (one diagram: an s-channel gluon), the
// light-quark channel of p p > t t~ (MadGraph's u u~ > t t~, d d~ > t t~, ...
// modules of madflow's p p > t t~ run; no instance in the reference's tests).
// The HELAS wavefunctions of wavefunctions_flow.py (ixxxxx for the incoming
// quark and the outgoing anti-top, oxxxxx for the incoming antiquark and the
// outgoing top), the two fermion bilinears c_mu = F1^T S(e_mu) F2 (so that
// F1^T S(V) F2 = sum_mu c_mu V^mu) and the gluon propagator contract them:
//   amp = GC_11^2 (c_t . c_q) / s  (up to a phase),
// and the colour algebra T^a_ij T^a_kl = (d_il d_kj - d_ij d_kl / 3) / 2 sums
// the colours to 2 |amp|^2.  Averaged over the initial spins (4) and colours
// (9).  T: the arithmetic of the spinors and bilinears (FP32 on the mixed
// path; the invariant s in FP64).
#pragma once
#include "mf_helas.cuh"
#include "mf_vertex.cuh"

// p [4][4]: q, q~, t, t~ (E, px, py, pz); g11sq = |GC_11|^2
template <class T> MF_D double uux_ttx_me(const double (*p)[4], double mt, double g11sq) {
  T q[4][4];
  for (int i = 0; i < 4; ++i)
    for (int c = 0; c < 4; ++c) q[i][c] = (T)p[i][c];
  W4<T> wq[2], wqb[2], wt[2], wtb[2];
  for (int b = 0; b < 2; ++b) {
    const T h = b ? T(1) : T(-1);
    wq[b] = ixxxxx<T>(q[0], T(0), h, T(1));
    wqb[b] = oxxxxx<T>(q[1], T(0), h, T(-1));
    wt[b] = oxxxxx<T>(q[2], (T)mt, h, T(1));
    wtb[b] = ixxxxx<T>(q[3], (T)mt, h, T(-1));
  }
  T tot = T(0);
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b) {
      cx<T> cq[4];
      for (int mu = 0; mu < 4; ++mu) cq[mu] = dot4(unit_row(wq[a], mu), wqb[b]);
      for (int c = 0; c < 2; ++c)
        for (int d = 0; d < 2; ++d) {
          cx<T> ct[4];
          for (int mu = 0; mu < 4; ++mu) ct[mu] = dot4(unit_row(wtb[c], mu), wt[d]);
          const cx<T> x = ct[0] * cq[0] - ct[1] * cq[1] - ct[2] * cq[2] - ct[3] * cq[3];
          tot += x.re * x.re + x.im * x.im;
        }
    }
  double P[4];
  for (int c = 0; c < 4; ++c) P[c] = p[0][c] + p[1][c];
  const double s = P[0] * P[0] - P[1] * P[1] - P[2] * P[2] - P[3] * P[3];
  return (double)tot * (g11sq * g11sq) / (s * s) * (2.0 / 36.0);
}
