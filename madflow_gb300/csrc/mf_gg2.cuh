// g g > t t~ in one thread per event: madflow's frozen module
// (tests/mockup_debug_me.py:454-543, Matrix_1_gg_ttx) evaluated straight
// from the momenta, without a per-event record.  Three diagrams: the
// s-channel gluon (VVV1P0_1 with GC_10) and the t- and u-channel tops
// (FFV1_1, FFV1_2 with GC_11), JAMP = (i a0 - a1, -i a0 - a2), colour
// matrix [[16, -2], [-2, 16]] / 3, summed over the 16 helicities and divided
// by 256 (mockup_debug_me.py:423-443, 506-537).
//
// Helicity recycling: the top-line bilinears serve the four gluon helicity
// pairs, the three-gluon current the four top pairs.  The three propagator
// invariants are FP64 (from the momenta, once per event); wavefunctions and
// amplitudes run in T (FP32 on the mixed path).
#pragma once
#include "mf_qq3.cuh"

// |M|^2 of g(p[0]) g(p[1]) > t(p[2]) t~(p[3]) averaged (/256); hel
// (optional) [16 * hstride]: per helicity configuration the unaveraged
// value of Matrix_1_gg_ttx.matrix, in madflow's helicity order (gluons,
// top, anti-top from the most significant bit; the anti-top runs +1, -1).
template <class T>
MF_D double gg2_me(const double (*p)[4], double mt, double wt, cx<double> gc10, cx<double> gc11, T sqh,
                   double* hel = nullptr, int64_t hstride = 1) {
  using namespace mfqq3;
  T pt[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int c = 0; c < 4; ++c) pt[i][c] = (T)p[i][c];
  // propagator factors i * coup / (P^2 - M^2 + i M W), P^2 in FP64
  double P[4];
  for (int c = 0; c < 4; ++c) P[c] = p[0][c] + p[1][c];
  const cx<T> cs = ic<T>(gc10, cx<T>{(T)(1.0 / (P[0] * P[0] - P[1] * P[1] - P[2] * P[2] - P[3] * P[3])), T(0)});
  cx<T> ctu[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    // t channel: the top after gluon 0 (p2 - p0); u channel: the anti-top (p3 - p0)
    for (int c = 0; c < 4; ++c) P[c] = p[2 + u][c] - p[0][c];
    const double d = P[0] * P[0] - P[1] * P[1] - P[2] * P[2] - P[3] * P[3] - mt * mt;
    const T dr = (T)d, di = (T)(mt * wt);
    const T inv = T(1) / (dr * dr + di * di);
    ctu[u] = ic<T>(gc11, cx<T>{dr * inv, -di * inv});
  }
  QW<T> G0[2], G1[2], Ot[2], Itb[2];
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    const T h = b ? T(1) : T(-1);
    G0[b] = external<T>(5, pt[0], T(0), h, sqh);
    G1[b] = external<T>(5, pt[1], T(0), h, sqh);
    Ot[b] = external<T>(2, pt[2], (T)mt, h, sqh);
    Itb[b] = external<T>(1, pt[3], (T)mt, h, sqh);
  }
  W4<T> vs[2][2];  // the s-channel gluon of (h0, h1)
#pragma unroll
  for (int a = 0; a < 2; ++a)
#pragma unroll
    for (int b = 0; b < 2; ++b) vs[a][b] = vvv1p0_1(G0[a], G1[b], cs).w;
  T tot = T(0);
  const double g11sq = gc11.re * gc11.re + gc11.im * gc11.im;  // the FFV1_0 factor -i GC_11
  // (rolled in FP64, where the unrolled form spills)
#pragma unroll(sizeof(T) == 4 ? 2 : 1)
  for (int h2 = 0; h2 < 2; ++h2)
#pragma unroll(sizeof(T) == 4 ? 2 : 1)
    for (int b3 = 0; b3 < 2; ++b3) {
      const int h3 = 1 - b3;  // the anti-top's +1 first
      const W4<T> c = bilinear(Itb[h3].w, Ot[h2].w);
#pragma unroll
      for (int h0 = 0; h0 < 2; ++h0) {
        const W4<T> dt = bilinear(Itb[h3].w, ffv1_1(Ot[h2], G0[h0], ctu[0], (T)mt).w);
        const W4<T> du = bilinear(ffv1_2(Itb[h3], G0[h0], ctu[1], (T)mt).w, Ot[h2].w);
#pragma unroll
        for (int h1 = 0; h1 < 2; ++h1) {
          const cx<T> a0 = contract(c, vs[h0][h1]), a1 = contract(dt, G1[h1].w), a2 = contract(du, G1[h1].w);
          const cx<T> j1 = cx<T>{-a0.im, a0.re} - a1;  // i a0 - a1
          const cx<T> j2 = cx<T>{a0.im, -a0.re} - a2;  // -i a0 - a2
          const T m = (T(16) * (abs2(j1) + abs2(j2)) - T(4) * (j1.re * j2.re + j1.im * j2.im)) * T(1.0 / 3.0);
          tot += m;
          if (hel) hel[(int64_t)((h0 << 3) | (h1 << 2) | (h2 << 1) | b3) * hstride] = (double)m * g11sq;
        }
      }
    }
  return (double)tot * g11sq / 256.0;
}
