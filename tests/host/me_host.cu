// Host-side harness for the generated colour-ordered recursion: compiles the
// product's device/host headers as host code so the CPU test suite can
// compare the generated matrix elements with the oracle without a GPU.
#include <cstdint>
#include <cstring>

#include "../../madflow_gb300/csrc/mf_helas.cuh"
#include "../../madflow_gb300/csrc/mf_vertex.cuh"
#include "../../madflow_gb300/csrc/generated/ttng2.cuh"
#include "../../madflow_gb300/csrc/generated/ttng3.cuh"
#include "../../madflow_gb300/csrc/generated/ttng4.cuh"

template <int K, class T> struct HostProc;
#define HOSTPROC(KK)                                                                                      \
  template <class T> struct HostProc<KK, T> {                                                             \
    static constexpr int NP = ttng##KK::NPERM, NC = ttng##KK::NCOMB;                                      \
    static void amps(const EvData<T, KK>& ev, const W4<T>* g, const W4<T>& wt, const W4<T>& wtb, cx<T>* A) { \
      ttng##KK##_amps<T>(ev, g, wt, wtb, A);                                                              \
    }                                                                                                     \
    static const signed char* hel(int h) { return ttng##KK::hel_h[h]; }                                  \
    static float col(int i) { return ttng##KK::colour_num_h[i]; }                                         \
    static constexpr double CDEN = ttng##KK::COLOUR_DEN, DEN = ttng##KK::DENOMINATOR;                     \
  };
HOSTPROC(2)
HOSTPROC(3)
HOSTPROC(4)

template <int K, class T>
static void partials(const double* p, const double* hel, const double* coup, double mt, double wt, cx<double>* out) {
  using P = HostProc<K, T>;
  double pd[K + 2][4];
  std::memcpy(pd, p, sizeof(pd));
  static EvData<T, K> ev;
  cx<double> c10 = {coup[0], coup[1]}, c11 = {coup[2], coup[3]}, c12 = {coup[4], coup[5]};
  for (int s = 0; s < (1 << K); ++s) evdata_subset<T, K>(ev, s, pd, mt, wt, c10, c11, c12);
  for (int i = 0; i < K + 2; ++i)
    for (int c = 0; c < 4; ++c) ev.pext[i][c] = (T)pd[i][c];
  ev.mt = (T)mt;
  const T sqh = (T)0.70710676908493042;
  W4<T> g[K];
  for (int q = 0; q < K; ++q) {
    int part = gluon_particle<K>(q);
    g[q] = vxxxxx<T>(ev.pext[part], T(0), (T)hel[part], part < 2 ? T(-1) : T(1), sqh);
  }
  W4<T> wtp = oxxxxx<T>(ev.pext[2], ev.mt, (T)hel[2], T(1));
  W4<T> wtb = ixxxxx<T>(ev.pext[3], ev.mt, (T)hel[3], T(-1));
  cx<T> A[P::NP];
  P::amps(ev, g, wtp, wtb, A);
  cx<double> ampf = mul_mi(c11);  // -i GC_11
  for (int i = 0; i < P::NP; ++i) out[i] = ampf * cx<double>{(double)A[i].re, (double)A[i].im};
}

template <int K, class T> static double smatrix(const double* p, const double* coup, double mt, double wt) {
  using P = HostProc<K, T>;
  double tot = 0.0;
  for (int h = 0; h < P::NC; ++h) {
    double hv[K + 2];
    for (int i = 0; i < K + 2; ++i) hv[i] = P::hel(h)[i];
    cx<double> A[P::NP];
    partials<K, T>(p, hv, coup, mt, wt, A);
    double s = 0.0;
    for (int a = 0; a < P::NP; ++a)
      for (int b = 0; b < P::NP; ++b) {
        cx<double> z = A[a] * conjg(A[b]);
        s += (double)P::col(a * P::NP + b) * z.re;
      }
    tot += s / P::CDEN;
  }
  return tot / P::DEN;
}

extern "C" int me_host_partials(int k, int prec, const double* p, const double* hel, const double* coup, double mt,
                                double wt, double* out) {
  cx<double> A[24];
  int np = k == 2 ? 2 : (k == 3 ? 6 : 24);
  if (k == 2) prec ? partials<2, float>(p, hel, coup, mt, wt, A) : partials<2, double>(p, hel, coup, mt, wt, A);
  else if (k == 3) prec ? partials<3, float>(p, hel, coup, mt, wt, A) : partials<3, double>(p, hel, coup, mt, wt, A);
  else if (k == 4) prec ? partials<4, float>(p, hel, coup, mt, wt, A) : partials<4, double>(p, hel, coup, mt, wt, A);
  else return 1;
  for (int i = 0; i < np; ++i) { out[2 * i] = A[i].re; out[2 * i + 1] = A[i].im; }
  return 0;
}

extern "C" int me_host_smatrix(int k, int prec, const double* p, int64_t N, const double* coup, double mt, double wt,
                               double* out) {
  int np = k + 2;
  for (int64_t e = 0; e < N; ++e) {
    const double* pe = p + 4 * np * e;
    if (k == 2) out[e] = prec ? smatrix<2, float>(pe, coup, mt, wt) : smatrix<2, double>(pe, coup, mt, wt);
    else if (k == 3) out[e] = prec ? smatrix<3, float>(pe, coup, mt, wt) : smatrix<3, double>(pe, coup, mt, wt);
    else if (k == 4) out[e] = prec ? smatrix<4, float>(pe, coup, mt, wt) : smatrix<4, double>(pe, coup, mt, wt);
    else return 1;
  }
  return 0;
}
