// CPU oracle entry points (extern "C", driven through ctypes by the tests and by
// the CPU-baseline leg of bench.py).  TEST INFRASTRUCTURE ONLY.
#include "mf_oracle.hpp"

#include <complex>
#include <cstdio>
#include <memory>
#include <numeric>
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace orc;
typedef Cx<double> C;
typedef WF<double> W;

// ---------------------------------------------------------------------------
// Philox / uniforms
// ---------------------------------------------------------------------------
extern "C" void orc_philox(const uint32_t* ctr, const uint32_t* key, uint32_t* out) { philox4x32_10(ctr, key, out); }

extern "C" void orc_uniforms(uint64_t seed, uint32_t stream, uint32_t iteration, uint64_t event0, int64_t N,
                             int ndim, double* u) {
  for (int64_t e = 0; e < N; ++e) philox_uniforms(seed, stream, iteration, event0 + (uint64_t)e, ndim, u + ndim * e);
}

// ---------------------------------------------------------------------------
// Phase space
// ---------------------------------------------------------------------------
extern "C" int orc_rambo(const double* x, int64_t N, int n, const double* sqrts, const double* masses, int f32q,
                         int rule, double* p, double* w) {
  RefConsts K = ref_consts(f32q != 0);
  bool massive = false;
  std::vector<double> m(n, 0.0);
  if (masses) {
    for (int i = 0; i < n; ++i) {
      m[i] = f32q ? (double)(float)masses[i] : masses[i];
      if (masses[i] != 0.0) massive = true;
    }
  }
  return rambo_batch<double>(x, N, n, sqrts, m.data(), massive, K, (NewtonRule)rule, p, w);
}

// ramboflow (phasespace.py:257-319) for nparticles >= 4.  p: [N][npart][4]
extern "C" int orc_ramboflow(const double* x, int64_t N, int npart, double com_sqrts, const double* masses, int f32q,
                             int rule, double* p, double* w, double* x1, double* x2) {
  RefConsts K = ref_consts(f32q != 0);
  int nout = npart - 2, ndim = 4 * nout + 2;
  double msum = 0.0;
  bool massive = false;
  std::vector<double> m(nout, 0.0);
  if (masses)
    for (int i = 0; i < nout; ++i) {
      msum += masses[i];
      m[i] = f32q ? (double)(float)masses[i] : masses[i];
      if (masses[i] != 0.0) massive = true;
    }
  double shat_min = msum * msum;
  double s_in = com_sqrts * com_sqrts;
  std::vector<double> xr((size_t)N * 4 * nout), roots(N), shat(N), pout((size_t)N * nout * 4), wps(N);
  for (int64_t e = 0; e < N; ++e) {
    const double* xe = x + ndim * e;
    get_x1x2<double>(xe, shat_min, s_in, shat[e], w[e], x1[e], x2[e]);
    roots[e] = std::sqrt(shat[e]);
    std::memcpy(&xr[(size_t)4 * nout * e], xe + 2, sizeof(double) * 4 * nout);
  }
  int it = rambo_batch<double>(xr.data(), N, nout, roots.data(), m.data(), massive, K, (NewtonRule)rule, pout.data(),
                               wps.data());
  for (int64_t e = 0; e < N; ++e) {
    double ein = roots[e] / 2.0;
    double* pe = p + (size_t)4 * npart * e;
    pe[0] = ein; pe[1] = 0; pe[2] = 0; pe[3] = ein;
    pe[4] = ein; pe[5] = 0; pe[6] = 0; pe[7] = -ein;
    std::memcpy(pe + 8, &pout[(size_t)4 * nout * e], sizeof(double) * 4 * nout);
    w[e] = w[e] * wps[e];
    w[e] = w[e] * K.gev2pb;
    w[e] = w[e] / (2.0 * shat[e]);
  }
  return it;
}

extern "C" void orc_boost_to_lab(double* p, int64_t N, int npart, const double* x1, const double* x2) {
  for (int64_t e = 0; e < N; ++e) boost_to_lab<double>(p + (size_t)4 * npart * e, npart, x1[e], x2[e]);
}

// ---------------------------------------------------------------------------
// Wavefunctions and ALOHA routines, batched for the tests.  Wavefunction
// arrays are [N][6] complex = [N][6][2] double.
// ---------------------------------------------------------------------------
static void put(const W& f, double* out) {
  for (int k = 0; k < 6; ++k) { out[2 * k] = f.w[k].re; out[2 * k + 1] = f.w[k].im; }
}
static W get(const double* in) {
  W f;
  for (int k = 0; k < 6; ++k) f.w[k] = C(in[2 * k], in[2 * k + 1]);
  return f;
}
extern "C" void orc_ixxxxx(const double* p, int64_t N, double m, double nhel, double nsf, double* out) {
  for (int64_t e = 0; e < N; ++e) { W f; ixxxxx<double>(p + 4 * e, m, nhel, nsf, f); put(f, out + 12 * e); }
}
extern "C" void orc_oxxxxx(const double* p, int64_t N, double m, double nhel, double nsf, double* out) {
  for (int64_t e = 0; e < N; ++e) { W f; oxxxxx<double>(p + 4 * e, m, nhel, nsf, f); put(f, out + 12 * e); }
}
extern "C" void orc_vxxxxx(const double* p, int64_t N, double m, double nhel, double nsv, int f32q, double* out) {
  double sqh = ref_consts(f32q != 0).sqh;
  for (int64_t e = 0; e < N; ++e) { W f; vxxxxx<double>(p + 4 * e, m, nhel, nsv, sqh, f); put(f, out + 12 * e); }
}
extern "C" void orc_sxxxxx(const double* p, int64_t N, double nss, double* out) {
  for (int64_t e = 0; e < N; ++e) {
    C s[3];
    sxxxxx<double>(p + 4 * e, nss, s);
    for (int k = 0; k < 3; ++k) { out[6 * e + 2 * k] = s[k].re; out[6 * e + 2 * k + 1] = s[k].im; }
  }
}
extern "C" void orc_FFV1_0(const double* F1, const double* F2, const double* V3, const double* coup, int64_t N,
                           double* out) {
  for (int64_t e = 0; e < N; ++e) {
    C a = FFV1_0<double>(get(F1 + 12 * e), get(F2 + 12 * e), get(V3 + 12 * e), C(coup[0], coup[1]));
    out[2 * e] = a.re; out[2 * e + 1] = a.im;
  }
}
extern "C" void orc_FFV1_1(const double* F2, const double* V3, const double* coup, double M, double Wd, int64_t N,
                           double* out) {
  for (int64_t e = 0; e < N; ++e) { W f; FFV1_1<double>(get(F2 + 12 * e), get(V3 + 12 * e), C(coup[0], coup[1]), M, Wd, f); put(f, out + 12 * e); }
}
extern "C" void orc_FFV1_2(const double* F1, const double* V3, const double* coup, double M, double Wd, int64_t N,
                           double* out) {
  for (int64_t e = 0; e < N; ++e) { W f; FFV1_2<double>(get(F1 + 12 * e), get(V3 + 12 * e), C(coup[0], coup[1]), M, Wd, f); put(f, out + 12 * e); }
}
extern "C" void orc_VVV1P0_1(const double* V2, const double* V3, const double* coup, double M, double Wd, int64_t N,
                             double* out) {
  for (int64_t e = 0; e < N; ++e) { W f; VVV1P0_1<double>(get(V2 + 12 * e), get(V3 + 12 * e), C(coup[0], coup[1]), M, Wd, f); put(f, out + 12 * e); }
}

// ---------------------------------------------------------------------------
// gg -> tt~ exactly as the frozen module (tests/mockup_debug_me.py:483-543)
// ---------------------------------------------------------------------------
static const double kHelGGTTX[16][4] = {
    {-1, -1, -1, 1}, {-1, -1, -1, -1}, {-1, -1, 1, 1}, {-1, -1, 1, -1}, {-1, 1, -1, 1}, {-1, 1, -1, -1},
    {-1, 1, 1, 1},   {-1, 1, 1, -1},   {1, -1, -1, 1}, {1, -1, -1, -1}, {1, -1, 1, 1},  {1, -1, 1, -1},
    {1, 1, -1, 1},   {1, 1, -1, -1},   {1, 1, 1, 1},   {1, 1, 1, -1}};

template <class R>
static R ggttx_matrix(const R* p /*[4][4]*/, const R* hel, R MT, R WT, Cx<R> GC10, Cx<R> GC11, R sqh) {
  WF<R> w0, w1, w2, w3, w4;
  R zero(0.0);
  vxxxxx<R>(p + 0, zero, hel[0], R(-1.0), sqh, w0);
  vxxxxx<R>(p + 4, zero, hel[1], R(-1.0), sqh, w1);
  oxxxxx<R>(p + 8, MT, hel[2], R(1.0), w2);
  ixxxxx<R>(p + 12, MT, hel[3], R(-1.0), w3);
  VVV1P0_1<R>(w0, w1, GC10, zero, zero, w4);
  Cx<R> amp0 = FFV1_0<R>(w3, w2, w4, GC11);
  FFV1_1<R>(w2, w0, GC11, MT, WT, w4);
  Cx<R> amp1 = FFV1_0<R>(w3, w4, w1, GC11);
  FFV1_2<R>(w3, w0, GC11, MT, WT, w4);
  Cx<R> amp2 = FFV1_0<R>(w4, w2, w1, GC11);
  Cx<R> jamp[2] = {mul_i(amp0) - amp1, mul_mi(amp0) - amp2};
  const R cf[2][2] = {{R(16.0), R(-2.0)}, {R(-2.0), R(16.0)}};
  Cx<R> m;
  for (int i = 0; i < 2; ++i) {
    Cx<R> zt;
    for (int j = 0; j < 2; ++j) zt = zt + cf[i][j] * jamp[j];
    m = m + (zt * conj(jamp[i])) / Cx<R>(R(3.0));
  }
  return m.re;
}

extern "C" void orc_smatrix_ggttx(const double* p, int64_t N, const double* prm, int f32q, double* out,
                                  double* hel_out) {
  double sqh = ref_consts(f32q != 0).sqh;
  C gc10(prm[2], prm[3]), gc11(prm[4], prm[5]);
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < N; ++e) {
    double ans = 0.0;
    for (int h = 0; h < 16; ++h) {
      double t = ggttx_matrix<double>(p + 16 * e, kHelGGTTX[h], prm[0], prm[1], gc10, gc11, sqh);
      if (hel_out) hel_out[h * N + e] = t;
      ans += t;
    }
    out[e] = ans / 256.0;
  }
}

// ---------------------------------------------------------------------------
// g g -> t t~ + (k-2) g through colour-ordered Berends-Giele recursion.
// Particle order as MadGraph emits it: 0,1 incoming gluons, 2 = t, 3 = t~,
// 4.. outgoing gluons.  Gluon label j in 0..k-1 maps to particle
// {0,1,4,5,6}[j].  A(sigma) multiplies (T^{a_sigma1} ... T^{a_sigmak})_{i_t j_tbar}.
// ---------------------------------------------------------------------------
struct TTNGPlan {
  int k = 0, nperm = 0, njnode = 0, nonode = 0;
  std::vector<std::vector<int>> jseq;              // J node -> gluon sequence
  std::vector<std::vector<std::pair<int, int>>> j2;  // 2-splits (left, right)
  std::vector<std::vector<std::array<int, 3>>> j3;   // 3-splits
  std::vector<std::vector<std::pair<int, int>>> oterms;  // O node: (O prefix, J block)
  std::vector<std::vector<std::pair<int, int>>> aterms;  // amplitude sigma: (O prefix, J block)
  std::vector<double> colour;                        // nperm x nperm
  std::vector<std::vector<double>> hels;             // ncomb x npart
  int npart = 0, ncomb = 0;
  double denominator = 0;
};

static int gluon_particle(int j) { return j < 2 ? j : j + 2; }

static void build_plan(TTNGPlan& P, int k) {
  P.k = k;
  P.npart = k + 2;
  std::map<std::vector<int>, int> jid, oid;
  // all ordered sequences of distinct labels, by length
  std::vector<std::vector<int>> bylen{{}};
  std::vector<std::vector<int>> frontier{{}};
  for (int len = 1; len <= k; ++len) {
    std::vector<std::vector<int>> next;
    for (auto& s : frontier)
      for (int g = 0; g < k; ++g)
        if (std::find(s.begin(), s.end(), g) == s.end()) {
          auto t = s;
          t.push_back(g);
          next.push_back(t);
        }
    for (auto& s : next) {
      int id = (int)P.jseq.size();
      jid[s] = id;
      P.jseq.push_back(s);
    }
    frontier = next;
  }
  P.njnode = (int)P.jseq.size();
  P.j2.resize(P.njnode);
  P.j3.resize(P.njnode);
  for (int id = 0; id < P.njnode; ++id) {
    auto& s = P.jseq[id];
    int L = (int)s.size();
    for (int i = 1; i < L; ++i)
      P.j2[id].push_back({jid[std::vector<int>(s.begin(), s.begin() + i)], jid[std::vector<int>(s.begin() + i, s.end())]});
    for (int i = 1; i < L; ++i)
      for (int j = i + 1; j < L; ++j)
        P.j3[id].push_back({jid[std::vector<int>(s.begin(), s.begin() + i)],
                            jid[std::vector<int>(s.begin() + i, s.begin() + j)],
                            jid[std::vector<int>(s.begin() + j, s.end())]});
  }
  // O nodes: prefixes of length 0..k-1
  std::vector<std::vector<int>> oseq{{}};
  oid[{}] = 0;
  P.oterms.push_back({});
  for (int id = 0; id < P.njnode; ++id) {
    auto& s = P.jseq[id];
    if ((int)s.size() >= k) continue;
    int o = (int)P.oterms.size();
    oid[s] = o;
    std::vector<std::pair<int, int>> terms;
    for (int i = 0; i < (int)s.size(); ++i)
      terms.push_back({oid[std::vector<int>(s.begin(), s.begin() + i)], jid[std::vector<int>(s.begin() + i, s.end())]});
    P.oterms.push_back(terms);
  }
  P.nonode = (int)P.oterms.size();
  // permutations in lexicographic order
  std::vector<int> sig(k);
  std::iota(sig.begin(), sig.end(), 0);
  do {
    std::vector<std::pair<int, int>> terms;
    for (int i = 0; i < k; ++i)
      terms.push_back({oid[std::vector<int>(sig.begin(), sig.begin() + i)], jid[std::vector<int>(sig.begin() + i, sig.end())]});
    P.aterms.push_back(terms);
  } while (std::next_permutation(sig.begin(), sig.end()));
  P.nperm = (int)P.aterms.size();
  // helicities: MadGraph order, the t~ (particle 3) runs +1 then -1
  P.ncomb = 1 << P.npart;
  for (int c = 0; c < P.ncomb; ++c) {
    std::vector<double> h(P.npart);
    for (int i = 0; i < P.npart; ++i) {
      int bit = (c >> (P.npart - 1 - i)) & 1;
      double v = bit ? 1.0 : -1.0;
      if (i == 3) v = -v;
      h[i] = v;
    }
    P.hels.push_back(h);
  }
  double iden = 1.0;
  for (int i = 2; i <= k - 2; ++i) iden *= i;
  P.denominator = 256.0 * iden;
}

// --- SU(3) generators (T = lambda/2) and structure constants
struct SU3 {
  std::complex<double> T[8][3][3];
  double f[8][8][8];
  SU3() {
    typedef std::complex<double> c;
    c I(0, 1);
    c L[8][3][3] = {};
    L[0][0][1] = 1; L[0][1][0] = 1;
    L[1][0][1] = -I; L[1][1][0] = I;
    L[2][0][0] = 1; L[2][1][1] = -1;
    L[3][0][2] = 1; L[3][2][0] = 1;
    L[4][0][2] = -I; L[4][2][0] = I;
    L[5][1][2] = 1; L[5][2][1] = 1;
    L[6][1][2] = -I; L[6][2][1] = I;
    L[7][0][0] = 1.0 / std::sqrt(3.0); L[7][1][1] = 1.0 / std::sqrt(3.0); L[7][2][2] = -2.0 / std::sqrt(3.0);
    for (int a = 0; a < 8; ++a)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T[a][i][j] = 0.5 * L[a][i][j];
    // f^{abc} = -2 i Tr([T^a, T^b] T^c)
    for (int a = 0; a < 8; ++a)
      for (int b = 0; b < 8; ++b)
        for (int cc = 0; cc < 8; ++cc) {
          c tr = 0;
          for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
              for (int l = 0; l < 3; ++l) tr += (T[a][i][j] * T[b][j][l] - T[b][i][j] * T[a][j][l]) * T[cc][l][i];
          f[a][b][cc] = (-2.0 * I * tr).real();
        }
  }
};
static const SU3& su3() {
  static SU3 s;
  return s;
}

// C_{sigma,tau} = sum over adjoint labels of Tr(T^{s1}..T^{sk} T^{tk}..T^{t1}),
// evaluated numerically with explicit generators (row sigma = identity, then
// C_{sigma,tau} = C_{id, sigma^-1 tau}).
extern "C" void orc_colour_matrix(int k, double* Cout) {
  typedef std::complex<double> c;
  const SU3& S = su3();
  std::vector<std::vector<int>> perms;
  std::vector<int> sig(k);
  std::iota(sig.begin(), sig.end(), 0);
  do perms.push_back(sig);
  while (std::next_permutation(sig.begin(), sig.end()));
  int np = (int)perms.size();
  int nb = 1;
  for (int i = 0; i < k; ++i) nb *= 8;
  // partial rows over fixed blocks of colour assignments, summed in block
  // order: the same matrix for any number of threads
  constexpr int kBlocks = 64;
  std::vector<double> part((size_t)kBlocks * np, 0.0);
#pragma omp parallel for schedule(dynamic, 1)
  for (int blk = 0; blk < kBlocks; ++blk) {
    double* rowp = &part[(size_t)blk * np];
    for (int bi = blk; bi < nb; bi += kBlocks) {
      int b[8];
      int t = bi;
      for (int i = 0; i < k; ++i) { b[i] = t % 8; t /= 8; }
      c X[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
      for (int i = 0; i < k; ++i) {
        c Y[3][3] = {};
        for (int r = 0; r < 3; ++r)
          for (int s = 0; s < 3; ++s)
            for (int u = 0; u < 3; ++u) Y[r][s] += X[r][u] * S.T[b[i]][u][s];
        std::memcpy(X, Y, sizeof(X));
      }
      for (int pi = 0; pi < np; ++pi) {
        // Y = (T^{b_pi(1)} ... T^{b_pi(k)}); contribution Tr(X Y^dagger)
        c Y[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
        for (int i = 0; i < k; ++i) {
          c Z[3][3] = {};
          for (int r = 0; r < 3; ++r)
            for (int s = 0; s < 3; ++s)
              for (int u = 0; u < 3; ++u) Z[r][s] += Y[r][u] * S.T[b[perms[pi][i]]][u][s];
          std::memcpy(Y, Z, sizeof(Y));
        }
        c tr = 0;
        for (int r = 0; r < 3; ++r)
          for (int s = 0; s < 3; ++s) tr += X[r][s] * std::conj(Y[r][s]);
        rowp[pi] += tr.real();
      }
    }
  }
  std::vector<double> row(np, 0.0);
  for (int blk = 0; blk < kBlocks; ++blk)
    for (int pi = 0; pi < np; ++pi) row[pi] += part[(size_t)blk * np + pi];
  // index of sigma^-1 tau
  std::map<std::vector<int>, int> idx;
  for (int i = 0; i < np; ++i) idx[perms[i]] = i;
  for (int s = 0; s < np; ++s) {
    std::vector<int> inv(k);
    for (int i = 0; i < k; ++i) inv[perms[s][i]] = i;
    for (int t = 0; t < np; ++t) {
      std::vector<int> comp(k);
      for (int i = 0; i < k; ++i) comp[i] = inv[perms[t][i]];
      Cout[s * np + t] = row[idx[comp]];
    }
  }
}

struct TTNGParams {
  double MT, WT;
  C gc10, gc11, gc12;
  C c3, c4;  // colour-ordered vertex factors
  double sqh;
};

// Colour-ordered partial amplitudes for one event and one helicity.
template <class R>
static void ttng_partials(const TTNGPlan& P, const R* p, const double* hel, const TTNGParams& Q, Cx<R>* amps,
                          std::vector<WF<R>>& J, std::vector<WF<R>>& O) {
  int k = P.k;
  R zero(0.0), MT(Q.MT), WT(Q.WT), sqh(Q.sqh);
  Cx<R> gc11(R(Q.gc11.re), R(Q.gc11.im));
  Cx<R> c3g = Cx<R>(R(Q.c3.re), R(Q.c3.im)) * Cx<R>(R(Q.gc10.re), R(Q.gc10.im));
  Cx<R> c4g = Cx<R>(R(Q.c4.re), R(Q.c4.im)) * Cx<R>(R(Q.gc12.re), R(Q.gc12.im));
  WF<R> wt, wtb;
  oxxxxx<R>(p + 8, MT, R(hel[2]), R(1.0), wt);
  ixxxxx<R>(p + 12, MT, R(hel[3]), R(-1.0), wtb);
  J.resize(P.njnode);
  O.resize(P.nonode);
  for (int id = 0; id < P.njnode; ++id) {
    const auto& s = P.jseq[id];
    if (s.size() == 1) {
      int part = gluon_particle(s[0]);
      vxxxxx<R>(p + 4 * part, zero, R(hel[part]), R(part < 2 ? -1.0 : 1.0), sqh, J[id]);
      continue;
    }
    WF<R> acc, t;
    bool first = true;
    for (auto& sp : P.j2[id]) {
      VVV1P0_1<R>(J[sp.first], J[sp.second], c3g, zero, zero, t);
      if (first) { acc = t; first = false; }
      else for (int c = 2; c < 6; ++c) acc.w[c] += t.w[c];
    }
    for (auto& sp : P.j3[id]) {
      VVVV_ord_1<R>(J[sp[0]], J[sp[1]], J[sp[2]], c4g, t);
      for (int c = 2; c < 6; ++c) acc.w[c] += t.w[c];
    }
    J[id] = acc;
  }
  O[0] = wt;
  for (int o = 1; o < P.nonode; ++o) {
    WF<R> acc, t;
    bool first = true;
    for (auto& tm : P.oterms[o]) {
      FFV1_1<R>(O[tm.first], J[tm.second], gc11, MT, WT, t);
      if (first) { acc = t; first = false; }
      else for (int c = 2; c < 6; ++c) acc.w[c] += t.w[c];
    }
    O[o] = acc;
  }
  for (int s = 0; s < P.nperm; ++s) {
    Cx<R> a;
    for (auto& tm : P.aterms[s]) a += FFV1_0<R>(wtb, O[tm.first], J[tm.second], gc11);
    amps[s] = a;
  }
}

template <class R>
static R colour_sum(const TTNGPlan& P, const Cx<R>* A) {
  R m(0.0);
  int np = P.nperm;
  for (int i = 0; i < np; ++i) {
    Cx<R> zt;
    for (int j = 0; j < np; ++j) {
      double c = P.colour[i * np + j];
      if (c != 0.0) zt += R(c) * A[j];
    }
    m += (zt * conj(A[i])).re;
  }
  return m;
}

extern "C" void* orc_ttng_create(int k, const double* colour) {
  auto* P = new TTNGPlan();
  build_plan(*P, k);
  P->colour.resize((size_t)P->nperm * P->nperm);
  if (colour) std::memcpy(P->colour.data(), colour, sizeof(double) * P->colour.size());
  else orc_colour_matrix(k, P->colour.data());
  return P;
}
extern "C" void orc_ttng_destroy(void* h) { delete (TTNGPlan*)h; }
extern "C" void orc_ttng_info(void* h, int* out) {
  auto* P = (TTNGPlan*)h;
  out[0] = P->k; out[1] = P->nperm; out[2] = P->njnode; out[3] = P->nonode; out[4] = P->ncomb; out[5] = P->npart;
}
extern "C" void orc_ttng_colour(void* h, double* out) {
  auto* P = (TTNGPlan*)h;
  std::memcpy(out, P->colour.data(), sizeof(double) * P->colour.size());
}
extern "C" void orc_ttng_helicities(void* h, double* out) {
  auto* P = (TTNGPlan*)h;
  for (int c = 0; c < P->ncomb; ++c)
    for (int i = 0; i < P->npart; ++i) out[c * P->npart + i] = P->hels[c][i];
}
extern "C" double orc_ttng_denominator(void* h) { return ((TTNGPlan*)h)->denominator; }

static TTNGParams make_params(const double* prm, int f32q) {
  // prm: MT, WT, GC10 (re, im), GC11 (re, im), GC12 (re, im), c3 (re, im), c4 (re, im)
  TTNGParams Q;
  Q.MT = prm[0]; Q.WT = prm[1];
  Q.gc10 = C(prm[2], prm[3]); Q.gc11 = C(prm[4], prm[5]); Q.gc12 = C(prm[6], prm[7]);
  Q.c3 = C(prm[8], prm[9]); Q.c4 = C(prm[10], prm[11]);
  Q.sqh = ref_consts(f32q != 0).sqh;
  return Q;
}

// partial amplitudes for one event and a given helicity vector: out[nperm][2]
extern "C" void orc_ttng_partials(void* h, const double* p, const double* hel, const double* prm, int f32q,
                                  double* out) {
  auto* P = (TTNGPlan*)h;
  TTNGParams Q = make_params(prm, f32q);
  std::vector<W> J, O;
  std::vector<C> A(P->nperm);
  ttng_partials<double>(*P, p, hel, Q, A.data(), J, O);
  for (int s = 0; s < P->nperm; ++s) { out[2 * s] = A[s].re; out[2 * s + 1] = A[s].im; }
}

extern "C" void orc_ttng_smatrix(void* h, const double* p, int64_t N, const double* prm, int f32q, double* out,
                                 double* hel_out) {
  auto* P = (TTNGPlan*)h;
  TTNGParams Q = make_params(prm, f32q);
  int np = P->npart;
#pragma omp parallel
  {
    std::vector<W> J, O;
    std::vector<C> A(P->nperm);
#pragma omp for schedule(dynamic, 16)
    for (int64_t e = 0; e < N; ++e) {
      double ans = 0.0;
      for (int c = 0; c < P->ncomb; ++c) {
        ttng_partials<double>(*P, p + (size_t)4 * np * e, P->hels[c].data(), Q, A.data(), J, O);
        double t = colour_sum<double>(*P, A.data());
        if (hel_out) hel_out[(size_t)c * N + e] = t;
        ans += t;
      }
      out[e] = ans / P->denominator;
    }
  }
}

// Operation count of the colour-ordered evaluation of one event (all
// helicities, no sharing between helicities), with complex mul = 6 real
// flops, complex add = 2, and sqrt/log/div = 1 each.
extern "C" double orc_ttng_flops(void* h, const double* p, const double* prm) {
  auto* P = (TTNGPlan*)h;
  TTNGParams Q = make_params(prm, 1);
  std::vector<WF<Flop>> J, O;
  std::vector<Cx<Flop>> A(P->nperm);
  std::vector<Flop> pf(4 * P->npart);
  for (int i = 0; i < 4 * P->npart; ++i) pf[i] = Flop(p[i]);
  Flop::count = 0;
  Flop ans(0.0);
  for (int c = 0; c < P->ncomb; ++c) {
    ttng_partials<Flop>(*P, pf.data(), P->hels[c].data(), Q, A.data(), J, O);
    ans += colour_sum<Flop>(*P, A.data());
  }
  ans = ans / Flop(P->denominator);
  return (double)Flop::count;
}
extern "C" double orc_ggttx_flops(const double* p, const double* prm) {
  std::vector<Flop> pf(16);
  for (int i = 0; i < 16; ++i) pf[i] = Flop(p[i]);
  Flop::count = 0;
  Flop ans(0.0);
  Cx<Flop> g10{Flop{prm[2]}, Flop{prm[3]}}, g11{Flop{prm[4]}, Flop{prm[5]}};
  for (int h = 0; h < 16; ++h) {
    Flop hel[4] = {kHelGGTTX[h][0], kHelGGTTX[h][1], kHelGGTTX[h][2], kHelGGTTX[h][3]};
    ans += ggttx_matrix<Flop>(pf.data(), hel, Flop(prm[0]), Flop(prm[1]), g10, g11, Flop(ref_consts(true).sqh));
  }
  ans = ans / Flop(256.0);
  return (double)Flop::count;
}

// ---------------------------------------------------------------------------
// Colour-dressed recursion with the full QCD Feynman rules, explicit colours:
// an independent check of the colour-ordered decomposition.  colours:
// [a_0 .. a_{k-1}] adjoint labels of the gluons (label order), then i_t, j_tbar.
// Vertex factors: s3 * GC10 * f^{abc} VVV1, T^a_{c c'} GC11 FFV1 along the
// quark line from the top, and kappa * GC12 * (f f) for the four-gluon vertex.
// ---------------------------------------------------------------------------
namespace {
struct GCur { W v[8]; bool nz[8]; };
struct FCur { W v[3]; bool nz[3]; };
}
static W zero_wf_mom(const W& like) { W z = like; for (int c = 2; c < 6; ++c) z.w[c] = C(); return z; }

extern "C" void orc_ttng_dressed(int k, const double* p, const double* hel, const int* colours, const double* prm,
                                 double s3, double kre, double kim, int f32q, double* out) {
  const SU3& S = su3();
  TTNGParams Q = make_params(prm, f32q);
  int nsub = 1 << k;
  std::vector<GCur> G(nsub);
  std::vector<W> ext(k);
  for (int j = 0; j < k; ++j) {
    int part = gluon_particle(j);
    vxxxxx<double>(p + 4 * part, 0.0, hel[part], part < 2 ? -1.0 : 1.0, Q.sqh, ext[j]);
  }
  C g3 = C(s3) * Q.gc10;
  C g4 = C(kre, kim) * Q.gc12;
  auto mom_wf = [&](int s) {
    W z;
    for (int j = 0; j < k; ++j)
      if (s >> j & 1) { z.w[0] += ext[j].w[0]; z.w[1] += ext[j].w[1]; }
    return z;
  };
  for (int s = 1; s < nsub; ++s) {
    GCur& g = G[s];
    W base = mom_wf(s);
    for (int a = 0; a < 8; ++a) { g.v[a] = base; g.nz[a] = false; }
    int pc = __builtin_popcount(s);
    if (pc == 1) {
      int j = __builtin_ctz(s);
      g.v[colours[j]] = ext[j];
      g.nz[colours[j]] = true;
      continue;
    }
    // unordered 2-partitions: s1 contains the lowest set bit of s
    int low = s & -s;
    for (int s1 = (s - 1) & s; s1 > 0; s1 = (s1 - 1) & s) {
      if (!(s1 & low)) continue;
      int s2 = s ^ s1;
      for (int b = 0; b < 8; ++b) {
        if (!G[s1].nz[b]) continue;
        for (int c = 0; c < 8; ++c) {
          if (!G[s2].nz[c]) continue;
          W t;
          VVV1P0_1<double>(G[s1].v[b], G[s2].v[c], g3, 0.0, 0.0, t);
          for (int a = 0; a < 8; ++a) {
            double f = S.f[a][b][c];
            if (f == 0.0) continue;
            for (int q = 2; q < 6; ++q) g.v[a].w[q] += C(f) * t.w[q];
            g.nz[a] = true;
          }
        }
      }
    }
    // unordered 3-partitions {s1, s2, s3}: s1 holds the lowest bit, s2 the lowest of the rest
    for (int s1 = s; s1 > 0; s1 = (s1 - 1) & s) {
      if (!(s1 & low) || s1 == s) continue;
      int rest = s ^ s1;
      int low2 = rest & -rest;
      for (int s2 = rest; s2 > 0; s2 = (s2 - 1) & rest) {
        if (!(s2 & low2) || s2 == rest) continue;
        int s3s = rest ^ s2;
        int parts[3] = {s1, s2, s3s};
        // momentum of the off-shell leg and propagator
        W V1 = mom_wf(s);
        double P1[4];
        mom_of<double>(V1, P1);
        for (int q = 0; q < 4; ++q) P1[q] = -P1[q];
        C den = prop_denom<double>(g4, P1, 0.0, 0.0);
        C ci = mul_i(den);
        for (int b = 0; b < 8; ++b) {
          if (!G[parts[0]].nz[b]) continue;
          for (int c = 0; c < 8; ++c) {
            if (!G[parts[1]].nz[c]) continue;
            for (int d = 0; d < 8; ++d) {
              if (!G[parts[2]].nz[d]) continue;
              const C* Vb = G[parts[0]].v[b].w + 2;
              const C* Vc = G[parts[1]].v[c].w + 2;
              const C* Vd = G[parts[2]].v[d].w + 2;
              C bd = mdot<double>(Vb, Vd), bc = mdot<double>(Vb, Vc), cd = mdot<double>(Vc, Vd);
              for (int a = 0; a < 8; ++a) {
                double f1 = 0, f2 = 0, f3 = 0;
                for (int e = 0; e < 8; ++e) {
                  f1 += S.f[a][b][e] * S.f[c][d][e];
                  f2 += S.f[a][c][e] * S.f[b][d][e];
                  f3 += S.f[a][d][e] * S.f[b][c][e];
                }
                if (f1 == 0 && f2 == 0 && f3 == 0) continue;
                for (int q = 0; q < 4; ++q) {
                  C term = C(f1) * (Vc[q] * bd - Vd[q] * bc) + C(f2) * (Vb[q] * cd - Vd[q] * bc) +
                           C(f3) * (Vb[q] * cd - Vc[q] * bd);
                  g.v[a].w[2 + q] += ci * term;
                }
                g.nz[a] = true;
              }
            }
          }
        }
      }
    }
  }
  // quark line from the top
  W wt, wtb;
  oxxxxx<double>(p + 8, Q.MT, hel[2], 1.0, wt);
  ixxxxx<double>(p + 12, Q.MT, hel[3], -1.0, wtb);
  std::vector<FCur> O(nsub);
  for (int c = 0; c < 3; ++c) { O[0].v[c] = zero_wf_mom(wt); O[0].nz[c] = false; }
  O[0].v[colours[k]] = wt;
  O[0].nz[colours[k]] = true;
  int full = nsub - 1;
  for (int s = 1; s < full; ++s) {
    FCur& o = O[s];
    bool init = false;
    for (int c = 0; c < 3; ++c) o.nz[c] = false;
    for (int b = s; b > 0; b = (b - 1) & s) {
      int a = s ^ b;
      for (int cc = 0; cc < 3; ++cc) {
        if (!O[a].nz[cc]) continue;
        for (int g = 0; g < 8; ++g) {
          if (!G[b].nz[g]) continue;
          W t;
          FFV1_1<double>(O[a].v[cc], G[b].v[g], Q.gc11, Q.MT, Q.WT, t);
          if (!init) { for (int c2 = 0; c2 < 3; ++c2) o.v[c2] = zero_wf_mom(t); init = true; }
          for (int c2 = 0; c2 < 3; ++c2) {
            std::complex<double> T = S.T[g][cc][c2];
            if (T == 0.0) continue;
            C tc(T.real(), T.imag());
            for (int q = 2; q < 6; ++q) o.v[c2].w[q] += tc * t.w[q];
            o.nz[c2] = true;
          }
        }
      }
    }
  }
  C amp;
  for (int b = full; b > 0; b = (b - 1) & full) {
    int a = full ^ b;
    for (int cc = 0; cc < 3; ++cc) {
      if (!O[a].nz[cc]) continue;
      for (int g = 0; g < 8; ++g) {
        if (!G[b].nz[g]) continue;
        std::complex<double> T = S.T[g][cc][colours[k + 1]];
        if (T == 0.0) continue;
        amp += C(T.real(), T.imag()) * FFV1_0<double>(wtb, O[a].v[cc], G[b].v[g], Q.gc11);
      }
    }
  }
  out[0] = amp.re;
  out[1] = amp.im;
}

// (T^{a_s1} ... T^{a_sk})_{i j} for explicit labels: out[2]
extern "C" void orc_colour_string(int k, const int* labels_in_order, int i, int j, double* out) {
  const SU3& S = su3();
  std::complex<double> X[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int m = 0; m < k; ++m) {
    std::complex<double> Y[3][3] = {};
    for (int r = 0; r < 3; ++r)
      for (int s = 0; s < 3; ++s)
        for (int u = 0; u < 3; ++u) Y[r][s] += X[r][u] * S.T[labels_in_order[m]][u][s];
    std::memcpy(X, Y, sizeof(X));
  }
  out[0] = X[i][j].real();
  out[1] = X[i][j].imag();
}

// ---------------------------------------------------------------------------
// Synthetic gluon PDF: x g(x) = A x^-0.2 (1-x)^5, A fixed by the momentum sum
// rule int_0^1 x g dx = 1/2, tabulated on 100 log-x nodes in [1e-6, 1] and 50
// log-Q^2 nodes in [1, 1e10] GeV^2, read back by bicubic convolution
// (Keys 1981, a = -1/2) in (log x, log Q^2) with clamped edge nodes.
// ---------------------------------------------------------------------------
static const int kNX = 100, kNQ = 50;
static double pdf_A() { return 0.5 / std::exp(std::lgamma(0.8) + std::lgamma(6.0) - std::lgamma(6.8)); }
// q q~ > t t~ (one diagram, an s-channel gluon), the light-quark channel of
// p p > t t~ at leading order.  No instance exists in the reference's tests;
// the evaluation follows the HELAS calls MadGraph makes for it (wavefunctions
// of wavefunctions_flow.py, FFV1P0_3 and FFV1_0 above) and the colour
// algebra T^a_ij T^a_kl = (d_il d_kj - d_ij d_kl / 3) / 2, which gives the
// colour sum 2 |amp|^2.  p [N][4][4] (q, q~, t, t~), prm = {MT, WT, GC_11 re,
// im}; out [N] = |M|^2 averaged over the initial spins (4) and colours (9).
template <class R> static R smatrix_uux_ttx(const R* p, const double* prm) {
  const R mt = R(prm[0]);
  const Cx<R> g11{R(prm[2]), R(prm[3])};
  R tot = R(0);
  for (int h0 = -1; h0 <= 1; h0 += 2)
    for (int h1 = -1; h1 <= 1; h1 += 2)
      for (int h2 = -1; h2 <= 1; h2 += 2)
        for (int h3 = -1; h3 <= 1; h3 += 2) {
          WF<R> wq, wqb, wt, wtb, g;
          ixxxxx<R>(p + 0, R(0), R(h0), R(1), wq);
          oxxxxx<R>(p + 4, R(0), R(h1), R(-1), wqb);
          oxxxxx<R>(p + 8, mt, R(h2), R(1), wt);
          ixxxxx<R>(p + 12, mt, R(h3), R(-1), wtb);
          FFV1P0_3<R>(wq, wqb, g11, R(0), R(0), g);
          Cx<R> amp = FFV1_0<R>(wtb, wt, g, g11);
          tot += amp.re * amp.re + amp.im * amp.im;
        }
  return tot * R(2.0) / R(36.0);
}

extern "C" void orc_smatrix_uux_ttx(const double* p, int64_t N, const double* prm, double* out) {
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < N; ++e) out[e] = smatrix_uux_ttx<double>(p + 16 * e, prm);
}

// ---------------------------------------------------------------------------
// p p > t t~ j at leading order: the channels with one light-quark line,
// q q~ > t t~ g, q g > t t~ q and q~ g > t t~ q~ (MadGraph's u u~ > t t~ g,
// u g > t t~ u, u~ g > t t~ u~ modules of a p p > t t~ j run; no instance in
// the reference's tests).  Five diagrams each, with the HELAS wavefunctions
// of wavefunctions_flow.py and the ALOHA routines above.  The light line runs
// from its i-type end I (ixxxxx: incoming quark or outgoing antiquark) to its
// o-type end O (oxxxxx: outgoing quark or incoming antiquark), the top line
// from the t~ (I_tb) to the t (O_t):
//   a1: gluon on the light line at I      colour (T^b T^a)_{O I} T^b_{t tb}
//   a2: gluon on the light line at O      colour (T^a T^b)_{O I} T^b_{t tb}
//   a3: gluon on the top line at the t    colour T^b_{O I} (T^a T^b)_{t tb}
//   a4: gluon on the top line at the t~   colour T^b_{O I} (T^b T^a)_{t tb}
//   a5: three-gluon vertex               colour f^{bac} T^b_{O I} T^c_{t tb}
// The colour matrix of these tensors, CM[d][d'] = sum over colours of
// C_d conj(C_d') (Gell-Mann generators, T^a = lambda^a / 2), is
//   [8/3 -1/3 7/3 -2/3 -3i; -1/3 8/3 -2/3 7/3 3i; 7/3 -2/3 8/3 -1/3 -3i;
//    -2/3 7/3 -1/3 8/3 3i; 3i -3i 3i -3i 6],
// with a5 = FFV1_0(I_tb, O_t, VVV1P0_1(V_light, G, GC_10), GC_11) as it
// stands (the sum agrees with an evaluation of the textbook Feynman rules,
// test).  Averages: 1/36 for q q~, 1/96 for q g and q~ g.
static const double kQQ3CmRe[5][5] = {{8.0 / 3, -1.0 / 3, 7.0 / 3, -2.0 / 3, 0},
                                      {-1.0 / 3, 8.0 / 3, -2.0 / 3, 7.0 / 3, 0},
                                      {7.0 / 3, -2.0 / 3, 8.0 / 3, -1.0 / 3, 0},
                                      {-2.0 / 3, 7.0 / 3, -1.0 / 3, 8.0 / 3, 0},
                                      {0, 0, 0, 0, 6}};
static const double kQQ3CmIm[5][5] = {{0, 0, 0, 0, -3}, {0, 0, 0, 0, 3}, {0, 0, 0, 0, -3}, {0, 0, 0, 0, 3},
                                      {3, -3, 3, -3, 0}};

template <class R>
static R qq3_helicity_sum(const WF<R> I[2], const WF<R> O[2], const WF<R> Ot[2], const WF<R> Itb[2],
                          const WF<R> G[2], Cx<R> gc10, Cx<R> gc11, R mt, R wt) {
  R tot = R(0);
  for (int hi = 0; hi < 2; ++hi)
    for (int ho = 0; ho < 2; ++ho) {
      WF<R> vs0;
      FFV1P0_3<R>(I[hi], O[ho], gc11, R(0), R(0), vs0);
      for (int hg = 0; hg < 2; ++hg) {
        WF<R> i1, o2, vs1, vs2, vs5;
        FFV1_2<R>(I[hi], G[hg], gc11, R(0), R(0), i1);
        FFV1P0_3<R>(i1, O[ho], gc11, R(0), R(0), vs1);
        FFV1_1<R>(O[ho], G[hg], gc11, R(0), R(0), o2);
        FFV1P0_3<R>(I[hi], o2, gc11, R(0), R(0), vs2);
        VVV1P0_1<R>(vs0, G[hg], gc10, R(0), R(0), vs5);
        for (int ht = 0; ht < 2; ++ht)
          for (int hb = 0; hb < 2; ++hb) {
            WF<R> ot3, itb4;
            FFV1_1<R>(Ot[ht], G[hg], gc11, mt, wt, ot3);
            FFV1_2<R>(Itb[hb], G[hg], gc11, mt, wt, itb4);
            Cx<R> a[5] = {FFV1_0<R>(Itb[hb], Ot[ht], vs1, gc11), FFV1_0<R>(Itb[hb], Ot[ht], vs2, gc11),
                          FFV1_0<R>(Itb[hb], ot3, vs0, gc11), FFV1_0<R>(itb4, Ot[ht], vs0, gc11),
                          FFV1_0<R>(Itb[hb], Ot[ht], vs5, gc11)};
            for (int d = 0; d < 5; ++d) {
              Cx<R> z;
              for (int e = 0; e < 5; ++e) z += Cx<R>{R(kQQ3CmRe[d][e]), R(kQQ3CmIm[d][e])} * conj(a[e]);
              tot += (a[d] * z).re;
            }
          }
      }
    }
  return tot;
}

// channel 0: q(p0) q~(p1) > t(p2) t~(p3) g(p4); 1: q(p0) g(p1) > t t~ q(p4);
// 2: q~(p0) g(p1) > t t~ q~(p4).  prm: mt, wt, GC_10 (re, im), GC_11 (re, im).
template <class R> static R smatrix_qq3(int channel, const R* p, const double* prm, double sqh_d) {
  const R mt = R(prm[0]), wt = R(prm[1]), sqh = R(sqh_d);
  const Cx<R> gc10{R(prm[2]), R(prm[3])}, gc11{R(prm[4]), R(prm[5])};
  WF<R> I[2], O[2], Ot[2], Itb[2], G[2];
  for (int b = 0; b < 2; ++b) {
    const R h = b ? R(1) : R(-1);
    oxxxxx<R>(p + 8, mt, h, R(1), Ot[b]);
    ixxxxx<R>(p + 12, mt, h, R(-1), Itb[b]);
    if (channel == 0) {
      ixxxxx<R>(p + 0, R(0), h, R(1), I[b]);
      oxxxxx<R>(p + 4, R(0), h, R(-1), O[b]);
      vxxxxx<R>(p + 16, R(0), h, R(1), sqh, G[b]);
    } else if (channel == 1) {
      ixxxxx<R>(p + 0, R(0), h, R(1), I[b]);
      oxxxxx<R>(p + 16, R(0), h, R(1), O[b]);
      vxxxxx<R>(p + 4, R(0), h, R(-1), sqh, G[b]);
    } else {
      oxxxxx<R>(p + 0, R(0), h, R(-1), O[b]);
      ixxxxx<R>(p + 16, R(0), h, R(-1), I[b]);
      vxxxxx<R>(p + 4, R(0), h, R(-1), sqh, G[b]);
    }
  }
  const R tot = qq3_helicity_sum<R>(I, O, Ot, Itb, G, gc10, gc11, mt, wt);
  return tot / R(channel == 0 ? 36.0 : 96.0);
}

// f32q: madflow's float32-rounded sqrt(1/2) in the gluon polarisations
// (wavefunctions_flow.py:10), else the exact value
extern "C" int orc_smatrix_qq3(int channel, const double* p, int64_t N, const double* prm, int f32q, double* out) {
  if (channel < 0 || channel > 2) return 1;
  const double sqh = ref_consts(f32q != 0).sqh;
#pragma omp parallel for schedule(static)
  for (int64_t e = 0; e < N; ++e) out[e] = smatrix_qq3<double>(channel, p + 20 * e, prm, sqh);
  return 0;
}

extern "C" void orc_pdf_table(double* table /*[kNQ][kNX]*/, double* lx0, double* dlx, double* lq0, double* dlq) {
  double A = pdf_A();
  *lx0 = std::log(1e-6); *dlx = (0.0 - *lx0) / (kNX - 1);
  *lq0 = std::log(1.0); *dlq = (std::log(1e10) - *lq0) / (kNQ - 1);
  for (int iq = 0; iq < kNQ; ++iq)
    for (int ix = 0; ix < kNX; ++ix) {
      double x = std::exp(*lx0 + ix * *dlx);
      if (ix == kNX - 1) x = 1.0;
      table[iq * kNX + ix] = A * std::pow(x, -0.2) * std::pow(1.0 - x, 5.0);
    }
}
// Synthetic quark densities beside the gluon (the configurations define only
// the gluon; p p > t t~ needs the light quarks too), x f(x) independent of Q:
//   valence  x u_v = A x^0.5 (1-x)^3 with int u_v = 2,
//            x d_v = A x^0.5 (1-x)^4 with int d_v = 1;
//   sea      x qbar = A x^-0.2 (1-x)^7 with momentum fractions int x qbar =
//            0.03 (ubar, dbar), 0.015 (s = sbar), 0.005 (c = cbar);
//   u = u_v + ubar, d = d_v + dbar.
// pdg: 21 gluon, 1..4 d u s c, -1..-4 their antiquarks.
static double beta_fn(double a, double b) { return std::exp(std::lgamma(a) + std::lgamma(b) - std::lgamma(a + b)); }
static double synth_xfx(int pdg, double x) {
  if (x >= 1.0) return 0.0;
  if (pdg == 21) return pdf_A() * std::pow(x, -0.2) * std::pow(1.0 - x, 5.0);
  const int a = pdg < 0 ? -pdg : pdg;
  const double frac = a <= 2 ? 0.03 : (a == 3 ? 0.015 : 0.005);
  double v = frac / beta_fn(0.8, 8.0) * std::pow(x, -0.2) * std::pow(1.0 - x, 7.0);
  if (pdg == 2) v += 2.0 / beta_fn(0.5, 4.0) * std::pow(x, 0.5) * std::pow(1.0 - x, 3.0);
  if (pdg == 1) v += 1.0 / beta_fn(0.5, 5.0) * std::pow(x, 0.5) * std::pow(1.0 - x, 4.0);
  return v;
}
extern "C" void orc_pdf_table_flavour(int pdg, double* table /*[kNQ][kNX]*/) {
  double lx0 = std::log(1e-6), dlx = (0.0 - lx0) / (kNX - 1);
  for (int iq = 0; iq < kNQ; ++iq)
    for (int ix = 0; ix < kNX; ++ix) {
      double x = std::exp(lx0 + ix * dlx);
      if (ix == kNX - 1) x = 1.0;
      table[iq * kNX + ix] = synth_xfx(pdg, x);
    }
}

static double keys_w(double t) {  // cubic convolution kernel, a = -1/2
  t = std::fabs(t);
  if (t <= 1.0) return (1.5 * t - 2.5) * t * t + 1.0;
  if (t < 2.0) return ((-0.5 * t + 2.5) * t - 4.0) * t + 2.0;
  return 0.0;
}
// bicubic lookup (Keys 1981, a = -1/2, clamped edge nodes) of a [kNQ][kNX] table
static double pdf_lookup(const double* tab, double x, double q2) {
  const double lx0 = std::log(1e-6), dlx = (0.0 - lx0) / (kNX - 1);
  const double lq0 = std::log(1.0), dlq = (std::log(1e10) - lq0) / (kNQ - 1);
  double u = (std::log(x) - lx0) / dlx, v = (std::log(q2) - lq0) / dlq;
  int iu = (int)std::floor(u), iv = (int)std::floor(v);
  double fu = u - iu, fv = v - iv;
  double s = 0.0;
  for (int a = -1; a <= 2; ++a) {
    int qi = std::min(std::max(iv + a, 0), kNQ - 1);
    double wv = keys_w(fv - a);
    for (int b = -1; b <= 2; ++b) {
      int xi = std::min(std::max(iu + b, 0), kNX - 1);
      s += wv * keys_w(fu - b) * tab[qi * kNX + xi];
    }
  }
  return s > 0.0 ? s : 0.0;
}
extern "C" void orc_pdf_xfx(const double* x, int64_t N, double q2, double* out) {
  static const std::vector<double> tab = [] {
    std::vector<double> t(kNX * kNQ);
    double a, b, c, d;
    orc_pdf_table(t.data(), &a, &b, &c, &d);
    return t;
  }();
  for (int64_t e = 0; e < N; ++e) out[e] = pdf_lookup(tab.data(), x[e], q2);
}
// x f(x, Q^2) of flavour pdg (21, +-1..+-4) from its table
extern "C" int orc_pdf_xfx_flavour(int pdg, const double* x, int64_t N, double q2, double* out) {
  static const std::map<int, std::vector<double>> tabs = [] {
    std::map<int, std::vector<double>> m;
    for (int f : {21, 1, 2, 3, 4, -1, -2, -3, -4}) {
      std::vector<double> t(kNX * kNQ);
      orc_pdf_table_flavour(f, t.data());
      m[f] = t;
    }
    return m;
  }();
  auto it = tabs.find(pdg);
  if (it == tabs.end()) return 1;
  for (int64_t e = 0; e < N; ++e) out[e] = pdf_lookup(it->second.data(), x[e], q2);
  return 0;
}

// ---------------------------------------------------------------------------
// VEGAS (G. P. Lepage, J. Comput. Phys. 27 (1978) 192): importance grid of
// nb bins per dimension on [0,1].  vegasflow is the reference's integrator and
// is not vendored; this follows the published algorithm.
// ---------------------------------------------------------------------------
extern "C" void orc_vegas_sample(const double* div /*ndim*(nb+1)*/, int ndim, int nb, const double* u, int64_t N,
                                 double* x, double* jac, int32_t* bins) {
  for (int64_t e = 0; e < N; ++e) {
    double j = 1.0;
    for (int d = 0; d < ndim; ++d) {
      double xn = u[ndim * e + d] * (double)nb;
      int i = (int)xn;
      if (i > nb - 1) i = nb - 1;
      double frac = xn - (double)i;
      double lo = div[d * (nb + 1) + i];
      double w = div[d * (nb + 1) + i + 1] - lo;
      x[ndim * e + d] = std::fma(w, frac, lo);
      j *= w * (double)nb;
      bins[ndim * e + d] = i;
    }
    jac[e] = j;
  }
}
// fw[e] = jac*f/N_iteration; accumulates sum fw, sum fw^2 and per-bin sum fw^2
extern "C" void orc_vegas_accumulate(const double* fw, const int32_t* bins, int64_t N, int ndim, int nb, double* sums,
                                     double* hist /*ndim*nb*/) {
  for (int64_t e = 0; e < N; ++e) {
    double f = fw[e], f2 = f * f;
    sums[0] += f;
    sums[1] += f2;
    for (int d = 0; d < ndim; ++d) hist[d * nb + bins[ndim * e + d]] += f2;
  }
}
// Grid refinement of one VEGAS iteration, alpha = damping exponent.
extern "C" void orc_vegas_refine(double* div, const double* hist, int ndim, int nb, double alpha) {
  std::vector<double> d(nb), r(nb), nd(nb + 1);
  for (int dim = 0; dim < ndim; ++dim) {
    const double* h = hist + dim * nb;
    double* g = div + dim * (nb + 1);
    // smoothing with neighbours
    d[0] = (h[0] + h[1]) / 2.0;
    for (int i = 1; i < nb - 1; ++i) d[i] = (h[i - 1] + h[i] + h[i + 1]) / 3.0;
    d[nb - 1] = (h[nb - 2] + h[nb - 1]) / 2.0;
    double tot = 0.0;
    for (int i = 0; i < nb; ++i) tot += d[i];
    if (!(tot > 0.0)) continue;
    double rsum = 0.0;
    for (int i = 0; i < nb; ++i) {
      double q = d[i] / tot;
      r[i] = (q > 0.0) ? std::pow((q - 1.0) / std::log(q), alpha) : 0.0;
      rsum += r[i];
    }
    if (!(rsum > 0.0)) continue;
    double per = rsum / (double)nb;
    // walk the old bins and place the new edges at equal shares of sum r
    nd[0] = g[0];
    nd[nb] = g[nb];
    int i = 0;
    double accum = 0.0;  // r collected below the current target inside old bins < i
    for (int j = 1; j < nb; ++j) {
      double target = per * (double)j;
      while (i < nb && accum + r[i] < target) { accum += r[i]; ++i; }
      if (i >= nb) { nd[j] = g[nb]; continue; }
      double frac = (target - accum) / r[i];
      nd[j] = g[i] + frac * (g[i + 1] - g[i]);
    }
    for (int j = 0; j <= nb; ++j) g[j] = nd[j];
  }
}

// ---------------------------------------------------------------------------
// Integrands.  kind 0: gg -> tt~ at fixed sqrt(s-hat) (rambo over 8 uniforms,
// flux 1/(2 s-hat), pb).  kind 1: hadronic ramboflow + synthetic PDF + cuts.
// ---------------------------------------------------------------------------
struct IntegrandCfg {
  int kind;        // 0 fixed sqrt(s-hat) gg->tt~, 1 hadronic tt~+ng
  int k;           // number of gluons (2 = gg->tt~)
  double sqrts;    // partonic (kind 0) or hadronic (kind 1)
  double mt, wt, alphas;
  double ptmin, etamax, drmin;  // cuts on outgoing gluons (ptmin <= 0: none)
  int newton_rule;
};

static double dphi(double a, double b) {
  double d = a - b;
  while (d > M_PI) d -= 2 * M_PI;
  while (d < -M_PI) d += 2 * M_PI;
  return d;
}
// cut decision on lab-frame momenta [npart][4]; outgoing gluons are particles 4..
extern "C" int orc_pass_cuts(const double* plab, int npart, double ptmin, double etamax, double drmin) {
  int ng = npart - 4;
  double eta[8], phi[8];
  for (int g = 0; g < ng; ++g) {
    const double* q = plab + 4 * (4 + g);
    double pt = std::sqrt(q[1] * q[1] + q[2] * q[2]);
    if (ptmin > 0 && !(pt > ptmin)) return 0;
    double pabs = std::sqrt(pt * pt + q[3] * q[3]);
    eta[g] = 0.5 * std::log((pabs + q[3]) / (pabs - q[3]));
    phi[g] = std::atan2(q[2], q[1]);
    if (etamax > 0 && !(std::fabs(eta[g]) < etamax)) return 0;
  }
  if (drmin > 0)
    for (int a = 0; a < ng; ++a)
      for (int b = a + 1; b < ng; ++b) {
        double de = eta[a] - eta[b], dp = dphi(phi[a], phi[b]);
        if (!(std::sqrt(de * de + dp * dp) > drmin)) return 0;
      }
  return 1;
}

// f[N] for x[N][ndim]; plan = tt~+ng handle (NULL for kind 0)
extern "C" void orc_integrand(const double* cfgv, void* plan, const double* x, int64_t N, double* f) {
  IntegrandCfg cfg;
  cfg.kind = (int)cfgv[0]; cfg.k = (int)cfgv[1]; cfg.sqrts = cfgv[2]; cfg.mt = cfgv[3]; cfg.wt = cfgv[4];
  cfg.alphas = cfgv[5]; cfg.ptmin = cfgv[6]; cfg.etamax = cfgv[7]; cfg.drmin = cfgv[8]; cfg.newton_rule = (int)cfgv[9];
  const int initial_states = (int)cfgv[10];  // 0: g g; 1: p p (g g + q q~ + q~ q, q = d u s c), k = 2 only
  // 1: madflow's dynamical scale (scripts/madflow_exec.py:428-431): per event
  // mu^2 = (sum over the outgoing particles of m_T / 2)^2 from the lab-frame
  // momenta, m_T^2 = p.p + p_T^2 (phasespace.py:406-415), the densities at
  // mu^2 and alpha_s(mu^2) from alpha_s(M_Z^2) = cfg.alphas at one loop with
  // five flavours (the stand-in for pdfflow's alphasQ2); every tree diagram
  // has k strong vertices, so the per-event couplings multiply |M|^2 by
  // (alpha_s(mu^2) / alpha_s(M_Z^2))^k
  const bool dyn = cfgv[11] != 0.0;
  // > 0: madflow's --pt_cut (scripts/madflow_exec.py:396-401): p_T >
  // float32(cut) for every outgoing particle, on the momenta before the boost
  // to the lab frame (phasespace.py:417-422, 458-466)
  const double pt_all = cfgv[12] > 0.0 ? (double)(float)cfgv[12] : 0.0;
  // PhaseSpaceGenerator.register_cut (phasespace.py:424-478): cfgv[13] cuts,
  // then per cut variable (0 pt, 1 mt, 2 mt2, 3 eta), particle, has_min,
  // has_max, min_val, max_val; strict, thresholds through float32, on the
  // momenta before the boost
  const int ncuts = (int)cfgv[13];
  auto pass_table = [&](const double* pe) {
    for (int c = 0; c < ncuts; ++c) {
      const double* cv = cfgv + 14 + 6 * c;
      const double* q = pe + 4 * (int)cv[1];
      const double pt = std::sqrt(q[1] * q[1] + q[2] * q[2]);
      double val = pt;
      const int var = (int)cv[0];
      if (var == 1 || var == 2) {
        const double mt2 = (q[0] * q[0] - ((q[1] * q[1] + q[2] * q[2]) + q[3] * q[3])) + pt * pt;
        val = var == 1 ? std::sqrt(mt2) : mt2;
      } else if (var == 3) {
        const double pabs = std::sqrt((q[1] * q[1] + q[2] * q[2]) + q[3] * q[3]);
        val = 0.5 * std::log((pabs + q[3]) / (pabs - q[3]));
      }
      if (cv[2] != 0.0 && !(val > (double)(float)cv[4])) return false;
      if (cv[3] != 0.0 && !(val < (double)(float)cv[5])) return false;
    }
    return true;
  };
  double gs = 2.0 * std::sqrt(M_PI * cfg.alphas);
  // MT, WT, GC_10 = -g, GC_11 = i g, GC_12 = i g^2, c3 = -i, c4 = -1
  double prm[12] = {cfg.mt, cfg.wt, -gs, 0.0, 0.0, gs, 0.0, gs * gs, 0.0, -1.0, -1.0, 0.0};
  if (cfg.kind == 0) {
    // gg -> tt~ at fixed sqrt(s-hat)
    std::vector<double> pout((size_t)N * 8), w(N), sq(N, cfg.sqrts), p((size_t)N * 16), me(N);
    double masses[2] = {cfg.mt, cfg.mt};
    orc_rambo(x, N, 2, sq.data(), masses, 1, cfg.newton_rule, pout.data(), w.data());
    double ein = cfg.sqrts / 2.0;
    for (int64_t e = 0; e < N; ++e) {
      double* pe = &p[16 * e];
      pe[0] = ein; pe[1] = 0; pe[2] = 0; pe[3] = ein; pe[4] = ein; pe[5] = 0; pe[6] = 0; pe[7] = -ein;
      std::memcpy(pe + 8, &pout[8 * e], 8 * sizeof(double));
    }
    double gp[6] = {cfg.mt, cfg.wt, -gs, 0.0, 0.0, gs};
    orc_smatrix_ggttx(p.data(), N, gp, 1, me.data(), nullptr);
    double flux = ref_consts(true).gev2pb / (2.0 * cfg.sqrts * cfg.sqrts);
    for (int64_t e = 0; e < N; ++e) f[e] = me[e] * w[e] * flux;
    return;
  }
  int npart = cfg.k + 2;
  std::vector<double> masses(npart - 2, 0.0);
  masses[0] = cfg.mt; masses[1] = cfg.mt;
  std::vector<double> p((size_t)N * 4 * npart), w(N), x1(N), x2(N), me(N, 0.0);
  orc_ramboflow(x, N, npart, cfg.sqrts, masses.data(), 1, cfg.newton_rule, p.data(), w.data(), x1.data(), x2.data());
  std::vector<char> pass(N, 1);
  std::vector<double> plab(4 * npart);
  std::vector<double> q2v((size_t)N, cfg.mt * cfg.mt), csv((size_t)N, 1.0);
  for (int64_t e = 0; e < N; ++e) {
    std::memcpy(plab.data(), &p[(size_t)4 * npart * e], sizeof(double) * 4 * npart);
    boost_to_lab<double>(plab.data(), npart, x1[e], x2[e]);
    pass[e] = (char)orc_pass_cuts(plab.data(), npart, cfg.ptmin, cfg.etamax, cfg.drmin);
    if (pt_all > 0.0)
      for (int i = 2; i < npart; ++i) {
        const double* q = &p[(size_t)4 * npart * e + 4 * i];
        if (!(std::sqrt(q[1] * q[1] + q[2] * q[2]) > pt_all)) pass[e] = 0;
      }
    if (ncuts > 0 && !pass_table(&p[(size_t)4 * npart * e])) pass[e] = 0;
    if (dyn) {
      double smt = 0.0;
      for (int i = 2; i < npart; ++i) {
        const double* q = &plab[4 * i];
        const double m2 = q[0] * q[0] - q[1] * q[1] - q[2] * q[2] - q[3] * q[3];
        const double pt = std::sqrt(q[1] * q[1] + q[2] * q[2]);
        smt += std::sqrt(m2 + pt * pt);
      }
      q2v[e] = (smt / 2.0) * (smt / 2.0);
      const double mz = 91.1876, b0 = 23.0 / (12.0 * M_PI);
      const double r = 1.0 / (1.0 + cfg.alphas * b0 * std::log(q2v[e] / (mz * mz)));
      csv[e] = std::pow(r, cfg.k);
    }
  }
  // x f(x) at the event's scale
  auto xf = [&](int pdg, const double* xs, int64_t e) {
    double o;
    if (pdg == 21) orc_pdf_xfx(xs + e, 1, q2v[e], &o);
    else orc_pdf_xfx_flavour(pdg, xs + e, 1, q2v[e], &o);
    return o;
  };
  // evaluate the matrix element on the passing events only
  std::vector<int64_t> idx;
  for (int64_t e = 0; e < N; ++e) if (pass[e]) idx.push_back(e);
  std::vector<double> pp((size_t)idx.size() * 4 * npart), mep(idx.size());
  for (size_t i = 0; i < idx.size(); ++i)
    std::memcpy(&pp[(size_t)4 * npart * i], &p[(size_t)4 * npart * idx[i]], sizeof(double) * 4 * npart);
  if (plan && !idx.empty()) orc_ttng_smatrix(plan, pp.data(), (int64_t)idx.size(), prm, 1, mep.data(), nullptr);
  std::vector<double> g1(N), g2(N);
  double q2 = cfg.mt * cfg.mt;
  if (dyn) {
    for (int64_t e = 0; e < N; ++e) {
      g1[e] = xf(21, x1.data(), e);
      g2[e] = xf(21, x2.data(), e);
    }
  } else {
    orc_pdf_xfx(x1.data(), N, q2, g1.data());
    orc_pdf_xfx(x2.data(), N, q2, g2.data());
  }
  for (int64_t e = 0; e < N; ++e) f[e] = 0.0;
  for (size_t i = 0; i < idx.size(); ++i) {
    int64_t e = idx[i];
    double lum = g1[e] * g2[e] / x1[e] / x2[e];
    f[e] = mep[i] * lum * w[e] * csv[e];
  }
  if (initial_states == 1 && cfg.k == 2 && !idx.empty()) {
    // madflow's integrand: sum over the processes of luminosity x |M|^2, the
    // luminosity summed over each process's initial states and their mirror
    // images (scripts/madflow_exec.py:444-458, utilities.py:25-39)
    std::vector<double> meq(idx.size()), qa((size_t)N), qb((size_t)N), qc((size_t)N), qd((size_t)N);
    double prmq[4] = {cfg.mt, cfg.wt, 0.0, gs};
    orc_smatrix_uux_ttx(pp.data(), (int64_t)idx.size(), prmq, meq.data());
    std::vector<double> lumq((size_t)N, 0.0);
    for (int q = 1; q <= 4; ++q) {
      if (dyn) {
        for (int64_t e = 0; e < N; ++e)
          lumq[e] += xf(q, x1.data(), e) * xf(-q, x2.data(), e) + xf(-q, x1.data(), e) * xf(q, x2.data(), e);
        continue;
      }
      orc_pdf_xfx_flavour(q, x1.data(), N, q2, qa.data());
      orc_pdf_xfx_flavour(-q, x2.data(), N, q2, qb.data());
      orc_pdf_xfx_flavour(-q, x1.data(), N, q2, qc.data());
      orc_pdf_xfx_flavour(q, x2.data(), N, q2, qd.data());
      for (int64_t e = 0; e < N; ++e) lumq[e] += qa[e] * qb[e] + qc[e] * qd[e];
    }
    for (size_t i = 0; i < idx.size(); ++i) {
      int64_t e = idx[i];
      f[e] += meq[i] * (lumq[e] / x1[e] / x2[e]) * w[e] * csv[e];
    }
  }
  if (initial_states == 1 && cfg.k == 3 && !idx.empty()) {
    // p p > t t~ j: q q~ > t t~ g, q g > t t~ q, q~ g > t t~ q~ and their
    // mirror images (the initial states swapped), q = d u s c
    const size_t M = idx.size();
    std::vector<double> swapped(pp);
    for (size_t i = 0; i < M; ++i)
      for (int c = 0; c < 4; ++c) std::swap(swapped[20 * i + c], swapped[20 * i + 4 + c]);
    double prm3[6] = {cfg.mt, cfg.wt, -gs, 0.0, 0.0, gs};
    std::vector<double> me[6];
    for (int ch = 0; ch < 3; ++ch) {
      me[2 * ch].resize(M);
      me[2 * ch + 1].resize(M);
      orc_smatrix_qq3(ch, pp.data(), (int64_t)M, prm3, 1, me[2 * ch].data());
      orc_smatrix_qq3(ch, swapped.data(), (int64_t)M, prm3, 1, me[2 * ch + 1].data());
    }
    std::vector<double> q1((size_t)N, 0.0), qb1((size_t)N, 0.0), t((size_t)N);
    for (int q = 1; q <= 4; ++q) {
      if (dyn) {
        for (int64_t e = 0; e < N; ++e) {
          q1[e] += xf(q, x1.data(), e);
          qb1[e] += xf(-q, x1.data(), e);
        }
        continue;
      }
      orc_pdf_xfx_flavour(q, x1.data(), N, q2, t.data());
      for (int64_t e = 0; e < N; ++e) q1[e] += t[e];
      orc_pdf_xfx_flavour(-q, x1.data(), N, q2, t.data());
      for (int64_t e = 0; e < N; ++e) qb1[e] += t[e];
    }
    double lq[6];
    for (size_t i = 0; i < M; ++i) {
      const int64_t e = idx[i];
      double s_qq = 0.0, s_qbq = 0.0, q_2 = 0.0, qb_2 = 0.0;
      for (int q = 1; q <= 4; ++q) {
        double a, b, c, d;
        orc_pdf_xfx_flavour(q, &x1[e], 1, q2v[e], &a);
        orc_pdf_xfx_flavour(-q, &x2[e], 1, q2v[e], &b);
        orc_pdf_xfx_flavour(-q, &x1[e], 1, q2v[e], &c);
        orc_pdf_xfx_flavour(q, &x2[e], 1, q2v[e], &d);
        s_qq += a * b;
        s_qbq += c * d;
        q_2 += d;
        qb_2 += b;
      }
      lq[0] = s_qq;               // q(x1) q~(x2)
      lq[1] = s_qbq;              // q~(x1) q(x2): q q~ mirrored
      lq[2] = q1[e] * g2[e];      // q(x1) g(x2)
      lq[3] = g1[e] * q_2;        // g(x1) q(x2)
      lq[4] = qb1[e] * g2[e];     // q~(x1) g(x2)
      lq[5] = g1[e] * qb_2;       // g(x1) q~(x2)
      double sum = 0.0;
      for (int c = 0; c < 6; ++c) sum += me[c][i] * lq[c];
      f[e] += sum / x1[e] / x2[e] * w[e] * csv[e];
    }
  }
}

extern "C" int orc_num_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
