// Helicity-recycling evaluation of g g > t t~ + (K-2) g: one thread block per
// event, currents shared between the helicity combinations that agree on the
// legs they depend on.
//
//   gluon currents J(s; h_s)            per canonical ordered gluon sequence s
//                                       and helicities of the gluons of s;
//   bare full-length contractions T0    wtb^T S(J(sigma; h_g)) wt, per
//                                       canonical sigma, h_g, h_t, h_tbar;
//   top-line currents O(a; h_t, h_a)    per ordered prefix a (the gluons
//                                       attached next to the top);
//   t~-side rows RW(b; h_tb, h_b)       wtb^T S(J(b)), per gluon sequence b;
//   partial amplitudes A(sigma; h) = T0 + sum_{sigma = a|b} RW(b) . O(a);
//   colour sum sum_{ab} C_ab Re(A_a A_b^*).
//
// Every stage is a loop over independent work items spread over the threads
// of the block (tid, nt); stages are separated by __syncthreads().  The
// stage functions are host-callable so the CPU test suite can run them one
// thread at a time against the oracle.  Tables come from the generated
// header of the process (namespace rec<K>, see codegen.emit_recycled_tables).
#pragma once
#include "mf_helas.cuh"
#include "mf_phasespace.cuh"
#include "mf_vertex.cuh"

template <int K> struct RecTraits;

#ifdef __CUDA_ARCH__
#define MF_TBL(NS, NAME, I) (NS::NAME[(I)])
#else
#define MF_TBL(NS, NAME, I) (NS::NAME##_h[(I)])
#endif

#define MF_DEFINE_REC(KK)                                                                             \
  template <> struct RecTraits<KK> {                                                                  \
    static constexpr int K = KK, NJ = rec##KK::NJ, J_TOTAL = rec##KK::J_TOTAL, NF = rec##KK::NF;      \
    static constexpr int NO = rec##KK::NO, O_TOTAL = rec##KK::O_TOTAL, NR = rec##KK::NR;              \
    static constexpr int R_TOTAL = rec##KK::R_TOTAL, BASE = rec##KK::BASE;                            \
    static constexpr int NPERM = ttng##KK::NPERM, NCOMB = ttng##KK::NCOMB;                            \
    static constexpr double DENOMINATOR = ttng##KK::DENOMINATOR, COLOUR_DEN = ttng##KK::COLOUR_DEN;   \
    MF_D static int jn_code(int i) { return MF_TBL(rec##KK, jn_code, i); }                            \
    MF_D static int jn_off(int i) { return MF_TBL(rec##KK, jn_off, i); }                              \
    MF_D static int jlen_first(int i) { return MF_TBL(rec##KK, jlen_first, i); }                      \
    MF_D static int seq_ref(int i) { return MF_TBL(rec##KK, seq_ref, i); }                            \
    MF_D static int seq_mask(int i) { return MF_TBL(rec##KK, seq_mask, i); }                          \
    MF_D static int fn_code(int i) { return MF_TBL(rec##KK, fn_code, i); }                            \
    MF_D static int perm_code(int i) { return MF_TBL(rec##KK, perm_code, i); }                        \
    MF_D static int perm_full(int i) { return MF_TBL(rec##KK, perm_full, i); }                        \
    MF_D static int on_code(int i) { return MF_TBL(rec##KK, on_code, i); }                            \
    MF_D static int on_off(int i) { return MF_TBL(rec##KK, on_off, i); }                              \
    MF_D static int olen_first(int i) { return MF_TBL(rec##KK, olen_first, i); }                      \
    MF_D static int opos(int i) { return MF_TBL(rec##KK, opos, i); }                                  \
    MF_D static int r_len(int i) { return MF_TBL(rec##KK, r_len, i); }                                \
    MF_D static int r_off(int i) { return MF_TBL(rec##KK, r_off, i); }                                \
    MF_D static int cfg_to_mg(int i) { return MF_TBL(rec##KK, cfg_to_mg, i); }                        \
    MF_D static float colour(int i) { return MF_TBL(ttng##KK, colour_num, i); }                       \
  };

// Workspace of one event (shared memory).
template <class T, int K> struct RecWS {
  using R = RecTraits<K>;
  W4<T> G[K][2];
  W4<T> WT[2], WTB[2];
  W4<T> J[R::J_TOTAL > 0 ? R::J_TOTAL : 1];
  cx<T> T0[R::NF][1 << K][4];
  W4<T> O[R::O_TOTAL];
  W4<T> RW[R::R_TOTAL];
  cx<T> A[1 << (K + 2)][R::NPERM];
};

template <int B> MF_D int pow_base(int e) {
  int p = 1;
  for (int i = 0; i < e; ++i) p *= B;
  return p;
}
// code of the ordered sub-sequence s[i:j]
template <int B> MF_D int sub_code(int code, int i, int j) { return (code / pow_base<B>(i)) % pow_base<B>(j - i); }
MF_D int bit_reverse(int hp, int len) {
  int r = 0;
  for (int j = 0; j < len; ++j) r |= ((hp >> j) & 1) << (len - 1 - j);
  return r;
}
// helicity pattern of the sequence `code` (length len) from gluon helicity bits hg
template <int B> MF_D int pack_hel(int hg, int code, int len) {
  int hp = 0;
  for (int j = 0; j < len; ++j) {
    int g = (code % B) - 1;
    code /= B;
    hp |= ((hg >> g) & 1) << j;
  }
  return hp;
}

template <class T, int K> MF_D W4<T> rec_cur(const RecWS<T, K>& ws, int ref, int len, int hp) {
  using R = RecTraits<K>;
  int id = ref >> 2;
  W4<T> w;
  if (id >= R::NJ) {
    w = ws.G[id - R::NJ][hp & 1];
  } else {
    int h = (ref & 2) ? bit_reverse(hp, len) : hp;
    w = ws.J[R::jn_off(id) + h];
  }
  return (ref & 1) ? neg(w) : w;
}

// colour-ordered gluon current of the ordered sequence `code` (length L)
template <class T, int K>
MF_D W4<T> rec_gluon_current(const RecWS<T, K>& ws, const EvData<T, K>& ev, int code, int L, int hp) {
  using R = RecTraits<K>;
  constexpr int B = R::BASE;
  W4<T> a3 = w4zero<T>(), a4 = w4zero<T>();
  for (int i = 1; i < L; ++i) {
    int cl = sub_code<B>(code, 0, i), cr = sub_code<B>(code, i, L);
    W4<T> a = rec_cur<T, K>(ws, R::seq_ref(cl), i, hp & ((1 << i) - 1));
    W4<T> b = rec_cur<T, K>(ws, R::seq_ref(cr), L - i, hp >> i);
    vvv_add<T>(a, ev.Qg[R::seq_mask(cl)], b, ev.Qg[R::seq_mask(cr)], a3);
  }
  for (int i = 1; i < L; ++i)
    for (int j = i + 1; j < L; ++j) {
      int c1 = sub_code<B>(code, 0, i), c2 = sub_code<B>(code, i, j), c3 = sub_code<B>(code, j, L);
      W4<T> a = rec_cur<T, K>(ws, R::seq_ref(c1), i, hp & ((1 << i) - 1));
      W4<T> b = rec_cur<T, K>(ws, R::seq_ref(c2), j - i, (hp >> i) & ((1 << (j - i)) - 1));
      W4<T> d = rec_cur<T, K>(ws, R::seq_ref(c3), L - j, hp >> j);
      vvvv_add<T>(a, b, d, a4);
    }
  int m = R::seq_mask(code);
  return combine<T>(ev.gv3[m], a3, ev.gv4[m], a4);
}

// stage 0: external wavefunctions (gluons for both helicities, t, t~)
template <class T, int K> MF_D void rec_st_ext(RecWS<T, K>& ws, const EvData<T, K>& ev, int tid, int nt) {
  const T sqh = (T)0.70710676908493042;  // madflow's float32-rounded sqrt(1/2)
  for (int i = tid; i < 2 * K + 4; i += nt) {
    if (i < 2 * K) {
      int q = i >> 1, b = i & 1;
      int part = gluon_particle<K>(q);
      ws.G[q][b] = vxxxxx<T>(ev.pext[part], T(0), b ? T(1) : T(-1), part < 2 ? T(-1) : T(1), sqh);
    } else if (i < 2 * K + 2) {
      int b = i - 2 * K;
      ws.WT[b] = oxxxxx<T>(ev.pext[2], ev.mt, b ? T(1) : T(-1), T(1));
    } else {
      int b = i - 2 * K - 2;
      ws.WTB[b] = ixxxxx<T>(ev.pext[3], ev.mt, b ? T(1) : T(-1), T(-1));
    }
  }
}

// stage J(L): gluon currents of length L (2 <= L <= K-1)
template <class T, int K> MF_D void rec_st_J(RecWS<T, K>& ws, const EvData<T, K>& ev, int L, int tid, int nt) {
  using R = RecTraits<K>;
  int first = R::jlen_first(L), cnt = R::jlen_first(L + 1) - first;
  for (int it = tid; it < (cnt << L); it += nt) {
    int node = first + (it >> L), hp = it & ((1 << L) - 1);
    ws.J[R::jn_off(node) + hp] = rec_gluon_current<T, K>(ws, ev, R::jn_code(node), L, hp);
  }
}

// row vector r = F1^T S(V): F1^T S(V) F2 = r . F2
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

// stage T0 + RW + O(1): all depend only on the gluon currents and externals
template <class T, int K> MF_D void rec_st_mid(RecWS<T, K>& ws, const EvData<T, K>& ev, int tid, int nt) {
  using R = RecTraits<K>;
  const int n_t0 = R::NF << K;
  const int n_o1 = R::olen_first(2) * 4;  // K prefixes of length 1, x 2 (h_t) x 2 (h)
  const int total = n_t0 + R::R_TOTAL + n_o1;
  for (int it = tid; it < total; it += nt) {
    if (it < n_t0) {
      int f = it >> K, hp = it & ((1 << K) - 1);
      W4<T> Jf = rec_gluon_current<T, K>(ws, ev, R::fn_code(f), K, hp);
      for (int q = 0; q < 4; ++q) ws.T0[f][hp][q] = dot4(sandwich_row(ws.WTB[q >> 1], Jf), ws.WT[q & 1]);
    } else if (it < n_t0 + R::R_TOTAL) {
      int idx = it - n_t0;
      int r = 0;
      while (r + 1 < R::NR && R::r_off(r + 1) <= idx) ++r;
      int L = R::r_len(r), rem = idx - R::r_off(r);
      int htb = rem >> L, hp = rem & ((1 << L) - 1);
      const W4<T>& J = (r >= R::NJ) ? ws.G[r - R::NJ][hp] : ws.J[R::jn_off(r) + hp];
      ws.RW[idx] = sandwich_row(ws.WTB[htb], J);
    } else {
      int idx = it - n_t0 - R::R_TOTAL;
      int node = idx >> 2, ht = (idx >> 1) & 1, hp = idx & 1;
      int code = R::on_code(node);
      W4<T> y = w4zero<T>();
      sv_add<T>(rec_cur<T, K>(ws, R::seq_ref(code), 1, hp), ws.WT[ht], y);
      int m = R::seq_mask(code);
      ws.O[R::on_off(node) + (ht << 1) + hp] = topprop<T>(ev.Qt[m], ev.mt, ev.tden[m], y);
    }
  }
}

// stage O(L), 2 <= L <= K-1: top-line currents with L gluons attached
template <class T, int K> MF_D void rec_st_O(RecWS<T, K>& ws, const EvData<T, K>& ev, int L, int tid, int nt) {
  using R = RecTraits<K>;
  constexpr int B = R::BASE;
  int first = R::olen_first(L), cnt = R::olen_first(L + 1) - first;
  for (int it = tid; it < (cnt << (L + 1)); it += nt) {
    int node = first + (it >> (L + 1)), rem = it & ((2 << L) - 1);
    int ht = rem >> L, hp = rem & ((1 << L) - 1);
    int code = R::on_code(node);
    W4<T> y = w4zero<T>();
    for (int i = 0; i < L; ++i) {
      int cb = sub_code<B>(code, i, L);
      W4<T> Jb = rec_cur<T, K>(ws, R::seq_ref(cb), L - i, hp >> i);
      if (i == 0) {
        sv_add<T>(Jb, ws.WT[ht], y);
      } else {
        int ca = sub_code<B>(code, 0, i);
        sv_add<T>(Jb, ws.O[R::on_off(R::opos(ca)) + (ht << i) + (hp & ((1 << i) - 1))], y);
      }
    }
    int m = R::seq_mask(code);
    ws.O[R::on_off(node) + (ht << L) + hp] = topprop<T>(ev.Qt[m], ev.mt, ev.tden[m], y);
  }
}

// stage A: partial amplitudes of every (helicity combination, ordering)
template <class T, int K> MF_D void rec_st_A(RecWS<T, K>& ws, int tid, int nt) {
  using R = RecTraits<K>;
  constexpr int B = R::BASE;
  constexpr int NC = 1 << (K + 2);
  for (int it = tid; it < NC * R::NPERM; it += nt) {
    int c = it / R::NPERM, s = it % R::NPERM;
    int hg = c & ((1 << K) - 1), ht = (c >> K) & 1, htb = (c >> (K + 1)) & 1;
    int code = R::perm_code(s), pf = R::perm_full(s);
    int hfull = pack_hel<B>(hg, code, K);
    int hcan = (pf & 2) ? bit_reverse(hfull, K) : hfull;
    cx<T> a = ws.T0[pf >> 2][hcan][ht | (htb << 1)];
    if (pf & 1) a = -a;
    for (int i = 1; i < K; ++i) {
      int ca = sub_code<B>(code, 0, i), cb = sub_code<B>(code, i, K);
      const W4<T>& O = ws.O[R::on_off(R::opos(ca)) + (ht << i) + (hfull & ((1 << i) - 1))];
      int ref = R::seq_ref(cb), id = ref >> 2, Lb = K - i;
      int hb = hfull >> i;
      if (ref & 2) hb = bit_reverse(hb, Lb);
      cx<T> t = dot4(ws.RW[R::r_off(id) + (htb << Lb) + hb], O);
      a = (ref & 1) ? a - t : a + t;
    }
    ws.A[c][s] = a;
  }
}

// stage colour: sum over this thread's (combination, row) items of
// C_aa |A_a|^2 + 2 sum_{b>a} C_ab Re(A_a A_b^*); cm = integer numerators
template <class T, int K> MF_D double rec_st_colour(const RecWS<T, K>& ws, const T* cm, int tid, int nt) {
  using R = RecTraits<K>;
  constexpr int NP = R::NPERM, NC = 1 << (K + 2);
  double acc = 0.0;
  for (int it = tid; it < NC * NP; it += nt) {
    int c = it / NP, a = it % NP;
    const cx<T>* A = ws.A[c];
    cx<T> z = {T(0), T(0)};
    for (int b = a + 1; b < NP; ++b) z += cm[a * NP + b] * A[b];
    T s = cm[a * NP + a] * (A[a].re * A[a].re + A[a].im * A[a].im) + T(2) * (A[a].re * z.re + A[a].im * z.im);
    acc += (double)s;
  }
  return acc;
}

// colour sum of one helicity combination c (for per-helicity outputs)
template <class T, int K> MF_D double rec_colour_one(const RecWS<T, K>& ws, const T* cm, int c) {
  using R = RecTraits<K>;
  constexpr int NP = R::NPERM;
  double acc = 0.0;
  for (int a = 0; a < NP; ++a) {
    const cx<T>* A = ws.A[c];
    cx<T> z = {T(0), T(0)};
    for (int b = a + 1; b < NP; ++b) z += cm[a * NP + b] * A[b];
    acc += (double)(cm[a * NP + a] * (A[a].re * A[a].re + A[a].im * A[a].im) + T(2) * (A[a].re * z.re + A[a].im * z.im));
  }
  return acc;
}

constexpr int MF_REC_NT = 128;  // threads per event block

template <class T, int K> struct RecSmem {
  RecWS<T, K> ws;
  EvData<T, K> ev;
  T cm[RecTraits<K>::NPERM * RecTraits<K>::NPERM];
  double pd[K + 2][4];
  double red[MF_REC_NT / 32];
};

#ifdef __CUDACC__
// Block-per-event |M|^2: ps [K+2][4][N]; couplings [N or 1][3] complex;
// skip (optional) [N]: events with skip[e] == 0 get out[e] = 0 without work;
// out [N]; hel_out (optional) [ncomb][N] MadGraph helicity order.
template <int K, class T>
__global__ void __launch_bounds__(MF_REC_NT) me_rec_kernel(const double* __restrict__ ps, int64_t N, double mt,
                                                          double wt, const double* __restrict__ coup,
                                                          int64_t cstride, const double* __restrict__ skip,
                                                          double* __restrict__ out, double* __restrict__ hel_out) {
  using R = RecTraits<K>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  RecSmem<T, K>& S = *reinterpret_cast<RecSmem<T, K>*>(smem_raw);
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < R::NPERM * R::NPERM; i += nt) S.cm[i] = (T)R::colour(i);
  const double scale_c = 1.0 / (R::COLOUR_DEN * R::DENOMINATOR);
  for (int64_t e = blockIdx.x; e < N; e += gridDim.x) {
    if (skip && skip[e] == 0.0) {
      if (tid == 0) out[e] = 0.0;
      continue;
    }
    __syncthreads();
    for (int i = tid; i < 4 * (K + 2); i += nt) S.pd[i / 4][i % 4] = ps[(int64_t)i * N + e];
    const double* cp = coup + 6 * cstride * e;
    cx<double> c10 = {cp[0], cp[1]}, c11 = {cp[2], cp[3]}, c12 = {cp[4], cp[5]};
    __syncthreads();
    for (int s = tid; s < (1 << K); s += nt) evdata_subset<T, K>(S.ev, s, S.pd, mt, wt, c10, c11, c12);
    for (int i = tid; i < 4 * (K + 2); i += nt) S.ev.pext[i / 4][i % 4] = (T)S.pd[i / 4][i % 4];
    if (tid == 0) S.ev.mt = (T)mt;
    __syncthreads();
    rec_st_ext<T, K>(S.ws, S.ev, tid, nt);
    __syncthreads();
    for (int L = 2; L < K; ++L) {
      rec_st_J<T, K>(S.ws, S.ev, L, tid, nt);
      __syncthreads();
    }
    rec_st_mid<T, K>(S.ws, S.ev, tid, nt);
    __syncthreads();
    for (int L = 2; L < K; ++L) {
      rec_st_O<T, K>(S.ws, S.ev, L, tid, nt);
      __syncthreads();
    }
    rec_st_A<T, K>(S.ws, tid, nt);
    __syncthreads();
    double part = rec_st_colour<T, K>(S.ws, S.cm, tid, nt);
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((tid & 31) == 0) S.red[tid >> 5] = part;
    const double sc = (c11.re * c11.re + c11.im * c11.im) * scale_c;
    if (hel_out)
      for (int c = tid; c < (1 << (K + 2)); c += nt)
        hel_out[(int64_t)R::cfg_to_mg(c) * N + e] = rec_colour_one<T, K>(S.ws, S.cm, c) * sc * R::DENOMINATOR;
    __syncthreads();
    if (tid == 0) {
      double tot = 0.0;
      for (int w = 0; w < nt / 32; ++w) tot += S.red[w];
      out[e] = tot * sc;
    }
  }
}
#endif
