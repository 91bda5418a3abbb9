// Helicity-recycling evaluation of g g > t t~ + (K-2) g: one thread block per
// event, every current computed once for the helicity combinations that
// agree on the legs it depends on.
//
//   J(s; h_s)        gluon current of every ordered gluon sequence s (length
//                    1..K-1; length 1 = the external gluons)
//   O(a; h_t, h_a)   top-line current with the ordered prefix a attached
//   R(b; h_tb, h_b)  the t~-side row wtb^T S(J(b))
//   A(sigma; h) = wtb^T S(J(sigma)) wt + sum_{sigma = a|b} R(b) . O(a)
//   |M|^2 = sum_h sum_{sigma,tau} C_{sigma tau} Re(A(sigma; h) A(tau; h)^*)
//
// The generator (codegen.emit_program) lays the evaluation out as a flat
// program: stage L computes the gluon currents of length L+1, the top
// currents and t~ rows of length L, and at L = K-1 the full-length
// contractions, which it writes straight into the amplitudes.  Each stage is
// a set of independent items spread over the block's threads (tid, nt), read
// from precomputed operand records; stages are separated by __syncthreads().
// The stage functions are host-callable so the CPU test suite can run them
// one thread at a time against the oracle.
#pragma once
#include <cstddef>
#include <type_traits>
#include "mf_helas.cuh"
#include "mf_phasespace.cuh"
#include "mf_vertex.cuh"

template <int K> struct RecTraits;

#ifdef __CUDA_ARCH__
#define MF_TBL(NS, NAME, I) (NS::NAME[(I)])
#define MF_TBLP(NS, NAME) (NS::NAME)
#else
#define MF_TBL(NS, NAME, I) (NS::NAME##_h[(I)])
#define MF_TBLP(NS, NAME) (NS::NAME##_h)
#endif

#define MF_DEFINE_REC(KK)                                                                                 \
  template <> struct RecTraits<KK> {                                                                      \
    static constexpr int K = KK, J_TOTAL = rec##KK::J_TOTAL, O_TOTAL = rec##KK::O_TOTAL;                  \
    static constexpr int R_TOTAL = rec##KK::R_TOTAL, NSTAGE = rec##KK::NSTAGE;                            \
    static constexpr bool USE_MP = rec##KK::USE_MP;                                                       \
    static constexpr int NPERM = ttng##KK::NPERM, NCOMB = ttng##KK::NCOMB;                                \
    static constexpr double DENOMINATOR = ttng##KK::DENOMINATOR, COLOUR_DEN = ttng##KK::COLOUR_DEN;       \
    MF_D static int prog(int i) { return MF_TBL(rec##KK, prog, i); }                                      \
    /* the 4-int group of the program at int index i (a multiple of 4) */                                  \
    MF_D static int4 prog4(int i) { return reinterpret_cast<const int4*>(MF_TBLP(rec##KK, prog))[i >> 2]; } \
    MF_D static int2 prog2(int i) { return reinterpret_cast<const int2*>(MF_TBLP(rec##KK, prog))[i >> 1]; } \
    MF_D static int pdesc(int i) { return MF_TBL(rec##KK, pdesc, i); }                                    \
    MF_D static int stage_first(int i) { return MF_TBL(rec##KK, stage_first, i); }                        \
    MF_D static int arec(int i) { return MF_TBL(rec##KK, arec, i); }                                      \
    MF_D static int2 arec2(int i) { return reinterpret_cast<const int2*>(MF_TBLP(rec##KK, arec))[i >> 1]; } \
    MF_D static int hpack(int i) { return MF_TBL(rec##KK, hpack, i); }                                    \
    MF_D static int hunpack(int i) { return MF_TBL(rec##KK, hunpack, i); }                                \
    MF_D static int jo_ext(int i) { return MF_TBL(rec##KK, jo_ext, i); }                                  \
    MF_D static int cfg_to_mg(int i) { return MF_TBL(rec##KK, cfg_to_mg, i); }                            \
    MF_D static float colour(int i) { return MF_TBL(ttng##KK, colour_num, i); }                           \
    MF_HD static constexpr int pdesc_c(int i) { return rec##KK::pdesc_c[i]; }                             \
    MF_HD static constexpr int stage_first_c(int i) { return rec##KK::stage_first_c[i]; }                 \
  };

// Currents in shared memory as 16-byte planes: plane p holds bytes
// [16p, 16p+16) of every element, so threads touching consecutive elements
// read consecutive 16-byte words (no bank conflicts).
template <class T, int N> struct W4Planes {
  static constexpr int NPL = (int)(sizeof(W4<T>) / 16);
  int4 pl[NPL][N > 0 ? N : 1];
  // memcpy keeps the 16-byte moves free of aliasing assumptions
  MF_D W4<T> get(int i) const {
    int4 t[NPL];
#pragma unroll
    for (int p = 0; p < NPL; ++p) t[p] = pl[p][i];
    W4<T> w;
    memcpy(&w, t, sizeof(w));
    return w;
  }
  MF_D void put(int i, const W4<T>& w) {
    int4 t[NPL];
    memcpy(t, &w, sizeof(w));
#pragma unroll
    for (int p = 0; p < NPL; ++p) pl[p][i] = t[p];
  }
};

template <class T, int K> struct RecWS {
  using R = RecTraits<K>;
  W4Planes<T, R::J_TOTAL> J;
  W4Planes<T, R::O_TOTAL> O;
  W4Planes<T, R::R_TOTAL> RW;
  W4Planes<T, (R::USE_MP ? 8 * K : 0)> MP;  // wtb[tb]^T S(e_mu) O(g): [2 o + tb], o a one-gluon top current
  W4<T> WT[2], WTB[2];
  cx<T> A[R::NPERM * (1 << (K + 2))];  // [ordering][helicity combination]
};

MF_D int bit_reverse(int hp, int len) {
  int r = 0;
  for (int j = 0; j < len; ++j) r |= ((hp >> j) & 1) << (len - 1 - j);
  return r;
}

// Per-event data of the evaluation, built by one thread per event (in the
// phase-space kernel of an iteration, or prep_kernel for mf_smatrix) and
// loaded by the event's block: subset momenta and propagators, the external
// wavefunctions for both helicities, and the |M|^2 scale factor.
template <class T, int K> struct alignas(16) PrepRec {
  EvData<T, K> ev;
  W4<T> G[K][2];
  W4<T> WT[2], WTB[2];
  double scale;  // |GC_11|^2 / (colour denominator x average)
};

template <class T, int K>
MF_D void prep_event(PrepRec<T, K>& r, const double (*p)[4], double mt, double wt, cx<double> c10, cx<double> c11,
                     cx<double> c12) {
  using R = RecTraits<K>;
  if constexpr (std::is_same<T, float>::value)
    evdata_all_ff<K>(r.ev, p, mt, wt, c10, c11, c12);
  else
    for (int s = 0; s < (1 << K); ++s) evdata_subset<T, K>(r.ev, s, p, mt, wt, c10, c11, c12);
  for (int i = 0; i < K + 2; ++i)
    for (int c = 0; c < 4; ++c) r.ev.pext[i][c] = (T)p[i][c];
  r.ev.mt = (T)mt;
  const T sqh = (T)0.70710676908493042;  // madflow's float32-rounded sqrt(1/2)
  for (int q = 0; q < K; ++q) {
    int part = gluon_particle<K>(q);
    for (int b = 0; b < 2; ++b)
      r.G[q][b] = vxxxxx<T>(r.ev.pext[part], T(0), b ? T(1) : T(-1), part < 2 ? T(-1) : T(1), sqh);
  }
  for (int b = 0; b < 2; ++b) {
    r.WT[b] = oxxxxx<T>(r.ev.pext[2], r.ev.mt, b ? T(1) : T(-1), T(1));
    r.WTB[b] = ixxxxx<T>(r.ev.pext[3], r.ev.mt, b ? T(1) : T(-1), T(-1));
  }
  // the top-line bilinears of the four (top, anti-top) spin combinations,
  // M[q][mu] = WTB[q>>1]^T S(e_mu) WT[q&1]: an amplitude in which the full
  // gluon current J meets the top line directly is J . M (S is linear in J)
  for (int q = 0; q < 4; ++q)
    for (int mu = 0; mu < 4; ++mu) r.ev.M[q][mu] = dot4(unit_row(r.WTB[q >> 1], mu), r.WT[q & 1]);
  r.scale = (c11.re * c11.re + c11.im * c11.im) / (R::COLOUR_DEN * R::DENOMINATOR);
}

// stage 0: the external wavefunctions go to their slots (gluons: the
// length-1 J entries)
template <class T, int K> MF_D void rec_st_ext(RecWS<T, K>& ws, const PrepRec<T, K>& pr, int tid, int nt) {
  using R = RecTraits<K>;
  for (int i = tid; i < 2 * K + 4; i += nt) {
    if (i < 2 * K) ws.J.put(R::jo_ext(i >> 1) + (i & 1), pr.G[i >> 1][i & 1]);
    else if (i < 2 * K + 2) ws.WT[i - 2 * K] = pr.WT[i - 2 * K];
    else ws.WTB[i - 2 * K - 2] = pr.WTB[i - 2 * K - 2];
  }
}

// The record of one event straight to where the stages read it: the
// per-event data to pr, the gluon wavefunctions to their J slots and the
// quark spinors to ws.WT / ws.WTB (record load and stage 0 in one pass).
// NT threads, tid in [0, NT).
template <class T, int K, int NT>
MF_D void rec_load(RecWS<T, K>& ws, PrepRec<T, K>& pr, const int4* __restrict__ src, int tid) {
  using R = RecTraits<K>;
  using P = PrepRec<T, K>;
  constexpr int NW = (int)(sizeof(P) / 16), NPL = (int)(sizeof(W4<T>) / 16);
  constexpr int OG = (int)(offsetof(P, G) / 16), OWT = (int)(offsetof(P, WT) / 16);
  constexpr int OWTB = (int)(offsetof(P, WTB) / 16), OEND = OWTB + 2 * NPL;
  static_assert(OWT == OG + 2 * K * NPL && OWTB == OWT + 2 * NPL, "record layout");
  int4* dpr = reinterpret_cast<int4*>(&pr);
  int4* dwt = reinterpret_cast<int4*>(ws.WT);
  int4* dwtb = reinterpret_cast<int4*>(ws.WTB);
  for (int w = tid; w < NW; w += NT) {
    const int4 v = src[w];
    if (w < OG || w >= OEND) {
      dpr[w] = v;
    } else if (w < OWT) {
      const int idx = w - OG, wv = idx / NPL;
      ws.J.pl[idx % NPL][R::jo_ext(wv >> 1) + (wv & 1)] = v;
    } else if (w < OWTB) {
      dwt[w - OWT] = v;
    } else {
      dwtb[w - OWTB] = v;
    }
  }
}

// rec_load in two halves, so that the global loads of the next event's
// record overlap the current event's colour stage: rec_fetch reads this
// thread's 16-byte words of the record into registers, rec_store puts them
// where rec_load would.
template <class T, int K, int NT> struct RecFetch {
  static constexpr int NW = (int)(sizeof(PrepRec<T, K>) / 16);
  static constexpr int PER = (NW + NT - 1) / NT;
  int4 v[PER];
};
template <class T, int K, int NT>
MF_D void rec_fetch(RecFetch<T, K, NT>& f, const int4* __restrict__ src, int tid) {
#pragma unroll
  for (int i = 0; i < RecFetch<T, K, NT>::PER; ++i) {
    const int w = tid + i * NT;
    if (w < RecFetch<T, K, NT>::NW) f.v[i] = src[w];
  }
}
template <class T, int K, int NT>
MF_D void rec_store(RecWS<T, K>& ws, PrepRec<T, K>& pr, const RecFetch<T, K, NT>& f, int tid) {
  using R = RecTraits<K>;
  using P = PrepRec<T, K>;
  constexpr int NW = (int)(sizeof(P) / 16), NPL = (int)(sizeof(W4<T>) / 16);
  constexpr int OG = (int)(offsetof(P, G) / 16), OWT = (int)(offsetof(P, WT) / 16);
  constexpr int OWTB = (int)(offsetof(P, WTB) / 16), OEND = OWTB + 2 * NPL;
  int4* dpr = reinterpret_cast<int4*>(&pr);
  int4* dwt = reinterpret_cast<int4*>(ws.WT);
  int4* dwtb = reinterpret_cast<int4*>(ws.WTB);
#pragma unroll
  for (int i = 0; i < RecFetch<T, K, NT>::PER; ++i) {
    const int w = tid + i * NT;
    if (w >= NW) break;
    const int4 v = f.v[i];
    if (w < OG || w >= OEND) {
      dpr[w] = v;
    } else if (w < OWT) {
      const int idx = w - OG, wv = idx / NPL;
      ws.J.pl[idx % NPL][R::jo_ext(wv >> 1) + (wv & 1)] = v;
    } else if (w < OWTB) {
      dwt[w - OWT] = v;
    } else {
      dwtb[w - OWTB] = v;
    }
  }
}

// colour-ordered gluon current from a record (see codegen.emit_program):
// group i (1..L-1) of the record is split i, then one group per triple of the
// contact term; m is the subset of the whole sequence
template <class T, int K>
MF_D W4<T> rec_current(const RecWS<T, K>& ws, const EvData<T, K>& ev, int r, int L, int m, int hp) {
  using R = RecTraits<K>;
  W4<T> a3 = w4zero<T>(), a4 = w4zero<T>();
  for (int i = 1; i < L; ++i) {
    const int4 g = R::prog4(r + 4 * i);  // J offsets and subsets of both sides
    W4<T> a = ws.J.get(g.x + (hp & ((1 << i) - 1)));
    W4<T> b = ws.J.get(g.y + (hp >> i));
    // every term of the vertex, also in FP32: the conserved-current form
    // (which drops the a.Qa and b.Qb terms) lost up to 1e-2 of |M|^2 where
    // two gluons are nearly collinear, since FP32 currents are conserved
    // only up to rounding
    vvv_add<T>(a, ev.Qg[g.z], b, ev.Qg[g.w], a3);
  }
  int q = r + 4 * L;
  for (int i = 1; i < L; ++i)
    for (int j = i + 1; j < L; ++j, q += 4) {
      const int4 t = R::prog4(q);
      W4<T> a = ws.J.get(t.x + (hp & ((1 << i) - 1)));
      W4<T> b = ws.J.get(t.y + ((hp >> i) & ((1 << (j - i)) - 1)));
      W4<T> d = ws.J.get(t.z + (hp >> j));
      vvvv_add<T>(a, b, d, a4);
    }
  return combine<T>(ev.gv3[m], a3, ev.gv4[m], a4);
}

// one item of a program part
template <class T, int K>
MF_D void rec_item(RecWS<T, K>& ws, const EvData<T, K>& ev, int type, int L, int r, int sub) {
  using R = RecTraits<K>;
  constexpr int NC = 1 << (K + 2);
  if (type == 0) {  // gluon current, written for s and reverse(s)
    const int4 h = R::prog4(r);  // out, reversed out, sign, subset
    W4<T> v = rec_current<T, K>(ws, ev, r, L, h.w, sub);
    ws.J.put(h.x + sub, v);
    ws.J.put(h.y + bit_reverse(sub, L), h.z < 0 ? neg(v) : v);
  } else if (type == 1) {  // full length: bare contractions into the amplitudes
    const int4 h = R::prog4(r);  // ordering, reversed ordering, sign, subset
    W4<T> Jf = rec_current<T, K>(ws, ev, r, K, h.w, sub);
    const int s = h.x, srev = h.y, sg = h.z;
    const int hg = R::hunpack(s * (1 << K) + sub);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const cx<T> t = Jf.v[0] * ev.M[q][0] + Jf.v[1] * ev.M[q][1] + Jf.v[2] * ev.M[q][2] + Jf.v[3] * ev.M[q][3];
      int c = hg | ((q & 1) << K) | ((q >> 1) << (K + 1));
      ws.A[s * NC + c] = t;
      ws.A[srev * NC + c] = sg < 0 ? -t : t;
    }
  } else if (type == 2) {  // top-line current: out, subset, then (previous, J suffix) per split
    const int ht = sub >> L, hp = sub & ((1 << L) - 1);
    int4 g[(2 + 2 * (K - 1) + 3) / 4];
    for (int k = 0; k < (2 + 2 * L + 3) / 4; ++k) g[k] = R::prog4(r + 4 * k);
    const int* f = reinterpret_cast<const int*>(g);
    W4<T> y = w4zero<T>();
    for (int i = 0; i < L; ++i) {
      const int prev = f[2 + 2 * i], jsuf = f[3 + 2 * i];
      W4<T> Jb = ws.J.get(jsuf + (hp >> i));
      if (prev < 0) sv_add<T>(Jb, ws.WT[ht], y);
      else sv_add<T>(Jb, ws.O.get(prev + (ht << i) + (hp & ((1 << i) - 1))), y);
    }
    const int m = f[1];
    ws.O.put(f[0] + sub, topprop<T>(ev.Qt[m], ev.mt, ev.tden[m], y));
  } else if (type == 3) {  // t~ row: out, J
    const int htb = sub >> L, hp = sub & ((1 << L) - 1);
    const int2 g = R::prog2(r);
    ws.RW.put(g.x + sub, sandwich_row(ws.WTB[htb], ws.J.get(g.y + hp)));
  } else {  // bilinears of the one-gluon top current o: wtb[tb]^T S(e_mu) O(o)
    const int o = R::prog4(r).x + sub;
    const W4<T> Oo = ws.O.get(o);
#pragma unroll
    for (int tb = 0; tb < 2; ++tb) {
      W4<T> m;
#pragma unroll
      for (int mu = 0; mu < 4; ++mu) m.v[mu] = dot4(unit_row(ws.WTB[tb], mu), Oo);
      ws.MP.put(2 * o + tb, m);
    }
  }
}

// one stage (1..K-1) of the program: the parts' items are dealt to the
// threads round-robin as if they formed one list
template <class T, int K>
MF_D void rec_stage(RecWS<T, K>& ws, const EvData<T, K>& ev, int stage, int tid, int nt) {
  using R = RecTraits<K>;
  const int p0 = R::stage_first(stage - 1), p1 = R::stage_first(stage);
  int base = 0;
  for (int p = p0; p < p1; ++p) {
    const int type = R::pdesc(5 * p), L = R::pdesc(5 * p + 1);
    const int lper = (type <= 1) ? L : L + 1;  // items per node = 1 << lper
    const int cnt = R::pdesc(5 * p + 2) << lper;
    const int rec0 = R::pdesc(5 * p + 3), rsz = R::pdesc(5 * p + 4);
    int first = (tid - base) % nt;
    if (first < 0) first += nt;
    for (int local = first; local < cnt; local += nt)
      rec_item<T, K>(ws, ev, type, L, rec0 + (local >> lper) * rsz, local & ((1 << lper) - 1));
    base += cnt;
  }
}

// Two top-line items of a part that differ in the top spin (type 2) or the
// anti-top spin (type 3) only: sub and sub + 2^L, sub < 2^L.  They share
// their gluon-current loads and the spin-independent products of those.
// Same results as rec_item on each.  (Pairing the gluon-current items the
// same way was measured slower: the paired currents need more registers.)
template <class T, int K, int TYPE, int L>
MF_D void rec_item2(RecWS<T, K>& ws, const EvData<T, K>& ev, int r, int sub) {
  using R = RecTraits<K>;
  static_assert(TYPE == 2 || TYPE == 3, "top-line items only");
  if constexpr (TYPE == 2) {
    const int hp = sub;  // top spin 0; its partner has top spin 1
    int4 g[(2 + 2 * L + 3) / 4];
#pragma unroll
    for (int k = 0; k < (2 + 2 * L + 3) / 4; ++k) g[k] = R::prog4(r + 4 * k);
    const int* f = reinterpret_cast<const int*>(g);
    W4<T> y0 = w4zero<T>(), y1 = w4zero<T>();
#pragma unroll
    for (int i = 0; i < L; ++i) {
      const int prev = f[2 + 2 * i], jsuf = f[3 + 2 * i];
      const W4<T> Jb = ws.J.get(jsuf + (hp >> i));
      if (prev < 0) {
        sv_add<T>(Jb, ws.WT[0], y0);
        sv_add<T>(Jb, ws.WT[1], y1);
      } else {
        const int o = prev + (hp & ((1 << i) - 1));
        sv_add<T>(Jb, ws.O.get(o), y0);
        sv_add<T>(Jb, ws.O.get(o + (1 << i)), y1);
      }
    }
    const int m = f[1];
    ws.O.put(f[0] + hp, topprop<T>(ev.Qt[m], ev.mt, ev.tden[m], y0));
    ws.O.put(f[0] + hp + (1 << L), topprop<T>(ev.Qt[m], ev.mt, ev.tden[m], y1));
  } else {
    const int2 g = R::prog2(r);  // out, J
    const W4<T> V = ws.J.get(g.y + sub);
    ws.RW.put(g.x + sub, sandwich_row(ws.WTB[0], V));
    ws.RW.put(g.x + sub + (1 << L), sandwich_row(ws.WTB[1], V));
  }
}

// items in parts P..PEND-1 of the part table
template <int K, int P, int PEND> MF_HD constexpr int rec_part_items() {
  using R = RecTraits<K>;
  if constexpr (P < PEND) {
    constexpr int type = R::pdesc_c(5 * P), L = R::pdesc_c(5 * P + 1);
    return (R::pdesc_c(5 * P + 2) << ((type <= 1) ? L : L + 1)) + rec_part_items<K, P + 1, PEND>();
  } else {
    return 0;
  }
}

// The same stage with the part table folded in at compile time (part P of
// stage STAGE; the item loops keep their run-time node index only).  With
// PAIR each thread takes the top-line items two at a time (rec_item2): used
// for four or more gluons where the stage has more items than threads.
template <class T, int K, int P, int PEND, int NT, bool PAIR>
MF_D void rec_stage_parts(RecWS<T, K>& ws, const EvData<T, K>& ev, int tid, int base) {
  if constexpr (P < PEND) {
    using R = RecTraits<K>;
    constexpr int type = R::pdesc_c(5 * P), L = R::pdesc_c(5 * P + 1);
    constexpr bool pair = PAIR && (type == 2 || type == 3);
    constexpr int lper = ((type <= 1) ? L : L + 1) - (pair ? 1 : 0);
    constexpr int cnt = R::pdesc_c(5 * P + 2) << lper;
    constexpr int rec0 = R::pdesc_c(5 * P + 3), rsz = R::pdesc_c(5 * P + 4);
    int first = (tid - base) % NT;
    if (first < 0) first += NT;
    for (int local = first; local < cnt; local += NT) {
      if constexpr (pair)
        rec_item2<T, K, type, L>(ws, ev, rec0 + (local >> lper) * rsz, local & ((1 << lper) - 1));
      else
        rec_item<T, K>(ws, ev, type, L, rec0 + (local >> lper) * rsz, local & ((1 << lper) - 1));
    }
    rec_stage_parts<T, K, P + 1, PEND, NT, PAIR>(ws, ev, tid, base + cnt);
  }
}
template <class T, int K, int STAGE, int NT>
MF_D void rec_stage_c(RecWS<T, K>& ws, const EvData<T, K>& ev, int tid) {
  using R = RecTraits<K>;
  constexpr int P0 = R::stage_first_c(STAGE - 1), P1 = R::stage_first_c(STAGE);
  // (measured: pairs pay from four gluons on; with three they cost 17-24%)
  constexpr bool PAIR = K >= 4 && rec_part_items<K, P0, P1>() > NT;
  rec_stage_parts<T, K, P0, P1, NT, PAIR>(ws, ev, tid, 0);
}
// stages STAGE..K-1, each followed by a block barrier (a warp barrier when
// one warp evaluates the event, NT = 32); a thread with on = false only
// takes part in the barriers
template <class T, int K, int STAGE, int NT>
MF_DO void rec_stages_c(RecWS<T, K>& ws, const EvData<T, K>& ev, int tid, bool on = true) {
  if constexpr (STAGE < K) {
    if (on) rec_stage_c<T, K, STAGE, NT>(ws, ev, tid);
    if constexpr (NT == 32)
      __syncwarp();
    else
      __syncthreads();
    rec_stages_c<T, K, STAGE + 1, NT>(ws, ev, tid, on);
  }
}

// stage A: add the top-line terms to every amplitude.  An item is one
// ordering and one assignment of the gluon helicities (in ordering
// position); it owns the four (top, anti-top) helicity combinations, so each
// top-line current and t~ row it reads serves two products.
template <class T, int K> MF_D void rec_st_A(RecWS<T, K>& ws, int tid, int nt) {
  using R = RecTraits<K>;
  constexpr int NC = 1 << (K + 2), NG = 1 << K;
  for (int it = tid; it < NG * R::NPERM; it += nt) {
    const int s = it / NG, hfull = it % NG;
    const int hg = R::hunpack(s * NG + hfull);
    cx<T> a[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) a[q] = ws.A[s * NC + (hg | ((q & 1) << K) | ((q >> 1) << (K + 1)))];
#pragma unroll
    for (int i = 1; i < K; ++i) {
      const int2 orr = R::arec2(s * 2 * (K - 1) + 2 * (i - 1));  // top current, t~ row
      const int oo = orr.x, ro = orr.y;
      const int lo = hfull & ((1 << i) - 1), hi = hfull >> i;
      if (R::USE_MP && i == 1) {
        // R(b) . O(a) = J(b) . MP(a) for the one-gluon prefix a (ro: the
        // J offset of the suffix b)
        const W4<T> Js = ws.J.get(ro + hi);
        const int o0 = oo + lo, o1 = oo + 2 + lo;
        a[0] += dot4(Js, ws.MP.get(2 * o0));
        a[1] += dot4(Js, ws.MP.get(2 * o1));
        a[2] += dot4(Js, ws.MP.get(2 * o0 + 1));
        a[3] += dot4(Js, ws.MP.get(2 * o1 + 1));
      } else {
        W4<T> O0 = ws.O.get(oo + lo), O1 = ws.O.get(oo + (1 << i) + lo);
        W4<T> R0 = ws.RW.get(ro + hi), R1 = ws.RW.get(ro + (1 << (K - i)) + hi);
        a[0] += dot4(R0, O0);
        a[1] += dot4(R0, O1);
        a[2] += dot4(R1, O0);
        a[3] += dot4(R1, O1);
      }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) ws.A[s * NC + (hg | ((q & 1) << K) | ((q >> 1) << (K + 1)))] = a[q];
  }
}

// Colour sum sum_c A(c)^dagger C A(c) with C real symmetric:
//   sum_a C_aa |A_a|^2 + 2 sum_{b>a} C_ab Re(A_a A_b^*).
// Rows a and NP-1-a together hold NP+1 matrix entries, so the NP/2 row pairs
// are equal shares; an item is one helicity combination and one of
// COLOUR_PARTS groups of row pairs.  The amplitudes of the combination sit in
// registers and the integer numerators are compile-time operands.
template <int K> MF_HD constexpr int colour_parts() {
  constexpr int np = RecTraits<K>::NPERM, nc = 1 << (K + 2);
  constexpr int want = 192 / nc > 0 ? 192 / nc : 1;
  return want < np / 2 ? want : np / 2;
}
template <class T, int K, int PART> MF_D T colour_rows(const RecWS<T, K>& ws, int c) {
  using R = RecTraits<K>;
  constexpr int NP = R::NPERM, NC = 1 << (K + 2), P = colour_parts<K>();
  static_assert(NP % 2 == 0, "row pairing needs an even number of orderings");
  cx<T> A[NP];
#pragma unroll
  for (int b = 0; b < NP; ++b) A[b] = ws.A[b * NC + c];
  T acc = T(0);
#pragma unroll
  for (int g = PART; g < NP / 2; g += P) {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int a = h ? NP - 1 - g : g;
      cx<T> z = {T(0), T(0)};
#pragma unroll
      for (int b = a + 1; b < NP; ++b) z += (T)R::colour(a * NP + b) * A[b];
      acc += (T)R::colour(a * NP + a) * (A[a].re * A[a].re + A[a].im * A[a].im) +
             T(2) * (A[a].re * z.re + A[a].im * z.im);
    }
  }
  return acc;
}
template <class T, int K, int PART, bool LAST = (PART == colour_parts<K>() - 1)> struct ColourDispatch {
  MF_D static T run(const RecWS<T, K>& ws, int c, int p) {
    if (p == PART) return colour_rows<T, K, PART>(ws, c);
    return ColourDispatch<T, K, PART + 1>::run(ws, c, p);
  }
};
template <class T, int K, int PART> struct ColourDispatch<T, K, PART, true> {
  MF_D static T run(const RecWS<T, K>& ws, int c, int) { return colour_rows<T, K, PART>(ws, c); }
};
// Colour sum for many flows (120 for five gluons): an item is one row a and
// one helicity combination c, z = sum_{b>a} C_ab A_b(c); neighbouring threads
// take neighbouring c, so C_ab is the same across a warp.
template <class T, int K> MF_D T rec_st_colour_rows(const RecWS<T, K>& ws, int tid, int nt) {
  using R = RecTraits<K>;
  constexpr int NP = R::NPERM, NC = 1 << (K + 2);
  T acc = T(0);
  for (int it = tid; it < NC * NP; it += nt) {
    const int a = it / NC, c = it % NC;
    cx<T> z = {T(0), T(0)};
    for (int b = a + 1; b < NP; ++b) z += (T)R::colour(a * NP + b) * ws.A[b * NC + c];
    const cx<T> Aa = ws.A[it];
    acc += (T)R::colour(a * NP + a) * (Aa.re * Aa.re + Aa.im * Aa.im) + T(2) * (Aa.re * z.re + Aa.im * z.im);
  }
  return acc;
}
template <class T, int K> MF_D T rec_st_colour(const RecWS<T, K>& ws, int tid, int nt) {
  if constexpr (RecTraits<K>::NPERM > 24) {
    return rec_st_colour_rows<T, K>(ws, tid, nt);
  } else {
    constexpr int NC = 1 << (K + 2), P = colour_parts<K>();
    T acc = T(0);
    for (int it = tid; it < NC * P; it += nt) acc += ColourDispatch<T, K, 0>::run(ws, it % NC, it / NC);
    return acc;
  }
}

// colour sum of one helicity combination c (per-helicity outputs)
template <class T, int K> MF_D double rec_colour_one(const RecWS<T, K>& ws, int c) {
  using R = RecTraits<K>;
  constexpr int NP = R::NPERM, NC = 1 << (K + 2);
  double acc = 0.0;
  for (int a = 0; a < NP; ++a) {
    cx<T> z = {T(0), T(0)};
    for (int b = a + 1; b < NP; ++b) z += (T)R::colour(a * NP + b) * ws.A[b * NC + c];
    cx<T> Aa = ws.A[a * NC + c];
    acc += (double)((T)R::colour(a * NP + a) * (Aa.re * Aa.re + Aa.im * Aa.im) + T(2) * (Aa.re * z.re + Aa.im * z.im));
  }
  return acc;
}

// the whole evaluation of one event by nt "threads" run one at a time (host tests)
template <class T, int K> struct RecHostRun {
  static double run(RecWS<T, K>& ws, const PrepRec<T, K>& pr, int nt) {
    for (int t = 0; t < nt; ++t) rec_st_ext<T, K>(ws, pr, t, nt);
    for (int st = 1; st < K; ++st)
      for (int t = 0; t < nt; ++t) rec_stage<T, K>(ws, pr.ev, st, t, nt);
    for (int t = 0; t < nt; ++t) rec_st_A<T, K>(ws, t, nt);
    double tot = 0.0;
    for (int t = 0; t < nt; ++t) tot += (double)rec_st_colour<T, K>(ws, t, nt);
    return tot;
  }
  // the same through the compile-time stage driver the kernels use (with
  // NT threads: every stage with more than NT items runs paired items)
  template <int NT> static double run_c(RecWS<T, K>& ws, const PrepRec<T, K>& pr) {
    for (int t = 0; t < NT; ++t) rec_st_ext<T, K>(ws, pr, t, NT);
    stages_c<1, NT>(ws, pr.ev);
    for (int t = 0; t < NT; ++t) rec_st_A<T, K>(ws, t, NT);
    double tot = 0.0;
    for (int t = 0; t < NT; ++t) tot += (double)rec_st_colour<T, K>(ws, t, NT);
    return tot;
  }
  template <int ST, int NT> static void stages_c(RecWS<T, K>& ws, const EvData<T, K>& ev) {
    if constexpr (ST < K) {
      for (int t = 0; t < NT; ++t) rec_stage_c<T, K, ST, NT>(ws, ev, t);
      stages_c<ST + 1, NT>(ws, ev);
    }
  }
};

constexpr int MF_REC_NT = 192;  // threads per event block

template <class T, int K> struct RecSmem {
  RecWS<T, K> ws;
  PrepRec<T, K> pr;
  T red[MF_REC_NT / 32];
  unsigned long long mbar;  // tensor-core colour stage: MMA completion
  uint32_t tmem;            // its tensor-memory accumulator
  int tc_err;               // a bounded wait ran out
};
template <class T, int K> MF_HD constexpr int prep_words() { return (int)(sizeof(PrepRec<T, K>) / 16); }

#include "mf_colour_tc.cuh"

#ifdef __CUDACC__
// Per-event records from momenta ps [K+2][4][N] and couplings [N or 1][3]
// complex (one thread per event).
template <int K, class T>
__global__ void __launch_bounds__(128) prep_kernel(const double* __restrict__ ps, int64_t N, double mt, double wt,
                                                   const double* __restrict__ coup, int64_t cstride,
                                                   int4* __restrict__ prep) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    double p[K + 2][4];
    for (int i = 0; i < K + 2; ++i)
      for (int c = 0; c < 4; ++c) p[i][c] = ps[((int64_t)i * 4 + c) * N + e];
    const double* cp = coup + 6 * cstride * e;
    PrepRec<T, K> r;
    prep_event<T, K>(r, p, mt, wt, {cp[0], cp[1]}, {cp[2], cp[3]}, {cp[4], cp[5]});
    const int4* src = reinterpret_cast<const int4*>(&r);
    int4* dst = prep + (int64_t)e * prep_words<T, K>();
    for (int w = 0; w < prep_words<T, K>(); ++w) dst[w] = src[w];
  }
}

// One event by the whole block with the SIMT colour sum (launches that mix
// processes): record load, stages, amplitudes, colour sum, block reduction.
// Returns |M|^2 in thread 0.
template <class T, int K, int NT> MF_DO double me_rec_event(RecSmem<T, K>& S, const int4* __restrict__ rec, int tid) {
  constexpr int nt = NT;
  rec_load<T, K, NT>(S.ws, S.pr, rec, tid);
  __syncthreads();
  rec_stages_c<T, K, 1, NT>(S.ws, S.pr.ev, tid);
  rec_st_A<T, K>(S.ws, tid, nt);
  __syncthreads();
  T part = rec_st_colour<T, K>(S.ws, tid, nt);
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((tid & 31) == 0) S.red[tid >> 5] = part;
  __syncthreads();
  double r = 0.0;
  if (tid == 0) {
    T tot = T(0);
    for (int w = 0; w < nt / 32; ++w) tot += S.red[w];
    r = (double)tot * S.pr.scale;
  }
  return r;
}

// After a bounded tensor-core wait ran out: the events e, e + stride, ...
// below N of a block get NaN in out (and hel_out), except events with
// skip[e] == +-0, which need no work and get 0 as usual.  Every thread of the
// block takes part (no barrier); thread tid writes the helicity rows tid,
// tid + nt, ...
template <int K>
MF_DO void mark_rest_nan(int64_t e, int64_t N, int64_t stride, const double* __restrict__ skip,
                         double* __restrict__ out, double* __restrict__ hel_out, int tid, int nt) {
  const double qnan = __longlong_as_double(0x7ff8000000000000ll);
  for (; e < N; e += stride) {
    const bool none = skip && (__double_as_longlong(skip[e]) << 1) == 0;
    if (tid == 0) out[e] = none ? 0.0 : qnan;
    if (hel_out && !none)
      for (int c = tid; c < (1 << (K + 2)); c += nt) hel_out[(int64_t)c * N + e] = qnan;
  }
}

// Processes whose workspace does not fit in shared memory (five gluons: 523
// KB in FP32) keep it in global memory, one per block (ws [gridDim]); the
// record and the reduction stay in shared memory.  Same stages and outputs
// as me_rec_kernel.  COLOUR = 1 (FP32, 128 helicity combinations, flows a
// multiple of 40): the colour sum on the tensor cores, one 128-row half of
// the amplitude matrix (Re, then Im) at a time, K in chunks of 40 flows
// (5 MMA K-steps each, A_hi and A_lo), C^T resident in shared memory, the
// accumulator (128 columns) in tensor memory; else the row-loop SIMT sum.
constexpr int MF_GWS_NT = 640;  // threads per block of the global-workspace kernel
template <class T, int K> struct RecSmemG {
  PrepRec<T, K> pr;
  T red[MF_GWS_NT / 32];
  unsigned long long mbar;
  uint32_t tmem;
  int tc_err;
};
constexpr int MF_GWS_KC = 40;  // flows per K chunk of the tensor-core colour sum
template <class T, int K> constexpr bool use_colour_tc_gws() {
  return MF_TCGEN05 && TcTraits<K>::enabled && sizeof(T) == 4 && (1 << (K + 2)) == 128 &&
         RecTraits<K>::NPERM % MF_GWS_KC == 0 && MF_GWS_NT >= 128;
}
// shared-memory bytes of the tensor-core colour operands: B (all flows),
// A_hi and A_lo of one 128-row half and one K chunk
template <int K> constexpr int gws_tc_bytes() {
  return TcTraits<K>::enabled ? (TcTraits<K>::N * RecTraits<K>::NPERM + 2 * 128 * MF_GWS_KC) * 4 : 0;
}
template <class T, int K> constexpr int gws_smem_bytes(int colour) {
  return colour == 1 && TcTraits<K>::enabled ? (int)((sizeof(RecSmemG<T, K>) + 1023) / 1024 * 1024) + gws_tc_bytes<K>()
                                             : (int)sizeof(RecSmemG<T, K>);
}
template <int K, class T, int COLOUR>
__global__ void __launch_bounds__(MF_GWS_NT)
    me_gws_kernel(const int4* __restrict__ prep, int64_t N, const double* __restrict__ skip,
                  double* __restrict__ out, double* __restrict__ hel_out, RecWS<T, K>* __restrict__ ws_all,
                  int* __restrict__ err, uint32_t wait_tries) {
  using R = RecTraits<K>;
  constexpr bool TC = COLOUR == 1 && use_colour_tc_gws<T, K>();
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  RecSmemG<T, K>& S = *reinterpret_cast<RecSmemG<T, K>*>(smem_raw);
  RecWS<T, K>& ws = ws_all[blockIdx.x];
  const int tid = threadIdx.x;
  constexpr int nt = MF_GWS_NT;  // launched with MF_GWS_NT threads
  constexpr int NW = prep_words<T, K>();
#if MF_TCGEN05
  float* tcB = nullptr;
  uint32_t phase = 0;
  if constexpr (TC) {
    constexpr int NP = R::NPERM;
    tcB = reinterpret_cast<float*>(smem_raw + (sizeof(RecSmemG<T, K>) + 1023) / 1024 * 1024);
    // C^T for every K chunk, resident for the whole launch
    const int4* src = reinterpret_cast<const int4*>(TcTraits<K>::b());
    int4* dB = reinterpret_cast<int4*>(tcB);
    for (int i = tid; i < TcTraits<K>::N * NP / 4; i += nt) dB[i] = src[i];
    if (tid < 32) tc_tmem_alloc(&S.tmem, 128);
    if (tid == 0) {
      tc_mbar_init(&S.mbar, 1);
      S.tc_err = 0;
    }
    tc_fence_proxy_async();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  }
#endif
  for (int64_t e = blockIdx.x; e < N; e += gridDim.x) {
    if (skip && (__double_as_longlong(skip[e]) << 1) == 0) {
      if (tid == 0) out[e] = 0.0;
      continue;
    }
    __syncthreads();
    rec_load<T, K, nt>(ws, S.pr, prep + e * NW, tid);
    __syncthreads();
    rec_stages_c<T, K, 1, nt>(ws, S.pr.ev, tid);
    rec_st_A<T, K>(ws, tid, nt);
    __syncthreads();
    T part = T(0);
    bool bad = false;
#if MF_TCGEN05
    if constexpr (TC) {
      constexpr int NP = R::NPERM, NC = 1 << (K + 2), KC = MF_GWS_KC, NCH = NP / KC;
      constexpr uint32_t SBA = (KC / 4) * 128;  // A chunk: 8-row groups
      constexpr uint32_t idesc = tc_idesc_tf32(128, TcTraits<K>::N);
      float* hi = tcB + TcTraits<K>::N * NP;
      float* lo = hi + 128 * KC;
      const uint32_t bB = tc_smem_u32(tcB), bh = tc_smem_u32(hi), bl = tc_smem_u32(lo);
      for (int h = 0; h < 2; ++h) {  // 0: Re rows, 1: Im rows
        for (int q = 0; q < NCH; ++q) {
          // A_hi, A_lo of rows c, flows [q KC, (q+1) KC), canonical K-major layout
          for (int it = tid; it < NC * (KC / 4); it += nt) {
            const int c = it % NC, k4 = it / NC;
            float vh[4], vl[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const cx<float> a = ws.A[(q * KC + 4 * k4 + j) * NC + c];
              const float v = h ? a.im : a.re;
              vh[j] = tc_hi(v);
              vl[j] = v - vh[j];
            }
            const int o = (c / 8) * (KC / 4) * 32 + k4 * 32 + (c % 8) * 4;
            *reinterpret_cast<float4*>(hi + o) = make_float4(vh[0], vh[1], vh[2], vh[3]);
            *reinterpret_cast<float4*>(lo + o) = make_float4(vl[0], vl[1], vl[2], vl[3]);
          }
          tc_fence_proxy_async();
          __syncthreads();
          if (tid == 0) {
            tc_fence_after();
#pragma unroll
            for (int s = 0; s < KC / 8; ++s) {
              const uint64_t db = tc_smem_desc(bB + 256 * (q * (KC / 8) + s), TcTraits<K>::LBO, TcTraits<K>::SBO);
              tc_mma_tf32(S.tmem, tc_smem_desc(bh + 256 * s, 128, SBA), db, idesc, (q > 0 || s > 0) ? 1u : 0u);
              tc_mma_tf32(S.tmem, tc_smem_desc(bl + 256 * s, 128, SBA), db, idesc, 1u);
            }
            tc_commit(&S.mbar);
          }
          // every thread waits: the next chunk overwrites the operands
          bool done = false;
          for (uint32_t spin = 0; spin < wait_tries; ++spin) {
            done = tc_mbar_try_wait(&S.mbar, phase, 1000000u);
            if (__all_sync(0xffffffffu, done)) break;
          }
          done = __all_sync(0xffffffffu, done);
          if (!done) S.tc_err = 1;
          phase ^= 1u;
          __syncthreads();
          if (S.tc_err) break;
        }
        if (S.tc_err) break;
        if (tid < 128) {
          tc_fence_after();
          const uint32_t ta = S.tmem + ((uint32_t)(32 * (tid >> 5)) << 16);
          float acc = 0.0f;
#pragma unroll
          for (int cb = 0; cb < NP; cb += 8) {
            float d[8];
            tc_ld_x8(ta + cb, d);
            tc_wait_ld();
#pragma unroll
            for (int t = 0; t < 8; ++t) {
              const cx<float> a = ws.A[(cb + t) * NC + tid];
              acc += d[t] * (h ? a.im : a.re);
            }
          }
          part += acc;
          tc_fence_before();
        }
        __syncthreads();  // the accumulator is read before the next half overwrites it
      }
      bad = S.tc_err != 0;
    } else
#endif
    {
      part = rec_st_colour<T, K>(ws, tid, nt);
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((tid & 31) == 0) S.red[tid >> 5] = part;
    const double sc = S.pr.scale;
    if (hel_out)
      for (int c = tid; c < (1 << (K + 2)); c += nt)
        hel_out[(int64_t)R::cfg_to_mg(c) * N + e] = rec_colour_one<T, K>(ws, c) * sc * R::DENOMINATOR;
    __syncthreads();
    if (tid == 0) {
      T tot = T(0);
      for (int w = 0; w < nt / 32; ++w) tot += S.red[w];
      out[e] = bad ? __longlong_as_double(0x7ff8000000000000ll) : (double)tot * sc;
      if (bad && err) atomicOr(err, 1);
    }
    if (bad) {
      // the tensor cores are no longer trusted: every later event of this
      // block that needs work gets NaN (no stale value survives in out)
      mark_rest_nan<K>(e + gridDim.x, N, gridDim.x, skip, out, hel_out, tid, nt);
      break;
    }
  }
#if MF_TCGEN05
  if constexpr (TC) {
    __syncthreads();
    if (S.tc_err) {
      bool done = false;
      for (uint32_t spin = 0; spin < 1000u && !done; ++spin) done = tc_mbar_try_wait(&S.mbar, phase ^ 1u, 1000000u);
    }
    if (tid < 32) {
      tc_fence_after();
      tc_tmem_dealloc(S.tmem, 128);
    }
  }
#endif
}

// Block-per-event |M|^2 from the per-event records prep [N][prep_words];
// skip (optional) [N]: events with skip[e] == 0 get out[e] = 0 without work;
// out [N]; hel_out (optional) [ncomb][N] in MadGraph helicity order.
// COLOUR = 1: FP32 processes with a tensor-core colour operand take the
// colour sum on the tensor cores (mf_colour_tc.cuh); err (optional) gets bit
// 0 set, and the remaining events of the block NaN, if a wait on the tensor
// cores ran out.  COLOUR = 0: the register-tiled SIMT colour sum.
template <class T, int K> constexpr bool use_colour_tc() {
  return MF_TCGEN05 && TcTraits<K>::enabled && sizeof(T) == 4 && (2 << (K + 2)) == 128 &&
         MF_REC_NT >= 128;
}
template <int K, class T, int COLOUR>
__global__ void __launch_bounds__(MF_REC_NT, sizeof(T) == 4 ? 4 : 2)
    me_rec_kernel(const int4* __restrict__ prep, int64_t N, const double* __restrict__ skip,
                  double* __restrict__ out, double* __restrict__ hel_out, int* __restrict__ err,
                  uint32_t wait_tries) {
  using R = RecTraits<K>;
  constexpr bool TC = COLOUR == 1 && use_colour_tc<T, K>();
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  RecSmem<T, K>& S = *reinterpret_cast<RecSmem<T, K>*>(smem_raw);
  // launched with MF_REC_NT threads: a compile-time stride for every item loop
  const int tid = threadIdx.x;
  constexpr int nt = MF_REC_NT;
  constexpr int NW = prep_words<T, K>();
#if MF_TCGEN05
  // operands in the shared memory of the top-line currents and t~ rows,
  // which are dead once the amplitudes are complete
  float* tc_region = nullptr;
  uint32_t phase = 0;
  if constexpr (TC) {
    static_assert(sizeof(S.ws.O) + sizeof(S.ws.RW) >= (size_t)tc_operand_bytes<K>() + 128, "operand space");
    uintptr_t o = reinterpret_cast<uintptr_t>(&S.ws.O);
    tc_region = reinterpret_cast<float*>((o + 127) & ~(uintptr_t)127);
    if (tid < 32) tc_tmem_alloc(&S.tmem, 32);
    if (tid == 0) {
      tc_mbar_init(&S.mbar, 1);
      S.tc_err = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
  }
#endif
  // the next event of this block that needs work (events with skip == 0
  // get out = 0 on the way), and the loading of its record + external slots
  // (the skip test on the bits: +-0.0, without the FP64 pipe)
  auto next_event = [&](int64_t e) {
    while (e < N && skip && (__double_as_longlong(skip[e]) << 1) == 0) {
      if (tid == 0) out[e] = 0.0;
      e += gridDim.x;
    }
    return e;
  };
  auto load_ext = [&](int64_t e) { rec_load<T, K, nt>(S.ws, S.pr, prep + e * NW, tid); };
  int64_t e = next_event(blockIdx.x);
  if (e < N) load_ext(e);
  while (e < N) {
    __syncthreads();
    rec_stages_c<T, K, 1, nt>(S.ws, S.pr.ev, tid);
    rec_st_A<T, K>(S.ws, tid, nt);
    __syncthreads();
    const double sc = S.pr.scale;
    const int64_t en = next_event(e + gridDim.x);
    T part = T(0);
    bool bad = false;

#if MF_TCGEN05
    if constexpr (TC) {
      constexpr int NP = R::NPERM, NC = 1 << (K + 2);
      tc_fill<K>(S.ws, tc_region, tid, nt);
      tc_fence_proxy_async();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        const uint32_t b = tc_smem_u32(tc_region);
        const uint32_t hi = b + TcTraits<K>::N * NP * 4, lo = hi + 2 * NC * NP * 4;
        constexpr uint32_t idesc = tc_idesc_tf32(2 * NC, TcTraits<K>::N);
        constexpr uint32_t L = TcTraits<K>::LBO, SB = TcTraits<K>::SBO;
#pragma unroll
        for (int s = 0; s < NP / 8; ++s)
          tc_mma_tf32(S.tmem, tc_smem_desc(hi + 256 * s, L, SB), tc_smem_desc(b + 256 * s, L, SB), idesc, s > 0);
#pragma unroll
        for (int s = 0; s < NP / 8; ++s)
          tc_mma_tf32(S.tmem, tc_smem_desc(lo + 256 * s, L, SB), tc_smem_desc(b + 256 * s, L, SB), idesc, 1);
        tc_commit(&S.mbar);
      }
      // while the tensor cores work: the next event's record and external
      // slots (its record, the gluon slots of J and the quark spinors; none
      // of them is an MMA operand or read by this event's epilogue)
      if (en < N) load_ext(en);
      if (tid < 2 * NC) {
        // bounded, warp-uniform wait (the accumulator loads are warp-collective)
        // (each try suspends for up to 1 ms; 1000 tries bound the wait to ~1 s)
        bool done = false;
        for (uint32_t spin = 0; spin < wait_tries; ++spin) {
          done = tc_mbar_try_wait(&S.mbar, phase, 1000000u);
          if (__all_sync(0xffffffffu, done)) break;
        }
        done = __all_sync(0xffffffffu, done);
        if (done) {
          tc_fence_after();
          float d[32];
          const uint32_t ta = S.tmem + ((uint32_t)(32 * (tid >> 5)) << 16);
          tc_ld_x16(ta, d);
          tc_ld_x8(ta + 16, d + 16);
          tc_wait_ld();
          const int c = tid % NC, im = tid / NC;
          float acc = 0.0f;
#pragma unroll
          for (int t = 0; t < NP; ++t) {
            const cx<float> a = S.ws.A[t * NC + c];
            acc += d[t] * (im ? a.im : a.re);
          }
          part = acc;
        } else {
          S.tc_err = 1;
        }
        tc_fence_before();
      }
      phase ^= 1u;
    } else
#endif
    {
      part = rec_st_colour<T, K>(S.ws, tid, nt);
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((tid & 31) == 0) S.red[tid >> 5] = part;
    if (hel_out)
      for (int c = tid; c < (1 << (K + 2)); c += nt)
        hel_out[(int64_t)R::cfg_to_mg(c) * N + e] = rec_colour_one<T, K>(S.ws, c) * sc * R::DENOMINATOR;
    __syncthreads();
    if constexpr (TC) bad = S.tc_err != 0;
    if (tid == 0) {
      T tot = T(0);
      for (int w = 0; w < nt / 32; ++w) tot += S.red[w];
      out[e] = bad ? __longlong_as_double(0x7ff8000000000000ll) : (double)tot * sc;
      if (bad && err) atomicOr(err, 1);
    }
    if (bad) {
      // every later event of this block that needs work gets NaN
      mark_rest_nan<K>(en, N, gridDim.x, skip, out, hel_out, tid, nt);
      break;
    }
    if constexpr (!TC)
      if (en < N) load_ext(en);
    e = en;
  }
#if MF_TCGEN05
  if constexpr (TC) {
    __syncthreads();
    if (S.tc_err) {
      // let an unfinished MMA drain (bounded) before its accumulator is freed
      bool done = false;
      for (uint32_t spin = 0; spin < 1000u && !done; ++spin) done = tc_mbar_try_wait(&S.mbar, phase ^ 1u, 1000000u);
    }
    if (tid < 32) {
      tc_fence_after();
      tc_tmem_dealloc(S.tmem, 32);
    }
  }
#endif
}
// Processes with few helicities and colour flows (two and three gluons) run
// one event per warp; four and five gluons one event per block.
template <int K> constexpr bool one_warp_per_event() { return K <= 3; }

// One warp per event (two and three gluons): every warp of the grid follows
// its own sequence of events (warp w of the grid takes w, w + W, w + 2W, ...,
// W the warps in the grid), with its own record in shared memory and only
// warp barriers between the stages, so no warp waits for another.  The
// warp looks for its next event and fetches its record into registers
// before the colour stage, which hides their loads.
// Warp-uniform: the warp's next event at or after cursor c (stride G) that
// needs work (e, -1 if none); the skipped ones before it get out = 0.
MF_DO int64_t next_warp_event(int64_t c, int64_t G, int64_t N, const double* __restrict__ skip,
                              double* __restrict__ out, int lane, int64_t& e) {
  for (;;) {
    const int64_t cand = c + (int64_t)lane * G;
    const bool inrange = cand < N;
    const bool need = inrange && !(skip && (__double_as_longlong(skip[cand]) << 1) == 0);
    const unsigned nm = __ballot_sync(0xffffffffu, need);
    if (__ballot_sync(0xffffffffu, inrange) == 0) {
      e = -1;
      return c;
    }
    if (nm) {
      const int first = __ffs(nm) - 1;
      if (lane < first && inrange) out[cand] = 0.0;
      e = c + (int64_t)first * G;
      return c + (int64_t)(first + 1) * G;
    }
    if (inrange) out[cand] = 0.0;
    c += 32 * G;
  }
}

template <int K, class T>
__global__ void __launch_bounds__(MF_REC_NT, sizeof(T) == 4 ? 4 : 2)
    me_rec_warp_kernel(const int4* __restrict__ prep, int64_t N, const double* __restrict__ skip,
                       double* __restrict__ out, double* __restrict__ hel_out) {
  using R = RecTraits<K>;
  constexpr int WPB = MF_REC_NT / 32, NW = prep_words<T, K>();
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  RecSmem<T, K>& S = reinterpret_cast<RecSmem<T, K>*>(smem_raw)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int64_t G = (int64_t)gridDim.x * WPB;
  int64_t e;
  int64_t c = next_warp_event((int64_t)blockIdx.x * WPB + (threadIdx.x >> 5), G, N, skip, out, lane, e);
  if (e >= 0) rec_load<T, K, 32>(S.ws, S.pr, prep + e * NW, lane);
  while (e >= 0) {
    __syncwarp();
    rec_stages_c<T, K, 1, 32>(S.ws, S.pr.ev, lane);
    rec_st_A<T, K>(S.ws, lane, 32);
    __syncwarp();
    int64_t en;
    c = next_warp_event(c, G, N, skip, out, lane, en);
    RecFetch<T, K, 32> nf;
    if (en >= 0) rec_fetch<T, K, 32>(nf, prep + en * NW, lane);
    T part = rec_st_colour<T, K>(S.ws, lane, 32);
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    const double sc = S.pr.scale;
    if (hel_out)
      for (int cc = lane; cc < (1 << (K + 2)); cc += 32)
        hel_out[(int64_t)R::cfg_to_mg(cc) * N + e] = rec_colour_one<T, K>(S.ws, cc) * sc * R::DENOMINATOR;
    if (lane == 0) out[e] = (double)part * sc;
    __syncwarp();
    if (en >= 0) rec_store<T, K, 32>(S.ws, S.pr, nf, lane);
    e = en;
  }
}
#endif
