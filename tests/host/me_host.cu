// Host-side harness for the helicity-recycling matrix-element stages: the
// product's stage functions (mf_me_rec.cuh) are run one "thread" at a time
// on the CPU, stage by stage, so the CPU test suite can compare the generated
// evaluation with the oracle without a GPU.
#include <cstdint>
#include <cstring>
#include <memory>

#include "../../madflow_gb300/csrc/mf_me_rec.cuh"
#include "../../madflow_gb300/csrc/generated/ttng2.cuh"
#include "../../madflow_gb300/csrc/generated/ttng3.cuh"
#include "../../madflow_gb300/csrc/generated/ttng4.cuh"
#include "../../madflow_gb300/csrc/generated/ttng5.cuh"

MF_DEFINE_REC(2)
MF_DEFINE_REC(3)
MF_DEFINE_REC(4)
MF_DEFINE_REC(5)

// |M|^2 of one event; hel_out (optional) [ncomb] in MadGraph helicity order.
template <int K, class T>
static double smatrix_one(const double* p, const double* coup, double mt, double wt, double* hel_out,
                          bool compiled = false) {
  using R = RecTraits<K>;
  auto ws = std::make_unique<RecWS<T, K>>();
  auto pr = std::make_unique<PrepRec<T, K>>();
  double pd[K + 2][4];
  std::memcpy(pd, p, sizeof(pd));
  cx<double> c10 = {coup[0], coup[1]}, c11 = {coup[2], coup[3]}, c12 = {coup[4], coup[5]};
  prep_event<T, K>(*pr, pd, mt, wt, c10, c11, c12);
  const int nt = 7;  // an odd "block size" exercises the item striding
  double tot = compiled ? RecHostRun<T, K>::template run_c<7>(*ws, *pr) : RecHostRun<T, K>::run(*ws, *pr, nt);
  double sc = pr->scale;
  if (hel_out)
    for (int c = 0; c < (1 << (K + 2)); ++c)
      hel_out[R::cfg_to_mg(c)] = rec_colour_one<T, K>(*ws, c) * sc * R::DENOMINATOR;
  return tot * sc;
}

extern "C" int me_host_smatrix(int k, int prec, const double* p, int64_t N, const double* coup, double mt, double wt,
                               double* out) {
  int np = k + 2;
  for (int64_t e = 0; e < N; ++e) {
    const double* pe = p + 4 * np * e;
    if (k == 2) out[e] = prec ? smatrix_one<2, float>(pe, coup, mt, wt, nullptr) : smatrix_one<2, double>(pe, coup, mt, wt, nullptr);
    else if (k == 3) out[e] = prec ? smatrix_one<3, float>(pe, coup, mt, wt, nullptr) : smatrix_one<3, double>(pe, coup, mt, wt, nullptr);
    else if (k == 4) out[e] = prec ? smatrix_one<4, float>(pe, coup, mt, wt, nullptr) : smatrix_one<4, double>(pe, coup, mt, wt, nullptr);
    else if (k == 5) out[e] = prec ? smatrix_one<5, float>(pe, coup, mt, wt, nullptr) : smatrix_one<5, double>(pe, coup, mt, wt, nullptr);
    else return 1;
  }
  return 0;
}

// The same through the kernels' compile-time stage driver (paired items in
// every stage with more than 7 items).
extern "C" int me_host_smatrix_compiled(int k, int prec, const double* p, int64_t N, const double* coup, double mt,
                                        double wt, double* out) {
  int np = k + 2;
  for (int64_t e = 0; e < N; ++e) {
    const double* pe = p + 4 * np * e;
    if (k == 2) out[e] = prec ? smatrix_one<2, float>(pe, coup, mt, wt, nullptr, true) : smatrix_one<2, double>(pe, coup, mt, wt, nullptr, true);
    else if (k == 3) out[e] = prec ? smatrix_one<3, float>(pe, coup, mt, wt, nullptr, true) : smatrix_one<3, double>(pe, coup, mt, wt, nullptr, true);
    else if (k == 4) out[e] = prec ? smatrix_one<4, float>(pe, coup, mt, wt, nullptr, true) : smatrix_one<4, double>(pe, coup, mt, wt, nullptr, true);
    else if (k == 5) out[e] = prec ? smatrix_one<5, float>(pe, coup, mt, wt, nullptr, true) : smatrix_one<5, double>(pe, coup, mt, wt, nullptr, true);
    else return 1;
  }
  return 0;
}

// ---- operation count of the recycled evaluation ------------------------------
// A scalar that counts every +, -, *, / and sqrt (complex mul = 6, add = 2,
// the convention the oracle's count uses).
struct CountF {
  double v;
  static inline unsigned long long n = 0;
  CountF() : v(0) {}
  template <class A> CountF(A x) : v((double)x) {}
  explicit operator double() const { return v; }
  explicit operator int() const { return (int)v; }
};
inline CountF operator+(CountF a, CountF b) { ++CountF::n; return CountF(a.v + b.v); }
inline CountF operator-(CountF a, CountF b) { ++CountF::n; return CountF(a.v - b.v); }
inline CountF operator*(CountF a, CountF b) { ++CountF::n; return CountF(a.v * b.v); }
inline CountF operator/(CountF a, CountF b) { ++CountF::n; return CountF(a.v / b.v); }
inline CountF operator-(CountF a) { return CountF(-a.v); }
inline CountF& operator+=(CountF& a, CountF b) { a = a + b; return a; }
inline bool operator==(CountF a, CountF b) { return a.v == b.v; }
inline bool operator!=(CountF a, CountF b) { return a.v != b.v; }
inline bool operator<(CountF a, CountF b) { return a.v < b.v; }
inline bool operator>(CountF a, CountF b) { return a.v > b.v; }
inline CountF sqrt(CountF a) { ++CountF::n; return CountF(std::sqrt(a.v)); }
inline CountF fabs(CountF a) { return CountF(std::fabs(a.v)); }
inline CountF fmin(CountF a, CountF b) { return a.v < b.v ? a : b; }
inline CountF fmax(CountF a, CountF b) { return a.v < b.v ? b : a; }
inline CountF floor(CountF a) { return CountF(std::floor(a.v)); }

// Flops of one event of the recycled evaluation (all helicity combinations)
// as the matrix-element kernel runs it: the stages, amplitudes and colour sum
// from a ready record (the record itself is built by the phase-space kernel).
template <int K> static double stage_flops(const double* p, const double* coup, double mt, double wt) {
  auto ws = std::make_unique<RecWS<CountF, K>>();
  auto pr = std::make_unique<PrepRec<CountF, K>>();
  double pd[K + 2][4];
  std::memcpy(pd, p, sizeof(pd));
  prep_event<CountF, K>(*pr, pd, mt, wt, {coup[0], coup[1]}, {coup[2], coup[3]}, {coup[4], coup[5]});
  CountF::n = 0;
  double tot = RecHostRun<CountF, K>::run(*ws, *pr, 7);
  (void)tot;
  return (double)CountF::n;
}
extern "C" double me_host_flops(int k, const double* p, const double* coup, double mt, double wt) {
  if (k == 2) return stage_flops<2>(p, coup, mt, wt);
  if (k == 3) return stage_flops<3>(p, coup, mt, wt);
  if (k == 4) return stage_flops<4>(p, coup, mt, wt);
  if (k == 5) return stage_flops<5>(p, coup, mt, wt);
  return 0.0;
}

extern "C" int me_host_helicities(int k, const double* p, const double* coup, double mt, double wt, double* hel_out) {
  if (k == 2) smatrix_one<2, double>(p, coup, mt, wt, hel_out);
  else if (k == 3) smatrix_one<3, double>(p, coup, mt, wt, hel_out);
  else if (k == 4) smatrix_one<4, double>(p, coup, mt, wt, hel_out);
  else if (k == 5) smatrix_one<5, double>(p, coup, mt, wt, hel_out);
  else return 1;
  return 0;
}
