// External wavefunctions (madflow wavefunctions_flow.py), device side.
// Each routine returns slots 2-5 of the HELAS wavefunction; slots 0-1 (the
// momentum flow) are p*nsv (vector, outgoing fermion) or -p*nsf (incoming
// fermion) and are produced by the batched API wrappers only.
#pragma once
#include "mf_common.cuh"

template <class T> MF_D T tf_sign(T y) { return y > T(0) ? T(1) : (y < T(0) ? T(-1) : T(0)); }
// floor(a / 2) of the small integers the helicity projectors take, in T
template <class T> MF_D int floordiv2(T a) { return (int)floor(a * T(0.5)); }

// pp + p3 of a massive fermion (pp = |p|).  For a fermion moving along -z
// the sum cancels; in FP32 it is then formed as (p1^2 + p2^2) / (pp - p3),
// which is exact algebra without the cancellation (a top quark running along
// a beam lost up to 4e-2 of |M|^2 to the rounded difference).  FP64 keeps
// the reference's sum (wavefunctions_flow.py:214, :418).
template <class T> MF_D T pp_plus_p3(const T* p, T pp) {
  if constexpr (sizeof(T) == 4)
    if (p[3] < T(0)) return (p[1] * p[1] + p[2] * p[2]) / (pp - p[3]);
  return fmax(pp + p[3], T(0));
}

// _ox_massive_pp_zero (wavefunctions_flow.py:370-392)
template <class T> MF_D void ox_massive_pp_zero(T fmass, T nsf, int ip, int im, W4<T>& f) {
  T s0 = sqrt(fabs(fmass));
  T sqm[2] = {s0, s0 * tf_sign(fmass)};
  int aim = im < 0 ? -im : im, aip = ip < 0 ? -ip : ip;
  f.v[0] = {T(im) * sqm[aim], T(0)};
  f.v[1] = {T(ip) * nsf * sqm[aim], T(0)};
  f.v[2] = {T(im) * nsf * sqm[aip], T(0)};
  f.v[3] = {T(ip) * sqm[aip], T(0)};
}

// ixxxxx (wavefunctions_flow.py:56-85 and 159-330)
template <class T> MF_D W4<T> ixxxxx(const T* p, T fmass, T nhel, T nsf) {
  W4<T> f;
  T nh = nhel * nsf;
  if (fmass != T(0)) {
    T pp = fmin(p[0], sqrt(p[1] * p[1] + p[2] * p[2] + p[3] * p[3]));
    int ip = floordiv2<T>(T(1) + nh), im = floordiv2<T>(T(1) - nh);
    if (pp == T(0)) {
      ox_massive_pp_zero<T>(fmass, nsf, im, ip, f);
      return f;
    }
    T sf0 = (T(1) + nsf + (T(1) - nsf) * nh) * T(0.5);
    T sf1 = (T(1) + nsf - (T(1) - nsf) * nh) * T(0.5);
    T sq = sqrt(p[0] + pp);
    T om[2] = {sq, fmass / sq};
    T sfo0 = sf0 * om[ip], sfo1 = sf1 * om[im];
    T pp3 = pp_plus_p3<T>(p, pp);
    cx<T> chi1;
    if (pp3 == T(0)) chi1 = {-nh, T(0)};
    else {
      T r = sqrt(T(2) * pp * pp3);
      chi1 = {nh * p[1] / r, p[2] / r};
    }
    cx<T> chi[2] = {{sqrt(pp3 * T(0.5) / pp), T(0)}, chi1};
    f.v[0] = sfo0 * chi[im];
    f.v[1] = sfo0 * chi[ip];
    f.v[2] = sfo1 * chi[im];
    f.v[3] = sfo1 * chi[ip];
    return f;
  }
  T sq = sqrt(fmax(p[0] + p[3], T(0))) * nsf;
  cx<T> chi1 = (sq == T(0)) ? cx<T>{-nhel * sqrt(T(2) * p[0]), T(0)} : cx<T>{nh * p[1] / sq, p[2] / sq};
  cx<T> chi0 = {sq, T(0)};
  cx<T> z = {T(0), T(0)};
  if (nh == T(1)) { f.v[0] = z; f.v[1] = z; f.v[2] = chi0; f.v[3] = chi1; }
  else { f.v[0] = chi1; f.v[1] = chi0; f.v[2] = z; f.v[3] = z; }
  return f;
}

// oxxxxx (wavefunctions_flow.py:89-116 and 336-462)
template <class T> MF_D W4<T> oxxxxx(const T* p, T fmass, T nhel, T nsf) {
  W4<T> f;
  T nh = nhel * nsf;
  if (fmass != T(0)) {
    T pp = fmin(p[0], sqrt(p[1] * p[1] + p[2] * p[2] + p[3] * p[3]));
    if (pp == T(0)) {
      int ipz = -floordiv2<T>(T(1) - nh) * (int)nhel;
      int imz = floordiv2<T>(T(1) + nh) * (int)nhel;
      ox_massive_pp_zero<T>(fmass, nsf, ipz, imz, f);
      return f;
    }
    T sf0 = (T(1) + nsf + (T(1) - nsf) * nh) * T(0.5);
    T sf1 = (T(1) + nsf - (T(1) - nsf) * nh) * T(0.5);
    T sq = sqrt(p[0] + pp);
    T om[2] = {sq, fmass / sq};
    int ip = floordiv2<T>(T(1) + nh), im = floordiv2<T>(T(1) - nh);
    T sfo0 = sf0 * om[ip], sfo1 = sf1 * om[im];
    T pp3 = pp_plus_p3<T>(p, pp);
    cx<T> chi1;
    if (pp3 == T(0)) chi1 = {-nh, T(0)};
    else {
      T r = sqrt(T(2) * pp * pp3);
      chi1 = {nh * p[1] / r, -p[2] / r};
    }
    cx<T> chi[2] = {{sqrt(pp3 * T(0.5) / pp), T(0)}, chi1};
    f.v[0] = sfo1 * chi[im];
    f.v[1] = sfo1 * chi[ip];
    f.v[2] = sfo0 * chi[im];
    f.v[3] = sfo0 * chi[ip];
    return f;
  }
  T sq = sqrt(fmax(p[0] + p[3], T(0))) * nsf;
  cx<T> chi0 = (sq == T(0)) ? cx<T>{-nhel * sqrt(T(2) * p[0]), T(0)} : cx<T>{nh * p[1] / sq, -p[2] / sq};
  cx<T> csq = {sq, T(0)};
  cx<T> z = {T(0), T(0)};
  if (nh == T(1)) { f.v[0] = csq; f.v[1] = chi0; f.v[2] = z; f.v[3] = z; }
  else { f.v[0] = z; f.v[1] = z; f.v[2] = chi0; f.v[3] = csq; }
  return f;
}

// vxxxxx (wavefunctions_flow.py:120-154 and 469-747); nhel = 4 is the BRST
// check (polarisation replaced by the momentum).
template <class T> MF_D W4<T> vxxxxx(const T* p, T vmass, T nhel, T nsv, T sqh) {
  W4<T> f;
  T pt2 = p[1] * p[1] + p[2] * p[2];
  T pp = fmin(p[0], sqrt(pt2 + p[3] * p[3]));
  T pt = fmin(pp, sqrt(pt2));
  T hel0 = T(1) - fabs(nhel);
  T nsvahl = nsv * fabs(nhel);
  if (nhel == T(4)) {
    T d = (vmass == T(0)) ? p[0] : vmass;
#pragma unroll
    for (int k = 0; k < 4; ++k) f.v[k] = {p[k] / d, T(0)};
    return f;
  }
  if (vmass != T(0)) {
    if (pp == T(0)) {
      f.v[0] = {T(1), T(0)};
      f.v[1] = {-nhel * sqh, T(0)};
      f.v[2] = {T(0), nsvahl * sqh};
      f.v[3] = {hel0, T(0)};
      return f;
    }
    T emp = p[0] / (vmass * pp);
    f.v[0] = {hel0 * pp / vmass, T(0)};
    f.v[3] = {hel0 * p[3] * emp + nhel * pt / pp * sqh, T(0)};
    if (pt != T(0)) {
      T pzpt = p[3] / (pp * pt) * sqh * nhel;
      f.v[1] = {hel0 * p[1] * emp - p[1] * pzpt, -nsvahl * p[2] / pt * sqh};
      f.v[2] = {hel0 * p[2] * emp - p[2] * pzpt, nsvahl * p[1] / pt * sqh};
    } else {
      f.v[1] = {-nhel * sqh, T(0)};
      f.v[2] = {T(0), nsvahl * (sqh * tf_sign(p[3]))};
    }
    return f;
  }
  T ppl = p[0];
  T ptl = sqrt(pt2);
  f.v[0] = {T(0), T(0)};
  f.v[3] = {nhel * ptl / ppl * sqh, T(0)};
  if (ptl != T(0)) {
    T pzpt = p[3] / (ppl * ptl) * sqh * nhel;
    f.v[1] = {-p[1] * pzpt, -nsv * p[2] / ptl * sqh};
    f.v[2] = {-p[2] * pzpt, nsv * p[1] / ptl * sqh};
  } else {
    f.v[1] = {-nhel * sqh, T(0)};
    f.v[2] = {T(0), nsv * (sqh * tf_sign(p[3]))};
  }
  return f;
}
