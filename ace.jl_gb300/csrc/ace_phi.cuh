// ace_phi.cuh -- per-neighbour one-particle basis on the GPU: the transformed,
// enveloped radial polynomials R_n and the complex spherical harmonics
// Y_l^m, with their Cartesian gradients, in any of the arithmetic types of
// ace_arith.cuh (float, double, double-float).
//
// Same recursions and operation order as ACE.jl:
//   radial   src/polynomials/orthpolys.jl:32-60,253-306 (evaluate!, evaluate_ed!)
//   SH       src/polynomials/sphericalharmonics.jl:167-197 (ALP evaluate!),
//            :212-267 (_evaluate_ed!, P/sin(theta) storage for m>0),
//            :379-403 (cYlm!), :410-443 (cYlm_ed!), :60-65 (dspher_to_dcart)
// cos(phi), sin(phi) are formed as x/rho, y/rho instead of through atan and
// sincos (identical values up to rounding, no transcendental calls).
#pragma once
#include <cstdint>

#include "ace_arith.cuh"

// double-float complex products through dot2 (one renormalisation per
// component) instead of four products and two sums
#ifndef ACE_DF_DOT2
#define ACE_DF_DOT2 1
#endif

namespace ace {

template <typename T> struct cpx { T re, im; };

template <typename T> __device__ __forceinline__ cpx<T> cmul(cpx<T> a, cpx<T> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
#if ACE_DF_DOT2
template <> __device__ __forceinline__ cpx<df> cmul<df>(cpx<df> a, cpx<df> b) {
  return {dot2(a.re, b.re, -a.im, b.im), dot2(a.re, b.im, a.im, b.re)};
}
#endif
template <typename T> __device__ __forceinline__ cpx<T> cadd(cpx<T> a, cpx<T> b) {
  return {a.re + b.re, a.im + b.im};
}
template <typename T> __device__ __forceinline__ cpx<T> cscale(cpx<T> a, T s) {
  return {a.re * s, a.im * s};
}
// a b + c d and a b + c, fused in double-float
template <typename T> __device__ __forceinline__ T dot2g(T a, T b, T c, T d) { return a * b + c * d; }
template <typename T> __device__ __forceinline__ T fmag(T a, T b, T c) { return a * b + c; }
#if ACE_DF_DOT2
template <> __device__ __forceinline__ df dot2g<df>(df a, df b, df c, df d) { return dot2(a, b, c, d); }
template <> __device__ __forceinline__ df fmag<df>(df a, df b, df c) { return fma_df(a, b, c); }
#endif
// acc + a s (real s)
template <typename T> __device__ __forceinline__ cpx<T> cfma(cpx<T> acc, cpx<T> a, T s) {
  return cadd(acc, cscale(a, s));
}
#if ACE_DF_DOT2
template <> __device__ __forceinline__ cpx<df> cfma<df>(cpx<df> acc, cpx<df> a, df s) {
  return {fma_df(a.re, s, acc.re), fma_df(a.im, s, acc.im)};
}
#endif

__host__ __device__ constexpr int size_p(int L) { return (L + 1) * (L + 2) / 2; }
__host__ __device__ constexpr int size_y(int L) { return (L + 1) * (L + 1); }
__host__ __device__ constexpr int idx_p(int l, int m) { return m + (l * (l + 1)) / 2; }
__host__ __device__ constexpr int idx_y(int l, int m) { return m + l + l * l; }

// Coefficient table layout (host builds it in double; the kernel holds a copy
// in shared memory in its own arithmetic type):
//   rA rB rC [nR] | alpA alpB [size_p(L)] | alpC alpD [L+1] | tl tr a0 sq3 sq15 sqhalfpi invsqrt2
__host__ __device__ inline int table_size(int nR, int L) { return 3 * nR + 2 * size_p(L) + 2 * (L + 1) + 7; }

template <typename T> struct Tables {
  const T *rA, *rB, *rC, *alpA, *alpB, *alpC, *alpD;
  T tl, tr, a0, sq3, sq15, sqhalfpi, invsqrt2;
  int nR, L, pl, pr, tp;
  __device__ __forceinline__ void bind(const T *tab, int nR_, int L_, int pl_, int pr_, int tp_) {
    nR = nR_; L = L_; pl = pl_; pr = pr_; tp = tp_;
    const int szP = size_p(L);
    rA = tab; rB = tab + nR; rC = tab + 2 * nR;
    alpA = tab + 3 * nR; alpB = alpA + szP;
    alpC = alpB + szP; alpD = alpC + (L + 1);
    const T *k = alpD + (L + 1);
    tl = k[0]; tr = k[1]; a0 = k[2]; sq3 = k[3]; sq15 = k[4]; sqhalfpi = k[5]; invsqrt2 = k[6];
  }
};

template <typename T> __device__ __forceinline__ T ipow(T x, int p) {
  T y = Arith<T>::one();
  for (int i = 0; i < p; ++i) y = (i == 0) ? x : y * x;
  return y;
}

// Radial values R_n(r) (and dR_n/dr when GRAD).
template <typename T, bool GRAD>
__device__ __forceinline__ void radial_eval(const Tables<T> &tb, T r, T *R, T *dR) {
  const T one = Arith<T>::one();
  const T u = one + r;
  const T x = tb.a0 / u;
  const T t = ipow(x, tb.tp);
  const bool outside = (tb.pl > 0 && t < tb.tl) || (tb.pr > 0 && t > tb.tr);
  const T f = outside ? Arith<T>::zero() : ipow(t - tb.tl, tb.pl) * ipow(t - tb.tr, tb.pr);
  R[0] = tb.rA[0] * f;
  T dtdr = Arith<T>::zero(), dP0 = Arith<T>::zero(), dP1 = Arith<T>::zero();
  if (GRAD) {
    dtdr = Arith<T>::from((double)tb.tp) * ipow(x, tb.tp - 1) * (-(tb.a0 / (u * u)));
    T fd = Arith<T>::zero();
    if (!outside) {
      if (tb.pl > 0) fd = fd + Arith<T>::from((double)tb.pl) * ipow(t - tb.tl, tb.pl - 1) * ipow(t - tb.tr, tb.pr);
      if (tb.pr > 0) fd = fd + ipow(t - tb.tl, tb.pl) * (Arith<T>::from((double)tb.pr) * ipow(t - tb.tr, tb.pr - 1));
    }
    dP0 = tb.rA[0] * fd;
    dR[0] = dP0 * dtdr;
  }
  if (tb.nR == 1) return;
  T al = tb.rA[1] * t + tb.rB[1];
  R[1] = al * R[0];
  if (GRAD) { dP1 = al * dP0 + tb.rA[1] * R[0]; dR[1] = dP1 * dtdr; }
  for (int n = 2; n < tb.nR; ++n) {
    al = fmag(tb.rA[n], t, tb.rB[n]);
    R[n] = dot2g(al, R[n - 1], tb.rC[n], R[n - 2]);
    if (GRAD) {
      const T dP2 = al * dP1 + tb.rC[n] * dP0 + tb.rA[n] * R[n - 1];
      dR[n] = dP2 * dtdr;
      dP0 = dP1; dP1 = dP2;
    }
  }
}

// ---------------------------------------------------------------------------
// Column-parallel spherical harmonics: one thread per (neighbour, m), m = 0..L.
// The associated Legendre recursion of sphericalharmonics.jl:167-267 is a
// recurrence in l for each fixed m, seeded from the diagonal P(m, m)
// (itself a short recurrence in m), so each column m is computed in
// registers by its own thread: seed, P(m+1, m) = sqrt(2m+3) cos(theta) P(m, m),
// then the three-term recurrence.  Each thread writes Y(l, +-m) (and dY) for
// l = m..L.  The constants (alpA, alpB, alpC, alpD) are those of the
// reference's ALP recursion (sphericalharmonics.jl:146-165).

template <typename T> struct Angles { T cost, sint, cosp, sinp, r; };

template <typename T> __device__ __forceinline__ Angles<T> angles(T x, T y, T z) {
  Angles<T> g;
  const T rho2 = x * x + y * y;
  g.r = Arith<T>::sqrt_(rho2 + z * z);
  const T rho = Arith<T>::sqrt_(rho2);
  g.cost = z / g.r;
  g.sint = rho / g.r;
  g.cosp = Arith<T>::one();
  g.sinp = Arith<T>::zero();
  if (Arith<T>::positive(rho)) { g.cosp = x / rho; g.sinp = y / rho; }
  return g;
}

// cYlm! (values) for column m
template <typename T>
__device__ __forceinline__ void sh_col_values(const Tables<T> &tb, const Angles<T> &g, int m, cpx<T> *Y) {
  const int L = tb.L;
  const T zero = Arith<T>::zero();
  T pmm = tb.sqhalfpi;
  for (int mm = 1; mm <= m; ++mm) pmm = tb.alpD[mm] * g.sint * pmm;
  cpx<T> ep = {tb.invsqrt2, zero};
  const cpx<T> ef = {g.cosp, g.sinp};
  for (int mm = 1; mm <= m; ++mm) ep = cmul(ep, ef);
  const cpx<T> em = (m & 1) ? cpx<T>{-ep.re, ep.im} : cpx<T>{ep.re, -ep.im};
  T p2 = zero, p1 = pmm;
  for (int l = m; l <= L; ++l) {
    T p;
    if (l == m) p = pmm;
    else if (l == m + 1) p = g.cost * tb.alpC[l] * pmm;
    else p = tb.alpA[idx_p(l, m)] * dot2g(g.cost, p1, tb.alpB[idx_p(l, m)], p2);
    if (l > m) { p2 = p1; p1 = p; }
    if (m == 0) {
      Y[idx_y(l, 0)] = {p * tb.invsqrt2, zero};
    } else {
      Y[idx_y(l, -m)] = cscale(em, p);
      Y[idx_y(l, m)] = cscale(ep, p);
    }
  }
}

// cYlm_ed! (values and Cartesian gradients) for column m
template <typename T>
__device__ __forceinline__ void sh_col_grad(const Tables<T> &tb, const Angles<T> &g, int m, cpx<T> *Y, cpx<T> *dY) {
  const int L = tb.L;
  const T zero = Arith<T>::zero();
  const T s2 = g.sint * g.sint;
  const T rinv = Arith<T>::one() / (g.r + Arith<T>::from(2.220446049250313e-16));
  const T cc = g.cosp * g.cost, sc = g.sinp * g.cost;
  // seed: P(m, m) (stored divided by sin(theta) for m > 0) and its theta-derivative
  T t1 = tb.sqhalfpi, td = zero;
  if (m >= 1) {
    const T t0 = tb.sqhalfpi;
    t1 = tb.alpD[1] * t0;
    td = tb.alpD[1] * (g.cost * t0);
    for (int l = 2; l <= m; ++l) {
      const T f = tb.alpD[l];
      const T nt1 = f * g.sint * t1;
      const T ntd = f * (g.cost * t1 * g.sint + g.sint * td);
      t1 = nt1;
      td = ntd;
    }
  }
  cpx<T> ep = {tb.invsqrt2, zero};
  const cpx<T> ef = {g.cosp, g.sinp};
  for (int mm = 1; mm <= m; ++mm) ep = cmul(ep, ef);
  const cpx<T> em = (m & 1) ? cpx<T>{-ep.re, ep.im} : cpx<T>{ep.re, -ep.im};
  const T fm = Arith<T>::from((double)m);
  const cpx<T> dep = {-(fm * ep.im), fm * ep.re};
  const cpx<T> dem = {fm * em.im, -(fm * em.re)};
  T p2 = zero, p1 = t1, d2 = zero, d1 = td;
  for (int l = m; l <= L; ++l) {
    T p, dp;
    if (l == m) { p = t1; dp = td; }
    else if (m == 0) {
      if (l == 1) { p = g.cost * tb.sq3 * t1; dp = -g.sint * tb.sq3 * t1 + g.cost * tb.sq3 * td; }
      else {
        const T A = tb.alpA[idx_p(l, 0)], B = tb.alpB[idx_p(l, 0)];
        p = A * (g.cost * p1 + B * p2);
        dp = A * (-g.sint * p1 + g.cost * d1 + B * d2);
      }
    } else if (l == m + 1) {
      const T q = tb.alpC[l];
      p = q * g.cost * t1;
      dp = q * (-s2 * t1 + g.cost * td);
    } else {
      const T A = tb.alpA[idx_p(l, m)], B = tb.alpB[idx_p(l, m)];
      p = A * (g.cost * p1 + B * p2);
      dp = A * (-s2 * p1 + g.cost * d1 + B * d2);
    }
    if (l > m) { p2 = p1; p1 = p; d2 = d1; d1 = dp; }
    if (m == 0) {
      Y[idx_y(l, 0)] = {p * tb.invsqrt2, zero};
      const T ft = dp * tb.invsqrt2;
      cpx<T> *d = dY + 3 * idx_y(l, 0);
      d[0] = {(cc * ft) * rinv, zero};
      d[1] = {(sc * ft) * rinv, zero};
      d[2] = {(-(g.sint * ft)) * rinv, zero};
    } else {
      Y[idx_y(l, -m)] = cscale(cscale(em, p), g.sint);
      Y[idx_y(l, m)] = cscale(cscale(ep, p), g.sint);
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const cpx<T> fps = cscale(s == 0 ? dem : dep, p);
        const cpx<T> ft = cscale(s == 0 ? em : ep, dp);
        cpx<T> *d = dY + 3 * idx_y(l, s == 0 ? -m : m);
        d[0] = {(-(g.sinp * fps.re) + cc * ft.re) * rinv, (-(g.sinp * fps.im) + cc * ft.im) * rinv};
        d[1] = {((g.cosp * fps.re) + sc * ft.re) * rinv, ((g.cosp * fps.im) + sc * ft.im) * rinv};
        d[2] = {(-(g.sint * ft.re)) * rinv, (-(g.sint * ft.im)) * rinv};
      }
    }
  }
}

}  // namespace ace
