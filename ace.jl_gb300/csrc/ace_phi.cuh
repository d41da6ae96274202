// ace_phi.cuh -- per-neighbour one-particle basis on the GPU: the transformed,
// enveloped radial polynomials R_n and the complex spherical harmonics
// Y_l^m, with their Cartesian gradients.
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

namespace ace {

template <typename T> struct cpx { T re, im; };

template <typename T> __device__ __forceinline__ cpx<T> cmul(cpx<T> a, cpx<T> b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename T> __device__ __forceinline__ cpx<T> cadd(cpx<T> a, cpx<T> b) {
  return {a.re + b.re, a.im + b.im};
}
template <typename T> __device__ __forceinline__ cpx<T> cscale(cpx<T> a, T s) {
  return {a.re * s, a.im * s};
}

__host__ __device__ constexpr int size_p(int L) { return (L + 1) * (L + 2) / 2; }
__host__ __device__ constexpr int size_y(int L) { return (L + 1) * (L + 1); }
__host__ __device__ constexpr int idx_p(int l, int m) { return m + (l * (l + 1)) / 2; }
__host__ __device__ constexpr int idx_y(int l, int m) { return m + l + l * l; }

// Coefficient tables, resident in shared memory during a kernel.
template <typename T> struct Tables {
  const T *rA, *rB, *rC;    // radial recursion, nR each
  const T *alpA, *alpB;     // ALP recursion, size_p(L) each
  int nR, L, pl, pr, tp;
  T tl, tr, r0;
};

template <typename T> __device__ __forceinline__ T ipow(T x, int p) {
  T y = T(1);
  for (int i = 0; i < p; ++i) y = (i == 0) ? x : y * x;
  return y;
}

// Per-neighbour slab layout (in units of T):
//   R[nR] dR[nR] P[szP] dP[szP] Y[2 nY] dY[6 nY]   (dY: [iy][axis] complex)
template <typename T> struct Slab {
  __host__ __device__ static int size(int nR, int L) {
    return 2 * nR + 2 * size_p(L) + 8 * size_y(L);
  }
};

// Radial values R_n(r) (and dR_n/dr when GRAD).
template <typename T, bool GRAD>
__device__ __forceinline__ void radial_eval(const Tables<T> &tb, T r, T *R, T *dR) {
  const T a = T(1) + tb.r0;
  const T u = T(1) + r;
  const T x = a / u;
  const T t = ipow(x, tb.tp);
  const bool outside = (tb.pl > 0 && t < tb.tl) || (tb.pr > 0 && t > tb.tr);
  T f = outside ? T(0) : ipow(t - tb.tl, tb.pl) * ipow(t - tb.tr, tb.pr);
  R[0] = tb.rA[0] * f;
  T dtdr = T(0), dP0 = T(0), dP1 = T(0), dP2 = T(0);
  if (GRAD) {
    dtdr = T(tb.tp) * ipow(x, tb.tp - 1) * (-(a / (u * u)));
    T fd = T(0);
    if (!outside) {
      if (tb.pl > 0) fd += T(tb.pl) * ipow(t - tb.tl, tb.pl - 1) * ipow(t - tb.tr, tb.pr);
      if (tb.pr > 0) fd += ipow(t - tb.tl, tb.pl) * (T(tb.pr) * ipow(t - tb.tr, tb.pr - 1));
    }
    dP0 = tb.rA[0] * fd;
    dR[0] = dP0 * dtdr;
  }
  if (tb.nR == 1) return;
  T al = tb.rA[1] * t + tb.rB[1];
  R[1] = al * R[0];
  if (GRAD) { dP1 = al * dP0 + tb.rA[1] * R[0]; dR[1] = dP1 * dtdr; }
  for (int n = 2; n < tb.nR; ++n) {
    al = tb.rA[n] * t + tb.rB[n];
    R[n] = al * R[n - 1] + tb.rC[n] * R[n - 2];
    if (GRAD) {
      dP2 = al * dP1 + tb.rC[n] * dP0 + tb.rA[n] * R[n - 1];
      dR[n] = dP2 * dtdr;
      dP0 = dP1; dP1 = dP2;
    }
  }
}

struct SphCoords { };

// Complex Y_l^m (index_y order) at direction (x, y, z), and when GRAD the
// Cartesian gradients dY[3*iy + a].  P and dP are scratch of size_p(L).
template <typename T, bool GRAD>
__device__ __forceinline__ void sh_eval(const Tables<T> &tb, T x, T y, T z, T *P, T *dP,
                                        cpx<T> *Y, cpx<T> *dY) {
  const int L = tb.L;
  const T rho2 = x * x + y * y;
  const T r = sqrt(rho2 + z * z);
  const T rho = sqrt(rho2);
  const T cost = z / r;
  const T sint = rho / r;
  T cosp = T(1), sinp = T(0);
  if (rho > T(0)) { cosp = x / rho; sinp = y / rho; }
  const T *A = tb.alpA, *B = tb.alpB;
  const T invsqrt2 = T(0.70710678118654752440084436210484903928);
  T temp = T(0.39894228040143267793994605993438186848);  // sqrt(0.5/pi)
  if (!GRAD) {
    // ALP evaluate! (sphericalharmonics.jl:167-197)
    P[idx_p(0, 0)] = temp;
    if (L > 0) {
      P[idx_p(1, 0)] = cost * T(1.7320508075688772935274463415058723670) * temp;
      temp = -T(1.2247448713915890490986420373529456960) * sint * temp;
      P[idx_p(1, 1)] = temp;
      for (int l = 2; l <= L; ++l) {
        const int il = (l * (l + 1)) / 2, ilm1 = il - l, ilm2 = ilm1 - l + 1;
        for (int m = 0; m <= l - 2; ++m)
          P[il + m] = A[il + m] * (cost * P[ilm1 + m] + B[il + m] * P[ilm2 + m]);
        P[il + l - 1] = cost * sqrt(T(2 * (l - 1) + 3)) * temp;
        temp = -sqrt(T(1) + T(0.5) / T(l)) * sint * temp;
        P[il + l] = temp;
      }
    }
    // cYlm! (sphericalharmonics.jl:379-403)
    for (int l = 0; l <= L; ++l) Y[idx_y(l, 0)] = {P[idx_p(l, 0)] * invsqrt2, T(0)};
    cpx<T> ep = {invsqrt2, T(0)};
    const cpx<T> ef = {cosp, sinp};
    T sig = T(1);
    for (int m = 1; m <= L; ++m) {
      sig = -sig;
      ep = cmul(ep, ef);
      const cpx<T> em = {sig * ep.re, -(sig * ep.im)};
      for (int l = m; l <= L; ++l) {
        const T p = P[idx_p(l, m)];
        Y[idx_y(l, -m)] = cscale(em, p);
        Y[idx_y(l, m)] = cscale(ep, p);
      }
    }
    return;
  }
  // _evaluate_ed! (sphericalharmonics.jl:212-267)
  const T sq3 = T(1.7320508075688772935274463415058723670);
  const T sq15 = T(1.2247448713915890490986420373529456960);
  P[idx_p(0, 0)] = temp;
  T temp_d = T(0);
  dP[idx_p(0, 0)] = temp_d;
  if (L > 0) {
    P[idx_p(1, 0)] = cost * sq3 * temp;
    dP[idx_p(1, 0)] = -sint * sq3 * temp + cost * sq3 * temp_d;
    T temp1 = -sq15 * temp;
    temp_d = -sq15 * (cost * temp + sint * temp_d);
    P[idx_p(1, 1)] = temp1;
    dP[idx_p(1, 1)] = temp_d;
    const T s2 = sint * sint;
    for (int l = 2; l <= L; ++l) {
      P[idx_p(l, 0)] = A[idx_p(l, 0)] * (cost * P[idx_p(l - 1, 0)] + B[idx_p(l, 0)] * P[idx_p(l - 2, 0)]);
      dP[idx_p(l, 0)] = A[idx_p(l, 0)] * (-sint * P[idx_p(l - 1, 0)] + cost * dP[idx_p(l - 1, 0)] +
                                          B[idx_p(l, 0)] * dP[idx_p(l - 2, 0)]);
      for (int m = 1; m <= l - 2; ++m) {
        P[idx_p(l, m)] = A[idx_p(l, m)] * (cost * P[idx_p(l - 1, m)] + B[idx_p(l, m)] * P[idx_p(l - 2, m)]);
        dP[idx_p(l, m)] = A[idx_p(l, m)] * (-s2 * P[idx_p(l - 1, m)] + cost * dP[idx_p(l - 1, m)] +
                                            B[idx_p(l, m)] * dP[idx_p(l - 2, m)]);
      }
      const T q = sqrt(T(2 * (l - 1) + 3));
      P[idx_p(l, l - 1)] = q * cost * temp1;
      dP[idx_p(l, l - 1)] = q * (-s2 * temp1 + cost * temp_d);
      const T f = -sqrt(T(1) + T(0.5) / T(l));
      const T nt1 = f * sint * temp1;
      const T ntd = f * (cost * temp1 * sint + sint * temp_d);
      temp1 = nt1;
      temp_d = ntd;
      P[idx_p(l, l)] = temp1;
      dP[idx_p(l, l)] = temp_d;
    }
  }
  // cYlm_ed! (sphericalharmonics.jl:410-443) with dspher_to_dcart (:60-65)
  const T rinv = T(1) / (r + T(2.220446049250313e-16));
  const T cc = cosp * cost, sc = sinp * cost;
  for (int l = 0; l <= L; ++l) {
    Y[idx_y(l, 0)] = {P[idx_p(l, 0)] * invsqrt2, T(0)};
    const T ft = dP[idx_p(l, 0)] * invsqrt2;
    cpx<T> *d = dY + 3 * idx_y(l, 0);
    d[0] = {(cc * ft) * rinv, T(0)};
    d[1] = {(sc * ft) * rinv, T(0)};
    d[2] = {(-(sint * ft)) * rinv, T(0)};
  }
  cpx<T> ep = {invsqrt2 * cosp, invsqrt2 * sinp};
  const cpx<T> ef = {cosp, sinp};
  T sig = T(1);
  for (int m = 1; m <= L; ++m) {
    sig = -sig;
    if (m > 1) ep = cmul(ep, ef);
    const cpx<T> em = {sig * ep.re, -(sig * ep.im)};
    const T fm = T(m);
    const cpx<T> dep = {-fm * ep.im, fm * ep.re};
    const cpx<T> dem = {fm * em.im, -fm * em.re};
    for (int l = m; l <= L; ++l) {
      const T p = P[idx_p(l, m)];
      const T dp = dP[idx_p(l, m)];
      Y[idx_y(l, -m)] = cscale(cscale(em, p), sint);
      Y[idx_y(l, m)] = cscale(cscale(ep, p), sint);
#pragma unroll
      for (int s = 0; s < 2; ++s) {
        const cpx<T> fps = cscale(s == 0 ? dem : dep, p);
        const cpx<T> ft = cscale(s == 0 ? em : ep, dp);
        cpx<T> *d = dY + 3 * idx_y(l, s == 0 ? -m : m);
        d[0] = {(-(sinp * fps.re) + cc * ft.re) * rinv, (-(sinp * fps.im) + cc * ft.im) * rinv};
        d[1] = {((cosp * fps.re) + sc * ft.re) * rinv, ((cosp * fps.im) + sc * ft.im) * rinv};
        d[2] = {(-(sint * ft.re)) * rinv, (-(sint * ft.im)) * rinv};
      }
    }
  }
}

}  // namespace ace
