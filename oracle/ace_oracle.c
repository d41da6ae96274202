/*
 * ace_oracle.c -- FP64 CPU restatement of ACE.jl's evaluation hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the correctness oracle and the
 * timed CPU baseline; the product (libace_b200) never links or calls it.
 *
 * It restates, loop for loop and in the same floating-point operation order
 * (compile with -ffp-contract=off, as Julia does not contract), the
 * reference's evaluation of a linear ACE model and of its symmetric basis:
 *
 *   radial     OrthPolyBasis evaluate!/evaluate_ed!   src/polynomials/orthpolys.jl:32-60,253-306
 *   transform  polytransform + ForwardDiff chain      src/transforms/distancetransforms.jl:16,
 *                                                     src/chain.jl:40-52, src/transforms/lambdas.jl:34-42
 *   SH         cart2spher, ALP evaluate!/_evaluate_ed!, cYlm!, cYlm_ed!, dspher_to_dcart
 *                                                     src/polynomials/sphericalharmonics.jl:43-65,146-267,379-443
 *   A, dA      Product1pBasis add_into_A! / _add_into_A_dA!
 *                                                     src/product_1pbasis.jl:99-134,169-244
 *   energy     ProductEvaluator evaluate              src/evaluator.jl:121-147
 *   forces     _rrule_evaluate (grad_config)          src/evaluator.jl:161-200,
 *                                                     _AA_local_adjoints!  src/pibasis.jl:338-390
 *   basis      SymmetricBasis evaluate / evaluate_ed  src/symmbasis.jl:248-264,297-336,
 *                                                     PIBasis evaluate!/_evaluate_ed!  src/pibasis.jl:265-275,402-432
 *
 * Environments are independent; OpenMP runs one environment per thread.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "ace_oracle.h"

typedef struct { double re, im; } cplx;

static inline cplx cmul(cplx a, cplx b) {
  cplx r;
  r.re = a.re * b.re - a.im * b.im;
  r.im = a.re * b.im + a.im * b.re;
  return r;
}
static inline cplx cadd(cplx a, cplx b) { cplx r = {a.re + b.re, a.im + b.im}; return r; }
static inline cplx crmul(cplx a, double s) { cplx r = {a.re * s, a.im * s}; return r; }

static double ipow(double x, int p) {
  /* Float64^Int: integer power by repeated multiplication (p is 0..4) */
  double y = 1.0;
  for (int i = 0; i < p; ++i) y = (i == 0) ? x : y * x;
  return y;
}

/* ---------------------------------------------------------------- radial */

static inline double transform_t(const oracle_spec *s, double r) {
  /* "r -> ((1+r0)/(1+r))^p" */
  double x = (1.0 + s->r0) / (1.0 + r);
  return ipow(x, s->tp);
}

static inline double transform_dt(const oracle_spec *s, double r) {
  /* ForwardDiff.derivative of the same expression:
     d/dr [(a/(1+r))^p] = p x^(p-1) * (-(a)/(1+r)^2),  x = a/(1+r) */
  double a = 1.0 + s->r0;
  double u = 1.0 + r;
  double x = a / u;
  double dx = -(a / (u * u));
  return (double)s->tp * ipow(x, s->tp - 1) * dx;
}

static inline double fcut(const oracle_spec *s, double t) {
  if ((s->pl > 0 && t < s->tl) || (s->pr > 0 && t > s->tr)) return 0.0;
  return ipow(t - s->tl, s->pl) * ipow(t - s->tr, s->pr);
}

static inline double fcut_d(const oracle_spec *s, double t) {
  if ((s->pl > 0 && t < s->tl) || (s->pr > 0 && t > s->tr)) return 0.0;
  double d = 0.0;
  if (s->pl > 0) d += (double)s->pl * ipow(t - s->tl, s->pl - 1) * ipow(t - s->tr, s->pr);
  if (s->pr > 0) d += ipow(t - s->tl, s->pl) * ((double)s->pr * ipow(t - s->tr, s->pr - 1));
  return d;
}

/* evaluate! (orthpolys.jl:253-263) */
static void radial_eval(const oracle_spec *s, double t, double *P) {
  int N = s->nR;
  P[0] = s->rA[0] * fcut(s, t);
  if (N == 1) return;
  P[1] = (s->rA[1] * t + s->rB[1]) * P[0];
  for (int n = 2; n < N; ++n)
    P[n] = (s->rA[n] * t + s->rB[n]) * P[n - 1] + s->rC[n] * P[n - 2];
}

/* evaluate_ed! (orthpolys.jl:287-306) */
static void radial_eval_ed(const oracle_spec *s, double t, double *P, double *dP) {
  int N = s->nR;
  P[0] = s->rA[0] * fcut(s, t);
  dP[0] = s->rA[0] * fcut_d(s, t);
  if (N == 1) return;
  double a = s->rA[1] * t + s->rB[1];
  P[1] = a * P[0];
  dP[1] = a * dP[0] + s->rA[1] * P[0];
  for (int n = 2; n < N; ++n) {
    a = s->rA[n] * t + s->rB[n];
    P[n] = a * P[n - 1] + s->rC[n] * P[n - 2];
    dP[n] = a * dP[n - 1] + s->rC[n] * dP[n - 2] + s->rA[n] * P[n - 1];
  }
}

/* ------------------------------------------------------- spherical harmonics */

#define IDX_P(l, m) ((m) + ((l) * ((l) + 1)) / 2)
#define IDX_Y(l, m) ((m) + (l) + (l) * (l))

typedef struct { double r, cosp, sinp, cost, sint; } spher;

static spher cart2spher(const double *R) {
  spher S;
  S.r = sqrt(R[0] * R[0] + R[1] * R[1] + R[2] * R[2]);
  double phi = atan2(R[1], R[0]);
  S.sinp = sin(phi);
  S.cosp = cos(phi);
  S.cost = R[2] / S.r;
  S.sint = sqrt(R[0] * R[0] + R[1] * R[1]) / S.r;
  return S;
}

/* ALPolynomials coefficients (sphericalharmonics.jl:146-159) */
static void alp_coeffs(int L, double *A, double *B) {
  int sz = (L + 1) * (L + 2) / 2;
  for (int i = 0; i < sz; ++i) { A[i] = 0.0; B[i] = 0.0; }
  for (int l = 2; l <= L; ++l) {
    double ls = (double)(l * l), lm1s = (double)((l - 1) * (l - 1));
    for (int m = 0; m <= l - 2; ++m) {
      double ms = (double)(m * m);
      A[IDX_P(l, m)] = sqrt((4 * ls - 1.0) / (ls - ms));
      B[IDX_P(l, m)] = -sqrt((lm1s - ms) / (4 * lm1s - 1.0));
    }
  }
}

/* evaluate! (sphericalharmonics.jl:167-197) */
static void alp_eval(int L, const double *A, const double *B, const spher *S, double *P) {
  double temp = sqrt(0.5 / M_PI);
  P[IDX_P(0, 0)] = temp;
  if (L == 0) return;
  P[IDX_P(1, 0)] = S->cost * sqrt(3.0) * temp;
  temp = -sqrt(1.5) * S->sint * temp;
  P[IDX_P(1, 1)] = temp;
  for (int l = 2; l <= L; ++l) {
    int il = (l * (l + 1)) / 2;
    int ilm1 = il - l;
    int ilm2 = ilm1 - l + 1;
    for (int m = 0; m <= l - 2; ++m)
      P[il + m] = A[il + m] * (S->cost * P[ilm1 + m] + B[il + m] * P[ilm2 + m]);
    P[il + l - 1] = S->cost * sqrt((double)(2 * (l - 1) + 3)) * temp;
    temp = -sqrt(1.0 + 0.5 / l) * S->sint * temp;
    P[il + l] = temp;
  }
}

/* _evaluate_ed! (sphericalharmonics.jl:212-267); P holds P/sin(theta) for m>0 */
static void alp_eval_ed(int L, const double *A, const double *B, const spher *S,
                        double *P, double *dP) {
  double temp = sqrt(0.5 / M_PI);
  P[IDX_P(0, 0)] = temp;
  double temp_d = 0.0;
  dP[IDX_P(0, 0)] = temp_d;
  if (L == 0) return;
  P[IDX_P(1, 0)] = S->cost * sqrt(3.0) * temp;
  dP[IDX_P(1, 0)] = -S->sint * sqrt(3.0) * temp + S->cost * sqrt(3.0) * temp_d;
  double temp1 = -sqrt(1.5) * temp;
  temp_d = -sqrt(1.5) * (S->cost * temp + S->sint * temp_d);
  P[IDX_P(1, 1)] = temp1;
  dP[IDX_P(1, 1)] = temp_d;
  double s2 = S->sint * S->sint;
  for (int l = 2; l <= L; ++l) {
    int m = 0;
    P[IDX_P(l, m)] = A[IDX_P(l, m)] * (S->cost * P[IDX_P(l - 1, m)] + B[IDX_P(l, m)] * P[IDX_P(l - 2, m)]);
    dP[IDX_P(l, m)] = A[IDX_P(l, m)] * (-S->sint * P[IDX_P(l - 1, m)] + S->cost * dP[IDX_P(l - 1, m)]
                                        + B[IDX_P(l, m)] * dP[IDX_P(l - 2, m)]);
    for (m = 1; m <= l - 2; ++m) {
      P[IDX_P(l, m)] = A[IDX_P(l, m)] * (S->cost * P[IDX_P(l - 1, m)] + B[IDX_P(l, m)] * P[IDX_P(l - 2, m)]);
      dP[IDX_P(l, m)] = A[IDX_P(l, m)] * (-s2 * P[IDX_P(l - 1, m)] + S->cost * dP[IDX_P(l - 1, m)]
                                          + B[IDX_P(l, m)] * dP[IDX_P(l - 2, m)]);
    }
    double q = sqrt((double)(2 * (l - 1) + 3));
    P[IDX_P(l, l - 1)] = q * S->cost * temp1;
    dP[IDX_P(l, l - 1)] = q * (-s2 * temp1 + S->cost * temp_d);
    double f = -sqrt(1.0 + 0.5 / l);
    double nt1 = f * S->sint * temp1;
    double ntd = f * (S->cost * temp1 * S->sint + S->sint * temp_d);
    temp1 = nt1;
    temp_d = ntd;
    P[IDX_P(l, l)] = temp1;
    dP[IDX_P(l, l)] = temp_d;
  }
}

/* cYlm! (sphericalharmonics.jl:379-403) */
static void cylm(int L, const spher *S, const double *P, cplx *Y) {
  cplx ep = {1.0 / sqrt(2.0), 0.0};
  for (int l = 0; l <= L; ++l) {
    double p = P[IDX_P(l, 0)];
    Y[IDX_Y(l, 0)].re = p * ep.re;
    Y[IDX_Y(l, 0)].im = p * ep.im;
  }
  int sig = 1;
  cplx ef = {S->cosp, S->sinp};
  for (int m = 1; m <= L; ++m) {
    sig *= -1;
    ep = cmul(ep, ef);
    cplx em = {sig * ep.re, sig * (-ep.im)};
    for (int l = m; l <= L; ++l) {
      double p = P[IDX_P(l, m)];
      Y[IDX_Y(l, -m)] = crmul(em, p);
      Y[IDX_Y(l, m)] = crmul(ep, p);
    }
  }
}

static inline void dspher_to_dcart(const spher *S, cplx fps, cplx ft, cplx *out) {
  double r = S->r + 2.220446049250313e-16; /* S.r + eps() */
  double cc = S->cosp * S->cost, sc = S->sinp * S->cost;
  cplx x, y, z;
  x.re = -(S->sinp * fps.re) + cc * ft.re;  x.im = -(S->sinp * fps.im) + cc * ft.im;
  y.re = (S->cosp * fps.re) + sc * ft.re;   y.im = (S->cosp * fps.im) + sc * ft.im;
  z.re = -(S->sint * ft.re);                z.im = -(S->sint * ft.im);
  out[0].re = x.re / r; out[0].im = x.im / r;
  out[1].re = y.re / r; out[1].im = y.im / r;
  out[2].re = z.re / r; out[2].im = z.im / r;
}

/* cYlm_ed! (sphericalharmonics.jl:410-443); dY has 3 entries per (l,m) */
static void cylm_ed(int L, const spher *S, const double *P, const double *dP, cplx *Y, cplx *dY) {
  double ep0 = 1.0 / sqrt(2.0);
  for (int l = 0; l <= L; ++l) {
    Y[IDX_Y(l, 0)].re = P[IDX_P(l, 0)] * ep0;
    Y[IDX_Y(l, 0)].im = 0.0;
    cplx z0 = {0.0, 0.0}, ft = {dP[IDX_P(l, 0)] * ep0, 0.0};
    dspher_to_dcart(S, z0, ft, &dY[3 * IDX_Y(l, 0)]);
  }
  int sig = 1;
  cplx ef = {S->cosp, S->sinp};
  cplx ep = {ep0 * ef.re, ep0 * ef.im}; /* first ep *= ep_fact is real * complex */
  for (int m = 1; m <= L; ++m) {
    sig *= -1;
    if (m > 1) ep = cmul(ep, ef);
    cplx em = {sig * ep.re, sig * (-ep.im)};
    cplx dep = {-(double)m * ep.im, (double)m * ep.re};   /* im*m*ep */
    cplx dem = {(double)m * em.im, -(double)m * em.re};   /* im*(-m)*em */
    for (int l = m; l <= L; ++l) {
      double p = P[IDX_P(l, m)];
      Y[IDX_Y(l, -m)] = crmul(crmul(em, p), S->sint);
      Y[IDX_Y(l, m)] = crmul(crmul(ep, p), S->sint);
      double dp = dP[IDX_P(l, m)];
      dspher_to_dcart(S, crmul(dem, p), crmul(em, dp), &dY[3 * IDX_Y(l, -m)]);
      dspher_to_dcart(S, crmul(dep, p), crmul(ep, dp), &dY[3 * IDX_Y(l, m)]);
    }
  }
}

/* --------------------------------------------------------------- workspace */

typedef struct {
  double *alpA, *alpB, *P, *dP, *R, *dR;
  cplx *Y, *dY, *A, *dA, *dAco, *dAAdA;
  double *AA, *dAA;
  int Lw;
} work_t;

static int work_init(work_t *w, const oracle_spec *s, int maxJ, int want_dA, int want_dAA) {
  memset(w, 0, sizeof(*w));
  int L = s->L;
  int szP = (L + 1) * (L + 2) / 2, szY = (L + 1) * (L + 1);
  w->alpA = malloc(sizeof(double) * szP);
  w->alpB = malloc(sizeof(double) * szP);
  w->P = malloc(sizeof(double) * szP);
  w->dP = malloc(sizeof(double) * szP);
  w->R = malloc(sizeof(double) * s->nR);
  w->dR = malloc(sizeof(double) * s->nR);
  w->Y = malloc(sizeof(cplx) * szY);
  w->dY = malloc(sizeof(cplx) * 3 * szY);
  w->A = malloc(sizeof(cplx) * s->nA);
  w->dAco = malloc(sizeof(cplx) * s->nA);
  w->dAAdA = malloc(sizeof(cplx) * (s->maxord + 1));
  w->dA = want_dA ? malloc(sizeof(cplx) * 3 * (size_t)s->nA * (maxJ > 0 ? maxJ : 1)) : NULL;
  w->AA = malloc(sizeof(double) * (s->nAA > 0 ? s->nAA : 1));
  w->dAA = want_dAA ? malloc(sizeof(double) * 3 * (size_t)s->nAA * (maxJ > 0 ? maxJ : 1)) : NULL;
  if (!w->alpA || !w->alpB || !w->P || !w->dP || !w->R || !w->dR || !w->Y || !w->dY ||
      !w->A || !w->dAco || !w->dAAdA || !w->AA || (want_dA && !w->dA) || (want_dAA && !w->dAA))
    return -1;
  alp_coeffs(L, w->alpA, w->alpB);
  return 0;
}

static void work_free(work_t *w) {
  free(w->alpA); free(w->alpB); free(w->P); free(w->dP); free(w->R); free(w->dR);
  free(w->Y); free(w->dY); free(w->A); free(w->dAco); free(w->dAAdA); free(w->dA);
  free(w->AA); free(w->dAA);
}

static inline int species_of(const int32_t *species, int64_t j) { return species ? species[j] : 0; }

/* A = sum_j phi(X_j) through the evaluate path (product_1pbasis.jl:99-134) */
static void eval_A(const oracle_spec *s, work_t *w, const double *rr, const int32_t *sp, int64_t J,
                   int64_t o) {
  for (int i = 0; i < s->nA; ++i) { w->A[i].re = 0.0; w->A[i].im = 0.0; }
  for (int64_t j = 0; j < J; ++j) {
    const double *x = rr + 3 * j;
    double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    if (s->Rext) memcpy(w->R, s->Rext + (o + j) * s->nR, sizeof(double) * s->nR);
    else radial_eval(s, transform_t(s, r), w->R);
    spher S = cart2spher(x);
    alp_eval(s->L, w->alpA, w->alpB, &S, w->P);
    cylm(s->L, &S, w->P, w->Y);
    int mu = species_of(sp, j);
    for (int i = 0; i < s->nA; ++i) {
      if (s->a_mu && s->a_mu[i] != mu) continue;
      cplx t = crmul(w->Y[s->a_iy[i]], w->R[s->a_n[i]]);
      w->A[i] = cadd(w->A[i], t);
    }
  }
}

/* A and materialised dA[i, j] through the evaluate_ed path
   (product_1pbasis.jl:169-244) */
static void eval_A_dA(const oracle_spec *s, work_t *w, const double *rr, const int32_t *sp, int64_t J,
                      int64_t o) {
  for (int i = 0; i < s->nA; ++i) { w->A[i].re = 0.0; w->A[i].im = 0.0; }
  for (int64_t j = 0; j < J; ++j) {
    const double *x = rr + 3 * j;
    double r = sqrt(x[0] * x[0] + x[1] * x[1] + x[2] * x[2]);
    double t = transform_t(s, r);
    /* dR_n = P_n'(t) * (t'(r) * rr/r) */
    double dt = transform_dt(s, r);
    if (s->Rext) {
      memcpy(w->R, s->Rext + (o + j) * s->nR, sizeof(double) * s->nR);
      memcpy(w->dR, s->dRext + (o + j) * s->nR, sizeof(double) * s->nR);
      dt = 1.0;  /* dRext is already dR/dr */
    } else {
      radial_eval_ed(s, t, w->R, w->dR);
    }
    double g[3] = {dt * (x[0] / r), dt * (x[1] / r), dt * (x[2] / r)};
    spher S = cart2spher(x);
    alp_eval_ed(s->L, w->alpA, w->alpB, &S, w->P, w->dP);
    cylm_ed(s->L, &S, w->P, w->dP, w->Y, w->dY);
    int mu = species_of(sp, j);
    for (int i = 0; i < s->nA; ++i) {
      cplx *d = &w->dA[3 * ((size_t)j * s->nA + i)];
      if (s->a_mu && s->a_mu[i] != mu) {
        d[0].re = d[0].im = d[1].re = d[1].im = d[2].re = d[2].im = 0.0;
        continue;
      }
      int n = s->a_n[i], iy = s->a_iy[i];
      double Rn = w->R[n];
      cplx Y = w->Y[iy];
      w->A[i] = cadd(w->A[i], crmul(Y, Rn));
      for (int a = 0; a < 3; ++a) {
        double dRa = w->dR[n] * g[a];
        cplx v = {0.0 + dRa * Y.re, 0.0 + dRa * Y.im};
        d[a] = cadd(v, crmul(w->dY[3 * iy + a], Rn));
      }
    }
  }
}

/* _AA_local_adjoints! (pibasis.jl:338-390); returns real(AA) */
static double aa_local_adjoints(const oracle_spec *s, const cplx *A, int64_t iAA, cplx *d) {
  int ord = s->orders[iAA];
  const int32_t *v = s->iAA2iA + iAA * s->maxord;
  if (ord == 1) { d[0].re = 1.0; d[0].im = 0.0; return A[v[0]].re; }
  cplx A1 = A[v[0]], A2 = A[v[1]];
  if (ord == 2) { d[0] = A2; d[1] = A1; return cmul(A1, A2).re; }
  d[0].re = 1.0; d[0].im = 0.0;
  d[1] = A1;
  cplx fwd = cmul(A1, A2);
  for (int a = 2; a < ord - 1; ++a) { d[a] = fwd; fwd = cmul(fwd, A[v[a]]); }
  d[ord - 1] = fwd;
  cplx Aend = A[v[ord - 1]];
  double aa = cmul(fwd, Aend).re;
  cplx bwd = Aend;
  for (int a = ord - 2; a >= 2; --a) { d[a] = cmul(d[a], bwd); bwd = cmul(bwd, A[v[a]]); }
  d[1] = cmul(d[1], bwd);
  bwd = cmul(bwd, A2);
  d[0] = cmul(d[0], bwd);
  return aa;
}

/* ProductEvaluator evaluate (evaluator.jl:121-147) */
static double energy_from_A(const oracle_spec *s, const cplx *A) {
  double val = 0.0;
  int64_t i0 = 0;
  if (s->nAA > 0 && s->orders[0] == 0) { val += s->ctilde[0]; i0 = 1; }
  for (int64_t iAA = i0; iAA < s->nAA; ++iAA) {
    const int32_t *v = s->iAA2iA + iAA * s->maxord;
    cplx aa = A[v[0]];
    for (int t = 1; t < s->orders[iAA]; ++t) aa = cmul(aa, A[v[t]]);
    val += aa.re * s->ctilde[iAA];
  }
  return val;
}

int oracle_energy(const oracle_spec *s, int64_t nEnv, const int64_t *offsets,
                  const double *rr, const int32_t *species, double *E, int nthreads) {
  int err = 0;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(| : err)
#endif
  {
    work_t w;
    if (work_init(&w, s, 0, 0, 0) != 0) err |= 1;
    else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
      for (int64_t e = 0; e < nEnv; ++e) {
        int64_t o = offsets[e], J = offsets[e + 1] - offsets[e];
        eval_A(s, &w, rr + 3 * o, species ? species + o : NULL, J, o);
        E[e] = energy_from_A(s, w.A);
      }
    }
    work_free(&w);
  }
  return err ? -1 : 0;
}

/* _rrule_evaluate (evaluator.jl:161-200): G[3*j + a] = dE/drr_j[a] */
static void grad_env(const oracle_spec *s, work_t *w, const double *rr, const int32_t *sp,
                     int64_t J, int64_t o, double *G) {
  eval_A_dA(s, w, rr, sp, J, o);
  for (int i = 0; i < s->nA; ++i) { w->dAco[i].re = 0.0; w->dAco[i].im = 0.0; }
  int64_t i0 = (s->nAA > 0 && s->orders[0] == 0) ? 1 : 0;
  for (int64_t iAA = i0; iAA < s->nAA; ++iAA) {
    aa_local_adjoints(s, w->A, iAA, w->dAAdA);
    const int32_t *v = s->iAA2iA + iAA * s->maxord;
    double c = s->ctilde[iAA];
    for (int t = 0; t < s->orders[iAA]; ++t)
      w->dAco[v[t]] = cadd(w->dAco[v[t]], crmul(w->dAAdA[t], c));
  }
  for (int64_t j = 0; j < J; ++j) {
    double g0 = 0.0, g1 = 0.0, g2 = 0.0;
    for (int i = 0; i < s->nA; ++i) {
      const cplx *d = &w->dA[3 * ((size_t)j * s->nA + i)];
      cplx c = w->dAco[i];
      g0 += cmul(c, d[0]).re;
      g1 += cmul(c, d[1]).re;
      g2 += cmul(c, d[2]).re;
    }
    G[3 * j + 0] = g0; G[3 * j + 1] = g1; G[3 * j + 2] = g2;
  }
}

static int64_t max_J(int64_t nEnv, const int64_t *offsets) {
  int64_t m = 0;
  for (int64_t e = 0; e < nEnv; ++e) if (offsets[e + 1] - offsets[e] > m) m = offsets[e + 1] - offsets[e];
  return m;
}

int oracle_grad_config(const oracle_spec *s, int64_t nEnv, const int64_t *offsets,
                       const double *rr, const int32_t *species, double *G, int nthreads) {
  int err = 0;
  int64_t mJ = max_J(nEnv, offsets);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(| : err)
#endif
  {
    work_t w;
    if (work_init(&w, s, (int)mJ, 1, 0) != 0) err |= 1;
    else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
      for (int64_t e = 0; e < nEnv; ++e) {
        int64_t o = offsets[e], J = offsets[e + 1] - offsets[e];
        grad_env(s, &w, rr + 3 * o, species ? species + o : NULL, J, o, G + 3 * o);
      }
    }
    work_free(&w);
  }
  return err ? -1 : 0;
}

int oracle_energy_forces(const oracle_spec *s, int64_t nEnv, const int64_t *offsets,
                         const double *rr, const int32_t *species, double *E, double *G,
                         int nthreads) {
  int err = 0;
  int64_t mJ = max_J(nEnv, offsets);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(| : err)
#endif
  {
    work_t w;
    if (work_init(&w, s, (int)mJ, 1, 0) != 0) err |= 1;
    else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
      for (int64_t e = 0; e < nEnv; ++e) {
        int64_t o = offsets[e], J = offsets[e + 1] - offsets[e];
        const int32_t *sp = species ? species + o : NULL;
        eval_A(s, &w, rr + 3 * o, sp, J, o);
        E[e] = energy_from_A(s, w.A);
        grad_env(s, &w, rr + 3 * o, sp, J, o, G + 3 * o);
      }
    }
    work_free(&w);
  }
  return err ? -1 : 0;
}

int oracle_A(const oracle_spec *s, int64_t nEnv, const int64_t *offsets, const double *rr,
             const int32_t *species, double *Aout /* nEnv x nA x 2 */, int nthreads) {
  int err = 0;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(| : err)
#endif
  {
    work_t w;
    if (work_init(&w, s, 0, 0, 0) != 0) err |= 1;
    else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
      for (int64_t e = 0; e < nEnv; ++e) {
        int64_t o = offsets[e], J = offsets[e + 1] - offsets[e];
        eval_A(s, &w, rr + 3 * o, species ? species + o : NULL, J, o);
        memcpy(Aout + 2 * (size_t)e * s->nA, w.A, sizeof(cplx) * s->nA);
      }
    }
    work_free(&w);
  }
  return err ? -1 : 0;
}

/* SymmetricBasis evaluate (symmbasis.jl:297-316): B = real(U * real(AA)) */
int oracle_basis(const oracle_spec *s, int64_t nEnv, const int64_t *offsets, const double *rr,
                 const int32_t *species, double *B /* nEnv x nB */, int nthreads) {
  int err = 0;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(| : err)
#endif
  {
    work_t w;
    if (work_init(&w, s, 0, 0, 0) != 0) err |= 1;
    else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
      for (int64_t e = 0; e < nEnv; ++e) {
        int64_t o = offsets[e], J = offsets[e + 1] - offsets[e];
        eval_A(s, &w, rr + 3 * o, species ? species + o : NULL, J, o);
        /* PIBasis evaluate! (pibasis.jl:265-275) */
        for (int64_t iAA = 0; iAA < s->nAA; ++iAA) {
          const int32_t *v = s->iAA2iA + iAA * s->maxord;
          cplx aa = {1.0, 0.0};
          for (int t = 0; t < s->orders[iAA]; ++t) aa = cmul(aa, w.A[v[t]]);
          w.AA[iAA] = aa.re;
        }
        /* genmul! (symmbasis.jl:248-264): rows accumulate columns in ascending order */
        double *Be = B + (size_t)e * s->nB;
        for (int64_t b = 0; b < s->nB; ++b) {
          double acc = 0.0;
          for (int64_t k = s->U_indptr[b]; k < s->U_indptr[b + 1]; ++k)
            acc += s->U_data[k] * w.AA[s->U_indices[k]];
          Be[b] = acc;
        }
      }
    }
    work_free(&w);
  }
  return err ? -1 : 0;
}

/* SymmetricBasis evaluate_ed (symmbasis.jl:322-334, pibasis.jl:402-432):
   B[e, b] and dB[(o_e + j) * nB + b][a] = dB_b / drr_j[a] */
int oracle_basis_d(const oracle_spec *s, int64_t nEnv, const int64_t *offsets, const double *rr,
                   const int32_t *species, double *B, double *dB, int nthreads) {
  int err = 0;
  int64_t mJ = max_J(nEnv, offsets);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(| : err)
#endif
  {
    work_t w;
    if (work_init(&w, s, (int)mJ, 1, 1) != 0) err |= 1;
    else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 2)
#endif
      for (int64_t e = 0; e < nEnv; ++e) {
        int64_t o = offsets[e], J = offsets[e + 1] - offsets[e];
        eval_A_dA(s, &w, rr + 3 * o, species ? species + o : NULL, J, o);
        int64_t i0 = 0;
        if (s->nAA > 0 && s->orders[0] == 0) {
          w.AA[0] = 1.0;
          for (int64_t j = 0; j < J; ++j) {
            double *d0 = &w.dAA[3 * ((size_t)j * s->nAA)];
            d0[0] = d0[1] = d0[2] = 0.0;
          }
          i0 = 1;
        }
        for (int64_t iAA = i0; iAA < s->nAA; ++iAA) {
          w.AA[iAA] = aa_local_adjoints(s, w.A, iAA, w.dAAdA);
          const int32_t *v = s->iAA2iA + iAA * s->maxord;
          int ord = s->orders[iAA];
          for (int64_t j = 0; j < J; ++j) {
            for (int a = 0; a < 3; ++a) {
              cplx acc = cmul(w.dAAdA[0], w.dA[3 * ((size_t)j * s->nA + v[0]) + a]);
              for (int t = 1; t < ord; ++t)
                acc = cadd(acc, cmul(w.dAAdA[t], w.dA[3 * ((size_t)j * s->nA + v[t]) + a]));
              w.dAA[3 * ((size_t)j * s->nAA + iAA) + a] = acc.re;
            }
          }
        }
        double *Be = B + (size_t)e * s->nB;
        for (int64_t b = 0; b < s->nB; ++b) {
          double acc = 0.0;
          for (int64_t k = s->U_indptr[b]; k < s->U_indptr[b + 1]; ++k)
            acc += s->U_data[k] * w.AA[s->U_indices[k]];
          Be[b] = acc;
        }
        for (int64_t j = 0; j < J; ++j) {
          double *dBj = dB + 3 * ((size_t)(o + j) * s->nB);
          for (int64_t b = 0; b < s->nB; ++b) {
            double a0 = 0.0, a1 = 0.0, a2 = 0.0;
            for (int64_t k = s->U_indptr[b]; k < s->U_indptr[b + 1]; ++k) {
              const double *d = &w.dAA[3 * ((size_t)j * s->nAA + s->U_indices[k])];
              double u = s->U_data[k];
              a0 += u * d[0]; a1 += u * d[1]; a2 += u * d[2];
            }
            dBj[3 * b] = a0; dBj[3 * b + 1] = a1; dBj[3 * b + 2] = a2;
          }
        }
      }
    }
    work_free(&w);
  }
  return err ? -1 : 0;
}

/* ------------------------------------------------- component access (tests) */

/* Y (and dY when dY != NULL) at one point, through cYlm! or cYlm_ed! */
/* dE/dR_n(r_j): the adjoint dAco of grad_env contracted with Y instead of dA
   (the chain rule of src/evaluator.jl:187-192 stopped at the radial values) */
int oracle_radial_adjoint(const oracle_spec *s, int64_t nEnv, const int64_t *offsets,
                          const double *rr, const int32_t *species, double *E, double *GR,
                          int nthreads) {
  int err = 0;
  int64_t mJ = max_J(nEnv, offsets);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(| : err)
#endif
  {
    work_t w;
    if (work_init(&w, s, (int)mJ, 1, 0) != 0) err |= 1;
    else {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
      for (int64_t e = 0; e < nEnv; ++e) {
        int64_t o = offsets[e], J = offsets[e + 1] - offsets[e];
        const int32_t *sp = species ? species + o : NULL;
        eval_A(s, &w, rr + 3 * o, sp, J, o);
        E[e] = energy_from_A(s, w.A);
        for (int i = 0; i < s->nA; ++i) { w.dAco[i].re = 0.0; w.dAco[i].im = 0.0; }
        int64_t i0 = (s->nAA > 0 && s->orders[0] == 0) ? 1 : 0;
        for (int64_t iAA = i0; iAA < s->nAA; ++iAA) {
          aa_local_adjoints(s, w.A, iAA, w.dAAdA);
          const int32_t *v = s->iAA2iA + iAA * s->maxord;
          double c = s->ctilde[iAA];
          for (int t = 0; t < s->orders[iAA]; ++t)
            w.dAco[v[t]] = cadd(w.dAco[v[t]], crmul(w.dAAdA[t], c));
        }
        for (int64_t j = 0; j < J; ++j) {
          const double *x = rr + 3 * (o + j);
          spher S = cart2spher(x);
          alp_eval(s->L, w.alpA, w.alpB, &S, w.P);
          cylm(s->L, &S, w.P, w.Y);
          double *g = GR + (o + j) * s->nR;
          for (int n = 0; n < s->nR; ++n) g[n] = 0.0;
          int mu = species_of(sp, j);
          for (int i = 0; i < s->nA; ++i) {
            if (s->a_mu && s->a_mu[i] != mu) continue;
            g[s->a_n[i]] += cmul(w.dAco[i], w.Y[s->a_iy[i]]).re;
          }
        }
      }
    }
    work_free(&w);
  }
  return err ? -1 : 0;
}

int oracle_sh(int L, const double *x, double *Y /* (L+1)^2 x 2 */, double *dY /* (L+1)^2 x 3 x 2 */) {
  int szP = (L + 1) * (L + 2) / 2;
  double *A = malloc(sizeof(double) * szP), *B = malloc(sizeof(double) * szP);
  double *P = malloc(sizeof(double) * szP), *dP = malloc(sizeof(double) * szP);
  if (!A || !B || !P || !dP) { free(A); free(B); free(P); free(dP); return -1; }
  alp_coeffs(L, A, B);
  spher S = cart2spher(x);
  if (dY) {
    alp_eval_ed(L, A, B, &S, P, dP);
    cylm_ed(L, &S, P, dP, (cplx *)Y, (cplx *)dY);
  } else {
    alp_eval(L, A, B, &S, P);
    cylm(L, &S, P, (cplx *)Y);
  }
  free(A); free(B); free(P); free(dP);
  return 0;
}

/* R_n(r) and dR_n/dr at radii r[k] */
int oracle_radial(const oracle_spec *s, int64_t n, const double *r, double *R, double *dR) {
  double *dP = malloc(sizeof(double) * s->nR);
  if (!dP) return -1;
  for (int64_t k = 0; k < n; ++k) {
    double t = transform_t(s, r[k]);
    radial_eval_ed(s, t, R + k * s->nR, dP);
    double dt = transform_dt(s, r[k]);
    for (int i = 0; i < s->nR; ++i) dR[k * s->nR + i] = dP[i] * dt;
  }
  free(dP);
  return 0;
}
