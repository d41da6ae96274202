/*
 * ace_oracle.h -- FP64 CPU restatement of ACE.jl's evaluation hot path.
 * TEST INFRASTRUCTURE ONLY (correctness oracle and CPU baseline).
 */
#ifndef ACE_ORACLE_H
#define ACE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  /* radial basis (OrthPolyBasis + polytransform) */
  int nR;
  const double *rA, *rB, *rC;
  int pl, pr;
  double tl, tr;
  int tp;          /* transform exponent p */
  double r0;       /* transform r0 */
  /* spherical harmonics degree to evaluate */
  int L;
  /* A spec: radial index (0-based), index_y (0-based), species (NULL = one species) */
  int nA;
  const int32_t *a_n, *a_iy, *a_mu;
  /* AA spec: orders and row-major iAA2iA (0-based, -1 padded), c~ */
  int64_t nAA;
  int maxord;
  const int32_t *orders;
  const int32_t *iAA2iA;
  const double *ctilde;
  /* U as CSR (nB x nAA) */
  int64_t nB;
  const int64_t *U_indptr;
  const int32_t *U_indices;
  const double *U_data;
  /* externally supplied radial channels (learned radial form): when non-NULL,
     R_n(r_j) = Rext[j * nR + n] and dR_n/dr(r_j) = dRext[j * nR + n] for the
     batch's neighbour j (absolute index) replace the polynomial radial basis */
  const double *Rext, *dRext;
} oracle_spec;

int oracle_energy(const oracle_spec *s, int64_t nEnv, const int64_t *offsets,
                  const double *rr, const int32_t *species, double *E, int nthreads);
int oracle_grad_config(const oracle_spec *s, int64_t nEnv, const int64_t *offsets,
                       const double *rr, const int32_t *species, double *G, int nthreads);
int oracle_energy_forces(const oracle_spec *s, int64_t nEnv, const int64_t *offsets,
                         const double *rr, const int32_t *species, double *E, double *G,
                         int nthreads);
int oracle_A(const oracle_spec *s, int64_t nEnv, const int64_t *offsets, const double *rr,
             const int32_t *species, double *Aout, int nthreads);
int oracle_basis(const oracle_spec *s, int64_t nEnv, const int64_t *offsets, const double *rr,
                 const int32_t *species, double *B, int nthreads);
int oracle_basis_d(const oracle_spec *s, int64_t nEnv, const int64_t *offsets, const double *rr,
                   const int32_t *species, double *B, double *dB, int nthreads);

/* dE/dR_n(r_j) = sum_{i: a_n[i] == n} Re(dAco_i Y_{a_iy[i]}(rhat_j)) for every
   neighbour j and radial channel n (GR is nNbr x nR), and E */
int oracle_radial_adjoint(const oracle_spec *s, int64_t nEnv, const int64_t *offsets,
                          const double *rr, const int32_t *species, double *E, double *GR,
                          int nthreads);

int oracle_sh(int L, const double *x, double *Y, double *dY);
int oracle_radial(const oracle_spec *s, int64_t n, const double *r, double *R, double *dR);

#ifdef __cplusplus
}
#endif
#endif
