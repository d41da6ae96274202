/*
 * ace_b200.h -- C ABI of libace_b200, a GB300 (sm_103a) evaluator for linear
 * ACE models.  Plain pointers and sizes only; every call returns an int
 * status (ACE_OK == 0) and no exception crosses the ABI.
 *
 * The library replaces the CPU evaluation that ACE.jl performs through Julia
 * dispatch (the reference has no FFI; the entry points below are what a
 * Julia `ccall` shim, or any C caller, binds):
 *
 *   ace_ctx_create      <- LinearACEModel(basis, c; evaluator=:standard)
 *                          src/linearmodel.jl:44-56, ProductEvaluator(basis, c)
 *                          src/evaluator.jl:30-31
 *   ace_set_params      <- set_params!(m, c)  src/linearmodel.jl:67-71,
 *                          src/evaluator.jl:48-56 (c~ = U^T c, :59-60)
 *   ace_energy          <- evaluate(m::LinearACEModel, cfg)
 *                          src/linearmodel.jl:107-108 -> src/evaluator.jl:121-147
 *   ace_energy_forces   <- evaluate + grad_config(m, cfg)
 *                          src/linearmodel.jl:110-111 -> src/evaluator.jl:150-200
 *   ace_basis           <- evaluate(basis::SymmetricBasis, cfg) and
 *                          evaluate_d / evaluate_ed   src/symmbasis.jl:297-336
 *                          (grad_params = B, grad_params_config = dB,
 *                          src/linearmodel.jl:114-128)
 *   ace_adjoint_eval_d  <- adjoint_EVAL_D(m, cfg, w)  src/evaluator.jl:204-244
 *
 * Many environments are evaluated per call: environment e owns neighbours
 * offsets[e] .. offsets[e+1]-1 of the position array (CSR).  Positions are
 * rr_j = X_j - X_centre, stored as x,y,z triples (the memory layout of a
 * Julia Vector{SVector{3,Float64}}).
 *
 * Ownership: the caller owns all input and output buffers; the context owns
 * every device allocation it makes.  Threading: one context per host thread
 * (or per stream); calls on one context must not overlap.
 */
#ifndef ACE_B200_H
#define ACE_B200_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ACE_SPEC_VERSION 1

/* status codes */
enum {
  ACE_OK = 0,
  ACE_ERR_INVALID = 1,      /* invalid argument or input data (see ace_last_error_string) */
  ACE_ERR_CUDA = 2,         /* a CUDA runtime call failed */
  ACE_ERR_ALLOC = 3,        /* device or host allocation failed */
  ACE_ERR_KERNEL = 4,       /* a kernel reported a bad status word */
  ACE_ERR_UNSUPPORTED = 5,  /* the spec exceeds a compiled limit */
  ACE_ERR_EMPTY_ENV = 6     /* informational: an environment had no neighbours */
};

/* precision modes */
enum {
  ACE_PREC_FP64 = 0,        /* all arithmetic in FP64 */
  ACE_PREC_FP32 = 1,        /* everything in FP32 (per-environment sums in FP64) */
  ACE_PREC_FP32_BF16X3 = 2, /* reserved: ace_ctx_create rejects it with ACE_ERR_UNSUPPORTED */
  ACE_PREC_LEARNED = 3,     /* reserved; the learned radial form is ace_set_radial_mlp */
  ACE_PREC_FP32X2 = 4,      /* energy path (Rn, Ylm, A, AA) in double-float (pairs of FP32
                               with error-free transformations), adjoint and forces in FP32 */
  ACE_PREC_FP32_COMP = 5    /* compensated: Rn, Ylm and A in double-float; the correlation
                               products, adjoint and forces in FP32 on A rounded to FP32, the
                               energy summed in double-float and corrected to first order for
                               that rounding (E += Re sum_i dE/dA_i A_lo_i); environments whose
                               estimated energy error exceeds a tolerance are evaluated again in
                               double-float (ace_set_energy_tolerance); every other path as
                               ACE_PREC_FP32X2 */
};

/* flags for the evaluation calls */
enum {
  ACE_INPUTS_ON_DEVICE = 1,   /* offsets/rr/species are device pointers */
  ACE_OUTPUTS_ON_DEVICE = 2,  /* E/dEdrr/B/dB are device pointers */
  ACE_ASYNC = 4               /* with device inputs and outputs: do not synchronise */
};

/*
 * The basis specification (the product of basis construction; see the
 * spec builder in the host package).  All arrays are host memory and are
 * copied by ace_ctx_create.
 *
 *   radial:  R_n(r) = P_n(t(r)), t(r) = ((1+r0)/(1+r))^tp,
 *            P_1 = rA[0] fcut(t), P_2 = (rA[1] t + rB[1]) P_1,
 *            P_n = (rA[n-1] t + rB[n-1]) P_{n-1} + rC[n-1] P_{n-2},
 *            fcut(t) = (t-tl)^pl (t-tr)^pr, zero if pl>0 && t<tl or pr>0 && t>tr
 *   1p:      A_i = sum_j [mu_j == a_mu[i]] R_{a_n[i]}(r_j) Y_{a_l[i]}^{a_m[i]}(rhat_j)
 *            (a_n 0-based; a_mu may be NULL for one species)
 *   AA:      AA_k = prod_{t < orders[k]} A_{iAA2iA[k*maxord + t]}  (row-major, -1 padded)
 *   U:       B = U AA  (CSR, nB x nAA)
 */
typedef struct {
  int32_t version;
  int32_t nR;
  const double *rA, *rB, *rC;
  int32_t pl, pr;
  double tl, tr;
  int32_t tp;
  double r0;
  int32_t nA;
  const int32_t *a_n, *a_l, *a_m, *a_mu;
  int32_t nspecies;
  int64_t nAA;
  int32_t maxord;
  const int32_t *orders;
  const int32_t *iAA2iA;
  int64_t nB;
  const int64_t *U_indptr;
  const int32_t *U_indices;
  const double *U_data;
} ace_spec_bundle;

typedef struct ace_ctx ace_ctx;

/* Create a context on CUDA device `device`: copies the spec to the device
   and prepares the evaluation tables.  Coefficients start at zero. */
int ace_ctx_create(const ace_spec_bundle *spec, int32_t precision_mode, int32_t device,
                   ace_ctx **out);
int ace_ctx_destroy(ace_ctx *ctx);

/* set_params!: B-basis coefficients c (length nB); c~ = U^T c is formed on the host. */
int ace_set_params(ace_ctx *ctx, const double *c, int64_t nB);
/* The AA-basis coefficients c~ directly (length nAA). */
int ace_set_ctilde(ace_ctx *ctx, const double *ctilde, int64_t nAA);

/* Multi-property models (c::Vector{SVector{N}}, src/linearmodel.jl:28-35):
   nprop coefficient sets for one basis, property-major c[p*nB + b]. */
int ace_set_params_multi(ace_ctx *ctx, const double *c, int64_t nB, int32_t nprop);
/* Complex AA coefficients for nprop properties, ct[(p*nAA + k)*2 + {0,1}] =
   (re, im): property p evaluates Re(sum_k ct_pk AA_k).  This is how an
   EuclideanVector model (src/properties.jl:154-248, B_b = Re(U_b . AA) in
   R^3 with complex U) is evaluated: one property per Cartesian component
   with c~^(i) = U_i^T c.  Needs the item schedule; then evaluate with
   ace_energy_forces_multi. */
int ace_set_ctilde_complex(ace_ctx *ctx, const double *ct, int64_t nAA, int32_t nprop);

/* Energies E[p*nEnv + e] and gradients dEdrr[(p*nNbr + j)*3 + a] of every
   property set by ace_set_params_multi or ace_set_ctilde_complex
   (property-major outputs). */
int ace_energy_forces_multi(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                            const int32_t *species, double *E, double *dEdrr, int32_t flags, void *stream);

/* Site energies E[e] and gradients dEdrr[3*j + a] = dE_{e(j)}/d rr_j[a]
   (grad_config; forces on neighbours are -dEdrr).  dEdrr may be NULL.
   species may be NULL for a one-species spec.  `stream` is a cudaStream_t
   (NULL = the legacy default stream). */
int ace_energy_forces(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                      const int32_t *species, double *E, double *dEdrr, int32_t flags,
                      void *stream);
int ace_energy(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
               const int32_t *species, double *E, int32_t flags, void *stream);

/* Error control of the compensated form (ACE_PREC_FP32_COMP; other modes
   return ACE_ERR_UNSUPPORTED).  Its rounding errors are those of the FP32
   correlation products; products that share a rounding (the prefix of a
   task, the terms of an item) form a group g with summed magnitude S_g, and
   every single-property ace_energy_forces launch with gradients estimates
   each environment's energy error as est_e = k sqrt(sum_g S_g^2) 2^-24,
   k = 5 on the task schedule and 7 on the item runs (measured against FP64
   on orders 4 and 5: errors up to 3.9 and 5.5 times the root sum square).
   Environments with est_e > tol * max(|E_e|, rms of E over the launch) are
   then evaluated again in double-float (ACE_PREC_FP32X2 arithmetic, energy
   error ~1e-12) within the same call, on the device (no synchronisation:
   the call stays asynchronous and capturable).  tol = 0 turns the
   re-evaluation off; the default is 1e-6.  Energy-only calls (ace_energy,
   or dEdrr = NULL) of a compensated context run the double-float energy
   kernel (no adjoint needed, energy error ~1e-12) and make no estimates.
   No counterpart in the reference (its evaluation is FP64). */
int ace_set_energy_tolerance(ace_ctx *ctx, double tol);
/* est_e of the last single-property energy/gradient call's first nEnv environments
   (est: host array, may be NULL; the estimate of the compensated
   evaluation also for re-evaluated environments) and the number of
   environments re-evaluated since the context was created (refined, may be
   NULL).  Synchronises with the context's work. */
int ace_energy_error_estimates(ace_ctx *ctx, int64_t nEnv, double *est, int64_t *refined);

/* Symmetric basis B[e*nB + b]; if dB != NULL also
   dB[(j*nB + b)*3 + a] = dB_b(env of j)/d rr_j[a]. */
int ace_basis(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
              const int32_t *species, double *B, double *dB, int32_t flags, void *stream);

/* adjoint_EVAL_D (src/evaluator.jl:204-244): out[e*nB + b] =
   sum_{j in e} sum_a w[3*j + a] * dB_b/d rr_j[a] -- the mixed derivative used
   for force matching, without forming dB.  w lives where rr lives (flags). */
int ace_adjoint_eval_d(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                       const int32_t *species, const double *w, double *out, int32_t flags, void *stream);

/* The symmetric basis B (as ace_basis, without dB) for callers that must not
   allocate device memory while they run -- e.g. an MD engine that owns the
   device memory pool after start-up, or a service with a fixed footprint.
   No counterpart in the reference (ACE.jl allocates per call).  Allocates
   nothing: inputs and B must be device pointers; its scratch is a 16 MiB
   static device array held by every GPU that loads the library.  Specs whose
   per-environment AA vector (nAA x 8 bytes, or x 4 in FP32 mode) exceeds
   16 MiB are rejected with ACE_ERR_UNSUPPORTED, as is the learned radial
   form.  ace_ctx_create looks up the array's device address and loads this
   entry point's device code, so only context creation allocates: every call
   of ace_basis_noalloc, the first included, allocates nothing.  The saved
   address does not survive a cudaDeviceReset of the device.  Runs
   asynchronously on `stream` (ace_sync reports the kernels' status).  All
   calls share the scratch: calls that overlap on the GPU race and must be
   serialised by the caller. */
int ace_basis_noalloc(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                      const int32_t *species, double *B, void *stream);

/* Autotuner: times the energy/force kernel on a representative batch (device
   pointers; E and dEdrr are overwritten) for each candidate launch
   configuration -- correlation algorithm (task schedule for orders >= 3,
   item runs, or trie walk; the compensated form has no trie walk) and
   shared-memory region size -- and keeps the fastest for this context.
   *choice (optional) receives region_kb + 1000 * algorithm (0 trie walk,
   1 item runs, 2 task schedule, 3 task schedule with the high-occupancy
   register bound).
   No counterpart in the reference (a GPU launch-configuration choice). */
int ace_autotune(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                 const int32_t *species, double *E, double *dEdrr, int32_t reps, void *stream,
                 int32_t *choice);

/* ---------------------------------------------------------------------
   Learned radial form.  No counterpart in the reference: it replaces the
   radial basis x species one-hot of the 1p basis (src/b1pcomponents/Rn.jl:
   17-29 times src/discrete1pbasis.jl:78-123) by K channels per l computed
   by a small MLP of (transformed distance, neighbour species):

     t = ((1 + r0)/(1 + r))^p and the envelope fe(t) of the spec's radial basis
     x = 2 (t - tl)/(tmax - tl) - 1,  f = [T_0(x) .. T_{Q-1}(x), onehot(s)]
     h1 = silu(W1 f + b1), h2 = silu(W2 h1 + b2)   (H = 64)
     R_{k + K l}(r, s) = fe(t) (W3 h2 + b3)_{k + K l}

   params = [W1 (H x (Q+S)) | b1 (H) | W2 (H x H) | b2 (H) | W3 (C x H) | b3 (C)],
   C = K (L + 1), row-major FP32.  The context's spec must be single-species
   with nR = K; A entry (n, l, m) then reads channel (n - 1) + K l.  After
   ace_set_radial_mlp the context's ace_energy_forces / ace_energy /
   ace_basis / ace_adjoint_eval_d evaluate the learned form (species index
   the MLP's one-hot); ace_basis_noalloc returns ACE_ERR_UNSUPPORTED.  Each
   learned-form call reads the batch's neighbour count back to the host (to
   size its radial buffer) and so synchronises its stream.  The training
   entry points below take device pointers only and run asynchronously on
   `stream`. */
typedef struct ace_radial_mlp {
  int32_t version;  /* 1 */
  int32_t K, Q, nspecies, H;
  double tmax;      /* feature scale: transform value mapped to x = +1 */
  const float *params;
  int64_t nparams;
} ace_radial_mlp;

/* Switch the context to the learned form (first call) or replace the
   parameters (later calls, same shape). */
int ace_set_radial_mlp(ace_ctx *ctx, const ace_radial_mlp *mlp);

/* Device pointer to the context's parameter array (updated in place by
   training) and its length. */
int ace_radial_mlp_params(ace_ctx *ctx, float **d_params, int64_t *nparams);

/* Copy the parameters out (host memory, or device memory with
   ACE_OUTPUTS_ON_DEVICE); synchronous. */
int ace_radial_mlp_get_params(ace_ctx *ctx, float *params, int32_t flags);

/* R[j][c] = R_c(r_j) and R[j][C + c] = dR_c/dr for nNbr neighbours (device). */
int ace_radial_mlp_forward(ace_ctx *ctx, int64_t nNbr, const double *rr, const int32_t *species, float *R,
                           void *stream);

/* The radials the evaluation calls use (R and dR/dr as above): on GB300 a
   tensor-core kernel (tcgen05.mma, BF16 operands, FP32 accumulation) when
   Q + nspecies <= 16 and K (L+1) <= 128, else the FP32 kernel;
   ACE_B200_MLP=fp32 in the environment at ace_set_radial_mlp keeps FP32.
   ace_energy_radial_adjoint (training) always uses the FP32 MLP. */
int ace_radial_mlp_infer(ace_ctx *ctx, int64_t nNbr, const double *rr, const int32_t *species, float *R,
                         void *stream);

/* gparams += sum_j wj[j] sum_c gR[j][c] dR_c(r_j)/dparams (device; wj may be
   NULL for weights 1). */
int ace_radial_mlp_backward(ace_ctx *ctx, int64_t nNbr, const double *rr, const int32_t *species,
                            const float *gR, const float *wj, float *gparams, void *stream);

/* Energies (and dE/drr when dEdrr is not NULL) of the learned form, and
   GR[j][c] = dE/dR_c(r_j): the adjoint of src/evaluator.jl:161-200 stopped
   at the radial values (device pointers). */
int ace_energy_radial_adjoint(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                              const int32_t *species, double *E, double *dEdrr, float *GR, void *stream);

/* One Adam step on n parameters (device): m, v moments; step >= 1. */
int ace_adam_step(int64_t n, float *w, const float *g, float *m, float *v, float lr, float beta1, float beta2,
                  float eps, int32_t step, void *stream);

/* Wait for the context's outstanding work; returns the kernels' status. */
int ace_sync(ace_ctx *ctx);

/* sizes[0..3] = nA, nAA, nB, maxord */
int ace_get_spec_sizes(const ace_ctx *ctx, int64_t *sizes);

/* Last error message of this context (or of the calling thread's last failed create when ctx
   is NULL). */
const char *ace_last_error_string(const ace_ctx *ctx);

/* Number of kernel launches this context has issued (for accounting). */
int64_t ace_launch_count(const ace_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif /* ACE_B200_H */
