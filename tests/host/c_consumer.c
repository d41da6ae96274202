/* A plain C99 consumer of the C ABI (include/ace_b200.h): builds a one-entry
   spec bundle and calls every entry point's signature through function
   pointers, so that the header compiles as C without any C++ or CUDA types.
   Compiled (not run) by tests/test_abi.py. */
#include <stddef.h>
#include <stdint.h>

#include "ace_b200.h"

typedef int (*ef_fn)(ace_ctx *, int64_t, const int64_t *, const double *, const int32_t *, double *, double *,
                     int32_t, void *);
typedef void (*any_fn)(void);

int main(void) {
  const double rA[1] = {1.0}, rB[1] = {0.0}, rC[1] = {0.0};
  const int32_t an[1] = {0}, al[1] = {0}, am[1] = {0};
  const int32_t orders[1] = {1}, iAA2iA[1] = {0};
  const int64_t Uptr[2] = {0, 1};
  const int32_t Uidx[1] = {0};
  const double Uval[1] = {1.0};
  ace_spec_bundle b;
  b.version = ACE_SPEC_VERSION;
  b.nR = 1; b.rA = rA; b.rB = rB; b.rC = rC; b.pl = 2; b.pr = 0; b.tl = 0.1; b.tr = 4.0; b.tp = 2; b.r0 = 1.0;
  b.nA = 1; b.a_n = an; b.a_l = al; b.a_m = am; b.a_mu = NULL; b.nspecies = 1;
  b.nAA = 1; b.maxord = 1; b.orders = orders; b.iAA2iA = iAA2iA;
  b.nB = 1; b.U_indptr = Uptr; b.U_indices = Uidx; b.U_data = Uval;
  ef_fn ef = ace_energy_forces;
  ace_radial_mlp m;
  m.version = 1; m.K = 1; m.Q = 1; m.nspecies = 1; m.H = 64; m.tmax = 4.0; m.params = NULL; m.nparams = 0;
  any_fn fns[] = {(any_fn)ace_ctx_create, (any_fn)ace_ctx_destroy, (any_fn)ace_set_params, (any_fn)ace_set_ctilde,
                 (any_fn)ace_set_params_multi, (any_fn)ace_set_ctilde_complex, (any_fn)ace_energy_forces_multi,
                 (any_fn)ace_energy, (any_fn)ace_basis, (any_fn)ace_adjoint_eval_d, (any_fn)ace_basis_noalloc,
                 (any_fn)ace_autotune, (any_fn)ace_set_radial_mlp, (any_fn)ace_radial_mlp_params,
                 (any_fn)ace_radial_mlp_get_params, (any_fn)ace_radial_mlp_forward, (any_fn)ace_radial_mlp_infer,
                 (any_fn)ace_radial_mlp_backward, (any_fn)ace_energy_radial_adjoint, (any_fn)ace_adam_step,
                 (any_fn)ace_sync, (any_fn)ace_get_spec_sizes, (any_fn)ace_last_error_string,
                 (any_fn)ace_launch_count};
  (void)b; (void)m; (void)ef;
  return (int)(sizeof(fns) / sizeof(fns[0])) == 24 ? 0 : 1;
}
