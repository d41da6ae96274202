// ace_ctx.h -- the evaluation context behind the opaque ace_ctx handle.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#define ACE_MAX_NR 32
#define ACE_MAX_L 20
#define ACE_MAX_ORD 6

// device status word bits (set by kernels, read back by the host)
#define ACE_STATUS_BAD_OFFSETS 1
#define ACE_STATUS_BAD_SPECIES 2
#define ACE_STATUS_BAD_POSITION 4
#define ACE_STATUS_SCRATCH 8
#define ACE_STATUS_TIMEOUT 16

struct ace_ctx {
  int device = 0, prec = 0, nsm = 0, smem_optin = 0;
  int nR = 0, L = 0, nA = 0, maxord = 0, nspecies = 1, ntab = 0;
  int pl = 0, pr = 0, tp = 0;
  double tl = 0, tr = 0, r0 = 0;
  int64_t nAA = 0, nB = 0;
  bool has_const = false;

  // device copies of the spec
  double *d_tabD = nullptr;   // coefficient tables (table_size entries) in double,
  float *d_tabF = nullptr;    // float,
  float *d_tabDF = nullptr;   // and double-float pairs
  int16_t *d_an = nullptr, *d_aiy = nullptr, *d_amu = nullptr;
  uint8_t *d_ord = nullptr;
  uint16_t *d_idx = nullptr;  // [maxord][nAA], flat products (basis path)
  int64_t *d_Uptr = nullptr;
  int32_t *d_Uidx = nullptr;
  double *d_UvalD = nullptr;
  float *d_UvalF = nullptr;
  int *d_status = nullptr;
  int *h_status = nullptr;

  // correlation schedule (ace_sched.h)
  int64_t sn = 0;
  bool halved = false;
  int64_t sched_nodes = 0;
  int64_t slen = 0;            // interleaved slots per thread
  uint4 *d_srec = nullptr;     // [slen * nt] packed records (ace_sched.h)
  void *d_sc = nullptr;        // [slen * nt] coefficients w * c~ in the energy type
  std::vector<int64_t> sslot;  // slot -> AA index (-1: empty slot)
  std::vector<uint8_t> sw;     // slot -> weight
  // item schedule (ace_sched.h build_items)
  bool use_items = true;
  // task schedule (ace_sched.h build_tasks; orders >= 3): the default
  // correlation walk of single-property energy/force calls
  bool has_tasks = false, use_tasks = false;
  bool task_high = false;      // the high-occupancy instantiation of the task kernels
  int64_t trows = 0;
  int32_t twrow[5] = {0, 0, 0, 0, 0};
  uint4 *d_trec = nullptr;
  void *d_tc = nullptr;        // [rows * (G+1) * 32] coefficients in the energy type
  float *d_tc32 = nullptr;     // the same in FP32 (compensated form)
  std::vector<int64_t> tk;     // AA index of each task-schedule coefficient (-1: none)
  std::vector<uint8_t> tw;     // weights
  // compensated form (ACE_PREC_FP32_COMP): prec is ACE_PREC_FP32X2 for every
  // other path; the single-property item kernel reads FP32 coefficients d_ic32
  bool comp = false;
  float *d_ic32 = nullptr;     // [(G+1) * item_n] coefficients in FP32
  // its error control (ace_set_energy_tolerance, ace_guard.cu): the kernels
  // write each environment's rounding scale to d_gest (offset guard_off
  // within the call, for the chunks of the host-buffer pipeline); the
  // environments over the tolerance are listed in d_glist and evaluated
  // again by the double-float kernel; d_gsum holds a launch's sum of E^2
  // and list length, d_gtotal the re-evaluations since creation
  double guard_tol = 0.0;
  float *d_gest = nullptr;
  int64_t *d_glist = nullptr;
  int64_t guard_cap = 0, guard_off = 0, guard_last = 0;
  double guard_kappa_last = 0.0;  // the factor of the last call's estimates
  void *d_gsum = nullptr;
  unsigned long long *d_gtotal = nullptr;
  int64_t item_n = 0;
  uint4 *d_irec = nullptr;
  void *d_ic = nullptr;        // [(G+1) * item_n] coefficients in the energy type
  std::vector<int64_t> ik;     // [(G+1) * item_n] AA index (-1: none)
  std::vector<uint8_t> iw;     // weights
  // multi-property coefficient sets (property-major); cplx: complex c~
  // (EuclideanVector components), item coefficients in two planes
  bool cplx = false;
  std::vector<int64_t> apartner;   // AA partner (halved schedules)
  std::vector<int8_t> amsign;      // (-1)^{sum m} of each AA function
  int nprop = 0;
  std::vector<double> ctilde_multi;   // [nprop * nAA]
  void *d_ic_multi = nullptr;         // [nprop * (G+1) * item_n] in the energy type

  // host copies
  std::vector<double> ctilde;
  std::vector<int64_t> U_indptr;
  std::vector<int32_t> U_indices;
  std::vector<double> U_data;

  // staging and scratch (grown on demand, owned by the context)
  void *d_stage = nullptr;
  size_t stage_bytes = 0;
  void *d_scratch = nullptr;
  size_t scratch_bytes = 0;
  void *d_wstage = nullptr;
  size_t wstage_bytes = 0;

  // launch configuration chosen at create time (and by ace_autotune)
  int region_kb = 40;          // shared region for neighbour slabs / private adjoint bins
  int nt = 128, chunkE = 32, chunkG = 16, npriv = 32, grid = 0;
  int grid_df[2] = {0, 0};     // compensated context: its double-float kernels' grids (energy, E+F)
  size_t smem = 0, smem_comp = 0;
  int aa_chunk = 32, aa_grid = 0;
  size_t aa_smem = 0;
  // fused symmetric basis (ace_sched.h build_urows); false: AA materialised
  bool fused_basis = true;
  int64_t ulen = 0;
  uint4 *d_urec = nullptr;
  void *d_uval = nullptr;      // U values in the energy type, slot order
  int ub_chunk = 8, ub_grid = 0;
  size_t ub_smem = 0;

  // learned radial form (ace_set_radial_mlp): the spec's radial index n is a
  // channel k < K of an MLP (transform features, species one-hot) -> K (L+1)
  // outputs; A entry (n, l, m) reads channel n + K l
  bool learned = false;
  int mlpK = 0, mlpQ = 0, mlpS = 0, mlpH = 0, mlpC = 0, mlpD = 0;
  int64_t mlp_np = 0;
  double mlp_tmax = 0;
  float *d_mlp = nullptr;       // parameters [W1 b1 W2 b2 W3 b3]
  float *d_Rext = nullptr;      // [nNbr][2 C] radial values and r-derivatives
  int64_t rext_cap = 0;         // neighbours d_Rext can hold
  int mlp_grid_f = 0, mlp_grid_b = 0, mlp_grid_tc = 0;
  bool mlp_tc = false;          // tensor-core (BF16) inference of the radial MLP
  size_t mlp_smem_f = 0, mlp_smem_b = 0;
  int64_t tc_wait_limit = int64_t(1) << 26;  // polls of an MMA completion before giving up

  // host-buffer pipeline (copy in, compute, copy out)
  cudaStream_t s_in = nullptr, s_comp = nullptr, s_out = nullptr;
  std::vector<cudaEvent_t> pipe_ev;

  // ace_basis_noalloc: device address of the static scratch array, looked up
  // at context creation (noalloc_rc != 0: the look-up failed, noalloc_err why)
  void *noalloc_scratch = nullptr;
  int noalloc_rc = 0;
  std::string noalloc_err;

  std::vector<void *> allocs;
  int64_t launches = 0;
  std::string err;
};

namespace ace {
int kernels_prepare(ace_ctx *ctx);
int launch_energy_forces(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr,
                         const int32_t *sp, double *E, double *G, cudaStream_t st,
                         const void *ic = nullptr, double c0 = 0.0, bool cpx = false);
// complex-coefficient (item schedule) energy/force kernels (ace_launch_cplx.cu)
void *ef_func_cplx(const ace_ctx *ctx, bool grad);
// compensated-form energy/force kernels (ace_launch_comp.cu)
void *ef_func_comp(const ace_ctx *ctx);
// task-schedule energy/force kernels (ace_launch_tasks.cu); _df: the
// double-float kernel also in a compensated context (its re-evaluations)
void *ef_func_tasks(const ace_ctx *ctx, bool grad);
void *ef_func_tasks_df(const ace_ctx *ctx, bool grad);
// error control of the compensated form (ace_guard.cu): guard_prepare grows
// the estimate and list arrays to n environments; guard_flag lists the
// launch's environments whose estimate est[0 .. nEnv) is over the tolerance
// (their number at guard_count, on the device)
int guard_prepare(ace_ctx *ctx, int64_t n);
double guard_kappa(const ace_ctx *ctx);
int guard_flag(ace_ctx *ctx, int64_t nEnv, const double *E, const float *est, cudaStream_t st);
const int32_t *guard_count(const ace_ctx *ctx);
int launch_basis(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr,
                 const int32_t *sp, double *B, double *dB, cudaStream_t st);
int launch_dbasis(ace_ctx *ctx, int64_t nEnv, const int64_t *off_d, const int64_t *off_h, const double *rr,
                  const int32_t *sp, double *dB, cudaStream_t st);
// learned radial form (ace_mlp.cu)
int mlp_prepare(ace_ctx *ctx);
int mlp_forward(ace_ctx *ctx, int64_t nEnv, const int64_t *off, int64_t nNbr, const double *rr, const int32_t *sp,
                float *R, cudaStream_t st);
int mlp_infer(ace_ctx *ctx, int64_t nEnv, const int64_t *off, int64_t nNbr, const double *rr, const int32_t *sp,
              float *R, cudaStream_t st);
// radial channels of the batch into the context's buffer; infer = false keeps
// the FP32 MLP (training), true allows the tensor-core inference kernel
int learned_radials(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr, const int32_t *sp,
                    cudaStream_t st, bool infer = true);
int launch_radial_adjoint(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr, const int32_t *sp,
                          double *E, double *G, float *GR, cudaStream_t st);
// ace_noalloc.cu: the static scratch's device address for this context's
// device (called by ace_ctx_create; the outcome is kept in the context)
int noalloc_prepare(ace_ctx *ctx);
int launch_adjoint_eval_d(ace_ctx *ctx, int64_t nEnv, const int64_t *off_d, const int64_t *off_h,
                          const double *rr, const int32_t *sp, const double *w, double *out, cudaStream_t st);
}  // namespace ace
