// ace_ctx.h -- the evaluation context behind the opaque ace_ctx handle.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#define ACE_MAX_NR 32
#define ACE_MAX_L 20
#define ACE_MAX_ORD 8

// device status word bits (set by kernels, read back by the host)
#define ACE_STATUS_BAD_OFFSETS 1
#define ACE_STATUS_BAD_SPECIES 2
#define ACE_STATUS_BAD_POSITION 4
#define ACE_STATUS_SCRATCH 8

struct ace_ctx {
  int device = 0, prec = 0, nsm = 0, smem_optin = 0;
  int nR = 0, L = 0, nA = 0, maxord = 0, nspecies = 1, ntab = 0;
  int pl = 0, pr = 0, tp = 0;
  double tl = 0, tr = 0, r0 = 0;
  int64_t nAA = 0, nB = 0;
  bool has_const = false;

  // device copies of the spec
  double *d_tabD = nullptr;   // rA rB rC alpA alpB
  float *d_tabF = nullptr;
  int16_t *d_an = nullptr, *d_aiy = nullptr, *d_amu = nullptr;
  uint8_t *d_ord = nullptr;
  uint16_t *d_idx = nullptr;  // [maxord][nAA]
  double *d_ctD = nullptr;
  float *d_ctF = nullptr;
  int64_t *d_Uptr = nullptr;
  int32_t *d_Uidx = nullptr;
  double *d_UvalD = nullptr;
  float *d_UvalF = nullptr;
  int *d_status = nullptr;
  int *h_status = nullptr;

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

  // launch configuration chosen at create time
  int ef_block = 256, ef_chunk = 32, ef_grid = 0;
  size_t ef_smem = 0;

  std::vector<void *> allocs;
  int64_t launches = 0;
  std::string err;
};

namespace ace {
int kernels_prepare(ace_ctx *ctx);
int launch_energy_forces(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr,
                         const int32_t *sp, double *E, double *G, cudaStream_t st);
int launch_basis(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr,
                 const int32_t *sp, double *B, double *dB, cudaStream_t st);
}  // namespace ace
