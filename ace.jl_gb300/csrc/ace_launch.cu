// ace_launch.cu -- launch configuration and dispatch of the evaluation kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "../../include/ace_b200.h"
#include "ace_ctx.h"
#include "ace_kernels.cuh"

namespace ace {

static constexpr int NT = 128;  // threads per CTA of the energy/forces kernel

template <typename TE, typename TG, bool GRAD, bool ITEMS>
static void *ef_func_k(int K) {
  switch (K) {
    case 1:
    case 2: return (void *)ef_kernel<TE, TG, 2, NT, GRAD, ITEMS>;
    case 3: return (void *)ef_kernel<TE, TG, 3, NT, GRAD, ITEMS>;
    case 4: return (void *)ef_kernel<TE, TG, 4, NT, GRAD, ITEMS>;
    case 5: return (void *)ef_kernel<TE, TG, 5, NT, GRAD, ITEMS>;
    default: return (void *)ef_kernel<TE, TG, 6, NT, GRAD, ITEMS>;
  }
}

template <typename TE, typename TG>
static void *ef_func_t(const ace_ctx *ctx, bool grad) {
  if (ctx->use_items) return grad ? ef_func_k<TE, TG, true, true>(ctx->maxord) : ef_func_k<TE, TG, false, true>(ctx->maxord);
  return grad ? ef_func_k<TE, TG, true, false>(ctx->maxord) : ef_func_k<TE, TG, false, false>(ctx->maxord);
}

static void *ef_func(const ace_ctx *ctx, bool grad) {
  switch (ctx->prec) {
    case ACE_PREC_FP64: return ef_func_t<double, double>(ctx, grad);
    case ACE_PREC_FP32X2: return ef_func_t<df, float>(ctx, grad);
    default: return ef_func_t<float, float>(ctx, grad);
  }
}

static void *aa_func(const ace_ctx *ctx) {
  switch (ctx->prec) {
    case ACE_PREC_FP64: return (void *)aa_kernel<double, double>;
    case ACE_PREC_FP32X2: return (void *)aa_kernel<df, double>;
    default: return (void *)aa_kernel<float, float>;
  }
}

static void *ub_func(const ace_ctx *ctx) {
  switch (ctx->prec) {
    case ACE_PREC_FP64: return (void *)ub_fused_kernel<double>;
    case ACE_PREC_FP32X2: return (void *)ub_fused_kernel<df>;
    default: return (void *)ub_fused_kernel<float>;
  }
}

// the compensated kernels replace the double-float item kernels for the
// single-property energy/force calls of a compensated context
static bool uses_comp(const ace_ctx *ctx) { return ctx->comp && ctx->use_items && !ctx->learned; }
// single-property energy/force calls walk the task schedule (orders >= 3)
static bool uses_tasks(const ace_ctx *ctx) { return ctx->has_tasks && ctx->use_tasks && !ctx->learned; }

// the kernel a context's single-property energy/force calls launch, its
// coefficient array and its shared-memory size
static void *ef_main(const ace_ctx *ctx, bool grad, const void **coef, size_t *smem) {
  const bool comp = uses_comp(ctx);
  *smem = comp ? ctx->smem_comp : ctx->smem;
  if (uses_tasks(ctx)) {
    *coef = comp ? (const void *)ctx->d_tc32 : ctx->d_tc;
    return ef_func_tasks(ctx, grad);
  }
  if (comp) {
    *coef = ctx->d_ic32;
    return ef_func_comp(ctx);
  }
  *coef = ctx->d_ic;
  return ef_func(ctx, grad);
}

static void type_sizes(const ace_ctx *ctx, int &sE, int &sG, bool &same) {
  switch (ctx->prec) {
    case ACE_PREC_FP64: sE = 8; sG = 8; same = true; break;
    case ACE_PREC_FP32X2: sE = 8; sG = 4; same = false; break;
    default: sE = 4; sG = 4; same = true; break;
  }
}

// The maximum dynamic shared memory of a kernel is a process-wide attribute
// of the function, shared by every context: it is set to the device's
// opt-in limit (never lowered by a context with a smaller spec); each launch
// passes its own size, and the occupancy queries use the context's size.
int kernels_prepare(ace_ctx *ctx) {
  int sE, sG;
  bool same;
  type_sizes(ctx, sE, sG, same);
  ctx->nt = NT;
  // one region (ctx->region_kb) holds the neighbour slabs (phases 1, 3) or the
  // private adjoint bins (phase 2); smaller regions raise occupancy
  const int region = ctx->region_kb * 1024;
  // column-parallel 1p basis: (L+1) threads per neighbour
  const int nRs = ctx->learned ? ctx->mlpC : ctx->nR;
  const bool radj = ctx->learned;
  const int slabE = (nRs + 2 * size_y(ctx->L)) * sE;
  const int slabG = (2 * nRs + 8 * size_y(ctx->L) + (radj ? nRs : 0)) * sG;
  const int lanes = NT / (ctx->L + 1);
  ctx->chunkE = std::max(1, std::min(lanes, region / slabE));
  ctx->chunkG = std::max(1, std::min(lanes, region / slabG));
  ctx->npriv = std::max(1, std::min(ctx->nA, region / (NT * 2 * sG)));
  EFLayout lay = ef_layout(ctx->ntab, nRs, ctx->L, ctx->nA, ctx->chunkE, ctx->chunkG, ctx->npriv, NT, sE, sG, same,
                           radj);
  while (lay.total > (size_t)ctx->smem_optin && (ctx->chunkE > 1 || ctx->chunkG > 1 || ctx->npriv > 1)) {
    ctx->chunkE = std::max(1, ctx->chunkE / 2);
    ctx->chunkG = std::max(1, ctx->chunkG / 2);
    ctx->npriv = std::max(1, ctx->npriv / 2);
    lay = ef_layout(ctx->ntab, nRs, ctx->L, ctx->nA, ctx->chunkE, ctx->chunkG, ctx->npriv, NT, sE, sG, same, radj);
  }
  if (lay.total > (size_t)ctx->smem_optin) {
    ctx->err = "spec too large for shared memory";
    return ACE_ERR_UNSUPPORTED;
  }
  ctx->smem = lay.total;
  // the compensated kernel's A_hi / A_lo arrays take the place of the
  // double-float A and its FP32 copy: a smaller layout of its own
  ctx->smem_comp = ef_layout(ctx->ntab, nRs, ctx->L, ctx->nA, ctx->chunkE, ctx->chunkG, ctx->npriv, NT, sE, sG, same,
                             radj, true).total;
  int occ = 1;
  std::vector<void *> fs = {ef_func(ctx, false), ef_func(ctx, true)};
  if (uses_comp(ctx)) fs.push_back(ef_func_comp(ctx));
  if (ctx->has_tasks) { fs.push_back(ef_func_tasks(ctx, false)); fs.push_back(ef_func_tasks(ctx, true)); }
  // (a compensated context's re-evaluations: the double-float task kernels)
  if (ctx->comp && ctx->has_tasks) { fs.push_back(ef_func_tasks_df(ctx, false)); fs.push_back(ef_func_tasks_df(ctx, true)); }
  for (void *f : fs)
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->smem_optin) != cudaSuccess) {
      ctx->err = "cudaFuncSetAttribute failed";
      return ACE_ERR_CUDA;
    }
  {
    // the grid follows the occupancy of the kernel the context's E+F calls run
    const void *coef;
    size_t sm;
    void *f = ef_main(ctx, true, &coef, &sm);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, f, NT, sm);
  }
  ctx->grid = ctx->nsm * std::max(occ, 1);
  // a compensated context's double-float launches (energies only, and the
  // re-evaluations) have their own occupancy: a grid of more CTAs than can
  // be resident would run its last CTAs' environments in a second wave
  if (ctx->comp) {
    for (int g = 0; g < 2; ++g) {
      void *f = uses_tasks(ctx) ? ef_func_tasks_df(ctx, g == 1) : ef_func_t<df, float>(ctx, g == 1);
      int o = 1;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, f, NT, ctx->smem);
      ctx->grid_df[g] = ctx->nsm * std::max(o, 1);
    }
  }
  // basis path (AA materialisation)
  ctx->aa_chunk = std::max(1, std::min(256 / (ctx->L + 1), (32 * 1024) / slabE));
  EFLayout la = ef_layout(ctx->ntab, nRs, ctx->L, ctx->nA, ctx->aa_chunk, 1, 0, 256, sE, sE, true);
  ctx->aa_smem = la.total;
  void *fa = aa_func(ctx);
  if (cudaFuncSetAttribute(fa, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->smem_optin) != cudaSuccess) {
    ctx->err = "cudaFuncSetAttribute failed";
    return ACE_ERR_CUDA;
  }
  int occa = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occa, fa, 256, la.total);
  ctx->aa_grid = ctx->nsm * std::max(occa, 1);
  // fused basis: 128 threads, neighbour slabs within 16 KB
  ctx->ub_chunk = std::max(1, std::min(128 / (ctx->L + 1), (16 * 1024) / slabE));
  EFLayout lu = ef_layout(ctx->ntab, nRs, ctx->L, ctx->nA, ctx->ub_chunk, 1, 0, 128, sE, sE, true);
  ctx->ub_smem = lu.total;
  void *fu = ub_func(ctx);
  if (cudaFuncSetAttribute(fu, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->smem_optin) != cudaSuccess) {
    ctx->err = "cudaFuncSetAttribute failed";
    return ACE_ERR_CUDA;
  }
  int occu = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occu, fu, 128, lu.total);
  ctx->ub_grid = ctx->nsm * std::max(occu, 1);
  return ACE_OK;
}

int launch_energy_forces(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr, const int32_t *sp,
                         double *E, double *G, cudaStream_t st, const void *ic, double c0, bool cpx) {
  if (nEnv == 0) return ACE_OK;
  if (ctx->learned) {
    int rc = learned_radials(ctx, nEnv, off, rr, sp, st);
    if (rc) return rc;
  }
  EFArgs a = make_args(ctx, nEnv, off, rr, sp, E, G);
  if (ic) { a.ic = ic; a.c0 = c0; }
  void *f = ef_func(ctx, G != nullptr);
  size_t smem = ctx->smem;
  // energies only in a compensated context: the double-float energy kernel,
  // which needs no adjoint (the compensated energy's correction does), is
  // faster there and exact to ~1e-12
  const bool comp_eonly = !ic && !cpx && uses_comp(ctx) && G == nullptr;
  if (comp_eonly) {
    if (uses_tasks(ctx)) {
      f = ef_func_tasks_df(ctx, false);
      a.tc = ctx->d_tc;
    } else {
      f = ef_func_t<df, float>(ctx, false);
      a.ic = ctx->d_ic;
    }
    ctx->guard_last = 0;  // (no estimates)
  } else if (!ic && !cpx) {
    // the single-property kernel: task schedule, compensated form or item runs
    const void *coef;
    f = ef_main(ctx, G != nullptr, &coef, &smem);
    if (uses_tasks(ctx)) a.tc = coef;
    else a.ic = coef;
  }
  if (cpx) {
    f = ef_func_cplx(ctx, G != nullptr);
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->smem_optin) != cudaSuccess) {
      ctx->err = "cudaFuncSetAttribute failed";
      return ACE_ERR_CUDA;
    }
  }
  // the compensated form estimates each environment's rounding error
  // (ace_guard.cu) and, with a tolerance set, evaluates the environments
  // over it again in double-float
  const bool guard = !ic && !cpx && uses_comp(ctx) && !comp_eonly;
  if (guard) {
    int rc = guard_prepare(ctx, ctx->guard_off + nEnv);
    if (rc) return rc;
    a.est = ctx->d_gest + ctx->guard_off;
    ctx->guard_last = ctx->guard_off + nEnv;
    ctx->guard_kappa_last = guard_kappa(ctx);
  }
  const int grid = (int)std::min<int64_t>(nEnv, comp_eonly ? ctx->grid_df[0] : ctx->grid);
  void *args[] = {&a};
  cudaError_t e = cudaLaunchKernel(f, dim3(grid), dim3(NT), args, smem, st);
  ctx->launches += 1;
  if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); return ACE_ERR_CUDA; }
  if (guard && ctx->guard_tol > 0.0) {
    int rc = guard_flag(ctx, nEnv, E, a.est, st);
    if (rc) return rc;
    EFArgs b = make_args(ctx, nEnv, off, rr, sp, E, G);
    b.elist = ctx->d_glist;
    b.ecount = guard_count(ctx);
    // (the schedule the context was tuned to)
    void *g;
    if (uses_tasks(ctx)) {
      g = ef_func_tasks_df(ctx, G != nullptr);
      b.tc = ctx->d_tc;
    } else {
      g = ef_func_t<df, float>(ctx, G != nullptr);
      b.ic = ctx->d_ic;
    }
    void *bargs[] = {&b};
    const int gridb = (int)std::min<int64_t>(nEnv, ctx->grid_df[G != nullptr ? 1 : 0]);
    e = cudaLaunchKernel(g, dim3(gridb), dim3(NT), bargs, ctx->smem, st);
    ctx->launches += 1;
    if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); return ACE_ERR_CUDA; }
  }
  return ACE_OK;
}

static int ensure_scratch(ace_ctx *ctx, size_t bytes) {
  if (bytes <= ctx->scratch_bytes) return ACE_OK;
  if (ctx->d_scratch) { cudaFree(ctx->d_scratch); ctx->d_scratch = nullptr; ctx->scratch_bytes = 0; }
  if (cudaMalloc(&ctx->d_scratch, bytes) != cudaSuccess) { ctx->err = "scratch allocation failed"; return ACE_ERR_ALLOC; }
  ctx->scratch_bytes = bytes;
  return ACE_OK;
}

int launch_radial_adjoint(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr, const int32_t *sp,
                          double *E, double *G, float *GR, cudaStream_t st) {
  if (nEnv == 0) return ACE_OK;
  int rc = learned_radials(ctx, nEnv, off, rr, sp, st, false);
  if (rc) return rc;
  EFArgs a = make_args(ctx, nEnv, off, rr, sp, E, G);
  a.GR = GR;
  void *f = ef_func(ctx, true);
  const int grid = (int)std::min<int64_t>(nEnv, ctx->grid);
  void *args[] = {&a};
  cudaError_t e = cudaLaunchKernel(f, dim3(grid), dim3(NT), args, ctx->smem, st);
  ctx->launches += 1;
  if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); return ACE_ERR_CUDA; }
  return ACE_OK;
}

int launch_basis(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr, const int32_t *sp,
                 double *B, double *dB, cudaStream_t st) {
  (void)dB;  // the derivative is produced by launch_dbasis
  if (nEnv == 0) return ACE_OK;
  if (ctx->learned) {
    int rc = learned_radials(ctx, nEnv, off, rr, sp, st);
    if (rc) return rc;
  }
  if (ctx->fused_basis) {
    EFArgs a = make_args(ctx, nEnv, off, rr, sp, nullptr, nullptr);
    a.chunkE = ctx->ub_chunk;
    const uint4 *urec = ctx->d_urec;
    const void *uval = ctx->d_uval;
    int64_t ulen = ctx->ulen, nB = ctx->nB;
    const int grid = (int)std::min<int64_t>(nEnv, ctx->ub_grid);
    void *args[] = {&a, &urec, &uval, &ulen, &nB, &B};
    cudaError_t e = cudaLaunchKernel(ub_func(ctx), dim3(grid), dim3(128), args, ctx->ub_smem, st);
    ctx->launches += 1;
    if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); return ACE_ERR_CUDA; }
    return ACE_OK;
  }
  const bool f32 = (ctx->prec == ACE_PREC_FP32 || ctx->prec == ACE_PREC_FP32_BF16X3);
  const size_t ts = f32 ? 4 : 8;
  int64_t per = std::max<int64_t>(1, (int64_t)((512ull << 20) / (ctx->nAA * ts)));
  per = std::min<int64_t>(per, nEnv);
  int rc = ensure_scratch(ctx, (size_t)per * ctx->nAA * ts);
  if (rc) return rc;
  void *fa = aa_func(ctx);
  for (int64_t e0 = 0; e0 < nEnv; e0 += per) {
    const int64_t ne = std::min(per, nEnv - e0);
    EFArgs a = make_args(ctx, ne, off + e0, rr, sp, nullptr, nullptr);
    a.chunkE = ctx->aa_chunk;
    a.AAout = ctx->d_scratch;
    a.ldE = ne;
    const int grid = (int)std::min<int64_t>(ne, ctx->aa_grid);
    void *args[] = {&a};
    cudaError_t err = cudaLaunchKernel(fa, dim3(grid), dim3(256), args, ctx->aa_smem, st);
    ctx->launches += 1;
    if (err != cudaSuccess) { ctx->err = cudaGetErrorString(err); return ACE_ERR_CUDA; }
    dim3 g2((unsigned)((ne + 127) / 128), (unsigned)std::min<int64_t>(ctx->nB, 65535));
    if (!f32)
      ub_kernel<double><<<g2, 128, 0, st>>>(ne, e0, ne, ctx->nB, ctx->d_Uptr, ctx->d_Uidx, ctx->d_UvalD,
                                             (const double *)ctx->d_scratch, B);
    else
      ub_kernel<float><<<g2, 128, 0, st>>>(ne, e0, ne, ctx->nB, ctx->d_Uptr, ctx->d_Uidx, ctx->d_UvalF,
                                            (const float *)ctx->d_scratch, B);
    ctx->launches += 1;
    err = cudaGetLastError();
    if (err != cudaSuccess) { ctx->err = cudaGetErrorString(err); return ACE_ERR_CUDA; }
  }
  return ACE_OK;
}

}  // namespace ace
