// ace_noalloc.cu -- ace_basis_noalloc: the symmetric-basis evaluation
// (B = U AA, as ace_basis computes it) without any device allocation.
//
// Why: some callers must not allocate device memory once they are running.
// A molecular-dynamics engine that reserves its device memory pool at
// start-up and forbids other libraries to call cudaMalloc afterwards, or a
// long-running service that keeps its memory footprint fixed, can create a
// context during set-up (which allocates) and then evaluate through this
// entry point, which allocates nothing: no cudaMalloc, no cudaFree, no
// staging buffers.  cudaMalloc also synchronises the device, which would stall
// the caller's other streams.
//
// How: ace_basis materialises real(AA) for a block of environments in a
// context-owned scratch buffer it grows with cudaMalloc.  Here that scratch is
// the file-scope array below, ACE_NOALLOC_SCRATCH_BYTES (16 MiB) of device
// memory that every GPU which loads this library holds until the process
// exits.  Its name is only a host-side handle: the device address is obtained
// once per device with cudaGetSymbolAddress (with that device current) and
// passed to the kernels.  ace_ctx_create performs this set-up (it allocates
// anyway), so that loading the module onto the device -- which takes device
// memory for the array and the code -- happens there and never inside
// ace_basis_noalloc.  A device reset (cudaDeviceReset) invalidates the saved
// address: the library must not be used across one.
//
// All calls share the array.  Each call overwrites every scratch element it
// reads before reading it, so nothing has to start at zero; calls that overlap
// on the GPU (on different streams, or from different contexts on the same
// device) race on the array and must be serialised by the caller.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/ace_b200.h"
#include "ace_ctx.h"
#include "ace_kernels.cuh"

#define ACE_NOALLOC_SCRATCH_BYTES (16u << 20)
#define ACE_NOALLOC_MAX_DEVICES 64

static __device__ __align__(256) unsigned char g_aa_scratch[ACE_NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_mu;
void *g_scratch_ptr[ACE_NOALLOC_MAX_DEVICES] = {};
bool g_ready[ACE_NOALLOC_MAX_DEVICES] = {};

int fail(ace_ctx *ctx, int code, const char *msg) {
  ctx->err = msg;
  return code;
}

}  // namespace

namespace ace {
// Called by ace_ctx_create with the context's device current: once per
// device, the scratch array's device address and the shared-memory opt-in of
// this file's kernel instances.  The result is kept in the context
// (noalloc_scratch, or noalloc_rc / noalloc_err when the set-up failed), so
// that ace_basis_noalloc itself makes no CUDA call that could load code.
int noalloc_prepare(ace_ctx *ctx) {
  std::lock_guard<std::mutex> lk(g_mu);
  const int dev = ctx->device;
  ctx->noalloc_scratch = nullptr;
  if (dev < 0 || dev >= ACE_NOALLOC_MAX_DEVICES) {
    ctx->noalloc_err = "device index too large for the static scratch table";
    return ctx->noalloc_rc = ACE_ERR_UNSUPPORTED;
  }
  if (!g_ready[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_aa_scratch);
    if (e != cudaSuccess) {
      ctx->noalloc_err = std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e);
      return ctx->noalloc_rc = ACE_ERR_CUDA;
    }
    const void *fns[] = {(const void *)ace::aa_kernel<double, double>, (const void *)ace::aa_kernel<ace::df, double>,
                         (const void *)ace::aa_kernel<float, float>};
    for (const void *f : fns) {
      e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->smem_optin);
      if (e != cudaSuccess) {
        ctx->noalloc_err = std::string("cudaFuncSetAttribute failed: ") + cudaGetErrorString(e);
        return ctx->noalloc_rc = ACE_ERR_CUDA;
      }
    }
    // load the code of the B = U AA kernels now (lazy module loading would
    // otherwise load it, taking device memory, at their first launch)
    const void *ub[] = {(const void *)ace::ub_kernel<double>, (const void *)ace::ub_kernel<float>};
    for (const void *f : ub) {
      cudaFuncAttributes fa;
      e = cudaFuncGetAttributes(&fa, f);
      if (e != cudaSuccess) {
        ctx->noalloc_err = std::string("cudaFuncGetAttributes failed: ") + cudaGetErrorString(e);
        return ctx->noalloc_rc = ACE_ERR_CUDA;
      }
    }
    g_scratch_ptr[dev] = p;
    g_ready[dev] = true;
  }
  ctx->noalloc_scratch = g_scratch_ptr[dev];
  return ctx->noalloc_rc = ACE_OK;
}
}  // namespace ace

extern "C" int ace_basis_noalloc(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                                 const int32_t *species, double *B, void *stream) {
  using namespace ace;
  if (!ctx) return ACE_ERR_INVALID;
  if (nEnv < 0 || !offsets || !rr || !B) return fail(ctx, ACE_ERR_INVALID, "NULL or negative argument");
  if (ctx->learned) return fail(ctx, ACE_ERR_UNSUPPORTED, "the learned radial form allocates its radial buffer");
  if (ctx->nB == 0) return fail(ctx, ACE_ERR_INVALID, "spec has no U");
  if (ctx->nspecies > 1 && !species) return fail(ctx, ACE_ERR_INVALID, "species required for a multi-species spec");
  const bool f32 = (ctx->prec == ACE_PREC_FP32 || ctx->prec == ACE_PREC_FP32_BF16X3);
  const size_t ts = f32 ? 4 : 8;
  const size_t per_env = (size_t)ctx->nAA * ts;
  if (per_env > ACE_NOALLOC_SCRATCH_BYTES)
    return fail(ctx, ACE_ERR_UNSUPPORTED,
                "ace_basis_noalloc: one environment's AA vector (nAA x element size) exceeds the 16 MiB "
                "static scratch; use ace_basis");
  if (ctx->noalloc_rc != ACE_OK || !ctx->noalloc_scratch) {
    ctx->err = "ace_basis_noalloc set-up failed at context creation: " + ctx->noalloc_err;
    return ctx->noalloc_rc != ACE_OK ? ctx->noalloc_rc : ACE_ERR_CUDA;
  }
  if (nEnv == 0) return ACE_OK;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, ACE_ERR_CUDA, "cudaSetDevice failed");
  void *scratch = ctx->noalloc_scratch;
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t per = std::min<int64_t>((int64_t)(ACE_NOALLOC_SCRATCH_BYTES / per_env), nEnv);
  void *fa = f32 ? (void *)aa_kernel<float, float>
                 : (ctx->prec == ACE_PREC_FP32X2 ? (void *)aa_kernel<df, double> : (void *)aa_kernel<double, double>);
  const int32_t *sp = ctx->nspecies > 1 ? species : nullptr;
  for (int64_t e0 = 0; e0 < nEnv; e0 += per) {
    const int64_t ne = std::min(per, nEnv - e0);
    EFArgs a = make_args(ctx, ne, offsets + e0, rr, sp, nullptr, nullptr);
    a.chunkE = ctx->aa_chunk;
    a.AAout = scratch;
    a.ldE = ne;
    const int grid = (int)std::min<int64_t>(ne, ctx->aa_grid);
    void *args[] = {&a};
    cudaError_t err = cudaLaunchKernel(fa, dim3(grid), dim3(256), args, ctx->aa_smem, st);
    ctx->launches += 1;
    if (err != cudaSuccess) return fail(ctx, ACE_ERR_CUDA, cudaGetErrorString(err));
    dim3 g2((unsigned)((ne + 127) / 128), (unsigned)std::min<int64_t>(ctx->nB, 65535));
    if (f32)
      ub_kernel<float><<<g2, 128, 0, st>>>(ne, e0, ne, ctx->nB, ctx->d_Uptr, ctx->d_Uidx, ctx->d_UvalF,
                                            (const float *)scratch, B);
    else
      ub_kernel<double><<<g2, 128, 0, st>>>(ne, e0, ne, ctx->nB, ctx->d_Uptr, ctx->d_Uidx, ctx->d_UvalD,
                                             (const double *)scratch, B);
    ctx->launches += 1;
    err = cudaGetLastError();
    if (err != cudaSuccess) return fail(ctx, ACE_ERR_CUDA, cudaGetErrorString(err));
  }
  return ACE_OK;
}
