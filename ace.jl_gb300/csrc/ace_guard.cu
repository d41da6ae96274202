// ace_guard.cu -- error control of the compensated form (ACE_PREC_FP32_COMP).
//
// The compensated kernels evaluate the correlation products in FP32 and
// write, per environment, the rounding scale s_e = sqrt(sum_g S_g^2) 2^-24,
// S_g the summed magnitude of the products that share a rounding (a task of
// the task schedule, an item of the item runs).  Their energy error is a sum
// of many independent roundings, so it is a small multiple of s_e: on the
// order-5 / degree-16 and order-4 bases, measured against FP64, at most 3.9
// s_e (task schedule) and 5.5 s_e (item runs).  After a launch, three more
// launches on the same stream
//   guard_sq_kernel    sum of E^2 over the launch (for its rms)
//   guard_flag_kernel  list the environments with kappa s_e > tol max(|E|, rms)
//   ef_kernel<df, ...> evaluate the listed environments again in
//                      double-float (energy error ~1e-12), overwriting E, G
// keep every environment's energy error under the tolerance without a host
// synchronisation (the call stays asynchronous and capturable).  The third
// launch is issued by launch_energy_forces (ace_launch.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/ace_b200.h"
#include "ace_ctx.h"
#include "ace_kernels.cuh"

namespace ace {

// est_e = kappa s_e, the bound the tolerance is compared with: measured on
// 100,000 environments of each of the order-5 / degree-16, order-4 /
// degree-12 and 4-species order-4 / degree-10 bases (and 4,000 at degree
// 14) against FP64, the error is at most 3.9 s_e on the task schedule and
// 5.5 s_e on the item runs (whose groups leave out the path products shared
// along a run); kappa keeps a margin of about 30 % over both
double guard_kappa(const ace_ctx *ctx) { return ctx->use_tasks && ctx->has_tasks ? 5.0 : 7.0; }

struct GuardSum {
  double sq;      // sum of E^2 over the launch's finite energies
  int32_t count;  // environments listed for re-evaluation
  int32_t pad;
};

__global__ void __launch_bounds__(256) guard_sq_kernel(const double *E, int64_t n, GuardSum *gs) {
  __shared__ double red[8];
  double s = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const double v = E[e];
    if (isfinite(v)) s += v * v;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    atomicAdd(&gs->sq, t);
  }
}

__global__ void __launch_bounds__(256) guard_flag_kernel(const double *E, const float *est, int64_t n, GuardSum *gs,
                                                         double kappa_over_tol, int64_t *list,
                                                         unsigned long long *total) {
  const double rms = sqrt(gs->sq / (double)(n > 0 ? n : 1));
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const double v = E[e];
    if (!isfinite(v)) continue;  // a rejected environment (status word) stays NaN
    if ((double)est[e] * kappa_over_tol > fmax(fabs(v), rms)) {
      list[atomicAdd(&gs->count, 1)] = e;
      atomicAdd(total, 1ull);
    }
  }
}

int guard_prepare(ace_ctx *ctx, int64_t n) {
  if (!ctx->d_gsum) {
    if (cudaMalloc(&ctx->d_gsum, sizeof(GuardSum)) != cudaSuccess ||
        cudaMalloc((void **)&ctx->d_gtotal, sizeof(unsigned long long)) != cudaSuccess) {
      ctx->err = "error-control allocation failed";
      return ACE_ERR_ALLOC;
    }
    ctx->allocs.push_back(ctx->d_gsum);
    ctx->allocs.push_back(ctx->d_gtotal);
    if (cudaMemset(ctx->d_gsum, 0, sizeof(GuardSum)) != cudaSuccess ||
        cudaMemset(ctx->d_gtotal, 0, sizeof(unsigned long long)) != cudaSuccess) {
      ctx->err = "cudaMemset failed";
      return ACE_ERR_CUDA;
    }
  }
  if (n <= ctx->guard_cap) return ACE_OK;
  if (ctx->d_gest) cudaFree(ctx->d_gest);
  if (ctx->d_glist) cudaFree(ctx->d_glist);
  ctx->d_gest = nullptr;
  ctx->d_glist = nullptr;
  ctx->guard_cap = 0;
  const int64_t cap = std::max<int64_t>(n, 1024);
  if (cudaMalloc((void **)&ctx->d_gest, cap * sizeof(float)) != cudaSuccess ||
      cudaMalloc((void **)&ctx->d_glist, cap * sizeof(int64_t)) != cudaSuccess) {
    ctx->err = "error-control allocation failed";
    return ACE_ERR_ALLOC;
  }
  ctx->guard_cap = cap;
  return ACE_OK;
}

int guard_flag(ace_ctx *ctx, int64_t nEnv, const double *E, const float *est, cudaStream_t st) {
  GuardSum *gs = (GuardSum *)ctx->d_gsum;
  cudaError_t ce = cudaMemsetAsync(gs, 0, sizeof(GuardSum), st);
  if (ce != cudaSuccess) { ctx->err = cudaGetErrorString(ce); return ACE_ERR_CUDA; }
  if (nEnv == 0) return ACE_OK;
  const int gb = (int)std::min<int64_t>((nEnv + 255) / 256, (int64_t)ctx->nsm * 8);
  guard_sq_kernel<<<gb, 256, 0, st>>>(E, nEnv, gs);
  guard_flag_kernel<<<gb, 256, 0, st>>>(E, est, nEnv, gs, guard_kappa(ctx) / ctx->guard_tol, ctx->d_glist,
                                        ctx->d_gtotal);
  ctx->launches += 2;
  ce = cudaGetLastError();
  if (ce != cudaSuccess) { ctx->err = cudaGetErrorString(ce); return ACE_ERR_CUDA; }
  return ACE_OK;
}

const int32_t *guard_count(const ace_ctx *ctx) { return &((const GuardSum *)ctx->d_gsum)->count; }

}  // namespace ace

using namespace ace;

extern "C" int ace_set_energy_tolerance(ace_ctx *ctx, double tol) {
  if (!ctx) return ACE_ERR_INVALID;
  if (!ctx->comp) {
    ctx->err = "energy tolerance: only the compensated form (ACE_PREC_FP32_COMP) estimates its error";
    return ACE_ERR_UNSUPPORTED;
  }
  if (!(tol >= 0.0) || std::isinf(tol)) {
    ctx->err = "energy tolerance must be finite and >= 0";
    return ACE_ERR_INVALID;
  }
  ctx->guard_tol = tol;
  return ACE_OK;
}

extern "C" int ace_energy_error_estimates(ace_ctx *ctx, int64_t nEnv, double *est, int64_t *refined) {
  if (!ctx) return ACE_ERR_INVALID;
  if (!ctx->comp) {
    ctx->err = "error estimates: only the compensated form (ACE_PREC_FP32_COMP) estimates its error";
    return ACE_ERR_UNSUPPORTED;
  }
  if (nEnv < 0 || (est && nEnv > ctx->guard_last)) {
    ctx->err = "error estimates: nEnv exceeds the last energy call's environments";
    return ACE_ERR_INVALID;
  }
  if (cudaSetDevice(ctx->device) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) {
    ctx->err = "cudaDeviceSynchronize failed";
    return ACE_ERR_CUDA;
  }
  if (est && nEnv > 0) {
    std::vector<float> s(nEnv);
    if (cudaMemcpy(s.data(), ctx->d_gest, nEnv * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess) {
      ctx->err = "cudaMemcpy failed";
      return ACE_ERR_CUDA;
    }
    for (int64_t e = 0; e < nEnv; ++e) est[e] = ctx->guard_kappa_last * (double)s[e];
  }
  if (refined) {
    unsigned long long t = 0;
    if (ctx->d_gtotal &&
        cudaMemcpy(&t, ctx->d_gtotal, sizeof(t), cudaMemcpyDeviceToHost) != cudaSuccess) {
      ctx->err = "cudaMemcpy failed";
      return ACE_ERR_CUDA;
    }
    *refined = (int64_t)t;
  }
  return ACE_OK;
}
