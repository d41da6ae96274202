// ace_launch_cplx.cu -- the complex-coefficient energy/force kernels (item
// schedule), in their own translation unit so they compile in parallel with
// the real-coefficient ones.
#include <cuda_runtime.h>

#include "../../include/ace_b200.h"
#include "ace_ctx.h"
#include "ace_kernels.cuh"

namespace ace {

static constexpr int NTC = 128;

template <typename TE, typename TG, bool GRAD>
static void *cf_k(int K) {
  switch (K) {
    case 1:
    case 2: return (void *)ef_kernel<TE, TG, 2, NTC, GRAD, true, true>;
    case 3: return (void *)ef_kernel<TE, TG, 3, NTC, GRAD, true, true>;
    case 4: return (void *)ef_kernel<TE, TG, 4, NTC, GRAD, true, true>;
    case 5: return (void *)ef_kernel<TE, TG, 5, NTC, GRAD, true, true>;
    default: return (void *)ef_kernel<TE, TG, 6, NTC, GRAD, true, true>;
  }
}

void *ef_func_cplx(const ace_ctx *ctx, bool grad) {
  switch (ctx->prec) {
    case ACE_PREC_FP64: return grad ? cf_k<double, double, true>(ctx->maxord) : cf_k<double, double, false>(ctx->maxord);
    case ACE_PREC_FP32X2: return grad ? cf_k<df, float, true>(ctx->maxord) : cf_k<df, float, false>(ctx->maxord);
    default: return grad ? cf_k<float, float, true>(ctx->maxord) : cf_k<float, float, false>(ctx->maxord);
  }
}

}  // namespace ace
