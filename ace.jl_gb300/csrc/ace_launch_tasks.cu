// ace_launch_tasks.cu -- the energy/force kernels on the task schedule
// (ace_sched.h build_tasks), orders 3-6, in their own translation unit so
// they compile in parallel with the others.
#include <cuda_runtime.h>

#include "../../include/ace_b200.h"
#include "ace_ctx.h"
#include "ace_kernels.cuh"

namespace ace {

static constexpr int NTT = 128;

template <typename TE, typename TG, bool GRAD, bool COMP>
static void *tk_k(int K) {
  switch (K) {
    case 3: return (void *)ef_kernel<TE, TG, 3, NTT, GRAD, true, false, COMP, true>;
    case 4: return (void *)ef_kernel<TE, TG, 4, NTT, GRAD, true, false, COMP, true>;
    case 5: return (void *)ef_kernel<TE, TG, 5, NTT, GRAD, true, false, COMP, true>;
    default: return (void *)ef_kernel<TE, TG, 6, NTT, GRAD, true, false, COMP, true>;
  }
}

void *ef_func_tasks(const ace_ctx *ctx, bool grad) {
  if (ctx->comp) return tk_k<df, float, true, true>(ctx->maxord);
  switch (ctx->prec) {
    case ACE_PREC_FP64: return grad ? tk_k<double, double, true, false>(ctx->maxord)
                                    : tk_k<double, double, false, false>(ctx->maxord);
    case ACE_PREC_FP32X2: return grad ? tk_k<df, float, true, false>(ctx->maxord) : tk_k<df, float, false, false>(ctx->maxord);
    default: return grad ? tk_k<float, float, true, false>(ctx->maxord) : tk_k<float, float, false, false>(ctx->maxord);
  }
}

}  // namespace ace
