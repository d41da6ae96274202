// ace_launch_tasks.cu -- the energy/force kernels on the task schedule
// (ace_sched.h build_tasks), orders 3-6, in their own translation unit so
// they compile in parallel with the others.
#include <cuda_runtime.h>

#include <type_traits>

#include "../../include/ace_b200.h"
#include "ace_ctx.h"
#include "ace_kernels.cuh"

namespace ace {

static constexpr int NTT = 128;

template <typename TE, typename TG, bool GRAD, bool COMP, int MINB>
static void *tk_k(int K) {
  switch (K) {
    case 3: return (void *)ef_kernel<TE, TG, 3, NTT, GRAD, true, false, COMP, true, MINB>;
    case 4: return (void *)ef_kernel<TE, TG, 4, NTT, GRAD, true, false, COMP, true, MINB>;
    case 5: return (void *)ef_kernel<TE, TG, 5, NTT, GRAD, true, false, COMP, true, MINB>;
    default: return (void *)ef_kernel<TE, TG, 6, NTT, GRAD, true, false, COMP, true, MINB>;
  }
}

// high occupancy (ctx->task_high): the register bound for 6 resident CTAs
// (double-float, compensated), 5 (FP64) or 7 (FP32), spill-free at orders
// 3-5; order 6 keeps the default bound
template <typename TE, typename TG, bool GRAD, bool COMP>
static void *tk_occ(const ace_ctx *ctx) {
  constexpr int HI = std::is_same<TE, double>::value ? 5 : std::is_same<TE, float>::value ? 7 : 6;
  if (ctx->task_high && ctx->maxord <= 5) {
    switch (ctx->maxord) {
      case 3: return (void *)ef_kernel<TE, TG, 3, NTT, GRAD, true, false, COMP, true, HI>;
      case 4: return (void *)ef_kernel<TE, TG, 4, NTT, GRAD, true, false, COMP, true, HI>;
      default: return (void *)ef_kernel<TE, TG, 5, NTT, GRAD, true, false, COMP, true, HI>;
    }
  }
  return tk_k<TE, TG, GRAD, COMP, 0>(ctx->maxord);
}

void *ef_func_tasks_df(const ace_ctx *ctx, bool grad) {
  return grad ? tk_k<df, float, true, false, 0>(ctx->maxord) : tk_k<df, float, false, false, 0>(ctx->maxord);
}

void *ef_func_tasks(const ace_ctx *ctx, bool grad) {
  if (ctx->comp) return tk_occ<df, float, true, true>(ctx);
  switch (ctx->prec) {
    case ACE_PREC_FP64: return grad ? tk_occ<double, double, true, false>(ctx) : tk_occ<double, double, false, false>(ctx);
    case ACE_PREC_FP32X2: return grad ? tk_occ<df, float, true, false>(ctx) : tk_occ<df, float, false, false>(ctx);
    default: return grad ? tk_occ<float, float, true, false>(ctx) : tk_occ<float, float, false, false>(ctx);
  }
}

}  // namespace ace
