// ace_launch_comp.cu -- the energy/force kernels of the compensated form
// (ACE_PREC_FP32_COMP: A in double-float, FP32 item products and adjoint, a
// first-order correction of the energy for A's FP32 rounding), in their own
// translation unit so they compile in parallel with the others.
#include <cuda_runtime.h>

#include "../../include/ace_b200.h"
#include "ace_ctx.h"
#include "ace_kernels.cuh"

namespace ace {

static constexpr int NTP = 128;

void *ef_func_comp(const ace_ctx *ctx) {
  switch (ctx->maxord) {
    case 1:
    case 2: return (void *)ef_kernel<df, float, 2, NTP, true, true, false, true>;
    case 3: return (void *)ef_kernel<df, float, 3, NTP, true, true, false, true>;
    case 4: return (void *)ef_kernel<df, float, 4, NTP, true, true, false, true>;
    case 5: return (void *)ef_kernel<df, float, 5, NTP, true, true, false, true>;
    default: return (void *)ef_kernel<df, float, 6, NTP, true, true, false, true>;
  }
}

}  // namespace ace
