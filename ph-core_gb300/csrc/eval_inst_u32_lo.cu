// eval_inst_u32_lo.cu -- instantiations of the elementwise kernels with
// uint32_t slots for the 0-2-input programs (split for parallel compilation).
#include "eval_kernels.cuh"

namespace phcu {

int32_t launch_eval_u32_lo(const EvalArgs& A) {
  switch (A.plan.nin) {
    case 0: return launch_eval_sn<uint32_t, 0>(A);
    case 1: return launch_eval_sn<uint32_t, 1>(A);
    case 2: return launch_eval_sn<uint32_t, 2>(A);
  }
  return fail(PHCU_ERR_INVALID, "input count %d not handled here", A.plan.nin);
}

}  // namespace phcu
