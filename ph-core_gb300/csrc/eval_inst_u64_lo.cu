// eval_inst_u64_lo.cu -- instantiations of the elementwise kernels with
// uint64_t slots for the 0-2-input programs (split for parallel compilation).
#include "eval_kernels.cuh"

namespace phcu {

int32_t launch_eval_u64_lo(const EvalArgs& A) {
  switch (A.plan.nin) {
    case 0: return launch_eval_sn<uint64_t, 0>(A);
    case 1: return launch_eval_sn<uint64_t, 1>(A);
    case 2: return launch_eval_sn<uint64_t, 2>(A);
  }
  return fail(PHCU_ERR_INVALID, "input count %d not handled here", A.plan.nin);
}

}  // namespace phcu
