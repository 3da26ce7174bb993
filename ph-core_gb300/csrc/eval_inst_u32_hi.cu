// eval_inst_u32_hi.cu -- instantiations of the elementwise kernels with
// uint32_t slots for the 3-4-input programs (split for parallel compilation).
#include "eval_kernels.cuh"

namespace phcu {

int32_t launch_eval_u32_hi(const EvalArgs& A) {
  switch (A.plan.nin) {
    case 3: return launch_eval_sn<uint32_t, 3>(A);
    case 4: return launch_eval_sn<uint32_t, 4>(A);
  }
  return fail(PHCU_ERR_INVALID, "input count %d not handled here", A.plan.nin);
}

}  // namespace phcu
