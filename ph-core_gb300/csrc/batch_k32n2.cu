// batch_k32n2.cu -- batch_kernel instantiations for 32-bit slots and two
// inputs, and the narrow reductions (each file its own translation unit, so
// the instantiations of the batched executor compile in parallel).
#include "batch_device.cuh"

namespace phcu {

BatchKernel batch_kernel_u32_nin2(int cls) {
  return batch_kernel_ew<uint32_t, 2>(cls);
}

BatchKernel batch_kernel_reduce(bool wide) {
  return wide ? batch_kernel<uint64_t, 2, true, BC_REDUCE> : batch_kernel<uint32_t, 2, false, BC_REDUCE>;
}

}  // namespace phcu
