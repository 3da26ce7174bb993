// batch_k32n4.cu -- batch_kernel instantiations for 32-bit slots and up to
// four inputs (its own translation unit, so the instantiations of the batched
// executor compile in parallel).
#include "batch_device.cuh"

namespace phcu {

BatchKernel batch_kernel_u32_nin4(int cls) {
  return batch_kernel_ew<uint32_t, 4>(cls);
}

}  // namespace phcu
