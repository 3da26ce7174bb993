// batch_k64.cu -- batch_kernel instantiations for 64-bit slots and up to
// four inputs (its own translation unit, so the instantiations of the batched
// executor compile in parallel).
#include "batch_device.cuh"

namespace phcu {

BatchKernel batch_kernel_u64(int cls) {
  return batch_kernel_ew<uint64_t, 4>(cls);
}

}  // namespace phcu
