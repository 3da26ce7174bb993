// batch_k32n4.cu -- batch_kernel<uint32_t, 4, false> (its own translation unit, so the
// instantiations of the batched executor compile in parallel).
#include "batch_device.cuh"

namespace phcu {

BatchKernel batch_kernel_u32_nin4() { return batch_kernel<uint32_t, 4, false>; }

}  // namespace phcu
