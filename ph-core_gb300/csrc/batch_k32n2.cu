// batch_k32n2.cu -- batch_kernel<uint32_t, 2, false> (its own translation unit, so the
// instantiations of the batched executor compile in parallel).
#include "batch_device.cuh"

namespace phcu {

BatchKernel batch_kernel_u32_nin2() { return batch_kernel<uint32_t, 2, false>; }

}  // namespace phcu
