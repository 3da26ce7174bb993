// batch_k64.cu -- batch_kernel<uint64_t, 4, true> (its own translation unit, so the
// instantiations of the batched executor compile in parallel).
#include "batch_device.cuh"

namespace phcu {

BatchKernel batch_kernel_u64() { return batch_kernel<uint64_t, 4, true>; }

}  // namespace phcu
