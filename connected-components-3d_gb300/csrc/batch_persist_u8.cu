// the persistent batch kernels of uint8_t volumes (cc3d_batch_persistent.cuh)
#include "cc3d_batch_persistent.cuh"
namespace cc3dgpu {
const void* persistent_kernel_u8(int conn) { return persistent_kernel<uint8_t>(conn); }
cudaError_t persistent_args_u8(const LabelArgs* a, cudaStream_t s) { return set_persistent_args(a, s); }
}  // namespace cc3dgpu
