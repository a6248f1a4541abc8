// the persistent batch kernels of uint16_t volumes (cc3d_batch_persistent.cuh)
#include "cc3d_batch_persistent.cuh"
namespace cc3dgpu {
const void* persistent_kernel_u16(int conn) { return persistent_kernel<uint16_t>(conn); }
cudaError_t persistent_args_u16(const LabelArgs* a, cudaStream_t s) { return set_persistent_args(a, s); }
}  // namespace cc3dgpu
