// the persistent batch kernels of uint32_t volumes (cc3d_batch_persistent.cuh)
#include "cc3d_batch_persistent.cuh"
namespace cc3dgpu {
const void* persistent_kernel_u32(int conn) { return persistent_kernel<uint32_t>(conn); }
cudaError_t persistent_args_u32(const LabelArgs* a, cudaStream_t s) { return set_persistent_args(a, s); }
}  // namespace cc3dgpu
