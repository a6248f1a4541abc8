// the persistent batch kernels of uint16_t volumes (cc3d_batch_persistent.cuh)
#include "cc3d_batch_persistent.cuh"
namespace cc3dgpu {
const void* persistent_kernel_u16(int conn) { return persistent_kernel<uint16_t>(conn); }
}  // namespace cc3dgpu
