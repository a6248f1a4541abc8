// label_u64.cu -- kernels and launchers instantiated for uint64_t volumes.
#include "cc3d_dtype_impl.cuh"

CC3D_DEFINE_DTYPE_LAUNCHERS(u64, uint64_t)
