// label_u32.cu -- kernels and launchers instantiated for uint32_t volumes.
#include "cc3d_dtype_impl.cuh"

CC3D_DEFINE_DTYPE_LAUNCHERS(u32, uint32_t)
