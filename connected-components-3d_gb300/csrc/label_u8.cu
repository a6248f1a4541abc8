// label_u8.cu -- kernels and launchers instantiated for uint8_t volumes.
#include "cc3d_dtype_impl.cuh"

CC3D_DEFINE_DTYPE_LAUNCHERS(u8, uint8_t)
