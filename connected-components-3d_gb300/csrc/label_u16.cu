// label_u16.cu -- kernels and launchers instantiated for uint16_t volumes.
#include "cc3d_dtype_impl.cuh"

CC3D_DEFINE_DTYPE_LAUNCHERS(u16, uint16_t)
