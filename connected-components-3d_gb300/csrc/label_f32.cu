// label_f32.cu -- kernels and launchers instantiated for float volumes.
#include "cc3d_dtype_impl.cuh"

CC3D_DEFINE_DTYPE_LAUNCHERS(f32, float)
