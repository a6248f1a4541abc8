// label_f64.cu -- kernels and launchers instantiated for double volumes.
#include "cc3d_dtype_impl.cuh"

CC3D_DEFINE_DTYPE_LAUNCHERS(f64, double)
