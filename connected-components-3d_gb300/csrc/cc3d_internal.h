// cc3d_internal.h -- declarations shared by the host runtime and the kernel
// translation units of libcc3d_gpu.so.  Not part of the public ABI.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "cc3d_label.cuh"
#include "cc3d_scan.cuh"
#include "cc3d_tile.cuh"

namespace cc3dgpu {

// per-dtype launchers of the tile labeller and the periodic wrap unions
// (one translation unit per element type: label_<type>.cu)
// tile-pass variants: the block-parallel pass (k_tile_runs) and the
// warp-per-tile raster scan (k_tile_scan)
constexpr int TILE_PASS_RUNS = 1;
constexpr int TILE_PASS_SCAN = 2;

#define CC3D_DECLARE_DTYPE_LAUNCHERS(SUF)                                              \
  cudaError_t launch_tile_local_##SUF(const LabelArgs& a, int conn, int mode,         \
                                      bool block8, int variant, int64_t ntiles,        \
                                      cudaStream_t s);                                 \
  cudaError_t launch_wrap_##SUF(const LabelArgs& a, int conn, int mode, cudaStream_t s); \
  cudaError_t launch_epl_##SUF(const void* in, int64_t sx, int64_t voxels,            \
                               Counters* ctr, cudaStream_t s);                        \
  cudaError_t launch_special_row_##SUF(const void* in, int64_t sx, int64_t row,       \
                                       int is_uint64, void* out, int out_dtype,        \
                                       Counters* ctr, cudaStream_t s);                \
  cudaError_t launch_minmax_##SUF(const void* in, int64_t voxels, int is_signed,      \
                                  unsigned long long* res, cudaStream_t s);

CC3D_DECLARE_DTYPE_LAUNCHERS(u8)
CC3D_DECLARE_DTYPE_LAUNCHERS(u16)
CC3D_DECLARE_DTYPE_LAUNCHERS(u32)
CC3D_DECLARE_DTYPE_LAUNCHERS(u64)
CC3D_DECLARE_DTYPE_LAUNCHERS(f32)
CC3D_DECLARE_DTYPE_LAUNCHERS(f64)

// cuTensorMapEncodeTiled from the driver (null if the driver lacks it);
// fetched once through the runtime, so the library needs no -lcuda
void* tensor_map_encoder();

// set the calling thread's error message (returns code); map a device error
// word to a return code (cc3d_capi.cu)
int api_fail(int code, const char* msg);
int api_device_errors(unsigned err);

// dtype-independent stages (cc3d_core.cu)
cudaError_t launch_merge_edges(const LabelArgs& a, cudaStream_t s);
cudaError_t launch_scan(const LabelArgs& a, int64_t nwords, uint32_t* block_sums,
                        int64_t nblocks, cudaStream_t s);
int64_t scan_blocks_needed(int64_t nwords);
cudaError_t launch_write(const LabelArgs& a, void* out, int out_dtype, int64_t ntiles,
                         cudaStream_t s);

// statistics (cc3d_stats.cu)
struct StatsArgs {
  const void* labels;
  int dtype;
  int64_t d0, d1, d2;
  int ndim;
  int c_order;
  uint64_t N;
  uint32_t* counts;              // [N+1]
  uint32_t* bmin;                // [(N+1) * 3]
  uint32_t* bmax;                // [(N+1) * 3]
  unsigned long long* sums;      // [(N+1) * 3]
};
cudaError_t launch_stats(const StatsArgs& a, cudaStream_t s);
cudaError_t launch_stats_finalize(const StatsArgs& a, void* bboxes, int bbox_dtype,
                                  double* centroids, cudaStream_t s);

}  // namespace cc3dgpu
