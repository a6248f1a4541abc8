// cc3d_internal.h -- declarations shared by the host runtime and the kernel
// translation units of libcc3d_gpu.so.  Not part of the public ABI.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "cc3d_label.cuh"
#include "cc3d_tile.cuh"
#include "cc3d_tile_list.cuh"

namespace cc3dgpu {

// per-dtype launchers of the tile labeller and the periodic wrap unions
// (one translation unit per element type: label_<type>.cu)
// tile-pass variants: the list pass (k_tile_list: multilabel and binary
// relations) and the run-union pass (k_tile_runs: every relation mode)
constexpr int TILE_PASS_RUNS = 1;
constexpr int TILE_PASS_LIST = 2;

// A tile-pass configuration (the CC3D_TILE_* codes of include/cc3d_gpu.h):
// variant in bits 0-3, 3D tile shape in bits 4-7 (0: 32x8x8, 1: 32x4x16,
// 2: 32x16x4), bit 8: the box by plain loads instead of one TMA copy.  2D
// images always use 32x64 tiles.
struct TileCfg {
  int variant;  // TILE_PASS_LIST or TILE_PASS_RUNS
  int ty, tz;
  bool plain;
};
inline TileCfg decode_tile_cfg(int code, bool d3) {
  TileCfg c;
  const int v = code & 15;
  c.variant = v == TILE_PASS_LIST ? TILE_PASS_LIST : TILE_PASS_RUNS;
  const int shape = (code >> 4) & 15;
  c.plain = (code & 0x100) != 0;
  if (!d3) { c.ty = 64; c.tz = 1; }
  else if (shape == 1) { c.ty = 4; c.tz = 16; }
  else if (shape == 2) { c.ty = 16; c.tz = 4; }
  else { c.ty = 8; c.tz = 8; }
  return c;
}
inline bool valid_tile_code(int code) {
  const int v = code & 15;
  return code == 0 || ((v == TILE_PASS_RUNS || v == TILE_PASS_LIST) && ((code >> 4) & 15) <= 2 &&
                       (code >> 9) == 0);
}

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
                                  unsigned long long* res, cudaStream_t s);            \
  cudaError_t launch_span_##SUF(const void* in, int64_t voxels, unsigned long long* res, \
                                cudaStream_t s);

CC3D_DECLARE_DTYPE_LAUNCHERS(u8)
CC3D_DECLARE_DTYPE_LAUNCHERS(u16)
CC3D_DECLARE_DTYPE_LAUNCHERS(u32)
CC3D_DECLARE_DTYPE_LAUNCHERS(u64)
CC3D_DECLARE_DTYPE_LAUNCHERS(f32)
CC3D_DECLARE_DTYPE_LAUNCHERS(f64)

// cuTensorMapEncodeTiled from the driver (null if the driver lacks it);
// fetched once through the runtime, so the library needs no -lcuda
void* tensor_map_encoder();

// whether a cost model has been trained or loaded (cc3d_costmodel.cu)
bool g_model_loaded();

// the tile pass CC3D_TILE_AUTO resolves to for a volume class (cc3d_capi.cu)
int tile_pass_for(int dtype, int eff_connectivity, int mode, int64_t voxels);
// record an autotuned choice for a volume class (cc3d_capi.cu)
void record_tile_pass(int dtype, int eff_connectivity, int mode, int64_t voxels, int variant);

// set the calling thread's error message (returns code); map a device error
// word to a return code (cc3d_capi.cu)
// True if a kernel of this device may dereference p: device or managed
// memory.  Host addresses (pinned or not) are refused, so that a wrong
// argument returns an error instead of faulting the device.
inline bool device_accessible(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

int api_fail(int code, const char* msg);
// iteration budget of every union-find loop set by cc3d_gpu_set_union_budget
// (0: the built-in limits)
int union_budget();
int api_device_errors(unsigned err);

// per-volume results of a batch (mirrors cc3d_gpu_volume_result)
struct BatchResult {
  uint64_t N;
  uint64_t epl;
  uint64_t provisional;
  int64_t first_row;
  int64_t last_row;
  int32_t out_dtype;
  int32_t status;
};

// dtype-independent stages (cc3d_core.cu)
cudaError_t launch_merge_edges(const LabelArgs& a, cudaStream_t s);
cudaError_t launch_scan(const LabelArgs& a, int64_t nwords, uint32_t* block_sums,
                        int64_t nblocks, cudaStream_t s);
int64_t scan_blocks_needed(int64_t nwords);
cudaError_t launch_write(const LabelArgs& a, void* out, int out_dtype, int64_t ntiles,
                         cudaStream_t s);
cudaError_t launch_write_tiles(const LabelArgs& a, void* out, int out_dtype, int64_t count, cudaStream_t s);
cudaError_t launch_batch_finalize(const LabelArgs& a, int nvol, int64_t nwords, BatchResult* res,
                                  cudaStream_t s);
cudaError_t launch_write_batch(const LabelArgs& a, int64_t ntiles, cudaStream_t s);
// the persistent batch kernels k_batch_persistent<T, conn> (batch_persist_*.cu)
const void* persistent_kernel_u8(int conn);
const void* persistent_kernel_u16(int conn);
const void* persistent_kernel_u32(int conn);
// write the labelling arguments the persistent kernels of a dtype read
cudaError_t persistent_args_u8(const LabelArgs* a, cudaStream_t s);
cudaError_t persistent_args_u16(const LabelArgs* a, cudaStream_t s);
cudaError_t persistent_args_u32(const LabelArgs* a, cudaStream_t s);

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
  unsigned int* err;             // set when a label exceeds N (its voxels are skipped)
};
cudaError_t launch_stats(const StatsArgs& a, cudaStream_t s);
cudaError_t launch_stats_finalize(const StatsArgs& a, void* bboxes, int bbox_dtype,
                                  double* centroids, cudaStream_t s);

}  // namespace cc3dgpu
