// cc3d_core.cu -- element-type independent stages of the labelling pipeline:
// the global edge merge, the numbering scan and the label writer.
#include "cc3d_internal.h"
#include "cc3d_stages.cuh"

namespace cc3dgpu {

void* tensor_map_encoder() {
  static void* fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      f = nullptr;
    return f;
  }();
  return fn;
}

// ------------------------------------------------------- K2: edge merges
// one warp per kMergeGroup tiles takes their edges 32 at a time (merge_group_edges)
__global__ void __launch_bounds__(256) k_merge_edges(LabelArgs p) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t g = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); g * kMergeGroup < p.ntiles;
       g += warps)
    merge_group_edges<kMergeGroup>(p, g * kMergeGroup, lane);
}

cudaError_t launch_merge_edges(const LabelArgs& a, cudaStream_t s) {
  // a warp per group of tiles, up to 32 warps per SM
  const int64_t groups = (a.ntiles + kMergeGroup - 1) / kMergeGroup;
  int64_t blocks = (groups + 7) / 8;
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  k_merge_edges<<<(unsigned)blocks, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// ------------------------------------------------------------ numbering scan
int64_t scan_blocks_needed(int64_t nwords) { return (nwords + kScanChunk - 1) / kScanChunk; }

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const uint32_t* bitmap, int64_t nwords,
                                                              uint32_t* bsum, const TileInfo* ti,
                                                              int64_t ntiles, Counters* ctr) {
  scan_reduce_chunk(bitmap, nwords, bsum, ti, ntiles, ctr, blockIdx.x, gridDim.x);
}

__global__ void __launch_bounds__(1024) k_scan_blocks(uint32_t* bsum, int64_t nblocks, Counters* ctr) {
  scan_chunk_sums<1024>(bsum, nblocks, ctr);
}

__global__ void __launch_bounds__(kScanThreads) k_scan_down(const uint32_t* bitmap, int64_t nwords,
                                                            const uint32_t* bsum, uint32_t* prefix) {
  scan_down_chunk(bitmap, nwords, bsum, prefix, blockIdx.x);
}

cudaError_t launch_scan(const LabelArgs& a, int64_t nwords, uint32_t* bsum, int64_t nblocks,
                        cudaStream_t s) {
  if (nblocks == 0) return cudaSuccess;
  k_scan_reduce<<<(unsigned)nblocks, kScanThreads, 0, s>>>(a.bitmap, nwords, bsum, a.tinfo, a.ntiles, a.ctr);
  k_scan_blocks<<<1, 1024, 0, s>>>(bsum, nblocks, a.ctr);
  k_scan_down<<<(unsigned)nblocks, kScanThreads, 0, s>>>(a.bitmap, nwords, bsum, a.prefix);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- writer
template <typename OUT>
cudaError_t launch_write_tiles_t(const LabelArgs& a, OUT* out, int64_t count, cudaStream_t s);

template <typename OUT>
cudaError_t launch_write_t(const LabelArgs& a, OUT* out, int64_t ntiles, cudaStream_t s) {
  return launch_write_tiles_t<OUT>(a, out, ntiles, s);
}

// ------------------------------------------------------------ batches
// one warp per volume of a batch (finalize_volume)
__global__ void __launch_bounds__(256) k_batch_finalize(LabelArgs p, int nvol, int64_t nwords,
                                                         cc3dgpu::BatchResult* res) {
  const int v = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (v >= nvol) return;
  finalize_volume(p, v, nvol, nwords, res, threadIdx.x & 31);
}

cudaError_t launch_batch_finalize(const LabelArgs& a, int nvol, int64_t nwords, BatchResult* res,
                                  cudaStream_t s) {
  k_batch_finalize<<<(unsigned)((nvol + 7) / 8), 256, 0, s>>>(a, nvol, nwords, res);
  return cudaGetLastError();
}

// A batch's labels, one warp per tile: the tile's run labels (resolve_tile),
// then its rows in the volume's output type (write_tile_warp; a batch's
// outputs are uint16 or uint32)
template <int TY, int TZ>
__global__ void __launch_bounds__(256) k_label_batch(LabelArgs p, int64_t ntiles) {
  const int64_t tile = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  if (tile >= ntiles) return;
  const int lane = threadIdx.x & 31;
  resolve_tile(p, tile, lane);
  __syncwarp();
  const VolGeo& v = p.vols[p.tile_vol[tile]];
  if (v.out_code == 2) write_tile_warp<uint16_t, TY, TZ>(p, tile, v, static_cast<uint16_t*>(v.out), lane);
  else write_tile_warp<uint32_t, TY, TZ>(p, tile, v, static_cast<uint32_t*>(v.out), lane);
}

cudaError_t launch_write_batch(const LabelArgs& a, int64_t ntiles, cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((ntiles + 7) / 8);
  if (a.ty == 8 && a.tz == 8) k_label_batch<8, 8><<<grid, 256, 0, s>>>(a, ntiles);
  else if (a.ty == 4 && a.tz == 16) k_label_batch<4, 16><<<grid, 256, 0, s>>>(a, ntiles);
  else if (a.ty == 16 && a.tz == 4) k_label_batch<16, 4><<<grid, 256, 0, s>>>(a, ntiles);
  else if (a.ty == 64 && a.tz == 1) k_label_batch<64, 1><<<grid, 256, 0, s>>>(a, ntiles);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

// labels of the tiles [a.tile_base, a.tile_base + count) of a single volume,
// resolved and written by one warp per tile
template <typename OUT>
cudaError_t launch_write_tiles_t(const LabelArgs& a, OUT* out, int64_t count, cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  const unsigned blocks = (unsigned)((count + kLabelWarps - 1) / kLabelWarps);
  constexpr int NT = kLabelWarps * 32;
  if (a.ty == 8 && a.tz == 8) k_label_write<OUT, 8, 8><<<blocks, NT, 0, s>>>(a, out, count);
  else if (a.ty == 4 && a.tz == 16) k_label_write<OUT, 4, 16><<<blocks, NT, 0, s>>>(a, out, count);
  else if (a.ty == 16 && a.tz == 4) k_label_write<OUT, 16, 4><<<blocks, NT, 0, s>>>(a, out, count);
  else if (a.ty == 64 && a.tz == 1) k_label_write<OUT, 64, 1><<<blocks, NT, 0, s>>>(a, out, count);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_write_tiles(const LabelArgs& a, void* out, int out_dtype, int64_t count, cudaStream_t s) {
  switch (out_dtype) {
    case 2: return launch_write_tiles_t<uint16_t>(a, (uint16_t*)out, count, s);
    case 3: return launch_write_tiles_t<uint32_t>(a, (uint32_t*)out, count, s);
    case 4: return launch_write_tiles_t<uint64_t>(a, (uint64_t*)out, count, s);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_write(const LabelArgs& a, void* out, int out_dtype, int64_t ntiles, cudaStream_t s) {
  switch (out_dtype) {
    case 2: return launch_write_t<uint16_t>(a, (uint16_t*)out, ntiles, s);
    case 3: return launch_write_t<uint32_t>(a, (uint32_t*)out, ntiles, s);
    case 4: return launch_write_t<uint64_t>(a, (uint64_t*)out, ntiles, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace cc3dgpu
