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
// one warp per 32 tiles takes their edges 32 at a time (merge_group_edges)
__global__ void __launch_bounds__(256) k_merge_edges(LabelArgs p) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t g = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); g * 32 < p.ntiles; g += warps)
    merge_group_edges(p, g * 32, lane);
}

cudaError_t launch_merge_edges(const LabelArgs& a, cudaStream_t s) {
  k_merge_edges<<<152 * 8, 256, 0, s>>>(a);
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

// ---------------------------------------------------------------- resolve
// Final label of every run: 1 + rank of the key of its component's root
// among the surviving keys.  A tile's components are named by their root runs
// (the runs whose component id is their own index): the labels of the root
// runs are resolved first, then every other run copies its root run's label
// into its own slot (slots of non-root runs are never read as component
// labels, so the copy is safe in place).  One warp per tile; each lane takes
// 8 runs at a time with all their loads in flight together.
__global__ void __launch_bounds__(256) k_resolve(LabelArgs p, int64_t ntiles) {
  const int lane = threadIdx.x & 31;
  const int64_t tile = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  if (tile >= ntiles) return;
  uint32_t C = p.tinfo[tile].C;
  if (C > kTV) C = kTV;
  const uint32_t node0 = (uint32_t)(tile * kTV);
  // a batch numbers each volume from 1: subtract the keys of the volumes before it
  const uint32_t rank0 = p.vols ? (uint32_t)p.vols[p.tile_vol[tile]].rank0 : 0u;
  constexpr int PER = 8;
  for (uint32_t base = 0; base < C; base += 32 * PER) {
    uint32_t rc[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const uint32_t c = base + lane + 32u * k;
      rc[k] = c < C ? (uint32_t)p.rcomp[node0 + c] : 0xFFFFFFFFu;
    }
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const uint32_t c = base + lane + 32u * k;
      if (rc[k] != c) continue;  // not a root run: no entry of its own
      const uint32_t R = gfind(p.E, node0 + c, node_count(p), p.ctr, limit_of(p.budget, kFindLimit));
      if (R == kBadNode) {
        p.label[node0 + c] = 0u;
        continue;
      }
      const uint32_t key = (uint32_t)(gload(p.E + R) >> 32);
      const uint32_t w = key >> 5;
      uint32_t lab = 0;
      if (w < p.nwords) {
        const uint32_t below = __ldg(p.bitmap + w) & ((1u << (key & 31)) - 1u);
        lab = __ldg(p.prefix + w) + __popc(below) + 1u - rank0;
      } else {
        atomicOr(&p.ctr->err, ERR_INDEX);
      }
      p.label[node0 + c] = lab;
    }
  }
  __syncwarp();
  for (uint32_t base = 0; base < C; base += 32 * PER) {
    uint32_t rc[PER], lab[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const uint32_t c = base + lane + 32u * k;
      rc[k] = c < C ? (uint32_t)p.rcomp[node0 + c] : c;
    }
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const uint32_t c = base + lane + 32u * k;
      lab[k] = (c < C && rc[k] != c && rc[k] < C) ? p.label[node0 + rc[k]] : 0u;
    }
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const uint32_t c = base + lane + 32u * k;
      if (c >= C || rc[k] == c) continue;
      if (rc[k] < C) p.label[node0 + c] = lab[k];
      else atomicOr(&p.ctr->err, ERR_INDEX);
    }
  }
}

static void launch_resolve_all(const LabelArgs& a, int64_t ntiles, cudaStream_t s) {
  if (ntiles > 0) k_resolve<<<(unsigned)((ntiles + 7) / 8), 256, 0, s>>>(a, ntiles);
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

cudaError_t launch_write_batch(const LabelArgs& a, int64_t ntiles, cudaStream_t s) {
  launch_resolve_all(a, ntiles, s);
  if (a.ty == 8 && a.tz == 8) k_write_batch<8, 8><<<(unsigned)ntiles, kThreads, 0, s>>>(a);
  else if (a.ty == 4 && a.tz == 16) k_write_batch<4, 16><<<(unsigned)ntiles, kThreads, 0, s>>>(a);
  else if (a.ty == 16 && a.tz == 4) k_write_batch<16, 4><<<(unsigned)ntiles, kThreads, 0, s>>>(a);
  else if (a.ty == 64 && a.tz == 1) k_write_batch<64, 1><<<(unsigned)ntiles, kThreads, 0, s>>>(a);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_resolve(const LabelArgs& a, cudaStream_t s) {
  launch_resolve_all(a, a.ntiles, s);
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
