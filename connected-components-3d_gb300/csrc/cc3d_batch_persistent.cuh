// cc3d_batch_persistent.cuh -- a batch of volumes labelled by ONE persistent
// kernel launch.
//
// The grid holds as many 256-thread blocks as the device keeps resident at
// once (a cooperative launch guarantees they all run together) and walks the
// stages of the labelling in order, each over the whole batch, with a grid
// barrier between stages:
//
//   0  tile -> volume map         one block per volume
//   1  tile pass                  one block per tile (tile_list_tile)
//   2  edge merges                one warp per 4 tiles (merge_group_edges)
//   3  chunk popcounts            one block per bitmap chunk
//   4  scan of the chunk sums     block 0
//   5  word prefixes              one block per bitmap chunk
//   6  per-volume results         one warp per volume (finalize_volume)
//   7  run labels                 one warp per tile (resolve_tile)
//   8  labels                     one block per tile (write_tile)
//
// Every argument -- the buffers, the tile and word counts, the volume
// descriptors -- comes from device memory written before the launch (the
// labelling arguments in constant memory, the rest in a header), so the
// launch itself does not depend on the batch's layout: the host captures it
// once into a CUDA graph and replays it for every batch.
// Every grid barrier is bounded: a block that waits too long sets ERR_WAIT
// and the kernel ends (the host reports the error).
#pragma once

#include "cc3d_internal.h"
#include "cc3d_stages.cuh"

namespace cc3dgpu {

// The labelling arguments of the batch being labelled (one copy per
// translation unit that includes this header: each dtype's kernels read their
// own, written by persistent_args_* of the same unit before each launch).
static __constant__ LabelArgs c_batch_args;

inline cudaError_t set_persistent_args(const LabelArgs* a, cudaStream_t s) {
  return cudaMemcpyToSymbolAsync(c_batch_args, a, sizeof(LabelArgs), 0, cudaMemcpyHostToDevice, s);
}

struct PersistentHeader {
  LabelArgs a;        // host staging of c_batch_args: a.ctr points at ctr below
  int64_t nwords;     // bitmap words of the whole batch
  int64_t nblocks;    // scan chunks
  uint32_t* bsum;     // [nblocks + 1] chunk sums
  BatchResult* res;   // [nvol]
  int nvol;
  // the counters and the two grid-barrier words each on cache lines of their
  // own: every waiting block polls the generation word, and traffic on its
  // line must not slow the counters' atomics or the header's reads
  alignas(128) Counters ctr;
  alignas(128) unsigned bar_count;  // blocks arrived at the current barrier
  alignas(128) unsigned bar_gen;    // barrier generation
  unsigned tail_pad[31];
};

constexpr int kBarrierLimit = 1 << 22;  // polls of one grid barrier before giving up

// Grid-wide barrier over all blocks of the (cooperatively launched) grid.
// False if this block gave up waiting (ERR_WAIT is set).
__device__ __forceinline__ bool grid_barrier(PersistentHeader* h) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* gen = &h->bar_gen;
    const unsigned g0 = *gen;
    int ok = 1;
    __threadfence();
    if (atomicAdd(&h->bar_count, 1u) == gridDim.x - 1) {
      h->bar_count = 0;
      __threadfence();
      atomicAdd(&h->bar_gen, 1u);
    } else {
      for (int it = 0; *gen == g0; ++it) {
        if (it >= kBarrierLimit) {
          atomicOr(&h->ctr.err, ERR_WAIT);
          ok = 0;
          break;
        }
        __nanosleep(256);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

template <typename T, int CONN>
__global__ void __launch_bounds__(kThreads, 6) k_batch_persistent(PersistentHeader* hdr) {
  constexpr bool D3 = (CONN == 26 || CONN == 18 || CONN == 6);
  constexpr int TY = D3 ? 8 : 64, TZ = D3 ? 8 : 1;
  const LabelArgs& p = c_batch_args;
  const int lane = threadIdx.x & 31;
  const int nv = hdr->nvol;
  const int64_t ntiles = p.ntiles, nwords = hdr->nwords, nblocks = hdr->nblocks;
  uint32_t* const bsum = hdr->bsum;
  BatchResult* const res = hdr->res;
  const int64_t gw = (int64_t)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5);
  const int64_t nwarps = (int64_t)gridDim.x * (kThreads / 32);

  // 0: the volume of every tile
  for (int v = blockIdx.x; v < nv; v += gridDim.x) {
    const int64_t t0 = p.vols[v].tile0, t1 = v + 1 < nv ? p.vols[v + 1].tile0 : ntiles;
    for (int64_t t = t0 + threadIdx.x; t < t1; t += kThreads) const_cast<uint32_t*>(p.tile_vol)[t] = (uint32_t)v;
  }
  if (!grid_barrier(hdr)) return;
  // 1: tile pass
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) tile_list_tile<T, CONN, TY, TZ, MODE_MULTI>(p, nullptr, 0, t);
  if (!grid_barrier(hdr)) return;
  // 2: edge merges
  for (int64_t g = gw; g * kMergeGroup < ntiles; g += nwarps) merge_group_edges<kMergeGroup>(p, g * kMergeGroup, lane);
  if (!grid_barrier(hdr)) return;
  // 3-5: numbering scan
  for (int64_t b = blockIdx.x; b < nblocks; b += gridDim.x)
    scan_reduce_chunk(p.bitmap, nwords, bsum, p.tinfo, ntiles, p.ctr, b, nblocks);
  if (!grid_barrier(hdr)) return;
  if (blockIdx.x == 0) scan_chunk_sums<kThreads>(bsum, nblocks, p.ctr);
  if (!grid_barrier(hdr)) return;
  for (int64_t b = blockIdx.x; b < nblocks; b += gridDim.x) scan_down_chunk(p.bitmap, nwords, bsum, p.prefix, b);
  if (!grid_barrier(hdr)) return;
  // 6: per-volume results
  for (int64_t v = gw; v < nv; v += nwarps) finalize_volume(p, (int)v, nv, nwords, res, lane);
  if (!grid_barrier(hdr)) return;
  // 7: run labels, one warp per tile
  for (int64_t t = gw; t < ntiles; t += nwarps) resolve_tile(p, t, lane);
  if (!grid_barrier(hdr)) return;
  // 8: the labels written, one block per tile (write_tile), in the volume's
  // output type
  for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
    const VolGeo& v = p.vols[p.tile_vol[t]];
    if (v.out_code == 2) write_tile<uint16_t, TY, TZ>(p, t, static_cast<uint16_t*>(v.out));
    else write_tile<uint32_t, TY, TZ>(p, t, static_cast<uint32_t*>(v.out));
  }
}

// the kernel of a dtype and connectivity (null if not built)
template <typename T>
const void* persistent_kernel(int conn) {
  switch (conn) {
    case 26: return (const void*)k_batch_persistent<T, 26>;
    case 18: return (const void*)k_batch_persistent<T, 18>;
    case 6: return (const void*)k_batch_persistent<T, 6>;
    case 8: return (const void*)k_batch_persistent<T, 8>;
    case 4: return (const void*)k_batch_persistent<T, 4>;
  }
  return nullptr;
}

}  // namespace cc3dgpu
