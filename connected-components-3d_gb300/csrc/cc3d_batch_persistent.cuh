// cc3d_batch_persistent.cuh -- a batch of volumes labelled by ONE persistent
// kernel launch.
//
// The grid holds as many 256-thread blocks as the device keeps resident at
// once (a cooperative launch guarantees they all run together) and walks the
// stages of the labelling in order, each over the whole batch, with a grid
// barrier between stages:
//
//   0  tile -> volume map         one block per volume
//   1  tile pass                  one block per tile (tile_list_tile), tiles
//                                 taken from a work queue
//   2  edge merges                one warp per 4 tiles (merge_group_edges)
//   3  chunk popcounts            one block per bitmap chunk
//   4  scan of the chunk sums     block 0
//   5  word prefixes              one block per bitmap chunk
//   6  per-volume results         one warp per volume (finalize_volume)
//   7  labels                     one warp per tile: its run labels
//                                 (resolve_tile), then its rows
//                                 (write_tile_warp)
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
  // the tile pass's work queue: the next tile a block takes (zero in the
  // uploaded header; a batch has fewer than 2^21 tiles)
  alignas(128) unsigned next_tile;
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

// A block's walk over the n items of a work queue.  A queue, not a fixed
// share per block: the SM's scheduler favours its older blocks, so with fixed
// shares the younger blocks of every SM finish last and the SM idles
// meanwhile.  Thread 0 takes items two ahead of their use: the item it
// publishes (to shared memory) before the body was fetched one body earlier,
// so no thread waits for the atomic.  The body must hold a block barrier that
// every thread reaches (the tile pass has several): thread 0 writes the next
// item before it, the others read it after it, and everyone has read the
// current item before thread 0 overwrites that slot one item later.
template <typename F>
__device__ __forceinline__ void drain_queue(unsigned* q, int64_t n, F&& body) {
  __shared__ unsigned s_item[2];
  unsigned ahead = 0;
  if (threadIdx.x == 0) {
    s_item[0] = atomicAdd(q, 1u);
    ahead = atomicAdd(q, 1u);
  }
  __syncthreads();
  for (int k = 0;; k ^= 1) {
    const unsigned t = s_item[k];
    if ((int64_t)t >= n) break;
    if (threadIdx.x == 0) {
      s_item[k ^ 1] = ahead;
      ahead = atomicAdd(q, 1u);
    }
    body((int64_t)t);
  }
}

// (seven blocks per SM for one- and two-byte voxels, as the tile pass alone)
template <typename T, int CONN>
__global__ void __launch_bounds__(kThreads, sizeof(T) <= 2 ? 7 : 6) k_batch_persistent(PersistentHeader* hdr) {
  constexpr bool D3 = (CONN == 26 || CONN == 18 || CONN == 6);
  constexpr int TY = D3 ? 8 : 64, TZ = D3 ? 8 : 1;
  const LabelArgs& p = c_batch_args;
  const int lane = threadIdx.x & 31;
  // (the header's fields are read where a stage needs them, not held in
  // registers across the stages: the tile pass needs every register)
  auto warp_id = [] { return (int64_t)blockIdx.x * (kThreads / 32) + (threadIdx.x >> 5); };
  auto warps = [] { return (int64_t)gridDim.x * (kThreads / 32); };

  // 0: the volume of every tile
  {
    const int nv = hdr->nvol;
    for (int v = blockIdx.x; v < nv; v += gridDim.x) {
      const int64_t t0 = p.vols[v].tile0, t1 = v + 1 < nv ? p.vols[v + 1].tile0 : p.ntiles;
      for (int64_t t = t0 + threadIdx.x; t < t1; t += kThreads) const_cast<uint32_t*>(p.tile_vol)[t] = (uint32_t)v;
    }
  }
  if (!grid_barrier(hdr)) return;
  // 1: tile pass, tiles in order from the queue
  drain_queue(&hdr->next_tile, p.ntiles,
              [&](int64_t t) { tile_list_tile<T, CONN, TY, TZ, MODE_MULTI, true>(p, nullptr, 0, t); });
  if (!grid_barrier(hdr)) return;
  // 2: edge merges
  for (int64_t g = warp_id(); g * kMergeGroup < p.ntiles; g += warps())
    merge_group_edges<kMergeGroup>(p, g * kMergeGroup, lane);
  if (!grid_barrier(hdr)) return;
  // 3-5: numbering scan
  for (int64_t b = blockIdx.x; b < hdr->nblocks; b += gridDim.x)
    scan_reduce_chunk(p.bitmap, hdr->nwords, hdr->bsum, p.tinfo, p.ntiles, p.ctr, b, hdr->nblocks);
  if (!grid_barrier(hdr)) return;
  if (blockIdx.x == 0) scan_chunk_sums<kThreads>(hdr->bsum, hdr->nblocks, p.ctr);
  if (!grid_barrier(hdr)) return;
  for (int64_t b = blockIdx.x; b < hdr->nblocks; b += gridDim.x)
    scan_down_chunk(p.bitmap, hdr->nwords, hdr->bsum, p.prefix, b);
  if (!grid_barrier(hdr)) return;
  // 6: per-volume results
  {
    const int nv = hdr->nvol;
    for (int64_t v = warp_id(); v < nv; v += warps()) finalize_volume(p, (int)v, nv, hdr->nwords, hdr->res, lane);
  }
  if (!grid_barrier(hdr)) return;
  // 7: the labels, one warp per tile: the tile's run labels (resolve_tile),
  // then its rows in the volume's output type (write_tile_warp)
  for (int64_t t = warp_id(); t < p.ntiles; t += warps()) {
    resolve_tile(p, t, lane);
    __syncwarp();
    const VolGeo& v = p.vols[p.tile_vol[t]];
    if (v.out_code == 2) write_tile_warp<uint16_t, TY, TZ>(p, t, v, static_cast<uint16_t*>(v.out), lane);
    else write_tile_warp<uint32_t, TY, TZ>(p, t, v, static_cast<uint32_t*>(v.out), lane);
    __syncwarp();
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
