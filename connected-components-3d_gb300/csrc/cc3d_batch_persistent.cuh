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
//   2  edge merges                one warp per 32 tiles (merge_group_edges)
//   3  chunk popcounts            one block per bitmap chunk
//   4  scan of the chunk sums     block 0
//   5  word prefixes              one block per bitmap chunk
//   6  per-volume results         one warp per volume (finalize_volume)
//   7  labels                     one warp per tile (write_batch_tile)
//
// Every argument -- the buffers, the tile and word counts, the volume
// descriptors -- comes from a header in device memory uploaded before the
// launch, so the launch itself does not depend on the batch's layout: the
// host captures it once into a CUDA graph and replays it for every batch.
// Every grid barrier is bounded: a block that waits too long sets ERR_WAIT
// and the kernel ends (the host reports the error).
#pragma once

#include "cc3d_internal.h"
#include "cc3d_stages.cuh"

namespace cc3dgpu {

struct PersistentHeader {
  LabelArgs a;        // a.ctr points at ctr below; a.vols, a.tile_vol into the arena
  int64_t nwords;     // bitmap words of the whole batch
  int64_t nblocks;    // scan chunks
  uint32_t* bsum;     // [nblocks + 1] chunk sums
  BatchResult* res;   // [nvol]
  int nvol;
  unsigned bar_count; // grid barrier: blocks arrived, generation
  unsigned bar_gen;
  unsigned pad;
  Counters ctr;
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
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Labels of one tile of a batch, by one warp: the labels of the tile's root
// runs (1 + rank of their root's key within the volume's key range), every
// other run's label (its root run's), then the tile's 64 rows in the
// volume's output type.  Run labels go through the per-run global slots.
template <int TY, int TZ>
__device__ __forceinline__ void write_batch_tile(const LabelArgs& p, int64_t tile, int lane) {
  const VolGeo& v = p.vols[p.tile_vol[tile]];
  const TileGeo g = tile_geo(p, tile);
  uint32_t C = p.tinfo[tile].C;
  if (C > kTV) {
    if (lane == 0) atomicOr(&p.ctr->err, ERR_INDEX);
    C = kTV;
  }
  const uint32_t node0 = (uint32_t)(tile * kTV);
  const uint32_t rank0 = (uint32_t)v.rank0;
  uint32_t* lab = p.label + node0;
  const uint2 ma = p.rmask[tile * kRowsPerTile + lane], mb = p.rmask[tile * kRowsPerTile + 32 + lane];
  const uint32_t ra = p.rrow[tile * kRowsPerTile + lane], rb = p.rrow[tile * kRowsPerTile + 32 + lane];
  for (uint32_t c = lane; c < C; c += 32) {
    if (p.rcomp[node0 + c] != c) continue;  // only root runs name components
    const uint32_t R = gfind(p.E, node0 + c, node_count(p), p.ctr, limit_of(p.budget, kFindLimit));
    uint32_t l = 0;
    if (R != kBadNode) {
      const uint32_t key = (uint32_t)(gload(p.E + R) >> 32);
      const uint32_t w = key >> 5;
      if (w < p.nwords) l = p.prefix[w] + __popc(p.bitmap[w] & ((1u << (key & 31)) - 1u)) + 1u - rank0;
      else atomicOr(&p.ctr->err, ERR_INDEX);
    }
    lab[c] = l;
  }
  __syncwarp();
  for (uint32_t c = lane; c < C; c += 32) {
    const uint32_t rc = p.rcomp[node0 + c];
    if (rc == c) continue;
    if (rc < C) lab[c] = lab[rc];
    else atomicOr(&p.ctr->err, ERR_INDEX);
  }
  __syncwarp();
  const int64_t x0 = (int64_t)g.tx * kTX, y0 = (int64_t)g.ty * TY, z0 = (int64_t)g.tz * TZ;
  const int64_t x = x0 + lane;
  const bool xin = x < g.sx;
  for (int ri = 0; ri < kRowsPerTile; ++ri) {
    const uint32_t F = __shfl_sync(FULL, ri < 32 ? ma.x : mb.x, ri & 31);
    const uint32_t S = __shfl_sync(FULL, ri < 32 ? ma.y : mb.y, ri & 31);
    const uint32_t b = __shfl_sync(FULL, ri < 32 ? ra : rb, ri & 31);
    const int ly = ri % TY, lz = ri / TY;
    const int64_t y = y0 + ly, z = z0 + lz;
    if (!xin || y >= g.sy || z >= g.sz) continue;
    uint32_t l = 0;
    if ((F >> lane) & 1u) {
      const int k = __popc(S & lanemask_le(lane)) - 1;
      const uint32_t r = b + (uint32_t)k;
      if (k >= 0 && r < C) l = lab[r];
      else atomicOr(&p.ctr->err, ERR_INDEX);
    }
    const int64_t i = (z * g.sy + y) * g.sx + x;
    if (v.out_code == 2) static_cast<uint16_t*>(v.out)[i] = (uint16_t)l;
    else static_cast<uint32_t*>(v.out)[i] = l;
  }
}

template <typename T, int CONN>
__global__ void __launch_bounds__(kThreads, 6) k_batch_persistent(PersistentHeader* hdr) {
  constexpr bool D3 = (CONN == 26 || CONN == 18 || CONN == 6);
  constexpr int TY = D3 ? 8 : 64, TZ = D3 ? 8 : 1;
  __shared__ LabelArgs sp;
  static_assert(sizeof(LabelArgs) % 4 == 0, "word copy");
  for (int i = threadIdx.x; i < (int)(sizeof(LabelArgs) / 4); i += blockDim.x)
    reinterpret_cast<uint32_t*>(&sp)[i] = reinterpret_cast<const uint32_t*>(&hdr->a)[i];
  __syncthreads();
  const LabelArgs& p = sp;
  const int lane = threadIdx.x & 31;
  const int nv = hdr->nvol;
  const int64_t ntiles = p.ntiles, nwords = hdr->nwords, nblocks = hdr->nblocks;
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
  for (int64_t g = gw; g * 32 < ntiles; g += nwarps) merge_group_edges(p, g * 32, lane);
  if (!grid_barrier(hdr)) return;
  // 3-5: numbering scan
  for (int64_t b = blockIdx.x; b < nblocks; b += gridDim.x)
    scan_reduce_chunk(p.bitmap, nwords, hdr->bsum, p.tinfo, ntiles, p.ctr, b, nblocks);
  if (!grid_barrier(hdr)) return;
  if (blockIdx.x == 0) scan_chunk_sums<kThreads>(hdr->bsum, nblocks, p.ctr);
  if (!grid_barrier(hdr)) return;
  for (int64_t b = blockIdx.x; b < nblocks; b += gridDim.x) scan_down_chunk(p.bitmap, nwords, hdr->bsum, p.prefix, b);
  if (!grid_barrier(hdr)) return;
  // 6: per-volume results
  for (int64_t v = gw; v < nv; v += nwarps) finalize_volume(p, (int)v, nv, nwords, hdr->res, lane);
  if (!grid_barrier(hdr)) return;
  // 7: labels
  for (int64_t t = gw; t < ntiles; t += nwarps) write_batch_tile<TY, TZ>(p, t, lane);
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
