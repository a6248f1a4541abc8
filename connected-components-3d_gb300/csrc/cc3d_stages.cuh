// cc3d_stages.cuh -- the element-type independent stages after the tile pass,
// written as device functions of one warp or one block, so that the staged
// kernels (cc3d_core.cu: one launch per stage) and the persistent batch kernel
// (cc3d_batch_persistent.cuh: every stage in one launch) run the same code.
#pragma once

#include "cc3d_internal.h"

namespace cc3dgpu {

// K2 of one tile, by one warp: every edge joins a tile component (x = its
// node) with the component that owns a halo voxel in the neighbouring tile
// (y = tile * 2048 + voxel index).
__device__ __forceinline__ void merge_tile_edges(const LabelArgs& p, int64_t tile, int lane) {
  const uint32_t n = p.tinfo[tile].nedges;
  const uint2* edges = p.edges + tile * p.edge_slots;
  for (uint32_t i = lane; i < n; i += 32) {
    const uint2 e = edges[i];
    const uint32_t otile = e.y / kTV, local = e.y % kTV;
    if (e.x >= (uint64_t)p.ntiles * kTV) {
      atomicOr(&p.ctr->err, ERR_INDEX);
      continue;
    }
    gunite(p.E, e.x, record_node(p, otile, (int)(local >> 5), (int)(local & 31)), node_count(p), p.bitmap,
           p.nwords, p.ctr, p.budget);
  }
}

// K2 of the G tiles [t0, t0 + G), by one warp: their edges are numbered one
// after the other (a scan of the tiles' edge counts over lanes 0..G-1) and
// taken 32 at a time, one per lane, so every round of dependent loads serves
// 32 edges (a tile has a few dozen edges; one warp per tile leaves most lanes
// of its last round idle).  G stays small so that the grid still has a warp
// for every few tiles.
constexpr int kMergeGroup = 4;
template <int G>
__device__ __forceinline__ void merge_group_edges(const LabelArgs& p, int64_t t0, int lane) {
  static_assert(G >= 1 && G <= 32 && (G & (G - 1)) == 0, "group of 1..32 tiles, a power of two");
  const int64_t tile = t0 + lane;
  const uint32_t n = (lane < G && tile < p.ntiles) ? p.tinfo[tile].nedges : 0u;
  uint32_t incl = n;
#pragma unroll
  for (int o = 1; o < G; o <<= 1) {
    const uint32_t y = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += y;
  }
  const uint32_t excl = incl - n;
  const uint32_t total = __shfl_sync(FULL, incl, G - 1);
  for (uint32_t base = 0; base < total; base += 32) {
    const uint32_t e = base + lane;
    // the tile whose edge range holds e: the last of lanes 0..G-1 with excl <= e
    int lo = 0;
#pragma unroll
    for (int step = G / 2; step > 0; step >>= 1) {
      const uint32_t ex = __shfl_sync(FULL, excl, lo + step);
      if (ex <= e) lo += step;
    }
    const uint32_t slot = e - __shfl_sync(FULL, excl, lo);
    if (e >= total) continue;
    const int64_t t = t0 + lo;
    const uint2 ed = p.edges[t * p.edge_slots + slot];
    const uint32_t otile = ed.y / kTV, local = ed.y % kTV;
    if (ed.x >= (uint64_t)p.ntiles * kTV) {
      atomicOr(&p.ctr->err, ERR_INDEX);
      continue;
    }
    gunite(p.E, ed.x, record_node(p, otile, (int)(local >> 5), (int)(local & 31)), node_count(p), p.bitmap,
           p.nwords, p.ctr, p.budget);
  }
}

// ------------------------------------------------------------ numbering scan
// The bitmap of surviving component keys is cut into chunks of kScanChunk
// words; chunk b's popcount goes to bsum[b], then an exclusive scan of the
// chunk sums, then each chunk writes the exclusive prefix of every word.
constexpr int kScanThreads = 256;
constexpr int kScanPer = 16;
constexpr int64_t kScanChunk = (int64_t)kScanThreads * kScanPer;

// Chunk b of nchunks, by a block of kScanThreads threads: its popcount sum;
// the block also reduces its share of the tile pass's per-tile results
// (estimate, provisional count, edges, first/last row) into the counters.
__device__ __forceinline__ void scan_reduce_chunk(const uint32_t* bitmap, int64_t nwords, uint32_t* bsum,
                                                  const TileInfo* ti, int64_t ntiles, Counters* ctr, int64_t b,
                                                  int64_t nchunks) {
  __shared__ uint32_t ws[kScanThreads / 32];
  __shared__ unsigned long long we[kScanThreads / 32], wp[kScanThreads / 32], wd[kScanThreads / 32];
  __shared__ long long wf[kScanThreads / 32], wl[kScanThreads / 32];
  const int64_t base = b * kScanChunk;
  uint32_t s = 0;
  for (int k = 0; k < kScanPer; ++k) {
    const int64_t w = base + (int64_t)k * kScanThreads + threadIdx.x;
    if (w < nwords) s += __popc(bitmap[w]);
  }
  unsigned long long epl = 0, prov = 0, edges = 0;
  long long f = 0x7FFFFFFFFFFFFFFFLL, l = -1;
  const int64_t per = (ntiles + nchunks - 1) / nchunks;
  const int64_t t0 = b * per, t1 = t0 + per < ntiles ? t0 + per : ntiles;
  for (int64_t t = t0 + threadIdx.x; t < t1; t += kScanThreads) {
    const TileInfo x = ti[t];
    epl += x.epl;
    prov += x.prov;
    edges += x.nedges;
    f = x.first_row < f ? x.first_row : f;
    l = x.last_row > l ? x.last_row : l;
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_down_sync(FULL, s, o);
    epl += __shfl_down_sync(FULL, epl, o);
    prov += __shfl_down_sync(FULL, prov, o);
    edges += __shfl_down_sync(FULL, edges, o);
    f = min(f, (long long)__shfl_down_sync(FULL, f, o));
    l = max(l, (long long)__shfl_down_sync(FULL, l, o));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { ws[warp] = s; we[warp] = epl; wp[warp] = prov; wd[warp] = edges; wf[warp] = f; wl[warp] = l; }
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) {
      t += ws[w];
      if (w) {
        epl += we[w]; prov += wp[w]; edges += wd[w];
        f = wf[w] < f ? wf[w] : f;
        l = wl[w] > l ? wl[w] : l;
      }
    }
    bsum[b] = t;
    if (epl) atomicAdd(&ctr->epl, epl);
    if (prov) atomicAdd(&ctr->prov, prov);
    if (edges) atomicAdd(&ctr->edges, (unsigned)edges);
    if (f != 0x7FFFFFFFFFFFFFFFLL) atomicMin(&ctr->first_row, f);
    if (l >= 0) atomicMax(&ctr->last_row, l);
  }
  __syncthreads();  // the block's shared words are free for its next chunk
}

// Exclusive scan of the nblocks chunk sums in place, by one block of NT
// threads; the total is the number of components (ctr->N).
template <int NT>
__device__ __forceinline__ void scan_chunk_sums(uint32_t* bsum, int64_t nblocks, Counters* ctr) {
  __shared__ uint32_t ws[32];
  unsigned long long carry = 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int64_t base = 0; base < nblocks; base += NT) {
    const int64_t i = base + threadIdx.x;
    const uint32_t v = i < nblocks ? bsum[i] : 0;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(FULL, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = lane < NT / 32 ? ws[lane] : 0u;
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(FULL, w, o);
        if (lane >= o) w += y;
      }
      if (lane < NT / 32) ws[lane] = w;
    }
    __syncthreads();
    const uint32_t excl = (warp ? ws[warp - 1] : 0) + x - v;
    if (i < nblocks) bsum[i] = (uint32_t)(carry + excl);
    const uint32_t chunk_total = ws[NT / 32 - 1];
    __syncthreads();
    carry += chunk_total;
  }
  if (threadIdx.x == 0) ctr->N = carry;
}

// Chunk b: the exclusive prefix of every word, by a block of kScanThreads.
__device__ __forceinline__ void scan_down_chunk(const uint32_t* bitmap, int64_t nwords, const uint32_t* bsum,
                                                uint32_t* prefix, int64_t b) {
  __shared__ uint32_t ws[kScanThreads / 32];
  const int64_t base = b * kScanChunk + (int64_t)threadIdx.x * kScanPer;
  uint32_t c[kScanPer];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    const int64_t w = base + k;
    c[k] = (w < nwords) ? __popc(bitmap[w]) : 0;
    s += c[k];
  }
  uint32_t total;
  uint32_t run = bsum[b] + block_exclusive_scan<kScanThreads>(s, ws, total);
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    const int64_t w = base + k;
    if (w < nwords) prefix[w] = run;
    run += c[k];
  }
  __syncthreads();  // the block's shared words are free for its next chunk
}

// Label of every run of one tile, by one warp: 1 + the rank of its
// component root's key among the surviving keys (minus the keys of the volumes
// before it, in a batch), into the per-run slots p.label.  The root runs
// (whose component id is their own index) are resolved first, then every
// other run copies its root run's label; eight runs per lane are in flight at
// once.
__device__ __forceinline__ void resolve_tile(const LabelArgs& p, int64_t tile, int lane) {
  uint32_t C = p.tinfo[tile].C;
  if (C > kTV) C = kTV;
  const uint32_t node0 = (uint32_t)(tile * kTV);
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
      uint32_t lab = 0;
      if (R != kBadNode) {
        const uint32_t key = (uint32_t)(gload(p.E + R) >> 32);
        const uint32_t w = key >> 5;
        if (w < p.nwords) {
          const uint32_t below = __ldg(p.bitmap + w) & ((1u << (key & 31)) - 1u);
          lab = __ldg(p.prefix + w) + __popc(below) + 1u - rank0;
        } else {
          atomicOr(&p.ctr->err, ERR_INDEX);
        }
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

// The labels of tile `tile` of a batch volume, by one warp, from the run
// labels resolve_tile left in p.label (read with coherent loads: they were
// written by this kernel).  Four rows per step: lane = 8 * (row of the four)
// + group, and a lane writes voxels 4 * group .. 4 * group + 3 of its row with
// one vector store where the row allows it.  A warp per tile, not a block,
// so that 48 tiles per SM have their dependent loads in flight at once.
template <typename OUT, int TY, int TZ>
__device__ __forceinline__ void write_tile_warp(const LabelArgs& p, int64_t tile, const VolGeo& v, OUT* out,
                                                int lane) {
  static_assert(sizeof(OUT) == 2 || sizeof(OUT) == 4, "batch outputs are uint16 or uint32");
  static_assert(TY * TZ == kRowsPerTile, "rows per tile");
  uint32_t C = p.tinfo[tile].C;
  if (C > kTV) {
    if (lane == 0) atomicOr(&p.ctr->err, ERR_INDEX);
    C = kTV;
  }
  const uint32_t local = (uint32_t)(tile - v.tile0);
  const uint32_t ntx = (uint32_t)v.ntx, nty = (uint32_t)v.nty;
  const uint32_t rest = local / ntx, tz = rest / nty;
  const int64_t x0 = (int64_t)(local - rest * ntx) * kTX;
  const int64_t y0 = (int64_t)(rest - tz * nty) * TY, z0 = (int64_t)tz * TZ;
  const uint32_t* lab = p.label + tile * kTV;
  const uint2 ma = p.rmask[tile * kRowsPerTile + lane], mb = p.rmask[tile * kRowsPerTile + 32 + lane];
  const uint32_t ra = p.rrow[tile * kRowsPerTile + lane], rb = p.rrow[tile * kRowsPerTile + 32 + lane];
  const int g4 = (lane & 7) * 4, rq = lane >> 3;
  const int64_t sx = v.sx, sy = v.sy, sz = v.sz, xg = x0 + g4, plane = sx * sy;
  const bool vec4 = (sx & 3) == 0 && (reinterpret_cast<uintptr_t>(out) & (4 * sizeof(OUT) - 1)) == 0 && xg + 3 < sx;
  const bool inner = y0 + TY <= sy && z0 + TZ <= sz;  // no row of the tile to check
  OUT* const base_ptr = out + z0 * plane + y0 * sx + xg;
#pragma unroll 1
  for (int r0 = 0; r0 < kRowsPerTile; r0 += 4) {
    const int ri = r0 + rq;
    const uint32_t F = __shfl_sync(FULL, r0 < 32 ? ma.x : mb.x, ri & 31);
    const uint32_t S = __shfl_sync(FULL, r0 < 32 ? ma.y : mb.y, ri & 31);
    const uint32_t b = __shfl_sync(FULL, r0 < 32 ? ra : rb, ri & 31);
    // the row's records hold together (no foreground before its first run
    // start, all its runs below C), checked once per row
    const bool ok = (F & ((S & (0u - S)) - 1u)) == 0u && b + (uint32_t)__popc(S) <= C;
    if (!ok) atomicOr(&p.ctr->err, ERR_INDEX);
    OUT o[4];
    // run of voxel g4 (the last run start at or before it), then of the next three
    uint32_t r = b + (uint32_t)__popc(S & lanemask_le(g4)) - 1u;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (i) r += (S >> (g4 + i)) & 1u;
      o[i] = OUT(0);
      if (ok && ((F >> (g4 + i)) & 1u)) o[i] = (OUT)lab[r];
    }
    const int ly = ri % TY, lz = ri / TY;
    if (!inner && (y0 + ly >= sy || z0 + lz >= sz)) continue;
    OUT* dst = base_ptr + lz * plane + ly * sx;
    if (vec4) {
      if constexpr (sizeof(OUT) == 2)
        *reinterpret_cast<uint2*>(dst) =
            make_uint2((uint32_t)o[0] | ((uint32_t)o[1] << 16), (uint32_t)o[2] | ((uint32_t)o[3] << 16));
      else
        *reinterpret_cast<uint4*>(dst) = make_uint4((uint32_t)o[0], (uint32_t)o[1], (uint32_t)o[2], (uint32_t)o[3]);
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (xg + i < sx) dst[i] = o[i];
    }
  }
}

// ------------------------------------------------------------ batches
// Volume v of a batch, by one warp: its estimate, provisional count,
// first/last foreground rows from its tiles; its number of components from the
// rank range of its bitmap words; the reference's output type for it
// (cc3d/fastcc3d.pyx:429-434: uint16 below 65535 estimated labels, else
// uint32; larger volumes are not batched).
__device__ __forceinline__ void finalize_volume(const LabelArgs& p, int v, int nvol, int64_t nwords,
                                                BatchResult* res, int lane) {
  VolGeo& g = p.vols[v];
  const int64_t t0 = g.tile0;
  const int64_t t1 = (v + 1 < nvol) ? p.vols[v + 1].tile0 : p.ntiles;
  unsigned long long epl = 0, prov = 0;
  long long f = 0x7FFFFFFFFFFFFFFFLL, l = -1;
  for (int64_t t = t0 + lane; t < t1; t += 32) {
    const TileInfo x = p.tinfo[t];
    epl += x.epl;
    prov += x.prov;
    f = x.first_row < f ? x.first_row : f;
    l = x.last_row > l ? x.last_row : l;
  }
  for (int o = 16; o > 0; o >>= 1) {
    epl += __shfl_down_sync(FULL, epl, o);
    prov += __shfl_down_sync(FULL, prov, o);
    f = min(f, (long long)__shfl_down_sync(FULL, f, o));
    l = max(l, (long long)__shfl_down_sync(FULL, l, o));
  }
  if (lane == 0) {
    const int64_t w1 = (v + 1 < nvol) ? p.vols[v + 1].word0 : nwords;
    const unsigned long long r0 = g.word0 < nwords ? p.prefix[g.word0] : p.ctr->N;
    const unsigned long long r1 = w1 < nwords ? p.prefix[w1] : p.ctr->N;
    const unsigned long long voxels = (unsigned long long)(g.sx * g.sy * g.sz);
    const unsigned long long max_labels = epl < voxels ? epl : voxels;
    g.rank0 = r0;
    g.out_code = max_labels < 65535ull ? 2 : 3;
    res[v].N = r1 - r0;
    res[v].epl = epl;
    res[v].provisional = prov;
    res[v].first_row = epl ? f : -1;
    res[v].last_row = epl ? l : -1;
    res[v].out_dtype = g.out_code;
    res[v].status = 0;
  }
}

}  // namespace cc3dgpu
