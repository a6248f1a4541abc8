// cc3d_core.cu -- element-type independent stages of the labelling pipeline:
// the global edge merge, the numbering scan and the label writer.
#include "cc3d_internal.h"

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
// Every edge joins a tile component (x = its node) with the component that
// owns a halo voxel in the neighbouring tile (y = tile * 2048 + voxel index).
// One warp per tile walks the tile's edge slots.
__global__ void __launch_bounds__(256) k_merge_edges(LabelArgs p) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t tile = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile < p.ntiles;
       tile += warps) {
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
}

cudaError_t launch_merge_edges(const LabelArgs& a, cudaStream_t s) {
  k_merge_edges<<<152 * 8, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// ------------------------------------------------------------ numbering scan
constexpr int kScanThreads = 256;
constexpr int kScanPer = 16;
constexpr int64_t kScanChunk = (int64_t)kScanThreads * kScanPer;

int64_t scan_blocks_needed(int64_t nwords) { return (nwords + kScanChunk - 1) / kScanChunk; }

// Per-block popcount sums of the bitmap; each block also reduces its share
// of the tile pass's per-tile results (estimate, provisional count, edges,
// first/last row) into the counters.
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const uint32_t* bitmap, int64_t nwords,
                                                              uint32_t* bsum, const TileInfo* ti,
                                                              int64_t ntiles, Counters* ctr) {
  const int64_t base = blockIdx.x * kScanChunk;
  uint32_t s = 0;
  for (int k = 0; k < kScanPer; ++k) {
    const int64_t w = base + (int64_t)k * kScanThreads + threadIdx.x;
    if (w < nwords) s += __popc(bitmap[w]);
  }
  unsigned long long epl = 0, prov = 0, edges = 0;
  long long f = 0x7FFFFFFFFFFFFFFFLL, l = -1;
  const int64_t per = (ntiles + gridDim.x - 1) / gridDim.x;
  const int64_t t0 = blockIdx.x * per, t1 = t0 + per < ntiles ? t0 + per : ntiles;
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
  __shared__ uint32_t ws[kScanThreads / 32];
  __shared__ unsigned long long we[kScanThreads / 32], wp[kScanThreads / 32], wd[kScanThreads / 32];
  __shared__ long long wf[kScanThreads / 32], wl[kScanThreads / 32];
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
    bsum[blockIdx.x] = t;
    if (epl) atomicAdd(&ctr->epl, epl);
    if (prov) atomicAdd(&ctr->prov, prov);
    if (edges) atomicAdd(&ctr->edges, (unsigned)edges);
    if (f != 0x7FFFFFFFFFFFFFFFLL) atomicMin(&ctr->first_row, f);
    if (l >= 0) atomicMax(&ctr->last_row, l);
  }
}

__global__ void __launch_bounds__(1024) k_scan_blocks(uint32_t* bsum, int64_t nblocks, Counters* ctr) {
  __shared__ uint32_t ws[32];
  unsigned long long carry = 0;
  for (int64_t base = 0; base < nblocks; base += 1024) {
    const int64_t i = base + threadIdx.x;
    const uint32_t v = i < nblocks ? bsum[i] : 0;
    uint32_t x = v;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(FULL, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
      uint32_t w = ws[lane];
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(FULL, w, o);
        if (lane >= o) w += y;
      }
      ws[lane] = w;
    }
    __syncthreads();
    const uint32_t excl = (warp ? ws[warp - 1] : 0) + x - v;
    if (i < nblocks) bsum[i] = (uint32_t)(carry + excl);
    const uint32_t chunk_total = ws[31];
    __syncthreads();
    carry += chunk_total;
  }
  if (threadIdx.x == 0) ctr->N = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_down(const uint32_t* bitmap, int64_t nwords,
                                                            const uint32_t* bsum, uint32_t* prefix) {
  __shared__ uint32_t ws[kScanThreads / 32];
  const int64_t base = blockIdx.x * kScanChunk + (int64_t)threadIdx.x * kScanPer;
  uint32_t c[kScanPer];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    const int64_t w = base + k;
    c[k] = (w < nwords) ? __popc(bitmap[w]) : 0;
    s += c[k];
  }
  uint32_t total;
  uint32_t run = bsum[blockIdx.x] + block_exclusive_scan<kScanThreads>(s, ws, total);
#pragma unroll
  for (int k = 0; k < kScanPer; ++k) {
    const int64_t w = base + k;
    if (w < nwords) prefix[w] = run;
    run += c[k];
  }
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
// Per volume of a batch (one warp each): its estimate, provisional count,
// first/last foreground rows from its tiles; its number of components from the
// rank range of its bitmap words; the reference's output type for it
// (cc3d/fastcc3d.pyx:429-434: uint16 below 65535 estimated labels, else
// uint32; larger volumes are not batched).
__global__ void __launch_bounds__(256) k_batch_finalize(LabelArgs p, int nvol, int64_t nwords,
                                                         cc3dgpu::BatchResult* res) {
  const int lane = threadIdx.x & 31;
  const int v = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (v >= nvol) return;
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
