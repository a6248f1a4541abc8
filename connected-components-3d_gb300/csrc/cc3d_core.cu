// cc3d_core.cu -- element-type independent stages of the labelling pipeline:
// the global edge merge, the numbering scan and the label writer.
#include "cc3d_internal.h"

namespace cc3dgpu {

// ------------------------------------------------------- K2: edge merges
// Every edge joins a tile component (x = its node) with the component that
// owns a halo voxel in the neighbouring tile (y = tile * 2048 + voxel index).
__global__ void __launch_bounds__(256) k_merge_edges(LabelArgs p) {
  unsigned n = *(volatile unsigned*)&p.ctr->edge_count;
  if (n > p.edge_cap) n = p.edge_cap;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint2 e = p.edges[i];
    const uint32_t otile = e.y / kTV;
    const uint16_t c = p.rec[e.y];
    gunite(p.E, e.x, otile * kTV + c, p.bitmap, p.ctr);
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

__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const uint32_t* bitmap, int64_t nwords,
                                                              uint32_t* bsum) {
  const int64_t base = blockIdx.x * kScanChunk;
  uint32_t s = 0;
  for (int k = 0; k < kScanPer; ++k) {
    const int64_t w = base + (int64_t)k * kScanThreads + threadIdx.x;
    if (w < nwords) s += __popc(bitmap[w]);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(FULL, s, o);
  __shared__ uint32_t ws[kScanThreads / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kScanThreads / 32; ++w) t += ws[w];
    bsum[blockIdx.x] = t;
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
  k_scan_reduce<<<(unsigned)nblocks, kScanThreads, 0, s>>>(a.bitmap, nwords, bsum);
  k_scan_blocks<<<1, 1024, 0, s>>>(bsum, nblocks, a.ctr);
  k_scan_down<<<(unsigned)nblocks, kScanThreads, 0, s>>>(a.bitmap, nwords, bsum, a.prefix);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- writer
template <typename OUT>
cudaError_t launch_write_t(const LabelArgs& a, OUT* out, int64_t ntiles, cudaStream_t s) {
  if (a.ty == 8 && a.tz == 8) k_write<OUT, 8, 8><<<(unsigned)ntiles, kThreads, 0, s>>>(a, out);
  else if (a.ty == 64 && a.tz == 1) k_write<OUT, 64, 1><<<(unsigned)ntiles, kThreads, 0, s>>>(a, out);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
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
