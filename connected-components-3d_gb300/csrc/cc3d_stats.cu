// cc3d_stats.cu -- per-label voxel counts, bounding boxes and centroids
// (replaces _statistics_helper2d/3d, cc3d/fastcc3d.pyx:767-938).
//
// One pass over the labels in memory order.  Each warp groups its 32 voxels
// by label (usually one or two labels: labels come in runs), reduces count,
// per-axis min/max and per-axis coordinate sums inside the group, and one lane
// per group issues the atomics.  Coordinate sums are exact 64-bit integers;
// the finaliser divides them in FP64, which reproduces the reference's
// one-by-one double accumulation bit for bit while the sums stay below 2^53.
#include "cc3d_internal.h"

namespace cc3dgpu {

__global__ void k_stats_init(uint32_t* counts, uint32_t* bmin, uint32_t* bmax,
                             unsigned long long* sums, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    counts[i] = 0;
    for (int a = 0; a < 3; ++a) {
      bmin[i * 3 + a] = 0xFFFFFFFFu;
      bmax[i * 3 + a] = 0;
      sums[i * 3 + a] = 0;
    }
  }
}

__device__ __forceinline__ unsigned long long warp_sum64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}

template <typename L>
__global__ void __launch_bounds__(256) k_stats(StatsArgs a) {
  const L* lab = static_cast<const L*>(a.labels);
  const int64_t n = a.d0 * a.d1 * a.d2;
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < n; base += stride) {
    const int64_t i = base + lane;
    const bool valid = i < n;
    unsigned long long l = valid ? (unsigned long long)lab[i] : 0;
    uint32_t c[3] = {0, 0, 0};
    if (valid) {
      if (a.c_order) {
        c[2] = (uint32_t)(i % a.d2);
        const int64_t r = i / a.d2;
        c[1] = (uint32_t)(r % a.d1);
        c[0] = (uint32_t)(r / a.d1);
      } else {
        c[0] = (uint32_t)(i % a.d0);
        const int64_t r = i / a.d0;
        c[1] = (uint32_t)(r % a.d1);
        c[2] = (uint32_t)(r / a.d1);
      }
    }
    unsigned active = __ballot_sync(FULL, valid);
    while (active) {
      const int leader = __ffs(active) - 1;
      const unsigned long long ll = __shfl_sync(FULL, l, leader);
      const bool mine = valid && l == ll;
      const unsigned grp = __ballot_sync(FULL, mine);
      uint32_t mn[3], mx[3];
      unsigned long long sm[3];
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) {
        mn[ax] = __reduce_min_sync(FULL, mine ? c[ax] : 0xFFFFFFFFu);
        mx[ax] = __reduce_max_sync(FULL, mine ? c[ax] : 0u);
        sm[ax] = warp_sum64(mine ? (unsigned long long)c[ax] : 0ull);
      }
      if (lane == leader) {
        atomicAdd(a.counts + ll, (uint32_t)__popc(grp));
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
          atomicMin(a.bmin + ll * 3 + ax, mn[ax]);
          atomicMax(a.bmax + ll * 3 + ax, mx[ax]);
          atomicAdd(a.sums + ll * 3 + ax, sm[ax]);
        }
      }
      active &= ~grp;
    }
  }
}

template <typename B>
__global__ void k_stats_finalize(StatsArgs a, B* bboxes, double* centroids) {
  const int64_t n = (int64_t)a.N + 1;
  const int nd = a.ndim;
  const uint32_t bmax_t = sizeof(B) == 2 ? 0xFFFFu : 0xFFFFFFFFu;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t cnt = a.counts[i];
    for (int ax = 0; ax < nd; ++ax) {
      const uint32_t lo = a.bmin[i * 3 + ax];
      bboxes[i * 2 * nd + 2 * ax] = (B)(lo > bmax_t ? bmax_t : lo);
      bboxes[i * 2 * nd + 2 * ax + 1] = (B)a.bmax[i * 3 + ax];
      centroids[i * nd + ax] = cnt == 0 ? __longlong_as_double(0x7FF8000000000000LL)
                                        : (double)a.sums[i * 3 + ax] / (double)cnt;
    }
  }
}

cudaError_t launch_stats(const StatsArgs& a, cudaStream_t s) {
  const int64_t n1 = (int64_t)a.N + 1;
  int64_t blocks = (n1 + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_stats_init<<<(unsigned)blocks, 256, 0, s>>>(a.counts, a.bmin, a.bmax, a.sums, n1);
  const int64_t n = a.d0 * a.d1 * a.d2;
  int64_t vb = (n + 255) / 256;
  if (vb > 152 * 32) vb = 152 * 32;
  if (vb < 1) vb = 1;
  switch (a.dtype) {
    case 1: k_stats<uint8_t><<<(unsigned)vb, 256, 0, s>>>(a); break;
    case 2: k_stats<uint16_t><<<(unsigned)vb, 256, 0, s>>>(a); break;
    case 3: k_stats<uint32_t><<<(unsigned)vb, 256, 0, s>>>(a); break;
    case 4: k_stats<uint64_t><<<(unsigned)vb, 256, 0, s>>>(a); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_stats_finalize(const StatsArgs& a, void* bboxes, int bbox_dtype,
                                  double* centroids, cudaStream_t s) {
  const int64_t n1 = (int64_t)a.N + 1;
  int64_t blocks = (n1 + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (bbox_dtype == 2) k_stats_finalize<uint16_t><<<(unsigned)blocks, 256, 0, s>>>(a, (uint16_t*)bboxes, centroids);
  else k_stats_finalize<uint32_t><<<(unsigned)blocks, 256, 0, s>>>(a, (uint32_t*)bboxes, centroids);
  return cudaGetLastError();
}

}  // namespace cc3dgpu
