// cc3d_stats.cu -- per-label voxel counts, bounding boxes and centroids
// (replaces _statistics_helper2d/3d, cc3d/fastcc3d.pyx:767-938).
//
// One pass over the labels in memory order.  Each warp groups its 32 voxels
// by label (usually one or two labels: labels come in runs), reduces count,
// per-axis min/max and per-axis coordinate sums inside the group, and one lane
// per group adds them in.  Frequent labels would serialise their atomics on a
// few global addresses (label 0, the background, lies in most warps of a
// labelled volume; a giant component in most warps of a dense binary one), so
// every block keeps a few labels in shared memory: slot 0 holds label 0, the
// others are claimed first come by the labels that hash to them, and the block
// adds its slots into the global tables once at the end.  Min, max and sums do
// not depend on the order of their terms, so the tables are the same.
// Coordinate sums are exact 64-bit integers; the finaliser divides them in
// FP64, which reproduces the reference's one-by-one double accumulation bit
// for bit while the sums stay below 2^53.
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

constexpr int kStatSlots = 32;                 // labels kept in shared memory per block
constexpr unsigned long long kFreeSlot = ~0ull;  // no label exceeds the voxel count

// WIDE: some axis is 2^27 or longer, so a warp's sum of 32 coordinates may
// not fit 32 bits and is reduced in 64 bits.
template <typename L, bool WIDE>
__global__ void __launch_bounds__(256) k_stats(StatsArgs a) {
  __shared__ unsigned long long s_lab[kStatSlots];
  __shared__ uint32_t s_cnt[kStatSlots], s_min[kStatSlots][3], s_max[kStatSlots][3];
  __shared__ unsigned long long s_sum[kStatSlots][3];
  for (int k = threadIdx.x; k < kStatSlots; k += blockDim.x) {
    s_lab[k] = k == 0 ? 0ull : kFreeSlot;
    s_cnt[k] = 0;
    for (int ax = 0; ax < 3; ++ax) {
      s_min[k][ax] = 0xFFFFFFFFu;
      s_max[k][ax] = 0;
      s_sum[k][ax] = 0;
    }
  }
  __syncthreads();

  const L* lab = static_cast<const L*>(a.labels);
  const int64_t n = a.d0 * a.d1 * a.d2;
  const int lane = threadIdx.x & 31;
  // coordinates in memory order (q0 fastest), advanced by the grid stride
  // with carries instead of a division per voxel
  const int64_t m0 = a.c_order ? a.d2 : a.d0, m1 = a.d1;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t s0 = stride % m0, s1 = (stride / m0) % m1, s2 = (stride / m0) / m1;
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int64_t q0 = i % m0, q1 = (i / m0) % m1, q2 = (i / m0) / m1;
  for (int64_t base = i - lane; base < n; base += stride) {
    const bool valid = i < n;
    const unsigned long long l = valid ? (unsigned long long)lab[i] : 0;
    uint32_t c[3];
    if (a.c_order) {
      c[0] = (uint32_t)q2; c[1] = (uint32_t)q1; c[2] = (uint32_t)q0;
    } else {
      c[0] = (uint32_t)q0; c[1] = (uint32_t)q1; c[2] = (uint32_t)q2;
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
        if constexpr (WIDE) sm[ax] = warp_sum64(mine ? (unsigned long long)c[ax] : 0ull);
        else sm[ax] = __reduce_add_sync(FULL, mine ? c[ax] : 0u);
      }
      if (lane == leader && ll > a.N) {
        // a label above the caller's N has no table row: skip it and report
        atomicOr(a.err, 1u);
      } else if (lane == leader) {
        int slot = -1;
        if (ll == 0) {
          slot = 0;
        } else {
          const int h = 1 + (int)(((ll * 0x9E3779B97F4A7C15ull) >> 59) % (kStatSlots - 1));
          const unsigned long long cur = *(volatile unsigned long long*)&s_lab[h];
          if (cur == ll) {
            slot = h;
          } else if (cur == kFreeSlot) {
            const unsigned long long old = atomicCAS(&s_lab[h], kFreeSlot, ll);
            if (old == kFreeSlot || old == ll) slot = h;
          }
        }
        const uint32_t cnt = (uint32_t)__popc(grp);
        if (slot >= 0) {
          atomicAdd(&s_cnt[slot], cnt);
#pragma unroll
          for (int ax = 0; ax < 3; ++ax) {
            atomicMin(&s_min[slot][ax], mn[ax]);
            atomicMax(&s_max[slot][ax], mx[ax]);
            atomicAdd(&s_sum[slot][ax], sm[ax]);
          }
        } else {
          atomicAdd(a.counts + ll, cnt);
#pragma unroll
          for (int ax = 0; ax < 3; ++ax) {
            atomicMin(a.bmin + ll * 3 + ax, mn[ax]);
            atomicMax(a.bmax + ll * 3 + ax, mx[ax]);
            atomicAdd(a.sums + ll * 3 + ax, sm[ax]);
          }
        }
      }
      active &= ~grp;
    }
    i += stride;
    q0 += s0;
    int carry = 0;
    if (q0 >= m0) { q0 -= m0; carry = 1; }
    q1 += s1 + carry;
    if (q1 >= m1) { q1 -= m1; q2 += 1; }
    q2 += s2;
  }

  // the block's slots into the global tables
  __syncthreads();
  for (int k = threadIdx.x; k < kStatSlots; k += blockDim.x) {
    const uint32_t cnt = s_cnt[k];
    if (!cnt) continue;
    const unsigned long long ll = s_lab[k];
    atomicAdd(a.counts + ll, cnt);
    for (int ax = 0; ax < 3; ++ax) {
      atomicMin(a.bmin + ll * 3 + ax, s_min[k][ax]);
      atomicMax(a.bmax + ll * 3 + ax, s_max[k][ax]);
      atomicAdd(a.sums + ll * 3 + ax, s_sum[k][ax]);
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
  const bool wide = a.d0 >= (1 << 27) || a.d1 >= (1 << 27) || a.d2 >= (1 << 27);
  switch (a.dtype * 2 + (wide ? 1 : 0)) {
    case 2: k_stats<uint8_t, false><<<(unsigned)vb, 256, 0, s>>>(a); break;
    case 3: k_stats<uint8_t, true><<<(unsigned)vb, 256, 0, s>>>(a); break;
    case 4: k_stats<uint16_t, false><<<(unsigned)vb, 256, 0, s>>>(a); break;
    case 5: k_stats<uint16_t, true><<<(unsigned)vb, 256, 0, s>>>(a); break;
    case 6: k_stats<uint32_t, false><<<(unsigned)vb, 256, 0, s>>>(a); break;
    case 7: k_stats<uint32_t, true><<<(unsigned)vb, 256, 0, s>>>(a); break;
    case 8: k_stats<uint64_t, false><<<(unsigned)vb, 256, 0, s>>>(a); break;
    case 9: k_stats<uint64_t, true><<<(unsigned)vb, 256, 0, s>>>(a); break;
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
