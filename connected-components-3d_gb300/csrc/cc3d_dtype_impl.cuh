// cc3d_dtype_impl.cuh -- element-type dependent kernels and their launchers.
// Included once per element type by label_<type>.cu, which instantiates the
// launchers declared in cc3d_internal.h through CC3D_DEFINE_DTYPE_LAUNCHERS.
#pragma once

#include <cstring>
#include <type_traits>

#include "cc3d_internal.h"

namespace cc3dgpu {

constexpr unsigned ERR_NAN = 16u;
constexpr unsigned ERR_OVERFLOW = 32u;

// ------------------------------------------------------------------ epl
// Provisional-label estimate: per row, [v[0] != 0] + #{x >= 1 : v[x] != v[x-1]
// and v[x] != 0}, and the first/last row holding foreground
// (cc3d/cc3d.hpp:287-315).  Work items are 1024-voxel segments of rows.
template <typename T>
__global__ void __launch_bounds__(256) k_epl(const T* in, int64_t sx, int64_t rows, Counters* ctr) {
  constexpr int SEG = 1024;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t segs = (sx + SEG - 1) / SEG;
  const int64_t items = rows * segs;
  unsigned long long acc = 0;
  long long f = 0x7FFFFFFFFFFFFFFFLL, l = -1;
  for (int64_t it = (int64_t)blockIdx.x * 8 + warp; it < items; it += (int64_t)gridDim.x * 8) {
    const int64_t row = it / segs, seg = it % segs;
    const T* rp = in + row * sx;
    const int64_t xs = seg * SEG, xe = (xs + SEG < sx) ? xs + SEG : sx;
    T carry = (xs > 0) ? rp[xs - 1] : T(0);
    unsigned cnt = 0;
    for (int64_t xb = xs; xb < xe; xb += 32) {
      const int64_t x = xb + lane;
      const T v = (x < xe) ? rp[x] : T(0);
      T prev = __shfl_up_sync(FULL, v, 1);
      if (lane == 0) prev = carry;
      cnt += __popc(__ballot_sync(FULL, (x < xe) && (v != prev) && (v != T(0))));
      carry = __shfl_sync(FULL, v, 31);
    }
    if (cnt) {
      acc += cnt;
      f = row < f ? row : f;
      l = row > l ? row : l;
    }
  }
  __shared__ unsigned long long sa[8];
  __shared__ long long sf[8], sl[8];
  if (lane == 0) { sa[warp] = acc; sf[warp] = f; sl[warp] = l; }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long a = 0;
    for (int w = 0; w < 8; ++w) {
      a += sa[w];
      f = sf[w] < f ? sf[w] : f;
      l = sl[w] > l ? sl[w] : l;
    }
    if (a) {
      atomicAdd(&ctr->epl, a);
      atomicMin(&ctr->first_row, f);
      atomicMax(&ctr->last_row, l);
    }
  }
}

// ------------------------------------------------------------ special row
// Single foreground row, labelled run by run with the previous run's value
// held as a C int64, exactly like the reference's Python loop
// (cc3d/fastcc3d.pyx:644-679).  Sequential by nature (a run continues while
// values equal the truncated value that opened it), so one thread does it.
template <typename T>
__device__ __forceinline__ bool to_int64(T v, int is_uint64, long long& out, unsigned& err) {
  if (sizeof(T) == 8 && (T)0.5 == T(0) && is_uint64) {  // unsigned 64-bit input
    if ((unsigned long long)v >= 0x8000000000000000ull) { err |= ERR_OVERFLOW; return false; }
    out = (long long)v;
    return true;
  }
  if ((T)0.5 != T(0)) {  // floating point
    const double d = (double)v;
    if (d != d) { err |= ERR_NAN; return false; }
    if (!(d > -9223372036854775809.0 && d < 9223372036854775808.0)) { err |= ERR_OVERFLOW; return false; }
    out = (long long)d;  // truncation, like Python's int()
    return true;
  }
  out = (long long)v;
  return true;
}

template <typename T, typename OUT>
__global__ void k_special_row(const T* in, int64_t sx, int64_t row, int is_uint64, OUT* out,
                              Counters* ctr) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const T* rp = in + row * sx;
  OUT* op = out + row * sx;
  unsigned long long N = 0;
  long long last = 0;
  unsigned err = 0;
  const bool is_float = (T)0.5 != T(0);
  for (int64_t i = 0; i < sx; ++i) {
    const T v = rp[i];
    if (v == T(0)) { last = 0; continue; }
    const bool same = is_float ? ((double)v == (double)last)
                               : ((unsigned long long)v == (unsigned long long)last);
    if (same) { op[i] = (OUT)N; continue; }
    ++N;
    op[i] = (OUT)N;
    if (!to_int64<T>(v, is_uint64, last, err)) break;
  }
  ctr->N = N;
  if (err) atomicOr(&ctr->err, err);
}

// ----------------------------------------------------------------- minmax
template <typename T>
__global__ void k_minmax_init(unsigned long long* res, int is_signed) {
  if (is_signed) {
    ((long long*)res)[0] = (long long)0x8000000000000000ull;
    ((long long*)res)[1] = 0x7FFFFFFFFFFFFFFFLL;
  } else {
    res[0] = 0;
    res[1] = ~0ull;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_minmax(const T* in, int64_t n, int is_signed,
                                                unsigned long long* res) {
  using ST = typename std::conditional<sizeof(T) == 1, int8_t,
             typename std::conditional<sizeof(T) == 2, int16_t,
             typename std::conditional<sizeof(T) == 4, int32_t, int64_t>::type>::type>::type;
  long long smax = (long long)0x8000000000000000ull, smin = 0x7FFFFFFFFFFFFFFFLL;
  unsigned long long umax = 0, umin = ~0ull;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T v = in[i];
    if (is_signed) {
      ST s;
      memcpy(&s, &v, sizeof(T));
      const long long w = (long long)s;
      smax = w > smax ? w : smax;
      smin = w < smin ? w : smin;
    } else {
      const unsigned long long w = (unsigned long long)v;
      umax = w > umax ? w : umax;
      umin = w < umin ? w : umin;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    smax = max(smax, (long long)__shfl_down_sync(FULL, smax, o));
    smin = min(smin, (long long)__shfl_down_sync(FULL, smin, o));
    umax = max(umax, (unsigned long long)__shfl_down_sync(FULL, umax, o));
    umin = min(umin, (unsigned long long)__shfl_down_sync(FULL, umin, o));
  }
  if ((threadIdx.x & 31) == 0) {
    if (is_signed) {
      atomicMax((long long*)res, smax);
      atomicMin((long long*)res + 1, smin);
    } else {
      atomicMax(res, umax);
      atomicMin(res + 1, umin);
    }
  }
}

// ------------------------------------------------------------- launchers
template <typename T>
constexpr CUtensorMapDataType tma_type() {
  return sizeof(T) == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8
         : sizeof(T) == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16
         : sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT32
                          : CU_TENSOR_MAP_DATA_TYPE_UINT64;
}

// A tensor map over the input for boxes of bw x bh x bd voxels, when the
// volume allows TMA: a 16-byte aligned base and rows whose byte length is a
// multiple of 16 (the copy engine's stride rule), one volume (a batch of
// volumes has one base per volume).  Returns 1 if the map was made; with 0
// the kernels load their boxes with plain loads.
template <typename T>
int encode_input_map(const LabelArgs& a, uint32_t bw, uint32_t bh, uint32_t bd, CUtensorMap* map) {
  memset(map, 0, sizeof(*map));
  const bool aligned = !a.vols && !a.no_tma && ((uintptr_t)a.in & 15u) == 0 && (a.sx * (int64_t)sizeof(T)) % 16 == 0 &&
                       a.sx < (1ll << 31) && a.sy < (1ll << 31) && a.sz < (1ll << 31);
  if (!aligned) return 0;
  using Encode = decltype(&cuTensorMapEncodeTiled);
  Encode enc = reinterpret_cast<Encode>(tensor_map_encoder());
  if (!enc) return 0;
  const cuuint64_t dims[3] = {(cuuint64_t)a.sx, (cuuint64_t)a.sy, (cuuint64_t)a.sz};
  const cuuint64_t strides[2] = {(cuuint64_t)(a.sx * sizeof(T)), (cuuint64_t)(a.sx * a.sy * sizeof(T))};
  const cuuint32_t box[3] = {bw, bh, bd};
  const cuuint32_t estr[3] = {1u, 1u, 1u};
  return enc(map, tma_type<T>(), 3, const_cast<void*>(a.in), dims, strides, box, estr,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the block-parallel pass: one CTA of 256 threads per tile, its box staged by
// one TMA copy
template <typename T, int CONN, int TY, int TZ, int MODE, bool BLOCK8>
cudaError_t launch_k1_runs(const LabelArgs& a, int64_t ntiles, cudaStream_t s) {
  using B = TileBox<CONN, TY, TZ>;
  CUtensorMap map;
  const int use_tma =
      ntiles > 0 ? encode_input_map<T>(a, (uint32_t)BoxRow<T>::W, (uint32_t)B::BY, (uint32_t)B::BZ, &map) : 0;
  k_tile_runs<T, CONN, TY, TZ, MODE, BLOCK8><<<(unsigned)ntiles, kThreads, 0, s>>>(a, map, use_tma);
  return cudaGetLastError();
}

// the list pass (multilabel and binary relations): one CTA of 256 threads per
// tile, its box staged by one TMA copy where the volume allows (else by
// plain loads, a kernel of its own)
template <typename T, int CONN, int TY, int TZ, int MODE>
cudaError_t launch_k1_list(const LabelArgs& a, int64_t ntiles, cudaStream_t s) {
  using B = TileBox<CONN, TY, TZ>;
  CUtensorMap map;
  const int use_tma =
      ntiles > 0 ? encode_input_map<T>(a, (uint32_t)BoxRow<T>::W, (uint32_t)B::BY, (uint32_t)B::BZ, &map) : 0;
  if (use_tma) k_tile_list<T, CONN, TY, TZ, MODE, true><<<(unsigned)ntiles, kThreads, 0, s>>>(a, map);
  else k_tile_list<T, CONN, TY, TZ, MODE, false><<<(unsigned)ntiles, kThreads, 0, s>>>(a, map);
  return cudaGetLastError();
}

// the list pass serves the multilabel and binary relations; the reference's
// binary 4-connected relation runs on the run-union pass
template <typename T, int CONN, int TY, int TZ, int MODE>
cudaError_t launch_k1(const LabelArgs& a, int64_t ntiles, int variant, cudaStream_t s) {
  if constexpr (MODE == MODE_MULTI || MODE == MODE_BINARY)
    if (variant == TILE_PASS_LIST) return launch_k1_list<T, CONN, TY, TZ, MODE>(a, ntiles, s);
  return launch_k1_runs<T, CONN, TY, TZ, MODE, false>(a, ntiles, s);
}

// 3D tiles of 2048 voxels: 32 x TY x TZ with TY * TZ = 64
template <typename T, int CONN, int MODE>
cudaError_t launch_k1_3d(const LabelArgs& a, int64_t ntiles, int variant, cudaStream_t s) {
  if (a.ty == 8 && a.tz == 8) return launch_k1<T, CONN, 8, 8, MODE>(a, ntiles, variant, s);
  if (a.ty == 4 && a.tz == 16) return launch_k1<T, CONN, 4, 16, MODE>(a, ntiles, variant, s);
  if (a.ty == 16 && a.tz == 4) return launch_k1<T, CONN, 16, 4, MODE>(a, ntiles, variant, s);
  return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t launch_tile_local_t(const LabelArgs& a, int conn, int mode, bool block8, int variant,
                                int64_t ntiles, cudaStream_t s) {
  const bool d3 = conn == 26 || conn == 18 || conn == 6;
  if (!d3 && (a.ty != 64 || a.tz != 1)) return cudaErrorInvalidValue;
  if (mode == MODE_GRAPH) {
    // voxel connectivity graphs are uint8 or uint32 bitfields
    if constexpr (std::is_same<T, uint8_t>::value || std::is_same<T, uint32_t>::value) {
      switch (conn) {
        case 26: return launch_k1_runs<T, 26, 8, 8, MODE_GRAPH, false>(a, ntiles, s);
        case 6: return launch_k1_runs<T, 6, 8, 8, MODE_GRAPH, false>(a, ntiles, s);
        case 8: return launch_k1_runs<T, 8, 64, 1, MODE_GRAPH, false>(a, ntiles, s);
        case 4: return launch_k1_runs<T, 4, 64, 1, MODE_GRAPH, false>(a, ntiles, s);
      }
    }
    return cudaErrorInvalidValue;
  }
  if (mode == MODE_CONT8Q) {
    if (conn != 8) return cudaErrorInvalidValue;
    return launch_k1_runs<T, 8, 64, 1, MODE_CONT8Q, false>(a, ntiles, s);
  }
  if (mode == MODE_CONT) {
    // continuous values: block-parallel pass, 32 x 8 x 8 tiles
    if (d3 && (a.ty != 8 || a.tz != 8)) return cudaErrorInvalidValue;
    switch (conn) {
      case 26: return launch_k1_runs<T, 26, 8, 8, MODE_CONT, false>(a, ntiles, s);
      case 18: return launch_k1_runs<T, 18, 8, 8, MODE_CONT, false>(a, ntiles, s);
      case 6: return launch_k1_runs<T, 6, 8, 8, MODE_CONT, false>(a, ntiles, s);
      case 8: return launch_k1_runs<T, 8, 64, 1, MODE_CONT, false>(a, ntiles, s);
      case 4: return launch_k1_runs<T, 4, 64, 1, MODE_CONT, false>(a, ntiles, s);
    }
    return cudaErrorInvalidValue;
  }
  const bool multi = mode == MODE_MULTI;
  switch (conn) {
    case 26:
      return multi ? launch_k1_3d<T, 26, MODE_MULTI>(a, ntiles, variant, s)
                   : launch_k1_3d<T, 26, MODE_BINARY>(a, ntiles, variant, s);
    case 18:
      return multi ? launch_k1_3d<T, 18, MODE_MULTI>(a, ntiles, variant, s)
                   : launch_k1_3d<T, 18, MODE_BINARY>(a, ntiles, variant, s);
    case 6:
      return multi ? launch_k1_3d<T, 6, MODE_MULTI>(a, ntiles, variant, s)
                   : launch_k1_3d<T, 6, MODE_BINARY>(a, ntiles, variant, s);
    case 8:
      // binary 8-connected images are numbered by 2x2 blocks: block-parallel pass only
      if (block8) return launch_k1_runs<T, 8, 64, 1, MODE_BINARY, true>(a, ntiles, s);
      return multi ? launch_k1<T, 8, 64, 1, MODE_MULTI>(a, ntiles, variant, s)
                   : launch_k1<T, 8, 64, 1, MODE_BINARY>(a, ntiles, variant, s);
    case 4:
      if (mode == MODE_BINARY4) return launch_k1<T, 4, 64, 1, MODE_BINARY4>(a, ntiles, variant, s);
      return multi ? launch_k1<T, 4, 64, 1, MODE_MULTI>(a, ntiles, variant, s)
                   : launch_k1<T, 4, 64, 1, MODE_BINARY>(a, ntiles, variant, s);
  }
  return cudaErrorInvalidValue;
}

template <typename T>
cudaError_t launch_wrap_t(const LabelArgs& a, int conn, int mode, cudaStream_t s) {
  const int64_t n = a.sy * a.sz + a.sx * a.sz + (conn == 6 ? a.sx * a.sy : 0) + 2;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  if (mode == MODE_MULTI) k_wrap_pairs<T, MODE_MULTI><<<(unsigned)blocks, 256, 0, s>>>(a, conn);
  else k_wrap_pairs<T, MODE_BINARY><<<(unsigned)blocks, 256, 0, s>>>(a, conn);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_epl_t(const void* in, int64_t sx, int64_t voxels, Counters* ctr, cudaStream_t s) {
  const int64_t rows = sx ? voxels / sx : 0;
  const int64_t items = rows * ((sx + 1023) / 1024);
  int64_t blocks = (items + 7) / 8;
  if (blocks > 152 * 32) blocks = 152 * 32;
  if (blocks < 1) blocks = 1;
  k_epl<T><<<(unsigned)blocks, 256, 0, s>>>(static_cast<const T*>(in), sx, rows, ctr);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_special_row_t(const void* in, int64_t sx, int64_t row, int is_uint64, void* out,
                                 int out_dtype, Counters* ctr, cudaStream_t s) {
  const T* tin = static_cast<const T*>(in);
  switch (out_dtype) {
    case 2: k_special_row<T, uint16_t><<<1, 1, 0, s>>>(tin, sx, row, is_uint64, (uint16_t*)out, ctr); break;
    case 3: k_special_row<T, uint32_t><<<1, 1, 0, s>>>(tin, sx, row, is_uint64, (uint32_t*)out, ctr); break;
    case 4: k_special_row<T, uint64_t><<<1, 1, 0, s>>>(tin, sx, row, is_uint64, (uint64_t*)out, ctr); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_minmax_t(const void* in, int64_t n, int is_signed, unsigned long long* res,
                            cudaStream_t s) {
  k_minmax_init<T><<<1, 1, 0, s>>>(res, is_signed);
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  k_minmax<T><<<(unsigned)blocks, 256, 0, s>>>(static_cast<const T*>(in), n, is_signed, res);
  return cudaGetLastError();
}

// ------------------------------------------------------------ image span
// The minimum and maximum the reference's continuous 2D 8-connected labeller
// folds over the whole image with std::min / std::max from element 0
// (cc3d/cc3d_continuous.hpp:275-280).  For floating point a NaN element makes
// the running value NaN and the next element replaces it, so the fold equals
// the plain minimum and maximum of the elements after the last NaN (NaN when
// the last element is NaN).  res[0], res[1]: minimum and maximum as element
// bits; res[2]: index of the last NaN (-1 if none); res[3]: scratch.
template <typename T>
__device__ __forceinline__ unsigned long long order_key(T v) {
  if constexpr (std::is_floating_point<T>::value) {
    using U = typename std::conditional<sizeof(T) == 4, uint32_t, uint64_t>::type;
    U u;
    memcpy(&u, &v, sizeof(T));
    const U sign = U(1) << (8 * sizeof(T) - 1);
    return (unsigned long long)((u & sign) ? U(~u) : U(u | sign));
  } else {
    return (unsigned long long)v;
  }
}
template <typename T>
__device__ __forceinline__ uint64_t key_bits(unsigned long long k) {
  if constexpr (std::is_floating_point<T>::value) {
    using U = typename std::conditional<sizeof(T) == 4, uint32_t, uint64_t>::type;
    const U sign = U(1) << (8 * sizeof(T) - 1);
    const U u = (U)k;
    return (uint64_t)((u & sign) ? U(u & ~sign) : U(~u));
  } else {
    return (uint64_t)k;
  }
}

template <typename T>
__global__ void k_span_init(unsigned long long* res) {
  res[0] = ~0ull;
  res[1] = 0;
  res[2] = (unsigned long long)-1ll;
  res[3] = 0;
}

template <typename T>
__global__ void __launch_bounds__(256) k_span_last_nan(const T* in, int64_t n, unsigned long long* res) {
  long long last = -1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (in[i] != in[i]) last = i;
  for (int o = 16; o > 0; o >>= 1) last = max(last, (long long)__shfl_down_sync(FULL, last, o));
  if ((threadIdx.x & 31) == 0 && last >= 0) atomicMax((long long*)&res[2], last);
}

template <typename T>
__global__ void __launch_bounds__(256) k_span(const T* in, int64_t n, unsigned long long* res) {
  const int64_t first = (long long)res[2] + 1;
  unsigned long long kmin = ~0ull, kmax = 0;
  for (int64_t i = first + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long k = order_key<T>(in[i]);
    kmin = k < kmin ? k : kmin;
    kmax = k > kmax ? k : kmax;
  }
  for (int o = 16; o > 0; o >>= 1) {
    kmin = min(kmin, (unsigned long long)__shfl_down_sync(FULL, kmin, o));
    kmax = max(kmax, (unsigned long long)__shfl_down_sync(FULL, kmax, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&res[0], kmin);
    atomicMax(&res[1], kmax);
  }
}

template <typename T>
__global__ void k_span_final(unsigned long long* res, int64_t n) {
  if constexpr (std::is_floating_point<T>::value) {
    if ((long long)res[2] + 1 >= n) {
      // nothing after the last NaN: both folds end in NaN
      const T nan = T(NAN);
      uint64_t b = 0;
      memcpy(&b, &nan, sizeof(T));
      res[0] = b;
      res[1] = b;
      return;
    }
  }
  res[0] = key_bits<T>(res[0]);
  res[1] = key_bits<T>(res[1]);
}

template <typename T>
cudaError_t launch_span_t(const void* in, int64_t n, unsigned long long* res, cudaStream_t s) {
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 8) blocks = 152 * 8;
  if (blocks < 1) blocks = 1;
  const T* p = static_cast<const T*>(in);
  k_span_init<T><<<1, 1, 0, s>>>(res);
  if (std::is_floating_point<T>::value) k_span_last_nan<T><<<(unsigned)blocks, 256, 0, s>>>(p, n, res);
  k_span<T><<<(unsigned)blocks, 256, 0, s>>>(p, n, res);
  k_span_final<T><<<1, 1, 0, s>>>(res, n);
  return cudaGetLastError();
}

}  // namespace cc3dgpu

#define CC3D_DEFINE_DTYPE_LAUNCHERS(SUF, T)                                               \
  namespace cc3dgpu {                                                                     \
  cudaError_t launch_tile_local_##SUF(const LabelArgs& a, int conn, int mode, bool block8,  \
                                      int variant, int64_t ntiles, cudaStream_t s) {      \
    return launch_tile_local_t<T>(a, conn, mode, block8, variant, ntiles, s);             \
  }                                                                                       \
  cudaError_t launch_wrap_##SUF(const LabelArgs& a, int conn, int mode, cudaStream_t s) { \
    return launch_wrap_t<T>(a, conn, mode, s);                                            \
  }                                                                                       \
  cudaError_t launch_epl_##SUF(const void* in, int64_t sx, int64_t voxels, Counters* ctr, \
                               cudaStream_t s) {                                          \
    return launch_epl_t<T>(in, sx, voxels, ctr, s);                                       \
  }                                                                                       \
  cudaError_t launch_special_row_##SUF(const void* in, int64_t sx, int64_t row,          \
                                       int is_uint64, void* out, int out_dtype,           \
                                       Counters* ctr, cudaStream_t s) {                   \
    return launch_special_row_t<T>(in, sx, row, is_uint64, out, out_dtype, ctr, s);       \
  }                                                                                       \
  cudaError_t launch_minmax_##SUF(const void* in, int64_t n, int is_signed,               \
                                  unsigned long long* res, cudaStream_t s) {              \
    return launch_minmax_t<T>(in, n, is_signed, res, s);                                  \
  }                                                                                       \
  cudaError_t launch_span_##SUF(const void* in, int64_t n, unsigned long long* res,       \
                                cudaStream_t s) {                                         \
    return launch_span_t<T>(in, n, res, s);                                               \
  }                                                                                       \
  }
