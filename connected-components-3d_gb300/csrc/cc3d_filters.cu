// cc3d_filters.cu -- per-label rewrites of a labelled volume, on the device:
// the element-wise halves of cc3d.dust and cc3d.largest_k
// (cc3d/__init__.py:71-155, 199-279).  The per-label decisions (which labels
// are dust, which are the k largest) are made on the small count table by the
// caller; these kernels apply them to every voxel.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "cc3d_gpu.h"
#include "cc3d_internal.h"

using namespace cc3dgpu;

namespace {

int failf(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int failf(int code, const char* fmt, ...) {
  char buf[256];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return api_fail(code, buf);
}

#define CKF(call)                                                                                \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return failf(CC3D_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <int B> struct UInt;
template <> struct UInt<1> { using type = uint8_t; };
template <> struct UInt<2> { using type = uint16_t; };
template <> struct UInt<4> { using type = uint32_t; };
template <> struct UInt<8> { using type = uint64_t; };

// out[i] = table[labels[i]]; a label outside the table sets *bad
template <typename L, typename O>
__global__ void __launch_bounds__(256) k_remap(const L* __restrict__ labels, int64_t n, const O* __restrict__ table,
                                               uint64_t tlen, O* __restrict__ out, unsigned* bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t l = (uint64_t)labels[i];
    O v = O(0);
    if (l < tlen) v = table[l];
    else atomicOr(bad, 1u);
    out[i] = v;
  }
}

// image[i] = 0 where zero[labels[i]] is set
template <typename I, typename L>
__global__ void __launch_bounds__(256) k_zero(I* __restrict__ image, const L* __restrict__ labels, int64_t n,
                                              const uint8_t* __restrict__ zero, uint64_t tlen, unsigned* bad) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t l = (uint64_t)labels[i];
    if (l < tlen) {
      if (zero[l]) image[i] = I(0);
    } else {
      atomicOr(bad, 1u);
    }
  }
}

unsigned grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  return (unsigned)(b < 1 ? 1 : b);
}

template <int LB, int OB>
void launch_remap(const void* labels, int64_t n, const void* table, uint64_t tlen, void* out, unsigned* bad,
                  cudaStream_t s) {
  using L = typename UInt<LB>::type;
  using O = typename UInt<OB>::type;
  k_remap<L, O><<<grid_for(n), 256, 0, s>>>((const L*)labels, n, (const O*)table, tlen, (O*)out, bad);
}

template <int IB, int LB>
void launch_zero(void* image, const void* labels, int64_t n, const uint8_t* zero, uint64_t tlen, unsigned* bad,
                 cudaStream_t s) {
  using I = typename UInt<IB>::type;
  using L = typename UInt<LB>::type;
  k_zero<I, L><<<grid_for(n), 256, 0, s>>>((I*)image, (const L*)labels, n, zero, tlen, bad);
}

bool valid_bytes(int b) { return b == 1 || b == 2 || b == 4 || b == 8; }

// small device flag per thread and device for out-of-table labels
thread_local unsigned* g_bad = nullptr;
thread_local int g_bad_dev = -1;
int bad_flag(unsigned** out) {
  int dev = 0;
  CKF(cudaGetDevice(&dev));
  if (!g_bad || g_bad_dev != dev) {
    CKF(cudaMalloc((void**)&g_bad, sizeof(unsigned)));
    g_bad_dev = dev;
  }
  *out = g_bad;
  return CC3D_OK;
}

int finish(unsigned* bad, cudaStream_t s) {
  unsigned h = 0;
  CKF(cudaGetLastError());
  CKF(cudaMemcpyAsync(&h, bad, sizeof(h), cudaMemcpyDeviceToHost, s));
  CKF(cudaStreamSynchronize(s));
  if (h) return failf(CC3D_ERR_INVALID, "a label is larger than the table (labels must be at most N)");
  return CC3D_OK;
}

}  // namespace

extern "C" int cc3d_gpu_remap_labels(const void* labels, int label_bytes, int64_t voxels, const void* table,
                                     int table_bytes, uint64_t table_len, void* out, void* stream) {
  if (!valid_bytes(label_bytes) || !valid_bytes(table_bytes) || voxels < 0 || (voxels && (!labels || !out)) ||
      !table || table_len == 0)
    return failf(CC3D_ERR_INVALID, "invalid arguments");
  if (voxels == 0) return CC3D_OK;
  if (!device_accessible(labels) || !device_accessible(table) || !device_accessible(out))
    return failf(CC3D_ERR_INVALID, "labels, table and output must be device memory");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned* bad;
  if (int rc = bad_flag(&bad)) return rc;
  CKF(cudaMemsetAsync(bad, 0, sizeof(unsigned), s));
#define REMAP_O(LB)                                                                       \
  switch (table_bytes) {                                                                  \
    case 1: launch_remap<LB, 1>(labels, voxels, table, table_len, out, bad, s); break;    \
    case 2: launch_remap<LB, 2>(labels, voxels, table, table_len, out, bad, s); break;    \
    case 4: launch_remap<LB, 4>(labels, voxels, table, table_len, out, bad, s); break;    \
    default: launch_remap<LB, 8>(labels, voxels, table, table_len, out, bad, s); break;   \
  }
  switch (label_bytes) {
    case 1: REMAP_O(1) break;
    case 2: REMAP_O(2) break;
    case 4: REMAP_O(4) break;
    default: REMAP_O(8) break;
  }
#undef REMAP_O
  return finish(bad, s);
}

extern "C" int cc3d_gpu_zero_labels(void* image, int image_bytes, const void* labels, int label_bytes,
                                    int64_t voxels, const uint8_t* zero, uint64_t table_len, void* stream) {
  if (!valid_bytes(label_bytes) || !valid_bytes(image_bytes) || voxels < 0 || (voxels && (!labels || !image)) ||
      !zero || table_len == 0)
    return failf(CC3D_ERR_INVALID, "invalid arguments");
  if (voxels == 0) return CC3D_OK;
  if (!device_accessible(image) || !device_accessible(labels) || !device_accessible(zero))
    return failf(CC3D_ERR_INVALID, "image, labels and table must be device memory");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned* bad;
  if (int rc = bad_flag(&bad)) return rc;
  CKF(cudaMemsetAsync(bad, 0, sizeof(unsigned), s));
#define ZERO_L(IB)                                                                      \
  switch (label_bytes) {                                                                \
    case 1: launch_zero<IB, 1>(image, labels, voxels, zero, table_len, bad, s); break;  \
    case 2: launch_zero<IB, 2>(image, labels, voxels, zero, table_len, bad, s); break;  \
    case 4: launch_zero<IB, 4>(image, labels, voxels, zero, table_len, bad, s); break;  \
    default: launch_zero<IB, 8>(image, labels, voxels, zero, table_len, bad, s); break; \
  }
  switch (image_bytes) {
    case 1: ZERO_L(1) break;
    case 2: ZERO_L(2) break;
    case 4: ZERO_L(4) break;
    default: ZERO_L(8) break;
  }
#undef ZERO_L
  return finish(bad, s);
}
