// cc3d_stack.cu -- the seam merge of connected_components_stack on the device
// (cc3d/__init__.py:324-501).
//
// The caller labels every slab of the stack on its own (local labels 1..n_k)
// and gives slab k the global labels offset_k + 1 .. offset_k + n_k.  The
// seam merge then works on one union-find table over all global labels, held
// in a caller-provided device work area:
//
//   begin    every label is its own group (parent[i] = i)
//   seam     every pair of labels that touch across one seam (the last plane
//            of slab k-1 against the first plane of slab k) joins its groups;
//            a root is only ever linked under a smaller root, so the root of
//            a group is its smallest label -- the reference's DisjointSet
//            (cc3d/__init__.py:296-321) keeps the smaller of two roots too
//   number   each group gets the rank of its smallest label among all the
//            groups' smallest labels (1..N): the reference renumbers the
//            remapped labels in sorted order (crackle.renumber)
//   relabel  out = number of (offset + local label), 0 for background
//
// Every union-find loop is bounded; a loop that runs out, or a label outside
// the table, sets the work area's error word and the call reports it.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include <cuda_fp16.h>

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

#define CKS(call)                                                                                \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return failf(CC3D_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

constexpr int kStackThreads = 256;
constexpr int kWordsPerBlock = 4096;  // bitmap words per block of the numbering scan
constexpr int kStackLimit = 1 << 22;  // iteration limit of every union-find loop
constexpr unsigned kErrBudget = 1u, kErrRange = 2u;

// Layout of the work area for a table of n = total + 1 entries.
struct StackWork {
  unsigned long long* parent;  // [n]: parent, then (number) the group number
  uint32_t* bitmap;            // [words]: one bit per group root
  unsigned long long* prefix;  // [words]: roots before each word
  unsigned long long* bsum;    // [blocks + 1]: roots before each block; [blocks] = N
  unsigned* err;               // [0] error bits, [1] a relabelled voxel was background
  uint64_t n, words, blocks;
};

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

StackWork carve(void* work, uint64_t total, size_t* bytes) {
  StackWork w;
  w.n = total + 1;
  w.words = (w.n + 31) / 32;
  w.blocks = (w.words + kWordsPerBlock - 1) / kWordsPerBlock;
  char* b = (char*)work;
  size_t off = 0;
  w.parent = (unsigned long long*)(b + off);
  off += up256(w.n * 8);
  w.bitmap = (uint32_t*)(b + off);
  off += up256(w.words * 4);
  w.prefix = (unsigned long long*)(b + off);
  off += up256(w.words * 8);
  w.bsum = (unsigned long long*)(b + off);
  off += up256((w.blocks + 1) * 8);
  w.err = (unsigned*)(b + off);
  off += 256;
  if (bytes) *bytes = off;
  return w;
}

__device__ __forceinline__ unsigned long long vload(const unsigned long long* p) {
  return *(const volatile unsigned long long*)p;
}

// root of x (path halving); ~0 on a parent outside the table or when the
// budget runs out (the error word says which)
__device__ unsigned long long sfind64(unsigned long long* P, unsigned long long x, uint64_t n, unsigned* err) {
  for (int it = 0; it < kStackLimit; ++it) {
    const unsigned long long p = vload(P + x);
    if (p == x) return x;
    if (p >= n) break;
    const unsigned long long g = vload(P + p);
    if (g >= n) break;
    if (g != p) *(volatile unsigned long long*)(P + x) = g;
    x = g;
  }
  atomicOr(err, kErrRange);
  return ~0ull;
}

__device__ void sunite64(unsigned long long* P, unsigned long long a, unsigned long long b, uint64_t n,
                         unsigned* err) {
  for (int it = 0; it < kStackLimit; ++it) {
    a = sfind64(P, a, n, err);
    b = sfind64(P, b, n, err);
    if (a == ~0ull || b == ~0ull || a == b) return;
    if (a < b) {
      const unsigned long long t = a;
      a = b;
      b = t;
    }
    // the larger root goes under the smaller one
    if (atomicCAS(P + a, a, b) == a) return;
  }
  atomicOr(err, kErrBudget);
}

__global__ void k_stack_begin(StackWork w) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += (uint64_t)gridDim.x * blockDim.x)
    w.parent[i] = i;
  if (blockIdx.x == 0 && threadIdx.x == 0) w.err[0] = w.err[1] = 0;
}

template <typename I>
__device__ __forceinline__ bool related(I a, I b, bool binary) {
  if (binary) return a != I(0) && b != I(0);
  return a == b;
}
template <>
__device__ __forceinline__ bool related<__half>(__half a, __half b, bool binary) {
  const float fa = __half2float(a), fb = __half2float(b);
  if (binary) return fa != 0.f && fb != 0.f;  // NaN is nonzero
  return fa == fb;
}

template <typename L>
__device__ __forceinline__ unsigned long long global_label(const void* lab, int64_t i, uint64_t off) {
  const unsigned long long l = (unsigned long long)static_cast<const L*>(lab)[i];
  return l ? off + l : 0ull;
}

__device__ __forceinline__ unsigned long long read_label(const void* lab, int bytes, int64_t i, uint64_t off) {
  switch (bytes) {
    case 1: return global_label<uint8_t>(lab, i, off);
    case 2: return global_label<uint16_t>(lab, i, off);
    case 4: return global_label<uint32_t>(lab, i, off);
    default: return global_label<uint64_t>(lab, i, off);
  }
}

// One thread per voxel of the bottom plane; planes are (sx, sy) with index
// x * sy + y.  6-connectivity: the voxel straight above; 26: the 3 x 3 patch
// above (the reference skips the patch once the voxel straight above joins;
// the patch voxels that relate to the bottom voxel then relate to the one
// above it too, so the groups come out the same).
template <typename I>
__global__ void k_stack_seam(const I* bimg, const I* timg, const void* blab, int bbytes, uint64_t boff,
                             const void* tlab, int tbytes, uint64_t toff, int64_t sx, int64_t sy, int conn,
                             bool binary, StackWork w) {
  const int64_t nvox = sx * sy;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nvox; i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long bl = read_label(blab, bbytes, i, boff);
    if (!bl) continue;
    const I bv = bimg[i];
    const int64_t x = i / sy, y = i - x * sy;
    const int r = conn == 26 ? 1 : 0;
    for (int dx = -r; dx <= r; ++dx) {
      const int64_t xx = x + dx;
      if (xx < 0 || xx >= sx) continue;
      for (int dy = -r; dy <= r; ++dy) {
        const int64_t yy = y + dy;
        if (yy < 0 || yy >= sy) continue;
        const int64_t j = xx * sy + yy;
        if (!related<I>(bv, timg[j], binary)) continue;
        const unsigned long long tl = read_label(tlab, tbytes, j, toff);
        if (!tl) continue;
        if (bl >= w.n || tl >= w.n) {
          atomicOr(w.err, kErrRange);
          continue;
        }
        sunite64(w.parent, bl, tl, w.n, w.err);
      }
    }
  }
}

// every label points at its root; roots set their bit (one warp per bitmap
// word, so every ballot has all 32 lanes)
__global__ void k_stack_flatten(StackWork w) {
  const int lane = threadIdx.x & 31;
  const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  for (uint64_t k = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < w.words; k += nwarps) {
    const uint64_t i = k * 32 + lane;
    bool root = false;
    if (i < w.n) {
      const unsigned long long r = sfind64(w.parent, i, w.n, w.err);
      if (r != ~0ull) w.parent[i] = r;  // an ancestor of i: safe while others still climb through i
      root = (r == i) && i > 0;
    }
    const unsigned m = __ballot_sync(0xFFFFFFFFu, root);
    if (lane == 0) w.bitmap[k] = m;
  }
}

// roots per block of words
__global__ void k_stack_count(StackWork w) {
  __shared__ unsigned long long part[kStackThreads / 32];
  const uint64_t w0 = (uint64_t)blockIdx.x * kWordsPerBlock;
  unsigned long long s = 0;
  for (uint64_t k = w0 + threadIdx.x; k < w0 + kWordsPerBlock && k < w.words; k += kStackThreads)
    s += __popc(w.bitmap[k]);
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int k = 0; k < kStackThreads / 32; ++k) t += part[k];
    w.bsum[blockIdx.x] = t;
  }
}

// exclusive prefix of the block counts (one thread: there are few blocks)
__global__ void k_stack_blocks(StackWork w) {
  unsigned long long run = 0;
  for (uint64_t b = 0; b < w.blocks; ++b) {
    const unsigned long long c = w.bsum[b];
    w.bsum[b] = run;
    run += c;
  }
  w.bsum[w.blocks] = run;
}

// word prefixes inside each block, then every label's number
__global__ void k_stack_words(StackWork w) {
  __shared__ unsigned long long warp_tot[kStackThreads / 32];
  const uint64_t w0 = (uint64_t)blockIdx.x * kWordsPerBlock;
  constexpr int PER = kWordsPerBlock / kStackThreads;
  const uint64_t mine = w0 + (uint64_t)threadIdx.x * PER;
  unsigned c[PER];
  unsigned long long s = 0;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    c[k] = (mine + k < w.words) ? __popc(w.bitmap[mine + k]) : 0u;
    s += c[k];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned long long x = s;
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xFFFFFFFFu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  unsigned long long before = w.bsum[blockIdx.x];
  for (int k = 0; k < warp; ++k) before += warp_tot[k];
  unsigned long long run = before + x - s;
#pragma unroll
  for (int k = 0; k < PER; ++k) {
    if (mine + k < w.words) w.prefix[mine + k] = run;
    run += c[k];
  }
}

__global__ void k_stack_number(StackWork w) {
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < w.n; i += (uint64_t)gridDim.x * blockDim.x) {
    if (i == 0) {
      w.parent[0] = 0;
      continue;
    }
    const unsigned long long r = w.parent[i];  // flattened: the root itself
    unsigned long long num = 0;
    if (r < w.n && r > 0) {
      num = w.prefix[r >> 5] + __popc(w.bitmap[r >> 5] & ((1u << (r & 31)) - 1u)) + 1ull;
    } else {
      atomicOr(w.err, kErrRange);
    }
    w.parent[i] = num;  // i's own entry: no other thread reads it any more
  }
}

// out[x, y, z] = number[offset + label[x, y, z]] (element strides)
template <typename L, typename O>
__global__ void k_stack_relabel(const L* lab, int64_t lsx, int64_t lsy, int64_t lsz, uint64_t off, O* out,
                                int64_t osx, int64_t osy, int64_t osz, int64_t sx, int64_t sy, int64_t sz,
                                StackWork w) {
  const int64_t nvox = sx * sy * sz;
  bool bg = false;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nvox; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = i % sx, rest = i / sx, y = rest % sy, z = rest / sy;
    const unsigned long long l = (unsigned long long)lab[x * lsx + y * lsy + z * lsz];
    O v = O(0);
    if (l) {
      const unsigned long long g = off + l;
      if (g < w.n) v = (O)w.parent[g];
      else atomicOr(w.err, kErrRange);
    }
    out[x * osx + y * osy + z * osz] = v;
    bg = bg || v == O(0);
  }
  if (bg) atomicOr(w.err + 1, 1u);
}

unsigned grid_for(uint64_t n) {
  uint64_t b = (n + kStackThreads - 1) / kStackThreads;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)(b < 1 ? 1 : b);
}

int read_err(const StackWork& w, cudaStream_t s, int* background = nullptr) {
  unsigned hw[2] = {0, 0};
  CKS(cudaGetLastError());
  CKS(cudaMemcpyAsync(hw, w.err, sizeof(hw), cudaMemcpyDeviceToHost, s));
  CKS(cudaStreamSynchronize(s));
  const unsigned h = hw[0];
  if (background) *background = hw[1] ? 1 : 0;
  if (h & kErrRange) return failf(CC3D_ERR_INVALID, "a label lies outside the stack's label table");
  if (h & kErrBudget) return failf(CC3D_ERR_DEVICE, "device error: stack union budget exhausted");
  return CC3D_OK;
}

bool label_width_ok(int b) { return b == 1 || b == 2 || b == 4 || b == 8; }

template <typename L>
int relabel_out(const StackWork& w, const L* lab, const int64_t* ls, uint64_t off, void* out, int out_bytes,
                const int64_t* os, int64_t sx, int64_t sy, int64_t sz, cudaStream_t s) {
  const unsigned g = grid_for((uint64_t)(sx * sy * sz));
#define RL(O) \
  k_stack_relabel<L, O><<<g, kStackThreads, 0, s>>>(lab, ls[0], ls[1], ls[2], off, (O*)out, os[0], os[1], os[2], sx, sy, sz, w)
  switch (out_bytes) {
    case 1: RL(uint8_t); break;
    case 2: RL(uint16_t); break;
    case 4: RL(uint32_t); break;
    default: RL(uint64_t); break;
  }
#undef RL
  return CC3D_OK;
}

}  // namespace

extern "C" uint64_t cc3d_gpu_stack_work_bytes(uint64_t total_labels) {
  size_t bytes = 0;
  carve(nullptr, total_labels, &bytes);
  return bytes;
}

extern "C" int cc3d_gpu_stack_begin(void* work, uint64_t total_labels, void* stream) {
  if (!work || total_labels >= (1ull << 62)) return failf(CC3D_ERR_INVALID, "invalid arguments");
  if (!device_accessible(work)) return failf(CC3D_ERR_INVALID, "the work area must be device memory");
  const StackWork w = carve(work, total_labels, nullptr);
  cudaStream_t s = (cudaStream_t)stream;
  k_stack_begin<<<grid_for(w.n), kStackThreads, 0, s>>>(w);
  CKS(cudaGetLastError());
  return CC3D_OK;
}

extern "C" int cc3d_gpu_stack_seam(const void* bottom_img, const void* top_img, int img_dtype,
                                   const void* bottom_labels, int bottom_label_bytes, uint64_t bottom_offset,
                                   const void* top_labels, int top_label_bytes, uint64_t top_offset, int64_t sx,
                                   int64_t sy, int64_t connectivity, int binary_image, void* work,
                                   uint64_t total_labels, void* stream) {
  if (connectivity != 6 && connectivity != 26)
    return failf(CC3D_ERR_INVALID, "Connectivity must be 6 or 26. Got: %lld", (long long)connectivity);
  if (!work || sx < 0 || sy < 0 || !label_width_ok(bottom_label_bytes) || !label_width_ok(top_label_bytes))
    return failf(CC3D_ERR_INVALID, "invalid arguments");
  if (sx * sy == 0) return CC3D_OK;
  if (!bottom_img || !top_img || !bottom_labels || !top_labels) return failf(CC3D_ERR_INVALID, "null plane");
  if (!device_accessible(bottom_img) || !device_accessible(top_img) || !device_accessible(bottom_labels) ||
      !device_accessible(top_labels) || !device_accessible(work))
    return failf(CC3D_ERR_INVALID, "planes, labels and the work area must be device memory");
  const StackWork w = carve(work, total_labels, nullptr);
  cudaStream_t s = (cudaStream_t)stream;
  const unsigned g = grid_for((uint64_t)(sx * sy));
  const int conn = (int)connectivity;
  const bool bin = binary_image != 0;
#define SEAM(I)                                                                                              \
  k_stack_seam<I><<<g, kStackThreads, 0, s>>>((const I*)bottom_img, (const I*)top_img, bottom_labels,        \
                                              bottom_label_bytes, bottom_offset, top_labels, top_label_bytes, \
                                              top_offset, sx, sy, conn, bin, w)
  switch (img_dtype) {
    case CC3D_U8: SEAM(uint8_t); break;
    case CC3D_U16: SEAM(uint16_t); break;
    case CC3D_U32: SEAM(uint32_t); break;
    case CC3D_U64: SEAM(uint64_t); break;
    case CC3D_F32: SEAM(float); break;
    case CC3D_F64: SEAM(double); break;
    case CC3D_F16: SEAM(__half); break;
    default: return failf(CC3D_ERR_INVALID, "unknown image dtype code %d", img_dtype);
  }
#undef SEAM
  CKS(cudaGetLastError());
  return CC3D_OK;
}

extern "C" int cc3d_gpu_stack_number(void* work, uint64_t total_labels, uint64_t* N, void* stream) {
  if (!work || !N) return failf(CC3D_ERR_INVALID, "invalid arguments");
  if (!device_accessible(work)) return failf(CC3D_ERR_INVALID, "the work area must be device memory");
  const StackWork w = carve(work, total_labels, nullptr);
  cudaStream_t s = (cudaStream_t)stream;
  k_stack_flatten<<<grid_for(w.words * 32), kStackThreads, 0, s>>>(w);
  k_stack_count<<<(unsigned)w.blocks, kStackThreads, 0, s>>>(w);
  k_stack_blocks<<<1, 1, 0, s>>>(w);
  k_stack_words<<<(unsigned)w.blocks, kStackThreads, 0, s>>>(w);
  k_stack_number<<<grid_for(w.n), kStackThreads, 0, s>>>(w);
  unsigned long long n = 0;
  CKS(cudaGetLastError());
  CKS(cudaMemcpyAsync(&n, w.bsum + w.blocks, sizeof(n), cudaMemcpyDeviceToHost, s));
  if (int rc = read_err(w, s)) return rc;
  *N = n;
  return CC3D_OK;
}

extern "C" int cc3d_gpu_stack_relabel(const void* labels, int label_bytes, const int64_t* label_strides,
                                      uint64_t offset, void* out, int out_bytes, const int64_t* out_strides,
                                      int64_t sx, int64_t sy, int64_t sz, void* work, uint64_t total_labels,
                                      int* has_background, void* stream) {
  if (!label_width_ok(label_bytes) || !label_width_ok(out_bytes) || !label_strides || !out_strides || !work ||
      sx < 0 || sy < 0 || sz < 0)
    return failf(CC3D_ERR_INVALID, "invalid arguments");
  if (has_background) *has_background = 0;
  if (sx * sy * sz == 0) return CC3D_OK;
  if (!labels || !out) return failf(CC3D_ERR_INVALID, "null buffer");
  if (!device_accessible(labels) || !device_accessible(out) || !device_accessible(work))
    return failf(CC3D_ERR_INVALID, "labels, output and the work area must be device memory");
  const StackWork w = carve(work, total_labels, nullptr);
  cudaStream_t s = (cudaStream_t)stream;
  CKS(cudaMemsetAsync(w.err + 1, 0, sizeof(unsigned), s));
  int rc;
  switch (label_bytes) {
    case 1: rc = relabel_out<uint8_t>(w, (const uint8_t*)labels, label_strides, offset, out, out_bytes, out_strides, sx, sy, sz, s); break;
    case 2: rc = relabel_out<uint16_t>(w, (const uint16_t*)labels, label_strides, offset, out, out_bytes, out_strides, sx, sy, sz, s); break;
    case 4: rc = relabel_out<uint32_t>(w, (const uint32_t*)labels, label_strides, offset, out, out_bytes, out_strides, sx, sy, sz, s); break;
    default: rc = relabel_out<uint64_t>(w, (const uint64_t*)labels, label_strides, offset, out, out_bytes, out_strides, sx, sy, sz, s); break;
  }
  if (rc) return rc;
  return read_err(w, s, has_background);
}
