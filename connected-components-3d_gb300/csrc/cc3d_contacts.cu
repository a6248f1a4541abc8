// cc3d_contacts.cu -- region adjacency of a labelled volume: cc3d.contacts
// and cc3d.region_graph (cc3d/fastcc3d.pyx:1180-1256,
// cc3d/cc3d_graphs.hpp:238-466).
//
// Every nonzero voxel looks at its backward neighbours (connectivity / 2 of
// them) exactly as the reference's neighbourhood table places them, including
// its treatment of the volume's faces: an offset component that would leave
// the volume is dropped from the sum, so at x = 0 the -x-y-z corner reads the
// -y-z voxel again, and in 2D the -x-y corner at y = 0 reads the -x voxel.
// A neighbour with another nonzero label adds one contact to the pair (lower
// label, higher label) in the offset's class: x face, y face, z face, or
// edge/corner.  Pairs are counted in an open-addressing hash table in device
// memory (64-bit keys low << 32 | high, integer counters per class), with the
// contacts of a warp that share a pair summed before they are inserted.  The
// caller turns the four counts into the reference's areas.
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

#define CKG(call)                                                                                \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return failf(CC3D_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

constexpr unsigned long long kEmpty = ~0ull;
constexpr unsigned ERR_TABLE_FULL = 1u;
constexpr unsigned ERR_WIDE_LABEL = 2u;

__device__ __forceinline__ unsigned long long mix(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  return x ^ (x >> 33);
}

struct Table {
  unsigned long long* keys;  // [cap]
  unsigned* counts;          // [cap][4]
  unsigned long long cap;    // power of two
  unsigned* flags;           // error bits
  unsigned long long* attempts;  // insert attempts (sizing pass)
};

__device__ void table_add(const Table& t, unsigned long long key, unsigned cls, unsigned n) {
  unsigned long long h = mix(key) & (t.cap - 1);
  for (unsigned long long probe = 0; probe < t.cap; ++probe) {
    const unsigned long long k = t.keys[h];
    if (k == key) {
      atomicAdd(&t.counts[h * 4 + cls], n);
      return;
    }
    if (k == kEmpty) {
      const unsigned long long seen = atomicCAS(&t.keys[h], kEmpty, key);
      if (seen == kEmpty || seen == key) {
        atomicAdd(&t.counts[h * 4 + cls], n);
        return;
      }
    }
    h = (h + 1) & (t.cap - 1);
  }
  atomicOr(t.flags, ERR_TABLE_FULL);
}

// Backward neighbour k (0 .. conn/2 - 1) of voxel (x, y, z) as the reference
// places it (cc3d/cc3d_graphs.hpp:238-298); returns the offset (0 = the voxel
// itself, which is skipped) and the contact class.
__device__ __forceinline__ int64_t neighbour3d(int k, int64_t x, int64_t y, int64_t z, int64_t sx, int64_t sy,
                                               int64_t sz, int conn, int& cls) {
  const int64_t sxy = sx * sy;
  const int64_t px = x < sx - 1, mx = -(int64_t)(x > 0);
  const int64_t py = sx * (y < sy - 1), my = -sx * (y > 0);
  const int64_t mz = -sxy * (z > 0);
  const int64_t c18 = conn > 6, c26 = conn > 18;
  cls = 3;
  switch (k) {
    case 0: cls = 0; return mx;
    case 1: cls = 1; return my;
    case 2: cls = 2; return mz;
    case 3: return c18 * (mx + my) * (mx && my);
    case 4: return c18 * (px + my) * (px && my);
    case 5: return c18 * (mx + mz) * (mx && mz);
    case 6: return c18 * (px + mz) * (px && mz);
    case 7: return c18 * (my + mz) * (my && mz);
    case 8: return c18 * (py + mz) * (py && mz);
    case 9: return c26 * (mx + my + mz) * (my && mz);
    case 10: return c26 * (px + my + mz) * (my && mz);
    case 11: return c26 * (mx + py + mz) * (py && mz);
    default: return c26 * (px + py + mz) * (py && mz);
  }
}

__device__ __forceinline__ int64_t neighbour2d(int k, int64_t x, int64_t y, int64_t sx, int conn, int& cls) {
  const int64_t px = x < sx - 1, mx = -(int64_t)(x > 0), my = -sx * (y > 0);
  const int64_t c8 = conn > 4;
  cls = 3;
  switch (k) {
    case 0: cls = 0; return mx;
    case 1: cls = 1; return my;
    case 2: return c8 * (mx + my);
    default: return c8 * (px + my);
  }
}

template <typename L>
__global__ void __launch_bounds__(256) k_contacts(const L* __restrict__ labels, int64_t sx, int64_t sy, int64_t sz,
                                                  int conn, int d2, Table t, int count_only) {
  const int64_t voxels = sx * sy * sz;
  const int lane = threadIdx.x & 31;
  const int nk = conn / 2;
  // grid-stride over voxels with whole warps in the loop (for the warp merge)
  for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < voxels; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = base + threadIdx.x;
    const bool in = i < voxels;
    const uint64_t cur = in ? (uint64_t)labels[i] : 0;
    int64_t x = 0, y = 0, z = 0;
    if (in) {
      x = i % sx;
      y = (i / sx) % sy;
      z = i / (sx * sy);
    }
    for (int k = 0; k < nk; ++k) {
      int cls = 3;
      unsigned long long key = kEmpty;
      if (in && cur != 0) {
        const int64_t off = d2 ? neighbour2d(k, x, y, sx, conn, cls) : neighbour3d(k, x, y, z, sx, sy, sz, conn, cls);
        const uint64_t lab = (uint64_t)labels[i + off];
        if (lab != 0 && lab != cur) {
          const uint64_t lo = cur < lab ? cur : lab, hi = cur < lab ? lab : cur;
          if (hi >> 32) atomicOr(t.flags, ERR_WIDE_LABEL);
          else key = (lo << 32) | hi;
        }
      }
      // contacts of the warp with the same pair and class are summed first
      const unsigned grp = __match_any_sync(FULL, key) & __match_any_sync(FULL, (unsigned)cls);
      const bool leader = key != kEmpty && lane == __ffs(grp) - 1;
      if (count_only) {
        const unsigned n = __popc(__ballot_sync(FULL, leader));
        if (lane == 0 && n) atomicAdd(t.attempts, (unsigned long long)n);
      } else if (leader) {
        table_add(t, key, (unsigned)cls, (unsigned)__popc(grp));
      }
    }
  }
}

// compact the occupied slots: out_keys[j], out_counts[j][4]
__global__ void k_compact(Table t, unsigned long long* out_keys, unsigned* out_counts, unsigned long long* n) {
  for (unsigned long long h = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x; h < t.cap;
       h += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long k = t.keys[h];
    if (k == kEmpty) continue;
    const unsigned long long j = atomicAdd(n, 1ull);
    out_keys[j] = k;
    for (int c = 0; c < 4; ++c) out_counts[j * 4 + c] = t.counts[h * 4 + c];
  }
}

unsigned grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  return (unsigned)(b < 1 ? 1 : b);
}

template <typename L>
void launch_contacts(const void* labels, int64_t sx, int64_t sy, int64_t sz, int conn, const Table& t,
                     int count_only, cudaStream_t s) {
  k_contacts<L><<<grid_for(sx * sy * sz), 256, 0, s>>>((const L*)labels, sx, sy, sz, conn, conn == 4 || conn == 8,
                                                         t, count_only);
}

// the table and its results live between the counting call and the copy-out
struct ContactState {
  void* dev = nullptr;
  size_t size = 0;
  unsigned long long n = 0;
  unsigned long long* keys = nullptr;
  unsigned* counts = nullptr;
};
thread_local ContactState g_contacts;

}  // namespace

extern "C" int cc3d_gpu_contacts(const void* labels, int label_bytes, int64_t sx, int64_t sy, int64_t sz,
                                 int64_t connectivity, uint64_t* npairs, void* stream) {
  if (!npairs || sx < 0 || sy < 0 || sz < 0 ||
      (label_bytes != 1 && label_bytes != 2 && label_bytes != 4 && label_bytes != 8))
    return failf(CC3D_ERR_INVALID, "invalid arguments");
  const int conn = (int)connectivity;
  if (conn != 4 && conn != 8 && conn != 6 && conn != 18 && conn != 26)
    return failf(CC3D_ERR_INVALID,
                 "Only (2d) 4, 8, (3d) 6, 18, and 26 connectivities are supported. Got: %d", conn);
  if ((conn == 4 || conn == 8) && sz != 1)
    return failf(CC3D_ERR_RUNTIME, "z thickness must be 1 for 2d region graph extraction.");
  *npairs = 0;
  g_contacts.n = 0;
  const int64_t voxels = sx * sy * sz;
  if (voxels == 0) return CC3D_OK;
  if (!device_accessible(labels)) return failf(CC3D_ERR_INVALID, "labels must be device memory");
  cudaStream_t s = (cudaStream_t)stream;
  ContactState& st = g_contacts;
  // pass 1: an upper bound on the pairs (warp-merged insert attempts)
  auto reserve = [&](size_t bytes) -> int {
    if (bytes <= st.size) return CC3D_OK;
    if (st.dev) cudaFree(st.dev);
    st.dev = nullptr;
    st.size = 0;
    if (cudaMalloc(&st.dev, bytes) != cudaSuccess) {
      cudaGetLastError();
      return failf(CC3D_ERR_NOMEM, "cannot allocate %zu bytes for the contact table", bytes);
    }
    st.size = bytes;
    return CC3D_OK;
  };
  if (int rc = reserve(256)) return rc;
  Table t;
  memset(&t, 0, sizeof(t));
  t.flags = (unsigned*)st.dev;
  t.attempts = (unsigned long long*)((char*)st.dev + 64);
  CKG(cudaMemsetAsync(st.dev, 0, 128, s));
  switch (label_bytes) {
    case 1: launch_contacts<uint8_t>(labels, sx, sy, sz, conn, t, 1, s); break;
    case 2: launch_contacts<uint16_t>(labels, sx, sy, sz, conn, t, 1, s); break;
    case 4: launch_contacts<uint32_t>(labels, sx, sy, sz, conn, t, 1, s); break;
    default: launch_contacts<uint64_t>(labels, sx, sy, sz, conn, t, 1, s); break;
  }
  unsigned long long attempts = 0;
  unsigned flags = 0;
  CKG(cudaMemcpyAsync(&attempts, t.attempts, sizeof(attempts), cudaMemcpyDeviceToHost, s));
  CKG(cudaMemcpyAsync(&flags, t.flags, sizeof(flags), cudaMemcpyDeviceToHost, s));
  CKG(cudaStreamSynchronize(s));
  if (flags & ERR_WIDE_LABEL)
    return failf(CC3D_ERR_UNSUPPORTED, "contacts on the GPU take labels below 2^32");
  if (attempts == 0) return CC3D_OK;
  unsigned long long cap = 1024;
  while (cap < attempts + attempts / 2) cap <<= 1;
  // table, then the compacted copy of at most cap entries
  const size_t o_keys = 256, o_counts = o_keys + cap * 8, o_okeys = o_counts + cap * 16,
               o_ocounts = o_okeys + cap * 8, total = o_ocounts + cap * 16;
  if (int rc = reserve(total)) return rc;
  t.flags = (unsigned*)st.dev;
  t.attempts = (unsigned long long*)((char*)st.dev + 64);
  unsigned long long* n_dev = (unsigned long long*)((char*)st.dev + 128);
  t.keys = (unsigned long long*)((char*)st.dev + o_keys);
  t.counts = (unsigned*)((char*)st.dev + o_counts);
  t.cap = cap;
  CKG(cudaMemsetAsync(st.dev, 0, 256, s));
  CKG(cudaMemsetAsync(t.keys, 0xFF, cap * 8, s));
  CKG(cudaMemsetAsync(t.counts, 0, cap * 16, s));
  switch (label_bytes) {
    case 1: launch_contacts<uint8_t>(labels, sx, sy, sz, conn, t, 0, s); break;
    case 2: launch_contacts<uint16_t>(labels, sx, sy, sz, conn, t, 0, s); break;
    case 4: launch_contacts<uint32_t>(labels, sx, sy, sz, conn, t, 0, s); break;
    default: launch_contacts<uint64_t>(labels, sx, sy, sz, conn, t, 0, s); break;
  }
  st.keys = (unsigned long long*)((char*)st.dev + o_okeys);
  st.counts = (unsigned*)((char*)st.dev + o_ocounts);
  k_compact<<<grid_for((int64_t)cap), 256, 0, s>>>(t, st.keys, st.counts, n_dev);
  CKG(cudaGetLastError());
  CKG(cudaMemcpyAsync(&flags, t.flags, sizeof(flags), cudaMemcpyDeviceToHost, s));
  CKG(cudaMemcpyAsync(&st.n, n_dev, sizeof(st.n), cudaMemcpyDeviceToHost, s));
  CKG(cudaStreamSynchronize(s));
  if (flags & ERR_TABLE_FULL) return failf(CC3D_ERR_DEVICE, "contact table overflow");
  *npairs = st.n;
  return CC3D_OK;
}

extern "C" int cc3d_gpu_contacts_copy(uint64_t* pairs, uint32_t* counts, uint64_t npairs) {
  if (npairs != g_contacts.n) return failf(CC3D_ERR_INVALID, "pair count does not match the last contacts call");
  if (npairs == 0) return CC3D_OK;
  if (!pairs || !counts) return failf(CC3D_ERR_INVALID, "invalid arguments");
  CKG(cudaMemcpy(pairs, g_contacts.keys, npairs * 8, cudaMemcpyDeviceToHost));
  CKG(cudaMemcpy(counts, g_contacts.counts, npairs * 16, cudaMemcpyDeviceToHost));
  return CC3D_OK;
}
