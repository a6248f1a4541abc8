// cc3d_runs.cu -- the run-length view of a labelled volume: the device half
// of cc3d.runs (cc3d/fastcc3d.pyx:1258-1277, extract_runs in
// cc3d/cc3d_graphs.hpp:470-502), on which cc3d.each and draw/erase build.
//
// A run starts wherever the label differs from the previous element in
// memory order.  The start positions (and the label there) are written in
// order with a two-pass compaction: per-block counts of starts, one scan of
// the block counts, then every block writes its starts at its offset.  The
// caller pairs consecutive starts into runs and drops the runs of label 0.
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

#define CKR(call)                                                                                \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return failf(CC3D_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

constexpr int kRunThreads = 256;
constexpr int kRunPer = 16;
constexpr int64_t kRunBlock = (int64_t)kRunThreads * kRunPer;

template <typename L>
__device__ __forceinline__ bool starts_run(const L* labels, int64_t i) {
  return i == 0 || labels[i] != labels[i - 1];
}

template <typename L>
__global__ void __launch_bounds__(kRunThreads) k_runs_count(const L* __restrict__ labels, int64_t n,
                                                             uint32_t* __restrict__ block_counts) {
  const int64_t base = blockIdx.x * kRunBlock + (int64_t)threadIdx.x * kRunPer;
  uint32_t c = 0;
#pragma unroll
  for (int k = 0; k < kRunPer; ++k) {
    const int64_t i = base + k;
    if (i < n && starts_run(labels, i)) ++c;
  }
  __shared__ uint32_t ws[kRunThreads / 32];
  uint32_t total;
  block_exclusive_scan<kRunThreads>(c, ws, total);
  if (threadIdx.x == 0) block_counts[blockIdx.x] = total;
}

// exclusive scan of the block counts in place (one block); *total = the sum
__global__ void __launch_bounds__(1024) k_runs_scan(uint32_t* counts, int64_t nblocks, unsigned long long* total) {
  __shared__ uint32_t ws[32];
  unsigned long long carry = 0;
  for (int64_t b0 = 0; b0 < nblocks; b0 += 1024) {
    const int64_t i = b0 + threadIdx.x;
    const uint32_t v = i < nblocks ? counts[i] : 0;
    uint32_t t;
    const uint32_t ex = block_exclusive_scan<1024>(v, ws, t);
    if (i < nblocks) counts[i] = (uint32_t)(carry + ex);
    carry += t;
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

template <typename L>
__global__ void __launch_bounds__(kRunThreads) k_runs_write(const L* __restrict__ labels, int64_t n,
                                                             const uint32_t* __restrict__ offsets,
                                                             uint64_t* __restrict__ pos, uint64_t* __restrict__ lab) {
  const int64_t base = blockIdx.x * kRunBlock + (int64_t)threadIdx.x * kRunPer;
  uint32_t c = 0;
#pragma unroll
  for (int k = 0; k < kRunPer; ++k) {
    const int64_t i = base + k;
    if (i < n && starts_run(labels, i)) ++c;
  }
  __shared__ uint32_t ws[kRunThreads / 32];
  uint32_t total;
  uint64_t o = (uint64_t)offsets[blockIdx.x] + block_exclusive_scan<kRunThreads>(c, ws, total);
#pragma unroll
  for (int k = 0; k < kRunPer; ++k) {
    const int64_t i = base + k;
    if (i < n && starts_run(labels, i)) {
      pos[o] = (uint64_t)i;
      lab[o] = (uint64_t)labels[i];
      ++o;
    }
  }
}

struct RunState {
  void* dev = nullptr;
  size_t size = 0;
  uint64_t n = 0;
  uint64_t* pos = nullptr;
  uint64_t* lab = nullptr;
};
thread_local RunState g_runs;

template <typename L>
int runs_t(const void* labels, int64_t n, cudaStream_t s) {
  RunState& st = g_runs;
  const int64_t nblocks = (n + kRunBlock - 1) / kRunBlock;
  auto reserve = [&](size_t bytes) -> int {
    if (bytes <= st.size) return CC3D_OK;
    if (st.dev) cudaFree(st.dev);
    st.dev = nullptr;
    st.size = 0;
    if (cudaMalloc(&st.dev, bytes) != cudaSuccess) {
      cudaGetLastError();
      return failf(CC3D_ERR_NOMEM, "cannot allocate %zu bytes for the runs", bytes);
    }
    st.size = bytes;
    return CC3D_OK;
  };
  const size_t o_tot = 0, o_cnt = 256, head = o_cnt + (((size_t)nblocks * 4 + 255) & ~size_t(255));
  if (int rc = reserve(head)) return rc;
  unsigned long long* tot = (unsigned long long*)((char*)st.dev + o_tot);
  uint32_t* counts = (uint32_t*)((char*)st.dev + o_cnt);
  const L* in = static_cast<const L*>(labels);
  k_runs_count<L><<<(unsigned)nblocks, kRunThreads, 0, s>>>(in, n, counts);
  k_runs_scan<<<1, 1024, 0, s>>>(counts, nblocks, tot);
  unsigned long long total = 0;
  CKR(cudaGetLastError());
  CKR(cudaMemcpyAsync(&total, tot, sizeof(total), cudaMemcpyDeviceToHost, s));
  CKR(cudaStreamSynchronize(s));
  // the output arrays follow the block counts (which they must not move)
  const size_t need = head + (size_t)total * 16;
  if (need > st.size) {
    void* grown = nullptr;
    if (cudaMalloc(&grown, need) != cudaSuccess) {
      cudaGetLastError();
      return failf(CC3D_ERR_NOMEM, "cannot allocate %zu bytes for the runs", need);
    }
    CKR(cudaMemcpyAsync(grown, st.dev, head, cudaMemcpyDeviceToDevice, s));
    CKR(cudaStreamSynchronize(s));
    cudaFree(st.dev);
    st.dev = grown;
    st.size = need;
    counts = (uint32_t*)((char*)st.dev + o_cnt);
  }
  st.pos = (uint64_t*)((char*)st.dev + head);
  st.lab = st.pos + total;
  k_runs_write<L><<<(unsigned)nblocks, kRunThreads, 0, s>>>(in, n, counts, st.pos, st.lab);
  CKR(cudaGetLastError());
  CKR(cudaStreamSynchronize(s));
  st.n = total;
  return CC3D_OK;
}

}  // namespace

extern "C" int cc3d_gpu_run_starts(const void* labels, int label_bytes, int64_t voxels, uint64_t* nstarts,
                                   void* stream) {
  if (!nstarts || voxels < 0 || (voxels && !labels) ||
      (label_bytes != 1 && label_bytes != 2 && label_bytes != 4 && label_bytes != 8))
    return failf(CC3D_ERR_INVALID, "invalid arguments");
  *nstarts = 0;
  g_runs.n = 0;
  if (voxels == 0) return CC3D_OK;
  if (!device_accessible(labels)) return failf(CC3D_ERR_INVALID, "labels must be device memory");
  cudaStream_t s = (cudaStream_t)stream;
  int rc;
  switch (label_bytes) {
    case 1: rc = runs_t<uint8_t>(labels, voxels, s); break;
    case 2: rc = runs_t<uint16_t>(labels, voxels, s); break;
    case 4: rc = runs_t<uint32_t>(labels, voxels, s); break;
    default: rc = runs_t<uint64_t>(labels, voxels, s); break;
  }
  if (rc) return rc;
  *nstarts = g_runs.n;
  return CC3D_OK;
}

extern "C" int cc3d_gpu_run_starts_copy(uint64_t* positions, uint64_t* labels, uint64_t nstarts) {
  if (nstarts != g_runs.n) return failf(CC3D_ERR_INVALID, "count does not match the last run_starts call");
  if (nstarts == 0) return CC3D_OK;
  if (!positions || !labels) return failf(CC3D_ERR_INVALID, "invalid arguments");
  CKR(cudaMemcpy(positions, g_runs.pos, nstarts * 8, cudaMemcpyDeviceToHost));
  CKR(cudaMemcpy(labels, g_runs.lab, nstarts * 8, cudaMemcpyDeviceToHost));
  return CC3D_OK;
}
