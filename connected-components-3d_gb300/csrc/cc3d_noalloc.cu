// cc3d_noalloc.cu -- labelling that allocates no memory.
//
// Every other entry point keeps its scratch in a per-thread device workspace
// that grows with cudaMalloc.  Some callers cannot let a library do that:
// applications whose device memory is owned by another allocator (a caching
// pool that has reserved most of the GPU, where an outside cudaMalloc fails or
// fragments the pool), services that must run in a fixed, pre-planned memory
// budget, and latency-critical loops, where cudaMalloc and cudaFree take an
// unbounded time and cudaFree waits for the whole device.  For them,
// cc3d_gpu_connected_components3d_noalloc runs the same kernels with all of
// their scratch carved out of one fixed array, `scratch` below, that is part
// of this library's device image.
//
//   * The array holds CC3D_NOALLOC_SCRATCH_BYTES (40 MiB).  Every GPU that
//     loads the library holds it until the process exits.  A volume whose
//     scratch does not fit is rejected with CC3D_ERR_INVALID and a message
//     giving the bytes it needs.
//   * The caller passes device input and output buffers; nothing is staged.
//   * The first call on a device looks up the array's device address
//     (cudaGetSymbolAddress, with that device current) and caches it; make
//     that first call before any stream capture.
//   * All calls share the one array, and it keeps the last call's contents.
//     The counters are reset on every call; every other buffer is written
//     before it is read (the 2x2-block bitmap of binary 8-connected images is
//     cleared first).  Calls whose work overlaps on the GPU -- from several
//     host threads, or on several streams without ordering between them --
//     race on the array and corrupt each other's results: order them.
//   * It calls no cudaMalloc, cudaFree or other allocating routine; device
//     results (N, error words) come back by a copy into host stack memory.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "cc3d_gpu.h"
#include "cc3d_internal.h"

using namespace cc3dgpu;

namespace {

static __device__ __align__(256) unsigned char scratch[CC3D_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 256;
std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

int failf(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int failf(int code, const char* fmt, ...) {
  char buf[256];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return api_fail(code, buf);
}

#define CKN(call)                                                                                \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return failf(CC3D_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// device address of `scratch` on the current device (looked up once per device)
int scratch_address(char** out) {
  int dev = 0;
  CKN(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return failf(CC3D_ERR_UNSUPPORTED, "device ordinal %d", dev);
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, scratch);
    if (e != cudaSuccess || !ptr)
      return failf(CC3D_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
    g_scratch_ptr[dev] = ptr;
  }
  *out = static_cast<char*>(g_scratch_ptr[dev]);
  return CC3D_OK;
}

size_t elem_size(int dt) {
  switch (dt) {
    case CC3D_U8: return 1;
    case CC3D_U16: return 2;
    case CC3D_U32: case CC3D_F32: return 4;
    case CC3D_U64: case CC3D_F64: return 8;
  }
  return 0;
}

#define NOALLOC_DISPATCH(dt, FN, ...)                \
  ([&]() -> cudaError_t {                            \
    switch (dt) {                                    \
      case CC3D_U8: return FN##_u8(__VA_ARGS__);     \
      case CC3D_U16: return FN##_u16(__VA_ARGS__);   \
      case CC3D_U32: return FN##_u32(__VA_ARGS__);   \
      case CC3D_U64: return FN##_u64(__VA_ARGS__);   \
      case CC3D_F32: return FN##_f32(__VA_ARGS__);   \
      case CC3D_F64: return FN##_f64(__VA_ARGS__);   \
    }                                                \
    return cudaErrorInvalidValue;                    \
  }())

}  // namespace

extern "C" int cc3d_gpu_connected_components3d_noalloc(const void* in, int dtype, int64_t sx, int64_t sy,
                                                       int64_t sz, int64_t max_labels,
                                                       int64_t connectivity, void* out, int out_dtype,
                                                       uint64_t* N, int periodic_boundary,
                                                       int binary_image, void* stream) {
  const size_t isz = elem_size(dtype);
  if (!isz) return failf(CC3D_ERR_INVALID, "unknown dtype code %d", dtype);
  if (out_dtype != CC3D_U16 && out_dtype != CC3D_U32 && out_dtype != CC3D_U64)
    return failf(CC3D_ERR_INVALID, "out_dtype must be uint16, uint32 or uint64 (code %d)", out_dtype);
  if (sx < 0 || sy < 0 || sz < 0 || !N) return failf(CC3D_ERR_INVALID, "invalid arguments");
  const int conn = (int)connectivity;
  if (conn != 26 && conn != 18 && conn != 6 && conn != 8 && conn != 4)
    return failf(CC3D_ERR_RUNTIME, "Only 4 and 8 2D and 6, 18, and 26 3D connectivities are supported.");
  if ((conn == 8 || conn == 4) && sz != 1)
    return failf(CC3D_ERR_RUNTIME, "sz must be 1 for 2D connectivities.");
  if (periodic_boundary && conn != 4 && conn != 8 && conn != 6)
    return failf(CC3D_ERR_INVALID, "periodic_boundary is only implemented for 4, 8 and 6 connectivity");
  *N = 0;
  int64_t voxels = 0;
  if (__builtin_mul_overflow(sx, sy, &voxels) || __builtin_mul_overflow(voxels, sz, &voxels))
    return failf(CC3D_ERR_INVALID, "volume size overflows int64");
  if (voxels == 0) return CC3D_OK;
  if (!device_accessible(in) || !device_accessible(out))
    return failf(CC3D_ERR_INVALID, "input and output must be device memory");
  // every voxel takes more than one byte of scratch: larger volumes cannot fit
  if (voxels > (int64_t)CC3D_NOALLOC_SCRATCH_BYTES)
    return failf(CC3D_ERR_INVALID,
                 "volume %lld x %lld x %lld is too large for the no-allocation entry point "
                 "(%llu bytes of scratch; use cc3d_gpu_connected_components3d)",
                 (long long)sx, (long long)sy, (long long)sz, (unsigned long long)CC3D_NOALLOC_SCRATCH_BYTES);
  const size_t osz = elem_size(out_dtype);
  cudaStream_t s = (cudaStream_t)stream;

  // the same geometry as the workspace path
  int eff = conn;
  if (sz == 1 && (conn == 26 || conn == 18)) eff = 8;
  if (sz == 1 && conn == 6) eff = 4;
  const int mode = !binary_image ? MODE_MULTI : (conn == 4 ? MODE_BINARY4 : MODE_BINARY);
  const bool block8 = binary_image && conn == 8;
  const bool d3 = (eff == 26 || eff == 18 || eff == 6);
  // the variant follows the thread's choice; 3D tiles stay 32x8x8, the shape
  // the scratch limit is stated for
  const TileCfg cfg = decode_tile_cfg(cc3d_gpu_tile_pass_choice(dtype, sx, sy, sz, connectivity, binary_image) & 15, d3);
  const int TY = block8 ? 64 : cfg.ty, TZ = block8 ? 1 : cfg.tz, HZ = d3 ? 1 : 0;
  LabelArgs a;
  memset(&a, 0, sizeof(a));
  a.budget = union_budget();
  a.sx = sx; a.sy = sy; a.sz = sz;
  a.ntx = (int)((sx + kTX - 1) / kTX);
  a.nty = (int)((sy + TY - 1) / TY);
  a.ntz = (int)((sz + TZ - 1) / TZ);
  a.ty = TY; a.tz = TZ;
  const int64_t ntiles = (int64_t)a.ntx * a.nty * a.ntz;
  int64_t nwords;
  if (block8) {
    a.wpr = (((sx + 1) >> 1) + 31) / 32;
    nwords = ((sy + 1) >> 1) * a.wpr;
  } else {
    a.wpr = a.ntx;
    nwords = sy * sz * a.wpr;
  }
  a.key_row = a.wpr * 32;
  a.nwords = nwords;
  a.edge_slots = (unsigned)((TY + 2) * (TZ + HZ) * 34 - kTV);
  a.ntiles = ntiles;
  a.tile_base = 0;
  a.tile_end = ntiles;
  a.want_epl = 0;
  a.want_prov = binary_image ? 1 : 0;
  const int64_t nblocks = scan_blocks_needed(nwords);

  // scratch layout: 256-byte aligned pieces, checked against the array's size
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t at = off;
    off += (bytes + 255) & ~size_t(255);
    return at;
  };
  const size_t o_ctr = take(sizeof(Counters));
  const size_t o_rm = take(ntiles * kRowsPerTile * sizeof(uint2));
  const size_t o_rr = take(ntiles * kRowsPerTile * sizeof(uint16_t));
  const size_t o_rc = take(ntiles * kTV * sizeof(uint16_t));
  const size_t o_E = take(ntiles * kTV * sizeof(unsigned long long));
  const size_t o_L = take(ntiles * kTV * sizeof(uint32_t));
  const size_t o_ti = take(ntiles * sizeof(TileInfo));
  const size_t o_bm = take(nwords * sizeof(uint32_t));
  const size_t o_pf = take(nwords * sizeof(uint32_t));
  const size_t o_bs = take((nblocks + 1) * sizeof(uint32_t));
  const size_t o_ed = take((size_t)ntiles * a.edge_slots * sizeof(uint2));
  if (off > (size_t)CC3D_NOALLOC_SCRATCH_BYTES)
    return failf(CC3D_ERR_INVALID,
                 "volume %lld x %lld x %lld needs %zu bytes of scratch; the no-allocation entry point "
                 "holds %zu (use cc3d_gpu_connected_components3d)",
                 (long long)sx, (long long)sy, (long long)sz, off, (size_t)CC3D_NOALLOC_SCRATCH_BYTES);

  char* base = nullptr;
  if (int rc = scratch_address(&base)) return rc;
  a.ctr = (Counters*)(base + o_ctr);
  a.rmask = (uint2*)(base + o_rm);
  a.rrow = (uint16_t*)(base + o_rr);
  a.rcomp = (uint16_t*)(base + o_rc);
  a.E = (unsigned long long*)(base + o_E);
  a.label = (uint32_t*)(base + o_L);
  a.tinfo = (TileInfo*)(base + o_ti);
  a.bitmap = (uint32_t*)(base + o_bm);
  a.prefix = (uint32_t*)(base + o_pf);
  a.edges = (uint2*)(base + o_ed);
  a.in = in;
  uint32_t* bsum = (uint32_t*)(base + o_bs);

  if (max_labels == 0) {  // the reference returns zeros before labelling
    CKN(cudaMemsetAsync(out, 0, voxels * osz, s));
    CKN(cudaStreamSynchronize(s));
    return CC3D_OK;
  }

  // what must start at zero: the counters (and the block bitmap)
  Counters h;
  memset(&h, 0, sizeof(h));
  h.first_row = 0x7FFFFFFFFFFFFFFFLL;
  h.last_row = -1;
  CKN(cudaMemcpyAsync(a.ctr, &h, sizeof(h), cudaMemcpyHostToDevice, s));
  if (block8) CKN(cudaMemsetAsync(a.bitmap, 0, nwords * sizeof(uint32_t), s));
  CKN(NOALLOC_DISPATCH(dtype, launch_tile_local, a, eff, mode, block8, cfg.variant, ntiles, s));
  CKN(launch_merge_edges(a, s));
  if (periodic_boundary) CKN(NOALLOC_DISPATCH(dtype, launch_wrap, a, eff, mode, s));
  CKN(launch_scan(a, nwords, bsum, nblocks, s));
  CKN(cudaMemcpyAsync(&h, a.ctr, sizeof(h), cudaMemcpyDeviceToHost, s));
  CKN(cudaStreamSynchronize(s));
  if (int rc = api_device_errors(h.err)) return rc;

  if (binary_image) {
    // the reference's binary labellers size their union-find from max_labels
    // with per-labeller caps and throw once a provisional label reaches it
    // (cc3d/cc3d_binary.hpp, cc3d/fastcc3d.pyx:381-434)
    const uint64_t V = (uint64_t)voxels;
    uint64_t L = (uint64_t)max_labels + 1;
    switch (conn) {
      case 26: L = (L < (V >> 2) + 1 ? L : (V >> 2) + 1) + 1; break;
      case 18: L = (L < V + 1 ? L : V + 1); break;
      case 8: L = (L < (V >> 1) + 1 ? L : (V >> 1) + 1); if (L < 1) L = 1; L += 1; break;
      default: L = (L < (V >> 1) + 1 ? L : (V >> 1) + 1) + 1; break;
    }
    const uint64_t outmax = out_dtype == CC3D_U16 ? 0xFFFFull : out_dtype == CC3D_U32 ? 0xFFFFFFFFull : ~0ull;
    if (L > outmax) L = outmax;
    if (h.prov >= L) return failf(CC3D_ERR_RUNTIME, "maximum length exception");
  }

  CKN(launch_write(a, out, out_dtype, ntiles, s));
  unsigned err = 0;
  CKN(cudaMemcpyAsync(&err, &a.ctr->err, sizeof(err), cudaMemcpyDeviceToHost, s));
  CKN(cudaStreamSynchronize(s));
  if (int rc = api_device_errors(err)) return rc;
  *N = h.N;
  return CC3D_OK;
}
