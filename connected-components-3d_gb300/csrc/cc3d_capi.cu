// cc3d_capi.cu -- host runtime behind include/cc3d_gpu.h.
//
// Owns the per-thread, per-device workspace (one grow-only device arena, a
// pinned counter block and a private stream for host-buffer calls), validates
// arguments like the reference's C++ entry points, stages host buffers, runs
// the kernel pipeline on the caller's stream and maps device error words to
// return codes.  No C++ exception crosses the ABI.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "cc3d_gpu.h"
#include "cc3d_internal.h"

using namespace cc3dgpu;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                       \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) return fail(CC3D_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

size_t dtype_size(int dt) {
  switch (dt) {
    case CC3D_U8: return 1;
    case CC3D_U16: return 2;
    case CC3D_U32: case CC3D_F32: return 4;
    case CC3D_U64: case CC3D_F64: return 8;
  }
  return 0;
}

struct Profile {
  bool on = false;
  double ms[CC3D_PROFILE_STAGES] = {0};
  uint64_t launches[CC3D_PROFILE_STAGES] = {0};
};
thread_local Profile g_prof;

// the labelling prepared by cc3d_gpu_label_prepare, finished by
// cc3d_gpu_label_finish on the same thread
struct Job {
  uint64_t token = 0;
  bool empty = false;
  bool ready = false;
  bool binary = false;
  int conn = 0;
  int64_t voxels = 0;
  int64_t ntiles = 0;
  uint64_t N = 0;
  uint64_t prov = 0;
  size_t out_staging_offset = 0;
  LabelArgs args;
};

// host <-> device copies of large volumes are cut into this many chunks of
// whole tile layers (z), overlapped with the tile pass / the writer
constexpr int kCopyChunks = 8;

struct Workspace {
  cudaEvent_t ev[CC3D_PROFILE_STAGES + 1] = {};
  cudaStream_t copy = nullptr;                 // second stream for chunked copies
  cudaEvent_t chunk_ev[kCopyChunks + 1] = {};  // ordering between the two streams
  Job job;
  uint64_t next_token = 0;
  void* spill = nullptr;
  void* dev = nullptr;
  size_t size = 0;
  Counters* host_ctr = nullptr;
  unsigned long long* host_small = nullptr;
  cudaStream_t own = nullptr;
};

// one workspace per (thread, device); released explicitly or at process exit
thread_local std::map<int, Workspace> g_ws;

int get_ws(Workspace*& out);

// entry points other than label_finish reuse the arena: forget a prepared job
int get_ws_fresh(Workspace*& out) {
  int rc = get_ws(out);
  if (rc == CC3D_OK) {
    out->job.ready = false;
    out->job.token = 0;
  }
  return rc;
}

int get_ws(Workspace*& out) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  Workspace& w = g_ws[dev];
  if (!w.host_ctr) {
    CK(cudaMallocHost((void**)&w.host_ctr, sizeof(Counters)));
    CK(cudaMallocHost((void**)&w.host_small, 64));
    CK(cudaStreamCreateWithFlags(&w.own, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&w.copy, cudaStreamNonBlocking));
    for (auto& e : w.ev) CK(cudaEventCreate(&e));
    for (auto& e : w.chunk_ev) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  out = &w;
  return CC3D_OK;
}

int reserve(Workspace& w, size_t bytes) {
  if (bytes <= w.size) return CC3D_OK;
  w.job.ready = false;  // a prepared labelling lived in the old arena
  if (w.dev) {
    cudaFree(w.dev);
    w.dev = nullptr;
    w.size = 0;
  }
  size_t want = bytes + bytes / 8 + (64u << 20);
  cudaError_t e = cudaMalloc(&w.dev, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    e = cudaMalloc(&w.dev, bytes);
    want = bytes;
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    w.dev = nullptr;
    return fail(CC3D_ERR_NOMEM, "cannot allocate %zu bytes of device workspace", bytes);
  }
  w.size = want;
  return CC3D_OK;
}

// carves aligned sub-buffers out of the arena
struct Carver {
  size_t off = 0;
  size_t take(size_t bytes) {
    const size_t at = off;
    off += (bytes + 255) & ~size_t(255);
    return at;
  }
};

// Tile layers [l0, l1) of chunk k out of n (whole z layers of tiles), and the
// voxel range they cover; volumes with fewer than kCopyChunks tile layers, or
// under 64 MiB, are one chunk.
int copy_chunks(const LabelArgs& a, int64_t bytes) {
  return (a.ntz >= kCopyChunks && bytes >= (64ll << 20)) ? kCopyChunks : 1;
}
void chunk_range(const LabelArgs& a, int k, int n, int64_t& t0, int64_t& t1, int64_t& v0, int64_t& v1) {
  const int64_t l0 = (int64_t)a.ntz * k / n, l1 = (int64_t)a.ntz * (k + 1) / n;
  const int64_t layer = (int64_t)a.ntx * a.nty;
  t0 = l0 * layer;
  t1 = l1 * layer;
  const int64_t plane = a.sx * a.sy;
  v0 = std::min<int64_t>(l0 * a.tz, a.sz) * plane;
  v1 = std::min<int64_t>(l1 * a.tz, a.sz) * plane;
}

cudaStream_t pick_stream(Workspace& w, void* stream, int mem_flags) {
  if (stream) return (cudaStream_t)stream;
  return mem_flags ? (cudaStream_t)0 : w.own;
}

int check_device_errors(unsigned err) {
  if (!err) return CC3D_OK;
  return fail(CC3D_ERR_DEVICE,
              "device kernel gave up (error bits 0x%x: %s%s%s%s%s%s)", err,
              (err & ERR_UNITE_BUDGET) ? "union budget " : "",
              (err & ERR_FIND_BUDGET) ? "find budget " : "",
              (err & ERR_EDGE_OVERFLOW) ? "edge buffer overflow " : "",
              (err & ERR_LOCAL_BUDGET) ? "tile union budget " : "",
              (err & ERR_WAIT) ? "a bounded wait ran out (input copy or grid barrier) " : "",
              (err & ERR_INDEX) ? "index range check" : "");
}

Counters fresh_counters() {
  Counters c;
  memset(&c, 0, sizeof(c));
  c.first_row = 0x7FFFFFFFFFFFFFFFLL;
  c.last_row = -1;
  return c;
}

#define DISPATCH_DTYPE(dt, FN, ...)                  \
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

// Stage timer: mark(k) records the end of stage k (the start is the previous
// mark); finish() adds the elapsed times of the marked stages after the
// stream has been synchronised.
struct StageTimer {
  Workspace& w;
  cudaStream_t s;
  int last = -1;
  int order[CC3D_PROFILE_STAGES + 1];
  int n = 0;
  StageTimer(Workspace& w_, cudaStream_t s_) : w(w_), s(s_) {
    if (g_prof.on) { cudaEventRecord(w.ev[0], s); order[n++] = -1; }
  }
  void mark(int stage) {
    if (!g_prof.on || n > CC3D_PROFILE_STAGES) return;
    cudaEventRecord(w.ev[n], s);
    order[n++] = stage;
  }
  void finish() {
    if (!g_prof.on) return;
    for (int i = 1; i < n; ++i) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, w.ev[i - 1], w.ev[i]) == cudaSuccess) {
        g_prof.ms[order[i]] += ms;
        g_prof.launches[order[i]] += 1;
      }
    }
  }
};

}  // namespace

// ------------------------------------------------------------ tile-pass choice
// The variant a thread asked for (CC3D_TILE_AUTO: the autotuner's choice for
// the volume's class, else the default), and the autotuner's choices, shared
// by all threads.  A class is (dtype, effective connectivity, relation mode,
// size bucket of the voxel count).
namespace {
thread_local int g_tile_pass = CC3D_TILE_AUTO;
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, int> g_tuned;

int size_bucket(int64_t voxels) {
  int b = 0;
  while (voxels > 1 && b < 62) { voxels >>= 1; ++b; }
  return b / 3;  // classes of 8x in voxel count
}

int resolve_tile_pass(int dtype, int eff, int mode, int64_t voxels) {
  if (g_tile_pass != CC3D_TILE_AUTO && g_tile_pass != CC3D_TILE_MODEL) return g_tile_pass;
  std::lock_guard<std::mutex> lock(g_tune_mu);
  auto it = g_tuned.find(std::make_tuple(dtype, eff, mode, size_bucket(voxels)));
  if (it != g_tuned.end()) return it->second;
  // without tuning data: the list pass on 32 x 8 x 8 tiles, box by TMA
  (void)eff;
  (void)mode;
  (void)voxels;
  return CC3D_TILE_LIST;
}
}  // namespace

int cc3dgpu::tile_pass_for(int dtype, int eff_connectivity, int mode, int64_t voxels) {
  return resolve_tile_pass(dtype, eff_connectivity, mode, voxels);
}

void cc3dgpu::record_tile_pass(int dtype, int eff_connectivity, int mode, int64_t voxels, int variant) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tuned[std::make_tuple(dtype, eff_connectivity, mode, size_bucket(voxels))] = variant;
}

// iteration budget of the union-find loops (0: the built-in limits)
namespace {
std::atomic<int> g_union_budget{0};
}
int cc3dgpu::union_budget() { return g_union_budget.load(std::memory_order_relaxed); }

// error reporting shared with the other host translation units
int cc3dgpu::api_fail(int code, const char* msg) { return fail(code, "%s", msg); }
int cc3dgpu::api_device_errors(unsigned err) { return check_device_errors(err); }

extern "C" {

void cc3d_gpu_profile_enable(int enable) { g_prof.on = enable != 0; }

int cc3d_gpu_profile_read(double* ms, uint64_t* launches, int n) {
  if (n > CC3D_PROFILE_STAGES) n = CC3D_PROFILE_STAGES;
  for (int i = 0; i < n; ++i) {
    if (ms) ms[i] = g_prof.ms[i];
    if (launches) launches[i] = g_prof.launches[i];
    g_prof.ms[i] = 0;
    g_prof.launches[i] = 0;
  }
  return n;
}

const char* cc3d_gpu_last_error(void) { return g_err.c_str(); }

int cc3d_gpu_set_union_budget(int budget) {
  if (budget < 0) return fail(CC3D_ERR_INVALID, "the union budget must be >= 0 (0: the built-in limits)");
  return g_union_budget.exchange(budget);
}

const char* cc3d_gpu_version(void) { return "cc3d-gb300 0.1 (sm_103a)"; }

void cc3d_gpu_release_workspace(void) {
  for (auto& kv : g_ws) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(kv.first);
    if (kv.second.dev) cudaFree(kv.second.dev);
    if (kv.second.host_ctr) cudaFreeHost(kv.second.host_ctr);
    if (kv.second.host_small) cudaFreeHost(kv.second.host_small);
    if (kv.second.own) cudaStreamDestroy(kv.second.own);
    if (kv.second.copy) cudaStreamDestroy(kv.second.copy);
    for (auto& e : kv.second.chunk_ev)
      if (e) cudaEventDestroy(e);
    for (auto& e : kv.second.ev)
      if (e) cudaEventDestroy(e);
    cudaSetDevice(prev);
  }
  g_ws.clear();
}

int cc3d_gpu_estimate_provisional_label_count(const void* in, int dtype, int64_t sx, int64_t voxels,
                                              uint64_t* epl, int64_t* first_row,
                                              int64_t* last_row, int mem_flags, void* stream) {
  const size_t isz = dtype_size(dtype);
  if (!isz) return fail(CC3D_ERR_INVALID, "unknown dtype code %d", dtype);
  if (sx < 0 || voxels < 0 || !epl || !first_row || !last_row)
    return fail(CC3D_ERR_INVALID, "invalid arguments");
  if (voxels == 0 || sx == 0) {
    *epl = 0;
    *first_row = -1;
    *last_row = -1;
    return CC3D_OK;
  }
  Workspace* w;
  if (int rc = get_ws_fresh(w)) return rc;
  cudaStream_t s = pick_stream(*w, stream, mem_flags);
  Carver cv;
  const size_t o_ctr = cv.take(sizeof(Counters));
  const bool stage_in = !(mem_flags & CC3D_IN_DEVICE);
  const size_t o_in = stage_in ? cv.take(voxels * isz) : 0;
  if (int rc = reserve(*w, cv.off)) return rc;
  char* base = (char*)w->dev;
  Counters* ctr = (Counters*)(base + o_ctr);
  *w->host_ctr = fresh_counters();
  CK(cudaMemcpyAsync(ctr, w->host_ctr, sizeof(Counters), cudaMemcpyHostToDevice, s));
  StageTimer tm(*w, s);
  const void* din = in;
  if (stage_in) {
    CK(cudaMemcpyAsync(base + o_in, in, voxels * isz, cudaMemcpyHostToDevice, s));
    din = base + o_in;
    tm.mark(0);
  }
  CK(DISPATCH_DTYPE(dtype, launch_epl, din, sx, voxels, ctr, s));
  tm.mark(1);
  CK(cudaMemcpyAsync(w->host_ctr, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  tm.finish();
  *epl = w->host_ctr->epl;
  *first_row = w->host_ctr->epl ? w->host_ctr->first_row : -1;
  *last_row = w->host_ctr->epl ? w->host_ctr->last_row : -1;
  return CC3D_OK;
}

static int label_prepare(const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
                         int64_t connectivity, int periodic_boundary, int binary_image,
                         int mem_flags, void* stream, cc3d_gpu_prepared* info, int variant,
                         bool continuous = false, uint64_t delta_bits = 0, bool graph = false);

int cc3d_gpu_label_prepare_graph(const void* vcg, int dtype, int64_t sx, int64_t sy, int64_t sz,
                                 int64_t connectivity, int mem_flags, void* stream, cc3d_gpu_prepared* info) {
  if (dtype != CC3D_U8 && dtype != CC3D_U32)
    return fail(CC3D_ERR_INVALID, "voxel connectivity graphs are uint8 or uint32 (dtype code %d)", dtype);
  const int c = (int)connectivity;
  if (c != 26 && c != 6 && c != 4 && c != 8)
    return fail(CC3D_ERR_RUNTIME, "Only 4, 8, 6 and 26 connectivities are supported.");
  if (sz > 1 && c != 6 && c != 26) return fail(CC3D_ERR_RUNTIME, "Only 6 and 26 connectivity is supported in 3D.");
  // one plane: the 2D labellers (4 for 4 and 6, 8 for 8 and 26)
  const int64_t conn = sz == 1 ? ((c == 4 || c == 6) ? 4 : 8) : c;
  return label_prepare(vcg, dtype, sx, sy, sz, conn, 0, 0, mem_flags, stream, info, CC3D_TILE_RUNS, false, 0,
                       true);
}

int cc3d_gpu_label_prepare_continuous(const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
                                      int64_t connectivity, const void* delta, int mem_flags, void* stream,
                                      cc3d_gpu_prepared* info) {
  const size_t isz = dtype_size(dtype);
  if (!isz || !delta) return fail(CC3D_ERR_INVALID, "invalid arguments");
  uint64_t bits = 0;
  memcpy(&bits, delta, isz);
  return label_prepare(in, dtype, sx, sy, sz, connectivity, 0, 0, mem_flags, stream, info, CC3D_TILE_RUNS,
                       true, bits);
}

int cc3d_gpu_label_prepare(const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
                           int64_t connectivity, int periodic_boundary, int binary_image,
                           int mem_flags, void* stream, cc3d_gpu_prepared* info) {
  int code = CC3D_TILE_AUTO;
  if (g_tile_pass == CC3D_TILE_MODEL && (mem_flags & CC3D_IN_DEVICE) && sx > 0 && sy > 0 && sz > 0 &&
      g_model_loaded()) {
    int choice = 0, confident = 0;
    if (cc3d_gpu_cost_model_choose(in, dtype, sx, sy, sz, connectivity, binary_image, mem_flags, stream, 0.05f,
                                   &choice, &confident) == CC3D_OK)
      code = choice;
  }
  return label_prepare(in, dtype, sx, sy, sz, connectivity, periodic_boundary, binary_image, mem_flags,
                       stream, info, code);
}

static int label_prepare(const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
                         int64_t connectivity, int periodic_boundary, int binary_image,
                         int mem_flags, void* stream, cc3d_gpu_prepared* info, int variant,
                         bool continuous, uint64_t delta_bits, bool graph) {
  const size_t isz = dtype_size(dtype);
  if (!isz) return fail(CC3D_ERR_INVALID, "unknown dtype code %d", dtype);
  if (sx < 0 || sy < 0 || sz < 0 || !info) return fail(CC3D_ERR_INVALID, "invalid arguments");
  const int conn = (int)connectivity;
  if (conn != 26 && conn != 18 && conn != 6 && conn != 8 && conn != 4)
    return fail(CC3D_ERR_RUNTIME, "Only 4 and 8 2D and 6, 18, and 26 3D connectivities are supported.");
  if ((conn == 8 || conn == 4) && sz != 1)
    return fail(CC3D_ERR_RUNTIME, "sz must be 1 for 2D connectivities.");
  if (periodic_boundary && conn != 4 && conn != 8 && conn != 6)
    return fail(CC3D_ERR_INVALID, "periodic_boundary is only implemented for 4, 8 and 6 connectivity");
  if (continuous && (periodic_boundary || binary_image))
    return fail(CC3D_ERR_RUNTIME, "periodic_boundary is not currently supported for continuous data.");
  if ((mem_flags & CC3D_IN_DEVICE) && sx * sy * sz > 0 && !device_accessible(in))
    return fail(CC3D_ERR_INVALID, "the input must be device memory with CC3D_IN_DEVICE");
  memset(info, 0, sizeof(*info));
  info->first_row = -1;
  info->last_row = -1;
  const int64_t voxels = sx * sy * sz;
  Workspace* w;
  if (int rc = get_ws(w)) return rc;
  Job& job = w->job;
  job = Job();
  job.token = ++w->next_token;
  info->token = job.token;
  job.voxels = voxels;
  job.conn = conn;
  job.binary = binary_image != 0;
  if (voxels == 0) {
    job.empty = true;
    return CC3D_OK;
  }
  cudaStream_t s = pick_stream(*w, stream, mem_flags);

  // effective neighbourhood: a single z plane makes 26/18 equal to 8 and 6 to 4
  int eff = conn;
  if (sz == 1 && (conn == 26 || conn == 18)) eff = 8;
  if (sz == 1 && conn == 6) eff = 4;
  // continuous values (cc3d/cc3d_continuous.hpp:394-455): the 3D labeller
  // (any plane count) joins on |a - b| <= delta; the 2D 8-connected one has
  // its own decision tree
  const int mode = graph ? MODE_GRAPH
                 : continuous ? (conn == 8 ? MODE_CONT8Q : MODE_CONT)
                              : (!binary_image ? MODE_MULTI : (conn == 4 ? MODE_BINARY4 : MODE_BINARY));
  const bool block8 = binary_image && conn == 8;
  const bool d3 = (eff == 26 || eff == 18 || eff == 6);
  // tile-pass configuration: the caller's, the autotuned one for this class, or the default
  if (continuous || graph) variant = CC3D_TILE_RUNS;
  if (variant == CC3D_TILE_AUTO) variant = resolve_tile_pass(dtype, eff, mode, voxels);
  const TileCfg cfg = decode_tile_cfg(variant, d3);
  const int TY = block8 ? 64 : cfg.ty, TZ = block8 ? 1 : cfg.tz, HZ = d3 ? 1 : 0;

  LabelArgs& a = job.args;
  memset(&a, 0, sizeof(a));
  a.budget = union_budget();
  a.no_tma = cfg.plain ? 1 : 0;
  a.sx = sx; a.sy = sy; a.sz = sz;
  a.ntx = (int)((sx + kTX - 1) / kTX);
  a.nty = (int)((sy + TY - 1) / TY);
  a.ntz = (int)((sz + TZ - 1) / TZ);
  a.ty = TY; a.tz = TZ;
  const int64_t ntiles = (int64_t)a.ntx * a.nty * a.ntz;
  if (ntiles * kTV >= 0xFFFFFFFFLL)
    return fail(CC3D_ERR_UNSUPPORTED, "volume too large: %lld tiles of 2048 voxels exceed 32-bit node ids",
                (long long)ntiles);
  int64_t nwords;
  if (block8) {
    const int64_t osx = (sx + 1) >> 1, osy = (sy + 1) >> 1;
    a.wpr = (osx + 31) / 32;
    a.key_row = a.wpr * 32;
    nwords = osy * a.wpr;
  } else {
    a.wpr = a.ntx;
    a.key_row = a.wpr * 32;
    nwords = sy * sz * a.wpr;
  }
  if (nwords * 32 >= 0xFFFFFFFFLL)
    return fail(CC3D_ERR_UNSUPPORTED, "volume too large for 32-bit component keys");
  a.nwords = nwords;
  // at most one edge per halo run head or halo column voxel
  a.edge_slots = (unsigned)((TY + 2) * (TZ + HZ) * 34 - kTV);
  a.ntiles = ntiles;
  a.tile_base = 0;
  a.tile_end = ntiles;
  a.want_epl = (binary_image || graph) ? 0 : 1;
  a.want_prov = binary_image ? 1 : 0;

  const bool stage_in = !(mem_flags & CC3D_IN_DEVICE);
  const int64_t nblocks = scan_blocks_needed(nwords);
  Carver cv;
  const size_t o_ctr = cv.take(sizeof(Counters));
  const size_t o_in = stage_in ? cv.take(voxels * isz) : 0;
  const size_t o_rm = cv.take(ntiles * kRowsPerTile * sizeof(uint2));
  const size_t o_rr = cv.take(ntiles * kRowsPerTile * sizeof(uint16_t));
  const size_t o_rc = cv.take(ntiles * kTV * sizeof(uint16_t));
  const size_t o_E = cv.take(ntiles * kTV * sizeof(unsigned long long));
  const size_t o_L = cv.take(ntiles * kTV * sizeof(uint32_t));
  const size_t o_cc = cv.take(ntiles * sizeof(TileInfo));
  const size_t o_bm = cv.take(nwords * sizeof(uint32_t));
  const size_t o_pf = cv.take(nwords * sizeof(uint32_t));
  const size_t o_bs = cv.take((nblocks + 1) * sizeof(uint32_t));
  const size_t o_ed = cv.take((size_t)ntiles * a.edge_slots * sizeof(uint2));
  const size_t o_sp = cv.take(4 * sizeof(unsigned long long));
  // host outputs are staged after the job's buffers (room for uint64 labels)
  job.out_staging_offset = cv.take((mem_flags & CC3D_OUT_DEVICE) ? 0 : voxels * 8);
  if (int rc = reserve(*w, cv.off)) return rc;
  char* base = (char*)w->dev;
  Counters* ctr = (Counters*)(base + o_ctr);
  a.ctr = ctr;
  a.rmask = (uint2*)(base + o_rm);
  a.rrow = (uint16_t*)(base + o_rr);
  a.rcomp = (uint16_t*)(base + o_rc);
  a.E = (unsigned long long*)(base + o_E);
  a.label = (uint32_t*)(base + o_L);
  a.tinfo = (TileInfo*)(base + o_cc);
  a.bitmap = (uint32_t*)(base + o_bm);
  a.prefix = (uint32_t*)(base + o_pf);
  a.edges = (uint2*)(base + o_ed);
  a.delta_bits = delta_bits;
  a.span = (unsigned long long*)(base + o_sp);
  uint32_t* bsum = (uint32_t*)(base + o_bs);

  *w->host_ctr = fresh_counters();
  CK(cudaMemcpyAsync(ctr, w->host_ctr, sizeof(Counters), cudaMemcpyHostToDevice, s));
  if (block8) CK(cudaMemsetAsync(a.bitmap, 0, nwords * sizeof(uint32_t), s));
  StageTimer tm(*w, s);
  a.in = in;
  // (the continuous 2D 8-connected pass needs the whole image's span first)
  const int nchunks = (stage_in && mode != MODE_CONT8Q) ? copy_chunks(a, voxels * (int64_t)isz) : 1;
  if (nchunks > 1) {
    // the input arrives chunk by chunk on the copy stream; the tile pass of a
    // chunk starts once it (and so every chunk before it, whose last plane is
    // its halo) has landed
    a.in = base + o_in;
    CK(cudaEventRecord(w->chunk_ev[kCopyChunks], s));  // earlier work on this arena
    CK(cudaStreamWaitEvent(w->copy, w->chunk_ev[kCopyChunks], 0));
    for (int k = 0; k < nchunks; ++k) {
      int64_t t0, t1, v0, v1;
      chunk_range(a, k, nchunks, t0, t1, v0, v1);
      CK(cudaMemcpyAsync(base + o_in + v0 * isz, (const char*)in + v0 * isz, (v1 - v0) * isz,
                         cudaMemcpyHostToDevice, w->copy));
      CK(cudaEventRecord(w->chunk_ev[k], w->copy));
    }
    for (int k = 0; k < nchunks; ++k) {
      int64_t t0, t1, v0, v1;
      chunk_range(a, k, nchunks, t0, t1, v0, v1);
      CK(cudaStreamWaitEvent(s, w->chunk_ev[k], 0));
      if (t1 == t0) continue;
      LabelArgs ak = a;
      ak.tile_base = t0;
      ak.tile_end = t1;
      CK(DISPATCH_DTYPE(dtype, launch_tile_local, ak, eff, mode, block8, cfg.variant, t1 - t0, s));
    }
    tm.mark(2);
  } else {
    if (stage_in) {
      CK(cudaMemcpyAsync(base + o_in, in, voxels * isz, cudaMemcpyHostToDevice, s));
      a.in = base + o_in;
      tm.mark(0);
    }
    if (mode == MODE_CONT8Q)
      CK(DISPATCH_DTYPE(dtype, launch_span, a.in, voxels, (unsigned long long*)a.span, s));
    CK(DISPATCH_DTYPE(dtype, launch_tile_local, a, eff, mode, block8, cfg.variant, ntiles, s));
    tm.mark(2);
  }
  CK(launch_merge_edges(a, s));
  tm.mark(3);
  if (periodic_boundary) {
    CK(DISPATCH_DTYPE(dtype, launch_wrap, a, eff, mode, s));
    tm.mark(4);
  }
  CK(launch_scan(a, nwords, bsum, nblocks, s));
  tm.mark(5);
  CK(cudaMemcpyAsync(w->host_ctr, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  tm.finish();
  const Counters& h = *w->host_ctr;
  if (int rc = check_device_errors(h.err)) return rc;
  job.ntiles = ntiles;
  job.ready = true;
  job.N = h.N;
  job.prov = h.prov;
  info->N = h.N;
  info->provisional = h.prov;
  info->edges = h.edges;
  if (binary_image) {
    info->epl = (uint64_t)voxels;
    info->first_row = 0;
    info->last_row = sy;
  } else {
    info->epl = h.epl;
    info->first_row = h.epl ? h.first_row : -1;
    info->last_row = h.epl ? h.last_row : -1;
  }
  return CC3D_OK;
}

int cc3d_gpu_label_finish(uint64_t token, int64_t max_labels, void* out, int out_dtype, uint64_t* N,
                          int mem_flags, void* stream) {
  if (out_dtype != CC3D_U16 && out_dtype != CC3D_U32 && out_dtype != CC3D_U64)
    return fail(CC3D_ERR_INVALID, "out_dtype must be uint16, uint32 or uint64 (code %d)", out_dtype);
  if (!N) return fail(CC3D_ERR_INVALID, "invalid arguments");
  Workspace* w;
  if (int rc = get_ws(w)) return rc;
  Job& job = w->job;
  if (job.token != token || token == 0)
    return fail(CC3D_ERR_INVALID, "no prepared labelling with this token on this thread");
  *N = 0;
  if (job.empty) return CC3D_OK;
  if (!job.ready) return fail(CC3D_ERR_INVALID, "the prepared labelling did not complete");
  if ((mem_flags & CC3D_OUT_DEVICE) && !device_accessible(out))
    return fail(CC3D_ERR_INVALID, "the output must be device memory with CC3D_OUT_DEVICE");
  const size_t osz = dtype_size(out_dtype);
  const int64_t voxels = job.voxels;
  cudaStream_t s = pick_stream(*w, stream, mem_flags);
  if (max_labels == 0) {  // the reference returns before labelling
    if (mem_flags & CC3D_OUT_DEVICE) {
      CK(cudaMemsetAsync(out, 0, voxels * osz, s));
      CK(cudaStreamSynchronize(s));
    } else {
      memset(out, 0, voxels * osz);
    }
    return CC3D_OK;
  }
  if (job.binary) {
    // the reference's binary labellers size their union-find from max_labels
    // with per-labeller caps and throw when a provisional label reaches it
    const uint64_t V = (uint64_t)voxels;
    uint64_t L = (uint64_t)max_labels + 1;
    switch (job.conn) {
      case 26: L = (L < (V >> 2) + 1 ? L : (V >> 2) + 1) + 1; break;
      case 18: L = (L < V + 1 ? L : V + 1); break;
      case 8: L = (L < (V >> 1) + 1 ? L : (V >> 1) + 1); if (L < 1) L = 1; L += 1; break;
      default: L = (L < (V >> 1) + 1 ? L : (V >> 1) + 1) + 1; break;
    }
    const uint64_t outmax = out_dtype == CC3D_U16 ? 0xFFFFull : out_dtype == CC3D_U32 ? 0xFFFFFFFFull : ~0ull;
    if (L > outmax) L = outmax;
    if (job.prov >= L) return fail(CC3D_ERR_RUNTIME, "maximum length exception");
  }
  const bool stage_out = !(mem_flags & CC3D_OUT_DEVICE);
  void* dout = out;
  if (stage_out) {
    // grow the arena past the job's buffers without moving them
    const size_t need = job.out_staging_offset + voxels * osz;
    if (need > w->size) {
      void* extra = nullptr;
      CK(cudaMalloc(&extra, voxels * osz));
      w->spill = extra;
      dout = extra;
    } else {
      dout = (char*)w->dev + job.out_staging_offset;
    }
  }
  StageTimer tm(*w, s);
  const int nchunks = stage_out ? copy_chunks(job.args, voxels * (int64_t)osz) : 1;
  if (nchunks > 1) {
    // labels leave chunk by chunk on the copy stream while the writer
    // produces the next chunk
    for (int k = 0; k < nchunks; ++k) {
      int64_t t0, t1, v0, v1;
      chunk_range(job.args, k, nchunks, t0, t1, v0, v1);
      if (t1 > t0) {
        LabelArgs ak = job.args;
        ak.tile_base = t0;
        ak.tile_end = t1;
        CK(launch_write_tiles(ak, dout, out_dtype, t1 - t0, s));
      }
      CK(cudaEventRecord(w->chunk_ev[k], s));
      CK(cudaStreamWaitEvent(w->copy, w->chunk_ev[k], 0));
      CK(cudaMemcpyAsync((char*)out + v0 * osz, (const char*)dout + v0 * osz, (v1 - v0) * osz,
                         cudaMemcpyDeviceToHost, w->copy));
    }
    CK(cudaEventRecord(w->chunk_ev[kCopyChunks], w->copy));
    CK(cudaStreamWaitEvent(s, w->chunk_ev[kCopyChunks], 0));
    tm.mark(6);
  } else {
    CK(launch_write(job.args, dout, out_dtype, job.ntiles, s));
    tm.mark(6);
    if (stage_out) {
      CK(cudaMemcpyAsync(out, dout, voxels * osz, cudaMemcpyDeviceToHost, s));
      tm.mark(7);
    }
  }
  CK(cudaMemcpyAsync(w->host_ctr, job.args.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  tm.finish();
  if (w->spill) {
    cudaFree(w->spill);
    w->spill = nullptr;
  }
  if (int rc = check_device_errors(w->host_ctr->err)) return rc;
  *N = job.N;
  return CC3D_OK;
}

int cc3d_gpu_connected_components3d(const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
                                    int64_t max_labels, int64_t connectivity, double delta,
                                    void* out, int out_dtype, uint64_t* N, int periodic_boundary,
                                    int binary_image, int mem_flags, void* stream) {
  if (!N) return fail(CC3D_ERR_INVALID, "invalid arguments");
  if (out_dtype != CC3D_U16 && out_dtype != CC3D_U32 && out_dtype != CC3D_U64)
    return fail(CC3D_ERR_INVALID, "out_dtype must be uint16, uint32 or uint64 (code %d)", out_dtype);
  cc3d_gpu_prepared info;
  if (delta != 0.0 && !binary_image) {
    if (periodic_boundary)
      return fail(CC3D_ERR_RUNTIME, "periodic_boundary is not currently supported for continuous data.");
    // delta in the element type, as the template argument T delta
    unsigned char d[8] = {0};
    switch (dtype) {
      case CC3D_U8: { const uint8_t v = (uint8_t)delta; memcpy(d, &v, 1); break; }
      case CC3D_U16: { const uint16_t v = (uint16_t)delta; memcpy(d, &v, 2); break; }
      case CC3D_U32: { const uint32_t v = (uint32_t)delta; memcpy(d, &v, 4); break; }
      case CC3D_U64: { const uint64_t v = (uint64_t)delta; memcpy(d, &v, 8); break; }
      case CC3D_F32: { const float v = (float)delta; memcpy(d, &v, 4); break; }
      case CC3D_F64: { memcpy(d, &delta, 8); break; }
      default: return fail(CC3D_ERR_INVALID, "unknown dtype code %d", dtype);
    }
    if (delta < 0.0) return fail(CC3D_ERR_INVALID, "delta must be >= 0");
    if (int rc = cc3d_gpu_label_prepare_continuous(in, dtype, sx, sy, sz, connectivity, d, mem_flags, stream,
                                                   &info))
      return rc;
  } else if (int rc = cc3d_gpu_label_prepare(in, dtype, sx, sy, sz, connectivity, periodic_boundary,
                                             binary_image, mem_flags, stream, &info)) {
    return rc;
  }
  return cc3d_gpu_label_finish(info.token, max_labels, out, out_dtype, N, mem_flags & CC3D_OUT_DEVICE,
                               stream);
}

int cc3d_gpu_special_row(const void* in, int dtype, int is_uint64, int64_t sx, int64_t sy, int64_t sz,
                         int64_t row, void* out, int out_dtype, uint64_t* N, int mem_flags,
                         void* stream) {
  const size_t isz = dtype_size(dtype), osz = dtype_size(out_dtype);
  if (!isz || (out_dtype != CC3D_U16 && out_dtype != CC3D_U32 && out_dtype != CC3D_U64) || !N)
    return fail(CC3D_ERR_INVALID, "invalid arguments");
  if (row < 0 || row >= sy * sz) return fail(CC3D_ERR_INVALID, "row %lld out of range", (long long)row);
  Workspace* w;
  if (int rc = get_ws_fresh(w)) return rc;
  cudaStream_t s = pick_stream(*w, stream, mem_flags);
  const bool stage_in = !(mem_flags & CC3D_IN_DEVICE), stage_out = !(mem_flags & CC3D_OUT_DEVICE);
  Carver cv;
  const size_t o_ctr = cv.take(sizeof(Counters));
  const size_t o_in = stage_in ? cv.take(sx * isz) : 0;
  const size_t o_out = stage_out ? cv.take(sx * osz) : 0;
  if (int rc = reserve(*w, cv.off)) return rc;
  char* base = (char*)w->dev;
  Counters* ctr = (Counters*)(base + o_ctr);
  *w->host_ctr = fresh_counters();
  CK(cudaMemcpyAsync(ctr, w->host_ctr, sizeof(Counters), cudaMemcpyHostToDevice, s));
  const char* rin = (const char*)in + row * sx * isz;
  char* rout = (char*)out + row * sx * osz;
  const void* din = rin;
  void* dout = rout;
  if (stage_in) {
    CK(cudaMemcpyAsync(base + o_in, rin, sx * isz, cudaMemcpyHostToDevice, s));
    din = base + o_in;
  }
  if (stage_out) {
    CK(cudaMemcpyAsync(base + o_out, rout, sx * osz, cudaMemcpyHostToDevice, s));
    dout = base + o_out;
  }
  CK(DISPATCH_DTYPE(dtype, launch_special_row, din, sx, 0, is_uint64, dout, out_dtype, ctr, s));
  if (stage_out) CK(cudaMemcpyAsync(rout, dout, sx * osz, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(w->host_ctr, ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  const unsigned err = w->host_ctr->err;
  if (err & 16u) return fail(CC3D_ERR_NAN, "cannot convert float NaN to integer");
  if (err & 32u) return fail(CC3D_ERR_OVERFLOW, "Python int too large to convert to C long");
  *N = w->host_ctr->N;
  return CC3D_OK;
}

int cc3d_gpu_label_minmax(const void* labels, int dtype, int is_signed, int64_t voxels, uint64_t* vmax,
                          int64_t* vmin, int mem_flags, void* stream) {
  const size_t isz = dtype_size(dtype);
  if (!isz || dtype == CC3D_F32 || dtype == CC3D_F64 || !vmax || !vmin || voxels <= 0)
    return fail(CC3D_ERR_INVALID, "invalid arguments");
  Workspace* w;
  if (int rc = get_ws_fresh(w)) return rc;
  cudaStream_t s = pick_stream(*w, stream, mem_flags);
  const bool stage_in = !(mem_flags & CC3D_IN_DEVICE);
  Carver cv;
  const size_t o_res = cv.take(16);
  const size_t o_in = stage_in ? cv.take(voxels * isz) : 0;
  if (int rc = reserve(*w, cv.off)) return rc;
  char* base = (char*)w->dev;
  unsigned long long* res = (unsigned long long*)(base + o_res);
  const void* din = labels;
  if (stage_in) {
    CK(cudaMemcpyAsync(base + o_in, labels, voxels * isz, cudaMemcpyHostToDevice, s));
    din = base + o_in;
  }
  CK(DISPATCH_DTYPE(dtype, launch_minmax, din, voxels, is_signed, res, s));
  CK(cudaMemcpyAsync(w->host_small, res, 16, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  *vmax = w->host_small[0];
  *vmin = (int64_t)w->host_small[1];
  return CC3D_OK;
}

int cc3d_gpu_statistics(const void* labels, int dtype, int64_t d0, int64_t d1, int64_t d2, int ndim,
                        int c_order, uint64_t N, uint32_t* counts, void* bboxes, int bbox_dtype,
                        double* centroids, int mem_flags, void* stream) {
  const size_t isz = dtype_size(dtype);
  if (!isz || dtype == CC3D_F32 || dtype == CC3D_F64)
    return fail(CC3D_ERR_INVALID, "statistics needs unsigned integer labels");
  if ((ndim != 2 && ndim != 3) || d0 <= 0 || d1 <= 0 || d2 <= 0 || (ndim == 2 && d2 != 1))
    return fail(CC3D_ERR_INVALID, "invalid shape");
  if (bbox_dtype != CC3D_U16 && bbox_dtype != CC3D_U32) return fail(CC3D_ERR_INVALID, "bbox dtype");
  const int64_t voxels = d0 * d1 * d2;
  if (N > (uint64_t)voxels) return fail(CC3D_ERR_INVALID, "N exceeds the voxel count");
  if ((mem_flags & CC3D_IN_DEVICE) && !device_accessible(labels))
    return fail(CC3D_ERR_INVALID, "labels must be device memory with CC3D_IN_DEVICE");
  if ((mem_flags & CC3D_OUT_DEVICE) &&
      !(device_accessible(counts) && device_accessible(bboxes) && device_accessible(centroids)))
    return fail(CC3D_ERR_INVALID, "outputs must be device memory with CC3D_OUT_DEVICE");
  Workspace* w;
  if (int rc = get_ws_fresh(w)) return rc;
  cudaStream_t s = pick_stream(*w, stream, mem_flags);
  const int64_t n1 = (int64_t)N + 1;
  const bool stage_in = !(mem_flags & CC3D_IN_DEVICE), stage_out = !(mem_flags & CC3D_OUT_DEVICE);
  const size_t bsz = dtype_size(bbox_dtype);
  Carver cv;
  const size_t o_in = stage_in ? cv.take(voxels * isz) : 0;
  const size_t o_cnt = cv.take(n1 * 4);
  const size_t o_min = cv.take(n1 * 3 * 4);
  const size_t o_max = cv.take(n1 * 3 * 4);
  const size_t o_sum = cv.take(n1 * 3 * 8);
  const size_t o_err = cv.take(sizeof(unsigned int));
  const size_t o_bb = stage_out ? cv.take(n1 * 2 * ndim * bsz) : 0;
  const size_t o_ce = stage_out ? cv.take(n1 * ndim * 8) : 0;
  if (int rc = reserve(*w, cv.off)) return rc;
  char* base = (char*)w->dev;
  StatsArgs a;
  a.labels = labels;
  if (stage_in) {
    CK(cudaMemcpyAsync(base + o_in, labels, voxels * isz, cudaMemcpyHostToDevice, s));
    a.labels = base + o_in;
  }
  a.dtype = dtype;
  a.d0 = d0; a.d1 = d1; a.d2 = d2;
  a.ndim = ndim;
  a.c_order = c_order;
  a.N = N;
  a.counts = (stage_out ? (uint32_t*)(base + o_cnt) : counts);
  a.bmin = (uint32_t*)(base + o_min);
  a.bmax = (uint32_t*)(base + o_max);
  a.sums = (unsigned long long*)(base + o_sum);
  a.err = (unsigned int*)(base + o_err);
  CK(cudaMemsetAsync(a.err, 0, sizeof(unsigned int), s));
  void* dbb = stage_out ? (void*)(base + o_bb) : bboxes;
  double* dce = stage_out ? (double*)(base + o_ce) : centroids;
  CK(launch_stats(a, s));
  CK(launch_stats_finalize(a, dbb, bbox_dtype, dce, s));
  if (stage_out) {
    CK(cudaMemcpyAsync(counts, a.counts, n1 * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(bboxes, dbb, n1 * 2 * ndim * bsz, cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(centroids, dce, n1 * ndim * 8, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaMemcpyAsync(w->host_small, a.err, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (*(const unsigned int*)w->host_small)
    return fail(CC3D_ERR_DEVICE, "a label exceeds N = %llu (its voxels were skipped)", (unsigned long long)N);
  return CC3D_OK;
}

int cc3d_gpu_set_tile_pass(int code) {
  if (!valid_tile_code(code) && code != CC3D_TILE_MODEL)
    return fail(CC3D_ERR_INVALID, "unknown tile pass configuration %d", code);
  const int prev = g_tile_pass;
  g_tile_pass = code;
  return prev;
}

int cc3d_gpu_tile_pass_choice(int dtype, int64_t sx, int64_t sy, int64_t sz, int64_t connectivity,
                              int binary_image) {
  const int conn = (int)connectivity;
  int eff = conn;
  if (sz == 1 && (conn == 26 || conn == 18)) eff = 8;
  if (sz == 1 && conn == 6) eff = 4;
  const int mode = !binary_image ? MODE_MULTI : (conn == 4 ? MODE_BINARY4 : MODE_BINARY);
  if (binary_image && conn == 8) return CC3D_TILE_RUNS;
  int code = resolve_tile_pass(dtype, eff, mode, sx * sy * sz);
  if (!(eff == 26 || eff == 18 || eff == 6)) code &= ~0xF0;  // 2D: one tile shape
  return code;
}

int cc3d_gpu_autotune(const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz, int64_t connectivity,
                      int binary_image, int mem_flags, void* stream, int repeats, int* best,
                      double* ms) {
  if (!best) return fail(CC3D_ERR_INVALID, "invalid arguments");
  if (repeats < 1) repeats = 1;
  const int conn = (int)connectivity;
  int eff = conn;
  if (sz == 1 && (conn == 26 || conn == 18)) eff = 8;
  if (sz == 1 && conn == 6) eff = 4;
  const bool d3 = eff == 26 || eff == 18 || eff == 6;
  const int mode = !binary_image ? MODE_MULTI : (conn == 4 ? MODE_BINARY4 : MODE_BINARY);
  const int ncfg = d3 ? CC3D_TILE_CONFIGS : 4;  // 2D: the 8x8 entries (one tile shape)
  double t[CC3D_TILE_CONFIGS];
  int bi = 0;
  for (int k = 0; k < CC3D_TILE_CONFIGS; ++k) t[k] = -1.0;
  for (int k = 0; k < ncfg; ++k) {
    const int code = cc3d_gpu_tile_config(k);
    double bestt = 1e300;
    for (int r = 0; r < repeats + 1; ++r) {  // the first run warms up
      cc3d_gpu_prepared info;
      const auto t0 = std::chrono::steady_clock::now();
      if (int rc = label_prepare(in, dtype, sx, sy, sz, connectivity, 0, binary_image, mem_flags, stream,
                                 &info, code))
        return rc;
      const double dt = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      if (r > 0 && dt < bestt) bestt = dt;
    }
    t[k] = bestt;
    if (bestt < t[bi]) bi = k;
  }
  const int choice = cc3d_gpu_tile_config(bi);
  {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tuned[std::make_tuple(dtype, eff, mode, size_bucket(sx * sy * sz))] = choice;
  }
  *best = choice;
  if (ms)
    for (int k = 0; k < CC3D_TILE_CONFIGS; ++k) ms[k] = t[k];
  return CC3D_OK;
}

int cc3d_gpu_tile_config(int index) {
  static const int codes[CC3D_TILE_CONFIGS] = {
      CC3D_TILE_LIST | CC3D_TILE_8x8,  CC3D_TILE_LIST | CC3D_TILE_8x8 | CC3D_TILE_PLAIN,
      CC3D_TILE_RUNS | CC3D_TILE_8x8,  CC3D_TILE_RUNS | CC3D_TILE_8x8 | CC3D_TILE_PLAIN,
      CC3D_TILE_LIST | CC3D_TILE_4x16, CC3D_TILE_LIST | CC3D_TILE_4x16 | CC3D_TILE_PLAIN,
      CC3D_TILE_RUNS | CC3D_TILE_4x16, CC3D_TILE_RUNS | CC3D_TILE_4x16 | CC3D_TILE_PLAIN,
      CC3D_TILE_LIST | CC3D_TILE_16x4, CC3D_TILE_LIST | CC3D_TILE_16x4 | CC3D_TILE_PLAIN,
      CC3D_TILE_RUNS | CC3D_TILE_16x4, CC3D_TILE_RUNS | CC3D_TILE_16x4 | CC3D_TILE_PLAIN};
  if (index < 0 || index >= CC3D_TILE_CONFIGS) return -1;
  return codes[index];
}

void cc3d_gpu_autotune_reset(void) {
  std::lock_guard<std::mutex> lock(g_tune_mu);
  g_tuned.clear();
}

}  // extern "C"
