// cc3d_batch.cu -- many volumes labelled by one launch of each stage.
//
// The volumes' tiles are numbered one after the other and their bitmap word
// ranges laid end to end (VolGeo, cc3d_label.cuh), so the tile pass, the edge
// merge, the numbering scan, the per-volume finalisation and the writer each
// run once for the whole batch.  The stage sequence -- descriptor upload,
// counter reset, the five stages, the copy of the per-volume results -- is
// captured once into a CUDA graph per batch layout (dtype, connectivity,
// variant and the list of shapes) and replayed while the layout repeats; the
// volumes' buffer addresses live in the uploaded descriptors, so new buffers
// need no new graph.
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "cc3d_gpu.h"
#include "cc3d_batch_persistent.cuh"
#include "cc3d_internal.h"

using namespace cc3dgpu;

static_assert(sizeof(BatchResult) == sizeof(cc3d_gpu_volume_result), "result layouts must match");

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

#define CKB(call)                                                                                \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess) return failf(CC3D_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

struct BatchState {
  // device arena and pinned host mirrors
  char* dev = nullptr;
  size_t dev_size = 0;
  char* host = nullptr;
  size_t host_size = 0;
  cudaStream_t own = nullptr;
  // the captured graph and the layout it was captured for
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<int64_t> layout;
  int nvol = 0;
  // offsets of the host mirrors
  size_t h_vols = 0, h_res = 0, h_ctr = 0, h_fresh = 0;
  Counters* d_ctr = nullptr;
};

thread_local std::map<int, BatchState> g_batch;

// the persistent path: one arena per device, and the graph holding the one
// cooperative launch, captured for a kernel, grid and header address
struct PersistState {
  char* dev = nullptr;
  size_t dev_size = 0;
  char* host = nullptr;
  size_t host_size = 0;
  cudaStream_t own = nullptr;
  cudaGraphExec_t exec = nullptr;
  const void* kernel = nullptr;
  void* hdr = nullptr;
  int grid = 0;
};
thread_local std::map<int, PersistState> g_persist;
std::mutex g_persist_args_mu;
thread_local int g_batch_mode = CC3D_BATCH_PERSISTENT;

void drop_graph(BatchState& b) {
  if (b.exec) cudaGraphExecDestroy(b.exec);
  if (b.graph) cudaGraphDestroy(b.graph);
  b.exec = nullptr;
  b.graph = nullptr;
  b.layout.clear();
}

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

static int label_batch(const cc3d_gpu_volume* vols, int n, int dtype, int64_t connectivity,
                       cc3d_gpu_volume_result* results, void* stream, int forced_variant);

static int label_batch_persistent(const cc3d_gpu_volume* vols, int n, int dtype, int64_t connectivity,
                                  cc3d_gpu_volume_result* results, void* stream);

extern "C" int cc3d_gpu_label_batch(const cc3d_gpu_volume* vols, int n, int dtype, int64_t connectivity,
                                    cc3d_gpu_volume_result* results, void* stream) {
  if (g_batch_mode == CC3D_BATCH_PERSISTENT)
    return label_batch_persistent(vols, n, dtype, connectivity, results, stream);
  return label_batch(vols, n, dtype, connectivity, results, stream, CC3D_TILE_AUTO);
}

extern "C" int cc3d_gpu_set_batch_mode(int mode) {
  if (mode != CC3D_BATCH_PERSISTENT && mode != CC3D_BATCH_STAGED)
    return failf(CC3D_ERR_INVALID, "unknown batch mode %d", mode);
  const int prev = g_batch_mode;
  g_batch_mode = mode;
  return prev;
}

// Times every tile-pass variant on this batch (the first run of each captures
// its graph) and records the faster one for the batch's class (dtype,
// connectivity, mean volume size).
extern "C" int cc3d_gpu_autotune_batch(const cc3d_gpu_volume* vols, int n, int dtype, int64_t connectivity,
                                       cc3d_gpu_volume_result* results, void* stream, int repeats, int* best,
                                       double* ms) {
  if (!best) return failf(CC3D_ERR_INVALID, "invalid arguments");
  if (repeats < 1) repeats = 1;
  const bool d3 = connectivity == 26 || connectivity == 18 || connectivity == 6;
  // (batches read their boxes with plain loads whatever the load-path bit
  // says, so only the configurations without it are timed)
  const int ncfg = d3 ? CC3D_TILE_CONFIGS : 4;
  double t[CC3D_TILE_CONFIGS];
  int bi = 0;
  for (int k = 0; k < CC3D_TILE_CONFIGS; ++k) t[k] = -1.0;
  for (int k = 0; k < ncfg; ++k) {
    if (cc3d_gpu_tile_config(k) & CC3D_TILE_PLAIN) continue;
    t[k] = 1e300;
    for (int r = 0; r < repeats + 1; ++r) {
      const auto t0 = std::chrono::steady_clock::now();
      if (int rc = label_batch(vols, n, dtype, connectivity, results, stream, cc3d_gpu_tile_config(k)))
        return rc;
      const double dt = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      if (r > 0 && dt < t[k]) t[k] = dt;
    }
    if (t[k] < t[bi]) bi = k;
  }
  int64_t voxels = 0, nonempty = 0;
  for (int i = 0; i < n; ++i) {
    const int64_t vx = vols[i].sx * vols[i].sy * vols[i].sz;
    voxels += vx;
    nonempty += vx > 0;
  }
  *best = cc3d_gpu_tile_config(bi);
  if (nonempty) record_tile_pass(dtype, (int)connectivity, MODE_MULTI, voxels / nonempty, *best);
  if (ms)
    for (int k = 0; k < CC3D_TILE_CONFIGS; ++k) ms[k] = t[k];
  return CC3D_OK;
}

static int label_batch(const cc3d_gpu_volume* vols, int n, int dtype, int64_t connectivity,
                       cc3d_gpu_volume_result* results, void* stream, int forced_variant) {
  if (n < 0 || (n > 0 && (!vols || !results))) return failf(CC3D_ERR_INVALID, "invalid arguments");
  if (dtype != CC3D_U8 && dtype != CC3D_U16 && dtype != CC3D_U32)
    return failf(CC3D_ERR_INVALID, "batches take uint8, uint16 or uint32 volumes (dtype code %d)", dtype);
  const int conn = (int)connectivity;
  if (conn != 26 && conn != 18 && conn != 6 && conn != 8 && conn != 4)
    return failf(CC3D_ERR_RUNTIME, "Only 4 and 8 2D and 6, 18, and 26 3D connectivities are supported.");
  const bool d3 = conn == 26 || conn == 18 || conn == 6;
  const int mode = MODE_MULTI;

  // tile-pass configuration: forced, or the autotuned one for the batch's
  // class (mean volume size), else the default
  int64_t vx_sum = 0, vx_n = 0;
  for (int i = 0; i < n; ++i) {
    const int64_t vx = vols[i].sx * vols[i].sy * vols[i].sz;
    if (vx > 0) {
      if (!device_accessible(vols[i].in) || !device_accessible(vols[i].out))
        return failf(CC3D_ERR_INVALID, "volume %d: input and output must be device memory", i);
      vx_sum += vx;
      ++vx_n;
    }
  }
  const int code = forced_variant != CC3D_TILE_AUTO ? forced_variant
                                                    : tile_pass_for(dtype, conn, mode, vx_n ? vx_sum / vx_n : 0);
  const TileCfg cfg = decode_tile_cfg(code, d3);
  const int variant = cfg.variant;
  const int TY = cfg.ty, TZ = cfg.tz, HZ = d3 ? 1 : 0;

  // geometry of every non-empty volume, in order
  std::vector<VolGeo> geo;
  std::vector<int> index;  // batch slot of each non-empty volume
  int64_t tiles = 0, words = 0, voxels_total = 0;
  for (int i = 0; i < n; ++i) {
    const cc3d_gpu_volume& v = vols[i];
    if (v.sx < 0 || v.sy < 0 || v.sz < 0) return failf(CC3D_ERR_INVALID, "volume %d: negative shape", i);
    if (!d3 && v.sz != 1) return failf(CC3D_ERR_RUNTIME, "sz must be 1 for 2D connectivities.");
    memset(&results[i], 0, sizeof(results[i]));
    results[i].first_row = -1;
    results[i].last_row = -1;
    results[i].out_dtype = CC3D_U16;
    const int64_t voxels = v.sx * v.sy * v.sz;
    if (voxels == 0) continue;
    if (!v.in || !v.out) return failf(CC3D_ERR_INVALID, "volume %d: null buffer", i);
    if (voxels >= 0xFFFFFFFFLL) return failf(CC3D_ERR_UNSUPPORTED, "volume %d is too large for a batch", i);
    VolGeo g;
    memset(&g, 0, sizeof(g));
    g.in = v.in;
    g.out = v.out;
    g.sx = v.sx; g.sy = v.sy; g.sz = v.sz;
    g.ntx = (int)((v.sx + kTX - 1) / kTX);
    g.nty = (int)((v.sy + TY - 1) / TY);
    g.ntz = (int)((v.sz + TZ - 1) / TZ);
    g.tile0 = tiles;
    g.word0 = words;
    tiles += (int64_t)g.ntx * g.nty * g.ntz;
    words += v.sy * v.sz * g.ntx;
    voxels_total += voxels;
    geo.push_back(g);
    index.push_back(i);
  }
  const int nv = (int)geo.size();
  if (nv == 0) return CC3D_OK;
  if (tiles * kTV >= 0xFFFFFFFFLL || words * 32 >= 0xFFFFFFFFLL)
    return failf(CC3D_ERR_UNSUPPORTED, "batch too large: %lld tiles, %lld bitmap words (32-bit ids and keys)",
                 (long long)tiles, (long long)words);

  int dev_id = 0;
  CKB(cudaGetDevice(&dev_id));
  BatchState& b = g_batch[dev_id];
  if (!b.own) CKB(cudaStreamCreateWithFlags(&b.own, cudaStreamNonBlocking));
  // graphs are captured on a stream of our own when the caller passes the
  // legacy default stream (it cannot be captured)
  cudaStream_t s = stream ? (cudaStream_t)stream : b.own;
  if (!stream) CKB(cudaStreamSynchronize(0));  // work the caller queued on the legacy stream

  std::vector<int64_t> layout;
  layout.reserve(4 + 3 * (size_t)nv);
  layout.push_back(dtype);
  layout.push_back(conn);
  layout.push_back(code);
  layout.push_back(nv);
  for (const VolGeo& g : geo) {
    layout.push_back(g.sx);
    layout.push_back(g.sy);
    layout.push_back(g.sz);
  }

  const unsigned edge_slots = (unsigned)((TY + 2) * (TZ + HZ) * 34 - kTV);
  const int64_t nblocks = scan_blocks_needed(words);
  // device layout
  size_t off = 0;
  auto take = [&](size_t bytes) { const size_t at = off; off += up256(bytes); return at; };
  const size_t o_ctr = take(sizeof(Counters));
  const size_t o_vols = take(nv * sizeof(VolGeo));
  const size_t o_tv = take(tiles * sizeof(uint32_t));
  const size_t o_res = take(nv * sizeof(BatchResult));
  const size_t o_rm = take(tiles * kRowsPerTile * sizeof(uint2));
  const size_t o_rr = take(tiles * kRowsPerTile * sizeof(uint16_t));
  const size_t o_rc = take(tiles * kTV * sizeof(uint16_t));
  const size_t o_E = take(tiles * kTV * sizeof(unsigned long long));
  const size_t o_L = take(tiles * kTV * sizeof(uint32_t));
  const size_t o_ti = take(tiles * sizeof(TileInfo));
  const size_t o_bm = take(words * sizeof(uint32_t));
  const size_t o_pf = take(words * sizeof(uint32_t));
  const size_t o_bs = take((nblocks + 1) * sizeof(uint32_t));
  const size_t o_ed = take((size_t)tiles * edge_slots * sizeof(uint2));
  // host mirror layout: descriptors, tile -> volume map, results, counters
  size_t hoff = 0;
  auto htake = [&](size_t bytes) { const size_t at = hoff; hoff += up256(bytes); return at; };
  const size_t h_vols = htake(nv * sizeof(VolGeo));
  const size_t h_tv = htake(tiles * sizeof(uint32_t));
  const size_t h_res = htake(nv * sizeof(BatchResult));
  const size_t h_ctr = htake(sizeof(Counters));
  const size_t h_fresh = htake(sizeof(Counters));

  const bool same_layout = b.exec && b.layout == layout;
  if (!same_layout) {
    drop_graph(b);
    if (off > b.dev_size) {
      if (b.dev) cudaFree(b.dev);
      b.dev = nullptr;
      b.dev_size = 0;
      if (cudaMalloc((void**)&b.dev, off) != cudaSuccess) {
        cudaGetLastError();
        return failf(CC3D_ERR_NOMEM, "cannot allocate %zu bytes of batch workspace", off);
      }
      b.dev_size = off;
    }
    if (hoff > b.host_size) {
      if (b.host) cudaFreeHost(b.host);
      b.host = nullptr;
      b.host_size = 0;
      CKB(cudaMallocHost((void**)&b.host, hoff));
      b.host_size = hoff;
    }
    b.h_vols = h_vols;
    b.h_res = h_res;
    b.h_ctr = h_ctr;
    b.h_fresh = h_fresh;
    // the tile -> volume map depends on the layout only
    uint32_t* tv = (uint32_t*)(b.host + h_tv);
    for (int v = 0; v < nv; ++v) {
      const int64_t t1 = v + 1 < nv ? geo[v + 1].tile0 : tiles;
      for (int64_t t = geo[v].tile0; t < t1; ++t) tv[t] = (uint32_t)v;
    }
    Counters* fresh = (Counters*)(b.host + h_fresh);
    memset(fresh, 0, sizeof(Counters));
    fresh->first_row = 0x7FFFFFFFFFFFFFFFLL;
    fresh->last_row = -1;
  }
  // descriptors carry this call's buffer addresses
  memcpy(b.host + b.h_vols, geo.data(), nv * sizeof(VolGeo));

  if (!same_layout) {
    LabelArgs a;
    memset(&a, 0, sizeof(a));
    a.budget = union_budget();
    a.ty = TY;
    a.tz = TZ;
    a.ntiles = tiles;
    a.tile_base = 0;
    a.tile_end = tiles;
    a.nwords = words;
    a.edge_slots = edge_slots;
    a.want_epl = 1;
    a.want_prov = 0;
    a.ctr = (Counters*)(b.dev + o_ctr);
    a.vols = (VolGeo*)(b.dev + o_vols);
    a.tile_vol = (const uint32_t*)(b.dev + o_tv);
    a.rmask = (uint2*)(b.dev + o_rm);
    a.rrow = (uint16_t*)(b.dev + o_rr);
    a.rcomp = (uint16_t*)(b.dev + o_rc);
    a.E = (unsigned long long*)(b.dev + o_E);
    a.label = (uint32_t*)(b.dev + o_L);
    a.tinfo = (TileInfo*)(b.dev + o_ti);
    a.bitmap = (uint32_t*)(b.dev + o_bm);
    a.prefix = (uint32_t*)(b.dev + o_pf);
    a.edges = (uint2*)(b.dev + o_ed);
    // ntx/nty of the single-volume fields are unused in a batch (tile_geo)
    a.ntx = 1;
    a.nty = 1;
    uint32_t* bsum = (uint32_t*)(b.dev + o_bs);
    BatchResult* d_res = (BatchResult*)(b.dev + o_res);
    b.d_ctr = a.ctr;

    CKB(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
    auto capture = [&]() -> cudaError_t {
      cudaError_t e;
      if ((e = cudaMemcpyAsync(a.vols, b.host + b.h_vols, nv * sizeof(VolGeo), cudaMemcpyHostToDevice, s))) return e;
      if ((e = cudaMemcpyAsync((void*)a.tile_vol, b.host + h_tv, tiles * sizeof(uint32_t), cudaMemcpyHostToDevice, s)))
        return e;
      if ((e = cudaMemcpyAsync(a.ctr, b.host + b.h_fresh, sizeof(Counters), cudaMemcpyHostToDevice, s))) return e;
      switch (dtype) {
        case CC3D_U8: e = launch_tile_local_u8(a, conn, mode, false, variant, tiles, s); break;
        case CC3D_U16: e = launch_tile_local_u16(a, conn, mode, false, variant, tiles, s); break;
        default: e = launch_tile_local_u32(a, conn, mode, false, variant, tiles, s); break;
      }
      if (e) return e;
      if ((e = launch_merge_edges(a, s))) return e;
      if ((e = launch_scan(a, words, bsum, nblocks, s))) return e;
      if ((e = launch_batch_finalize(a, nv, words, d_res, s))) return e;
      if ((e = launch_write_batch(a, tiles, s))) return e;
      if ((e = cudaMemcpyAsync(b.host + b.h_res, d_res, nv * sizeof(BatchResult), cudaMemcpyDeviceToHost, s))) return e;
      return cudaMemcpyAsync(b.host + b.h_ctr, a.ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s);
    };
    const cudaError_t ce = capture();
    cudaGraph_t graph = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(s, &graph);
    if (ce != cudaSuccess || ee != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      return failf(CC3D_ERR_CUDA, "capturing the batch graph: %s",
                   cudaGetErrorString(ce != cudaSuccess ? ce : ee));
    }
    b.graph = graph;
    CKB(cudaGraphInstantiate(&b.exec, b.graph, 0));
    b.layout = layout;
    b.nvol = nv;
  }

  CKB(cudaGraphLaunch(b.exec, s));
  CKB(cudaStreamSynchronize(s));
  const Counters* hc = (const Counters*)(b.host + b.h_ctr);
  if (int rc = api_device_errors(hc->err)) return rc;
  const BatchResult* hr = (const BatchResult*)(b.host + b.h_res);
  for (int v = 0; v < nv; ++v) memcpy(&results[index[v]], &hr[v], sizeof(BatchResult));
  return CC3D_OK;
}

extern "C" void cc3d_gpu_release_batch(void) {
  for (auto& kv : g_persist) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(kv.first);
    PersistState& b = kv.second;
    if (b.exec) cudaGraphExecDestroy(b.exec);
    if (b.dev) cudaFree(b.dev);
    if (b.host) cudaFreeHost(b.host);
    if (b.own) cudaStreamDestroy(b.own);
    cudaSetDevice(prev);
  }
  g_persist.clear();
  for (auto& kv : g_batch) {
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(kv.first);
    BatchState& b = kv.second;
    drop_graph(b);
    if (b.dev) cudaFree(b.dev);
    if (b.host) cudaFreeHost(b.host);
    if (b.own) cudaStreamDestroy(b.own);
    cudaSetDevice(prev);
  }
  g_batch.clear();
}

// ---------------------------------------------------------------- persistent
// One cooperative launch of k_batch_persistent labels the whole batch; its
// header (the buffers, counts and fresh counters) and the volume descriptors
// are uploaded by one copy, the per-volume results and counters come back by
// two.  The launch is captured into a CUDA graph once per kernel, grid and
// arena and replayed for every batch, whatever its layout.  3D volumes use
// the list pass with 32 x 8 x 8 tiles, 2D images 32 x 64.
static int label_batch_persistent(const cc3d_gpu_volume* vols, int n, int dtype, int64_t connectivity,
                                  cc3d_gpu_volume_result* results, void* stream) {
  if (n < 0 || (n > 0 && (!vols || !results))) return failf(CC3D_ERR_INVALID, "invalid arguments");
  if (dtype != CC3D_U8 && dtype != CC3D_U16 && dtype != CC3D_U32)
    return failf(CC3D_ERR_INVALID, "batches take uint8, uint16 or uint32 volumes (dtype code %d)", dtype);
  const int conn = (int)connectivity;
  if (conn != 26 && conn != 18 && conn != 6 && conn != 8 && conn != 4)
    return failf(CC3D_ERR_RUNTIME, "Only 4 and 8 2D and 6, 18, and 26 3D connectivities are supported.");
  const bool d3 = conn == 26 || conn == 18 || conn == 6;
  const int TY = d3 ? 8 : 64, TZ = d3 ? 8 : 1, HZ = d3 ? 1 : 0;

  std::vector<VolGeo> geo;
  std::vector<int> index;
  int64_t tiles = 0, words = 0;
  for (int i = 0; i < n; ++i) {
    const cc3d_gpu_volume& v = vols[i];
    if (v.sx < 0 || v.sy < 0 || v.sz < 0) return failf(CC3D_ERR_INVALID, "volume %d: negative shape", i);
    if (!d3 && v.sz != 1) return failf(CC3D_ERR_RUNTIME, "sz must be 1 for 2D connectivities.");
    memset(&results[i], 0, sizeof(results[i]));
    results[i].first_row = -1;
    results[i].last_row = -1;
    results[i].out_dtype = CC3D_U16;
    const int64_t voxels = v.sx * v.sy * v.sz;
    if (voxels == 0) continue;
    if (!v.in || !v.out) return failf(CC3D_ERR_INVALID, "volume %d: null buffer", i);
    if (!device_accessible(v.in) || !device_accessible(v.out))
      return failf(CC3D_ERR_INVALID, "volume %d: input and output must be device memory", i);
    if (voxels >= 0xFFFFFFFFLL) return failf(CC3D_ERR_UNSUPPORTED, "volume %d is too large for a batch", i);
    VolGeo g;
    memset(&g, 0, sizeof(g));
    g.in = v.in;
    g.out = v.out;
    g.sx = v.sx; g.sy = v.sy; g.sz = v.sz;
    g.ntx = (int)((v.sx + kTX - 1) / kTX);
    g.nty = (int)((v.sy + TY - 1) / TY);
    g.ntz = (int)((v.sz + TZ - 1) / TZ);
    g.tile0 = tiles;
    g.word0 = words;
    tiles += (int64_t)g.ntx * g.nty * g.ntz;
    words += v.sy * v.sz * g.ntx;
    geo.push_back(g);
    index.push_back(i);
  }
  const int nv = (int)geo.size();
  if (nv == 0) return CC3D_OK;
  if (tiles * kTV >= 0xFFFFFFFFLL || words * 32 >= 0xFFFFFFFFLL)
    return failf(CC3D_ERR_UNSUPPORTED, "batch too large: %lld tiles, %lld bitmap words (32-bit ids and keys)",
                 (long long)tiles, (long long)words);

  int dev_id = 0;
  CKB(cudaGetDevice(&dev_id));
  PersistState& b = g_persist[dev_id];
  if (!b.own) CKB(cudaStreamCreateWithFlags(&b.own, cudaStreamNonBlocking));
  cudaStream_t s = stream ? (cudaStream_t)stream : b.own;
  if (!stream) CKB(cudaStreamSynchronize(0));  // work the caller queued on the legacy stream

  const unsigned edge_slots = (unsigned)((TY + 2) * (TZ + HZ) * 34 - kTV);
  const int64_t nblocks = scan_blocks_needed(words);
  size_t off = 0;
  auto take = [&](size_t bytes) { const size_t at = off; off += up256(bytes); return at; };
  // header and descriptors first: they are uploaded by one copy
  const size_t o_hdr = take(sizeof(PersistentHeader));
  const size_t o_vols = take(nv * sizeof(VolGeo));
  const size_t up_bytes = off;
  const size_t o_res = take(nv * sizeof(BatchResult));
  const size_t o_tv = take(tiles * sizeof(uint32_t));
  const size_t o_rm = take(tiles * kRowsPerTile * sizeof(uint2));
  const size_t o_rr = take(tiles * kRowsPerTile * sizeof(uint16_t));
  const size_t o_rc = take(tiles * kTV * sizeof(uint16_t));
  const size_t o_E = take(tiles * kTV * sizeof(unsigned long long));
  const size_t o_L = take(tiles * kTV * sizeof(uint32_t));
  const size_t o_ti = take(tiles * sizeof(TileInfo));
  const size_t o_bm = take(words * sizeof(uint32_t));
  const size_t o_pf = take(words * sizeof(uint32_t));
  const size_t o_bs = take((nblocks + 1) * sizeof(uint32_t));
  const size_t o_ed = take((size_t)tiles * edge_slots * sizeof(uint2));
  const size_t host_bytes = up_bytes + up256(nv * sizeof(BatchResult));

  if (off > b.dev_size) {
    if (b.exec) cudaGraphExecDestroy(b.exec);
    b.exec = nullptr;
    if (b.dev) cudaFree(b.dev);
    b.dev = nullptr;
    b.dev_size = 0;
    if (cudaMalloc((void**)&b.dev, off) != cudaSuccess) {
      cudaGetLastError();
      return failf(CC3D_ERR_NOMEM, "cannot allocate %zu bytes of batch workspace", off);
    }
    b.dev_size = off;
  }
  if (host_bytes > b.host_size) {
    if (b.host) cudaFreeHost(b.host);
    b.host = nullptr;
    b.host_size = 0;
    CKB(cudaMallocHost((void**)&b.host, host_bytes));
    b.host_size = host_bytes;
  }

  PersistentHeader* h = (PersistentHeader*)(b.host + o_hdr);
  memset(h, 0, sizeof(*h));
  LabelArgs& a = h->a;
  a.budget = union_budget();
  a.ty = TY;
  a.tz = TZ;
  a.ntiles = tiles;
  a.tile_base = 0;
  a.tile_end = tiles;
  a.nwords = words;
  a.edge_slots = edge_slots;
  a.want_epl = 1;
  a.want_prov = 0;
  PersistentHeader* dh = (PersistentHeader*)(b.dev + o_hdr);
  a.ctr = &dh->ctr;
  a.vols = (VolGeo*)(b.dev + o_vols);
  a.tile_vol = (const uint32_t*)(b.dev + o_tv);
  a.rmask = (uint2*)(b.dev + o_rm);
  a.rrow = (uint16_t*)(b.dev + o_rr);
  a.rcomp = (uint16_t*)(b.dev + o_rc);
  a.E = (unsigned long long*)(b.dev + o_E);
  a.label = (uint32_t*)(b.dev + o_L);
  a.tinfo = (TileInfo*)(b.dev + o_ti);
  a.bitmap = (uint32_t*)(b.dev + o_bm);
  a.prefix = (uint32_t*)(b.dev + o_pf);
  a.edges = (uint2*)(b.dev + o_ed);
  a.ntx = 1;  // (the single-volume geometry fields are unused in a batch)
  a.nty = 1;
  h->nwords = words;
  h->nblocks = nblocks;
  h->bsum = (uint32_t*)(b.dev + o_bs);
  h->res = (BatchResult*)(b.dev + o_res);
  h->nvol = nv;
  h->ctr.first_row = 0x7FFFFFFFFFFFFFFFLL;
  h->ctr.last_row = -1;
  memcpy(b.host + o_vols, geo.data(), nv * sizeof(VolGeo));

  const void* kernel = dtype == CC3D_U8 ? persistent_kernel_u8(conn)
                       : dtype == CC3D_U16 ? persistent_kernel_u16(conn)
                                           : persistent_kernel_u32(conn);
  if (!kernel) return failf(CC3D_ERR_UNSUPPORTED, "no persistent batch kernel for connectivity %d", conn);
  int per_sm = 0, sms = 0;
  CKB(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0));
  CKB(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev_id));
  const int grid = per_sm * sms;
  if (grid < 1) return failf(CC3D_ERR_CUDA, "the persistent batch kernel does not fit on this device");

  if (!b.exec || b.kernel != kernel || b.hdr != (void*)dh || b.grid != grid) {
    if (b.exec) cudaGraphExecDestroy(b.exec);
    b.exec = nullptr;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void* args[] = {(void*)&dh};
    CKB(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const cudaError_t le = cudaLaunchKernelExC(&cfg, kernel, args);
    cudaGraph_t graph = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(s, &graph);
    if (le != cudaSuccess || ee != cudaSuccess) {
      if (graph) cudaGraphDestroy(graph);
      cudaGetLastError();
      return failf(CC3D_ERR_CUDA, "capturing the persistent batch launch: %s",
                   cudaGetErrorString(le != cudaSuccess ? le : ee));
    }
    const cudaError_t ie = cudaGraphInstantiate(&b.exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ie != cudaSuccess) {
      b.exec = nullptr;
      return failf(CC3D_ERR_CUDA, "instantiating the persistent batch graph: %s", cudaGetErrorString(ie));
    }
    b.kernel = kernel;
    b.hdr = (void*)dh;
    b.grid = grid;
  }
  // the kernels read their arguments from one constant-memory copy per
  // dtype: batches of several host threads take turns
  std::lock_guard<std::mutex> args_lock(g_persist_args_mu);
  CKB(cudaMemcpyAsync(b.dev, b.host, up_bytes, cudaMemcpyHostToDevice, s));
  CKB(dtype == CC3D_U8 ? persistent_args_u8(&h->a, s)
                       : dtype == CC3D_U16 ? persistent_args_u16(&h->a, s) : persistent_args_u32(&h->a, s));
  CKB(cudaGraphLaunch(b.exec, s));
  BatchResult* hres = (BatchResult*)(b.host + up_bytes);
  CKB(cudaMemcpyAsync(hres, b.dev + o_res, nv * sizeof(BatchResult), cudaMemcpyDeviceToHost, s));
  Counters* hc = &h->ctr;
  CKB(cudaMemcpyAsync(hc, &dh->ctr, sizeof(Counters), cudaMemcpyDeviceToHost, s));
  CKB(cudaStreamSynchronize(s));
  if (int rc = api_device_errors(hc->err)) return rc;
  for (int v = 0; v < nv; ++v) memcpy(&results[index[v]], &hres[v], sizeof(BatchResult));
  return CC3D_OK;
}
