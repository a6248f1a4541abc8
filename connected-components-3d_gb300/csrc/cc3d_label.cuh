// cc3d_label.cuh -- labelling kernels of the GB300 path (sm_103a).
//
// Pipeline for one volume (512^3 uint32 figures in brackets):
//
//   k_tile_runs   one CTA per 32 x TY x TZ tile of 2048 voxels [65536 CTAs].
//                 Stages the tile plus a one-voxel backward halo in shared
//                 memory by one TMA copy (rows of 32 values with the two halo
//                 columns).  Rows are cut into runs of related voxels with warp
//                 ballots; only run heads take part in the tile's union-find,
//                 so trees stay shallow.  Every row is matched with its
//                 backward rows (the connectivity's neighbour rows) by ballots
//                 (dx = 0, and dx = -1/+1 where the primary neighbour does not
//                 decide) and one union per pair of overlapping runs.  One edge
//                 per halo run joined to a tile component leaves the tile,
//                 except where the same-owner voxel just before it already
//                 carries the same join.  (k_tile_list, the list pass of
//                 cc3d_tile_list.cuh, produces the same records.)  Writes
//                   rmask[tile][row]   (foreground mask, run-start mask)
//                   rrow[tile][row]    first run of the row in rcomp
//                   rcomp[tile][run]   16-bit local component of every run:
//                                      the index of the component's root run
//                   E[tile*2048 + c]   (key << 32 | node) of component c,
//                                      key = row-padded raster index of the
//                                      component's first voxel (or first
//                                      2x2 block)
//                   bitmap             one bit per component key
//                   edges              (component node, halo voxel) pairs
//                 and, in the same read of the input, the provisional-label
//                 estimate and first/last foreground row (cc3d/cc3d.hpp:287-315)
//                 and the provisional-label count of the reference's binary
//                 labellers.
//   k_merge_edges global union-find over component nodes: a root is only ever
//                 linked under a root with a smaller key (64-bit atomicCAS on the
//                 packed (key, parent) word), so the root of every tree is the
//                 component's first voxel.  A root that gets linked clears its
//                 bit in the numbering bitmap.
//   k_wrap_pairs  periodic boundaries: unions across wrapped faces.
//   scan          exclusive popcount prefix of the bitmap: the rank of every
//                 surviving key = the component's number minus one.
//   k_label_write label of each run = 1 + rank(key of its component's root),
//                 then the run-length records expand to the output volume
//                 (batches: resolve_tile + write_tile_warp, cc3d_stages.cuh).
//
// Every loop that waits on other threads (the union-find retries) carries an
// iteration budget; when it runs out it sets a bit in the device error word
// and stops, and the host reports an error.
#pragma once

#include <cstdint>
#include <cstring>
#include <cuda_runtime.h>

namespace cc3dgpu {

constexpr int kTX = 32;          // tile width in x (one warp per row)
constexpr int kTV = 2048;        // voxels per tile (every tile shape)
constexpr int kThreads = 256;    // threads per CTA of the tile kernels
constexpr int kRowsPerTile = 64; // 2048 / 32
constexpr unsigned FULL = 0xFFFFFFFFu;

// relation modes
constexpr int MODE_MULTI = 0;    // neighbours join when equal and nonzero
constexpr int MODE_BINARY = 1;   // neighbours join when both nonzero
constexpr int MODE_BINARY4 = 2;  // the reference's binary 4-connected relation
constexpr int MODE_CONT = 3;     // continuous values: neighbours join when |a - b| <= delta
constexpr int MODE_CONT8Q = 4;   // the reference's continuous 2D 8-connected decision tree
constexpr int MODE_GRAPH = 5;    // a voxel connectivity graph: every voxel is a node, and it
                                 // joins a backward neighbour where its own bit says so

// device error bits
constexpr unsigned ERR_UNITE_BUDGET = 1u;
constexpr unsigned ERR_FIND_BUDGET = 2u;
constexpr unsigned ERR_EDGE_OVERFLOW = 4u;
constexpr unsigned ERR_LOCAL_BUDGET = 8u;
constexpr unsigned ERR_INDEX = 64u;  // an index failed its range check (access skipped)

constexpr int kFindLimit = 1 << 24;
constexpr int kUniteLimit = 1 << 20;
constexpr int kLocalLimit = 1 << 16;
// the iteration limit of a loop: the call's budget (LabelArgs::budget, set
// by cc3d_gpu_set_union_budget) where one is given, else the default
__host__ __device__ __forceinline__ int limit_of(int budget, int dflt) { return budget > 0 ? budget : dflt; }

struct Counters {
  unsigned int edges;        // total edges written by the tile pass
  unsigned int err;
  unsigned long long prov;   // provisional labels of the reference's binary labellers
  unsigned long long N;
  unsigned long long epl;
  long long first_row;
  long long last_row;
  unsigned long long pad[2];
};

// per-tile results of the tile pass (no same-address atomics in that pass:
// the scan kernel reduces these)
struct TileInfo {
  uint32_t C;          // runs; a component is named by its root run's index (< C)
  uint32_t nedges;     // edges in the tile's edge slots
  uint32_t epl;        // provisional-label estimate of the tile's row segments
  uint32_t prov;       // provisional labels of the reference's binary labellers
  long long first_row; // first/last row holding foreground (INT64_MAX / -1 if none)
  long long last_row;
};

// One volume of a batch.  A batch numbers the tiles of all its volumes one
// after the other and lays their bitmap word ranges end to end, so that one
// launch of each stage covers every volume: node ids and keys stay unique
// across volumes, and a volume's labels are ranks within its word range.
struct VolGeo {
  const void* in;
  void* out;
  int64_t sx, sy, sz;
  int ntx, nty, ntz;
  int out_code;      // output element type (2 = uint16, 3 = uint32), set by k_batch_finalize
  int64_t tile0;     // first tile of the volume in the batch
  int64_t word0;     // first bitmap word of the volume
  uint64_t rank0;    // number of keys before the volume's range (set by k_batch_finalize)
};

struct LabelArgs {
  const void* in;
  int64_t sx, sy, sz;
  int ntx, nty, ntz;
  int ty, tz;                  // tile shape (TY, TZ) at run time
  int64_t wpr;                 // bitmap words per padded row (block rows for 2x2 numbering)
  int64_t key_row;             // wpr * 32
  uint2* rmask;                // [tiles][64] (foreground, run starts)
  uint16_t* rrow;              // [tiles][64] first run of each row
  uint16_t* rcomp;             // [tiles][2048] component of each run
  unsigned long long* E;       // [tiles][2048]
  uint32_t* label;             // [tiles][2048] final label of each component
  TileInfo* tinfo;             // [tiles]
  int64_t ntiles;
  uint32_t* bitmap;
  uint32_t* prefix;
  int64_t nwords;              // words of bitmap and prefix
  uint2* edges;                // [tiles][edge_slots]
  unsigned int edge_slots;     // edge capacity of one tile (one per halo node)
  Counters* ctr;
  int want_epl;
  int want_prov;
  VolGeo* vols;                // batch descriptors (null for a single volume)
  const uint32_t* tile_vol;    // [tiles] volume of every tile of a batch
  int64_t tile_base;           // first tile of this launch of the tile pass or the writer
  int64_t tile_end;            // one past its last tile
  // continuous modes: delta as the bits of one input element, and (2D
  // 8-connected) the image's minimum and maximum as element bits on the device
  uint64_t delta_bits;
  const unsigned long long* span;
  int budget;                  // iteration limit of every union-find loop (0: the defaults)
  int no_tma;                  // read tile boxes with plain loads even where TMA could
};

// Geometry of the volume a tile belongs to, and the tile's place in it.
struct TileGeo {
  const void* in;
  int64_t sx, sy, sz;
  int ntx, nty;
  int64_t wpr, key_row;  // bitmap words per row, key stride of a row
  int64_t tile0;         // first tile of the volume (0 for a single volume)
  int64_t word0;         // first bitmap word of the volume
  int tx, ty, tz;        // tile coordinates inside the volume
};

__device__ __forceinline__ TileGeo tile_geo(const LabelArgs& p, int64_t tile) {
  TileGeo g;
  if (p.vols) {
    const VolGeo& v = p.vols[p.tile_vol[tile]];
    g.in = v.in; g.sx = v.sx; g.sy = v.sy; g.sz = v.sz; g.ntx = v.ntx; g.nty = v.nty;
    g.wpr = v.ntx; g.key_row = (int64_t)v.ntx * 32; g.tile0 = v.tile0; g.word0 = v.word0;
  } else {
    g.in = p.in; g.sx = p.sx; g.sy = p.sy; g.sz = p.sz; g.ntx = p.ntx; g.nty = p.nty;
    g.wpr = p.wpr; g.key_row = p.key_row; g.tile0 = 0; g.word0 = 0;
  }
  // tile indices of a volume fit 32 bits (node ids do), so 32-bit division
  const uint32_t local = (uint32_t)(tile - g.tile0);
  const uint32_t ntx = (uint32_t)g.ntx, nty = (uint32_t)g.nty;
  const uint32_t rest = local / ntx;
  g.tx = (int)(local - rest * ntx);
  const uint32_t tz = rest / nty;
  g.ty = (int)(rest - tz * nty);
  g.tz = (int)tz;
  return g;
}

// ---------------------------------------------------------------- neighbours
// Backward neighbour rows of a connectivity: (dy, dz) and which x offsets of
// that row are neighbours (bit 0: dx = -1, bit 1: dx = 0, bit 2: dx = +1).
// The left neighbour in the same row (dx = -1, dy = dz = 0) is carried by the
// runs themselves.
template <int CONN> struct RowNb;
template <> struct RowNb<26> { static constexpr int n = 4; };
template <> struct RowNb<18> { static constexpr int n = 4; };
template <> struct RowNb<6> { static constexpr int n = 2; };
template <> struct RowNb<8> { static constexpr int n = 1; };
template <> struct RowNb<4> { static constexpr int n = 1; };

template <int CONN>
__host__ __device__ __forceinline__ void row_nb(int k, int& dy, int& dz, int& dxs) {
  if (CONN == 26) {
    const int t[4][3] = {{-1, 0, 7}, {-1, -1, 7}, {0, -1, 7}, {1, -1, 7}};
    dy = t[k][0]; dz = t[k][1]; dxs = t[k][2];
  } else if (CONN == 18) {
    const int t[4][3] = {{-1, 0, 7}, {-1, -1, 2}, {0, -1, 7}, {1, -1, 2}};
    dy = t[k][0]; dz = t[k][1]; dxs = t[k][2];
  } else if (CONN == 6) {
    dy = (k == 0) ? -1 : 0; dz = (k == 0) ? 0 : -1; dxs = 2;
  } else if (CONN == 8) {
    dy = -1; dz = 0; dxs = 7;
  } else {
    dy = -1; dz = 0; dxs = 2;
  }
}

template <typename T, int MODE> struct Stored { using type = T; };
template <typename T> struct Stored<T, MODE_BINARY> { using type = uint8_t; };

template <typename S, typename T, int MODE>
__device__ __forceinline__ S to_stored(T v) {
  if (MODE == MODE_BINARY) return (S)(v != T(0) ? 1 : 0);
  return (S)v;
}

template <typename S>
__device__ __forceinline__ bool is_fg(S v) { return v != S(0); }

// relation between a foreground voxel `a` and a neighbour `b` off its row
template <int MODE, typename S>
__device__ __forceinline__ bool rel(S a, S b) {
  if (MODE == MODE_MULTI) return a == b;
  return is_fg(b);
}

// ------------------------------------------- voxel connectivity graphs
// Bit (0-based) of direction (dx, dy, dz) in a 3D voxel connectivity graph:
// faces +x -x +y -y +z -z, then edges and corners in the order of
// cc3d/cc3d_graphs.hpp:81-96; -1 for the centre.
__host__ __device__ __forceinline__ int dir_bit3(int dx, int dy, int dz) {
  constexpr signed char t[27] = {
      25, 17, 24, 15, 5, 14, 23, 16, 22,   // dz = -1
      9, 3, 8, 1, -1, 0, 7, 2, 6,          // dz = 0
      21, 13, 20, 11, 4, 10, 19, 12, 18};  // dz = +1
  return t[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)];
}
// 2D graphs: +x -x +y -y, then xy, -xy, x-y, -x-y (cc3d/cc3d_graphs.hpp:25-29)
__host__ __device__ __forceinline__ int dir_bit2(int dx, int dy) {
  constexpr signed char t[9] = {7, 3, 6, 1, -1, 0, 5, 2, 4};
  return t[(dx + 1) + 3 * (dy + 1)];
}

// ---------------------------------------------------- continuous values
// An input element from its bits (the low sizeof(T) bytes).
template <typename T>
__host__ __device__ __forceinline__ T from_bits(uint64_t b) {
  T v;
  memcpy(&v, &b, sizeof(T));
  return v;
}

__device__ __forceinline__ float abs_diff(float a, float b) { return fabsf(a - b); }
__device__ __forceinline__ double abs_diff(double a, double b) { return fabs(a - b); }
template <typename T>
__device__ __forceinline__ T abs_diff(T a, T b) { return a > b ? T(a - b) : T(b - a); }

// |a - b| <= delta in the element type, as cc3d::match
// (cc3d/cc3d_continuous.hpp:80-88): unsigned without underflow, floating
// point by the rounded difference (NaN never matches).
template <typename T>
__device__ __forceinline__ bool cmatch(T a, T b, T delta) {
  return abs_diff(a, b) <= delta;
}

// The 2D 8-connected continuous labeller's second shortcut
// (cc3d/cc3d_continuous.hpp:301-309): a pixel takes the label above it when
// both lie within delta of the image's minimum and maximum, whether or not
// they match each other.  std::min / std::max order, so a NaN operand fails.
template <typename T>
__device__ __forceinline__ bool span_shortcut(T cur, T up, T gmin, T gmax, T delta) {
  const T mn = (up < cur) ? up : cur;
  const T mx = (cur < up) ? up : cur;
  return (T)(mn - gmin) <= delta && (T)(gmax - mx) <= delta;
}

__device__ __forceinline__ uint32_t lanemask_le(int lane) { return (2u << lane) - 1u; }
__device__ __forceinline__ int head_of(uint32_t starts, int lane) {
  return 31 - __clz(starts & lanemask_le(lane));
}

// ------------------------------------------------------ shared union-find
__device__ __forceinline__ unsigned short sfind(volatile unsigned short* par, unsigned short n,
                                                int lim = kLocalLimit) {
  for (int it = 0; it < lim; ++it) {
    unsigned short p = par[n];
    if (p == n) return n;
    unsigned short g = par[p];
    if (g != p) par[n] = g;
    n = g;
  }
  return n;
}

// find without path compression: used once the unions are done, when every
// thread only reads the forest (no write may race with the flattening)
static __device__ __forceinline__ unsigned short sfind_ro(const volatile unsigned short* par, unsigned short n,
                                                          int lim = kLocalLimit) {
  for (int it = 0; it < lim; ++it) {
    const unsigned short p = par[n];
    if (p == n) return n;
    n = p;
  }
  return n;
}

// Inlined into its one call site in the block-parallel pass (the union
// runner); callers with many sites use sunite_outlined.
static __device__ __forceinline__ bool sunite(unsigned short* par, unsigned short a, unsigned short b,
                                              int lim = kLocalLimit) {
  volatile unsigned short* vp = par;
  for (int it = 0; it < lim; ++it) {
    a = sfind(vp, a, lim);
    b = sfind(vp, b, lim);
    if (a == b) return true;
    if (a < b) { unsigned short t = a; a = b; b = t; }
    // link the larger root under the smaller one
    if (atomicCAS(par + a, a, b) == a) return true;
  }
  return false;
}

// One shared copy of sunite for kernels that call it from many sites, which
// keeps their code inside the instruction cache.
static __device__ __noinline__ bool sunite_outlined(unsigned short* par, unsigned short a, unsigned short b) {
  return sunite(par, a, b);
}

// ------------------------------------------------------ global union-find
__device__ __forceinline__ unsigned long long gload(const unsigned long long* p) {
  return *(const volatile unsigned long long*)p;
}

// Root of node n among the nn nodes of E.  Every parent is range-checked: a
// parent outside [0, nn) sets ERR_INDEX and returns kBadNode, so a corrupt
// entry raises the error word instead of reading outside E.  When the budget
// runs out the node reached so far is returned (with ERR_FIND_BUDGET set).
constexpr uint32_t kBadNode = 0xFFFFFFFFu;
__device__ __forceinline__ uint32_t gfind(unsigned long long* E, uint32_t n, uint32_t nn, Counters* ctr,
                                          int lim = kFindLimit) {
  if (n >= nn) {
    atomicOr(&ctr->err, ERR_INDEX);
    return kBadNode;
  }
  for (int it = 0; it < lim; ++it) {
    unsigned long long e = gload(E + n);
    uint32_t p = (uint32_t)e;
    if (p == n) return n;
    if (p >= nn) break;
    unsigned long long e2 = gload(E + p);
    uint32_t g = (uint32_t)e2;
    if (g >= nn) break;
    if (g != p) *(volatile unsigned long long*)(E + n) = e2;  // path halving
    n = g;
    if (it + 1 == lim) {
      atomicOr(&ctr->err, ERR_FIND_BUDGET);
      return n;
    }
  }
  atomicOr(&ctr->err, ERR_INDEX);
  return kBadNode;
}

__device__ __forceinline__ void gunite(unsigned long long* E, uint32_t a, uint32_t b, uint32_t nn,
                                       uint32_t* bitmap, int64_t nwords, Counters* ctr, int budget = 0) {
  const int flim = limit_of(budget, kFindLimit);
  for (int it = 0, ulim = limit_of(budget, kUniteLimit); it < ulim; ++it) {
    a = gfind(E, a, nn, ctr, flim);
    b = gfind(E, b, nn, ctr, flim);
    if (a == kBadNode || b == kBadNode) return;
    if (a == b) return;
    unsigned long long ea = gload(E + a), eb = gload(E + b);
    if ((uint32_t)ea != a || (uint32_t)eb != b) continue;
    uint32_t ka = (uint32_t)(ea >> 32), kb = (uint32_t)(eb >> 32);
    if (ka < kb) {
      uint32_t t = a; a = b; b = t;
      unsigned long long te = ea; ea = eb; eb = te;
      uint32_t tk = ka; ka = kb; kb = tk;
    }
    const unsigned long long want = ((unsigned long long)kb << 32) | b;
    if (atomicCAS(E + a, ea, want) == ea) {
      if ((int64_t)(ka >> 5) < nwords) atomicAnd(bitmap + (ka >> 5), ~(1u << (ka & 31)));
      else atomicOr(&ctr->err, ERR_INDEX);
      return;
    }
  }
  atomicOr(&ctr->err, ERR_UNITE_BUDGET);
}

// number of component nodes of a labelling (node ids fit 32 bits)
__device__ __forceinline__ uint32_t node_count(const LabelArgs& p) {
  const uint64_t n = (uint64_t)p.ntiles * kTV;
  return n < 0xFFFFFFFFull ? (uint32_t)n : 0xFFFFFFFFu;
}

// component node of a voxel given its tile and in-tile position (x & 31, row);
// indices are range-checked so that a corrupt record raises the error word
// instead of reading outside the buffers
__device__ __forceinline__ uint32_t record_node(const LabelArgs& p, int64_t tile, int row, int lx) {
  if (tile < 0 || tile >= p.ntiles || row < 0 || row >= kRowsPerTile) {
    atomicOr(&p.ctr->err, ERR_INDEX);
    return 0;
  }
  const uint2 m = p.rmask[tile * kRowsPerTile + row];
  const int k = __popc(m.y & lanemask_le(lx)) - 1;
  const int run = (int)p.rrow[tile * kRowsPerTile + row] + k;
  if (k < 0 || run >= kTV) {
    atomicOr(&p.ctr->err, ERR_INDEX);
    return (uint32_t)(tile * kTV);
  }
  const uint16_t c = p.rcomp[tile * kTV + run];
  if (c >= p.tinfo[tile].C) {
    atomicOr(&p.ctr->err, ERR_INDEX);
    return (uint32_t)(tile * kTV);
  }
  return (uint32_t)(tile * kTV + c);
}

// --------------------------------------------------------- block helpers
template <int NT>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* ws, uint32_t& total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(FULL, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = (lane < NT / 32) ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(FULL, w, o);
      if (lane >= o) w += y;
    }
    if (lane < NT / 32) ws[lane] = w;
  }
  __syncthreads();
  total = ws[NT / 32 - 1];
  const uint32_t before = warp ? ws[warp - 1] : 0;
  return before + x - v;
}

// K1 (the tile pass) lives in cc3d_tile.cuh.

// ------------------------------------------------ periodic wrap unions
__device__ __forceinline__ uint32_t voxel_node(const LabelArgs& p, int64_t x, int64_t y, int64_t z) {
  const int64_t tile = (x >> 5) + (int64_t)p.ntx * ((y / p.ty) + (int64_t)p.nty * (z / p.tz));
  const int row = (int)((y % p.ty) + p.ty * (z % p.tz));
  return record_node(p, tile, row, (int)(x & 31));
}

template <typename T, int MODE>
__device__ __forceinline__ bool wrap_related(T a, T b) {
  if (MODE == MODE_MULTI) return a != T(0) && a == b;
  return a != T(0) && b != T(0);
}

// conn: 6 (x, y, z faces), 4 (x, y faces), 8 (x, y faces with diagonals and
// the two corner pairs).  One thread per base position of each face family.
template <typename T, int MODE>
__global__ void k_wrap_pairs(LabelArgs p, int conn) {
  const T* in = static_cast<const T*>(p.in);
  const int64_t sx = p.sx, sy = p.sy, sz = p.sz;
  const int64_t nA = sy * sz, nB = sx * sz, nC = (conn == 6) ? sx * sy : 0, nD = (conn == 8) ? 2 : 0;
  const int64_t total = nA + nB + nC + nD;
  auto at = [&](int64_t x, int64_t y, int64_t z) { return in[(z * sy + y) * sx + x]; };
  auto pair = [&](int64_t ax, int64_t ay, int64_t az, int64_t bx, int64_t by, int64_t bz) {
    if (wrap_related<T, MODE>(at(ax, ay, az), at(bx, by, bz)))
      gunite(p.E, voxel_node(p, ax, ay, az), voxel_node(p, bx, by, bz), node_count(p), p.bitmap, p.nwords, p.ctr,
             p.budget);
  };
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (i < nA) {  // x faces: (0, y, z) with (sx-1, y', z)
      const int64_t y = i % sy, z = i / sy;
      pair(0, y, z, sx - 1, y, z);
      if (conn == 8) {
        if (y > 0) pair(0, y, z, sx - 1, y - 1, z);
        if (y < sy - 1) pair(0, y, z, sx - 1, y + 1, z);
      }
    } else if (i < nA + nB) {  // y faces: (x, 0, z) with (x', sy-1, z)
      const int64_t j = i - nA, x = j % sx, z = j / sx;
      pair(x, 0, z, x, sy - 1, z);
      if (conn == 8) {
        if (x > 0) pair(x, 0, z, x - 1, sy - 1, z);
        if (x < sx - 1) pair(x, 0, z, x + 1, sy - 1, z);
      }
    } else if (i < nA + nB + nC) {  // z faces
      const int64_t j = i - nA - nB, x = j % sx, y = j / sx;
      pair(x, y, 0, x, y, sz - 1);
    } else {  // corners of 8-connected images
      if (i - nA - nB - nC == 0) pair(0, 0, 0, sx - 1, sy - 1, 0);
      else pair(sx - 1, 0, 0, 0, sy - 1, 0);
    }
  }
}

// -------------------------------------------------------------- K3: write
// Label resolution and label writing of a single volume, one warp per tile:
// the labels of the tile's root runs (1 + rank of their root's key among the
// surviving keys), then every run's label (a non-root run copies its root
// run's), then the tile's 64 rows.  Up to 256 runs keep their labels in the
// warp's shared-memory table; a tile with more runs keeps them in the global
// per-run label slots.  With a warp (not a block) per tile, 64 tiles per SM
// have their dependent loads in flight at once.
constexpr int kLabelWarps = 4;
template <typename OUT, int TY, int TZ>
__global__ void __launch_bounds__(kLabelWarps * 32, 12)
k_label_write(LabelArgs p, OUT* out, int64_t count) {
  __shared__ uint32_t slab[kLabelWarps][256];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t t = (int64_t)blockIdx.x * kLabelWarps + w;
  if (t >= count) return;
  const int64_t tile = p.tile_base + t;
  uint32_t* lab = slab[w];
  const uint32_t ntx = (uint32_t)p.ntx, nty = (uint32_t)p.nty;
  const uint32_t rest = (uint32_t)tile / ntx, tz = rest / nty;
  const int64_t x0 = (int64_t)((uint32_t)tile - rest * ntx) * kTX;
  const int64_t y0 = (int64_t)(rest - tz * nty) * TY, z0 = (int64_t)tz * TZ;
  uint32_t C = p.tinfo[tile].C;
  if (C > kTV) {
    if (lane == 0) atomicOr(&p.ctr->err, ERR_INDEX);
    C = kTV;
  }
  const uint32_t node0 = (uint32_t)(tile * kTV);
  // row records of rows lane and lane + 32, fetched while the labels resolve
  const uint2 ma = __ldg(p.rmask + tile * kRowsPerTile + lane), mb = __ldg(p.rmask + tile * kRowsPerTile + 32 + lane);
  const uint32_t ra = __ldg(p.rrow + tile * kRowsPerTile + lane), rb = __ldg(p.rrow + tile * kRowsPerTile + 32 + lane);
  auto root_label = [&](uint32_t c) -> uint32_t {
    const uint32_t R = gfind(p.E, node0 + c, node_count(p), p.ctr, limit_of(p.budget, kFindLimit));
    if (R == kBadNode) return 0u;
    const uint32_t key = (uint32_t)(gload(p.E + R) >> 32);
    const uint32_t wd = key >> 5;
    if (wd >= p.nwords) {
      atomicOr(&p.ctr->err, ERR_INDEX);
      return 0u;
    }
    return __ldg(p.prefix + wd) + __popc(__ldg(p.bitmap + wd) & ((1u << (key & 31)) - 1u)) + 1u;
  };
  const bool fast = C <= 256;
  uint32_t* glab = p.label + node0;
  constexpr int PER = 8;
  for (uint32_t base = 0; base < C; base += 32 * PER) {
    uint32_t rc[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const uint32_t c = base + lane + 32u * k;
      rc[k] = c < C ? (uint32_t)__ldg(p.rcomp + node0 + c) : 0xFFFFFFFFu;
    }
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const uint32_t c = base + lane + 32u * k;
      if (rc[k] != c) continue;  // only root runs name components
      const uint32_t v = root_label(c);
      if (fast) lab[c] = v;
      else glab[c] = v;
    }
  }
  __syncwarp();
  for (uint32_t base = 0; base < C; base += 32 * PER) {
    uint32_t rc[PER], v[PER];
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const uint32_t c = base + lane + 32u * k;
      rc[k] = c < C ? (uint32_t)__ldg(p.rcomp + node0 + c) : c;
    }
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const uint32_t c = base + lane + 32u * k;
      v[k] = 0u;
      if (c < C && rc[k] != c) {
        if (rc[k] < C) v[k] = fast ? lab[rc[k]] : glab[rc[k]];
        else atomicOr(&p.ctr->err, ERR_INDEX);
      }
    }
#pragma unroll
    for (int k = 0; k < PER; ++k) {
      const uint32_t c = base + lane + 32u * k;
      if (c < C && rc[k] != c) {
        if (fast) lab[c] = v[k];
        else glab[c] = v[k];
      }
    }
  }
  __syncwarp();
  // the rows, four per step: lane = 8 * (row of the four) + group; a lane
  // writes the 4 consecutive voxels 4 * group .. 4 * group + 3 of its row
  // with one vector store where the output allows it
  const int g4 = (lane & 7) * 4, rq = lane >> 3;
  const int64_t xg = x0 + g4;
  const bool vec = ((p.sx & 3) == 0) && ((reinterpret_cast<uintptr_t>(out) & (4 * sizeof(OUT) - 1)) == 0) &&
                   (sizeof(OUT) <= 4 || (reinterpret_cast<uintptr_t>(out) & 15) == 0);
  const bool vec4 = vec && xg + 3 < p.sx;  // this lane's four voxels by one store
  // a tile whose rows all lie inside the volume checks no row
  const bool inner = y0 + TY <= p.sy && z0 + TZ <= p.sz;
  const int64_t plane = p.sx * p.sy;
  OUT* base_ptr = out + z0 * plane + y0 * p.sx + xg;
#pragma unroll 2
  for (int r0 = 0; r0 < kRowsPerTile; r0 += 4) {
    const int ri = r0 + rq;
    const uint32_t F = __shfl_sync(FULL, r0 < 32 ? ma.x : mb.x, ri & 31);
    const uint32_t S = __shfl_sync(FULL, r0 < 32 ? ma.y : mb.y, ri & 31);
    const uint32_t b = __shfl_sync(FULL, r0 < 32 ? ra : rb, ri & 31);
    // the row's records hold together (no foreground before its first run
    // start, all its runs below C), checked once per row: then every
    // foreground voxel's run index is in range
    const bool ok = (F & ((S & (0u - S)) - 1u)) == 0u && b + (uint32_t)__popc(S) <= C;
    if (!ok) atomicOr(&p.ctr->err, ERR_INDEX);
    OUT v[4];
    // run of voxel g4 (the last run start at or before it), then of the next three
    uint32_t r = b + (uint32_t)__popc(S & lanemask_le(g4)) - 1u;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (i) r += (S >> (g4 + i)) & 1u;
      v[i] = OUT(0);
      if (ok && ((F >> (g4 + i)) & 1u)) v[i] = (OUT)(fast ? lab[r] : glab[r]);
    }
    const int ly = ri % TY, lz = ri / TY;
    if (!inner && (y0 + ly >= p.sy || z0 + lz >= p.sz)) continue;
    OUT* dst = base_ptr + lz * plane + ly * p.sx;
    if (vec4) {
      if constexpr (sizeof(OUT) == 2) {
        *reinterpret_cast<uint2*>(dst) = make_uint2((uint32_t)v[0] | ((uint32_t)v[1] << 16),
                                                    (uint32_t)v[2] | ((uint32_t)v[3] << 16));
      } else if constexpr (sizeof(OUT) == 4) {
        *reinterpret_cast<uint4*>(dst) = make_uint4((uint32_t)v[0], (uint32_t)v[1], (uint32_t)v[2], (uint32_t)v[3]);
      } else {
        *reinterpret_cast<ulonglong2*>(dst) = make_ulonglong2((unsigned long long)v[0], (unsigned long long)v[1]);
        *reinterpret_cast<ulonglong2*>(dst + 2) = make_ulonglong2((unsigned long long)v[2], (unsigned long long)v[3]);
      }
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (xg + i < p.sx) dst[i] = v[i];
    }
  }
}

}  // namespace cc3dgpu
