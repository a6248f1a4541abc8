// cc3d_label.cuh -- labelling kernels of the GB300 path (sm_103a).
//
// Pipeline for one volume (sizes for a 512^3 uint32 volume in brackets):
//
//   k_tile_local  one CTA per 32 x TY x TZ tile (2048 voxels) [65536 CTAs].
//                 Stages the tile plus a one-voxel backward halo in shared
//                 memory, unions equal-valued neighbours inside the tile with a
//                 shared-memory union-find whose root is the minimum index,
//                 groups halo voxels that are connected inside their own tile,
//                 and unions tile voxels with halo voxels.  Writes
//                   rec[tile][voxel]   16-bit local component id (0xFFFF = bg)
//                   E[tile*2048 + c]   (key << 32 | node) for every component,
//                                      key = row-padded raster index of the
//                                      component's first voxel in the tile
//                   bitmap             one bit per component key
//                   edges              (component node, halo voxel) pairs, one
//                                      per halo group touching the component
//                 and, optionally, the provisional-label estimate (epl) and the
//                 first/last foreground row, which need the same read.
//   k_merge_edges global union-find over component nodes: the parent of a root
//                 is only ever set to a root with a smaller key (atomicCAS on the
//                 packed (key, parent) word), so every tree's root holds the
//                 component's first voxel.  A root that is linked clears its
//                 bit in the numbering bitmap.
//   k_wrap_pairs  periodic boundaries: unions across the wrapped faces.
//   scan          exclusive popcount prefix of the bitmap = the rank of every
//                 surviving key, i.e. the component's number minus one.
//   k_write       label of every component = 1 + rank(key of its root);
//                 every voxel's label is its component's label.
//
// All loops that wait for other threads (the union-find retries) carry an
// iteration budget; when it runs out they set a bit in the device error word
// and stop, and the host turns that into an error return.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace cc3dgpu {

constexpr int kTX = 32;          // tile width in x (one warp per row)
constexpr int kTV = 2048;        // voxels per tile (every tile shape)
constexpr int kThreads = 256;    // threads per CTA of the tile kernels
constexpr uint16_t kBg = 0xFFFF; // local component id of background voxels
constexpr unsigned FULL = 0xFFFFFFFFu;

// relation modes
constexpr int MODE_MULTI = 0;    // neighbours join when equal and nonzero
constexpr int MODE_BINARY = 1;   // neighbours join when both nonzero
constexpr int MODE_BINARY4 = 2;  // the reference's binary 4-connected relation

// device error bits
constexpr unsigned ERR_UNITE_BUDGET = 1u;
constexpr unsigned ERR_FIND_BUDGET = 2u;
constexpr unsigned ERR_EDGE_OVERFLOW = 4u;
constexpr unsigned ERR_LOCAL_BUDGET = 8u;

constexpr int kFindLimit = 1 << 24;
constexpr int kUniteLimit = 1 << 20;
constexpr int kLocalLimit = 1 << 16;

struct Counters {
  unsigned int edge_count;
  unsigned int err;
  unsigned long long prov;   // provisional labels of the reference's binary labellers
  unsigned long long N;
  unsigned long long epl;
  long long first_row;
  long long last_row;
  unsigned long long pad[2];
};

struct LabelArgs {
  const void* in;
  int64_t sx, sy, sz;
  int ntx, nty, ntz;
  int ty, tz;                  // tile shape (TY, TZ) at run time
  int64_t wpr;                 // bitmap words per padded row
  int64_t key_row;             // wpr * 32
  uint16_t* rec;
  unsigned long long* E;
  uint32_t* ccount;
  uint32_t* bitmap;
  uint32_t* prefix;
  uint2* edges;
  unsigned int edge_cap;
  Counters* ctr;
  int want_epl;
  int want_prov;
};

// ---------------------------------------------------------------- neighbours
template <int CONN> struct NbCount;
template <> struct NbCount<26> { static constexpr int n = 13; };
template <> struct NbCount<18> { static constexpr int n = 9; };
template <> struct NbCount<6> { static constexpr int n = 3; };
template <> struct NbCount<8> { static constexpr int n = 4; };
template <> struct NbCount<4> { static constexpr int n = 2; };

// backward neighbour k of the connectivity: raster-earlier voxels
template <int CONN>
__device__ __forceinline__ void nb_off(int k, int& dx, int& dy, int& dz) {
  if (CONN == 26) {
    if (k < 9) { dz = -1; dy = k / 3 - 1; dx = k % 3 - 1; }
    else if (k < 12) { dz = 0; dy = -1; dx = k - 10; }
    else { dz = 0; dy = 0; dx = -1; }
  } else if (CONN == 18) {
    const int t[9][3] = {{0, -1, -1}, {-1, 0, -1}, {0, 0, -1}, {1, 0, -1}, {0, 1, -1},
                         {-1, -1, 0}, {0, -1, 0}, {1, -1, 0}, {-1, 0, 0}};
    dx = t[k][0]; dy = t[k][1]; dz = t[k][2];
  } else if (CONN == 6) {
    dx = (k == 2) ? -1 : 0; dy = (k == 1) ? -1 : 0; dz = (k == 0) ? -1 : 0;
  } else if (CONN == 8) {
    if (k < 3) { dz = 0; dy = -1; dx = k - 1; } else { dz = 0; dy = 0; dx = -1; }
  } else {  // 4
    dz = 0; dy = (k == 0) ? -1 : 0; dx = (k == 1) ? -1 : 0;
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

// ------------------------------------------------------ shared union-find
__device__ __forceinline__ unsigned short sfind(volatile unsigned short* par, unsigned short n) {
  for (int it = 0; it < kLocalLimit; ++it) {
    unsigned short p = par[n];
    if (p == n) return n;
    unsigned short g = par[p];
    if (g != p) par[n] = g;
    n = g;
  }
  return n;
}

__device__ __forceinline__ bool sunite(unsigned short* par, unsigned short a, unsigned short b) {
  volatile unsigned short* vp = par;
  for (int it = 0; it < kLocalLimit; ++it) {
    a = sfind(vp, a);
    b = sfind(vp, b);
    if (a == b) return true;
    if (a < b) { unsigned short t = a; a = b; b = t; }
    // link the larger root under the smaller one
    if (atomicCAS(par + a, a, b) == a) return true;
  }
  return false;
}

// ------------------------------------------------------ global union-find
__device__ __forceinline__ unsigned long long gload(const unsigned long long* p) {
  return *(const volatile unsigned long long*)p;
}

__device__ __forceinline__ uint32_t gfind(unsigned long long* E, uint32_t n, Counters* ctr) {
  for (int it = 0; it < kFindLimit; ++it) {
    unsigned long long e = gload(E + n);
    uint32_t p = (uint32_t)e;
    if (p == n) return n;
    unsigned long long e2 = gload(E + p);
    uint32_t g = (uint32_t)e2;
    if (g != p) *(volatile unsigned long long*)(E + n) = e2;  // path halving
    n = g;
  }
  atomicOr(&ctr->err, ERR_FIND_BUDGET);
  return n;
}

__device__ __forceinline__ void gunite(unsigned long long* E, uint32_t a, uint32_t b,
                                       uint32_t* bitmap, Counters* ctr) {
  for (int it = 0; it < kUniteLimit; ++it) {
    a = gfind(E, a, ctr);
    b = gfind(E, b, ctr);
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
      atomicAnd(bitmap + (ka >> 5), ~(1u << (ka & 31)));
      return;
    }
  }
  atomicOr(&ctr->err, ERR_UNITE_BUDGET);
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

// ------------------------------------------------------------ K1: tiles
template <typename T, int CONN, int TY, int TZ, int MODE, bool BLOCK8>
__global__ void __launch_bounds__(kThreads)
k_tile_local(LabelArgs p) {
  using S = typename Stored<T, MODE>::type;
  constexpr bool D3 = (CONN == 26 || CONN == 18 || CONN == 6);
  constexpr int HZ = D3 ? 1 : 0;
  constexpr int BX = kTX + 2, BY = TY + 2, BZ = TZ + HZ;
  constexpr int BOX = BX * BY * BZ;
  constexpr int NODES = kTV + BOX;
  constexpr int NW = kThreads / 32;
  constexpr int NB = NbCount<CONN>::n;
  static_assert(kTX * TY * TZ == kTV, "tile must hold 2048 voxels");
  static_assert(NODES < 65535, "node ids must fit 16 bits");

  __shared__ S sv[BOX];
  __shared__ unsigned short par[NODES];
  __shared__ unsigned short cid[kTV];
  __shared__ uint8_t grp[BOX];
  __shared__ uint32_t ws[NW];
  __shared__ uint32_t minblk[BLOCK8 ? kTV : 1];
  __shared__ unsigned long long red_epl[NW];
  __shared__ long long red_first[NW], red_last[NW];
  __shared__ unsigned int red_prov[NW];
  __shared__ unsigned int local_err;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t tile = blockIdx.x;
  const int tx = (int)(tile % p.ntx);
  const int64_t rest = tile / p.ntx;
  const int ty = (int)(rest % p.nty);
  const int tz = (int)(rest / p.nty);
  const int64_t x0 = (int64_t)tx * kTX, y0 = (int64_t)ty * TY, z0 = (int64_t)tz * TZ;
  const T* in = static_cast<const T*>(p.in);

  if (tid == 0) local_err = 0;

  // ---- phase 0: stage tile + halo; epl on the tile's own rows
  unsigned long long epl_acc = 0;
  long long frow = 0x7FFFFFFFFFFFFFFFLL, lrow = -1;
  for (int r = warp; r < BY * BZ; r += NW) {
    const int by = r % BY, bz = r / BY;
    const int64_t y = y0 - 1 + by, z = z0 - HZ + bz;
    const bool rowin = (y >= 0) && (y < p.sy) && (z >= 0) && (z < p.sz);
    const int64_t x = x0 + lane;
    T v = T(0), vl = T(0), vr = T(0);
    if (rowin) {
      const T* rowp = in + (z * p.sy + y) * p.sx;
      if (x < p.sx) v = rowp[x];
      if (lane == 0 && x0 > 0) vl = rowp[x0 - 1];
      if (lane == 0 && x0 + kTX < p.sx) vr = rowp[x0 + kTX];
    }
    S* row = sv + r * BX;
    row[lane + 1] = to_stored<S, T, MODE>(v);
    if (lane == 0) {
      row[0] = to_stored<S, T, MODE>(vl);
      row[BX - 1] = to_stored<S, T, MODE>(vr);
    }
    if (p.want_epl && by >= 1 && by <= TY && bz >= HZ) {
      T prev = __shfl_up_sync(FULL, v, 1);
      if (lane == 0) prev = vl;
      const bool t = rowin && (x < p.sx) && (v != prev) && (v != T(0));
      const unsigned m = __ballot_sync(FULL, t);
      if (m) {
        epl_acc += __popc(m);
        const long long rg = (long long)(y + p.sy * z);
        frow = rg < frow ? rg : frow;
        lrow = rg > lrow ? rg : lrow;
      }
    }
  }
  for (int n = tid; n < NODES; n += kThreads) par[n] = (unsigned short)n;
  __syncthreads();

  auto tile_box = [&](int t) -> int {
    const int lx = t & 31, ri = t >> 5, ly = ri % TY, lz = ri / TY;
    return ((lz + HZ) * BY + (ly + 1)) * BX + lx + 1;
  };
  auto in_tile = [&](int bx, int by, int bz) -> bool {
    return bx >= 1 && bx <= kTX && by >= 1 && by <= TY && bz >= HZ;
  };
  auto owner = [&](int bx, int by, int bz) -> int {
    const int ox = bx == 0 ? 0 : (bx == BX - 1 ? 2 : 1);
    const int oy = by == 0 ? 0 : (by == BY - 1 ? 2 : 1);
    const int oz = bz < HZ ? 0 : 1;
    return ox + 3 * (oy + 3 * oz);
  };
  // relation between box positions a (later voxel) and b = a + (dx,dy,dz)
  auto related = [&](int a, int b, int dy, int dz, int64_t gy, int64_t gz) -> bool {
    const S va = sv[a], vb = sv[b];
    if (MODE == MODE_BINARY) return is_fg(va) && is_fg(vb);
    if (MODE == MODE_MULTI) return is_fg(va) && va == vb;
    // MODE_BINARY4: vertical pairs join when both are foreground; horizontal
    // pairs of the first row join only when equal, later rows skip the link
    // when both pixels have foreground directly above.
    if (!(is_fg(va) && is_fg(vb))) return false;
    if (dy != 0 || dz != 0) return true;
    if (gy == 0 && gz == 0) return va == vb;
    return !(is_fg(sv[a - BX]) && is_fg(sv[b - BX]));
  };

  // ---- phase 1: tile-tile and same-owner halo-halo unions
  for (int t = tid; t < kTV; t += kThreads) {
    const int lx = t & 31, ri = t >> 5, ly = ri % TY, lz = ri / TY;
    const int a = tile_box(t);
    if (!is_fg(sv[a])) continue;
#pragma unroll
    for (int k = 0; k < NB; ++k) {
      int dx, dy, dz;
      nb_off<CONN>(k, dx, dy, dz);
      const int nx = lx + dx, ny = ly + dy, nz = lz + dz;
      if (nx < 0 || nx >= kTX || ny < 0 || ny >= TY || nz < 0 || nz >= TZ) continue;
      const int b = a + dx + BX * (dy + BY * dz);
      if (related(a, b, dy, dz, y0 + ly, z0 + lz)) {
        if (!sunite(par, (unsigned short)t, (unsigned short)(nx + kTX * (ny + TY * nz)))) local_err = 1;
      }
    }
  }
  for (int a = tid; a < BOX; a += kThreads) {
    const int bx = a % BX, by = (a / BX) % BY, bz = a / (BX * BY);
    if (in_tile(bx, by, bz) || !is_fg(sv[a])) continue;
    const int own = owner(bx, by, bz);
#pragma unroll
    for (int k = 0; k < NB; ++k) {
      int dx, dy, dz;
      nb_off<CONN>(k, dx, dy, dz);
      if (MODE == MODE_BINARY4 && dy == 0) continue;  // needs the row above the box
      const int nx = bx + dx, ny = by + dy, nz = bz + dz;
      if (nx < 0 || nx >= BX || ny < 0 || ny >= BY || nz < 0 || nz >= BZ) continue;
      if (in_tile(nx, ny, nz) || owner(nx, ny, nz) != own) continue;
      const int b = a + dx + BX * (dy + BY * dz);
      if (related(a, b, dy, dz, y0 - 1 + by, z0 - HZ + bz)) {
        if (!sunite(par, (unsigned short)(kTV + a), (unsigned short)(kTV + b))) local_err = 1;
      }
    }
  }
  __syncthreads();

  // ---- phase 1.5: halo groups (roots of the halo-only forest)
  for (int a = tid; a < BOX; a += kThreads) {
    const int bx = a % BX, by = (a / BX) % BY, bz = a / (BX * BY);
    grp[a] = (!in_tile(bx, by, bz) && is_fg(sv[a]) &&
              sfind(par, (unsigned short)(kTV + a)) == kTV + a) ? 1 : 0;
  }
  __syncthreads();

  // ---- phase 2: tile-halo unions
  for (int t = tid; t < kTV; t += kThreads) {
    const int lx = t & 31, ri = t >> 5, ly = ri % TY, lz = ri / TY;
    const int a = tile_box(t);
    if (!is_fg(sv[a])) continue;
#pragma unroll
    for (int k = 0; k < NB; ++k) {
      int dx, dy, dz;
      nb_off<CONN>(k, dx, dy, dz);
      const int nx = lx + dx, ny = ly + dy, nz = lz + dz;
      if (!(nx < 0 || nx >= kTX || ny < 0 || ny >= TY || nz < 0 || nz >= TZ)) continue;
      const int b = a + dx + BX * (dy + BY * dz);
      if (related(a, b, dy, dz, y0 + ly, z0 + lz)) {
        if (!sunite(par, (unsigned short)t, (unsigned short)(kTV + b))) local_err = 1;
      }
    }
  }
  __syncthreads();

  // ---- phase 3a: roots of tile nodes -> dense component ids (tile raster order)
  constexpr int NPT = kTV / kThreads;
  uint32_t cnt = 0, rootbits = 0;
#pragma unroll
  for (int k = 0; k < NPT; ++k) {
    const int t = tid * NPT + k;
    if (is_fg(sv[tile_box(t)])) {
      const unsigned short r = sfind(par, (unsigned short)t);
      par[t] = r;
      if (r == t) { rootbits |= 1u << k; ++cnt; }
    }
  }
  uint32_t C;
  uint32_t base = block_exclusive_scan<kThreads>(cnt, ws, C);
#pragma unroll
  for (int k = 0; k < NPT; ++k)
    if (rootbits >> k & 1u) cid[tid * NPT + k] = (unsigned short)(base++);
  if (BLOCK8)
    for (uint32_t c = tid; c < C; c += kThreads) minblk[c] = 0xFFFFFFFFu;
  __syncthreads();

  // ---- phase 3b: local component of every voxel
  uint16_t* rec = p.rec + tile * kTV;
  for (int t = tid; t < kTV; t += kThreads) {
    const bool f = is_fg(sv[tile_box(t)]);
    const unsigned short c = f ? cid[par[t]] : kBg;
    rec[t] = c;
    if (BLOCK8 && f) {
      const int lx = t & 31, ly = t >> 5;
      const uint32_t blk = (uint32_t)(((y0 + ly) >> 1) * p.key_row + ((x0 + lx) >> 1));
      atomicMin(&minblk[c], blk);
    }
  }
  if (BLOCK8) __syncthreads();

  // ---- phase 3c: component nodes, keys and the numbering bitmap
  const uint32_t node0 = (uint32_t)(tile * kTV);
  for (int t = tid; t < kTV; t += kThreads) {
    if (!is_fg(sv[tile_box(t)]) || par[t] != t) continue;
    const uint32_t c = cid[t];
    uint32_t key;
    if (BLOCK8) {
      key = minblk[c];
      atomicOr(p.bitmap + (key >> 5), 1u << (key & 31));
    } else {
      const int lx = t & 31, ri = t >> 5, ly = ri % TY, lz = ri / TY;
      key = (uint32_t)(((z0 + lz) * p.sy + (y0 + ly)) * p.key_row + x0 + lx);
    }
    p.E[node0 + c] = ((unsigned long long)key << 32) | (node0 + c);
  }
  if (!BLOCK8) {
    for (int ri = warp; ri < TY * TZ; ri += NW) {
      const int t = ri * kTX + lane;
      const bool root = is_fg(sv[tile_box(t)]) && par[t] == t;
      const unsigned m = __ballot_sync(FULL, root);
      const int ly = ri % TY, lz = ri / TY;
      const int64_t y = y0 + ly, z = z0 + lz;
      if (lane == 0 && y < p.sy && z < p.sz) p.bitmap[(z * p.sy + y) * p.wpr + tx] = m;
    }
  }

  // ---- phase 3d: one edge per halo group that joined a tile component
  for (int a = tid; a < BOX; a += kThreads) {
    if (!grp[a]) continue;
    const unsigned short r = sfind(par, (unsigned short)(kTV + a));
    if (r >= kTV) continue;
    const int bx = a % BX, by = (a / BX) % BY, bz = a / (BX * BY);
    const int64_t gx = x0 - 1 + bx, gy = y0 - 1 + by, gz = z0 - HZ + bz;
    const int64_t otile = (gx >> 5) + (int64_t)p.ntx * ((gy / TY) + (int64_t)p.nty * (gz / TZ));
    const uint32_t local = (uint32_t)((gx & 31) + kTX * ((gy % TY) + TY * (gz % TZ)));
    const unsigned slot = atomicAdd(&p.ctr->edge_count, 1u);
    if (slot < p.edge_cap) p.edges[slot] = make_uint2(node0 + cid[r], (uint32_t)(otile * kTV + local));
    else atomicOr(&p.ctr->err, ERR_EDGE_OVERFLOW);
  }

  // ---- provisional labels the reference's binary labeller would open
  unsigned int prov = 0;
  if (p.want_prov) {
    if (BLOCK8) {
      // 2x2 blocks: Y Z / X W at (x, y); C D E F above, B A to the left
      for (int q = tid; q < kTV / 4; q += kThreads) {
        const int bxq = q & 15, byq = q >> 4;
        const int lx = 2 * bxq, ly = 2 * byq;
        const int a = tile_box(lx + kTX * ly);
        const bool Y = is_fg(sv[a]), Z = is_fg(sv[a + 1]);
        const bool X = is_fg(sv[a + BX]), W = is_fg(sv[a + BX + 1]);
        if (!(Y || Z || X || W)) continue;
        const bool Cc = is_fg(sv[a - BX - 1]), D = is_fg(sv[a - BX]);
        const bool Ee = is_fg(sv[a - BX + 1]), F = is_fg(sv[a - BX + 2]);
        const bool B = is_fg(sv[a - 1]), A = is_fg(sv[a + BX - 1]);
        const bool linked = (Y && (Cc || D || Ee || B || A)) || (Z && (D || Ee || F)) || (X && (B || A));
        prov += linked ? 0u : 1u;
      }
    } else {
      for (int t = tid; t < kTV; t += kThreads) {
        const int lx = t & 31, ri = t >> 5, ly = ri % TY, lz = ri / TY;
        const int a = tile_box(t);
        if (!is_fg(sv[a])) continue;
        bool linked = false;
#pragma unroll
        for (int k = 0; k < NB; ++k) {
          int dx, dy, dz;
          nb_off<CONN>(k, dx, dy, dz);
          const int b = a + dx + BX * (dy + BY * dz);
          if (MODE == MODE_BINARY4 && dy == 0 && dz == 0 && y0 + ly == 0 && z0 + lz == 0)
            linked |= (sv[a] == sv[b]);
          else
            linked |= is_fg(sv[b]);
        }
        (void)lx;
        prov += linked ? 0u : 1u;
      }
    }
  }

  // ---- reductions
  if (lane == 0) {
    red_epl[warp] = epl_acc;
    red_first[warp] = frow;
    red_last[warp] = lrow;
  }
  unsigned int pw = prov;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) pw += __shfl_down_sync(FULL, pw, o);
  if (lane == 0) red_prov[warp] = pw;
  __syncthreads();
  if (tid == 0) {
    unsigned long long e = 0, pv = 0;
    long long f = 0x7FFFFFFFFFFFFFFFLL, l = -1;
    for (int w = 0; w < NW; ++w) {
      e += red_epl[w];
      pv += red_prov[w];
      f = red_first[w] < f ? red_first[w] : f;
      l = red_last[w] > l ? red_last[w] : l;
    }
    if (p.want_epl && e) {
      atomicAdd(&p.ctr->epl, e);
      atomicMin(&p.ctr->first_row, f);
      atomicMax(&p.ctr->last_row, l);
    }
    if (pv) atomicAdd(&p.ctr->prov, pv);
    p.ccount[tile] = C;
    if (local_err) atomicOr(&p.ctr->err, ERR_LOCAL_BUDGET);
  }
}

// ------------------------------------------------------ K2: edge merges
__global__ void k_merge_edges(LabelArgs p);

// ------------------------------------------------ periodic wrap unions
// node of voxel (x, y, z): its tile's component node
__device__ __forceinline__ uint32_t voxel_node(const LabelArgs& p, int64_t x, int64_t y, int64_t z) {
  const int64_t tile = (x >> 5) + (int64_t)p.ntx * ((y / p.ty) + (int64_t)p.nty * (z / p.tz));
  const int64_t local = (x & 31) + kTX * ((y % p.ty) + p.ty * (z % p.tz));
  return (uint32_t)(tile * kTV + p.rec[tile * kTV + local]);
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
      gunite(p.E, voxel_node(p, ax, ay, az), voxel_node(p, bx, by, bz), p.bitmap, p.ctr);
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
template <typename OUT, int TY, int TZ>
__global__ void __launch_bounds__(kThreads)
k_write(LabelArgs p, OUT* out) {
  __shared__ uint32_t lab[kTV];
  const int tid = threadIdx.x;
  const int64_t tile = blockIdx.x;
  const int tx = (int)(tile % p.ntx);
  const int64_t rest = tile / p.ntx;
  const int ty = (int)(rest % p.nty);
  const int tz = (int)(rest / p.nty);
  const int64_t x0 = (int64_t)tx * kTX, y0 = (int64_t)ty * TY, z0 = (int64_t)tz * TZ;
  const uint32_t C = p.ccount[tile];
  const uint32_t node0 = (uint32_t)(tile * kTV);
  for (uint32_t c = tid; c < C; c += kThreads) {
    const uint32_t R = gfind(p.E, node0 + c, p.ctr);
    const uint32_t key = (uint32_t)(gload(p.E + R) >> 32);
    const uint32_t w = key >> 5;
    const uint32_t below = __ldg(p.bitmap + w) & ((1u << (key & 31)) - 1u);
    lab[c] = __ldg(p.prefix + w) + __popc(below) + 1u;
  }
  __syncthreads();
  const uint16_t* rec = p.rec + tile * kTV;
  for (int t = tid; t < kTV; t += kThreads) {
    const int lx = t & 31, ri = t >> 5, ly = ri % TY, lz = ri / TY;
    const int64_t x = x0 + lx, y = y0 + ly, z = z0 + lz;
    if (x >= p.sx || y >= p.sy || z >= p.sz) continue;
    const uint16_t c = rec[t];
    out[(z * p.sy + y) * p.sx + x] = (c == kBg) ? OUT(0) : (OUT)lab[c];
  }
}

}  // namespace cc3dgpu
