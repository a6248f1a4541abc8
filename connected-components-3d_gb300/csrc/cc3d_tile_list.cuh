// cc3d_tile_list.cuh -- the tile pass (K1) for multilabel and binary volumes,
// "list" variant.
//
// One 256-thread CTA labels one 32 x TY x TZ tile (2048 voxels) together with
// its one-voxel backward halo, all in shared memory, and writes the same
// records as k_tile_runs (run masks, run components, component keys, the
// numbering bitmap, one edge per halo run joined to a tile component).  It is
// built around how few voxels need more than one test:
//
//   * Every voxel of the 18- and 26-connected labellers (cc3d/cc3d.hpp:344-755)
//     and of the 8-connected one (:1287-1421) that relates to its "primary"
//     neighbour -- the voxel below (z - 1) for 26, below and behind (y - 1) for
//     18, behind for 8 -- needs no other test: each of its other backward
//     neighbours is also a neighbour of the primary one, earlier in raster
//     order, and related to it when related to the voxel, so that pair is
//     joined by induction over the raster order.  The voxel's own join with
//     its link row (below in 3D, behind in 2D) is one union per pair of runs
//     (this row's run, the link row's run) where the pair starts; the first
//     such pair of every run is a direct parent link to the link row's run,
//     so union-find trees are short chains along z.
//   * The other ("needy") voxels are few (background faces and isolated
//     values): they go to a per-warp list and each is then handled by one
//     lane, which tests its remaining backward neighbours itself.  A voxel
//     that continues a run (equal to its left neighbour) skips the neighbours
//     that its left neighbour already sees, and a diagonal relation is skipped
//     where the same neighbour run is already joined through the dx = 0
//     relation.
//   * 6- and 4-connected labellers have no primary neighbour: every row pair
//     contributes one union per starting pair of runs, found by ballots.
//
// Indices are 32-bit (tile and node ids fit 32 bits), and the geometry of
// every box row (its tile, its row inside that tile, its global row, its
// same-owner predecessor) comes from tables built once per tile.  A
// component is named by its root run: the smallest node of its tree, i.e.
// its first run in tile raster order; the name is that run's index in the
// tile's run order, so no separate component numbering is needed.
//
// Phases: 0 box by TMA (or plain loads), row tables; 1 run masks of every box
// row, union-find nodes of the run heads, the provisional-label estimate
// (cc3d/cc3d.hpp:287-315); 2a primary relations, direct links, the warp's
// union list; 2b its unions; 3 roots, run records, keys, bitmap (halo heads
// are pointed at their roots); 4 halo edges, the binary labellers'
// provisional count, per-tile results.
#pragma once

#include <type_traits>

#include "cc3d_tile.cuh"

namespace cc3dgpu {

// Backward relations that a needy voxel tests itself, per connectivity: the
// neighbour row (RowNb order, row_nb), the x offset, and whether the relation
// is implied through the left neighbour when the voxel continues a run (the
// neighbour is then also a backward neighbour of the left voxel).  The
// primary row's dx = 0 relation is not listed: it is the row-level pair.
// Packed 4 bits per relation: bits 0-1 row, bit 2-3 dx + 1; a mask of the
// relations implied through the left neighbour.
template <int CONN> struct NeedRels;
// 26: rows (dy, dz) = (-1, 0), (-1, -1), (0, -1) [primary], (1, -1); all dx.
template <> struct NeedRels<26> {
  static constexpr int n = 11;
  //                  (0,-1) (0,0) (0,1) (1,-1) (1,0) (1,1) (2,-1) (2,1) (3,-1) (3,0) (3,1)
  static constexpr unsigned long long code =
      (0x0ull << 0) | (0x4ull << 4) | (0x8ull << 8) | (0x1ull << 12) | (0x5ull << 16) | (0x9ull << 20) |
      (0x2ull << 24) | (0xAull << 28) | (0x3ull << 32) | (0x7ull << 36) | (0xBull << 40);
  static constexpr unsigned left = 0b01101011011u;  // relations with dx <= 0
};
// 18: row 0 (behind) all dx, row 1 dx = 0, row 2 (below, primary) dx = -1 and
// +1, row 3 dx = 0.  Implied through the left neighbour: row 0 dx <= 0, row 2
// dx = -1.
template <> struct NeedRels<18> {
  static constexpr int n = 7;
  //                  (0,-1) (0,0) (0,1) (1,0) (2,-1) (2,1) (3,0)
  static constexpr unsigned long long code =
      (0x0ull << 0) | (0x4ull << 4) | (0x8ull << 8) | (0x5ull << 12) | (0x2ull << 16) | (0xAull << 20) |
      (0x7ull << 24);
  static constexpr unsigned left = 0b0010011u;
};
// 8: the row behind (primary) at dx = -1 and +1.
template <> struct NeedRels<8> {
  static constexpr int n = 2;
  static constexpr unsigned long long code = (0x0ull << 0) | (0x8ull << 4);
  static constexpr unsigned left = 0b01u;
};
template <> struct NeedRels<6> {
  static constexpr int n = 0;
  static constexpr unsigned long long code = 0;
  static constexpr unsigned left = 0;
};
template <> struct NeedRels<4> {
  static constexpr int n = 0;
  static constexpr unsigned long long code = 0;
  static constexpr unsigned left = 0;
};

// Union-find over parent words in shared memory: 32-bit words (a native
// shared-memory CAS) where the tile fits the static shared-memory budget with
// them, else 16-bit words (8-byte elements).  A root is linked under the
// smaller root, so the root of every tree is its smallest node.  Every loop
// is bounded.
template <typename PT>
static __device__ __forceinline__ uint32_t lfind(volatile PT* par, uint32_t n, int lim) {
  for (int it = 0; it < lim; ++it) {
    const uint32_t p = par[n];
    if (p == n) return n;
    const uint32_t g = par[p];
    if (g != p) par[n] = (PT)g;  // path halving
    n = g;
  }
  return n;
}
template <typename PT>
static __device__ __forceinline__ uint32_t lfind_ro(const volatile PT* par, uint32_t n, int lim) {
  for (int it = 0; it < lim; ++it) {
    const uint32_t p = par[n];
    if (p == n) return n;
    n = p;
  }
  return n;
}
template <typename PT>
static __device__ __forceinline__ bool lunite(PT* par, uint32_t a, uint32_t b, int lim) {
  volatile PT* vp = par;
  for (int it = 0; it < lim; ++it) {
    a = lfind<PT>(vp, a, lim);
    b = lfind<PT>(vp, b, lim);
    if (a == b) return true;
    if (a < b) { const uint32_t t = a; a = b; b = t; }
    if ((uint32_t)atomicCAS(par + a, (PT)a, (PT)b) == a) return true;
  }
  return false;
}

// Tile rows of warp w: the j-th of its 8 rows.  A warp owns whole columns of
// rows along the link direction (z in 3D, y in 2D) and takes them from the
// bottom up, so the link row of its j-th row is, for all but its first rows,
// one of its own earlier rows: by the time a warp resolves a row's roots, the
// link row's runs already point at theirs and the finds stay short.
template <int TY>
__device__ __forceinline__ int warp_row(int w, int j) {
  if constexpr (TY == 16) return (w + 8 * (j & 1)) + 16 * (j >> 1);
  else if constexpr (TY == 8) return w + 8 * j;
  else if constexpr (TY == 4) return (w & 3) + 4 * (8 * (w >> 2) + j);
  else return 8 * w + j;  // 2D: 64 x 1 tiles
}

// One tile of the list pass, by the whole 256-thread block: the kernel below
// runs one per block; the persistent batch kernel (cc3d_batch_persistent.cu)
// runs many in a row (the block's shared memory is free again once it
// returns).  `tmap` is used only when use_tma is set.
// The unions of a warp's pair buffer q[0, n), lane i taking entries i, i + 32,
// ... (pairs (a << 16) | b).  Not inlined: every site that flushes the buffer
// shares one copy of the union-find code.  Returns 1 if a union ran out of
// budget.
template <typename PT>
static __device__ __noinline__ int list_unions(const uint32_t* q, int n, PT* par, int lim, int lane) {
  __syncwarp();
  int err = 0;
  for (int r0 = 0; r0 < n; r0 += 32) {
    if (r0 + lane < n) {
      const uint32_t e = q[r0 + lane];
      if (!lunite<PT>(par, e >> 16, e & 0xFFFFu, lim)) err = 1;
    }
  }
  __syncwarp();
  return err;
}

// LOOP: the caller labels tile after tile in one block (the persistent batch)
template <typename T, int CONN, int TY, int TZ, int MODE, bool LOOP = false>
__device__ __forceinline__ void tile_list_tile(const LabelArgs& p, const CUtensorMap* tmap, int use_tma,
                                               int64_t tile) {
  static_assert(MODE == MODE_MULTI || MODE == MODE_BINARY, "multilabel or binary relation");
  constexpr bool D3 = (CONN == 26 || CONN == 18 || CONN == 6);
  constexpr int HZ = D3 ? 1 : 0;
  constexpr int BY = TY + 2, BZ = TZ + HZ;
  constexpr int NRB = BY * BZ;           // box rows (tile + halo)
  constexpr int NR = TY * TZ;            // tile rows
  constexpr int NHR = NRB - NR;          // halo rows
  constexpr int HNODE = kTV;             // halo-row run heads: HNODE + (halo row) * 32 + x
  constexpr int CNODE = kTV + NHR * 32;  // columns: CNODE + rb (x0 - 1), CNODE + NRB + rb (x0 + 32)
  constexpr int NODES = CNODE + 2 * NRB;
  constexpr int NW = kThreads / 32;
  constexpr int RPW = NR / NW;           // tile rows per warp
  constexpr int NRN = RowNb<CONN>::n;
  constexpr int W = BoxRow<T>::W, PADX = BoxRow<T>::PADX;
  // a primary neighbour row decides most voxels (26, 18: below; 8: behind)
  constexpr bool PRIMARY = (CONN == 26 || CONN == 18 || CONN == 8);
  // the link row: every run's first pair of runs with it becomes a direct
  // parent link (below in 3D, behind in 2D)
  constexpr int LOFF = D3 ? -BY : -1;
  constexpr int LSTEP = D3 ? TY : 1;     // tile-row distance to the link row
  constexpr int LROW0 = D3 ? TY : 1;     // first tile row whose link row is a tile row
  constexpr int QN = RPW * 32;           // list capacity: every voxel of the warp's rows
  using NRel = NeedRels<CONN>;
  constexpr int NB = NRel::n;
  static_assert(kTX * NR == kTV, "tile must hold 2048 voxels");
  static_assert(NR == kRowsPerTile, "64 rows per tile");
  static_assert(RPW == 8, "8 rows per warp");
  static_assert(NODES < 16384, "node ids must fit 14 bits");
  static_assert(W <= 256 && BY <= 256 && BZ <= 256, "TMA box dimensions");

  __shared__ __align__(128) T box[NRB * W];
  __shared__ __align__(8) uint64_t tbar;
  __shared__ uint32_t smask[NRB], fmask[NRB];
  using PT = typename std::conditional<sizeof(T) == 8, unsigned short, uint32_t>::type;
  __shared__ __align__(16) PT par[NODES];
  __shared__ unsigned short nbase[NRB];     // node id of every box row's voxel 0
  // per box row: the tile holding its 32 voxels and the row's index inside
  // that tile; the same-owner box row before it (one back in y, else in z;
  // 255: none)
  __shared__ unsigned char rloc[NRB], rprev[NRB], rown[NRB];
  __shared__ TileGeo sgeo;  // the tile's place in its volume (one warp works it out)
  // the tile's list: one entry per voxel that has unions to run,
  // (needy << 14) | (row-level pairs << 11) | (tile row << 5) | x; in phase C
  // each warp's slice holds the run heads of its rows
  __shared__ unsigned short ulist[NW][QN];
  // per tile row: the ballot of its relations with its link row (M) and, for
  // 18 and 6, with the row behind; for 6 and 4 whether x = 0 relates to the
  // column x0 - 1
  __shared__ uint32_t mmask[NR], m2mask[NR];
  __shared__ unsigned char colb[NR];
  __shared__ unsigned int list_fill;
  // per warp: union pairs (h << 16) | t waiting for a dense round
  constexpr int PC = 64;
  __shared__ uint32_t pairs[NW][PC];
  __shared__ unsigned short rbase[NR + 1];  // first run of every tile row
  __shared__ uint32_t rootm[NR];            // root runs of every tile row
  __shared__ unsigned long long red_epl[NW];
  __shared__ int red_first[NW], red_last[NW];
  __shared__ unsigned int red_prov[NW];
  __shared__ unsigned int local_err;
  __shared__ unsigned int edge_fill;

  // In a loop over tiles the thread index passes through an empty asm, so
  // that what is derived from it is worked out again for every tile: the
  // block would otherwise keep all of it live across the whole loop and
  // spill.  (A single tile keeps the plain form, which issues fewer
  // instructions.)
  int tid_in = threadIdx.x;
  if constexpr (LOOP) asm volatile("" : "+r"(tid_in));
  const int tid = tid_in, lane = tid & 31, warp = tid >> 5;
  const uint32_t utile = (uint32_t)tile;  // tile ids and node ids fit 32 bits
  const uint32_t node0 = utile * (uint32_t)kTV;
  const uint32_t lt = (1u << lane) - 1u;
  const int llim = limit_of(p.budget, kLocalLimit);

  auto rb_of = [&](int ri) -> int { return (ri / TY + HZ) * BY + (ri % TY) + 1; };
  // box row of halo row h: the whole first plane in 3D, then the two y faces
  // of every tile plane
  auto halo_rb = [&](int h) -> int {
    const int q = h - HZ * BY;
    return q < 0 ? h : (HZ + (q >> 1)) * BY + ((q & 1) ? BY - 1 : 0);
  };
  auto at = [&](int rb, int x) -> T { return box[rb * W + PADX + x]; };
  // relation of a foreground voxel with value a and a neighbour b
  auto R = [&](T a, T b) -> bool {
    if (MODE == MODE_MULTI) return a == b;
    return b != T(0);
  };
  // box-row offset of neighbour row k
  auto row_off = [&](int k) -> int {
    int dy, dz, dxs;
    row_nb<CONN>(k, dy, dz, dxs);
    return dy + BY * dz;
  };

  // ---- phase 0: the box arrives while the node bases are set up
  if (warp == 0) {
    const TileGeo gg = tile_geo(p, tile);
    if (lane == 0) {
      sgeo = gg;
      local_err = 0;
      edge_fill = 0;
      list_fill = 0;
      if (use_tma) {
        mbar_init(&tbar, 1);
        fence_mbar_init();
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&tbar, (uint32_t)(NRB * W * sizeof(T)));
        tma_load_3d(box, tmap, &tbar, (int)(gg.tx * kTX - PADX), (int)((int64_t)gg.ty * TY - 1),
                    (int)((int64_t)gg.tz * TZ - HZ));
      }
    }
  }
  if (!use_tma) {
    const TileGeo g = tile_geo(p, tile);
    const int64_t x0 = (int64_t)g.tx * kTX, y0 = (int64_t)g.ty * TY, z0 = (int64_t)g.tz * TZ;
    const T* in = static_cast<const T*>(g.in);
    for (int rb = warp; rb < NRB; rb += NW) {
      const int by = rb % BY, bz = rb / BY;
      const int64_t y = y0 - 1 + by, z = z0 - HZ + bz;
      const bool rowin = (y >= 0) && (y < g.sy) && (z >= 0) && (z < g.sz);
      const int64_t x = x0 + lane;
      T v = T(0), vl = T(0), vr = T(0);
      if (rowin) {
        const T* rowp = in + (z * g.sy + y) * g.sx;
        if (x < g.sx) v = rowp[x];
        if (lane == 0 && x0 > 0) vl = rowp[x0 - 1];
        if (lane == 0 && x0 + kTX < g.sx) vr = rowp[x0 + kTX];
      }
      box[rb * W + PADX + lane] = v;
      if (lane == 0) {
        box[rb * W + PADX - 1] = vl;
        box[rb * W + PADX + 32] = vr;
      }
    }
  }
  if (tid < NRB) {
    const int rb = tid, by = rb % BY, bz = rb / BY;
    const bool trow = by >= 1 && by <= TY && bz >= HZ;
    const int hidx = bz < HZ ? by : HZ * BY + (bz - HZ) * 2 + (by == 0 ? 0 : 1);
    nbase[rb] = (unsigned short)(trow ? ((bz - HZ) * TY + by - 1) * 32 : HNODE + hidx * 32);
    const int dy = by == 0 ? -1 : (by == BY - 1 ? 1 : 0);
    const int dz = bz < HZ ? -1 : 0;
    const int ly = by == 0 ? TY - 1 : (by == BY - 1 ? 0 : by - 1);
    const int lz = bz < HZ ? TZ - 1 : bz - HZ;
    rloc[rb] = (unsigned char)(ly + TY * lz);
    rown[rb] = (unsigned char)((dy + 1) + 3 * (dz + 1));
    // which tile holds a box row: its y and z offsets from this tile
    auto owner = [&](int r) -> int {
      const int b = r % BY, c = r / BY;
      return (b == 0 ? 0 : (b == BY - 1 ? 2 : 1)) + 3 * (c < HZ ? 0 : 1);
    };
    const int own = (dy + 1) + 3 * (dz + 1);
    int prev = 255;
    if (by > 0 && owner(rb - 1) == own) prev = rb - 1;
    else if (bz > 0 && owner(rb - BY) == own) prev = rb - BY;
    rprev[rb] = (unsigned char)prev;
  }
  if (tid < 2 * NRB) par[CNODE + tid] = (PT)(CNODE + tid);
  if (use_tma) {
    __syncthreads();  // the barrier is initialised before anyone polls it
    if (!mbar_wait_bounded(&tbar, 0)) {
      local_err = 3;
      mbar_wait_bounded(&tbar, 0);  // let a late copy land before the CTA moves on
    }
  }
  __syncthreads();
  const TileGeo g = sgeo;
  const int64_t x0 = (int64_t)g.tx * kTX, y0 = (int64_t)g.ty * TY, z0 = (int64_t)g.tz * TZ;
  (void)x0;

  // ---- phase A: run masks of every box row; run heads become nodes; the
  // provisional-label estimate (cc3d/cc3d.hpp:287-315) on the tile rows
  unsigned long long epl_acc = 0;
  int frb = NRB, lrb = -1;  // first / last box rows with estimate transitions
  auto masks = [&](int rb, uint32_t& F, uint32_t& E) {
    const T v = at(rb, lane), vl = at(rb, lane - 1);
    const bool fg = v != T(0);
    // a voxel whose left neighbour (the real one, also across the x seam)
    // does not relate to it
    const bool diff = (MODE == MODE_MULTI) ? (v != vl) : (vl == T(0));
    F = __ballot_sync(FULL, fg);
    E = __ballot_sync(FULL, fg && diff);
    const uint32_t S = E | (F & 1u);  // runs are cut at the tile's x seam
    fmask[rb] = F;
    smask[rb] = S;
    return S;
  };
#pragma unroll 2
  for (int j = 0; j < RPW; ++j) {
    const int ri = warp_row<TY>(warp, j), rb = rb_of(ri);
    uint32_t F, E;
    const uint32_t S = masks(rb, F, E);
    if ((S >> lane) & 1u) par[ri * 32 + lane] = (PT)(ri * 32 + lane);
    rootm[ri] = 0u;
    // relations with the link row (dx = 0) and, for 18 and 6, the row behind
    const T v = at(rb, lane);
    const bool fg = (F >> lane) & 1u;
    mmask[ri] = __ballot_sync(FULL, fg && R(v, at(rb + LOFF, lane)));
    if constexpr (CONN == 18 || CONN == 6) m2mask[ri] = __ballot_sync(FULL, fg && R(v, at(rb - 1, lane)));
    if constexpr (CONN == 6 || CONN == 4) colb[ri] = (unsigned char)((F & 1u) && R(at(rb, 0), at(rb, -1)));
    if (MODE == MODE_MULTI && E) {
      epl_acc += __popc(E);
      frb = rb < frb ? rb : frb;
      lrb = rb > lrb ? rb : lrb;
    }
  }
  for (int h = warp; h < NHR; h += NW) {
    const int rb = halo_rb(h);
    uint32_t F, E;
    const uint32_t S = masks(rb, F, E);
    if ((S >> lane) & 1u) par[HNODE + h * 32 + lane] = (PT)(HNODE + h * 32 + lane);
  }
  __syncthreads();

  // ---- phase B1: row-level relations, one lane per tile row (warps 0 and
  // 1), on the row masks.  The first pair of every run with its link row
  // becomes a direct parent link (to the link row's run's parent at that
  // moment: a smaller node, so roots stay the smallest node of their tree);
  // where the link row is a halo row, each halo run's first pair links the
  // halo run under the tile run instead.  The other row-level pairs and the
  // needy voxels go to the tile's list, whose unions run in phase B2 (no
  // union runs before every direct link is in place).
  if (warp < 2) {
    const int ri = warp * 32 + lane, rb = rb_of(ri), rl = rb + LOFF;
    const uint32_t F = fmask[rb], Sc = smask[rb], Sl = smask[rl], M = mmask[ri];
    const uint32_t P = M & (Sc | Sl | ~(M << 1));
    uint32_t NEED = 0, K1 = 0, K4 = 0, K2 = 0;
    if constexpr (CONN == 26 || CONN == 8) {
      // a needy voxel that continues a run whose next voxel relates to its
      // primary neighbour needs nothing: it only has dx = +1 relations of its
      // own, and each of them is that next voxel's dx = 0 relation, implied
      NEED = F & ~M & ~(~Sc & (M >> 1) & ~(Sc >> 1) & 0x7FFFFFFFu);
    } else if constexpr (CONN == 18) {
      NEED = F & ~(M & m2mask[ri]);
    } else {
      // 6: every starting pair of runs with the row behind; 6 and 4: x = 0
      // with the column x0 - 1
      if constexpr (CONN == 6) {
        const uint32_t M0 = m2mask[ri];
        K1 = M0 & (Sc | smask[rb - 1] | ~(M0 << 1));
      }
      K4 = colb[ri] ? 1u : 0u;
    }
    // walk the pair starts in x order: a run's (halo run's) first pair is the
    // first pair start seen under its head
    uint32_t rest = P;
    int last = -1;
    while (rest) {
      const int x = __ffs(rest) - 1;
      rest &= rest - 1u;
      if (ri >= LROW0) {
        const int hx = head_of(Sc, x);
        if (hx != last) {
          last = hx;
          const uint32_t tl = (uint32_t)((ri - LSTEP) * 32 + head_of(Sl, x));
          par[ri * 32 + hx] = ((const volatile PT*)par)[tl];
        } else {
          K2 |= 1u << x;
        }
      } else {
        const int hl = head_of(Sl, x);
        if (hl != last) {
          last = hl;
          par[nbase[rl] + hl] = (PT)(ri * 32 + head_of(Sc, x));
        } else {
          K2 |= 1u << x;
        }
      }
    }
    // this row's list entries, placed after the earlier lanes' of the warp
    const uint32_t U = NEED | K1 | K2 | K4;
    const unsigned cnt = __popc(U);
    unsigned incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned y = __shfl_up_sync(FULL, incl, o);
      if (lane >= o) incl += y;
    }
    unsigned base = 0;
    if (lane == 31) base = atomicAdd(&list_fill, incl);
    base = __shfl_sync(FULL, base, 31) + incl - cnt;
    unsigned short* tl_ = &ulist[0][0];
    uint32_t u = U;
    while (u) {
      const int x = __ffs(u) - 1;
      u &= u - 1u;
      const unsigned km = ((K1 >> x) & 1u) | (((K2 >> x) & 1u) << 1) | (((K4 >> x) & 1u) << 2);
      tl_[base++] = (unsigned short)((((NEED >> x) & 1u) << 14) | (km << 11) | ((unsigned)ri << 5) | (unsigned)x);
    }
  } else if (warp == 2) {
    // exclusive prefix of the run counts over the tile rows (two per lane)
    const uint32_t a0 = __popc(smask[rb_of(2 * lane)]), a1 = __popc(smask[rb_of(2 * lane + 1)]);
    uint32_t sa = a0 + a1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t ya = __shfl_up_sync(FULL, sa, o);
      if (lane >= o) sa += ya;
    }
    rbase[2 * lane] = (unsigned short)(sa - a0 - a1);
    rbase[2 * lane + 1] = (unsigned short)(sa - a1);
    if (lane == 31) rbase[NR] = (unsigned short)sa;
  }
  __syncthreads();

  // ---- phase B2: the tile's list, 32 entries per warp and round
  const int un = (int)list_fill;
  const unsigned short* tlist = &ulist[0][0];
  unsigned short* ul = ulist[warp];
  // the warp's list, one entry per lane: each lane tests its voxel's
  // relations one after the other (a needy voxel's own relation tests; the
  // column x0 - 1 of its row; the row-level pair with the row behind (6); the
  // row-level pair with the link row), and after each relation the lanes
  // that hold it append their pair to the warp's pair buffer in one step;
  // the buffer's unions run in dense rounds of one union per lane.
  int err = 0;
  int pc = 0;  // warp-uniform pair fill
  uint32_t* pw = pairs[warp];
  for (int r0 = warp * 32; r0 < un; r0 += NW * 32) {
    const int i = r0 + lane;
    unsigned e = 0;
    int x = 0, rb = 0;
    uint32_t h = 0;
    if (i < un) {
      e = tlist[i];
      x = (int)(e & 31u);
      rb = rb_of((int)((e >> 5) & 63u));
      h = (uint32_t)(((e >> 5) & 63u) * 32u + head_of(smask[rb], x));
    }
    // append pair (h, t) for every lane with `has`
    auto emit = [&](bool has, uint32_t t) {
      const uint32_t act = __ballot_sync(FULL, has);
      if (!act) return;
      if (pc + __popc(act) > PC) {
        err |= list_unions<PT>(pw, pc, par, llim, lane);
        pc = 0;
      }
      if (has) pw[pc + __popc(act & lt)] = (h << 16) | t;
      pc += __popc(act);
    };
    // the target node of column xn of box row rbk
    auto node_at = [&](int rbk, int xn) -> uint32_t {
      if (xn < 0) return (uint32_t)(CNODE + rbk);
      if (xn > 31) return (uint32_t)(CNODE + NRB + rbk);
      return (uint32_t)(nbase[rbk] + head_of(smask[rbk], xn));
    };
    if constexpr (PRIMARY) {
      // a needy voxel tests its remaining relations itself
      const bool needy = (e >> 14) & 1u;
      const T v = at(rb, x);
      const bool head = (smask[rb] >> x) & 1u;
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        const unsigned c = (unsigned)((NRel::code >> (4 * j)) & 15u);
        const int k = (int)(c & 3u), dx = (int)(c >> 2) - 1;
        const int rbk = rb + row_off(k);
        bool rel = needy && (head || !((NRel::left >> j) & 1u)) && R(v, at(rbk, x + dx));
        if (dx != 0) {
          // the neighbour run of column x + dx already joined through the
          // dx = 0 relation when it also covers column x
          const int xn = x + dx;
          const uint32_t Sk = smask[rbk];
          const bool same = (xn >= 0 && xn <= 31) && !((Sk >> (dx > 0 ? xn : x)) & 1u);
          rel = rel && !(same && R(v, at(rbk, x)));
        }
        emit(rel, node_at(rbk, x + dx));
      }
      // the column x0 - 1 of the voxel's own row
      emit(needy && x == 0 && R(v, at(rb, -1)), (uint32_t)(CNODE + rb));
    } else {
      emit(((e >> 11) & 4u) != 0u, (uint32_t)(CNODE + rb));
      if constexpr (CONN == 6) emit(((e >> 11) & 1u) != 0u, node_at(rb - 1, x));
    }
    emit(((e >> 11) & 2u) != 0u, node_at(rb + LOFF, x));
  }
  err |= list_unions<PT>(pw, pc, par, llim, lane);
  if (err) local_err = 1;
  __syncthreads();

  // ---- phase C: roots, run records, keys, bitmap.  A component is named by
  // its root run (the smallest node of its tree, its first run in raster
  // order): the run's index in the tile's run order.  Each warp gathers the
  // run heads of its rows (bottom of its columns first) into its list and
  // resolves them 32 at a time, one per lane.  Halo heads and the halo
  // columns are only pointed at their roots, for the edges below.
  const uint32_t C = rbase[NR];
  auto rid_of = [&](unsigned r) -> unsigned {
    return rbase[r >> 5] + __popc(smask[rb_of((int)(r >> 5))] & ((1u << (r & 31u)) - 1u));
  };
  const uint32_t wpr = (uint32_t)g.wpr, tx = (uint32_t)g.tx;
  const uint32_t sy32 = (uint32_t)g.sy;
  // bitmap word of the tile's row (ly, lz) = bw0 + (lz * sy + ly) * wpr
  const uint32_t bw0 = (uint32_t)g.word0 + ((uint32_t)z0 * sy32 + (uint32_t)y0) * wpr + tx;
  int nh = 0;  // warp-uniform head count
  for (int j = 0; j < RPW; ++j) {
    const int ri = warp_row<TY>(warp, j);
    const uint32_t S = smask[rb_of(ri)];
    if ((S >> lane) & 1u) ul[nh + __popc(S & lt)] = (unsigned short)(ri * 32 + lane);
    nh += __popc(S);
  }
  __syncwarp();
  for (int h0 = 0; h0 < nh; h0 += 32) {
    if (h0 + lane < nh) {
      const uint32_t n = ul[h0 + lane];
      const int ri = (int)(n >> 5), x = (int)(n & 31u);
      uint32_t r = lfind_ro<PT>(par, n, llim);
      if (par[r] != r) {
        // the find ran out of budget: the run becomes a root of its own (the
        // call reports the error), so every component it names has a key
        local_err = 1;
        r = n;
      }
      par[n] = (PT)r;
      const unsigned c = rid_of(r);
      const unsigned own = rbase[ri] + __popc(smask[rb_of(ri)] & ((1u << x) - 1u));
      p.rcomp[node0 + own] = (uint16_t)c;
      if (r == n) {
        const uint32_t bw = bw0 + ((uint32_t)(ri / TY) * sy32 + (uint32_t)(ri % TY)) * wpr;
        p.E[node0 + c] = ((unsigned long long)(bw * 32u + (uint32_t)x) << 32) | (node0 + c);
        atomicOr(&rootm[ri], 1u << x);
      }
    }
  }
  for (int h = warp; h < NHR; h += NW) {
    const uint32_t S = smask[halo_rb(h)];
    if ((S >> lane) & 1u) {
      const uint32_t n = (uint32_t)(HNODE + h * 32 + lane);
      uint32_t r = lfind_ro<PT>(par, n, llim);
      if (par[r] != r) {
        local_err = 1;
        r = n;
      }
      par[n] = (PT)r;
    }
  }
  if (tid < 2 * NRB) {
    const uint32_t n = (uint32_t)(CNODE + tid);
    uint32_t r = lfind_ro<PT>(par, n, llim);
    if (par[r] != r) {
      local_err = 1;
      r = n;
    }
    par[n] = (PT)r;
  }
  __syncwarp();
  // the row records of the warp's rows, one lane per row
  if (lane < RPW) {
    const int ri = warp_row<TY>(warp, lane), rb = rb_of(ri);
    const uint32_t rr = utile * (uint32_t)kRowsPerTile + (uint32_t)ri;
    p.rmask[rr] = make_uint2(fmask[rb], smask[rb]);
    p.rrow[rr] = rbase[ri];
    const int ly = ri % TY, lz = ri / TY;
    if (y0 + ly < g.sy && z0 + lz < g.sz)
      p.bitmap[bw0 + ((uint32_t)lz * sy32 + (uint32_t)ly) * wpr] = rootm[ri];
  }
  __syncthreads();

  // ---- phase D: one edge per halo run / halo-column voxel joined to a tile
  // component, except where the same-owner voxel just before it (one row back
  // in y, else in z) relates to it and joined the same component: both lie
  // in one component of their own tile, so that edge would repeat
  uint2* edges = p.edges + (size_t)utile * p.edge_slots;
  // the tile holding box row rb (rows outside the volume hold no foreground,
  // so their tile id is unused)
  const uint32_t ntx = (uint32_t)g.ntx, ntxy = ntx * (uint32_t)g.nty;
  auto rtile = [&](int rb) -> uint32_t {
    const int own = rown[rb];
    return utile + (uint32_t)(own % 3 - 1) * ntx + (uint32_t)(own / 3 - 1) * ntxy;
  };
  constexpr int NCC = (2 * NRB + 31) / 32;  // 32-voxel chunks of the two halo columns
  constexpr int NHW = (NHR + 31) / 32;      // warps that take the halo rows, one lane per row
  static_assert(NHW + 1 <= NW, "warps left for the halo columns");
  if (warp < NHW) {
    // halo row h: its run heads in x order
    const int h = warp * 32 + lane;
    if (h < NHR) {
      const int rb = halo_rb(h), rp = rprev[rb];
      uint32_t heads = smask[rb];
      const uint32_t Sp = rp != 255 ? smask[rp] : 0u;
      while (heads) {
        const int x = __ffs(heads) - 1;
        heads &= heads - 1u;
        const uint32_t r = par[HNODE + h * 32 + x];
        if (r >= kTV) continue;
        if (rp != 255) {
          const T a = at(rb, x), b = at(rp, x);
          if (b != T(0) && (MODE == MODE_MULTI ? a == b : true) && par[nbase[rp] + head_of(Sp, x)] == r) continue;
        }
        const unsigned slot = atomicAdd(&edge_fill, 1u);
        if (slot < p.edge_slots)
          edges[slot] = make_uint2(node0 + rid_of(r), (rtile(rb) * (uint32_t)kRowsPerTile + rloc[rb]) * 32u + x);
      }
    }
  } else {
    for (int it = warp - NHW; it < NCC; it += NW - NHW) {
      bool has = false;
      uint2 e = make_uint2(0u, 0u);
      const int c = it * 32 + lane;
      if (c < 2 * NRB) {
        const int side = c >= NRB ? 1 : 0, rb = c - side * NRB, xi = side ? 32 : -1;
        if (at(rb, xi) != T(0)) {
          const uint32_t r = par[CNODE + c];
          if (r < kTV) {
            has = true;
            const int rp = rprev[rb];
            if (rp != 255) {
              const T a = at(rb, xi), b = at(rp, xi);
              if (b != T(0) && (MODE == MODE_MULTI ? a == b : true) && par[CNODE + side * NRB + rp] == r)
                has = false;
            }
            // the column voxel lies in the tile left (x0 - 1) or right
            // (x0 + 32) of the row's tile, at x 31 or 0 of that tile
            if (has)
              e = make_uint2(node0 + rid_of(r),
                             ((rtile(rb) + (side ? 1u : 0xFFFFFFFFu)) * (uint32_t)kRowsPerTile + rloc[rb]) * 32u +
                                 (side ? 0u : 31u));
          }
        }
      }
      const unsigned m = __ballot_sync(FULL, has);
      if (!m) continue;
      unsigned base = 0;
      if (lane == 0) base = atomicAdd(&edge_fill, (unsigned)__popc(m));
      base = __shfl_sync(FULL, base, 0);
      if (has) {
        const unsigned slot = base + __popc(m & lt);
        if (slot < p.edge_slots) edges[slot] = e;
      }
    }
  }

  // ---- provisional labels the reference's binary labellers would open: a
  // foreground voxel none of whose backward neighbours is foreground
  unsigned int prov = 0;
  if (MODE == MODE_BINARY && p.want_prov) {
    auto colfg = [&](int rb, int xi) -> uint32_t { return at(rb, xi) != T(0) ? 1u : 0u; };
    for (int ri = warp; ri < NR; ri += NW) {
      const int rb = rb_of(ri);
      const uint32_t F = fmask[rb];
      uint32_t Lk = (F << 1) | colfg(rb, -1);
#pragma unroll
      for (int k = 0; k < NRN; ++k) {
        int dy, dz, dxs;
        row_nb<CONN>(k, dy, dz, dxs);
        const int rbp = rb + dy + BY * dz;
        const uint32_t Fp = fmask[rbp];
        if (dxs & 2) Lk |= Fp;
        if (dxs & 1) Lk |= (Fp << 1) | colfg(rbp, -1);
        if (dxs & 4) Lk |= (Fp >> 1) | (colfg(rbp, 32) << 31);
      }
      if (lane == 0) prov += __popc(F & ~Lk);
    }
  }

  // ---- per-tile results (reduced by the numbering scan, no same-address
  // atomics here)
  if (lane == 0) {
    red_epl[warp] = epl_acc;
    red_first[warp] = frb;
    red_last[warp] = lrb;
    red_prov[warp] = prov;
  }
  __syncthreads();
  if (tid == 0) {
    unsigned long long e = 0, pv = 0;
    int f = NRB, l = -1;
    for (int w = 0; w < NW; ++w) {
      e += red_epl[w];
      pv += red_prov[w];
      // box-row order is raster order for rows inside the volume
      f = red_first[w] < f ? red_first[w] : f;
      l = red_last[w] > l ? red_last[w] : l;
    }
    auto grow = [&](int rb) -> long long {
      return (long long)(y0 - 1 + rb % BY) + (long long)g.sy * (long long)(z0 - HZ + rb / BY);
    };
    const uint32_t nedges = edge_fill;
    TileInfo ti;
    ti.C = C;
    ti.nedges = nedges < p.edge_slots ? nedges : p.edge_slots;
    ti.epl = (uint32_t)e;
    ti.prov = (uint32_t)pv;
    ti.first_row = f < NRB ? grow(f) : 0x7FFFFFFFFFFFFFFFLL;
    ti.last_row = l >= 0 ? grow(l) : -1;
    p.tinfo[tile] = ti;
    if (nedges > p.edge_slots) atomicOr(&p.ctr->err, ERR_EDGE_OVERFLOW);
    if (local_err)
      atomicOr(&p.ctr->err, local_err == 3 ? ERR_WAIT : (local_err == 2 ? ERR_INDEX : ERR_LOCAL_BUDGET));
  }
}

// TMA: the box arrives by one TMA copy (else by plain loads); two kernels, so
// that each holds only its own way of loading and keeps its registers for the
// phases after it.  Seven blocks per SM for one- and two-byte voxels, whose
// boxes leave the shared memory for it (32 registers a thread then, against
// 40 at six: measured faster all the same); six for wider voxels.
template <typename T, int CONN, int TY, int TZ, int MODE, bool TMA>
__global__ void __launch_bounds__(kThreads, sizeof(T) <= 2 ? 7 : 6)
k_tile_list(LabelArgs p, const __grid_constant__ CUtensorMap tmap) {
  tile_list_tile<T, CONN, TY, TZ, MODE>(p, &tmap, TMA ? 1 : 0, p.tile_base + blockIdx.x);
}

}  // namespace cc3dgpu
