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
//     the primary neighbour is one union per pair of runs (this row's run,
//     the neighbour row's run) where the pair starts.
//   * The other ("needy") voxels are few (background faces and isolated
//     values): their x positions go to a per-warp list and each is then
//     handled by one lane, which tests its remaining backward neighbours
//     itself.  A voxel that continues a run (equal to its left neighbour)
//     skips the neighbours that its left neighbour already sees, and a
//     diagonal relation is skipped where the same neighbour run is already
//     joined through the dx = 0 relation.
//   * 6- and 4-connected labellers have no primary neighbour: every row pair
//     contributes one union per starting pair of runs, found by ballots.
//
// Row-level work is therefore a handful of warp instructions per 32-voxel row
// (two ballots for the run masks, one for the primary relation, two list
// appends); unions run from the lists with one lane per entry.
//
// Phases: 0 box by TMA (or plain loads), node table; 1 run masks of every box
// row, union-find nodes of the run heads, the provisional-label estimate
// (cc3d/cc3d.hpp:287-315); 2 primary relations and lists, then the unions of
// the warp's own lists; 3 roots (path-compressed), per-row counts, prefix;
// 4 records, keys, bitmap, halo edges, the binary labellers' provisional
// count, per-tile results.
#pragma once

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

template <typename T, int CONN, int TY, int TZ, int MODE>
__global__ void __launch_bounds__(kThreads, 4)
k_tile_list(LabelArgs p, const __grid_constant__ CUtensorMap tmap, int use_tma) {
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
  constexpr int NRN = RowNb<CONN>::n;
  constexpr int W = BoxRow<T>::W, PADX = BoxRow<T>::PADX;
  // a primary neighbour row decides most voxels (box-row offset of the
  // row-level pair: below in 3D, behind in 2D)
  constexpr bool PRIMARY = (CONN == 26 || CONN == 18 || CONN == 8);
  constexpr int POFF = (CONN == 8) ? -1 : -BY;
  constexpr int QN = (NR / NW) * 32;     // list capacity: every voxel of the warp's rows
  using NRel = NeedRels<CONN>;
  static_assert(kTX * NR == kTV, "tile must hold 2048 voxels");
  static_assert(NR == kRowsPerTile, "64 rows per tile");
  static_assert(NR % NW == 0, "rows per warp");
  static_assert(NODES < 16384, "node ids must fit 14 bits");
  static_assert(W <= 256 && BY <= 256 && BZ <= 256, "TMA box dimensions");
  static_assert(NRB < 256, "box rows fit a byte");

  __shared__ __align__(128) T box[NRB * W];
  __shared__ __align__(8) uint64_t tbar;
  __shared__ uint32_t smask[NRB], fmask[NRB];
  __shared__ __align__(16) unsigned short par[NODES];
  __shared__ unsigned short nbase[NRB];  // node id of a box row's voxel 0
  __shared__ unsigned short plist[NW][QN], nlist[NW][QN];
  __shared__ uint32_t rootm[NR];
  __shared__ unsigned short rbase[NR + 1], cbase[NR + 1];
  __shared__ unsigned long long red_epl[NW];
  __shared__ long long red_first[NW], red_last[NW];
  __shared__ unsigned int red_prov[NW];
  __shared__ unsigned int local_err;
  __shared__ unsigned int edge_fill;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t tile = p.tile_base + blockIdx.x;
  const TileGeo g = tile_geo(p, tile);
  const int tx = g.tx;
  const int64_t x0 = (int64_t)tx * kTX, y0 = (int64_t)g.ty * TY, z0 = (int64_t)g.tz * TZ;
  const uint32_t lt = (1u << lane) - 1u;

  auto is_tile_row = [&](int rb) -> bool {
    const int by = rb % BY, bz = rb / BY;
    return by >= 1 && by <= TY && bz >= HZ;
  };
  auto tile_row_of = [&](int rb) -> int { return (rb % BY - 1) + TY * (rb / BY - HZ); };
  auto box_row_of = [&](int ri) -> int { return (ri / TY + HZ) * BY + (ri % TY) + 1; };
  // index of a halo box row among the halo rows (the whole first plane in
  // 3D, then the two y faces of every tile plane)
  auto halo_row_of = [&](int rb) -> int {
    const int by = rb % BY, bz = rb / BY;
    return bz < HZ ? by : HZ * BY + (bz - HZ) * 2 + (by == 0 ? 0 : 1);
  };
  // which neighbouring tile holds a halo row
  auto row_owner = [&](int rb) -> int {
    const int by = rb % BY, bz = rb / BY;
    return (by == 0 ? 0 : (by == BY - 1 ? 2 : 1)) + 3 * (bz < HZ ? 0 : 1);
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

  // ---- phase 0: the box arrives while the node table is set up
  if (tid == 0) {
    local_err = 0;
    edge_fill = 0;
    if (use_tma) {
      mbar_init(&tbar, 1);
      fence_mbar_init();
      fence_proxy_async_smem();
      mbar_arrive_expect_tx(&tbar, (uint32_t)(NRB * W * sizeof(T)));
      tma_load_3d(box, &tmap, &tbar, (int)(x0 - PADX), (int)(y0 - 1), (int)(z0 - HZ));
    }
  }
  if (!use_tma) {
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
  for (int rb = tid; rb < NRB; rb += kThreads) {
    nbase[rb] = (unsigned short)(is_tile_row(rb) ? tile_row_of(rb) * 32 : HNODE + halo_row_of(rb) * 32);
    par[CNODE + rb] = (unsigned short)(CNODE + rb);
    par[CNODE + NRB + rb] = (unsigned short)(CNODE + NRB + rb);
  }
  if (use_tma) {
    __syncthreads();  // the barrier is initialised before anyone polls it
    if (!mbar_wait_bounded(&tbar, 0)) {
      local_err = 3;
      mbar_wait_bounded(&tbar, 0);  // let a late copy land before the CTA moves on
    }
  }
  __syncthreads();

  // ---- phase 1: run masks of every box row; the run heads become nodes
  unsigned long long epl_acc = 0;
  int frb = NRB, lrb = -1;  // first / last box rows with estimate transitions
  for (int rb = warp; rb < NRB; rb += NW) {
    const T v = at(rb, lane), vl = at(rb, lane - 1);
    const bool fg = v != T(0);
    // a voxel whose left neighbour (the real one, also across the x seam)
    // does not relate to it
    const bool diff = (MODE == MODE_MULTI) ? (v != vl) : (vl == T(0));
    const uint32_t F = __ballot_sync(FULL, fg);
    const uint32_t E = __ballot_sync(FULL, fg && diff);
    const uint32_t S = E | (F & 1u);  // runs are cut at the tile's x seam
    if (lane == 0) {
      fmask[rb] = F;
      smask[rb] = S;
    }
    if ((S >> lane) & 1u) {
      const unsigned short n = (unsigned short)(nbase[rb] + lane);
      par[n] = n;
    }
    if (MODE == MODE_MULTI && p.want_epl && E && is_tile_row(rb)) {
      epl_acc += __popc(E);
      frb = rb < frb ? rb : frb;
      lrb = rb > lrb ? rb : lrb;
    }
  }
  __syncthreads();

  // ---- phase 2: row-level relations and the warp's lists, then its unions
  int pn = 0, nn = 0;  // warp-uniform list fills
  unsigned short* pl = plist[warp];
  unsigned short* nl = nlist[warp];
  for (int ri = warp; ri < NR; ri += NW) {
    const int rb = box_row_of(ri);
    const T v = at(rb, lane);
    const uint32_t F = fmask[rb], Sc = smask[rb];
    const bool fg = (F >> lane) & 1u;
    uint32_t P, NEED = 0, km = 1u;
    if constexpr (PRIMARY) {
      const uint32_t M = __ballot_sync(FULL, fg && R(v, at(rb + POFF, lane)));
      P = M & (Sc | smask[rb + POFF] | ~(M << 1));
      uint32_t cov = M;
      if constexpr (CONN == 18) cov &= __ballot_sync(FULL, fg && R(v, at(rb - 1, lane)));
      NEED = F & ~cov;
    } else {
      // behind (and below for 6): one union per starting pair of runs; lane
      // 0 also relates to the column x0 - 1 of its own row
      const uint32_t M0 = __ballot_sync(FULL, fg && R(v, at(rb - 1, lane)));
      const uint32_t P0 = M0 & (Sc | smask[rb - 1] | ~(M0 << 1));
      uint32_t P1 = 0;
      if constexpr (CONN == 6) {
        const uint32_t M1 = __ballot_sync(FULL, fg && R(v, at(rb - BY, lane)));
        P1 = M1 & (Sc | smask[rb - BY] | ~(M1 << 1));
      }
      const bool lc = lane == 0 && fg && R(v, at(rb, -1));
      km = ((P0 >> lane) & 1u) | (((P1 >> lane) & 1u) << 1) | (lc ? 4u : 0u);
      P = __ballot_sync(FULL, km != 0u);
    }
    if ((P >> lane) & 1u) pl[pn + __popc(P & lt)] = (unsigned short)((km << 11) | (ri << 5) | lane);
    pn += __popc(P);
    if (PRIMARY) {
      if ((NEED >> lane) & 1u) nl[nn + __popc(NEED & lt)] = (unsigned short)((ri << 5) | lane);
      nn += __popc(NEED);
    }
  }
  __syncwarp();
  int err = 0;
  // pairs found at row level: lane i takes entry i of each round
  for (int r0 = 0; r0 < pn; r0 += 32) {
    const int i = r0 + lane;
    if (i < pn) {
      const unsigned e = pl[i];
      const int x = (int)(e & 31u), ri = (int)((e >> 5) & 63u);
      const int rb = box_row_of(ri);
      const unsigned short h = (unsigned short)(ri * 32 + head_of(smask[rb], x));
      unsigned m = PRIMARY ? 1u : (e >> 11);
      while (m) {
        const int j = __ffs(m) - 1;
        m &= m - 1u;
        unsigned short t;
        if (j == 2) {
          t = (unsigned short)(CNODE + rb);
        } else {
          const int rbk = rb + (PRIMARY ? POFF : (j == 0 ? -1 : -BY));
          t = (unsigned short)(nbase[rbk] + head_of(smask[rbk], x));
        }
        if (!sunite(par, h, t)) err = 1;
      }
    }
  }
  // needy voxels: one lane each tests the voxel's remaining relations
  if constexpr (PRIMARY) {
    for (int r0 = 0; r0 < nn; r0 += 32) {
      const int i = r0 + lane;
      if (i < nn) {
        const unsigned e = nl[i];
        const int x = (int)(e & 31u), ri = (int)(e >> 5);
        const int rb = box_row_of(ri);
        const T v = at(rb, x);
        const uint32_t Sc = smask[rb];
        const bool head = (Sc >> x) & 1u;
        const unsigned short h = (unsigned short)(ri * 32 + head_of(Sc, x));
        uint32_t m = 0;
#pragma unroll
        for (int j = 0; j < NRel::n; ++j) {
          const unsigned c = (unsigned)((NRel::code >> (4 * j)) & 15u);
          const int k = (int)(c & 3u), dx = (int)(c >> 2) - 1;
          if (((NRel::left >> j) & 1u) && !head) continue;
          const int rbk = rb + row_off(k);
          bool rel = R(v, at(rbk, x + dx));
          if (dx != 0 && rel) {
            // the neighbour run of column x + dx already joined through the
            // dx = 0 relation when it also covers column x
            const int xn = x + dx;
            if (xn >= 0 && xn <= 31) {
              const uint32_t Sk = smask[rbk];
              const bool same = dx > 0 ? !((Sk >> xn) & 1u) : !((Sk >> x) & 1u);
              if (same && R(v, at(rbk, x))) rel = false;
            }
          }
          if (rel) m |= 1u << j;
        }
        // the column x0 - 1 of the voxel's own row
        if (x == 0 && R(v, at(rb, -1))) m |= 1u << NRel::n;
        while (m) {
          const int j = __ffs(m) - 1;
          m &= m - 1u;
          unsigned short t;
          if (j == NRel::n) {
            t = (unsigned short)(CNODE + rb);
          } else {
            const unsigned c = (unsigned)((NRel::code >> (4 * j)) & 15u);
            const int k = (int)(c & 3u), xn = x + (int)(c >> 2) - 1;
            const int rbk = rb + (k == 0 ? row_off(0) : (k == 1 ? row_off(1) : (k == 2 ? row_off(2) : row_off(3))));
            if (xn < 0) t = (unsigned short)(CNODE + rbk);
            else if (xn > 31) t = (unsigned short)(CNODE + NRB + rbk);
            else t = (unsigned short)(nbase[rbk] + head_of(smask[rbk], xn));
          }
          if (!sunite(par, h, t)) err = 1;
        }
      }
    }
  }
  if (err) local_err = 1;
  __syncthreads();

  // ---- phase 3: roots (every head points at its root afterwards), counts
  for (int rb = warp; rb < NRB; rb += NW) {
    const uint32_t S = smask[rb];
    bool root = false;
    if ((S >> lane) & 1u) {
      const unsigned short n = (unsigned short)(nbase[rb] + lane);
      const unsigned short r = sfind_ro(par, n);
      par[n] = r;
      root = (r == n);
    }
    if (is_tile_row(rb)) {
      const uint32_t rm = __ballot_sync(FULL, root);
      if (lane == 0) {
        const int ri = tile_row_of(rb);
        rootm[ri] = rm;
        rbase[ri + 1] = (unsigned short)__popc(S);
        cbase[ri + 1] = (unsigned short)__popc(rm);
      }
    }
  }
  for (int c = tid; c < 2 * NRB; c += kThreads) {
    const unsigned short n = (unsigned short)(CNODE + c);
    par[n] = sfind_ro(par, n);
  }
  __syncthreads();
  if (warp == 0) {
    // exclusive prefix over the 64 rows (two per lane)
    const uint32_t a0 = rbase[2 * lane + 1], a1 = rbase[2 * lane + 2];
    const uint32_t c0 = cbase[2 * lane + 1], c1 = cbase[2 * lane + 2];
    uint32_t sa = a0 + a1, sc = c0 + c1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t ya = __shfl_up_sync(FULL, sa, o), yc = __shfl_up_sync(FULL, sc, o);
      if (lane >= o) { sa += ya; sc += yc; }
    }
    rbase[2 * lane + 1] = (unsigned short)(sa - a1);
    rbase[2 * lane + 2] = (unsigned short)sa;
    cbase[2 * lane + 1] = (unsigned short)(sc - c1);
    cbase[2 * lane + 2] = (unsigned short)sc;
    if (lane == 0) { rbase[0] = 0; cbase[0] = 0; }
  }
  __syncthreads();
  const uint32_t C = cbase[NR];
  // dense component id of a root (a tile run head) in tile raster order
  auto cid_of = [&](unsigned r) -> unsigned {
    return cbase[r >> 5] + __popc(rootm[r >> 5] & ((1u << (r & 31u)) - 1u));
  };

  // ---- phase 4: run records, keys, bitmap
  const uint32_t node0 = (uint32_t)(tile * kTV);
  for (int ri = warp; ri < NR; ri += NW) {
    const int rb = box_row_of(ri);
    const uint32_t S = smask[rb], F = fmask[rb], rm = rootm[ri];
    const int64_t y = y0 + ri % TY, z = z0 + ri / TY;
    if (lane == 0) {
      p.rmask[tile * kRowsPerTile + ri] = make_uint2(F, S);
      p.rrow[tile * kRowsPerTile + ri] = rbase[ri];
      if (y < g.sy && z < g.sz) p.bitmap[g.word0 + (z * g.sy + y) * g.wpr + tx] = rm;
    }
    if ((S >> lane) & 1u) {
      const unsigned r = par[ri * 32 + lane];
      const unsigned c = cid_of(r);
      p.rcomp[tile * kTV + rbase[ri] + __popc(S & lt)] = (uint16_t)c;
      if ((rm >> lane) & 1u) {
        const uint32_t key = (uint32_t)(g.word0 * 32 + (z * g.sy + y) * g.key_row + x0 + lane);
        p.E[node0 + c] = ((unsigned long long)key << 32) | (node0 + c);
      }
    }
  }

  // ---- one edge per halo run / halo-column voxel joined to a tile component,
  // except where the same-owner voxel just before it (one row back in y, else
  // in z) relates to it and joined the same component: both lie in one
  // component of their own tile, so that edge would repeat
  auto prev_row = [&](int rb) -> int {
    const int by = rb % BY, bz = rb / BY, own = row_owner(rb);
    if (by > 0 && row_owner(rb - 1) == own) return rb - 1;
    if (bz > 0 && row_owner(rb - BY) == own) return rb - BY;
    return -1;
  };
  auto halo_edge = [&](int h, uint2& e) -> bool {
    int rb, lx, xi;
    int64_t gx;
    unsigned short node;
    if (h < NRB * 32) {
      rb = h >> 5;
      lx = h & 31;
      if (!((smask[rb] >> lx) & 1u)) return false;  // run heads stand for their runs
      xi = lx;
      gx = x0 + lx;
      node = (unsigned short)(nbase[rb] + lx);
    } else {
      const int c = h - NRB * 32;
      rb = c % NRB;
      xi = (c < NRB) ? -1 : 32;
      gx = x0 + xi;
      lx = (int)(gx & 31);
      node = (unsigned short)(CNODE + c);
      if (at(rb, xi) == T(0)) return false;
    }
    const unsigned short r = par[node];
    if (r >= kTV) return false;
    const int rp = prev_row(rb);
    if (rp >= 0) {
      const T a = at(rb, xi), b = at(rp, xi);
      if (b != T(0) && (MODE == MODE_MULTI ? a == b : true)) {
        unsigned short np;
        if (xi < 0) np = (unsigned short)(CNODE + rp);
        else if (xi > 31) np = (unsigned short)(CNODE + NRB + rp);
        else np = (unsigned short)(nbase[rp] + head_of(smask[rp], xi));
        if (par[np] == r) return false;
      }
    }
    const int by = rb % BY, bz = rb / BY;
    const int64_t gy = y0 - 1 + by, gz = z0 - HZ + bz;
    const int64_t otile = g.tile0 + (gx >> 5) + (int64_t)g.ntx * ((gy / TY) + (int64_t)g.nty * (gz / TZ));
    const uint32_t local = (uint32_t)(lx + kTX * ((gy % TY) + TY * (gz % TZ)));
    e = make_uint2(node0 + cid_of(r), (uint32_t)(otile * kTV + local));
    return true;
  };
  uint2* edges = p.edges + tile * p.edge_slots;
  constexpr int NCC = (2 * NRB + 31) / 32;  // 32-voxel chunks of the two halo columns
  for (int it = warp; it < NRB + NCC; it += NW) {
    int h;
    if (it < NRB) {
      if (is_tile_row(it)) continue;
      h = it * 32 + lane;
    } else {
      const int c = (it - NRB) * 32 + lane;
      h = c < 2 * NRB ? NRB * 32 + c : -1;
    }
    uint2 e;
    const bool has = h >= 0 && halo_edge(h, e);
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

  // ---- provisional labels the reference's binary labellers would open: a
  // foreground voxel none of whose backward neighbours is foreground
  unsigned int prov = 0;
  if (MODE == MODE_BINARY && p.want_prov) {
    auto colfg = [&](int rb, int xi) -> uint32_t { return at(rb, xi) != T(0) ? 1u : 0u; };
    for (int ri = warp; ri < NR; ri += NW) {
      const int rb = box_row_of(ri);
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
    auto grow = [&](int rb) -> long long { return (y0 - 1 + rb % BY) + g.sy * (z0 - HZ + rb / BY); };
    red_epl[warp] = epl_acc;
    red_first[warp] = frb < NRB ? grow(frb) : 0x7FFFFFFFFFFFFFFFLL;
    red_last[warp] = lrb >= 0 ? grow(lrb) : -1;
    red_prov[warp] = prov;
  }
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
    const uint32_t nedges = edge_fill;
    TileInfo ti;
    ti.C = C;
    ti.nedges = nedges < p.edge_slots ? nedges : p.edge_slots;
    ti.epl = (uint32_t)e;
    ti.prov = (uint32_t)pv;
    ti.first_row = f;
    ti.last_row = l;
    p.tinfo[tile] = ti;
    if (nedges > p.edge_slots) atomicOr(&p.ctr->err, ERR_EDGE_OVERFLOW);
    if (local_err)
      atomicOr(&p.ctr->err, local_err == 3 ? ERR_WAIT : (local_err == 2 ? ERR_INDEX : ERR_LOCAL_BUDGET));
  }
}

}  // namespace cc3dgpu
