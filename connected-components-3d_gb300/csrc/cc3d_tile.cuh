// cc3d_tile.cuh -- the tile pass (K1) of the labelling pipeline.
//
// One CTA labels one 32 x TY x TZ tile (2048 voxels) with a one-voxel backward
// halo, all in shared memory:
//
//   phase 0  the box (the tile, its halo rows and the two halo columns, padded
//            in x to 16-byte boundaries) arrives by one TMA copy while the
//            threads initialise the union-find; out-of-volume voxels are
//            zero-filled by the copy engine, which is exactly the background
//            the labelling needs at volume faces.  (Inputs whose rows are not
//            16-byte multiples, and batches, load the box with plain loads.)
//            Foreground and run-start masks come from warp ballots, and the
//            provisional-label estimate (cc3d/cc3d.hpp:287-315) is counted on
//            the tile's own rows.
//   phase 2  every tile row is related to its backward rows.  Equalities at
//            dx = 0 are one ballot per neighbour row; a union is queued only
//            where a pair of overlapping runs starts.  Where the connectivity
//            allows it, a voxel equal to its "primary" neighbour (the voxel
//            below for 26, below and behind for 18, the row behind for 8)
//            needs nothing else: each of its other backward neighbours that it
//            relates to is also a neighbour of the primary one, related to it,
//            and earlier in raster order, so that pair is joined by induction
//            over the raster order.  Only the remaining voxels test their
//            dx = +-1 neighbours (the halo columns at the x faces), again as
//            ballots, and a union is queued only for a pair of runs that
//            neither the voxel before it nor the dx = 0 relation already
//            joins.  Unions go through small per-warp queues and are run in
//            dense rounds (lane i takes entry i), every lane at one call site.
//   phase 3  roots -> component ids (the index of the root run in the
//            tile's run order), run-length records, component keys, the
//            numbering bitmap, one edge per
//            halo run (or halo-column voxel) joined to a tile component --
//            except where the same-owner voxel just before it (dx = 0, one row
//            back in y, else in z) has the same value and joined the same
//            component: both lie in one component of their own tile, so that
//            edge would repeat -- and the binary labellers' provisional count.
#pragma once

#include "cc3d_tma.cuh"

namespace cc3dgpu {

// Box geometry of a 32 x TY x TZ tile with its backward halo: rows rb =
// bz * BY + by; tile rows have by in [1, TY] and bz >= HZ.  Union-find nodes:
// tile run heads ri * 32 + x, halo run heads kTV + rb * 32 + x, halo columns
// CNODE + rb (x0 - 1) and CNODE + NRB + rb (x0 + 32).
template <int CONN, int TY, int TZ>
struct TileBox {
  static constexpr bool D3 = (CONN == 26 || CONN == 18 || CONN == 6);
  static constexpr int HZ = D3 ? 1 : 0;
  static constexpr int BY = TY + 2, BZ = TZ + HZ;
  static constexpr int NRB = BY * BZ;
  static constexpr int HNODE = kTV;
  static constexpr int CNODE = kTV + NRB * 32;
  static constexpr int NODES = CNODE + 2 * NRB;
  __device__ static __forceinline__ bool is_tile_row(int rb) {
    const int by = rb % BY, bz = rb / BY;
    return by >= 1 && by <= TY && bz >= HZ;
  }
};


// Staged box of one tile: box rows of W values, the tile's column x0 + x at
// index PADX + x (x in [-1, 32]); the row starts 16-byte aligned in memory
// and in the volume, as a TMA copy needs.
template <typename T>
struct BoxRow {
  static constexpr int PADX = 16 / (int)sizeof(T);
  static constexpr int W = 32 + 2 * PADX;
};

// Runs the queued unions q[from, to) of one warp, lane i taking entry from + i
// of each round of 32.  Entries are (a << 16) | b.  Not inlined, so that every
// queue site shares one copy of the union-find code.  Returns 2 for a node id
// out of range, 1 if a union ran out of budget, else 0.
static __device__ __noinline__ int run_unions(const uint32_t* q, int from, int to, unsigned short* par, int nodes,
                                       int lane, int lim) {
  __syncwarp();
  int err = 0;
  for (int r = from; r < to; r += 32) {
    const int i = r + lane;
    if (i < to) {
      const uint32_t e = q[i];
      const int a = (int)(e >> 16), b = (int)(e & 0xFFFFu);
      if (a >= nodes || b >= nodes) err = 2;
      else if (!sunite(par, (unsigned short)a, (unsigned short)b, lim)) err = 1;
    }
  }
  __syncwarp();
  return err;
}

template <typename T, int CONN, int TY, int TZ, int MODE, bool BLOCK8>
__global__ void __launch_bounds__(kThreads, 4)
k_tile_runs(LabelArgs p, const __grid_constant__ CUtensorMap tmap, int use_tma) {
  using S = typename Stored<T, MODE>::type;
  constexpr bool D3 = (CONN == 26 || CONN == 18 || CONN == 6);
  constexpr int HZ = D3 ? 1 : 0;
  constexpr int BY = TY + 2, BZ = TZ + HZ;
  constexpr int NRB = BY * BZ;                 // box rows (tile + halo)
  constexpr int NR = TY * TZ;                  // tile rows
  constexpr int HNODE = kTV;                   // halo-row heads: HNODE + rb*32 + lane
  constexpr int CNODE = kTV + NRB * 32;        // columns: CNODE + rb (x0-1), + NRB + rb (x0+32)
  constexpr int NODES = CNODE + 2 * NRB;
  constexpr int NW = kThreads / 32;
  constexpr int NRN = RowNb<CONN>::n;
  constexpr int W = BoxRow<T>::W, PADX = BoxRow<T>::PADX;
  // neighbour rows (indices into row_nb) whose dx = 0 match makes a voxel's
  // other backward relations implied; -1 = none
  // (a connectivity graph implies nothing: every relation is its own bit)
  constexpr bool GRAPH = MODE == MODE_GRAPH;
  constexpr int PRI0 = GRAPH ? -1 : ((CONN == 26) ? 2 : (CONN == 18 ? 2 : (CONN == 8 ? 0 : -1)));
  constexpr int PRI1 = (!GRAPH && CONN == 18) ? 0 : -1;
  constexpr bool HAS_DX = (CONN == 26 || CONN == 18 || CONN == 8);
  constexpr bool CONT = (MODE == MODE_CONT || MODE == MODE_CONT8Q);
  constexpr bool EQUAL_JOINS = (MODE == MODE_MULTI || CONT);  // equal neighbours always join
  static_assert(MODE != MODE_CONT8Q || CONN == 8, "the 2D 8-connected decision tree");
  constexpr int QN = 128;                      // per-warp queue capacity
  static_assert(kTX * NR == kTV, "tile must hold 2048 voxels");
  static_assert(NR == kRowsPerTile, "64 rows per tile");
  static_assert(NODES < 16384, "node ids must fit 14 bits");
  static_assert(!HAS_DX || MODE != MODE_BINARY4, "the binary 4-connected relation has no diagonals");
  static_assert(W <= 256 && BY <= 256 && BZ <= 256, "TMA box dimensions");

  __shared__ __align__(128) T box[NRB * W];
  __shared__ __align__(8) uint64_t tbar;
  __shared__ uint32_t smask[NRB], fmask[NRB];
  __shared__ __align__(16) unsigned short par[NODES];
  // component ids (phase 3) share their storage with the phase-2 union queues
  __shared__ __align__(16) unsigned short cid[kTV];
  __shared__ uint32_t rootm[NR];
  __shared__ unsigned short rbase[NR + 1];
  __shared__ uint32_t minblk[BLOCK8 ? kTV : 1];
  static_assert(NW * QN * sizeof(uint32_t) <= sizeof(unsigned short) * kTV,
                "queues must fit in the component-id storage");
  uint32_t (*uq)[QN] = reinterpret_cast<uint32_t (*)[QN]>(cid);  // (a << 16) | b
  __shared__ unsigned long long red_epl[NW];
  __shared__ long long red_first[NW], red_last[NW];
  __shared__ unsigned int red_prov[NW];
  __shared__ unsigned int local_err;
  __shared__ unsigned int edge_fill;
  __shared__ unsigned short nbase[NRB];  // node id of a box row's voxel 0
  __shared__ unsigned char vcol[GRAPH ? NRB : 1];  // graphs: bit 0 / 1: column x0-1 / x0+32 in the volume
  __shared__ unsigned char brow[NR];     // box row of each tile row

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t tile = p.tile_base + blockIdx.x;
  const TileGeo g = tile_geo(p, tile);
  const int tx = g.tx;
  const int64_t x0 = (int64_t)tx * kTX, y0 = (int64_t)g.ty * TY, z0 = (int64_t)g.tz * TZ;
  const uint32_t lt = (1u << lane) - 1u;
  const int llim = limit_of(p.budget, kLocalLimit);

  auto is_tile_row = [&](int rb) -> bool {
    const int by = rb % BY, bz = rb / BY;
    return by >= 1 && by <= TY && bz >= HZ;
  };
  auto tile_row_of = [&](int rb) -> int { return (rb % BY - 1) + TY * (rb / BY - HZ); };
  auto box_row_of = [&](int ri) -> int { return (ri / TY + HZ) * BY + (ri % TY) + 1; };
  // owner code of a halo row / column: which neighbouring tile holds it
  auto row_owner = [&](int rb) -> int {
    const int by = rb % BY, bz = rb / BY;
    return (by == 0 ? 0 : (by == BY - 1 ? 2 : 1)) + 3 * (bz < HZ ? 0 : 1);
  };
  // the box row of tile row ri, from the table filled in phase 0
  auto box_row = [&](int ri) -> int { return brow[ri]; };
  static_assert(NRB < 256, "box rows fit a byte");
  // stored value of box row rb at tile column x (x in [-1, 32])
  auto sv = [&](int rb, int x) -> S { return to_stored<S, T, MODE>(box[rb * W + PADX + x]); };
  // relation of a foreground voxel a with a neighbour b
  const T delta = from_bits<T>(p.delta_bits);
  auto R = [&](S a, S b) -> bool {
    if constexpr (CONT) return is_fg(b) && cmatch<T>((T)a, (T)b, delta);
    else return rel<MODE>(a, b);
  };
  // continuous 2D 8-connected: a pixel that takes the label above it and
  // nothing else (cc3d/cc3d_continuous.hpp:296-309)
  const T gmin = MODE == MODE_CONT8Q ? from_bits<T>(p.span[0]) : T(0);
  const T gmax = MODE == MODE_CONT8Q ? from_bits<T>(p.span[1]) : T(0);
  auto up_only = [&](S a, S up) -> bool {
    return is_fg(a) && is_fg(up) && (a == up || span_shortcut<T>((T)a, (T)up, gmin, gmax, delta));
  };
  // graphs: the bit of voxel value a for direction (dx, dy, dz); a single
  // plane reads uint8 graphs in the 2D layout and uint32 graphs in the 3D one
  // (the two 8-connected labellers, cc3d/cc3d_graphs.hpp:831-1017)
  auto gbit = [&](S a, int dx, int dy, int dz) -> bool {
    const int b = (D3 || sizeof(T) == 4) ? dir_bit3(dx, dy, dz) : dir_bit2(dx, dy);
    return ((uint32_t)a >> b) & 1u;
  };

  // ---- phase 0: the box arrives (TMA, or plain loads) while the forest is set up
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
  for (int rb = tid; rb < NRB; rb += kThreads)
    nbase[rb] = (unsigned short)(is_tile_row(rb) ? tile_row_of(rb) * 32 : HNODE + rb * 32);
  for (int ri = tid; ri < NR; ri += kThreads) brow[ri] = (unsigned char)box_row_of(ri);
  {
    // identity forest, four nodes per store
    uint2* p4 = reinterpret_cast<uint2*>(par);
    for (int n = tid; n < NODES / 4; n += kThreads) {
      const uint32_t b = 4u * n;
      p4[n] = make_uint2(b | ((b + 1) << 16), (b + 2) | ((b + 3) << 16));
    }
    for (int n = (NODES / 4) * 4 + tid; n < NODES; n += kThreads) par[n] = (unsigned short)n;
  }
  if (use_tma) {
    __syncthreads();  // the barrier is initialised before anyone polls it
    if (!mbar_wait_bounded(&tbar, 0)) {
      local_err = 3;
      mbar_wait_bounded(&tbar, 0);  // let a late copy land before the CTA moves on
    }
  }
  __syncthreads();

  // ---- masks of every box row, epl on the tile's own rows
  unsigned long long epl_acc = 0;
  // first and last box rows with foreground runs (box-row order is raster
  // order for rows inside the volume); -1 / NRB when none
  int frb = NRB, lrb = -1;
  for (int rb = warp; rb < NRB; rb += NW) {
    const int by = rb % BY, bz = rb / BY;
    const T v = box[rb * W + PADX + lane];
    const bool trow = by >= 1 && by <= TY && bz >= HZ;
    if (p.want_epl && trow) {
      T prev = __shfl_up_sync(FULL, v, 1);
      if (lane == 0) prev = box[rb * W + PADX - 1];
      const unsigned m = __ballot_sync(FULL, (v != prev) && (v != T(0)));
      if (m) {
        epl_acc += __popc(m);
        frb = rb < frb ? rb : frb;
        lrb = rb > lrb ? rb : lrb;
      }
    }
    if (GRAPH) {
      // every voxel inside the volume is a node; it links to its left
      // neighbour where its own -x bit is set
      const int64_t gy = y0 - 1 + by, gz = z0 - HZ + bz;
      const bool rowin = gy >= 0 && gy < g.sy && gz >= 0 && gz < g.sz;
      const bool in = rowin && x0 + lane < g.sx;
      const uint32_t F = __ballot_sync(FULL, in);
      const uint32_t L = __ballot_sync(FULL, in && lane > 0 && gbit((S)v, -1, 0, 0));
      if (lane == 0) {
        fmask[rb] = F;
        smask[rb] = F & ~L;
        vcol[GRAPH ? rb : 0] = (unsigned char)((rowin && x0 > 0 ? 1 : 0) | (rowin && x0 + kTX < g.sx ? 2 : 0));
      }
    } else if (MODE != MODE_BINARY4) {
      const S s = to_stored<S, T, MODE>(v);
      const S sl = (S)__shfl_up_sync(FULL, s, 1);
      const bool fg = is_fg(s);
      bool link = lane > 0 && fg && is_fg(sl);
      if (MODE == MODE_MULTI) link = link && (s == sl);
      if (CONT) link = link && R(s, sl);
      if (MODE == MODE_CONT8Q) {
        // a pixel that takes the label above it has no left link; halo rows
        // keep single-pixel runs (their links depend on rows outside the box)
        link = link && trow && !up_only(s, sv(rb - 1 < 0 ? 0 : rb - 1, lane));
      }
      const uint32_t F = __ballot_sync(FULL, fg);
      const uint32_t L = __ballot_sync(FULL, link);
      if (lane == 0) {
        fmask[rb] = F;
        smask[rb] = F & ~L;
      }
    }
  }

  if (MODE == MODE_BINARY4) {
    // horizontal links of the reference's binary 4-connected labeller: the
    // first image row links equal values only; later rows drop the link when
    // both pixels have foreground directly above (they are joined through the
    // row above).  Halo rows keep single-voxel runs.
    for (int rb = warp; rb < NRB; rb += NW) {
      const S s = sv(rb, lane);
      const S sl = (S)__shfl_up_sync(FULL, s, 1);
      const bool fg = is_fg(s);
      bool link = lane > 0 && fg && is_fg(sl);
      const int64_t gy = y0 - 1 + rb % BY;
      if (!is_tile_row(rb)) {
        link = false;
      } else if (gy == 0) {
        link = link && (s == sl);
      } else {
        const S a = sv(rb - 1, lane);
        const S al = (S)__shfl_up_sync(FULL, a, 1);
        link = link && !(is_fg(a) && is_fg(al));
      }
      const uint32_t F = __ballot_sync(FULL, fg);
      const uint32_t L = __ballot_sync(FULL, link);
      if (lane == 0) {
        fmask[rb] = F;
        smask[rb] = F & ~L;
      }
    }
  }
  __syncthreads();

  // ---- phase 2: unions through per-warp queues
  int uqn = 0;  // warp-uniform queue fill, below 32 between neighbour rows
  uint32_t* myq = uq[warp];
  // lanes in m append (a, b)
  auto push = [&](uint32_t m, unsigned a, unsigned b) {
    if ((m >> lane) & 1u) myq[uqn + __popc(m & lt)] = (a << 16) | (b & 0xFFFFu);
    uqn += __popc(m);
  };
  // run whole rounds of 32 from the top of the queue
  auto flush = [&](int keep) {
    if (uqn > keep) {
      const int e = run_unions(myq, keep, uqn, par, NODES, lane, llim);
      if (e) local_err = e;
      uqn = keep;
    }
  };

  // tile rows.  A union is queued for the first voxel of each pair of runs
  // (this row's run, the neighbour row's run) that a relation joins; pairs
  // that a voxel's primary neighbour implies are left out.
  for (int ri = warp; ri < NR; ri += NW) {
    const int rb = box_row(ri);
    const S s = sv(rb, lane);
    const uint32_t F = fmask[rb], Sr = smask[rb];
    const bool fg = (F >> lane) & 1u;
    const unsigned nR = (unsigned)(ri * 32 + head_of(Sr, lane));
    uint32_t M0[NRN], Sp[NRN];
    S Wn[NRN];
#pragma unroll
    for (int k = 0; k < NRN; ++k) {
      int dy, dz, dxs;
      row_nb<CONN>(k, dy, dz, dxs);
      const int rbp = rb + dy + BY * dz;
      Wn[k] = sv(rbp, lane);
      Sp[k] = smask[rbp];
      if (GRAPH) M0[k] = __ballot_sync(FULL, fg && gbit(s, 0, dy, dz) && ((fmask[rbp] >> lane) & 1u));
      else M0[k] = __ballot_sync(FULL, fg && R(s, Wn[k]));
    }
    uint32_t SC = 0;
    if (MODE == MODE_CONT8Q) {
      // the decision tree's first two branches: the pixel above and nothing else
      SC = __ballot_sync(FULL, up_only(s, Wn[0]));
      M0[0] |= SC;
    } else if (CONT) {
      // an exactly equal primary neighbour stands in for the voxel (equality
      // carries every match over to it)
      if (PRI0 >= 0) SC = __ballot_sync(FULL, fg && s == Wn[PRI0 < 0 ? 0 : PRI0]);
      if (PRI1 >= 0) SC &= __ballot_sync(FULL, fg && s == Wn[PRI1 < 0 ? 0 : PRI1]);
    } else {
      if (PRI0 >= 0) SC = M0[PRI0 < 0 ? 0 : PRI0];
      if (PRI1 >= 0) SC &= M0[PRI1 < 0 ? 0 : PRI1];
    }
    const uint32_t NEED = (PRI0 >= 0) ? (F & ~SC) : F;
    if (HAS_DX && (NEED & 1u)) {
      // the same row's left neighbour across the x seam
      const bool r0 = lane == 0 && (GRAPH ? (gbit(s, -1, 0, 0) && (vcol[GRAPH ? rb : 0] & 1u)) : R(s, sv(rb, -1)));
      push(__ballot_sync(FULL, r0), nR, (unsigned)(CNODE + rb));
    }
    if (!HAS_DX && (F & 1u)) {
      // same-row neighbour across the x seam
      const S s0 = (S)__shfl_sync(FULL, s, 0);
      const S c0 = sv(rb, -1);
      bool r0;
      if (GRAPH) r0 = gbit(s0, -1, 0, 0) && (vcol[GRAPH ? rb : 0] & 1u);
      else if (MODE == MODE_MULTI) r0 = (s0 == c0);
      else if (CONT) r0 = R(s0, c0);
      else if (MODE == MODE_BINARY4) {
        const int64_t gy = y0 - 1 + rb % BY;
        r0 = is_fg(c0) && (gy == 0 ? (s0 == c0) : !(is_fg(sv(rb - 1, 0)) && is_fg(sv(rb - 1, -1))));
      } else r0 = is_fg(c0);
      if (r0) push(1u, (unsigned)(ri * 32), (unsigned)(CNODE + rb));
    }
#pragma unroll
    for (int k = 0; k < NRN; ++k) {
      int dy, dz, dxs;
      row_nb<CONN>(k, dy, dz, dxs);
      const int rbp = rb + dy + BY * dz;
      const bool primary = (k == PRI0) || (k == PRI1);
      uint32_t U = M0[k] & (Sr | Sp[k] | ~(M0[k] << 1));
      if (!primary) U &= NEED;
      const unsigned nb = nbase[rbp];
      if (U) push(U, nR, nb + head_of(Sp[k], lane));
      if (HAS_DX && NEED) {
        // Voxels not covered by their primary neighbour relate to the dx = -1
        // and dx = +1 voxels of the neighbour rows.  The pair (this run, the
        // neighbour's run) of voxel x repeats that of x - 1 when neither run
        // starts between them, and it is the dx = 0 pair when the neighbour's
        // run goes on from x to x -+ 1: both are left out.
        const uint32_t candL = NEED & ~(M0[k] & ~Sp[k] & ~1u);
        const uint32_t candR = NEED & ~(M0[k] & ~(Sp[k] >> 1) & 0x7FFFFFFFu);
        // voxels whose diagonal relations stand for joins: all of them where
        // the primary neighbour implies them, only NEED where a voxel that
        // takes the label above drops its other relations (continuous 2D 8)
        const bool mine = MODE != MODE_CONT8Q || ((NEED >> lane) & 1u);
        if ((dxs & 1) && candL) {
          S wl = (S)__shfl_up_sync(FULL, Wn[k], 1);
          if (lane == 0) wl = sv(rbp, -1);
          const bool rl = GRAPH ? (gbit(s, -1, dy, dz) && (lane > 0 ? ((fmask[rbp] >> (lane - 1)) & 1u)
                                                                     : (vcol[GRAPH ? rbp : 0] & 1u)))
                                : R(s, wl);
          const uint32_t ML = __ballot_sync(FULL, fg && mine && rl);
          const uint32_t UL = ML & candL & (Sr | (Sp[k] << 1) | ~(ML << 1));
          if (UL) push(UL, nR, lane == 0 ? (unsigned)(CNODE + rbp) : nb + head_of(Sp[k], lane - 1));
        }
        if ((dxs & 4) && candR) {
          S wr = (S)__shfl_down_sync(FULL, Wn[k], 1);
          if (lane == 31) wr = sv(rbp, 32);
          const bool rr = GRAPH ? (gbit(s, 1, dy, dz) && (lane < 31 ? ((fmask[rbp] >> (lane + 1)) & 1u)
                                                                     : ((vcol[GRAPH ? rbp : 0] >> 1) & 1u)))
                                : R(s, wr);
          const uint32_t MR = __ballot_sync(FULL, fg && mine && rr);
          const uint32_t UR = MR & candR & (Sr | (Sp[k] >> 1) | 0x80000000u | ~(MR << 1));
          if (UR)
            push(UR, nR, lane == 31 ? (unsigned)(CNODE + NRB + rbp) : nb + head_of(Sp[k], lane + 1));
        }
      }
      // at most 1 + 3 * 32 entries were added since the queue held < 32
      if (uqn >= 32) flush(uqn & 31);
    }
  }
  flush(0);
  __syncthreads();

  // ---- phase 3a: component roots per tile row, run counts per row
  for (int ri = warp; ri < NR; ri += NW) {
    const int rb = box_row(ri);
    const uint32_t Sr = smask[rb];
    bool root = false;
    if ((Sr >> lane) & 1u) {
      const unsigned short n = (unsigned short)(ri * 32 + lane);
      unsigned short r = sfind_ro(par, n, llim);
      if (par[r] != r) {
        // the find ran out of budget: the run becomes a root of its own (the
        // call reports the error), so every component id stays defined
        local_err = 1;
        r = n;
      }
      par[n] = r;
      root = (r == n);
    }
    const uint32_t rm = __ballot_sync(FULL, root);
    if (lane == 0) {
      rootm[ri] = rm;
      rbase[ri + 1] = (unsigned short)__popc(Sr);
    }
  }
  __syncthreads();
  if (warp == 0) {
    // exclusive prefix of the run counts over the 64 rows (two per lane)
    const uint32_t a0 = rbase[2 * lane + 1], a1 = rbase[2 * lane + 2];
    uint32_t sa = a0 + a1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t ya = __shfl_up_sync(FULL, sa, o);
      if (lane >= o) sa += ya;
    }
    rbase[2 * lane + 1] = (unsigned short)(sa - a1);
    rbase[2 * lane + 2] = (unsigned short)sa;
    if (lane == 0) rbase[0] = 0;
  }
  __syncthreads();
  // a component is named by the index of its root run in the tile's run
  // order; ids run up to the tile's run count C
  for (int ri = warp; ri < NR; ri += NW) {
    const uint32_t rm = rootm[ri];
    if ((rm >> lane) & 1u)
      cid[ri * 32 + lane] = (unsigned short)(rbase[ri] + __popc(smask[box_row(ri)] & lt));
  }
  const uint32_t C = rbase[NR];
  if (BLOCK8)
    for (uint32_t c = tid; c < C; c += kThreads) minblk[c] = 0xFFFFFFFFu;
  __syncthreads();

  // ---- phase 3b: run records, keys, bitmap
  const uint32_t node0 = (uint32_t)(tile * kTV);
  for (int ri = warp; ri < NR; ri += NW) {
    const int rb = box_row(ri);
    const uint32_t Sr = smask[rb], F = fmask[rb];
    const int ly = ri % TY, lz = ri / TY;
    const int64_t y = y0 + ly, z = z0 + lz;
    if (lane == 0) {
      p.rmask[tile * kRowsPerTile + ri] = make_uint2(F, Sr);
      p.rrow[tile * kRowsPerTile + ri] = rbase[ri];
    }
    if ((Sr >> lane) & 1u) {
      const unsigned short r = par[ri * 32 + lane];
      const unsigned short c = cid[r];
      p.rcomp[tile * kTV + rbase[ri] + __popc(Sr & lt)] = c;
      if (BLOCK8) atomicMin(&minblk[c], (uint32_t)((y >> 1) * g.key_row + ((x0 + lane) >> 1)));
    }
    if (!BLOCK8) {
      const uint32_t rm = rootm[ri];
      if ((rm >> lane) & 1u) {
        const uint32_t key = (uint32_t)(g.word0 * 32 + (z * g.sy + y) * g.key_row + x0 + lane);
        const uint32_t c = cid[ri * 32 + lane];
        p.E[node0 + c] = ((unsigned long long)key << 32) | (node0 + c);
      }
      if (lane == 0 && y < g.sy && z < g.sz) p.bitmap[g.word0 + (z * g.sy + y) * g.wpr + tx] = rm;
    }
  }
  if (BLOCK8) {
    __syncthreads();
    for (uint32_t c = tid; c < C; c += kThreads) {
      const uint32_t key = minblk[c];
      if (key == 0xFFFFFFFFu) continue;  // not a root run
      atomicOr(p.bitmap + (key >> 5), 1u << (key & 31));
      p.E[node0 + c] = ((unsigned long long)key << 32) | (node0 + c);
    }
  }

  // ---- phase 3c: one edge per halo run / halo-column voxel joined to a tile
  // component, into the tile's own edge slots
  // the same-owner box row just before rb (one back in y, else in z), or -1
  auto prev_row = [&](int rb) -> int {
    const int by = rb % BY, bz = rb / BY, own = row_owner(rb);
    if (by > 0 && row_owner(rb - 1) == own) return rb - 1;
    if (bz > 0 && row_owner(rb - BY) == own) return rb - BY;
    return -1;
  };
  auto halo_edge = [&](int h, uint2& e) -> bool {
    int rb, lx, xi;  // xi: the voxel's tile column (-1 and 32 for the halo columns)
    int64_t gx;
    unsigned short node;
    if (h < NRB * 32) {
      rb = h >> 5;
      lx = h & 31;
      if (is_tile_row(rb)) return false;
      if (!((smask[rb] >> lx) & 1u)) return false;  // run heads stand for their runs
      xi = lx;
      gx = x0 + lx;
      node = (unsigned short)(HNODE + h);
    } else {
      const int c = h - NRB * 32;
      rb = c % NRB;
      xi = (c < NRB) ? -1 : 32;
      gx = x0 + xi;
      lx = (int)(gx & 31);
      node = (unsigned short)(CNODE + c);
      if (GRAPH ? !((vcol[GRAPH ? rb : 0] >> (c < NRB ? 0 : 1)) & 1u) : !is_fg(sv(rb, xi))) return false;
    }
    unsigned short r = sfind_ro(par, node, llim);
    if (r >= kTV) return false;
    // a find that ran out of budget ends on a tile run head, whose parent is
    // its root after phase 3a (the error is already recorded)
    if (par[r] != r) r = par[r];
    const int rp = MODE == MODE_BINARY4 ? -1 : prev_row(rb);
    if (rp >= 0) {
      const S a = sv(rb, xi), b = sv(rp, xi);
      // joined inside their own tile: equal values, or (graphs) the later
      // voxel's bit towards the earlier one, with both in the volume
      bool joined;
      if (GRAPH) {
        const bool rp_in = xi < 0 ? (vcol[GRAPH ? rp : 0] & 1u) : (xi > 31 ? ((vcol[GRAPH ? rp : 0] >> 1) & 1u)
                                                                           : ((fmask[rp] >> xi) & 1u));
        joined = rp_in && (rp == rb - 1 ? gbit(a, 0, -1, 0) : gbit(a, 0, 0, -1));
      } else {
        joined = is_fg(b) && (EQUAL_JOINS ? a == b : true);
      }
      if (joined) {
        unsigned short np;
        if (xi < 0) np = (unsigned short)(CNODE + rp);
        else if (xi > 31) np = (unsigned short)(CNODE + NRB + rp);
        else np = (unsigned short)(HNODE + rp * 32 + head_of(smask[rp], xi));
        if (sfind_ro(par, np, llim) == r) return false;
      }
    }
    const int by = rb % BY, bz = rb / BY;
    const int64_t gy = y0 - 1 + by, gz = z0 - HZ + bz;
    const int64_t otile = g.tile0 + (gx >> 5) + (int64_t)g.ntx * ((gy / TY) + (int64_t)g.nty * (gz / TZ));
    const uint32_t local = (uint32_t)(lx + kTX * ((gy % TY) + TY * (gz % TZ)));
    e = make_uint2(node0 + cid[r], (uint32_t)(otile * kTV + local));
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

  // ---- provisional labels the reference's binary labeller would open
  unsigned int prov = 0;
  if (p.want_prov) {
    auto colfg = [&](int rb, int xi) -> uint32_t { return is_fg(sv(rb, xi)) ? 1u : 0u; };
    if (BLOCK8) {
      // 2x2 blocks Y Z / X W; C D E F in the row above, B A to the left
      for (int q = tid; q < kTV / 4; q += kThreads) {
        const int b = q & 15, ri = 2 * (q >> 4);
        const int rb = box_row(ri);
        const uint32_t Fa = fmask[rb - 1], F0 = fmask[rb], F1 = fmask[rb + 1];
        const uint32_t ca = colfg(rb - 1, -1), c0 = colfg(rb, -1);
        const uint32_t c1 = colfg(rb + 1, -1), ra = colfg(rb - 1, 32);
        const int x = 2 * b;
        const bool Y = (F0 >> x) & 1u, Z = (F0 >> (x + 1)) & 1u;
        const bool X = (F1 >> x) & 1u, W_ = (F1 >> (x + 1)) & 1u;
        if (!(Y || Z || X || W_)) continue;
        const bool Cc = x == 0 ? ca : (Fa >> (x - 1)) & 1u;
        const bool D = (Fa >> x) & 1u, Ee = (Fa >> (x + 1)) & 1u;
        const bool Fq = x + 2 == 32 ? ra : (Fa >> (x + 2)) & 1u;
        const bool B = x == 0 ? c0 : (F0 >> (x - 1)) & 1u;
        const bool A = x == 0 ? c1 : (F1 >> (x - 1)) & 1u;
        const bool linked = (Y && (Cc || D || Ee || B || A)) || (Z && (D || Ee || Fq)) || (X && (B || A));
        prov += linked ? 0u : 1u;
      }
    } else {
      for (int ri = warp; ri < NR; ri += NW) {
        const int rb = box_row(ri);
        const uint32_t F = fmask[rb];
        const S s = sv(rb, lane);
        uint32_t Lk;
        const int64_t gy = y0 + ri % TY, gz = z0 + ri / TY;
        if (MODE == MODE_BINARY4 && gy == 0 && gz == 0) {
          S sl = (S)__shfl_up_sync(FULL, s, 1);
          if (lane == 0) sl = sv(rb, -1);
          Lk = __ballot_sync(FULL, is_fg(s) && s == sl);
        } else {
          Lk = (F << 1) | colfg(rb, -1);
        }
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
  }

  // ---- reductions
  if (lane == 0) {
    // global row index y + sy * z of a box row
    auto grow = [&](int rb) -> long long { return (y0 - 1 + rb % BY) + g.sy * (z0 - HZ + rb / BY); };
    red_epl[warp] = epl_acc;
    red_first[warp] = frb < NRB ? grow(frb) : 0x7FFFFFFFFFFFFFFFLL;
    red_last[warp] = lrb >= 0 ? grow(lrb) : -1;
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
