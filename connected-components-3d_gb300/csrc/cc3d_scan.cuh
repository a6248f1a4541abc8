// cc3d_scan.cuh -- the tile pass as a label-copying raster scan.
//
// One warp labels one 32 x TY x TZ tile (2048 voxels) together with its
// one-voxel backward halo, visiting the box rows in raster order (z, then y),
// 32 voxels of a row per warp instruction:
//
//   * rows arrive through TMA (cp.async.bulk.tensor) into a three-slot ring
//     of chunks in shared memory, one chunk ahead of the scan, completion
//     tracked by mbarriers; out-of-volume reads are zero-filled by the copy
//     engine, which is exactly the background the scan needs at volume edges;
//   * a row is cut into runs with warp ballots; every run takes the smallest
//     root label among its related backward neighbours (a copy, no write to the
//     union-find) and only a run with none opens a new label.  Where a run
//     touches two different roots they are merged with an atomicCAS union --
//     the rare case, e.g. where two branches of a component meet;
//   * as in a decision tree, a voxel equal to its primary neighbour (below for
//     26, below and behind for 18, behind for 8) needs no other test: every
//     other backward neighbour it relates to also neighbours the primary one,
//     relates to it and precedes it in raster order, so that pair was joined
//     already;
//   * halo rows and the two halo columns take labels from same-owner halo
//     neighbours only, so a halo label names a group of halo voxels that are
//     connected inside their own tile; one edge per group that joined a tile
//     component leaves the tile.
//
// At the end the warp numbers the tile's components in raster order of their
// first voxel and writes the run-length records, keys, numbering bitmap and
// edges that the rest of the pipeline (cc3d_label.cuh) consumes.
#pragma once

#include "cc3d_tma.cuh"

namespace cc3dgpu {

constexpr int kScanWarps = 2;           // tiles (warps) per CTA
constexpr uint16_t kNoLabel = 0xFFFF;
constexpr uint16_t kCompFlag = 0x8000;  // par[root] = flag | component id, final pass only

template <typename T, int CONN, int TY, int TZ>
struct ScanGeom {
  static constexpr bool D3 = (CONN == 26 || CONN == 18 || CONN == 6);
  static constexpr int HZ = D3 ? 1 : 0;
  static constexpr int BY = TY + 2, BZ = TZ + HZ;
  static constexpr int NRB = BY * BZ;               // box rows
  static constexpr int CH = D3 ? BY : 8;            // rows per loaded chunk (a plane in 3D)
  static constexpr int NCH = (NRB + CH - 1) / CH;   // chunks
  static constexpr int NS = 3;                      // ring slots: previous, current, next
  static constexpr int PADX = 16 / (int)sizeof(T);  // box starts 16-byte aligned before x0
  static constexpr int W = 32 + 2 * PADX;           // elements per loaded row
  // ring slot stride: TMA writes to 128-byte aligned shared memory
  static constexpr int SLOT = (int)(((CH * W * sizeof(T) + 127) / 128 * 128) / sizeof(T));
  // label slots: 3D keeps the previous and the current plane, 2D the
  // previous and the current row
  static constexpr int LS = D3 ? 2 * BY : 2;
  static constexpr int NHL = (NRB - TY * TZ) * 32 + 2 * NRB;  // halo labels
  static constexpr int NLAB = kTV + NHL;
  static_assert(NLAB < (int)kCompFlag, "labels must leave the flag bit free");
};

template <typename T, int CONN, int TY, int TZ>
struct alignas(128) ScanSmem {
  using G = ScanGeom<T, CONN, TY, TZ>;
  T vals[G::NS][G::SLOT];
  uint64_t bar[G::NS];
  uint16_t lab[G::LS][34];    // labels of recent rows; [0] = column x0-1, [33] = column x0+32
  uint32_t fmr[G::LS];        // foreground masks of recent rows
  uint32_t colfg[G::LS];      // bit 0: column x0-1 foreground, bit 1: column x0+32
  uint16_t par[G::NLAB];      // union-find over labels
  uint16_t hpos[G::NHL];      // halo label -> rb * 34 + i of the voxel that opened it
  uint16_t runlab[kTV];       // label of every tile run, in tile raster order
  uint32_t rowF[TY * TZ], rowS[TY * TZ];
  uint16_t rowbase[TY * TZ + 1];
};

// dynamic shared memory of one CTA (+128 to align the base by hand)
template <typename T, int CONN, int TY, int TZ>
constexpr size_t scan_smem_bytes() {
  return sizeof(ScanSmem<T, CONN, TY, TZ>) * kScanWarps + 128;
}

template <typename T, int CONN, int TY, int TZ, int MODE>
__global__ void __launch_bounds__(kScanWarps * 32, 1)
k_tile_scan(LabelArgs p, const __grid_constant__ CUtensorMap tmap, int use_tma) {
  using G = ScanGeom<T, CONN, TY, TZ>;
  using SMem = ScanSmem<T, CONN, TY, TZ>;
  constexpr int BY = G::BY, HZ = G::HZ, NRB = G::NRB, CH = G::CH, NS = G::NS;
  constexpr int NR = TY * TZ;
  constexpr int NRN = RowNb<CONN>::n;
  constexpr int PRI0 = (CONN == 26) ? 2 : (CONN == 18 ? 2 : (CONN == 8 ? 0 : -1));
  constexpr int PRI1 = (CONN == 18) ? 0 : -1;
  static_assert(NR == kRowsPerTile, "64 rows per tile");

  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t mis = smem_addr(smem_raw) & 127u;
  SMem& sm = reinterpret_cast<SMem*>(smem_raw + (mis ? 128u - mis : 0u))[warp];
  const int64_t tile = p.tile_base + (int64_t)blockIdx.x * kScanWarps + warp;
  if (tile >= p.tile_end) return;  // the whole warp leaves
  const TileGeo g = tile_geo(p, tile);
  const int tx = g.tx;
  const int64_t x0 = (int64_t)tx * kTX, y0 = (int64_t)g.ty * TY, z0 = (int64_t)g.tz * TZ;
  const uint32_t lt = (1u << lane) - 1u;
  unsigned err = 0;

  // an empty tile record, for a tile that cannot be labelled
  auto give_up = [&]() {
    if (lane == 0) {
      TileInfo ti = {};
      ti.first_row = 0x7FFFFFFFFFFFFFFFLL;
      ti.last_row = -1;
      p.tinfo[tile] = ti;
      if (err) atomicOr(&p.ctr->err, err);
    }
  };
  // once one warp's copy never arrived the launch is failing: the remaining
  // tiles skip their copies, so that the launch ends quickly
  if (*(volatile unsigned*)&p.ctr->err & ERR_WAIT) {
    give_up();
    return;
  }

  auto find = [&](uint16_t n) -> uint16_t { return sfind(sm.par, n); };

  // ---- ring of chunks: chunk c holds box rows [c * CH, c * CH + CH)
  if (lane == 0 && use_tma) {
    for (int s = 0; s < NS; ++s) mbar_init(&sm.bar[s], 1);
    fence_mbar_init();
  }
  __syncwarp();
  const int chunk_y = (int)(y0 - 1), chunk_z = (int)(z0 - HZ);
  auto issue = [&](int c) {
    if (c >= G::NCH) return;
    const int slot = c % NS;
    const int cy = G::D3 ? chunk_y : chunk_y + c * CH;
    const int cz = G::D3 ? chunk_z + c : chunk_z;
    if (use_tma) {
      if (lane == 0) {
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&sm.bar[slot], (uint32_t)(CH * G::W * sizeof(T)));
        tma_load_3d(&sm.vals[slot][0], &tmap, &sm.bar[slot], (int)(x0 - G::PADX), cy, cz);
      }
    } else {
      const T* in = static_cast<const T*>(g.in);
      for (int i = lane; i < CH * G::W; i += 32) {
        const int r = i / G::W, xi = i % G::W;
        const int64_t gx = x0 - G::PADX + xi, gy = cy + r, gz = cz;
        T v = T(0);
        if (gx >= 0 && gx < g.sx && gy >= 0 && gy < g.sy && gz >= 0 && gz < g.sz)
          v = in[(gz * g.sy + gy) * g.sx + gx];
        sm.vals[slot][r * G::W + xi] = v;
      }
    }
  };
  auto wait = [&](int c) {
    if (use_tma) {
      const int slot = c % NS;
      const uint32_t parity = (uint32_t)((c / NS) & 1);
      bool ok = false;
      for (int it = 0; it < kWaitLimit && !ok; ++it) ok = mbar_try_wait(&sm.bar[slot], parity);
      if (!__all_sync(FULL, ok)) {
        err |= ERR_WAIT;
        // let the copy land (bounded) before the warp gives up on the tile
        for (int it = 0; it < kWaitLimit && !ok; ++it) ok = mbar_try_wait(&sm.bar[slot], parity);
      }
    }
    __syncwarp();
  };

  // ---- the scan
  uint32_t tl = 0, hl = kTV;  // next tile / halo label
  uint32_t rbase = 0;         // runs of the tile rows seen so far
  unsigned long long epl_acc = 0;
  long long frow = 0x7FFFFFFFFFFFFFFFLL, lrow = -1;
  uint32_t prov = 0;
  // Box row (by, bz) = rb: its values by column i (0 = x0 - 1, 1..32 = the
  // tile's columns, 33 = x0 + 32) and its label slot.  3D chunks are whole
  // planes, so a row's chunk is its plane.
  auto vrow = [&](int r, int by_, int bz_) -> const T* {
    if (G::D3) return &sm.vals[bz_ % NS][by_ * G::W + G::PADX - 1];
    return &sm.vals[(r / CH) % NS][(r % CH) * G::W + G::PADX - 1];
  };
  auto lslot = [&](int r, int by_, int bz_) -> int { return G::D3 ? (bz_ & 1) * BY + by_ : (r & 1); };
  auto owner_of = [&](int by_, int bz_) -> int {
    return (by_ == 0 ? 0 : (by_ == BY - 1 ? 2 : 1)) + 3 * (bz_ < HZ ? 0 : 1);
  };
  constexpr int NC = 2 * NRN + 1;  // candidate slots of a voxel

  issue(0);
  int by = 0, bz = 0;
  for (int rb = 0; rb < NRB; ++rb) {
    if (rb % CH == 0) {
      const int c = rb / CH;
      wait(c);
      if (err & ERR_WAIT) break;  // a chunk that never arrived: report, start no more copies
      issue(c + 1);
    }
    {
      const bool trow = by >= 1 && by <= TY && bz >= HZ;
      const int own = owner_of(by, bz);
      const T* vc = vrow(rb, by, bz);
      const int ls = lslot(rb, by, bz);
      uint16_t* lc = sm.lab[ls];
      // backward neighbour rows (warp-uniform); grp: a halo or column voxel of
      // this row may group with that row (dx = 0, inside the box, same owner)
      const T* vn[NRN];
      const uint16_t* ln[NRN];
      bool grp[NRN], grp_row[NRN];
      int lsn[NRN];
#pragma unroll
      for (int k = 0; k < NRN; ++k) {
        int dy, dz, dxs;
        row_nb<CONN>(k, dy, dz, dxs);
        const int byp = by + dy, bzp = bz + dz;
        const bool inbox = byp >= 0 && byp < BY && bzp >= 0;
        const int byq = inbox ? byp : by, bzq = inbox ? bzp : bz;
        vn[k] = vrow(rb + (inbox ? dy + BY * dz : 0), byq, bzq);
        lsn[k] = lslot(rb + (inbox ? dy + BY * dz : 0), byq, bzq);
        ln[k] = sm.lab[lsn[k]];
        grp[k] = inbox && (dxs & 2) && owner_of(byp, bzp) == own;
        grp_row[k] = grp[k] && !(byp >= 1 && byp <= TY && bzp >= HZ);
      }
      // -- the two halo columns of this row (lanes 0 and 1)
      {
        const int ci = lane == 0 ? 0 : 33;
        uint32_t lo = kNoLabel;
        bool differs = false, cfg = false;
        T cv = T(0);
        if (lane < 2) {
          cv = vc[ci];
          cfg = is_fg(cv);
#pragma unroll
          for (int k = 0; k < NRN; ++k) {
            if (cfg && grp[k] && rel<MODE>(cv, vn[k][ci])) {
              const uint32_t l = ln[k][ci];
              if (l != kNoLabel) {
                differs |= (lo != kNoLabel && l != lo);
                lo = l < lo ? l : lo;
              }
            }
          }
        }
        if (differs) {  // several labels meet (rare): join them
#pragma unroll
          for (int k = 0; k < NRN; ++k) {
            if (grp[k] && rel<MODE>(cv, vn[k][ci])) {
              const uint32_t l = ln[k][ci];
              if (l != kNoLabel && l != lo && !sunite_outlined(sm.par, (uint16_t)lo, (uint16_t)l)) err |= ERR_LOCAL_BUDGET;
            }
          }
        }
        uint32_t clab = lo == kNoLabel ? kNoLabel : find((uint16_t)lo);
        const bool cnew = cfg && lo == kNoLabel;
        const uint32_t nm = __ballot_sync(FULL, cnew);
        if (cnew) {
          clab = hl + __popc(nm & lt);
          sm.par[clab] = (uint16_t)clab;
          sm.hpos[clab - kTV] = (uint16_t)(rb * 34 + ci);
        }
        hl += __popc(nm);
        if (lane < 2) lc[ci] = (uint16_t)clab;
        if (lane == 0) sm.colfg[ls] = (is_fg(vc[0]) ? 1u : 0u) | (is_fg(vc[33]) ? 2u : 0u);
      }
      __syncwarp();

      // -- runs of the row
      const T v = vc[lane + 1];
      const bool fg = is_fg(v);
      const T sl = __shfl_up_sync(FULL, v, 1);
      bool link = lane > 0 && fg && is_fg(sl);
      const int64_t gy = y0 - 1 + by;
      if (MODE == MODE_MULTI) {
        link = link && (v == sl);
      } else if (MODE == MODE_BINARY4) {
        // the reference's binary 4-connected labeller links horizontal
        // neighbours of the first image row only when equal, and in later
        // rows not when both have foreground above (they meet through the
        // row above); halo rows keep single-voxel runs
        if (!trow) {
          link = false;
        } else if (gy == 0) {
          link = link && (v == sl);
        } else {
          const T a = vn[0][lane + 1];
          const T al = __shfl_up_sync(FULL, a, 1);
          link = link && !(is_fg(a) && is_fg(al));
        }
      }
      const uint32_t F = __ballot_sync(FULL, fg);
      const uint32_t Sm = F & ~__ballot_sync(FULL, link);
      const int head = head_of(Sm, lane);
      const int hsrc = fg ? head : lane;

      // -- labels of the related backward neighbours.  Of related neighbours
      // that are adjacent to each other only one needs to be taken: their
      // own join is already done (they precede this voxel), which is also
      // why a voxel equal to its primary neighbour takes that one alone.
      uint16_t cand[NC];
#pragma unroll
      for (int j = 0; j < NC; ++j) cand[j] = kNoLabel;
      if (fg) {
        if (trow) {
          bool m0[NRN];
#pragma unroll
          for (int k = 0; k < NRN; ++k) m0[k] = rel<MODE>(v, vn[k][lane + 1]);
          const bool covered =
              PRI0 >= 0 && m0[PRI0 < 0 ? 0 : PRI0] && (PRI1 < 0 || m0[PRI1 < 0 ? 0 : PRI1]);
#pragma unroll
          for (int k = 0; k < NRN; ++k) {
            int dy, dz, dxs;
            row_nb<CONN>(k, dy, dz, dxs);
            if (covered && k != PRI0 && k != PRI1) continue;
            if (m0[k]) {
              cand[2 * k] = ln[k][lane + 1];  // dx = -1 / +1, if related, are in its run
            } else {
              if ((dxs & 1) && rel<MODE>(v, vn[k][lane])) cand[2 * k] = ln[k][lane];
              if ((dxs & 4) && rel<MODE>(v, vn[k][lane + 2])) cand[2 * k + 1] = ln[k][lane + 2];
            }
          }
          if (!covered && lane == 0) {
            // same-row neighbour across the x seam
            const T c0 = vc[0];
            bool r0;
            if (MODE == MODE_MULTI) r0 = (v == c0);
            else if (MODE == MODE_BINARY4)
              r0 = is_fg(c0) && (gy == 0 ? (v == c0) : !(is_fg(vn[0][1]) && is_fg(vn[0][0])));
            else r0 = is_fg(c0);
            if (r0) cand[2 * NRN] = lc[0];
          }
        } else if (MODE != MODE_BINARY4) {
          // halo row: group with same-owner halo rows (dx = 0)
#pragma unroll
          for (int k = 0; k < NRN; ++k)
            if (grp_row[k] && rel<MODE>(v, vn[k][lane + 1])) cand[2 * k] = ln[k][lane + 1];
        }
      }
      uint32_t lo = kNoLabel;
#pragma unroll
      for (int j = 0; j < NC; ++j) lo = cand[j] < lo ? cand[j] : lo;
      bool differs = false;
#pragma unroll
      for (int j = 0; j < NC; ++j) differs |= (cand[j] != kNoLabel && cand[j] != lo);
      if (__any_sync(FULL, differs)) {
        // a voxel that touches several labels joins them (rare)
        if (differs) {
#pragma unroll
          for (int j = 0; j < NC; ++j)
            if (cand[j] != kNoLabel && cand[j] != lo && !sunite_outlined(sm.par, (uint16_t)lo, cand[j]))
              err |= ERR_LOCAL_BUDGET;
        }
        __syncwarp();
      }
      const uint32_t c1 = lo == kNoLabel ? kNoLabel : find((uint16_t)lo);

      // -- run label: smallest root over the run
      uint32_t m = c1;
      const uint32_t hc = __shfl_sync(FULL, m, hsrc);
      if (__ballot_sync(FULL, fg && m != hc)) {
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t t = __shfl_up_sync(FULL, m, o);
          if (fg && lane - o >= head && t < m) m = t;
        }
        const uint32_t after = (Sm | ~F) & ~lanemask_le(lane);
        const int last = after ? (__ffs(after) - 2) : 31;
        m = __shfl_sync(FULL, m, fg ? last : lane);
      } else {
        m = hc;
      }
      // runs without candidates open new labels
      const bool isnew = fg && lane == head && m == kNoLabel;
      const uint32_t nm = __ballot_sync(FULL, isnew);
      uint32_t lh = m;
      if (isnew) {
        if (trow) {
          lh = tl + __popc(nm & lt);
        } else {
          lh = hl + __popc(nm & lt);
          sm.hpos[lh - kTV] = (uint16_t)(rb * 34 + lane + 1);
        }
        sm.par[lh] = (uint16_t)lh;
      }
      if (trow) tl += __popc(nm); else hl += __popc(nm);
      const uint16_t RL = (uint16_t)__shfl_sync(FULL, lh, hsrc);
      // lanes whose root is not the run's join it (rare)
      const bool needmerge = fg && c1 != kNoLabel && c1 != RL;
      if (__any_sync(FULL, needmerge)) {
        if (needmerge && !sunite_outlined(sm.par, RL, (uint16_t)c1)) err |= ERR_LOCAL_BUDGET;
      }
      lc[lane + 1] = fg ? RL : kNoLabel;
      if (lane == 0) sm.fmr[ls] = F;

      if (trow) {
        const int ri = (by - 1) + TY * (bz - HZ);
        if (lane == 0) {
          sm.rowF[ri] = F;
          sm.rowS[ri] = Sm;
          sm.rowbase[ri] = (uint16_t)rbase;
        }
        if ((Sm >> lane) & 1u) sm.runlab[rbase + __popc(Sm & lt)] = RL;
        rbase += __popc(Sm);
        if (p.want_epl) {
          const T prev = lane == 0 ? vc[0] : sl;
          const unsigned em = __ballot_sync(FULL, (v != prev) && (v != T(0)));
          if (em) {
            epl_acc += __popc(em);
            const long long rg = (long long)((z0 - HZ + bz) * g.sy + gy);
            frow = rg < frow ? rg : frow;
            lrow = rg > lrow ? rg : lrow;
          }
        }
        if (p.want_prov) {
          // voxels the reference's binary labeller opens a label for: no
          // foreground among their backward neighbours
          uint32_t Lk;
          const int64_t gz = z0 - HZ + bz;
          if (MODE == MODE_BINARY4 && gy == 0 && gz == 0) {
            const T prev = lane == 0 ? vc[0] : sl;
            Lk = __ballot_sync(FULL, fg && is_fg(prev) && v == prev);
          } else {
            Lk = (F << 1) | (sm.colfg[ls] & 1u);
          }
#pragma unroll
          for (int k = 0; k < NRN; ++k) {
            int dy, dz, dxs;
            row_nb<CONN>(k, dy, dz, dxs);
            const uint32_t Fp = sm.fmr[lsn[k]], cf = sm.colfg[lsn[k]];
            if (dxs & 2) Lk |= Fp;
            if (dxs & 1) Lk |= (Fp << 1) | (cf & 1u);
            if (dxs & 4) Lk |= (Fp >> 1) | ((cf & 2u) ? 0x80000000u : 0u);
          }
          prov += __popc(F & ~Lk);
        }
      }
      __syncwarp();
    }
    if (++by == BY) {
      by = 0;
      ++bz;
    }
  }

  if (err & ERR_WAIT) {
    // the records of this tile are incomplete: publish an empty tile and the error
    give_up();
    return;
  }

  // ---- components in tile raster order of their first voxel
  auto rootf = [&](uint16_t n) -> uint16_t {
    for (int it = 0; it < kLocalLimit; ++it) {
      const uint16_t q = sm.par[n];
      if ((q & kCompFlag) || q == n) return n;
      n = q;
    }
    return n;
  };
  const uint32_t node0 = (uint32_t)(tile * kTV);
  uint32_t C = 0;
  for (int ri = 0; ri < NR; ++ri) {
    const uint32_t Sm = sm.rowS[ri], F = sm.rowF[ri];
    const uint32_t base = sm.rowbase[ri];
    const bool ishead = (Sm >> lane) & 1u;
    const uint32_t run = base + __popc(Sm & lt);
    uint16_t r = 0;
    bool isnewc = false;
    if (ishead) {
      r = rootf(sm.runlab[run]);
      isnewc = !(sm.par[r] & kCompFlag);
    }
    const uint32_t same = __match_any_sync(FULL, isnewc ? (uint32_t)r : 0x10000u + lane);
    const bool leader = isnewc && lane == __ffs(same) - 1;
    const uint32_t NL = __ballot_sync(FULL, leader);
    const int ly = ri % TY, lz = ri / TY;
    const int64_t y = y0 + ly, z = z0 + lz;
    if (leader) {
      const uint32_t cid = C + __popc(NL & lt);
      sm.par[r] = (uint16_t)(kCompFlag | cid);
      const uint32_t key = (uint32_t)(g.word0 * 32 + (z * g.sy + y) * g.key_row + x0 + lane);
      p.E[node0 + cid] = ((unsigned long long)key << 32) | (node0 + cid);
    }
    C += __popc(NL);
    __syncwarp();
    if (ishead) {
      const uint16_t q = sm.par[rootf(sm.runlab[run])];
      p.rcomp[tile * kTV + run] = (uint16_t)(q & (kCompFlag - 1));
    }
    if (lane == 0) {
      p.rmask[tile * kRowsPerTile + ri] = make_uint2(F, Sm);
      p.rrow[tile * kRowsPerTile + ri] = (uint16_t)base;
      if (y < g.sy && z < g.sz) p.bitmap[g.word0 + (z * g.sy + y) * g.wpr + tx] = NL;
    }
  }

  // ---- one edge per halo group that joined a tile component
  uint2* edges = p.edges + tile * p.edge_slots;
  uint32_t nedges = 0;
  for (uint32_t l0 = kTV; l0 < hl; l0 += 32) {
    const uint32_t l = l0 + lane;
    bool has = false;
    uint2 e;
    if (l < hl) {
      const uint16_t q = sm.par[rootf((uint16_t)l)];
      if (q & kCompFlag) {
        const int pos = sm.hpos[l - kTV];
        const int rb = pos / 34, i = pos % 34;
        const int by = rb % BY, bz = rb / BY;
        const int64_t gx = x0 - 1 + i, gy = y0 - 1 + by, gz = z0 - HZ + bz;
        const int64_t otile = g.tile0 + (gx >> 5) + (int64_t)g.ntx * ((gy / TY) + (int64_t)g.nty * (gz / TZ));
        const uint32_t local = (uint32_t)((gx & 31) + kTX * ((gy % TY) + TY * (gz % TZ)));
        e = make_uint2(node0 + (q & (kCompFlag - 1)), (uint32_t)(otile * kTV + local));
        has = true;
      }
    }
    const uint32_t m = __ballot_sync(FULL, has);
    if (has) {
      const uint32_t slot = nedges + __popc(m & lt);
      if (slot < p.edge_slots) edges[slot] = e;
    }
    nedges += __popc(m);
  }

  // ---- per-tile results
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const long long f2 = __shfl_down_sync(FULL, frow, o), l2 = __shfl_down_sync(FULL, lrow, o);
    frow = f2 < frow ? f2 : frow;
    lrow = l2 > lrow ? l2 : lrow;
  }
  if (lane == 0) {
    TileInfo ti;
    ti.C = C;
    ti.nedges = nedges < p.edge_slots ? nedges : p.edge_slots;
    ti.epl = (uint32_t)epl_acc;
    ti.prov = prov;
    ti.first_row = frow;
    ti.last_row = lrow;
    p.tinfo[tile] = ti;
    if (nedges > p.edge_slots) err |= ERR_EDGE_OVERFLOW;
  }
  err = __reduce_or_sync(FULL, err);
  if (lane == 0 && err) atomicOr(&p.ctr->err, err);
}

}  // namespace cc3dgpu
