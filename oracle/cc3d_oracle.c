/*
 * cc3d_oracle.c -- CPU restatement of cc3d's labelling semantics.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU path: it is
 * loaded by tests/, by __graft_entry__.smoke() and by the CPU-baseline leg of
 * bench.py, and by nothing in the product.  It is pinned against the reference
 * itself (oracle/_ref, the reference's own headers compiled by oracle/Makefile)
 * and against the golden vectors in tests/golden/.
 *
 * What it restates (paths relative to the cc3d source tree):
 *   - estimate_provisional_label_count   cc3d/cc3d.hpp:287-315
 *   - the labelling contract of connected_components3d
 *       dispatch                         cc3d/cc3d_continuous.hpp:394-455,
 *                                        cc3d/cc3d.hpp:1423-1471,
 *                                        cc3d/cc3d_binary.hpp:1266-1314
 *       neighbourhoods                   26: cc3d/cc3d.hpp:372-399 (13-voxel backward mask)
 *                                        18: cc3d/cc3d.hpp:597-755, 6: cc3d/cc3d.hpp:757-1076,
 *                                        8: cc3d/cc3d.hpp:1287-1421, 4: cc3d/cc3d.hpp:1096-1280
 *       periodic wrap pairs              6: cc3d/cc3d.hpp:1048-1073, 4: cc3d/cc3d.hpp:1265-1277,
 *                                        8: cc3d/cc3d.hpp:1377-1418,
 *                                        binary: cc3d/cc3d_binary.hpp:733-758, 938-950,
 *                                        cc3d/cc3d_binary.hpp:1170-1210
 *       continuous values (delta != 0)   cc3d/cc3d_continuous.hpp:90-392: the 3D labeller
 *                                        (26/18/6, with its exact-equality shortcut below),
 *                                        the 2D 4-connected one and the 2D 8-connected one
 *                                        with its image-span shortcut, restated branch by
 *                                        branch in oracle_connected_components_continuous
 *       numbering                        cc3d/cc3d.hpp:244-285 (relabel): components are
 *                                        numbered 1..N in raster order of their first voxel;
 *                                        binary 8-connected images use the 2x2-block
 *                                        labeller (cc3d/cc3d_binary.hpp:955-1263), which
 *                                        numbers components in block-raster order of their
 *                                        first 2x2 block.
 *
 * The algorithm is the classic two-pass scheme the reference also uses: a
 * raster pass assigns provisional labels (copying a matching backward
 * neighbour's label, uniting differing ones in a union-find over labels whose
 * root is the smallest label), the periodic wrap pairs are united, and a second
 * pass writes each voxel's component number.  Background voxels are written as
 * 0.  It is single-threaded, like the reference.
 *
 * Known, documented difference: for binary 8-connected images whose memory
 * dimensions are not both even, the reference's in-place relabel
 * (cc3d/cc3d_binary.hpp:1237-1260) leaves provisional block labels in some
 * background pixels outside each row's foreground span.  This oracle writes 0
 * there, as the GPU path does; foreground pixels match exactly.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define DT_U8 1
#define DT_U16 2
#define DT_U32 3
#define DT_U64 4
#define DT_F32 5
#define DT_F64 6

static inline uint32_t uf_find(uint32_t *p, uint32_t i) {
  while (p[i] != i) {
    p[i] = p[p[i]];
    i = p[i];
  }
  return i;
}

/* union-find over provisional labels 1..n; the root of a set is its
   smallest label, so a parent is always smaller than its child. */
typedef struct {
  uint32_t *par;
  uint32_t n, cap;
  int oom;
} Labels;

static uint32_t lab_new(Labels *L) {
  if (L->n + 1 >= L->cap) {
    uint32_t nc = L->cap ? L->cap * 2 : 1024;
    uint32_t *np_ = (uint32_t *)realloc(L->par, sizeof(uint32_t) * nc);
    if (!np_) { L->oom = 1; return L->n; }
    L->par = np_;
    L->cap = nc;
  }
  L->n++;
  L->par[L->n] = L->n;
  return L->n;
}

static uint32_t lab_unite(Labels *L, uint32_t a, uint32_t b) {
  a = uf_find(L->par, a);
  b = uf_find(L->par, b);
  if (a == b) return a;
  if (a < b) { L->par[b] = a; return a; }
  L->par[a] = b;
  return b;
}

/* backward offsets (dx, dy, dz) per connectivity */
static const int OFF26[13][3] = {
  {-1,-1,-1},{0,-1,-1},{1,-1,-1},{-1,0,-1},{0,0,-1},{1,0,-1},{-1,1,-1},{0,1,-1},{1,1,-1},
  {-1,-1,0},{0,-1,0},{1,-1,0},{-1,0,0}};
static const int OFF18[9][3] = {
  {0,-1,-1},{-1,0,-1},{0,0,-1},{1,0,-1},{0,1,-1},{-1,-1,0},{0,-1,0},{1,-1,0},{-1,0,0}};
static const int OFF6[3][3] = {{0,0,-1},{0,-1,0},{-1,0,0}};
static const int OFF8[4][3] = {{-1,-1,0},{0,-1,0},{1,-1,0},{-1,0,0}};
static const int OFF4[2][3] = {{0,-1,0},{-1,0,0}};

static int offsets_for(int conn, const int (**off)[3]) {
  switch (conn) {
    case 26: *off = OFF26; return 13;
    case 18: *off = OFF18; return 9;
    case 6: *off = OFF6; return 3;
    case 8: *off = OFF8; return 4;
    case 4: *off = OFF4; return 2;
  }
  return -1;
}

/* ---- per-type kernels, generated by macro ---------------------------- */

#define FG(v) ((v) != 0)
#define EQV(a, b) (binary ? (FG(a) && FG(b)) : (FG(a) && (a) == (b)))

#define DEFINE_TYPE(SUF, T)                                                     \
static uint64_t epl_##SUF(const T *in, int64_t sx, int64_t voxels,              \
                          int64_t *first, int64_t *last) {                      \
  uint64_t count = 0;                                                           \
  *first = -1; *last = -1;                                                      \
  int64_t row = 0;                                                              \
  for (int64_t loc = 0; loc < voxels; loc += sx, row++) {                       \
    uint64_t rc = (in[loc] != 0);                                               \
    for (int64_t x = 1; x < sx; x++)                                            \
      rc += (in[loc + x] != in[loc + x - 1] && in[loc + x] != 0);               \
    count += rc;                                                                \
    if (rc) { if (*first == -1) *first = row; *last = row; }                    \
  }                                                                             \
  return count;                                                                 \
}                                                                               \
/* Two-pass labelling with provisional labels, as the reference does: the   \
   first raster pass copies a matching backward neighbour's label (or opens  \
   a new one) and unites differing labels in a union-find over labels whose  \
   root is always the smallest label; periodic wrap pairs are united next.   \
   For 26-connectivity a voxel equal to the voxel below it (z-1) takes that  \
   label and needs no other test: every other backward neighbour it relates  \
   to is also a 26-neighbour of the voxel below, and that pair was already   \
   united earlier in the scan.  By the same argument an interior voxel that  \
   relates to the voxel behind it (y-1) or on its left (x-1) takes that      \
   label and only tests the backward neighbours not adjacent to it (26: 3    \
   and 4 of them; 18: 3 and 4, and 2 for the voxel below).  The relation     \
   is an equivalence (equal values, or both foreground), which the argument  \
   needs.  Returns the number of provisional labels.                         */ \
static uint32_t first_pass_##SUF(const T *in, int64_t sx, int64_t sy, int64_t sz, \
                                 int conn, int binary, int periodic,            \
                                 uint32_t *lab, Labels *L) {                    \
  const int (*off)[3];                                                          \
  int noff = offsets_for(conn, &off);                                           \
  const int64_t sxy = sx * sy;                                                  \
  int64_t doff[13];                                                             \
  for (int k = 0; k < noff; k++)                                                \
    doff[k] = off[k][0] + sx * off[k][1] + sxy * off[k][2];                     \
  /* binary 4-connected (cc3d/cc3d_binary.hpp:776-953): the first row links    \
     horizontal neighbours only when their values are equal (:833), and later   \
     rows skip the horizontal link when both pixels have foreground above      \
     (the SIMPLE state, :903-918), relying on the row above being linked.      \
     Together these define the reference's effective neighbour relation.     */ \
  const int row0_eq = binary && conn == 4;                                      \
  const int below_shortcut = (conn == 26);                                      \
  /* shortcuts of interior voxels: a related neighbour (below z-1, behind     \
     y-1, left x-1) and the backward neighbours not adjacent to it */          \
  int nsc = 0;                                                                  \
  int64_t sc_prim[3], sc_rest[3][4];                                            \
  int sc_n[3];                                                                  \
  if (conn == 26) {                                                             \
    /* below: handled before, for every voxel with z > 0 */                     \
    const int64_t behind[3] = {-1 + sx - sxy, sx - sxy, 1 + sx - sxy};          \
    const int64_t left[4] = {1 - sx - sxy, 1 - sxy, 1 + sx - sxy, 1 - sx};      \
    sc_prim[0] = -sx; sc_n[0] = 3; memcpy(sc_rest[0], behind, sizeof(behind));  \
    sc_prim[1] = -1; sc_n[1] = 4; memcpy(sc_rest[1], left, sizeof(left));       \
    nsc = 2;                                                                    \
  } else if (conn == 18 && !row0_eq) {                                          \
    const int64_t below[2] = {-1 - sx, 1 - sx};                                 \
    const int64_t behind[3] = {-1 - sxy, 1 - sxy, sx - sxy};                    \
    const int64_t left[4] = {-sx - sxy, 1 - sxy, sx - sxy, 1 - sx};             \
    sc_prim[0] = -sxy; sc_n[0] = 2; memcpy(sc_rest[0], below, sizeof(below));   \
    sc_prim[1] = -sx; sc_n[1] = 3; memcpy(sc_rest[1], behind, sizeof(behind));  \
    sc_prim[2] = -1; sc_n[2] = 4; memcpy(sc_rest[2], left, sizeof(left));       \
    nsc = 3;                                                                    \
  }                                                                             \
  for (int64_t z = 0; z < sz; z++)                                              \
    for (int64_t y = 0; y < sy; y++) {                                          \
      int64_t row = sx * (y + sy * z);                                          \
      int yz_in = (y >= 1) && (y + 1 < sy) && (z >= 1);                         \
      for (int64_t x = 0; x < sx; x++) {                                        \
        int64_t i = row + x;                                                    \
        T v = in[i];                                                            \
        if (!FG(v)) { lab[i] = 0; continue; }                                   \
        if (below_shortcut && z > 0 && EQV(v, in[i - sxy])) {                   \
          lab[i] = lab[i - sxy];                                                \
          continue;                                                             \
        }                                                                       \
        int interior = yz_in && x >= 1 && x + 1 < sx;                           \
        uint32_t cur = 0;                                                       \
        if (nsc && interior) {                                                  \
          int hit = -1;                                                         \
          for (int q = 0; q < nsc; q++)                                         \
            if (EQV(v, in[i + sc_prim[q]])) { hit = q; break; }                 \
          if (hit >= 0) {                                                       \
            cur = lab[i + sc_prim[hit]];                                        \
            for (int k = 0; k < sc_n[hit]; k++) {                               \
              const int64_t j = i + sc_rest[hit][k];                            \
              if (!EQV(v, in[j])) continue;                                     \
              const uint32_t l = lab[j];                                        \
              if (l != cur) cur = lab_unite(L, cur, l);                         \
            }                                                                   \
            lab[i] = cur;                                                       \
            continue;                                                           \
          }                                                                     \
        }                                                                       \
        for (int k = 0; k < noff; k++) {                                        \
          if (!interior) {                                                      \
            int64_t nx = x + off[k][0], ny = y + off[k][1], nz = z + off[k][2]; \
            if (nx < 0 || nx >= sx || ny < 0 || ny >= sy || nz < 0 || nz >= sz) \
              continue;                                                         \
          }                                                                     \
          int64_t j = i + doff[k];                                              \
          T w = in[j];                                                          \
          if (!EQV(v, w)) continue;                                             \
          if (row0_eq && off[k][1] == 0) {                                      \
            if (y == 0) { if (v != w) continue; }                               \
            else if (FG(in[i - sx]) && FG(in[j - sx])) continue;                \
          }                                                                     \
          uint32_t l = lab[j];                                                  \
          if (cur == 0) cur = l;                                                \
          else if (l != cur) cur = lab_unite(L, cur, l);                        \
        }                                                                       \
        if (cur == 0) cur = lab_new(L);                                         \
        lab[i] = cur;                                                           \
      }                                                                         \
    }                                                                           \
  if (periodic) {                                                               \
    /* wrap pairs: x faces, y faces (with diagonals for 8), z faces, corners */ \
    if (conn == 6 || conn == 4) {                                               \
      for (int64_t z = 0; z < sz; z++)                                          \
        for (int64_t y = 0; y < sy; y++) {                                      \
          int64_t a = sx * (y + sy * z), b = a + sx - 1;                        \
          if (EQV(in[a], in[b])) lab_unite(L, lab[a], lab[b]);                  \
        }                                                                       \
      for (int64_t z = 0; z < sz; z++)                                          \
        for (int64_t x = 0; x < sx; x++) {                                      \
          int64_t a = x + sxy * z, b = a + sx * (sy - 1);                       \
          if (EQV(in[a], in[b])) lab_unite(L, lab[a], lab[b]);                  \
        }                                                                       \
      if (conn == 6)                                                            \
        for (int64_t y = 0; y < sy; y++)                                        \
          for (int64_t x = 0; x < sx; x++) {                                    \
            int64_t a = x + sx * y, b = a + sxy * (sz - 1);                     \
            if (EQV(in[a], in[b])) lab_unite(L, lab[a], lab[b]);                \
          }                                                                     \
    } else if (conn == 8) {                                                     \
      const int64_t voxels = sx * sy;                                           \
      const int64_t bot = sx * (sy - 1);                                        \
      for (int64_t x = 0; x < sx; x++) {                                        \
        if (!FG(in[x])) continue;                                               \
        if (x > 0 && EQV(in[x], in[x - 1 + bot])) lab_unite(L, lab[x], lab[x - 1 + bot]); \
        if (EQV(in[x], in[x + bot])) lab_unite(L, lab[x], lab[x + bot]);       \
        if (x < sx - 1 && EQV(in[x], in[x + 1 + bot]))                          \
          lab_unite(L, lab[x], lab[x + 1 + bot]);                               \
      }                                                                         \
      if (EQV(in[0], in[voxels - 1])) lab_unite(L, lab[0], lab[voxels - 1]);   \
      if (EQV(in[sx - 1], in[bot])) lab_unite(L, lab[sx - 1], lab[bot]);       \
      for (int64_t y = 0; y < sy; y++) {                                        \
        int64_t a = sx * y;                                                     \
        if (!FG(in[a])) continue;                                               \
        if (EQV(in[a], in[a + sx - 1])) lab_unite(L, lab[a], lab[a + sx - 1]);  \
        if (y > 0 && EQV(in[a], in[a - 1])) lab_unite(L, lab[a], lab[a - 1]);   \
        if (y < sy - 1 && EQV(in[a], in[a + 2 * sx - 1]))                       \
          lab_unite(L, lab[a], lab[a + 2 * sx - 1]);                            \
      }                                                                         \
    }                                                                           \
  }                                                                             \
  return L->n;                                                                  \
}                                                                               \
static int fg_##SUF(const void *in, int64_t i) { return FG(((const T *)in)[i]); } \
/* Provisional labels the reference's binary labeller would create: a voxel  \
   (or, for 8-connected, a 2x2 block) opens a new label iff none of its       \
   backward-mask neighbours is foreground.                                   */ \
static uint64_t prov_##SUF(const T *in, int64_t sx, int64_t sy, int64_t sz,     \
                           int conn) {                                          \
  uint64_t P = 0;                                                               \
  if (conn == 8) {                                                              \
    for (int64_t y = 0; y < sy; y += 2)                                         \
      for (int64_t x = 0; x < sx; x += 2) {                                     \
        int Y = FG(in[x + sx * y]);                                             \
        int Z = x + 1 < sx && FG(in[x + 1 + sx * y]);                           \
        int X = y + 1 < sy && FG(in[x + sx * (y + 1)]);                         \
        int W = x + 1 < sx && y + 1 < sy && FG(in[x + 1 + sx * (y + 1)]);       \
        if (!(Y || Z || X || W)) continue;                                      \
        int up = y > 0;                                                         \
        int C = up && x > 0 && FG(in[x - 1 + sx * (y - 1)]);                    \
        int D = up && FG(in[x + sx * (y - 1)]);                                 \
        int E = up && x + 1 < sx && FG(in[x + 1 + sx * (y - 1)]);               \
        int F = up && x + 2 < sx && FG(in[x + 2 + sx * (y - 1)]);               \
        int B = x > 0 && FG(in[x - 1 + sx * y]);                                \
        int A = x > 0 && y + 1 < sy && FG(in[x - 1 + sx * (y + 1)]);            \
        int linked = (Y && (C || D || E || B || A)) || (Z && (D || E || F)) ||  \
                     (X && (B || A));                                           \
        if (!linked) P++;                                                       \
      }                                                                         \
    return P;                                                                   \
  }                                                                             \
  const int (*off)[3];                                                          \
  int noff = offsets_for(conn, &off);                                           \
  for (int64_t z = 0; z < sz; z++)                                              \
    for (int64_t y = 0; y < sy; y++)                                            \
      for (int64_t x = 0; x < sx; x++) {                                        \
        int64_t i = x + sx * (y + sy * z);                                      \
        if (!FG(in[i])) continue;                                               \
        int linked = 0;                                                         \
        for (int k = 0; k < noff && !linked; k++) {                             \
          int64_t nx = x + off[k][0], ny = y + off[k][1], nz = z + off[k][2];   \
          if (nx < 0 || nx >= sx || ny < 0 || ny >= sy || nz < 0 || nz >= sz)   \
            continue;                                                           \
          T w = in[nx + sx * (ny + sy * nz)];                                   \
          if (conn == 4 && y == 0 && off[k][1] == 0) linked = (w == in[i]);     \
          else linked = FG(w);                                                  \
        }                                                                       \
        if (!linked) P++;                                                       \
      }                                                                         \
  return P;                                                                     \
}

DEFINE_TYPE(u8, uint8_t)
DEFINE_TYPE(u16, uint16_t)
DEFINE_TYPE(u32, uint32_t)
DEFINE_TYPE(u64, uint64_t)
DEFINE_TYPE(f32, float)
DEFINE_TYPE(f64, double)

static void store_label(void *out, int out_dtype, int64_t i, uint64_t lab) {
  switch (out_dtype) {
    case DT_U16: ((uint16_t *)out)[i] = (uint16_t)lab; break;
    case DT_U32: ((uint32_t *)out)[i] = (uint32_t)lab; break;
    default: ((uint64_t *)out)[i] = lab; break;
  }
}

/* Provisional labels live in the output itself when it is uint32 (as the
   reference's labellers write into out_labels), else in a scratch array. */
static uint32_t *provisional_buffer(void *out, int out_dtype, int64_t voxels) {
  if (out_dtype == DT_U32) return (uint32_t *)out;
  return (uint32_t *)malloc(sizeof(uint32_t) * (size_t)voxels);
}

static void release_provisional(uint32_t *lab, void *out) {
  if ((void *)lab != out) free(lab);
}

/* Second pass: out[i] = fin[lab[i]] in the output's type, where fin maps a
   provisional label to its component number and fin[0] = 0.  lab may be the
   output itself (uint32): each element is read before it is overwritten. */
static void write_labels(void *out, int out_dtype, const uint32_t *lab, const uint32_t *fin,
                         int64_t voxels) {
  switch (out_dtype) {
    case DT_U16: {
      uint16_t *o = (uint16_t *)out;
      for (int64_t i = 0; i < voxels; i++) o[i] = (uint16_t)fin[lab[i]];
      break;
    }
    case DT_U32: {
      uint32_t *o = (uint32_t *)out;
      for (int64_t i = 0; i < voxels; i++) o[i] = fin[lab[i]];
      break;
    }
    default: {
      uint64_t *o = (uint64_t *)out;
      for (int64_t i = 0; i < voxels; i++) o[i] = fin[lab[i]];
      break;
    }
  }
}

/* Turns the flattened forest (par[p] = root of p) into fin[p] = component
   number of p, in place, given ren[root] = number; fin[0] = 0.  Returns the
   table to index with (a one-entry zero table when there are no labels). */
static const uint32_t *finish_table(Labels *L, const uint32_t *ren) {
  static const uint32_t none[1] = {0};
  if (!L->par) return none;
  for (uint32_t p = 1; p <= L->n; p++) L->par[p] = ren[L->par[p]];
  L->par[0] = 0;
  return L->par;
}

/* Per-label voxel counts, bounding boxes and coordinate sums of a label
 * array: a restatement of _statistics_helper2d/3d (cc3d/fastcc3d.pyx:767-938).
 * Axes are the array's own (x = axis 0, y = axis 1, z = axis 2, extents d0, d1,
 * d2; a 2D array has d2 = 1); c_order says whether the buffer is C or Fortran
 * ordered.  One pass in memory order: counts[l] (uint32, wrapping like the
 * reference's), bmin/bmax[3 l + a] (bmin starts at 0xFFFFFFFF, bmax at 0), and
 * centroids[3 l + a] = sum of coordinates / count, NaN for a count of 0.  The
 * reference adds coordinates into a double one by one; every partial sum is an
 * integer below 2^53, so the exact 64-bit sums divided once are the same
 * doubles.  Returns 0, -1 for a label above N or a bad width, -4 when out of
 * memory. */
#define STATS_PASS(T)                                                            \
  do {                                                                           \
    const T *lab = (const T *)labels;                                            \
    int64_t i = 0;                                                               \
    if (c_order) {                                                               \
      for (int64_t x = 0; x < d0; x++)                                           \
        for (int64_t y = 0; y < d1; y++)                                         \
          for (int64_t z = 0; z < d2; z++, i++) STATS_VOXEL((uint64_t)lab[i]);   \
    } else {                                                                     \
      for (int64_t z = 0; z < d2; z++)                                           \
        for (int64_t y = 0; y < d1; y++)                                         \
          for (int64_t x = 0; x < d0; x++, i++) STATS_VOXEL((uint64_t)lab[i]);   \
    }                                                                            \
  } while (0)
#define STATS_VOXEL(L)                                                           \
  do {                                                                           \
    const uint64_t l = (L);                                                      \
    if (l > N) { bad = 1; break; }                                               \
    const uint32_t c[3] = {(uint32_t)x, (uint32_t)y, (uint32_t)z};               \
    counts[l]++;                                                                 \
    for (int a = 0; a < 3; a++) {                                                \
      if (c[a] < bmin[3 * l + a]) bmin[3 * l + a] = c[a];                        \
      if (c[a] > bmax[3 * l + a]) bmax[3 * l + a] = c[a];                        \
      sums[3 * l + a] += c[a];                                                   \
    }                                                                            \
  } while (0)
int oracle_statistics(const void *labels, int label_bytes, int64_t d0, int64_t d1, int64_t d2,
                      int c_order, uint64_t N, uint32_t *counts, uint32_t *bmin, uint32_t *bmax,
                      double *centroids) {
  const uint64_t n1 = N + 1;
  uint64_t *sums = (uint64_t *)calloc((size_t)(3 * n1), sizeof(uint64_t));
  if (!sums) return -4;
  for (uint64_t l = 0; l < n1; l++) {
    counts[l] = 0;
    for (int a = 0; a < 3; a++) { bmin[3 * l + a] = 0xFFFFFFFFu; bmax[3 * l + a] = 0; }
  }
  int bad = 0;
  switch (label_bytes) {
    case 1: STATS_PASS(uint8_t); break;
    case 2: STATS_PASS(uint16_t); break;
    case 4: STATS_PASS(uint32_t); break;
    case 8: STATS_PASS(uint64_t); break;
    default: bad = 1;
  }
  if (!bad)
    for (uint64_t l = 0; l < n1; l++)
      for (int a = 0; a < 3; a++)
        centroids[3 * l + a] = counts[l] ? (double)sums[3 * l + a] / (double)counts[l] : NAN;
  free(sums);
  return bad ? -1 : 0;
}
#undef STATS_VOXEL
#undef STATS_PASS

/* Estimated provisional label count and first/last foreground row
 * (cc3d/cc3d.hpp:287-315).  Returns (uint64_t)-1 on an unknown dtype. */
uint64_t oracle_epl(const void *in, int dtype, int64_t sx, int64_t voxels,
                    int64_t *first, int64_t *last) {
  switch (dtype) {
    case DT_U8: return epl_u8((const uint8_t *)in, sx, voxels, first, last);
    case DT_U16: return epl_u16((const uint16_t *)in, sx, voxels, first, last);
    case DT_U32: return epl_u32((const uint32_t *)in, sx, voxels, first, last);
    case DT_U64: return epl_u64((const uint64_t *)in, sx, voxels, first, last);
    case DT_F32: return epl_f32((const float *)in, sx, voxels, first, last);
    case DT_F64: return epl_f64((const double *)in, sx, voxels, first, last);
  }
  return (uint64_t)-1;
}

/* Label `in` (x fastest, sx*sy*sz voxels) into `out` (uint16/32/64 by
 * out_dtype).  connectivity in {26,18,6} or {8,4} (sz must be 1).  Returns 0,
 * -1 on bad arguments, -2 when sz != 1 for a 2D connectivity, -3 when the
 * volume has 2^32 voxels or more, -4 on allocation failure, and -5 where the
 * reference's binary labeller would overflow its union-find and throw
 * "maximum length exception" (its table is sized from max_labels with
 * per-labeller caps: cc3d/cc3d_binary.hpp:49-54, 350-354, 532-537, 795-800,
 * 966-971; DisjointSet::add, cc3d/cc3d.hpp:106-115). */
int oracle_connected_components(const void *in, int dtype, int64_t sx,
                                int64_t sy, int64_t sz, int64_t max_labels,
                                int connectivity, int binary, int periodic,
                                void *out, int out_dtype, uint64_t *N) {
  const int (*off)[3];
  if (offsets_for(connectivity, &off) < 0) return -1;
  if ((connectivity == 8 || connectivity == 4) && sz != 1) return -2;
  const int64_t voxels = sx * sy * sz;
  *N = 0;
  if (voxels == 0) return 0;
  if (voxels >= (int64_t)0xFFFFFFFFLL) return -3;
  if (max_labels == 0) {
    for (int64_t i = 0; i < voxels; i++) store_label(out, out_dtype, i, 0);
    return 0;
  }
  if (binary) {
    uint64_t P = 0;
    switch (dtype) {
      case DT_U8: P = prov_u8((const uint8_t *)in, sx, sy, sz, connectivity); break;
      case DT_U16: P = prov_u16((const uint16_t *)in, sx, sy, sz, connectivity); break;
      case DT_U32: P = prov_u32((const uint32_t *)in, sx, sy, sz, connectivity); break;
      case DT_U64: P = prov_u64((const uint64_t *)in, sx, sy, sz, connectivity); break;
      case DT_F32: P = prov_f32((const float *)in, sx, sy, sz, connectivity); break;
      case DT_F64: P = prov_f64((const double *)in, sx, sy, sz, connectivity); break;
    }
    uint64_t L = (uint64_t)max_labels + 1, V = (uint64_t)voxels;
    uint64_t outmax = out_dtype == DT_U16 ? 0xFFFFull : out_dtype == DT_U32 ? 0xFFFFFFFFull : ~0ull;
    switch (connectivity) {
      case 26: L = (L < (V >> 2) + 1 ? L : (V >> 2) + 1) + 1; break;
      case 18: L = (L < V + 1 ? L : V + 1); break;
      case 8: L = (L < (V >> 1) + 1 ? L : (V >> 1) + 1); if (L < 1) L = 1; L += 1; break;
      default: L = (L < (V >> 1) + 1 ? L : (V >> 1) + 1) + 1; break;
    }
    if (L > outmax) L = outmax;
    if (P >= L) return -5;
  }
  uint32_t *lab = provisional_buffer(out, out_dtype, voxels);
  if (!lab) return -4;
  Labels L = {NULL, 0, 0, 0};
  int (*fg)(const void *, int64_t) = NULL;
  switch (dtype) {
#define CASE(D, SUF, T)                                                     \
    case D:                                                                 \
      first_pass_##SUF((const T *)in, sx, sy, sz, connectivity, binary,     \
                       periodic, lab, &L);                                  \
      fg = fg_##SUF;                                                        \
      break;
    CASE(DT_U8, u8, uint8_t)
    CASE(DT_U16, u16, uint16_t)
    CASE(DT_U32, u32, uint32_t)
    CASE(DT_U64, u64, uint64_t)
    CASE(DT_F32, f32, float)
    CASE(DT_F64, f64, double)
#undef CASE
    default: release_provisional(lab, out); return -1;
  }
  if (L.oom) { release_provisional(lab, out); free(L.par); return -4; }
  /* flatten: parents are smaller than children, so one increasing pass
     leaves every label pointing at its root */
  for (uint32_t p = 1; p <= L.n; p++) L.par[p] = L.par[L.par[p]];
  uint32_t *ren = (uint32_t *)calloc((size_t)L.n + 1, sizeof(uint32_t));
  if (!ren && L.n) { release_provisional(lab, out); free(L.par); return -4; }
  uint64_t n = 0;
  if (binary && connectivity == 8) {
    /* block-raster numbering: visit 2x2 blocks in raster order; a component
       takes its number at the first block that holds one of its pixels. */
    for (int64_t by = 0; by < sy; by += 2)
      for (int64_t bx = 0; bx < sx; bx += 2)
        for (int dy = 0; dy < 2; dy++)
          for (int dx = 0; dx < 2; dx++) {
            int64_t x = bx + dx, y = by + dy;
            if (x >= sx || y >= sy) continue;
            uint32_t l = lab[x + sx * y];
            if (!l) continue;
            uint32_t r = L.par[l];
            if (ren[r] == 0) ren[r] = (uint32_t)++n;
          }
  } else {
    /* the smallest provisional label of a component is the one its first
       voxel opened, so numbering roots in label order is raster order */
    for (uint32_t p = 1; p <= L.n; p++)
      if (L.par[p] == p) ren[p] = (uint32_t)++n;
  }
  write_labels(out, out_dtype, lab, finish_table(&L, ren), voxels);
  (void)fg;
  free(ren);
  free(L.par);
  release_provisional(lab, out);
  *N = n;
  return 0;
}


/* ---- continuous values (delta != 0) ------------------------------------ */

/* |a - b| <= delta as cc3d::match (cc3d/cc3d_continuous.hpp:80-88) */
#define UMATCH(a, b, d) (((a) > (b) ? (a) - (b) : (b) - (a)) <= (d))
#define FMATCH(a, b, d) (fabsf((a) - (b)) <= (d))
#define DMATCH(a, b, d) (fabs((a) - (b)) <= (d))

#define DEFINE_CONT(SUF, T, MATCH)                                              \
/* 3D labeller (cc3d/cc3d_continuous.hpp:90-180): neighbour table of           \
   compute_neighborhood (:36-76), the first connectivity/2 entries.         */ \
static void cont3d_##SUF(const T *in, int64_t sx, int64_t sy, int64_t sz,      \
                         int conn, T delta, uint32_t *lab, Labels *L) {        \
  static const int NB[13][3] = {                                               \
    {-1,0,0},{0,-1,0},{0,0,-1},{-1,-1,0},{1,-1,0},{0,-1,-1},{0,1,-1},          \
    {-1,0,-1},{1,0,-1},{-1,-1,-1},{1,-1,-1},{-1,1,-1},{1,1,-1}};               \
  const int64_t sxy = sx * sy;                                                 \
  const int nn = conn / 2;                                                     \
  for (int64_t z = 0; z < sz; z++)                                             \
    for (int64_t y = 0; y < sy; y++)                                           \
      for (int64_t x = 0; x < sx; x++) {                                       \
        const int64_t i = x + sx * (y + sy * z);                               \
        const T cur = in[i];                                                   \
        if (cur == 0) { lab[i] = 0; continue; }                                \
        if (z > 0 && conn == 26 && cur == in[i - sxy]) {                       \
          lab[i] = lab[i - sxy];                                               \
          continue;                                                            \
        }                                                                      \
        uint32_t c = 0;                                                        \
        for (int k = 0; k < nn; k++) {                                         \
          const int64_t nx = x + NB[k][0], ny = y + NB[k][1], nz = z + NB[k][2]; \
          if (nx < 0 || nx >= sx || ny < 0 || ny >= sy || nz < 0) continue;    \
          const int64_t j = i + NB[k][0] + sx * NB[k][1] + sxy * NB[k][2];     \
          const T w = in[j];                                                   \
          if (w == 0 || !(MATCH(cur, w, delta))) continue;                     \
          if (c) c = lab_unite(L, c, lab[j]);                                  \
          else c = lab[j];                                                     \
        }                                                                      \
        lab[i] = c ? c : lab_new(L);                                           \
      }                                                                        \
}                                                                              \
/* 2D 4-connected (cc3d/cc3d_continuous.hpp:182-259) */                        \
static void cont4_##SUF(const T *in, int64_t sx, int64_t sy, T delta,          \
                        uint32_t *lab, Labels *L) {                            \
  for (int64_t y = 0; y < sy; y++)                                             \
    for (int64_t x = 0; x < sx; x++) {                                         \
      const int64_t i = x + sx * y;                                            \
      const T cur = in[i];                                                     \
      if (cur == 0) { lab[i] = 0; continue; }                                  \
      if (x > 0 && in[i - 1] != 0 && (MATCH(cur, in[i - 1], delta))) {         \
        lab[i] = lab[i - 1];                                                   \
        if (y > 0 && cur != in[i - 1 - sx]) {                                  \
          if (in[i - sx] != 0 && (MATCH(cur, in[i - sx], delta)))              \
            lab_unite(L, lab[i], lab[i - sx]);                                 \
        }                                                                      \
      } else if (y > 0 && in[i - sx] != 0 && (MATCH(cur, in[i - sx], delta))) { \
        lab[i] = lab[i - sx];                                                  \
      } else {                                                                 \
        lab[i] = lab_new(L);                                                   \
      }                                                                        \
    }                                                                          \
}                                                                              \
/* 2D 8-connected (cc3d/cc3d_continuous.hpp:261-343), with the image's        \
   minimum and maximum folded by std::min / std::max from element 0         */ \
static void cont8_##SUF(const T *in, int64_t sx, int64_t sy, T delta,          \
                        uint32_t *lab, Labels *L) {                            \
  const int64_t voxels = sx * sy;                                              \
  T gmax = in[0], gmin = in[0];                                                \
  for (int64_t i = 1; i < voxels; i++) {                                       \
    gmax = (in[i] < gmax) ? gmax : in[i];   /* std::max(in[i], gmax) */        \
    gmin = (gmin < in[i]) ? gmin : in[i];   /* std::min(in[i], gmin) */        \
  }                                                                            \
  for (int64_t y = 0; y < sy; y++)                                             \
    for (int64_t x = 0; x < sx; x++) {                                         \
      const int64_t i = x + sx * y;                                            \
      const T cur = in[i];                                                     \
      if (cur == 0) { lab[i] = 0; continue; }                                  \
      if (y > 0) {                                                             \
        const T b = in[i - sx];                                                \
        if (cur == b) { lab[i] = lab[i - sx]; continue; }                      \
        if (b != 0) {                                                          \
          const T mn = (b < cur) ? b : cur, mx = (cur < b) ? b : cur;          \
          if ((T)(mn - gmin) <= delta && (T)(gmax - mx) <= delta) {            \
            lab[i] = lab[i - sx];                                              \
            continue;                                                          \
          }                                                                    \
        }                                                                      \
      }                                                                        \
      uint32_t c = 0;                                                          \
      if (y > 0 && in[i - sx] != 0 && (MATCH(cur, in[i - sx], delta))) c = lab[i - sx]; \
      if (x > 0 && y > 0 && in[i - 1 - sx] != 0 && (MATCH(cur, in[i - 1 - sx], delta))) \
        c = c ? lab_unite(L, c, lab[i - 1 - sx]) : lab[i - 1 - sx];            \
      if (x < sx - 1 && y > 0 && in[i + 1 - sx] != 0 && (MATCH(cur, in[i + 1 - sx], delta))) \
        c = c ? lab_unite(L, c, lab[i + 1 - sx]) : lab[i + 1 - sx];            \
      if (x > 0 && in[i - 1] != 0 && (MATCH(cur, in[i - 1], delta)))           \
        c = c ? lab_unite(L, c, lab[i - 1]) : lab[i - 1];                      \
      lab[i] = c ? c : lab_new(L);                                             \
    }                                                                          \
}

DEFINE_CONT(u8, uint8_t, UMATCH)
DEFINE_CONT(u16, uint16_t, UMATCH)
DEFINE_CONT(u32, uint32_t, UMATCH)
DEFINE_CONT(u64, uint64_t, UMATCH)
DEFINE_CONT(f32, float, FMATCH)
DEFINE_CONT(f64, double, DMATCH)

/* Continuous-value labelling of `in` (delta: one element of the input type
 * at `delta`), numbered 1..N in raster order of each component's first
 * voxel.  Returns 0, -1 on bad arguments, -2 when sz != 1 for a 2D
 * connectivity, -3 for 2^32 voxels or more, -4 on allocation failure. */
int oracle_connected_components_continuous(const void *in, int dtype, int64_t sx,
                                           int64_t sy, int64_t sz, int connectivity,
                                           const void *delta, void *out, int out_dtype,
                                           uint64_t *N) {
  const int (*off)[3];
  if (offsets_for(connectivity, &off) < 0 || !delta) return -1;
  if ((connectivity == 8 || connectivity == 4) && sz != 1) return -2;
  const int64_t voxels = sx * sy * sz;
  *N = 0;
  if (voxels == 0) return 0;
  if (voxels >= (int64_t)0xFFFFFFFFLL) return -3;
  uint32_t *lab = provisional_buffer(out, out_dtype, voxels);
  if (!lab) return -4;
  Labels L = {NULL, 0, 0, 0};
  switch (dtype) {
#define CASE(D, SUF, T)                                                          \
    case D: {                                                                    \
      T d;                                                                       \
      memcpy(&d, delta, sizeof(T));                                              \
      if (connectivity == 8) cont8_##SUF((const T *)in, sx, sy, d, lab, &L);     \
      else if (connectivity == 4) cont4_##SUF((const T *)in, sx, sy, d, lab, &L); \
      else cont3d_##SUF((const T *)in, sx, sy, sz, connectivity, d, lab, &L);    \
      break;                                                                     \
    }
    CASE(DT_U8, u8, uint8_t)
    CASE(DT_U16, u16, uint16_t)
    CASE(DT_U32, u32, uint32_t)
    CASE(DT_U64, u64, uint64_t)
    CASE(DT_F32, f32, float)
    CASE(DT_F64, f64, double)
#undef CASE
    default: release_provisional(lab, out); return -1;
  }
  if (L.oom) { release_provisional(lab, out); free(L.par); return -4; }
  for (uint32_t p = 1; p <= L.n; p++) L.par[p] = L.par[L.par[p]];
  uint32_t *ren = (uint32_t *)calloc((size_t)L.n + 1, sizeof(uint32_t));
  if (!ren && L.n) { release_provisional(lab, out); free(L.par); return -4; }
  uint64_t n = 0;
  for (uint32_t p = 1; p <= L.n; p++)
    if (L.par[p] == p) ren[p] = (uint32_t)++n;
  write_labels(out, out_dtype, lab, finish_table(&L, ren), voxels);
  free(ren);
  free(L.par);
  release_provisional(lab, out);
  *N = n;
  return 0;
}
