// cc3d_vcg.cu -- the voxel connectivity graph of a labelled volume on the
// device: cc3d.voxel_connectivity_graph (cc3d/fastcc3d.pyx:1021-1178,
// extract_voxel_connectivity_graph in cc3d/cc3d_graphs.hpp:31-240).
//
// Every voxel gets a bit per direction of its neighbourhood; a bit is cleared
// when the neighbour in that direction lies inside the volume and holds a
// different label, and stays set otherwise (also at the volume's faces).  The
// reference visits each pair once from its later voxel and clears both ends;
// here every voxel gathers its own bits, which gives the same field.
//
// A block of 32 x 8 threads covers 32 x 8 x 8 voxels: the box with its
// one-voxel halo (34 x 10 x 10) is staged in shared memory with coalesced
// loads, then every thread walks its 8 voxels along z.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "cc3d_gpu.h"
#include "cc3d_internal.h"

using namespace cc3dgpu;

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

constexpr int VX = 32, VY = 8, VZ = 8;                  // voxels per block
constexpr int BXW = VX + 2, BYW = VY + 2, BZW = VZ + 2;  // staged box with halo

// REV: the array is C-ordered, so memory runs its last axis fastest: with
// REV = 3 (3D arrays) memory offsets (a, b, c) are the field's directions
// (x, y, z) = (c, b, a); with REV = 2 (2D arrays) (x, y, z) = (b, a, c).
// sx, sy, sz are the memory extents, fastest first.
template <int REV, bool D3>
__device__ __forceinline__ int field_bit(int da, int db, int dc) {
  if (!D3) return REV ? dir_bit2(db, da) : dir_bit2(da, db);
  return REV == 3 ? dir_bit3(dc, db, da) : REV == 2 ? dir_bit3(db, da, dc) : dir_bit3(da, db, dc);
}

template <typename T, typename OUT, bool D3, int REV>
__global__ void __launch_bounds__(VX * VY) k_vcg(const T* __restrict__ in, int64_t sx, int64_t sy, int64_t sz,
                                                 OUT* __restrict__ out, uint32_t mask, int64_t nbx, int64_t nby) {
  constexpr int NZ = D3 ? BZW : 1;  // staged planes (one for 2D fields)
  __shared__ T box[NZ][BYW][BXW];
  const int tx = threadIdx.x, ty = threadIdx.y;
  int64_t b = blockIdx.x;
  const int64_t bx = b % nbx;
  b /= nbx;
  const int64_t by = b % nby, bz = b / nby;
  const int64_t x0 = bx * VX, y0 = by * VY, z0 = bz * VZ;
  // stage the box row by row, coalesced along x (out-of-volume entries are
  // never compared: their directions are set from the coordinates)
  for (int r = ty; r < NZ * BYW; r += VY) {
    const int lz = r / BYW, ly = r - lz * BYW;
    const int64_t gy = y0 - 1 + ly, gz = D3 ? z0 - 1 + lz : 0;
    const bool rowin = gy >= 0 && gy < sy && gz >= 0 && gz < sz;
    const T* row = in + (gz * sy + gy) * sx;
    for (int c = tx; c < BXW; c += VX) {
      const int64_t gx = x0 - 1 + c;
      box[lz][ly][c] = (rowin && gx >= 0 && gx < sx) ? row[gx] : T(0);
    }
  }
  __syncthreads();
  const int64_t x = x0 + tx, y = y0 + ty;
  if (x >= sx || y >= sy) return;
  const bool xm = x > 0, xp = x < sx - 1, ym = y > 0, yp = y < sy - 1;
  // directions whose neighbour lies outside the volume keep their bit
  uint32_t oob_xy = 0;
#pragma unroll
  for (int dc = -1; dc <= 1; ++dc)
#pragma unroll
    for (int db = -1; db <= 1; ++db)
#pragma unroll
      for (int da = -1; da <= 1; ++da) {
        if ((!D3 && dc) || (!da && !db && !dc)) continue;
        const bool out_ab = (da < 0 && !xm) || (da > 0 && !xp) || (db < 0 && !ym) || (db > 0 && !yp);
        if (out_ab) oob_xy |= 1u << field_bit<REV, D3>(da, db, dc);
      }
  if (!D3) {
    const T cur = box[0][ty + 1][tx + 1];
    uint32_t bits = oob_xy;
#pragma unroll
    for (int db = -1; db <= 1; ++db)
#pragma unroll
      for (int da = -1; da <= 1; ++da)
        if (da || db) bits |= (uint32_t)(box[0][ty + 1 + db][tx + 1 + da] == cur) << field_bit<REV, D3>(da, db, 0);
    out[y * sx + x] = (OUT)(bits & mask);
    return;
  }
  // slide a 3 x 3 x 3 window of registers along c (memory z)
  T w[3][3][3];  // [dc + 1][db + 1][da + 1]
#pragma unroll
  for (int k = 0; k < 2; ++k)
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int i = 0; i < 3; ++i) w[k + 1][j][i] = box[k][ty + j][tx + i];
  uint32_t up_bits = 0, down_bits = 0;  // the dc = +1 / -1 directions
#pragma unroll
  for (int db = -1; db <= 1; ++db)
#pragma unroll
    for (int da = -1; da <= 1; ++da) {
      up_bits |= 1u << field_bit<REV, D3>(da, db, 1);
      down_bits |= 1u << field_bit<REV, D3>(da, db, -1);
    }
  for (int lz = 0; lz < VZ; ++lz) {
    const int64_t z = z0 + lz;
    if (z >= sz) break;
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        w[0][j][i] = w[1][j][i];
        w[1][j][i] = w[2][j][i];
        w[2][j][i] = box[lz + 2][ty + j][tx + i];
      }
    const T cur = w[1][1][1];
    uint32_t bits = oob_xy | (z > 0 ? 0u : down_bits) | (z < sz - 1 ? 0u : up_bits);
#pragma unroll
    for (int dc = -1; dc <= 1; ++dc)
#pragma unroll
      for (int db = -1; db <= 1; ++db)
#pragma unroll
        for (int da = -1; da <= 1; ++da)
          if (da || db || dc) bits |= (uint32_t)(w[dc + 1][db + 1][da + 1] == cur) << field_bit<REV, D3>(da, db, dc);
    out[(z * sy + y) * sx + x] = (OUT)(bits & mask);
  }
}

template <typename T, typename OUT, bool D3>
void launch_vcg(const void* in, int64_t sx, int64_t sy, int64_t sz, void* out, uint32_t mask, int rev,
                cudaStream_t s) {
  const int64_t nbx = (sx + VX - 1) / VX, nby = (sy + VY - 1) / VY, nbz = (sz + VZ - 1) / VZ;
  const unsigned grid = (unsigned)(nbx * nby * nbz);
  const T* i = static_cast<const T*>(in);
  OUT* o = static_cast<OUT*>(out);
  if (rev == 3) k_vcg<T, OUT, D3, 3><<<grid, dim3(VX, VY), 0, s>>>(i, sx, sy, sz, o, mask, nbx, nby);
  else if (rev == 2) k_vcg<T, OUT, D3, 2><<<grid, dim3(VX, VY), 0, s>>>(i, sx, sy, sz, o, mask, nbx, nby);
  else k_vcg<T, OUT, D3, 0><<<grid, dim3(VX, VY), 0, s>>>(i, sx, sy, sz, o, mask, nbx, nby);
}

template <typename T>
void launch_vcg_t(const void* in, int64_t sx, int64_t sy, int64_t sz, int conn, void* out, int rev,
                  cudaStream_t s) {
  // 2D fields for 4 / 8 (one plane), 3D fields otherwise; 8-bit outputs for 4, 8, 6
  switch (conn) {
    case 26: launch_vcg<T, uint32_t, true>(in, sx, sy, sz, out, 0x3ffffffu, rev, s); break;
    case 18: launch_vcg<T, uint32_t, true>(in, sx, sy, sz, out, 0x3ffffu, rev, s); break;
    case 6: launch_vcg<T, uint8_t, true>(in, sx, sy, sz, out, 0x3fu, rev, s); break;
    case 8: launch_vcg<T, uint8_t, false>(in, sx, sy, sz, out, 0xffu, rev, s); break;
    default: launch_vcg<T, uint8_t, false>(in, sx, sy, sz, out, 0x0fu, rev, s); break;
  }
}

}  // namespace

extern "C" int cc3d_gpu_voxel_connectivity_graph(const void* labels, int label_bytes, int64_t sx, int64_t sy,
                                                 int64_t sz, int connectivity, int reversed_axes, void* graph,
                                                 void* stream) {
  if ((label_bytes != 1 && label_bytes != 2 && label_bytes != 4 && label_bytes != 8) || sx < 0 || sy < 0 ||
      sz < 0 || (reversed_axes != 0 && reversed_axes != 2 && reversed_axes != 3))
    return failf(CC3D_ERR_INVALID, "invalid arguments");
  if (connectivity != 26 && connectivity != 18 && connectivity != 6 && connectivity != 8 && connectivity != 4)
    return failf(CC3D_ERR_RUNTIME, "Only 4 and 8 2D and 6, 18, and 26 3D connectivities are supported.");
  // (a reversed 2D array has memory extents (sy, sx, 1): still one plane)
  if ((connectivity == 8 || connectivity == 4) && sz != 1)
    return failf(CC3D_ERR_RUNTIME, "sz must be 1 for 2D connectivities.");
  const int64_t voxels = sx * sy * sz;
  if (voxels == 0) return CC3D_OK;
  if (!device_accessible(labels) || !device_accessible(graph))
    return failf(CC3D_ERR_INVALID, "labels and graph must be device memory");
  if ((sx + VX - 1) / VX * ((sy + VY - 1) / VY) * ((sz + VZ - 1) / VZ) >= (1ll << 31))
    return failf(CC3D_ERR_UNSUPPORTED, "volume too large");
  cudaStream_t s = (cudaStream_t)stream;
  switch (label_bytes) {
    case 1: launch_vcg_t<uint8_t>(labels, sx, sy, sz, connectivity, graph, reversed_axes, s); break;
    case 2: launch_vcg_t<uint16_t>(labels, sx, sy, sz, connectivity, graph, reversed_axes, s); break;
    case 4: launch_vcg_t<uint32_t>(labels, sx, sy, sz, connectivity, graph, reversed_axes, s); break;
    default: launch_vcg_t<uint64_t>(labels, sx, sy, sz, connectivity, graph, reversed_axes, s); break;
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return failf(CC3D_ERR_CUDA, "voxel connectivity graph: %s", cudaGetErrorString(e));
  return CC3D_OK;
}
