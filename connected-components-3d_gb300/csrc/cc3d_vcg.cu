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
template <typename T, typename OUT, bool D3, int REV>
__global__ void __launch_bounds__(VX * VY) k_vcg(const T* __restrict__ in, int64_t sx, int64_t sy, int64_t sz,
                                                 OUT* __restrict__ out, uint32_t mask, int64_t nbx, int64_t nby) {
  __shared__ T box[BZW][BYW][BXW];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * VX + tx;
  int64_t b = blockIdx.x;
  const int64_t bx = b % nbx;
  b /= nbx;
  const int64_t by = b % nby, bz = b / nby;
  const int64_t x0 = bx * VX, y0 = by * VY, z0 = bz * VZ;
  // stage the box (out-of-volume entries are never compared)
  for (int i = tid; i < BZW * BYW * BXW; i += VX * VY) {
    const int lx = i % BXW, ly = (i / BXW) % BYW, lz = i / (BXW * BYW);
    const int64_t gx = x0 - 1 + lx, gy = y0 - 1 + ly, gz = z0 - 1 + lz;
    T v = T(0);
    if (gx >= 0 && gx < sx && gy >= 0 && gy < sy && gz >= 0 && gz < sz) v = in[(gz * sy + gy) * sx + gx];
    box[lz][ly][lx] = v;
  }
  __syncthreads();
  const int64_t x = x0 + tx, y = y0 + ty;
  if (x >= sx || y >= sy) return;
  // which neighbours exist, per axis and side
  const bool xm = x > 0, xp = x < sx - 1, ym = y > 0, yp = y < sy - 1;
  for (int lz = 0; lz < VZ; ++lz) {
    const int64_t z = z0 + lz;
    if (z >= sz) break;
    const bool zm = z > 0, zp = z < sz - 1;
    const T cur = box[lz + 1][ty + 1][tx + 1];
    uint32_t bits = 0;
    if (D3) {
#pragma unroll
      for (int dz = -1; dz <= 1; ++dz)
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
          for (int dx = -1; dx <= 1; ++dx) {
            if (!dx && !dy && !dz) continue;
            const bool exists = (dx < 0 ? xm : (dx > 0 ? xp : true)) && (dy < 0 ? ym : (dy > 0 ? yp : true)) &&
                                (dz < 0 ? zm : (dz > 0 ? zp : true));
            const bool differs = exists && box[lz + 1 + dz][ty + 1 + dy][tx + 1 + dx] != cur;
            if (!differs)
              bits |= 1u << (REV == 3 ? dir_bit3(dz, dy, dx) : REV == 2 ? dir_bit3(dy, dx, dz) : dir_bit3(dx, dy, dz));
          }
    } else {
#pragma unroll
      for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
          if (!dx && !dy) continue;
          const bool exists = (dx < 0 ? xm : (dx > 0 ? xp : true)) && (dy < 0 ? ym : (dy > 0 ? yp : true));
          const bool differs = exists && box[1][ty + 1 + dy][tx + 1 + dx] != cur;
          if (!differs) bits |= 1u << (REV ? dir_bit2(dy, dx) : dir_bit2(dx, dy));
        }
    }
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
  if (!labels || !graph) return failf(CC3D_ERR_INVALID, "invalid arguments");
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
