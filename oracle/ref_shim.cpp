// ref_shim.cpp -- exposes the reference's own labelling core through a C ABI.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/Makefile against the
// reference's unmodified headers (cc3d/cc3d.hpp, cc3d/cc3d_binary.hpp,
// cc3d/cc3d_continuous.hpp) where they lie in the reference source tree;
// the result goes to oracle/_ref/ and is used to pin oracle/cc3d_oracle.c and
// as the CPU baseline of bench.py when it exists.  Nothing here is shipped.
//
// The entry points mirror the template calls the reference's Cython layer
// makes: estimate_provisional_label_count<T> (cc3d/fastcc3d.pyx:168-242 ->
// cc3d/cc3d.hpp:287-315) and connected_components3d<T,OUT> with delta = 0 and
// with a nonzero delta (cc3d/fastcc3d.pyx:494-608 ->
// cc3d/cc3d_continuous.hpp:394-455).
#include <cstdint>
#include <cstring>
#include <exception>
#include "cc3d_continuous.hpp"

namespace {

template <typename T>
int label_out(const void* in, int64_t sx, int64_t sy, int64_t sz,
              int64_t max_labels, int64_t conn, void* out, int out_dtype,
              uint64_t* N, bool periodic, bool binary) {
  size_t n = 0;
  T* data = const_cast<T*>(static_cast<const T*>(in));
  switch (out_dtype) {
    case 2:
      cc3d::connected_components3d<T, uint16_t>(data, sx, sy, sz, max_labels, conn, T(0),
                                                static_cast<uint16_t*>(out), n, periodic, binary);
      break;
    case 3:
      cc3d::connected_components3d<T, uint32_t>(data, sx, sy, sz, max_labels, conn, T(0),
                                                static_cast<uint32_t*>(out), n, periodic, binary);
      break;
    case 4:
      cc3d::connected_components3d<T, uint64_t>(data, sx, sy, sz, max_labels, conn, T(0),
                                                static_cast<uint64_t*>(out), n, periodic, binary);
      break;
    default:
      return -1;
  }
  *N = n;
  return 0;
}

// connected_components3d<T,OUT> with a nonzero delta (the continuous labellers)
template <typename T>
int label_delta(const void* in, int64_t sx, int64_t sy, int64_t sz, int64_t max_labels, int64_t conn,
                const void* delta, void* out, int out_dtype, uint64_t* N) {
  size_t n = 0;
  T d;
  memcpy(&d, delta, sizeof(T));
  T* data = const_cast<T*>(static_cast<const T*>(in));
  switch (out_dtype) {
    case 2:
      cc3d::connected_components3d<T, uint16_t>(data, sx, sy, sz, max_labels, conn, d,
                                                static_cast<uint16_t*>(out), n, false, false);
      break;
    case 3:
      cc3d::connected_components3d<T, uint32_t>(data, sx, sy, sz, max_labels, conn, d,
                                                static_cast<uint32_t*>(out), n, false, false);
      break;
    case 4:
      cc3d::connected_components3d<T, uint64_t>(data, sx, sy, sz, max_labels, conn, d,
                                                static_cast<uint64_t*>(out), n, false, false);
      break;
    default:
      return -1;
  }
  *N = n;
  return 0;
}

template <typename T>
uint64_t epl(const void* in, int64_t sx, int64_t voxels, int64_t* first, int64_t* last) {
  int64_t f = 0, l = 0;
  T* data = const_cast<T*>(static_cast<const T*>(in));
  uint64_t c = cc3d::estimate_provisional_label_count<T>(data, sx, voxels, f, l);
  *first = f;
  *last = l;
  return c;
}

}  // namespace

extern "C" {

// dtype codes: 1 u8, 2 u16, 3 u32, 4 u64, 5 f32, 6 f64.  `out` must be zeroed
// by the caller, as the reference's Cython layer does (np.zeros).
int ref_connected_components(const void* in, int dtype, int64_t sx, int64_t sy,
                             int64_t sz, int64_t max_labels, int64_t conn, void* out,
                             int out_dtype, uint64_t* N, int periodic, int binary) {
  try {
    switch (dtype) {
      case 1: return label_out<uint8_t>(in, sx, sy, sz, max_labels, conn, out, out_dtype, N, periodic, binary);
      case 2: return label_out<uint16_t>(in, sx, sy, sz, max_labels, conn, out, out_dtype, N, periodic, binary);
      case 3: return label_out<uint32_t>(in, sx, sy, sz, max_labels, conn, out, out_dtype, N, periodic, binary);
      case 4: return label_out<uint64_t>(in, sx, sy, sz, max_labels, conn, out, out_dtype, N, periodic, binary);
      case 5: return label_out<float>(in, sx, sy, sz, max_labels, conn, out, out_dtype, N, periodic, binary);
      case 6: return label_out<double>(in, sx, sy, sz, max_labels, conn, out, out_dtype, N, periodic, binary);
    }
  } catch (const std::exception&) {
    return -2;
  }
  return -1;
}

int ref_connected_components_delta(const void* in, int dtype, int64_t sx, int64_t sy, int64_t sz,
                                   int64_t max_labels, int64_t conn, const void* delta, void* out,
                                   int out_dtype, uint64_t* N) {
  try {
    switch (dtype) {
      case 1: return label_delta<uint8_t>(in, sx, sy, sz, max_labels, conn, delta, out, out_dtype, N);
      case 2: return label_delta<uint16_t>(in, sx, sy, sz, max_labels, conn, delta, out, out_dtype, N);
      case 3: return label_delta<uint32_t>(in, sx, sy, sz, max_labels, conn, delta, out, out_dtype, N);
      case 4: return label_delta<uint64_t>(in, sx, sy, sz, max_labels, conn, delta, out, out_dtype, N);
      case 5: return label_delta<float>(in, sx, sy, sz, max_labels, conn, delta, out, out_dtype, N);
      case 6: return label_delta<double>(in, sx, sy, sz, max_labels, conn, delta, out, out_dtype, N);
    }
  } catch (const std::exception&) {
    return -2;
  }
  return -1;
}

uint64_t ref_epl(const void* in, int dtype, int64_t sx, int64_t voxels,
                 int64_t* first, int64_t* last) {
  switch (dtype) {
    case 1: return epl<uint8_t>(in, sx, voxels, first, last);
    case 2: return epl<uint16_t>(in, sx, voxels, first, last);
    case 3: return epl<uint32_t>(in, sx, voxels, first, last);
    case 4: return epl<uint64_t>(in, sx, voxels, first, last);
    case 5: return epl<float>(in, sx, voxels, first, last);
    case 6: return epl<double>(in, sx, voxels, first, last);
  }
  return (uint64_t)-1;
}

}  // extern "C"
