"""Drop-in front end for cc3d's labelling path on the GPU.

Mirrors the reference's Cython layer (cc3d/fastcc3d.pyx) argument by argument:
validation, dtype views, order handling, the provisional-label estimate that
fixes the output dtype, the single-foreground-row special case, output
allocation (including mmapped ``out_file``), the final reshape and the torch
round trip.  The labelling itself runs through the C ABI in
include/cc3d_gpu.h.

numpy arrays (and CPU torch tensors) are staged to the GPU by the library and
the result comes back as numpy (torch for torch input), as in the reference.
CUDA torch tensors stay on their device: the output is a CUDA tensor and the
work is ordered on the tensor's current stream.
"""
from __future__ import annotations

import ctypes
import operator
import os
from functools import reduce
from typing import Any, Optional, Sequence, Tuple, Union

import numpy as np

from . import _native as nat


class DimensionError(Exception):
    """The array has the wrong number of dimensions (cc3d/fastcc3d.pyx:123-125)."""


_UNSUPPORTED = (
    "Type {} is not currently supported. "
    "Supported: bool, int8, int16, int32, int64, uint8, uint16, uint32, uint64, float16, float32, float64"
)

_CODE = {
    np.dtype(np.bool_): nat.U8, np.dtype(np.uint8): nat.U8, np.dtype(np.int8): nat.U8,
    np.dtype(np.uint16): nat.U16, np.dtype(np.int16): nat.U16,
    np.dtype(np.uint32): nat.U32, np.dtype(np.int32): nat.U32,
    np.dtype(np.uint64): nat.U64, np.dtype(np.int64): nat.U64,
    np.dtype(np.float32): nat.F32, np.dtype(np.float64): nat.F64,
}
_OUT_CODE = {np.dtype(np.uint16): nat.U16, np.dtype(np.uint32): nat.U32, np.dtype(np.uint64): nat.U64}


# ----------------------------------------------------------------- helpers
def _is_torch(x) -> bool:
    return hasattr(x, "cpu") and hasattr(x, "is_cuda")


def _torch():
    import torch
    return torch


def _np_dtype_of_torch(t) -> np.dtype:
    torch = _torch()
    table = {
        torch.bool: np.bool_, torch.uint8: np.uint8, torch.int8: np.int8,
        torch.int16: np.int16, torch.int32: np.int32, torch.int64: np.int64,
        torch.float16: np.float16, torch.float32: np.float32, torch.float64: np.float64,
    }
    for name, npt in (("uint16", np.uint16), ("uint32", np.uint32), ("uint64", np.uint64)):
        if hasattr(torch, name):
            table[getattr(torch, name)] = npt
    if t.dtype not in table:
        raise TypeError(_UNSUPPORTED.format(t.dtype))
    return np.dtype(table[t.dtype])


def _torch_dtype(npd: np.dtype):
    torch = _torch()
    return {
        "bool": torch.bool, "uint8": torch.uint8, "int8": torch.int8, "int16": torch.int16,
        "int32": torch.int32, "int64": torch.int64, "float16": torch.float16,
        "float32": torch.float32, "float64": torch.float64,
        "uint16": getattr(torch, "uint16", None), "uint32": getattr(torch, "uint32", None),
        "uint64": getattr(torch, "uint64", None),
    }[np.dtype(npd).name]


def _contig_flags(shape: Sequence[int], strides: Sequence[int]) -> Tuple[bool, bool]:
    """numpy's C/F contiguity rules (size-1 axes are ignored) for element strides."""
    if any(s == 0 for s in shape):
        return True, True
    c = True
    expect = 1
    for n, st in zip(reversed(shape), reversed(strides)):
        if n != 1:
            if st != expect:
                c = False
                break
            expect *= n
    f = True
    expect = 1
    for n, st in zip(shape, strides):
        if n != 1:
            if st != expect:
                f = False
                break
            expect *= n
    return c, f


class _Dev:
    """A CUDA torch tensor seen through numpy-like attributes."""

    def __init__(self, t):
        self.t = t
        self.npdtype = _np_dtype_of_torch(t)

    @property
    def shape(self):
        return tuple(self.t.shape)

    @property
    def size(self):
        return self.t.numel()

    def flags(self):
        return _contig_flags(self.t.shape, self.t.stride())

    def ptr(self):
        return nat.dev_ptr(self.t)

    def stream(self):
        return ctypes.c_void_p(_torch().cuda.current_stream(self.t.device).cuda_stream)


def _even_ceil(n: int) -> int:
    return n << 1 if n & 1 else n


def _reshape_flat(arr: np.ndarray) -> np.ndarray:
    if arr.flags.f_contiguous:
        return arr.reshape(-1, order="F")
    if arr.flags.c_contiguous:
        return arr.reshape(-1, order="C")
    return np.ascontiguousarray(arr).reshape(-1)


# --------------------------------------------------------------- epl
def _epl_call(ptr, code, sx, voxels, mem, stream):
    lib = nat.load()
    epl, first, last = ctypes.c_uint64(0), ctypes.c_int64(0), ctypes.c_int64(0)
    nat.check(lib.cc3d_gpu_estimate_provisional_label_count(
        ptr, code, int(sx), int(voxels), ctypes.byref(epl), ctypes.byref(first),
        ctypes.byref(last), mem, stream))
    return int(epl.value), int(first.value), int(last.value)


def estimate_provisional_labels(data) -> Tuple[int, int, int]:
    """(epl, first_foreground_row, last_foreground_row) of `data`.

    Mirrors cc3d.estimate_provisional_labels (cc3d/fastcc3d.pyx:168-242); the
    count is done on the GPU.  float16 is not accepted here (the reference
    only accepts it through connected_components, which views it as uint16)."""
    if _is_torch(data) and data.is_cuda:
        d = _Dev(data)
        c, f = d.flags()
        if d.npdtype not in _CODE:
            raise TypeError(_UNSUPPORTED.format(d.npdtype))
        t = data if (c or f) else data.contiguous()
        if not (c or f):
            c, f = True, False
        sx = t.shape[0] if f else t.shape[-1]
        with _torch().cuda.device(t.device):
            return _epl_call(nat.dev_ptr(t), _CODE[d.npdtype], sx, t.numel(), nat.IN_DEVICE, d.stream())
    if _is_torch(data):
        data = data.cpu().numpy()
    if data.dtype not in _CODE:
        raise TypeError(_UNSUPPORTED.format(data.dtype))
    sx = data.shape[0] if data.flags.f_contiguous else data.shape[-1]
    linear = np.ascontiguousarray(_reshape_flat(data))
    if linear.size == 0:
        return (0, -1, -1)
    return _epl_call(linear.ctypes.data, _CODE[data.dtype], sx, linear.size, 0, None)


_CTYPE_NAME = {1: "uint8_t", 2: "uint16_t", 4: "uint32_t", 8: "uint64_t"}


def _delta_element(delta, dtype) -> ctypes.Array:
    """delta as one element of the type the labeller runs on (the unsigned
    view of integer data, or the float type), raising the OverflowError that
    Cython's conversion to that C type raises (cc3d/fastcc3d.pyx:494-608)."""
    dt = np.dtype(dtype)
    if dt.kind == "f":
        raw = np.array([delta], dtype=dt).tobytes()
    else:
        width = dt.itemsize
        d = int(delta)
        if d < 0:
            raise OverflowError(f"can't convert negative value to {_CTYPE_NAME[width]}")
        if d >= 1 << (8 * width):
            raise OverflowError(f"value too large to convert to {_CTYPE_NAME[width]}")
        raw = d.to_bytes(width, "little")
    return ctypes.create_string_buffer(raw, 8)


# ---------------------------------------------------------- main entry
def connected_components(
    data: Any,
    max_labels: int = -1,
    connectivity: int = 26,
    return_N: bool = False,
    delta: Union[int, float] = 0,
    out_dtype: Optional[Any] = None,
    out_file: Optional[Any] = None,
    periodic_boundary: bool = False,
    binary_image: bool = False,
):
    """Connected components of a 2D or 3D image, numbered 1..N.

    Same signature, return values, dtypes and exceptions as
    cc3d.connected_components (cc3d/fastcc3d.pyx:244-626), including
    continuous-value labelling (``delta`` > 0: neighbours join when their
    values differ by at most delta; cc3d/cc3d_continuous.hpp:90-392)."""
    is_torch = _is_torch(data)
    on_device = is_torch and data.is_cuda
    if is_torch and not on_device:
        data = data.cpu().numpy()

    shape0 = tuple(data.shape)
    dims = len(shape0)
    if dims not in (1, 2, 3):
        raise DimensionError("Only 1D, 2D, and 3D arrays supported. Got: " + str(dims))
    if dims == 2 and connectivity not in (4, 8, 6, 18, 26):
        raise ValueError("Only 4, 8, and 6, 18, 26 connectivities are supported for 2D images. Got: " + str(connectivity))
    elif dims != 2 and connectivity not in (6, 18, 26):
        raise ValueError("Only 6, 18, and 26 connectivities are supported for 3D images. Got: " + str(connectivity))
    if periodic_boundary and connectivity not in (4, 8, 6):
        raise ValueError(f"periodic_boundary is not yet implemented for {connectivity}-connectivity.")
    if periodic_boundary and delta != 0:
        raise ValueError("periodic_boundary is not yet implemented continuous data.")

    size = reduce(operator.mul, shape0, 1)
    if size == 0:
        dt = np.dtype(out_dtype) if out_dtype is not None else (
            _np_dtype_of_torch(data) if on_device else data.dtype)
        if on_device:
            out = _torch().zeros((0,), dtype=_torch_dtype(dt), device=data.device)
        else:
            out = np.zeros(shape=(0,), dtype=dt)
        return (out, 0) if return_N else out

    if on_device:
        dev = _Dev(data)
        cflag, fflag = dev.flags()
        order = "F" if fflag else "C"
        t = data
        while t.dim() < 3:
            t = t.unsqueeze(0) if order == "C" else t.unsqueeze(-1)
        c3, f3 = _contig_flags(t.shape, t.stride())
        if not c3 and not f3:
            t = t.contiguous()
        dtype = dev.npdtype
        if dtype == np.float16:
            if delta == 0:
                t = t.view(_torch().int16)
                dtype = np.dtype(np.uint16)
            else:
                raise TypeError("float16 is not supported for continuous images (delta != 0).")
        shape = list(t.shape)
    else:
        order = "F" if data.flags.f_contiguous else "C"
        while len(data.shape) < 3:
            data = data[np.newaxis, ...] if order == "C" else data[..., np.newaxis]
        if not data.flags.c_contiguous and not data.flags.f_contiguous:
            data = np.copy(data, order=order)
        if data.dtype == np.float16:
            if delta == 0:
                data = data.view(np.uint16)
            else:
                raise TypeError("float16 is not supported for continuous images (delta != 0).")
        dtype = data.dtype
        shape = list(data.shape)
    padded_shape = list(shape)
    if order == "C":
        shape.reverse()
    sx, sy, sz = (int(v) for v in shape)
    voxels = sx * sy * sz

    if np.dtype(dtype) not in _CODE:
        raise TypeError(_UNSUPPORTED.format(dtype))
    code = _CODE[np.dtype(dtype)]
    binary0 = bool(binary_image or (dtype == bool))
    # delta equal to the dtype's maximum makes any image binary (fastcc3d.pyx:397-403)
    if np.issubdtype(dtype, np.floating):
        delta = float(delta)
        binary_image = binary0 or (delta == np.finfo(dtype).max)
    else:
        delta = int(delta)
        binary_image = binary0 or (delta == np.iinfo(dtype).max)
    continuous = delta != 0 and not binary_image

    if on_device:
        stream = dev.stream()
        torch = _torch()
        devctx = torch.cuda.device(t.device)
        ptr = nat.dev_ptr(t)
    else:
        stream = None
        devctx = None
        flat = _reshape_flat(data)
        ptr = flat.ctypes.data
    mem_in = nat.IN_DEVICE if on_device else 0
    mem_out_hint = nat.OUT_DEVICE if (on_device and out_file is None) else 0
    lib = nat.load()

    def call(fn, *args):
        if devctx is not None:
            with devctx:
                return fn(*args)
        return fn(*args)

    # labelling up to the numbering; the same pass computes the estimate
    info = nat.Prepared()
    if continuous:
        dbuf = _delta_element(delta, dtype)
        nat.check(call(lib.cc3d_gpu_label_prepare_continuous, ptr, code, sx, sy, sz, int(connectivity),
                       dbuf, mem_in | mem_out_hint, stream, ctypes.byref(info)))
    else:
        nat.check(call(lib.cc3d_gpu_label_prepare, ptr, code, sx, sy, sz, int(connectivity),
                       int(bool(periodic_boundary)), int(binary_image), mem_in | mem_out_hint, stream,
                       ctypes.byref(info)))
    if binary0:
        epl, first_row, last_row = voxels, 0, sy
    elif binary_image:
        epl, first_row, last_row = call(_epl_call, ptr, code, sx, voxels, mem_in, stream)
        info = nat.Prepared()
        nat.check(call(lib.cc3d_gpu_label_prepare, ptr, code, sx, sy, sz, int(connectivity),
                       int(bool(periodic_boundary)), 1, mem_in | mem_out_hint, stream,
                       ctypes.byref(info)))
    else:
        epl, first_row, last_row = int(info.epl), int(info.first_row), int(info.last_row)
    max_labels = min(epl, voxels)

    ufv = _even_ceil(padded_shape[0]) * _even_ceil(padded_shape[1]) * _even_ceil(padded_shape[2])
    if binary_image:
        if connectivity in (4, 6):
            max_labels = min(max_labels, (ufv // 2) + 1)
        elif connectivity == (8, 18):  # never true, as in fastcc3d.pyx:412
            max_labels = min(max_labels, (ufv // 4) + 1)
        else:
            max_labels = min(max_labels, (ufv // 8) + 1)

    if out_dtype is not None:
        out_dtype = np.dtype(out_dtype)
        if out_dtype not in (np.uint16, np.uint32, np.uint64):
            raise ValueError(
                f"Explicitly defined out_dtype ({out_dtype}) must be one of: "
                f"np.uint16, np.uint32, np.uint64")
        if np.iinfo(out_dtype).max < max_labels:
            raise ValueError(
                f"Explicitly defined out_dtype ({out_dtype}) is too small "
                f"to contain the estimated maximum number of labels ({max_labels}).")
    elif max_labels < np.iinfo(np.uint16).max:
        out_dtype = np.dtype(np.uint16)
    elif max_labels < np.iinfo(np.uint32).max:
        out_dtype = np.dtype(np.uint32)
    else:
        out_dtype = np.dtype(np.uint64)

    special = (delta == 0 and first_row == last_row and first_row >= 0)

    # output buffer: host (numpy / memmap) or device (torch)
    if out_file is not None:
        if isinstance(out_file, str):
            with open(out_file, "wb") as f:
                os.ftruncate(f.fileno(), voxels * out_dtype.itemsize)
        out = np.memmap(out_file, order="F", dtype=out_dtype, shape=(voxels,))
        if special:
            out[:] = 0
        out_ptr, mem_out = out.ctypes.data, 0
    elif on_device:
        maker = torch.zeros if special else torch.empty
        out = maker((voxels,), dtype=_torch_dtype(out_dtype), device=t.device)
        out_ptr, mem_out = nat.dev_ptr(out), nat.OUT_DEVICE
    else:
        out = np.zeros((voxels,), dtype=out_dtype, order="F")
        out_ptr, mem_out = out.ctypes.data, 0

    n = ctypes.c_uint64(0)
    ocode = _OUT_CODE[out_dtype]
    if not special:
        _delta_element(delta, dtype)  # the template argument T delta must hold it
    if special:
        # the Cython layer's single-row loop (fastcc3d.pyx:469-470, 644-679)
        is_u64 = int(np.dtype(dtype) == np.uint64)
        nat.check(call(lib.cc3d_gpu_special_row, ptr, code, is_u64, sx, sy, sz, int(first_row),
                       out_ptr, ocode, ctypes.byref(n), mem_in | mem_out, stream))
    else:
        nat.check(call(lib.cc3d_gpu_label_finish, info.token, int(max_labels), out_ptr, ocode,
                       ctypes.byref(n), mem_out, stream))
    N = int(n.value)

    out = _final_reshape(out, sx, sy, sz, dims, order)
    if is_torch and not isinstance(out, _torch().Tensor):
        out = _torch().from_numpy(np.asarray(out))
    return (out, N) if return_N else out


def _final_reshape(out, sx, sy, sz, dims, order):
    """fastcc3d.pyx:628-642 (for torch: a view with the same memory layout)."""
    if isinstance(out, np.ndarray):
        if dims == 3:
            return out.reshape((sz, sy, sx) if order == "C" else (sx, sy, sz), order=order)
        if dims == 2:
            return out.reshape((sy, sx) if order == "C" else (sx, sy), order=order)
        return out.reshape((sx,), order=order)
    if dims == 3:
        shp = (sz, sy, sx)
    elif dims == 2:
        shp = (sy, sx)
    else:
        shp = (sx,)
    v = out.reshape(shp)
    if order == "F":
        v = v.permute(*reversed(range(v.dim())))
    return v


# ------------------------------------------------------------- statistics
def statistics(out_labels: Any, no_slice_conversion: bool = False) -> dict:
    """Voxel counts, bounding boxes and centroids per label.

    Mirrors cc3d.statistics (cc3d/fastcc3d.pyx:681-938): axes are the array's
    own axes (x = axis 0), counts are uint32, bounding boxes uint16 (uint32
    when an axis exceeds 65535) as (min, max) per axis, centroids float64 with
    NaN for absent labels.  CUDA torch input returns CUDA tensors."""
    on_device = _is_torch(out_labels) and out_labels.is_cuda
    if _is_torch(out_labels) and not on_device:
        out_labels = out_labels.cpu().numpy()
    if on_device:
        torch = _torch()
        t = out_labels
        while t.dim() < 2:
            t = t.unsqueeze(-1)
        npd = _np_dtype_of_torch(t)
        shape = tuple(t.shape)
    else:
        while out_labels.ndim < 2:
            out_labels = out_labels[..., np.newaxis]
        if out_labels.dtype == bool:
            out_labels = out_labels.view(np.uint8)
        npd = out_labels.dtype
        shape = out_labels.shape
    voxels = reduce(operator.mul, shape, 1)
    if voxels == 0:
        return {"voxel_counts": None, "bounding_boxes": None, "centroids": None}
    if len(shape) > 3:
        raise ValueError(f"Buffer has wrong number of dimensions (expected 3, got {len(shape)})")
    if npd == np.bool_:
        npd = np.dtype(np.uint8)
    if not np.issubdtype(npd, np.integer):
        raise TypeError("Function call with ambiguous argument types")
    code = _CODE[np.dtype(npd)]
    signed = np.issubdtype(npd, np.signedinteger)

    if on_device:
        c, f = _contig_flags(t.shape, t.stride())
        if not (c or f):
            t = t.contiguous()
            c, f = True, False
        c_order = 0 if (f and not c) else 1
        ptr, mem = nat.dev_ptr(t), nat.IN_DEVICE | nat.OUT_DEVICE
        stream = ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)
        devctx = torch.cuda.device(t.device)
    else:
        arr = out_labels
        if arr.flags.c_contiguous:
            c_order = 1
        elif arr.flags.f_contiguous:
            c_order = 0
        else:
            arr = np.ascontiguousarray(arr)
            c_order = 1
        ptr, mem, stream = arr.ctypes.data, 0, None
        devctx = None

    lib = nat.load()
    vmax, vmin = ctypes.c_uint64(0), ctypes.c_int64(0)

    def call(fn, *args):
        if devctx is not None:
            with devctx:
                return fn(*args)
        return fn(*args)

    nat.check(call(lib.cc3d_gpu_label_minmax, ptr, code, int(signed), voxels, ctypes.byref(vmax),
                   ctypes.byref(vmin), mem & nat.IN_DEVICE, stream))
    N = int(vmax.value)
    if signed:
        N = int(np.int64(np.uint64(N).view(np.int64)))
    if N > voxels:
        raise ValueError(
            f"Statistics can only be computed on volumes containing labels with values lower than the number of voxels. Max: {N}")
    if signed and vmin.value < 0:
        raise ValueError(
            f"Statistics can only be computed on volumes containing labels with values >= 0. Min: {vmin.value}")

    ndim = len(shape)
    d0, d1 = int(shape[0]), int(shape[1])
    d2 = int(shape[2]) if ndim > 2 else 1
    big = any(s > np.iinfo(np.uint16).max for s in (d0, d1, d2))
    bdt = np.dtype(np.uint32) if big else np.dtype(np.uint16)
    bcode = nat.U32 if big else nat.U16
    if on_device:
        counts = torch.empty((N + 1,), dtype=_torch_dtype(np.uint32), device=t.device)
        bboxes = torch.empty((N + 1, 2 * ndim), dtype=_torch_dtype(bdt), device=t.device)
        cents = torch.empty((N + 1, ndim), dtype=torch.float64, device=t.device)
        pc, pb, pcen = nat.dev_ptr(counts), nat.dev_ptr(bboxes), nat.dev_ptr(cents)
    else:
        counts = np.zeros(N + 1, dtype=np.uint32)
        bboxes = np.zeros((N + 1, 2 * ndim), dtype=bdt)
        cents = np.zeros((N + 1, ndim), dtype=np.float64)
        pc, pb, pcen = counts.ctypes.data, bboxes.ctypes.data, cents.ctypes.data
    nat.check(call(lib.cc3d_gpu_statistics, ptr, code, d0, d1, d2, ndim, c_order, N, pc, pb, bcode,
                   pcen, mem, stream))
    output = {"voxel_counts": counts, "bounding_boxes": bboxes, "centroids": cents}
    if no_slice_conversion:
        return output
    bb = bboxes.cpu().numpy() if on_device else bboxes
    slices = []
    for row in bb:
        starts, ends = row[0::2], row[1::2]
        if all(int(s) < voxels for s in starts):
            slices.append(tuple(slice(int(s), int(e) + 1) for s, e in zip(starts, ends)))
        else:
            slices.append(None)
    output["bounding_boxes"] = slices
    return output
