"""CPU oracle for the cc3d labelling path.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.

Two interchangeable cores sit under one Python front end that restates the
reference's Cython layer (cc3d/fastcc3d.pyx):

* ``"port"``      -- oracle/cc3d_oracle.c, a plain C restatement of the
                     labelling contract (always available; built by make).
* ``"reference"`` -- oracle/_ref/libcc3d_ref.so, the reference's own C++
                     headers compiled from its source tree by oracle/Makefile
                     (only where that tree exists).

Statistics are restated in numpy (cc3d/fastcc3d.pyx:681-938).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from functools import reduce
import operator

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libcc3d_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libcc3d_ref.so")

DT_CODES = {
    np.dtype(np.uint8): 1, np.dtype(np.uint16): 2, np.dtype(np.uint32): 3,
    np.dtype(np.uint64): 4, np.dtype(np.float32): 5, np.dtype(np.float64): 6,
}


class DimensionError(Exception):
    """The array has the wrong number of dimensions (cc3d/fastcc3d.pyx:123-125)."""


def build(quiet: bool = True) -> None:
    """Compile the oracle (and the reference shim when its sources exist)."""
    kw = dict(stdout=subprocess.DEVNULL, stderr=subprocess.STDOUT) if quiet else {}
    subprocess.run(["make", "-s", "-C", HERE], check=True, **kw)


_LIBS: dict = {}


def have_reference() -> bool:
    return os.path.exists(REF_LIB)


def _lib(kind: str):
    if kind in _LIBS:
        return _LIBS[kind]
    path = PORT_LIB if kind == "port" else REF_LIB
    if not os.path.exists(path):
        if kind == "port":
            build()
        else:
            raise FileNotFoundError(f"reference library not built: {path}")
    lib = ctypes.CDLL(path)
    i64, u64p, i64p = ctypes.c_int64, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int64)
    if kind == "port":
        lib.oracle_connected_components.argtypes = [
            ctypes.c_void_p, ctypes.c_int, i64, i64, i64, i64, ctypes.c_int, ctypes.c_int,
            ctypes.c_int, ctypes.c_void_p, ctypes.c_int, u64p]
        lib.oracle_connected_components.restype = ctypes.c_int
        lib.oracle_epl.argtypes = [ctypes.c_void_p, ctypes.c_int, i64, i64, i64p, i64p]
        lib.oracle_epl.restype = ctypes.c_uint64
        vp = ctypes.c_void_p
        lib.oracle_statistics.argtypes = [vp, ctypes.c_int, i64, i64, i64, ctypes.c_int, ctypes.c_uint64,
                                          vp, vp, vp, vp]
        lib.oracle_statistics.restype = ctypes.c_int
        lib.oracle_connected_components_continuous.argtypes = [
            ctypes.c_void_p, ctypes.c_int, i64, i64, i64, ctypes.c_int, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_int, u64p]
        lib.oracle_connected_components_continuous.restype = ctypes.c_int
    else:
        lib.ref_connected_components_delta.argtypes = [
            ctypes.c_void_p, ctypes.c_int, i64, i64, i64, i64, i64, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_int, u64p]
        lib.ref_connected_components_delta.restype = ctypes.c_int
        lib.ref_connected_components.argtypes = [
            ctypes.c_void_p, ctypes.c_int, i64, i64, i64, i64, i64, ctypes.c_void_p,
            ctypes.c_int, u64p, ctypes.c_int, ctypes.c_int]
        lib.ref_connected_components.restype = ctypes.c_int
        lib.ref_epl.argtypes = [ctypes.c_void_p, ctypes.c_int, i64, i64, i64p, i64p]
        lib.ref_epl.restype = ctypes.c_uint64
    _LIBS[kind] = lib
    return lib


def _core_dtype(dtype: np.dtype) -> np.dtype:
    """The unsigned/float view the reference dispatches on (fastcc3d.pyx:494-608)."""
    dtype = np.dtype(dtype)
    if dtype == bool or dtype in (np.int8, np.uint8):
        return np.dtype(np.uint8)
    if dtype in (np.int16, np.uint16):
        return np.dtype(np.uint16)
    if dtype in (np.int32, np.uint32):
        return np.dtype(np.uint32)
    if dtype in (np.int64, np.uint64):
        return np.dtype(np.uint64)
    if dtype in (np.float32, np.float64):
        return dtype
    raise TypeError(
        f"Type {dtype} is not currently supported. "
        f"Supported: bool, int8, int16, int32, int64, uint8, uint16, uint32, uint64, float16, float32, float64"
    )


def _reshape_flat(arr: np.ndarray) -> np.ndarray:
    """Memory-order flat view (fastcc3d.pyx:128-161 with shape=(size,))."""
    if arr.flags.f_contiguous:
        return arr.reshape(-1, order="F")
    if arr.flags.c_contiguous:
        return arr.reshape(-1, order="C")
    return arr.reshape(-1)


def estimate_provisional_labels(data: np.ndarray, backend: str = "port"):
    """(epl, first_foreground_row, last_foreground_row); fastcc3d.pyx:168-242."""
    sx = data.shape[0] if data.flags.f_contiguous else data.shape[-1]
    linear = _reshape_flat(data)
    cd = _core_dtype(data.dtype) if data.dtype != np.float16 else None
    if cd is None:
        raise TypeError(f"Type {data.dtype} is not currently supported.")
    linear = np.ascontiguousarray(linear.view(cd))
    first, last = ctypes.c_int64(0), ctypes.c_int64(0)
    lib = _lib(backend)
    fn = lib.oracle_epl if backend == "port" else lib.ref_epl
    epl = fn(linear.ctypes.data, DT_CODES[cd], int(sx), int(linear.size),
             ctypes.byref(first), ctypes.byref(last))
    return (int(epl), int(first.value), int(last.value))


def _even_ceil(n: int) -> int:
    return n << 1 if n & 1 else n


def _final_reshape(out, sx, sy, sz, dims, order):
    """fastcc3d.pyx:628-642."""
    if dims == 3:
        return out.reshape((sz, sy, sx) if order == "C" else (sx, sy, sz), order=order)
    if dims == 2:
        return out.reshape((sy, sx) if order == "C" else (sx, sy), order=order)
    return out.reshape((sx,), order=order)


def _special_row(row_values: np.ndarray, out_row: np.ndarray) -> int:
    """Run labelling of a single foreground row (fastcc3d.pyx:644-679).

    The previous value is kept in a C int64: floats are truncated, and values
    that do not fit raise like the reference does."""
    N = 0
    last = 0
    for i, v in enumerate(row_values):
        if v == 0:
            last = 0
            continue
        if v == last:
            out_row[i] = N
            continue
        N += 1
        out_row[i] = N
        if isinstance(v, (np.floating, float)):
            fv = float(v)
            if fv != fv:
                raise ValueError("cannot convert float NaN to integer")
            if fv in (float("inf"), float("-inf")) or not (-2**63 <= int(fv) < 2**63):
                raise OverflowError("Python int too large to convert to C long")
            last = int(fv)
        else:
            iv = int(v)
            if not (-2**63 <= iv < 2**63):
                raise OverflowError("Python int too large to convert to C long")
            last = iv
    return N


def connected_components(data, max_labels=-1, connectivity=26, return_N=False,
                         delta=0, out_dtype=None, out_file=None,
                         periodic_boundary=False, binary_image=False,
                         backend: str = "port"):
    """Restatement of cc3d.connected_components (fastcc3d.pyx:244-626)."""
    is_torch = hasattr(data, "cpu")
    if is_torch:
        data = data.cpu().numpy()
    dims = len(data.shape)
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
    if data.size == 0:
        dtype = out_dtype if out_dtype is not None else data.dtype
        out = np.zeros(shape=(0,), dtype=dtype)
        return (out, 0) if return_N else out

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
    shape = list(data.shape)
    if order == "C":
        shape.reverse()
    sx, sy, sz = shape
    voxels = sx * sy * sz
    dtype = data.dtype
    binary_image = binary_image or (dtype == bool)
    if binary_image:
        epl, first_row, last_row = voxels, 0, sy
    else:
        epl, first_row, last_row = estimate_provisional_labels(data, backend=backend)
    max_labels = min(epl, voxels)
    if np.issubdtype(dtype, np.floating):
        delta = float(delta)
        binary_image = binary_image or (delta == np.finfo(dtype).max)
    else:
        delta = int(delta)
        binary_image = binary_image or (delta == np.iinfo(dtype).max)
    ufv = _even_ceil(data.shape[0]) * _even_ceil(data.shape[1]) * _even_ceil(data.shape[2])
    if binary_image:
        if connectivity in (4, 6):
            max_labels = min(max_labels, (ufv // 2) + 1)
        elif connectivity == (8, 18):  # never true: mirrors fastcc3d.pyx:412
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

    if out_file is None:
        out = np.zeros((voxels,), dtype=out_dtype, order="F")
    else:
        if isinstance(out_file, str):
            with open(out_file, "wb") as f:
                os.ftruncate(f.fileno(), voxels * np.dtype(out_dtype).itemsize)
        out = np.memmap(out_file, order="F", dtype=out_dtype, shape=(voxels,))

    if delta == 0 and first_row == last_row and first_row >= 0:
        rz, ry = divmod(first_row, sy)
        row = data[:, ry, rz] if data.flags.f_contiguous else data[rz, ry, :]
        N = _special_row(row, out[first_row * sx:(first_row + 1) * sx])
    else:
        cd = _core_dtype(dtype)
        flat = np.ascontiguousarray(_reshape_flat(data).view(cd))
        n = ctypes.c_uint64(0)
        odt = DT_CODES[out_dtype]
        lib = _lib(backend)
        dbuf = _delta_bytes(delta, cd)
        if delta != 0 and not binary_image:
            if backend == "port":
                rc = lib.oracle_connected_components_continuous(
                    flat.ctypes.data, DT_CODES[cd], sx, sy, sz, int(connectivity), dbuf,
                    out.ctypes.data, odt, ctypes.byref(n))
            else:
                rc = lib.ref_connected_components_delta(
                    flat.ctypes.data, DT_CODES[cd], sx, sy, sz, int(max_labels), int(connectivity),
                    dbuf, out.ctypes.data, odt, ctypes.byref(n))
        elif backend == "port":
            rc = lib.oracle_connected_components(
                flat.ctypes.data, DT_CODES[cd], sx, sy, sz, int(max_labels), int(connectivity),
                int(bool(binary_image)), int(bool(periodic_boundary)),
                out.ctypes.data, odt, ctypes.byref(n))
        else:
            rc = lib.ref_connected_components(
                flat.ctypes.data, DT_CODES[cd], sx, sy, sz, int(max_labels),
                int(connectivity), out.ctypes.data, odt, ctypes.byref(n),
                int(bool(periodic_boundary)), int(bool(binary_image)))
        if rc == -2 and backend == "port":
            raise RuntimeError("sz must be 1 for 2D connectivities.")
        if rc == -5 or (rc == -2 and backend == "reference"):
            raise RuntimeError("maximum length exception")
        if rc != 0:
            raise RuntimeError(f"oracle failed with code {rc}")
        N = int(n.value)

    out = _final_reshape(out, sx, sy, sz, dims, order)
    if is_torch:
        import torch
        out = torch.from_numpy(out)
    return (out, N) if return_N else out


def _delta_bytes(delta, cd: np.dtype):
    """delta as one element of the labeller's type cd (Cython's conversion at
    the call, cc3d/fastcc3d.pyx:494-608: OverflowError outside an unsigned
    type's range)."""
    cd = np.dtype(cd)
    if cd.kind == "f":
        raw = np.array([delta], dtype=cd).tobytes()
    else:
        d = int(delta)
        name = {1: "uint8_t", 2: "uint16_t", 4: "uint32_t", 8: "uint64_t"}[cd.itemsize]
        if d < 0:
            raise OverflowError(f"can't convert negative value to {name}")
        if d >= 1 << (8 * cd.itemsize):
            raise OverflowError(f"value too large to convert to {name}")
        raw = d.to_bytes(cd.itemsize, "little")
    return ctypes.create_string_buffer(raw, 8)


def statistics(out_labels: np.ndarray, no_slice_conversion: bool = False) -> dict:
    """Restatement of cc3d.statistics (fastcc3d.pyx:681-938): the argument
    checks, output dtypes and slices here, the per-voxel pass in C
    (oracle_statistics, fastcc3d.pyx:767-938)."""
    while out_labels.ndim < 2:
        out_labels = out_labels[..., np.newaxis]
    if out_labels.dtype == bool:
        out_labels = out_labels.view(np.uint8)
    voxels = out_labels.size
    if voxels == 0:
        return {"voxel_counts": None, "bounding_boxes": None, "centroids": None}
    if not (np.issubdtype(out_labels.dtype, np.integer)):
        raise TypeError("Function call with ambiguous argument types")
    N = int(np.max(out_labels))
    if N > voxels:
        raise ValueError(
            f"Statistics can only be computed on volumes containing labels with values lower than the number of voxels. Max: {N}")
    if np.issubdtype(out_labels.dtype, np.signedinteger):
        mn = int(np.min(out_labels))
        if mn < 0:
            raise ValueError(
                f"Statistics can only be computed on volumes containing labels with values >= 0. Min: {mn}")
        out_labels = out_labels.view(f"u{out_labels.dtype.itemsize}")
    ndim = out_labels.ndim
    shape = out_labels.shape
    bdt = np.uint32 if any(s > np.iinfo(np.uint16).max for s in (list(shape) + [1])[:3]) else np.uint16
    # one pass of the C restatement over the buffer in its memory order
    if out_labels.flags.c_contiguous:
        buf, c_order = out_labels, 1
    elif out_labels.flags.f_contiguous:
        buf, c_order = out_labels, 0
    else:
        buf, c_order = np.ascontiguousarray(out_labels), 1
    d0, d1 = int(shape[0]), int(shape[1])
    d2 = int(shape[2]) if ndim > 2 else 1
    counts = np.empty(N + 1, dtype=np.uint32)
    bmin = np.empty((N + 1, 3), dtype=np.uint32)
    bmax_ = np.empty((N + 1, 3), dtype=np.uint32)
    cent3 = np.empty((N + 1, 3), dtype=np.float64)
    rc = _lib("port").oracle_statistics(
        buf.ctypes.data, buf.dtype.itemsize, d0, d1, d2, c_order, N, counts.ctypes.data,
        bmin.ctypes.data, bmax_.ctypes.data, cent3.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"oracle statistics failed with code {rc}")
    bmax = np.iinfo(bdt).max
    bb = np.zeros((N + 1, 2 * ndim), dtype=bdt)
    bb[:, 0::2] = np.minimum(bmin[:, :ndim], bmax).astype(bdt)  # absent labels keep the dtype max
    bb[:, 1::2] = bmax_[:, :ndim].astype(bdt)
    cent = np.ascontiguousarray(cent3[:, :ndim])
    output = {"voxel_counts": counts, "bounding_boxes": bb, "centroids": cent}
    if no_slice_conversion:
        return output
    slices = []
    for row in bb:
        starts = row[0::2]
        ends = row[1::2]
        if all(int(s) < voxels for s in starts):
            slices.append(tuple(slice(int(s), int(e) + 1) for s, e in zip(starts, ends)))
        else:
            slices.append(None)
    output["bounding_boxes"] = slices
    return output


def runs(labels: np.ndarray) -> dict:
    """{label: [(start, end), ...]} in memory order, labels ascending: a
    restatement of extract_runs (cc3d/cc3d_graphs.hpp:470-502) behind
    cc3d.fastcc3d.runs (cc3d/fastcc3d.pyx:1258-1277).  A one-element input is
    recorded whatever its label; an empty one raises like the reference."""
    flat = _reshape_flat(np.asarray(labels))
    if flat.dtype == np.bool_:
        flat = flat.view(np.uint8)
    if flat.dtype not in (np.uint8, np.uint16, np.uint32, np.uint64):
        raise TypeError("Unsupported type: " + str(flat.dtype))
    n = flat.size
    if n == 0:
        raise IndexError("Out of bounds on buffer access (axis 0)")
    if n == 1:
        return {int(flat[0]): [(0, 1)]}
    starts = np.concatenate(([0], np.flatnonzero(flat[1:] != flat[:-1]) + 1))
    ends = np.append(starts[1:], n)
    out: dict = {}
    for lab in np.unique(flat):
        if lab == 0:
            continue
        sel = flat[starts] == lab
        out[int(lab)] = list(zip(starts[sel].tolist(), ends[sel].tolist()))
    return out


# directions (dx, dy, dz) of the voxel connectivity graph's bits, 0-based, as
# laid out in cc3d/cc3d_graphs.hpp:25-29 (2D) and :81-96 (3D)
_VCG_BITS_2D = {(1, 0): 0, (-1, 0): 1, (0, 1): 2, (0, -1): 3, (1, 1): 4, (-1, 1): 5, (1, -1): 6, (-1, -1): 7}
_VCG_BITS_3D = {
    (1, 0, 0): 0, (-1, 0, 0): 1, (0, 1, 0): 2, (0, -1, 0): 3, (0, 0, 1): 4, (0, 0, -1): 5,
    (1, 1, 0): 6, (-1, 1, 0): 7, (1, -1, 0): 8, (-1, -1, 0): 9,
    (1, 0, 1): 10, (-1, 0, 1): 11, (0, 1, 1): 12, (0, -1, 1): 13,
    (1, 0, -1): 14, (-1, 0, -1): 15, (0, 1, -1): 16, (0, -1, -1): 17,
    (1, 1, 1): 18, (-1, 1, 1): 19, (1, -1, 1): 20, (-1, -1, 1): 21,
    (1, 1, -1): 22, (-1, 1, -1): 23, (1, -1, -1): 24, (-1, -1, -1): 25}


def voxel_connectivity_graph(data: np.ndarray, connectivity: int = 26) -> np.ndarray:
    """numpy restatement of cc3d.voxel_connectivity_graph
    (cc3d/fastcc3d.pyx:1021-1178, extract_voxel_connectivity_graph in
    cc3d/cc3d_graphs.hpp:31-240): every bit starts set; for each pair of
    neighbouring voxels (axes: x = numpy axis 0) with different labels both
    ends lose the bit pointing at the other; the field is then masked to the
    connectivity (18: 0x3ffff, 6: 0x3f, 4: 0x0f)."""
    dims = data.ndim
    if dims not in (1, 2, 3):
        raise DimensionError("Only 1D, 2D, and 3D arrays supported. Got: " + str(dims))
    if dims == 2 and connectivity not in (4, 8, 6, 18, 26):
        raise ValueError("Only 4, 8, and 6, 18, 26 connectivities are supported for 2D images. Got: "
                         + str(connectivity))
    elif dims != 2 and connectivity not in (6, 18, 26):
        raise ValueError("Only 6, 18, and 26 connectivities are supported for 3D images. Got: "
                         + str(connectivity))
    out_dtype = np.uint8 if connectivity in (4, 8, 6) else np.uint32
    if data.size == 0:
        return np.zeros(shape=(0,), dtype=out_dtype)
    if data.dtype not in (np.bool_, np.uint8, np.int8, np.uint16, np.int16, np.uint32, np.int32,
                          np.uint64, np.int64):
        raise TypeError("Type {} not currently supported.".format(data.dtype))
    shape = data.shape
    a = data.reshape(shape + (1,) * (3 - dims))
    two_d = connectivity in (4, 8)
    table = _VCG_BITS_2D if two_d else _VCG_BITS_3D
    g = np.full(a.shape, 0xFF if two_d else 0x3FFFFFF, dtype=np.uint64)

    for d, bit in table.items():
        dx, dy, dz = (d + (0,)) if two_d else d
        # a voxel at p and its neighbour at p + d, both inside the volume
        nb = a[slice(max(0, dx), a.shape[0] + min(0, dx)), slice(max(0, dy), a.shape[1] + min(0, dy)),
               slice(max(0, dz), a.shape[2] + min(0, dz))]
        cur_sl = (slice(max(0, -dx), a.shape[0] - max(0, dx)), slice(max(0, -dy), a.shape[1] - max(0, dy)),
                  slice(max(0, -dz), a.shape[2] - max(0, dz)))
        differ = a[cur_sl] != nb
        g[cur_sl] &= ~(differ.astype(np.uint64) << np.uint64(bit))
    mask = {26: 0x3FFFFFF, 18: 0x3FFFF, 6: 0x3F, 8: 0xFF, 4: 0x0F}[connectivity]
    g &= np.uint64(mask)
    return np.asfortranarray(g.astype(out_dtype)).reshape(shape, order="F")


def color_connectivity_graph(vcg: np.ndarray, connectivity: int = 26, return_N: bool = False):
    """Restatement of cc3d.color_connectivity_graph (cc3d/fastcc3d.pyx:941-1019,
    color_connectivity_graph_N and its labellers in
    cc3d/cc3d_graphs.hpp:558-1105): every voxel is a node; a voxel joins each
    backward neighbour inside the volume whose direction bit it has set (the
    2D layout for a single plane: 4-connected for 4/6, 8-connected for 8/26;
    the 3D layout otherwise, 6 or 26 directions); components are numbered
    1..N in raster order (x = numpy axis 0 fastest) of their first voxel, as
    the reference's simplified relabel does.  The components come from
    scipy's graph search over those edges."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import connected_components as graph_components
    dims = vcg.ndim
    if dims not in (2, 3):
        raise DimensionError("Only 2D, and 3D arrays supported. Got: " + str(dims))
    if dims == 2 and connectivity not in [4, 8, 6, 26]:
        raise ValueError(f"Only 4 and 8 connectivity is supported for 2D images. Got: {connectivity}")
    elif dims != 2 and connectivity not in [6, 26]:
        raise ValueError(f"Only 6 and 26 connectivity are supported for 3D images. Got: {connectivity}")
    if vcg.dtype not in [np.uint8, np.uint32]:
        raise ValueError(f"Only uint8 and uint32 are supported. Got: {vcg.dtype}")
    if vcg.size == 0:
        out = np.zeros([0] * dims, dtype=np.uint32, order="F")
        return (out, 0) if return_N else out
    shape = vcg.shape
    v = vcg.reshape(shape + (1,) * (3 - dims)).astype(np.uint64)
    sx, sy, sz = v.shape
    if connectivity in [18, 26] and sz > 1 and vcg.dtype != np.uint32:
        raise ValueError(f"Only uint32 is supported for 18 and 26 connected. Got: {vcg.dtype}")
    if sz == 1:
        # one plane: uint8 graphs use the 2D layout, uint32 graphs the 3D one
        # (the two color_connectivity_graph_8 overloads, cc3d/cc3d_graphs.hpp:831-1017)
        dirs = [(-1, 0, 0), (0, -1, 0)] if connectivity in (4, 6) else [(-1, 0, 0), (-1, -1, 0), (0, -1, 0), (1, -1, 0)]
        bit = {d: (_VCG_BITS_3D[d] if vcg.dtype == np.uint32 else _VCG_BITS_2D[d[:2]]) for d in dirs}
    else:
        if connectivity == 6:
            dirs = [(-1, 0, 0), (0, -1, 0), (0, 0, -1)]
        else:
            dirs = [d for d in _VCG_BITS_3D if d[2] < 0 or (d[2] == 0 and (d[1] < 0 or (d[1] == 0 and d[0] < 0)))]
        bit = {d: _VCG_BITS_3D[d] for d in dirs}
    idx = np.arange(sx * sy * sz, dtype=np.int64).reshape((sx, sy, sz), order="F")
    rows, cols = [], []
    for d in dirs:
        dx, dy, dz = d
        cur = (slice(max(0, -dx), sx - max(0, dx)), slice(max(0, -dy), sy - max(0, dy)),
               slice(max(0, -dz), sz - max(0, dz)))
        nb = (slice(max(0, dx), sx + min(0, dx)), slice(max(0, dy), sy + min(0, dy)),
              slice(max(0, dz), sz + min(0, dz)))
        on = ((v[cur] >> np.uint64(bit[d])) & np.uint64(1)).astype(bool)
        rows.append(idx[cur][on])
        cols.append(idx[nb][on])
    n = sx * sy * sz
    r = np.concatenate(rows) if rows else np.zeros(0, np.int64)
    c = np.concatenate(cols) if cols else np.zeros(0, np.int64)
    g = sp.coo_matrix((np.ones(r.size, np.int8), (r, c)), shape=(n, n))
    ncomp, comp = graph_components(g, directed=False)
    # number components by their first voxel in raster order (index order)
    _, first = np.unique(comp, return_index=True)
    rank = np.empty(ncomp, dtype=np.int64)
    rank[np.argsort(first)] = np.arange(ncomp)
    flat = (rank[comp] + 1).astype(np.uint32)
    out = flat.reshape((sx, sy, sz), order="F")
    while out.ndim > dims:
        out = out[..., 0]
    return (out, int(ncomp)) if return_N else out


def _stack_seam_pairs(bottom_img, bottom_lab, top_img, top_lab, connectivity: int, binary_image: bool):
    """(bottom label, top label) pairs joined across one seam: the reference's
    seam loops (cc3d/__init__.py:425-463) as array operations.  For 26 the
    reference skips a voxel's diagonals once the voxel straight above joins;
    those diagonals join top voxels already joined to that one, so every
    offset can be taken."""
    sx, sy = bottom_img.shape
    offs = [(0, 0)] if connectivity == 6 else [(dx, dy) for dx in (-1, 0, 1) for dy in (-1, 0, 1)]
    pairs = []
    for dx, dy in offs:
        bx = slice(max(0, -dx), sx - max(0, dx))
        by = slice(max(0, -dy), sy - max(0, dy))
        tx = slice(max(0, dx), sx + min(0, dx))
        ty = slice(max(0, dy), sy + min(0, dy))
        bl, tl = bottom_lab[bx, by], top_lab[tx, ty]
        bi, ti = bottom_img[bx, by], top_img[tx, ty]
        rel = (bi != 0) & (ti != 0) if binary_image else (bi == ti)
        m = (bl != 0) & (tl != 0) & rel
        if m.any():
            pairs.append(np.stack([bl[m], tl[m]], axis=1))
    return np.concatenate(pairs) if pairs else np.zeros((0, 2), np.uint64)


def connected_components_stack(stacked_images, connectivity: int = 26, return_N: bool = False,
                               binary_image: bool = False):
    """Restatement of cc3d.connected_components_stack (cc3d/__init__.py:324-501)
    on the CPU: every slab labelled by this oracle with uint64 labels offset by
    the slabs before it, seam pairs joined in a disjoint set whose root is the
    smallest label (cc3d/__init__.py:296-321), and the groups numbered 1..N in
    increasing order of their smallest label (crackle.renumber of the sorted
    labels).  Returns (labels in Fortran order, N, has_background) -- the
    crackle array itself is not restated."""
    if connectivity not in (6, 26):
        raise ValueError(f"Connectivity must be 6 or 26. Got: {connectivity}")
    slabs, pairs = [], []
    offset = 0
    prev_img = prev_lab = None
    for image in stacked_images:
        image = np.asarray(image)
        cc, n = connected_components(image, connectivity=connectivity, return_N=True, out_dtype=np.uint64,
                                     binary_image=bool(binary_image))
        cc = np.asarray(cc)
        if offset:
            np.add(cc, np.uint64(offset), out=cc, where=(cc != 0))
        if prev_img is not None:
            pairs.append(_stack_seam_pairs(prev_img, prev_lab, image[:, :, 0], cc[:, :, 0], connectivity,
                                           bool(binary_image)))
        offset += int(n)
        slabs.append(cc)
        prev_img, prev_lab = image[:, :, -1], cc[:, :, -1]
    if not slabs:
        raise ValueError("no images to stack")
    rep = np.arange(offset + 1, dtype=np.uint64)
    allp = np.concatenate(pairs) if pairs else np.zeros((0, 2), np.uint64)
    if len(allp):
        import scipy.sparse as sp
        from scipy.sparse.csgraph import connected_components as graph_components
        nodes, inv = np.unique(allp.reshape(-1), return_inverse=True)
        inv = inv.reshape(-1, 2)
        g = sp.coo_matrix((np.ones(len(inv), np.int8), (inv[:, 0], inv[:, 1])), shape=(len(nodes), len(nodes)))
        ncomp, comp = graph_components(g, directed=False)
        smallest = np.full(ncomp, np.iinfo(np.uint64).max, dtype=np.uint64)
        np.minimum.at(smallest, comp, nodes)
        rep[nodes.astype(np.int64)] = smallest[comp]
    uniq = np.unique(rep[1:])
    N = int(len(uniq))
    table = np.zeros(offset + 1, dtype=np.uint64)
    table[1:] = np.searchsorted(uniq, rep[1:]) + 1
    out_dtype = next(np.dtype(t) for t in (np.uint8, np.uint16, np.uint32, np.uint64) if N <= np.iinfo(t).max)
    table = table.astype(out_dtype)
    depth = sum(s.shape[2] for s in slabs)
    out = np.empty(slabs[0].shape[:2] + (depth,), dtype=out_dtype, order="F")
    z = 0
    has_bg = False
    for cc in slabs:
        d = cc.shape[2]
        out[:, :, z:z + d] = table[cc.astype(np.int64)]
        has_bg = has_bg or bool((cc == 0).any())
        z += d
    return (out, N, has_bg) if return_N else out
