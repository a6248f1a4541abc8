"""cc3d.contacts, cc3d.region_graph, cc3d.runs, cc3d.draw and cc3d.each on
the GPU (cc3d/fastcc3d.pyx:1180-1372).

The contacts of every pair of touching labels are counted on the device by
cc3d_gpu_contacts, with the reference's neighbourhood (including its handling
of the volume's faces); the counts are turned into the reference's areas here.
Areas with integer values (unit or integer anisotropy, or voxel counts) are
exactly the reference's float32 sums; others agree within float32 rounding of
a sum taken in another order.  Axes follow the reference: numpy axis 0 is x.
"""
from __future__ import annotations

import ctypes
from typing import Any, Dict, Tuple

import numpy as np

from . import _native as nat
from .api import _is_torch


def contacts(labels: Any, connectivity: int = 26, surface_area: bool = True,
             anisotropy=(1, 1, 1)) -> Dict[Tuple[int, int], float]:
    """{(label_1, label_2): contact area (or count of neighbouring voxels)}."""
    import torch
    if _is_torch(labels):
        t = labels
        while t.dim() < 3:
            t = t.unsqueeze(-1)
        dev = t.permute(*reversed(range(t.dim()))).contiguous()  # x fastest in memory
        if not dev.is_cuda:
            dev = dev.cuda()
        sx, sy, sz = (int(v) for v in t.shape)
        width = t.element_size()
        if t.is_floating_point():
            raise TypeError("contacts needs integer labels")
    else:
        a = np.asarray(labels)
        while a.ndim < 3:
            a = a[..., np.newaxis]
        if a.dtype.kind not in "uib":
            raise TypeError("contacts needs integer labels")
        f = np.asfortranarray(a)
        sx, sy, sz = (int(v) for v in f.shape)
        width = f.dtype.itemsize
        dev = torch.from_numpy(np.ravel(f, order="K").view(np.uint8)).cuda()
    while len(anisotropy) < 3:
        anisotropy = tuple(anisotropy) + (1,)
    if connectivity not in (4, 8, 6, 18, 26):
        raise ValueError(f"Only (2d) 4, 8, (3d) 6, 18, and 26 connectivities are supported. Got: {connectivity}")
    lib = nat.load()
    n = ctypes.c_uint64(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    with torch.cuda.device(dev.device):
        nat.check(lib.cc3d_gpu_contacts(nat.dev_ptr(dev), width, sx, sy, sz, int(connectivity), ctypes.byref(n),
                                        stream))
    npairs = int(n.value)
    if npairs == 0:
        return {}
    pairs = np.empty(npairs, np.uint64)
    counts = np.empty((npairs, 4), np.uint32)
    nat.check(lib.cc3d_gpu_contacts_copy(pairs.ctypes.data, counts.ctypes.data, npairs))
    wx, wy, wz = (float(v) for v in anisotropy[:3])
    if not surface_area:
        area = np.ones(4)
    elif connectivity in (4, 8):
        area = np.array([np.float32(wy), np.float32(wx), 0.0, 0.0])
    else:
        area = np.array([np.float32(np.float32(wy) * np.float32(wz)), np.float32(np.float32(wx) * np.float32(wz)),
                         np.float32(np.float32(wx) * np.float32(wy)), 0.0])
    vals = (counts.astype(np.float64) @ area).astype(np.float32)
    lo = (pairs >> np.uint64(32)).tolist()
    hi = (pairs & np.uint64(0xFFFFFFFF)).tolist()
    return {(a, b): float(v) for a, b, v in zip(lo, hi, vals.tolist())}


def region_graph(labels: Any, connectivity: int = 26) -> set:
    """The set of (label_1, label_2) pairs of touching labels."""
    return set(contacts(labels, connectivity=connectivity).keys())


def _flat_memory_order(labels):
    """(flat CUDA byte tensor in memory order, element width, element count)."""
    import torch
    if _is_torch(labels):
        t = labels
        if not t.is_contiguous():
            t = t.permute(*reversed(range(t.dim()))).contiguous()
        if not t.is_cuda:
            t = t.cuda()
        return t.reshape(-1).view(torch.uint8), t.element_size(), t.numel()
    a = np.asarray(labels)
    flat = a.reshape(-1, order="F" if a.flags.f_contiguous and not a.flags.c_contiguous else "C")
    flat = np.ascontiguousarray(flat)
    return torch.from_numpy(flat.view(np.uint8)).cuda(), flat.dtype.itemsize, flat.size


def runs(labels: Any) -> Dict[int, list]:
    """{label: [(start, end), ...]}: the runs of each nonzero label in memory
    order, labels ascending (cc3d/fastcc3d.pyx:1258-1277)."""
    import torch
    if not _is_torch(labels):
        labels = np.asarray(labels)
        if labels.dtype not in (np.uint8, np.uint16, np.uint32, np.uint64, np.bool_):
            raise TypeError("Unsupported type: " + str(labels.dtype))
    dev, width, n = _flat_memory_order(labels)
    if n == 0:  # the reference indexes the first element of the buffer
        raise IndexError("Out of bounds on buffer access (axis 0)")
    lib = nat.load()
    cnt = ctypes.c_uint64(0)
    with torch.cuda.device(dev.device):
        nat.check(lib.cc3d_gpu_run_starts(nat.dev_ptr(dev), width, n, ctypes.byref(cnt),
                                          ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    m = int(cnt.value)
    pos = np.empty(m, np.uint64)
    lab = np.empty(m, np.uint64)
    nat.check(lib.cc3d_gpu_run_starts_copy(pos.ctypes.data, lab.ctypes.data, m))
    if n == 1:  # the reference records the single element whatever its label
        return {int(lab[0]): [(0, 1)]}
    ends = np.append(pos[1:], np.uint64(n))
    keep = lab != 0
    pos, ends, lab = pos[keep], ends[keep], lab[keep]
    order = np.argsort(lab, kind="stable")
    pos, ends, lab = pos[order].tolist(), ends[order].tolist(), lab[order]
    out: Dict[int, list] = {}
    if len(lab) == 0:
        return out
    cut = np.flatnonzero(np.diff(lab)) + 1
    bounds = [0] + cut.tolist() + [len(lab)]
    for a, b in zip(bounds[:-1], bounds[1:]):
        out[int(lab[a])] = list(zip(pos[a:b], ends[a:b]))
    return out


def draw(label, runs_of_label, image: np.ndarray) -> np.ndarray:
    """Write `label` over the runs of a label (memory order) in `image`
    (cc3d/fastcc3d.pyx:1279-1308, set_run_voxels in
    cc3d/cc3d_graphs.hpp:505-523); bool images get label != 0.  As in the
    reference, an image that is neither C- nor F-contiguous is written through
    a copy (so it is returned unchanged) and an invalid run raises after the
    runs before it were drawn."""
    if image.dtype not in (np.bool_, np.uint8, np.uint16, np.uint32, np.uint64):
        raise TypeError("Unsupported type: " + str(image.dtype))
    if image.flags.f_contiguous:
        flat = image.reshape(-1, order="F")
    elif image.flags.c_contiguous:
        flat = image.reshape(-1, order="C")
    else:
        flat = image.reshape(-1)
    value = (label != 0) if image.dtype == bool else label
    n = flat.size
    for a, b in runs_of_label:
        if b > n or a >= b:
            raise RuntimeError("Invalid run.")
        flat[a:b] = value
    return image


def each(labels: np.ndarray, binary: bool = False, in_place: bool = False):
    """Iterator of (label, image of that label alone) over the nonzero labels
    (cc3d/fastcc3d.pyx:1322-1372); the runs come from the GPU."""
    all_runs = runs(labels)
    order = "F" if labels.flags["F_CONTIGUOUS"] else "C"
    dtype = bool if binary else labels.dtype

    class ImageIterator:
        def __len__(self):
            return len(all_runs) - int(0 in all_runs)

        def __iter__(self):
            for key, rns in all_runs.items():
                if key == 0:
                    continue
                img = np.zeros(labels.shape, dtype=dtype, order=order)
                draw(key, rns, img)
                yield (key, img)

    class InPlaceImageIterator(ImageIterator):
        def __iter__(self):
            img = np.zeros(labels.shape, dtype=dtype, order=order)
            for key, rns in all_runs.items():
                if key == 0:
                    continue
                draw(key, rns, img)
                img.setflags(write=0)
                yield (key, img)
                img.setflags(write=1)
                draw(0, rns, img)

    return InPlaceImageIterator() if in_place else ImageIterator()


_VCG_INPUT = {np.dtype(np.bool_): 1, np.dtype(np.uint8): 1, np.dtype(np.int8): 1, np.dtype(np.uint16): 2,
              np.dtype(np.int16): 2, np.dtype(np.uint32): 4, np.dtype(np.int32): 4, np.dtype(np.uint64): 8,
              np.dtype(np.int64): 8}


def _f_order_device(data):
    """(flat CUDA tensor of `data` in F order -- axis 0 fastest --, numpy dtype, shape)."""
    import torch
    if _is_torch(data):
        t = data if data.is_cuda else data.cuda()
        npd = np.dtype(str(t.dtype).replace("torch.", ""))
        flat = t.permute(*reversed(range(t.dim()))).contiguous().reshape(-1)
        return flat, npd, tuple(t.shape)
    a = np.asarray(data)
    flat = np.asfortranarray(a).reshape(-1, order="F")
    return torch.from_numpy(np.ascontiguousarray(flat)).cuda(), a.dtype, a.shape


def _from_f_order(flat, shape, like_torch: bool):
    """A flat F-ordered CUDA tensor back as an array of `shape` (numpy F order,
    or a CUDA tensor view with F strides)."""
    if like_torch:
        return flat.view(*reversed(shape)).permute(*reversed(range(len(shape))))
    return flat.cpu().numpy().reshape(shape, order="F")


def voxel_connectivity_graph(data: Any, connectivity: int = 26):
    """Bitfield of the directions in which each voxel's neighbour has the same
    label (cc3d/fastcc3d.pyx:1021-1178; cc3d/cc3d_graphs.hpp:31-240): uint8
    for 4, 8 and 6-connectivity, uint32 for 18 and 26.  Axes are the array's
    own (x = axis 0), as in the reference; a bit stays set at the volume's
    faces.  CUDA tensors give CUDA tensors."""
    from .api import DimensionError
    import torch
    dims = len(data.shape)
    if dims not in (1, 2, 3):
        raise DimensionError("Only 1D, 2D, and 3D arrays supported. Got: " + str(dims))
    if dims == 2 and connectivity not in (4, 8, 6, 18, 26):
        raise ValueError("Only 4, 8, and 6, 18, 26 connectivities are supported for 2D images. Got: "
                         + str(connectivity))
    elif dims != 2 and connectivity not in (6, 18, 26):
        raise ValueError("Only 6, 18, and 26 connectivities are supported for 3D images. Got: "
                         + str(connectivity))
    out_dtype = np.dtype(np.uint8) if connectivity in (4, 8, 6) else np.dtype(np.uint32)
    is_t = _is_torch(data)
    n = int(np.prod(data.shape))
    if n == 0:
        if is_t:
            return torch.zeros((0,), dtype=getattr(torch, out_dtype.name), device=data.device)
        return np.zeros(shape=(0,), dtype=out_dtype)
    npd = np.dtype(str(data.dtype).replace("torch.", "")) if is_t else np.asarray(data).dtype
    if npd not in _VCG_INPUT:
        raise TypeError("Type {} not currently supported.".format(npd))
    shape = tuple(int(v) for v in data.shape)
    # C-ordered arrays are read in place with the axes reversed (the kernel
    # maps memory offsets back to the reference's x = axis 0); anything else
    # goes through a Fortran-ordered copy
    if is_t:
        t = data if data.is_cuda else data.cuda()
        rev = dims > 1 and t.is_contiguous()
        flat = t.reshape(-1) if rev else t.permute(*reversed(range(dims))).contiguous().reshape(-1)
    else:
        a = np.asarray(data)
        rev = dims > 1 and a.flags.c_contiguous and not a.flags.f_contiguous
        host = np.ascontiguousarray(a).reshape(-1) if rev else np.asfortranarray(a).reshape(-1, order="F")
        flat = torch.from_numpy(np.ascontiguousarray(host)).cuda()
    ext = tuple(reversed(shape)) if rev else shape
    sx, sy, sz = (int(v) for v in ext + (1,) * (3 - dims))
    width = _VCG_INPUT[npd]  # labels compare as unsigned integers of this width
    out = torch.empty((n,), dtype=getattr(torch, out_dtype.name), device=flat.device)
    lib = nat.load()
    with torch.cuda.device(flat.device):
        nat.check(lib.cc3d_gpu_voxel_connectivity_graph(
            nat.dev_ptr(flat), width, sx, sy, sz, int(connectivity), dims if rev else 0, nat.dev_ptr(out),
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    if rev:
        res = out.view(*shape) if is_t else np.asfortranarray(out.cpu().numpy().reshape(shape))
    else:
        res = _from_f_order(out, shape, is_t)
    # CPU tensors in, CPU tensors out (as connected_components does)
    return res.cpu() if is_t and not data.is_cuda else res


def color_connectivity_graph(vcg: Any, connectivity: int = 26, return_N: bool = False):
    """Connected components of a voxel connectivity graph (uint8 or uint32
    bitfields in the layout voxel_connectivity_graph produces), as uint32
    labels 1..N; every voxel is a node and joins a backward neighbour where its
    own bit says so.  Mirrors cc3d.color_connectivity_graph
    (cc3d/fastcc3d.pyx:941-1019; cc3d/cc3d_graphs.hpp:558-1105), including
    its argument errors and its use of the 2D bit layout for a single plane.
    CUDA tensors give CUDA tensors."""
    from .api import DimensionError
    import torch
    dims = len(vcg.shape)
    if dims not in (2, 3):
        raise DimensionError("Only 2D, and 3D arrays supported. Got: " + str(dims))
    if dims == 2 and connectivity not in [4, 8, 6, 26]:
        raise ValueError(f"Only 4 and 8 connectivity is supported for 2D images. Got: {connectivity}")
    elif dims != 2 and connectivity not in [6, 26]:
        raise ValueError(f"Only 6 and 26 connectivity are supported for 3D images. Got: {connectivity}")
    is_t = _is_torch(vcg)
    npd = np.dtype(str(vcg.dtype).replace("torch.", "")) if is_t else np.asarray(vcg).dtype
    if npd not in [np.uint8, np.uint32]:
        raise ValueError(f"Only uint8 and uint32 are supported. Got: {npd}")
    n = int(np.prod(vcg.shape))
    if n == 0:
        if is_t:
            out = torch.zeros([0] * dims, dtype=torch.uint32, device=vcg.device)
        else:
            out = np.zeros([0] * dims, dtype=np.uint32, order="F")
        return (out, 0) if return_N else out
    shape3 = tuple(vcg.shape) + (1,) * (3 - dims)
    sx, sy, sz = (int(v) for v in shape3)
    if connectivity in [18, 26] and sz > 1 and npd != np.uint32:
        raise ValueError(f"Only uint32 is supported for 18 and 26 connected. Got: {npd}")
    flat, _, shape = _f_order_device(vcg)
    lib = nat.load()
    out = torch.empty((n,), dtype=torch.uint32, device=flat.device)
    cnt = ctypes.c_uint64(0)
    with torch.cuda.device(flat.device):
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        info = nat.Prepared()
        nat.check(lib.cc3d_gpu_label_prepare_graph(nat.dev_ptr(flat), nat.U8 if npd == np.uint8 else nat.U32,
                                                   sx, sy, sz, int(connectivity),
                                                   nat.IN_DEVICE | nat.OUT_DEVICE, stream, ctypes.byref(info)))
        nat.check(lib.cc3d_gpu_label_finish(info.token, n, nat.dev_ptr(out), nat.U32, ctypes.byref(cnt),
                                            nat.OUT_DEVICE, stream))
    labels = _from_f_order(out, tuple(shape), is_t)
    if is_t and not vcg.is_cuda:
        labels = labels.cpu()
    N = int(cnt.value)
    return (labels, N) if return_N else labels
