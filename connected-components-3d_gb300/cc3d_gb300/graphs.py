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
        nat.check(lib.cc3d_gpu_contacts(dev.data_ptr(), width, sx, sy, sz, int(connectivity), ctypes.byref(n),
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
        nat.check(lib.cc3d_gpu_run_starts(dev.data_ptr(), width, n, ctypes.byref(cnt),
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
