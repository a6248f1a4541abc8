"""cc3d.connected_components_stack on the GPU (cc3d/__init__.py:324-501).

Connected components of a volume that arrives as a sequence of slabs along
its third axis (numpy axis 2), each of the same width and height.  Every
slab goes to the device and is labelled there as it arrives
(connected_components; its labels stay on the device).  Slab k's labels
become the global labels offset_k + 1 .. offset_k + n_k.  The seams are
merged on the device (csrc/cc3d_stack.cu): a union-find table over all
global labels, one kernel per seam that joins the labels touching across it
(the previous slab's last plane against the new slab's first plane, 6- or
26-connected, equal values or both foreground for binary images), a
numbering pass that gives every group the rank of its smallest label (the
reference's DisjointSet keeps the smaller root; its crackle.renumber numbers
the remapped labels in sorted order), and a relabel that writes each slab's
final labels in place into the whole volume's output on the device.

The reference compresses the result into a crackle array, which needs the
crackle package; here the result is a LabelStack holding the labels (a numpy
array in Fortran order for numpy slabs, a CUDA tensor of the same layout for
CUDA tensor slabs) with the few methods of the crackle array that callers
use (indexing, decompress, num_labels).  Its dtype is the smallest unsigned
type that holds N.
"""
from __future__ import annotations

import ctypes
from typing import Any, Iterable

import numpy as np

from . import _native as nat
from .api import _is_torch, connected_components

F16 = 7  # CC3D_F16 (include/cc3d_gpu.h)


class LabelStack:
    """Labels of a stacked volume behind the interface of the reference's
    crackle array (``arr[...]``, ``decompress()``, ``num_labels()``,
    ``shape``, ``dtype``)."""

    def __init__(self, labels, n: int, has_background: bool):
        self._labels = labels
        self._n = n
        self._bg = has_background

    @property
    def shape(self):
        return tuple(self._labels.shape)

    @property
    def dtype(self):
        return self._labels.dtype

    def __getitem__(self, item):
        return self._labels[item]

    def __array__(self, dtype=None, copy=None):
        arr = self._labels.cpu().numpy() if _is_torch(self._labels) else self._labels
        return arr if dtype is None else arr.astype(dtype)

    def decompress(self):
        return self._labels

    def numpy(self) -> np.ndarray:
        return self.__array__()

    def num_labels(self) -> int:
        """Distinct values, background included (as a crackle array counts them)."""
        return self._n + (1 if self._bg else 0)


def _torch():
    import torch
    return torch


def _img_code(t) -> int:
    torch = _torch()
    if t.dtype == torch.float16:
        return F16
    if t.dtype == torch.float32:
        return nat.F32
    if t.dtype == torch.float64:
        return nat.F64
    return {1: nat.U8, 2: nat.U16, 4: nat.U32, 8: nat.U64}[t.element_size()]


def _img_plane(t):
    """A contiguous (sx, sy) device copy of one z plane; bool as uint8."""
    torch = _torch()
    if t.dtype == torch.bool:
        t = t.view(torch.uint8)
    return t.contiguous()


def _stream():
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def connected_components_stack(stacked_images: Iterable[Any], connectivity: int = 26, return_N: bool = False,
                               binary_image: bool = False):
    """Connected components of the volume the slabs form along axis 2
    (cc3d/__init__.py:324-501); returns a LabelStack (and N)."""
    if connectivity not in (6, 26):
        raise ValueError(f"Connectivity must be 6 or 26. Got: {connectivity}")
    torch = _torch()
    lib = nat.load()
    stream = _stream()
    slabs = []  # (labels on the device, n, first image plane, last image plane)
    xy = None
    host_input = True
    for image in stacked_images:
        if _is_torch(image):
            host_input = host_input and not image.is_cuda
            dev = image if image.is_cuda else image.cuda()
        else:
            image = np.asarray(image)
            dev = torch.from_numpy(image).cuda()
        if dev.dim() != 3:
            raise ValueError(f"stacked images must be 3D. Got: {dev.dim()}D")
        if xy is None:
            xy = tuple(dev.shape[:2])
        elif tuple(dev.shape[:2]) != xy:
            raise ValueError(f"every image needs the same width and height: {tuple(dev.shape[:2])} != {xy}")
        cc, n = connected_components(dev, connectivity=connectivity, return_N=True,
                                     binary_image=bool(binary_image))
        slabs.append((cc, int(n), _img_plane(dev[:, :, 0]), _img_plane(dev[:, :, -1])))
    if not slabs:
        raise ValueError("no images to stack")

    sx, sy = xy
    total = sum(n for _, n, _, _ in slabs)
    work = torch.empty(int(lib.cc3d_gpu_stack_work_bytes(total)), dtype=torch.uint8, device="cuda")
    wp = nat.dev_ptr(work)
    nat.check(lib.cc3d_gpu_stack_begin(wp, total, stream))
    offsets = np.concatenate([[0], np.cumsum([n for _, n, _, _ in slabs])]).astype(np.uint64)
    for k in range(1, len(slabs)):
        bcc, _, _, bimg = slabs[k - 1]
        tcc, _, timg, _ = slabs[k]
        blab = bcc[:, :, -1].contiguous()
        tlab = tcc[:, :, 0].contiguous()
        nat.check(lib.cc3d_gpu_stack_seam(nat.dev_ptr(bimg), nat.dev_ptr(timg), _img_code(timg),
                                          nat.dev_ptr(blab), blab.element_size(), int(offsets[k - 1]),
                                          nat.dev_ptr(tlab), tlab.element_size(), int(offsets[k]),
                                          sx, sy, connectivity, int(bool(binary_image)), wp, total, stream))
    N = ctypes.c_uint64(0)
    nat.check(lib.cc3d_gpu_stack_number(wp, total, ctypes.byref(N), stream))
    N = int(N.value)
    out_np = next(np.dtype(t) for t in (np.uint8, np.uint16, np.uint32, np.uint64) if N <= np.iinfo(t).max)
    width = out_np.itemsize
    depth = sum(int(cc.shape[2]) for cc, _, _, _ in slabs)
    # Fortran order, (sx, sy, depth): x fastest, slabs contiguous
    signed = {1: torch.uint8, 2: torch.int16, 4: torch.int32, 8: torch.int64}[width]
    out = torch.empty((depth, sy, sx), dtype=signed, device="cuda").permute(2, 1, 0)
    ostr = (ctypes.c_int64 * 3)(*out.stride())
    z = 0
    has_bg = False
    for k, (cc, _, _, _) in enumerate(slabs):
        d = int(cc.shape[2])
        dst = out[:, :, z:z + d]
        lstr = (ctypes.c_int64 * 3)(*cc.stride())
        bg = ctypes.c_int(0)
        nat.check(lib.cc3d_gpu_stack_relabel(nat.dev_ptr(cc), cc.element_size(), lstr, int(offsets[k]),
                                             nat.dev_ptr(dst), width, ostr, sx, sy, d, wp, total,
                                             ctypes.byref(bg), stream))
        has_bg = has_bg or bool(bg.value)
        z += d
    if host_input:
        labels = out.cpu().numpy().view(out_np)
    else:
        labels = out if width == 1 else out.view(getattr(torch, out_np.name))
    arr = LabelStack(labels, N, has_bg)
    return (arr, N) if return_N else arr
