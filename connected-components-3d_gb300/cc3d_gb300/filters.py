"""cc3d.dust and cc3d.largest_k on the GPU (cc3d/__init__.py:71-155, 199-279).

Same signatures, results, dtypes and return forms as the reference.  The
labelling and the voxel counts run on the device (connected_components,
statistics); the per-label decisions are made on the count table with the
same numpy calls the reference makes (so ties break the same way); the
voxel-wise rewrite is cc3d_gpu_zero_labels / cc3d_gpu_remap_labels.  numpy
inputs give numpy outputs, CUDA tensors give CUDA tensors.
"""
from __future__ import annotations

import ctypes
from typing import Any

import numpy as np

from . import _native as nat
from .api import _is_torch, connected_components, statistics

_UNSIGNED_VIEW = {np.dtype(np.int8): np.uint8, np.dtype(np.int16): np.uint16,
                  np.dtype(np.int32): np.uint32, np.dtype(np.int64): np.uint64}


def _torch():
    import torch
    return torch


def _np_dtype(x) -> np.dtype:
    if _is_torch(x):
        return np.dtype(str(x.dtype).replace("torch.", ""))
    return x.dtype


def _view_as_unsigned(img):
    """cc3d/__init__.py:280-292: signed integers viewed as the unsigned type of the same width."""
    dt = _np_dtype(img)
    if dt in _UNSIGNED_VIEW:
        if _is_torch(img):
            return img.view(getattr(_torch(), np.dtype(_UNSIGNED_VIEW[dt]).name))
        return img.view(_UNSIGNED_VIEW[dt])
    return img


def _flat_device(x):
    """A flat CUDA byte tensor of x's elements in logical (C) order."""
    torch = _torch()
    if _is_torch(x):
        t = x.contiguous().view(-1)
        if not t.is_cuda:
            t = t.cuda()
        return t.view(torch.uint8)
    a = np.ascontiguousarray(np.asarray(x)).reshape(-1)
    return torch.from_numpy(a.view(np.uint8)).cuda()


def _max_int(x) -> int:
    """Largest element of a labels array or tensor (0 if empty)."""
    if not _is_torch(x):
        return int(np.max(x)) if x.size else 0
    torch = _torch()
    if x.numel() == 0:
        return 0
    if x.dtype in (torch.uint8, torch.bool) or x.is_floating_point() or not str(x.dtype).startswith("torch.uint"):
        return int(x.max())
    signed = {2: torch.int16, 4: torch.int32, 8: torch.int64}[x.element_size()]
    wide = x.view(signed).to(torch.int64)
    if x.element_size() < 8:
        wide = wide & ((1 << (8 * x.element_size())) - 1)
    return int(wide.max())


def _stream():
    torch = _torch()
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _counts_host(cc_labels, N: int) -> np.ndarray:
    cts = statistics(cc_labels, no_slice_conversion=True)["voxel_counts"]
    return cts.cpu().numpy() if _is_torch(cts) else np.asarray(cts)


def dust(img: Any, threshold, connectivity: int = 26, in_place: bool = False, binary_image: bool = False,
         precomputed_ccl: bool = False, invert: bool = False, return_N: bool = False):
    """Remove connected components smaller than `threshold` voxels (or, for a
    (lower, upper) pair, outside [lower, upper)); `invert` keeps them instead.
    Mirrors cc3d.dust (cc3d/__init__.py:71-155), including its return dtype:
    the input's, or its unsigned view when nothing was removed."""
    torch = _torch() if _is_torch(img) else None
    orig_dtype = _np_dtype(img)
    img = _view_as_unsigned(img)
    if not in_place:
        img = img.clone() if torch is not None else np.copy(img)
    if precomputed_ccl:
        cc_labels = img
        N = _max_int(img)
    else:
        cc_labels, N = connected_components(img, connectivity=connectivity, return_N=True,
                                            binary_image=bool(binary_image))
    mask_sizes = _counts_host(cc_labels, N)
    sizes = mask_sizes[1:N + 1]
    if isinstance(threshold, (tuple, list)):
        in_mask = ~((threshold[0] <= sizes) & (sizes < threshold[1]))
    else:
        in_mask = sizes < threshold
    n_mask = int(in_mask.sum())
    dust_N = n_mask if invert else N - n_mask

    if n_mask == 0:
        if invert:
            if torch is not None:
                img = torch.zeros_like(img)
            else:
                img = np.zeros(img.shape, dtype=img.dtype, order="F")
        return (img, dust_N) if return_N else img

    # label -> zero this voxel?  (np.isin(cc_labels, to_mask, invert=invert))
    zero = np.zeros(N + 1, dtype=np.uint8)
    zero[1:] = (~in_mask if invert else in_mask).astype(np.uint8)
    zero[0] = 1 if invert else 0
    _zero_labels(img, cc_labels, zero)
    img = img.view(getattr(torch, orig_dtype.name)) if torch is not None else img.view(orig_dtype)
    return (img, dust_N) if return_N else img


def _zero_labels(img, cc_labels, zero: np.ndarray) -> None:
    """img[voxel] = 0 where zero[cc_labels[voxel]], in place (logical voxel order)."""
    torch = _torch()
    lib = nat.load()
    lab = _flat_device(cc_labels)
    ztab = torch.from_numpy(zero).cuda()
    lab_bytes = cc_labels.element_size() if _is_torch(cc_labels) else cc_labels.dtype.itemsize
    img_bytes = img.element_size() if _is_torch(img) else img.dtype.itemsize
    n = img.numel() if _is_torch(img) else img.size
    in_place = _is_torch(img) and img.is_cuda and img.is_contiguous()
    target = img.view(-1).view(torch.uint8) if in_place else _flat_device(img)
    nat.check(lib.cc3d_gpu_zero_labels(nat.dev_ptr(target), img_bytes, nat.dev_ptr(lab), lab_bytes, n,
                                       nat.dev_ptr(ztab), zero.size, _stream()))
    if _is_torch(img):
        if not in_place:
            img.copy_(target.view(img.dtype).view(img.shape))
        return
    img[...] = target.cpu().numpy().view(img.dtype).reshape(img.shape)


def _remap(cc_labels, table: np.ndarray, out_dtype, order: str = "C"):
    """out[voxel] = table[cc_labels[voxel]], shaped like cc_labels (numpy: in `order`)."""
    torch = _torch()
    lib = nat.load()
    lab = _flat_device(cc_labels)
    n = cc_labels.numel() if _is_torch(cc_labels) else cc_labels.size
    lab_bytes = cc_labels.element_size() if _is_torch(cc_labels) else cc_labels.dtype.itemsize
    table = np.ascontiguousarray(table)
    otab = torch.from_numpy(table.view(np.uint8)).cuda()
    width = table.dtype.itemsize
    out = torch.empty((max(1, n) * width,), dtype=torch.uint8, device=lab.device)
    nat.check(lib.cc3d_gpu_remap_labels(nat.dev_ptr(lab), lab_bytes, n, nat.dev_ptr(otab), width, table.size,
                                        nat.dev_ptr(out), _stream()))
    out = out[:n * width]
    if _is_torch(cc_labels):
        if out_dtype == np.bool_:
            res = out.view(torch.bool).view(cc_labels.shape)
        else:
            res = out.view(getattr(torch, np.dtype(out_dtype).name)).view(cc_labels.shape)
        return res if cc_labels.is_cuda else res.cpu()
    host = out.cpu().numpy().view(np.bool_ if out_dtype == np.bool_ else out_dtype).reshape(cc_labels.shape)
    return np.asfortranarray(host) if order == "F" else host


def largest_k(img: Any, k: int, connectivity: int = 26, delta=0, return_N: bool = False,
              binary_image: bool = False, precomputed_ccl: bool = False):
    """The k largest connected components, renumbered 1..k in increasing size
    (a boolean mask for k = 1).  Mirrors cc3d.largest_k
    (cc3d/__init__.py:199-279) as it runs without fastremap."""
    assert k >= 0
    torch = _torch() if _is_torch(img) else None
    if torch is None:
        order = "C" if img.flags.c_contiguous else "F"
    if k == 0:
        if torch is not None:
            return torch.zeros(img.shape, dtype=torch.int16, device=img.device).view(torch.uint16)
        return np.zeros(img.shape, dtype=np.uint16, order=order)
    if precomputed_ccl:
        cc_labels = img.clone() if torch is not None else np.copy(img, order="F")
        N = _max_int(cc_labels)
    else:
        cc_labels, N = connected_components(img, connectivity=connectivity, return_N=True, delta=delta,
                                            binary_image=bool(binary_image))
    if N <= k:
        return (cc_labels, N) if return_N else cc_labels
    cts = _counts_host(cc_labels, N)
    if k == 1:
        table = np.zeros(N + 1, dtype=np.bool_)
        table[np.argmax(cts[1:]) + 1] = True
        lab_order = "C" if (torch is not None or cc_labels.flags.c_contiguous) else "F"
        cc_out = _remap(cc_labels, table.view(np.uint8), np.bool_, lab_order)
        return (cc_out, 1) if return_N else cc_out
    preserve = np.argpartition(cts[1:], len(cts) - k - 1)[-k:]
    preserve += 1
    preserve_sorted = sorted(preserve, key=lambda label: cts[label])
    preserve_list = list(map(int, preserve_sorted))
    ldt = _np_dtype(cc_labels)
    ldt = np.dtype(_UNSIGNED_VIEW.get(ldt, ldt))
    table = np.zeros(N + 1, dtype=ldt)
    for i, label in enumerate(preserve_list):
        table[label] = i + 1
    lab_order = "C" if (torch is not None or cc_labels.flags.c_contiguous) else "F"
    cc_out = _remap(cc_labels, table, ldt, lab_order)
    return (cc_out, len(preserve_list)) if return_N else cc_out
