"""Many volumes in one go: include/cc3d_gpu.h cc3d_gpu_label_batch.

    outs = connected_components_batch([vol0, vol1, ...], connectivity=26)

gives, for every volume, exactly what ``connected_components(vol,
connectivity)`` gives (labels, N, and the output dtype the reference would
choose), but labels all of them together: by default with ONE persistent
kernel launch that walks every stage over the whole batch (replayed from a
CUDA graph captured once, whatever the shapes), or, after
``set_batch_mode("staged")``, with one launch of each stage replayed from a
CUDA graph while the list of shapes repeats.  The reference has no batch
call: its users loop over ``cc3d.connected_components``.

Volumes are CUDA tensors or numpy arrays (copied to the device) of one dtype
among uint8/16/32 (int8/16/32 and bool are viewed as the unsigned type of the
same width), C-ordered, 2D or 3D; multilabel only.
"""
from __future__ import annotations

import ctypes
from typing import Any, Dict, List, Sequence

import numpy as np

from . import _native as nat


class Volume(ctypes.Structure):
    """cc3d_gpu_volume."""
    _fields_ = [("in_", ctypes.c_void_p), ("out", ctypes.c_void_p),
                ("sx", ctypes.c_int64), ("sy", ctypes.c_int64), ("sz", ctypes.c_int64)]


class VolumeResult(ctypes.Structure):
    """cc3d_gpu_volume_result."""
    _fields_ = [("N", ctypes.c_uint64), ("epl", ctypes.c_uint64), ("provisional", ctypes.c_uint64),
                ("first_row", ctypes.c_int64), ("last_row", ctypes.c_int64),
                ("out_dtype", ctypes.c_int32), ("status", ctypes.c_int32)]


_UNSIGNED = {1: np.uint8, 2: np.uint16, 4: np.uint32}


def _as_device(torch, v):
    if not (hasattr(v, "is_cuda") and v.is_cuda):
        v = torch.from_numpy(np.ascontiguousarray(np.asarray(v)))
        v = v.cuda()
    return v.contiguous()


_VOLUME_DTYPE = np.dtype([("in", "<u8"), ("out", "<u8"), ("sx", "<i8"), ("sy", "<i8"), ("sz", "<i8")])
_RESULT_DTYPE = np.dtype([("N", "<u8"), ("epl", "<u8"), ("provisional", "<u8"), ("first_row", "<i8"),
                          ("last_row", "<i8"), ("out_dtype", "<i4"), ("status", "<i4")])
assert _VOLUME_DTYPE.itemsize == ctypes.sizeof(Volume) and _RESULT_DTYPE.itemsize == ctypes.sizeof(VolumeResult)


def _descriptors(volumes):
    """Device volumes, dtype code, the cc3d_gpu_volume and result arrays (numpy
    records with the C layouts) and the output views."""
    import torch
    devs = [_as_device(torch, v) for v in volumes]
    dt = devs[0].dtype
    if any(d.dtype != dt for d in devs):
        raise TypeError("all volumes of a batch must have one dtype")
    itemsize = devs[0].element_size()
    if itemsize not in _UNSIGNED or devs[0].is_floating_point():
        raise TypeError(f"batches take 8, 16 or 32-bit integer volumes, not {dt}")
    code = {1: nat.U8, 2: nat.U16, 4: nat.U32}[itemsize]
    n = len(devs)
    shapes = np.ones((n, 3), np.int64)
    for i, d in enumerate(devs):
        if d.dim() not in (2, 3):
            raise ValueError("batches take 2D or 3D volumes")
        shapes[i, 3 - d.dim():] = d.shape
    voxels = shapes.prod(axis=1)
    # one allocation for every output (4 bytes per voxel, 256-byte aligned slices)
    sizes = ((np.maximum(voxels, 1) * 4 + 255) // 256) * 256
    pool = torch.empty((int(sizes.sum()),), dtype=torch.uint8, device=devs[0].device)
    offs = np.concatenate([[0], np.cumsum(sizes)[:-1]])
    vols = np.empty(n, _VOLUME_DTYPE)
    vols["in"] = [nat.dev_ptr(d) for d in devs]
    vols["out"] = nat.dev_ptr(pool) + offs
    vols["sx"], vols["sy"], vols["sz"] = shapes[:, 2], shapes[:, 1], shapes[:, 0]
    res = np.zeros(n, _RESULT_DTYPE)
    outs = pool.split([int(v) for v in sizes])
    return devs, code, vols, res, outs


def _labels(devs, outs, res, return_N):
    import torch
    results = []
    codes, Ns = res["out_dtype"], res["N"]
    for i, d in enumerate(devs):
        if d.numel() == 0:
            # like the single-volume call (fastcc3d.pyx: empty input -> zeros((0,), input dtype))
            lab = torch.zeros((0,), dtype=d.dtype, device=d.device)
        else:
            tdt = torch.uint16 if codes[i] == nat.U16 else torch.uint32
            nbytes = d.numel() * (2 if tdt == torch.uint16 else 4)
            lab = outs[i][:nbytes].view(tdt).view(d.shape)
        results.append((lab, int(Ns[i])) if return_N else lab)
    return results


_MODES = {"persistent": 0, "staged": 1}


def set_batch_mode(mode: str) -> str:
    """This thread's batch mode, "persistent" (default) or "staged"; returns
    the previous one (cc3d_gpu_set_batch_mode)."""
    if mode not in _MODES:
        raise ValueError(f"unknown batch mode {mode!r}")
    prev = nat.load().cc3d_gpu_set_batch_mode(_MODES[mode])
    nat.check(min(prev, 0))
    return {v: k for k, v in _MODES.items()}[prev]


def connected_components_batch(volumes: Sequence[Any], connectivity: int = 26,
                               return_N: bool = False) -> List[Any]:
    """Label every volume; returns a list of CUDA tensors (or (tensor, N))."""
    import torch
    if len(volumes) == 0:
        return []
    devs, code, vols, res, outs = _descriptors(volumes)
    with torch.cuda.device(devs[0].device):
        nat.check(nat.load().cc3d_gpu_label_batch(vols.ctypes.data, len(devs), code, int(connectivity),
                                                  res.ctypes.data, None))
    return _labels(devs, outs, res, return_N)


def autotune_batch(volumes: Sequence[Any], connectivity: int = 26, repeats: int = 2) -> Dict[str, Any]:
    """Time every tile-pass configuration on this batch and record the fastest
    for its class (dtype, connectivity, mean volume size).  Returns
    {"best": name, "ms": {name: milliseconds}}."""
    import torch
    from .tuning import CONFIGS, config_name
    devs, code, vols, res, outs = _descriptors(volumes)
    best = ctypes.c_int(0)
    ms = (ctypes.c_double * len(CONFIGS))()
    with torch.cuda.device(devs[0].device):
        nat.check(nat.load().cc3d_gpu_autotune_batch(vols.ctypes.data, len(devs), code, int(connectivity),
                                                     res.ctypes.data, None, int(repeats), ctypes.byref(best), ms))
    return {"best": config_name(best.value),
            "ms": {CONFIGS[i]: ms[i] for i in range(len(CONFIGS)) if ms[i] >= 0}}
