"""Tile-pass variants and their autotuner (include/cc3d_gpu.h: cc3d_gpu_set_tile_pass,
cc3d_gpu_tile_pass_choice, cc3d_gpu_autotune, cc3d_gpu_autotune_reset).

Every variant labels identically; the autotuner only picks the faster one for a
class of volumes (dtype, effective connectivity, binary or not, voxel count
within a factor of 8) and the labelling entry points use that choice from then
on.  The reference has no counterpart: it runs one CPU algorithm per
connectivity.
"""
from __future__ import annotations

import ctypes
from typing import Any, Dict

import numpy as np

from . import _native as nat
from .api import _CODE, _is_torch

VARIANTS = ("list", "runs")
_VARIANT_BITS = {"runs": 1, "list": 2}
SHAPES = ("8x8", "4x16", "16x4")   # 3D tiles 32 x TY x TZ; 2D images always use 32 x 64
_SHAPE_BITS = {"8x8": 0x00, "4x16": 0x10, "16x4": 0x20}
LOADS = ("", "plain")              # the box by one TMA copy, or by plain loads
_PLAIN = 0x100
# configuration index -> name, in the order of cc3d_gpu_tile_config
CONFIGS = tuple(f"{v}/{s}" + (f"/{ld}" if ld else "") for s in SHAPES for v in VARIANTS for ld in LOADS)


def config_code(name: str) -> int:
    """CC3D_TILE_* code of "auto", "model", "list", "runs" or
    "<variant>/<shape>[/plain]"."""
    if name == "auto":
        return 0
    if name == "model":
        return 3
    parts = name.split("/")
    code = _VARIANT_BITS[parts[0]] | _SHAPE_BITS[parts[1] if len(parts) > 1 else "8x8"]
    if len(parts) > 2:
        if parts[2] != "plain":
            raise KeyError(name)
        code |= _PLAIN
    return code


def config_name(code: int) -> str:
    if code == 0:
        return "auto"
    if code == 3:
        return "model"
    variant = {b: v for v, b in _VARIANT_BITS.items()}[code & 15]
    return f"{variant}/{SHAPES[(code >> 4) & 15]}" + ("/plain" if code & _PLAIN else "")


def set_tile_pass(name: str) -> str:
    """Select the calling thread's tile-pass configuration: "auto", "list",
    "runs" (32x8x8 tiles) or "<variant>/<shape>[/plain]" such as "runs/4x16"
    or "list/16x4/plain" (the tile's box by plain loads instead of TMA).
    "model" lets the learned cost model choose per volume (the parameters
    shipped with the package are loaded if no model was trained or loaded).
    Returns the previous setting."""
    if name == "model":
        from . import costmodel
        try:
            costmodel.get_params()
        except ValueError:
            costmodel.load()
    prev = nat.load().cc3d_gpu_set_tile_pass(config_code(name))
    if prev < 0:
        nat.check(prev)
    return config_name(prev)


def _volume(data: Any):
    """(pointer, dtype code, sx, sy, sz, mem flags, stream, keepalive) of a numpy
    array or CUDA tensor, as the labelling entry points see it."""
    if _is_torch(data) and data.is_cuda:
        import torch
        t = data.contiguous()
        npd = np.dtype(str(t.dtype).replace("torch.", ""))
        if npd == np.float16:
            t, npd = t.view(torch.int16), np.dtype(np.uint16)
        npd = {np.dtype(np.int8): np.dtype(np.uint8), np.dtype(np.int16): np.dtype(np.uint16),
               np.dtype(np.int32): np.dtype(np.uint32), np.dtype(np.int64): np.dtype(np.uint64),
               np.dtype(np.bool_): np.dtype(np.uint8)}.get(npd, npd)
        shape = list(t.shape)
        ptr, mem = nat.dev_ptr(t), nat.IN_DEVICE
        stream = ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)
        keep = t
    else:
        a = np.ascontiguousarray(data.cpu().numpy() if _is_torch(data) else data)
        if a.dtype == np.float16:
            a = a.view(np.uint16)
        if a.dtype.kind in "ib":
            a = a.view({1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[a.dtype.itemsize])
        npd, shape, ptr, mem, stream, keep = a.dtype, list(a.shape), a.ctypes.data, 0, None, a
    if npd not in _CODE:
        raise TypeError(f"unsupported dtype {npd}")
    while len(shape) < 3:
        shape.insert(0, 1)
    sz, sy, sx = (int(v) for v in shape)
    return ptr, _CODE[npd], sx, sy, sz, mem, stream, keep


def tile_pass_choice(data: Any, connectivity: int = 26, binary_image: bool = False) -> str:
    """The configuration a labelling of `data` would use now."""
    ptr, code, sx, sy, sz, mem, stream, keep = _volume(data)
    return config_name(nat.load().cc3d_gpu_tile_pass_choice(code, sx, sy, sz, int(connectivity),
                                                           int(bool(binary_image))))


def autotune(data: Any, connectivity: int = 26, binary_image: bool = False, repeats: int = 2) -> Dict[str, Any]:
    """Time every tile-pass configuration on `data` and record the fastest for
    its class.  Returns {"best": name, "ms": {name: milliseconds}}."""
    ptr, code, sx, sy, sz, mem, stream, keep = _volume(data)
    best = ctypes.c_int(0)
    ms = (ctypes.c_double * len(CONFIGS))()
    nat.check(nat.load().cc3d_gpu_autotune(ptr, code, sx, sy, sz, int(connectivity), int(bool(binary_image)),
                                           mem, stream, int(repeats), ctypes.byref(best), ms))
    return {"best": config_name(best.value),
            "ms": {CONFIGS[i]: ms[i] for i in range(len(CONFIGS)) if ms[i] >= 0}}


def autotune_reset() -> None:
    """Forget every recorded choice."""
    nat.load().cc3d_gpu_autotune_reset()
