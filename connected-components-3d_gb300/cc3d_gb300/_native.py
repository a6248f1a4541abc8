"""ctypes binding of libcc3d_gpu.so (the C ABI declared in include/cc3d_gpu.h).

There is no CPU fallback: when the library is missing or no CUDA device is
usable, every call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import _build

U8, U16, U32, U64, F32, F64 = 1, 2, 3, 4, 5, 6
IN_DEVICE, OUT_DEVICE = 1, 2

OK = 0
ERR_INVALID = -1
ERR_UNSUPPORTED = -2
ERR_CUDA = -3
ERR_NOMEM = -4
ERR_RUNTIME = -5
ERR_DEVICE = -6
ERR_OVERFLOW = -7
ERR_NAN = -8

EXPORTED = (
    "cc3d_gpu_last_error",
    "cc3d_gpu_version",
    "cc3d_gpu_estimate_provisional_label_count",
    "cc3d_gpu_connected_components3d",
    "cc3d_gpu_label_prepare",
    "cc3d_gpu_label_prepare_continuous",
    "cc3d_gpu_voxel_connectivity_graph",
    "cc3d_gpu_label_prepare_graph",
    "cc3d_gpu_label_finish",
    "cc3d_gpu_special_row",
    "cc3d_gpu_label_minmax",
    "cc3d_gpu_statistics",
    "cc3d_gpu_profile_enable",
    "cc3d_gpu_profile_read",
    "cc3d_gpu_release_workspace",
    "cc3d_gpu_connected_components3d_noalloc",
    "cc3d_gpu_set_tile_pass",
    "cc3d_gpu_set_union_budget",
    "cc3d_gpu_tile_pass_choice",
    "cc3d_gpu_tile_config",
    "cc3d_gpu_autotune",
    "cc3d_gpu_autotune_reset",
    "cc3d_gpu_label_batch",
    "cc3d_gpu_release_batch",
    "cc3d_gpu_autotune_batch",
    "cc3d_gpu_set_batch_mode",
    "cc3d_gpu_volume_features",
    "cc3d_gpu_cost_model_train",
    "cc3d_gpu_cost_model_predict",
    "cc3d_gpu_cost_model_get",
    "cc3d_gpu_cost_model_set",
    "cc3d_gpu_cost_model_choose",
    "cc3d_gpu_remap_labels",
    "cc3d_gpu_zero_labels",
    "cc3d_gpu_contacts",
    "cc3d_gpu_contacts_copy",
    "cc3d_gpu_run_starts",
    "cc3d_gpu_run_starts_copy",
    "cc3d_gpu_stack_work_bytes",
    "cc3d_gpu_stack_begin",
    "cc3d_gpu_stack_seam",
    "cc3d_gpu_stack_number",
    "cc3d_gpu_stack_relabel",
)
PROFILE_STAGES = ("h2d", "epl", "tile_local", "merge_edges", "wrap_pairs", "scan", "write", "d2h")

class Prepared(ctypes.Structure):
    """cc3d_gpu_prepared (include/cc3d_gpu.h)."""
    _fields_ = [("token", ctypes.c_uint64), ("epl", ctypes.c_uint64), ("first_row", ctypes.c_int64),
                ("last_row", ctypes.c_int64), ("N", ctypes.c_uint64), ("provisional", ctypes.c_uint64),
                ("edges", ctypes.c_uint64)]


_lock = threading.Lock()
_lib = None


def library_path() -> str:
    return _build.LIB


def load() -> ctypes.CDLL:
    """Load the native library (it must have been built: cc3d_gb300.build())."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if not os.path.exists(path):
            raise ImportError(
                f"the CUDA extension is not built ({path} is missing); "
                "run cc3d_gb300.build() or __graft_entry__.build()")
        lib = ctypes.CDLL(path)
        vp, i64, u64p, i64p = ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int64)
        ci = ctypes.c_int
        lib.cc3d_gpu_last_error.restype = ctypes.c_char_p
        lib.cc3d_gpu_version.restype = ctypes.c_char_p
        lib.cc3d_gpu_estimate_provisional_label_count.argtypes = [vp, ci, i64, i64, u64p, i64p, i64p, ci, vp]
        lib.cc3d_gpu_connected_components3d.argtypes = [
            vp, ci, i64, i64, i64, i64, i64, ctypes.c_double, vp, ci, u64p, ci, ci, ci, vp]
        lib.cc3d_gpu_label_prepare.argtypes = [vp, ci, i64, i64, i64, i64, ci, ci, ci, vp,
                                               ctypes.POINTER(Prepared)]
        lib.cc3d_gpu_label_prepare_continuous.argtypes = [vp, ci, i64, i64, i64, i64, vp, ci, vp,
                                                          ctypes.POINTER(Prepared)]
        lib.cc3d_gpu_label_finish.argtypes = [ctypes.c_uint64, i64, vp, ci, u64p, ci, vp]
        lib.cc3d_gpu_voxel_connectivity_graph.argtypes = [vp, ci, i64, i64, i64, ci, ci, vp, vp]
        lib.cc3d_gpu_label_prepare_graph.argtypes = [vp, ci, i64, i64, i64, i64, ci, vp,
                                                     ctypes.POINTER(Prepared)]
        lib.cc3d_gpu_special_row.argtypes = [vp, ci, ci, i64, i64, i64, i64, vp, ci, u64p, ci, vp]
        lib.cc3d_gpu_label_minmax.argtypes = [vp, ci, ci, i64, u64p, i64p, ci, vp]
        lib.cc3d_gpu_statistics.argtypes = [vp, ci, i64, i64, i64, ci, ci, ctypes.c_uint64, vp, vp, ci, vp, ci, vp]
        lib.cc3d_gpu_release_workspace.restype = None
        lib.cc3d_gpu_connected_components3d_noalloc.argtypes = [
            vp, ci, i64, i64, i64, i64, i64, vp, ci, u64p, ci, ci, vp]
        lib.cc3d_gpu_connected_components3d_noalloc.restype = ctypes.c_int
        lib.cc3d_gpu_set_tile_pass.argtypes = [ci]
        lib.cc3d_gpu_set_tile_pass.restype = ci
        lib.cc3d_gpu_set_union_budget.argtypes = [ci]
        lib.cc3d_gpu_set_union_budget.restype = ci
        lib.cc3d_gpu_tile_pass_choice.argtypes = [ci, i64, i64, i64, i64, ci]
        lib.cc3d_gpu_tile_pass_choice.restype = ci
        lib.cc3d_gpu_tile_config.argtypes = [ci]
        lib.cc3d_gpu_tile_config.restype = ci
        lib.cc3d_gpu_autotune.argtypes = [vp, ci, i64, i64, i64, i64, ci, ci, vp, ci,
                                          ctypes.POINTER(ci), ctypes.POINTER(ctypes.c_double)]
        lib.cc3d_gpu_autotune.restype = ci
        lib.cc3d_gpu_autotune_reset.argtypes = []
        lib.cc3d_gpu_autotune_reset.restype = None
        lib.cc3d_gpu_label_batch.argtypes = [vp, ci, ci, i64, vp, vp]
        lib.cc3d_gpu_label_batch.restype = ci
        lib.cc3d_gpu_release_batch.argtypes = []
        lib.cc3d_gpu_release_batch.restype = None
        lib.cc3d_gpu_autotune_batch.argtypes = [vp, ci, ci, i64, vp, vp, ci, ctypes.POINTER(ci),
                                                ctypes.POINTER(ctypes.c_double)]
        lib.cc3d_gpu_autotune_batch.restype = ci
        lib.cc3d_gpu_set_batch_mode.argtypes = [ci]
        lib.cc3d_gpu_set_batch_mode.restype = ci
        fp = ctypes.POINTER(ctypes.c_float)
        lib.cc3d_gpu_volume_features.argtypes = [vp, ci, i64, i64, i64, i64, ci, ci, vp, fp]
        lib.cc3d_gpu_cost_model_train.argtypes = [vp, vp, ci, ci, ci, ctypes.c_float, ctypes.c_uint64, fp]
        lib.cc3d_gpu_cost_model_predict.argtypes = [vp, ci, vp]
        lib.cc3d_gpu_cost_model_get.argtypes = [vp, ci]
        lib.cc3d_gpu_cost_model_set.argtypes = [vp, ci]
        lib.cc3d_gpu_cost_model_choose.argtypes = [vp, ci, i64, i64, i64, i64, ci, ci, vp, ctypes.c_float,
                                                   ctypes.POINTER(ci), ctypes.POINTER(ci)]
        lib.cc3d_gpu_remap_labels.argtypes = [vp, ci, i64, vp, ci, ctypes.c_uint64, vp, vp]
        lib.cc3d_gpu_zero_labels.argtypes = [vp, ci, vp, ci, i64, vp, ctypes.c_uint64, vp]
        lib.cc3d_gpu_remap_labels.restype = ci
        lib.cc3d_gpu_contacts.argtypes = [vp, ci, i64, i64, i64, i64, u64p, vp]
        lib.cc3d_gpu_contacts.restype = ci
        lib.cc3d_gpu_contacts_copy.argtypes = [vp, vp, ctypes.c_uint64]
        lib.cc3d_gpu_contacts_copy.restype = ci
        lib.cc3d_gpu_run_starts.argtypes = [vp, ci, i64, u64p, vp]
        lib.cc3d_gpu_run_starts.restype = ci
        lib.cc3d_gpu_run_starts_copy.argtypes = [vp, vp, ctypes.c_uint64]
        lib.cc3d_gpu_run_starts_copy.restype = ci
        lib.cc3d_gpu_zero_labels.restype = ci
        u64 = ctypes.c_uint64
        lib.cc3d_gpu_stack_work_bytes.argtypes = [u64]
        lib.cc3d_gpu_stack_work_bytes.restype = u64
        lib.cc3d_gpu_stack_begin.argtypes = [vp, u64, vp]
        lib.cc3d_gpu_stack_seam.argtypes = [vp, vp, ci, vp, ci, u64, vp, ci, u64, i64, i64, i64, ci, vp, u64, vp]
        lib.cc3d_gpu_stack_number.argtypes = [vp, u64, u64p, vp]
        lib.cc3d_gpu_stack_relabel.argtypes = [vp, ci, i64p, u64, vp, ci, i64p, i64, i64, i64, vp, u64,
                                               ctypes.POINTER(ci), vp]
        for name in ("cc3d_gpu_stack_begin", "cc3d_gpu_stack_seam", "cc3d_gpu_stack_number",
                     "cc3d_gpu_stack_relabel"):
            getattr(lib, name).restype = ci
        for name in ("cc3d_gpu_volume_features", "cc3d_gpu_cost_model_train", "cc3d_gpu_cost_model_predict",
                     "cc3d_gpu_cost_model_get", "cc3d_gpu_cost_model_set", "cc3d_gpu_cost_model_choose"):
            getattr(lib, name).restype = ci
        lib.cc3d_gpu_profile_enable.argtypes = [ci]
        lib.cc3d_gpu_profile_enable.restype = None
        lib.cc3d_gpu_profile_read.argtypes = [ctypes.POINTER(ctypes.c_double), u64p, ci]
        for name in EXPORTED[2:9] + ("cc3d_gpu_profile_read",):
            getattr(lib, name).restype = ctypes.c_int
        _lib = lib
        return lib


def profile_enable(on: bool) -> None:
    load().cc3d_gpu_profile_enable(int(bool(on)))


def profile_read() -> dict:
    """Per-stage (milliseconds, launches) accumulated since the last read."""
    n = len(PROFILE_STAGES)
    ms = (ctypes.c_double * n)()
    cnt = (ctypes.c_uint64 * n)()
    load().cc3d_gpu_profile_read(ms, cnt, n)
    return {name: (ms[i], int(cnt[i])) for i, name in enumerate(PROFILE_STAGES)}


def dev_ptr(t) -> int:
    """The device address of a CUDA tensor; anything else is refused here, so
    that no host address ever reaches a kernel."""
    if not getattr(t, "is_cuda", False):
        raise RuntimeError("internal error: a device buffer was expected (got a host tensor)")
    return t.data_ptr()


def check(rc: int) -> None:
    """Raise the Python exception the reference raises for this failure."""
    if rc == OK:
        return
    msg = load().cc3d_gpu_last_error().decode(errors="replace")
    if rc == ERR_INVALID:
        raise ValueError(msg)
    if rc == ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    if rc == ERR_NOMEM:
        raise MemoryError(msg)
    if rc == ERR_OVERFLOW:
        raise OverflowError(msg)
    if rc == ERR_NAN:
        raise ValueError(msg)
    raise RuntimeError(msg)
