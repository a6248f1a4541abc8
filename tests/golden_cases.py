"""Loader and comparator for the golden fixtures made by golden/make_golden.py."""
from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_CACHE = {}


def load():
    if "g" not in _CACHE:
        with open(os.path.join(HERE, "golden", "cc3d_golden.json")) as f:
            meta = json.load(f)["cases"]
        arrays = np.load(os.path.join(HERE, "golden", "cc3d_golden.npz"))
        _CACHE["g"] = (meta, {k: arrays[k] for k in arrays.files})
    return _CACHE["g"]


def cases(kind):
    meta, arrays = load()
    return [(i, m) for i, m in enumerate(meta) if m["kind"] == kind]


def input_of(i, m):
    _, arrays = load()
    a = arrays[f"in{i}"]
    if m.get("order") == "F":
        a = np.asfortranarray(a)
    return a


def kwargs_of(m):
    kw = dict(m["kwargs"])
    if kw.get("out_dtype") is not None:
        kw["out_dtype"] = np.dtype(kw["out_dtype"])
    return kw


def check_cc(i, m, fn):
    """Run fn(data, return_N=True, **kwargs) and compare with the reference.

    Returns "ok", or "bg-defect" for the one documented difference (binary
    8-connected images where the reference leaves provisional labels in some
    background pixels).  Raises AssertionError on any other difference."""
    _, arrays = load()
    data = input_of(i, m)
    kw = kwargs_of(m)
    if "exc" in m:
        try:
            fn(data, return_N=True, **kw)
        except Exception as e:  # noqa: BLE001
            assert type(e).__name__ == m["exc"], (m["name"], type(e).__name__, m["exc"], str(e))
            return "ok"
        raise AssertionError(f"{m['name']}: expected {m['exc']}: {m['msg']}")
    out, N = fn(data, return_N=True, **kw)
    out = np.asarray(out)
    exp = arrays[f"out{i}"]
    assert N == m["N"], (m["name"], N, m["N"])
    assert str(out.dtype) == m["out_dtype"], (m["name"], out.dtype, m["out_dtype"])
    assert list(out.shape) == m["out_shape"], (m["name"], out.shape, m["out_shape"])
    if np.array_equal(out, exp):
        return "ok"
    binary8 = kw.get("connectivity") == 8 and (kw.get("binary_image") or m["dtype"] == "bool")
    if binary8:
        fg = data != 0
        assert np.array_equal(out[fg], exp[fg]), m["name"]
        assert not np.any(out[~fg]), m["name"]
        return "bg-defect"
    raise AssertionError(f"{m['name']}: labels differ")


def check_stats(i, m, fn):
    _, arrays = load()
    data = input_of(i, m)
    if "exc" in m:
        try:
            fn(data, no_slice_conversion=m["no_slice_conversion"])
        except Exception as e:  # noqa: BLE001
            assert type(e).__name__ == m["exc"], (m["name"], type(e).__name__, m["exc"])
            return
        raise AssertionError(f"{m['name']}: expected {m['exc']}")
    s = fn(data, no_slice_conversion=m["no_slice_conversion"])
    if m.get("empty"):
        assert s["voxel_counts"] is None and s["bounding_boxes"] is None and s["centroids"] is None
        return
    counts = np.asarray(s["voxel_counts"])
    assert counts.dtype == arrays[f"counts{i}"].dtype
    assert np.array_equal(counts, arrays[f"counts{i}"]), m["name"]
    cent = np.asarray(s["centroids"])
    assert np.array_equal(cent, arrays[f"cent{i}"], equal_nan=True), m["name"]
    if m["no_slice_conversion"]:
        bb = np.asarray(s["bounding_boxes"])
        assert bb.dtype == arrays[f"bbox{i}"].dtype, (bb.dtype, arrays[f"bbox{i}"].dtype)
        assert np.array_equal(bb, arrays[f"bbox{i}"]), m["name"]
    else:
        got = [None if sl is None else [[x.start, x.stop] for x in sl] for sl in s["bounding_boxes"]]
        assert got == m["slices"], m["name"]
