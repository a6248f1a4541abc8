"""Golden fixtures for continuous-value labelling (delta != 0), made by the
reference itself.

Run where make_golden.py has built the reference out of tree:

    python tests/golden/make_golden_continuous.py [--ref-build /tmp/cc3d_golden_ref]

Writes cc3d_continuous.npz (inputs and expected labels) and
cc3d_continuous.json (call arguments, N, output dtype, or the exception type
for inputs the reference rejects).  The cases cover the 3D labeller at 26, 18
and 6, the 2D 4- and 8-connected labellers (including the 8-connected one's
image-span shortcut, which joins pixels whose values do not match), every
input dtype, C and F order, NaN and infinity in floating point inputs, and the
argument errors.  Every input is built here from a seed.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-build", default="/tmp/cc3d_golden_ref")
    args = ap.parse_args()
    sys.path.insert(0, args.ref_build)
    import cc3d as R

    rng = np.random.default_rng(23)
    meta, arrays = [], {}

    def record(data, **kw):
        i = len(meta)
        arrays[f"in{i}"] = data
        m = {"dtype": str(data.dtype), "shape": list(data.shape),
             "order": "F" if data.flags.f_contiguous and not data.flags.c_contiguous else "C",
             "kwargs": {k: (float(v) if isinstance(v, (float, np.floating)) else v) for k, v in kw.items()}}
        try:
            out, N = R.connected_components(data, return_N=True, **kw)
        except Exception as e:  # the reference's own error for these arguments
            m["error"] = type(e).__name__
        else:
            arrays[f"out{i}"] = out
            m["N"] = int(N)
            m["out_dtype"] = str(out.dtype)
        meta.append(m)

    def volume(dtype, shape, spread):
        if np.dtype(dtype).kind == "f":
            a = rng.normal(0.0, spread, shape) * (rng.random(shape) < 0.85)
            return a.astype(dtype)
        if np.dtype(dtype).kind == "b":
            return rng.random(shape) < 0.5
        info = np.iinfo(dtype)
        hi = min(int(info.max), int(spread))
        lo = max(int(info.min), -int(spread)) if info.min < 0 else 0
        return rng.integers(lo, hi + 1, shape).astype(dtype)

    dtypes = ("uint8", "uint16", "uint32", "uint64", "int8", "int16", "int32", "int64",
              "float32", "float64")
    for dtype in dtypes:
        for shape, conns in (((29, 23), (4, 8, 6, 18, 26)), ((13, 11, 9), (6, 18, 26)),
                             ((1, 40, 17), (6, 18, 26)), ((64, 1), (4, 8))):
            for conn in conns:
                spread = rng.choice([6, 40])
                a = volume(dtype, shape, spread)
                if rng.random() < 0.5:
                    a = np.asfortranarray(a)
                delta = (float(rng.choice([0.25, 1.0, 3.5])) if np.dtype(dtype).kind == "f"
                         else int(rng.choice([1, 2, 4])))
                record(a, connectivity=conn, delta=delta)
    # image-span shortcut of the 2D 8-connected labeller: a few distinct levels
    # with a delta just below the level spacing
    for k in range(8):
        a = (rng.integers(0, 4, (31, 27)) * 10).astype(np.uint16)
        if k % 2:
            a = np.asfortranarray(a)
        record(a, connectivity=8, delta=int(rng.choice([9, 10, 15, 25])))
        record(a.astype(np.float32), connectivity=8, delta=9.5)
    # NaN and infinity
    for dtype in ("float32", "float64"):
        for conn, shape in ((8, (25, 19)), (4, (25, 19)), (26, (9, 8, 7)), (6, (9, 8, 7))):
            a = volume(dtype, shape, 5.0)
            flat = a.reshape(-1)
            flat[rng.integers(0, a.size, 6)] = np.nan
            flat[rng.integers(0, a.size, 3)] = np.inf
            record(a, connectivity=conn, delta=2.0)
        a = volume(dtype, (20, 20), 5.0)
        a.reshape(-1)[-1] = np.nan  # the span fold ends in NaN
        record(a, connectivity=8, delta=1.0)
    # larger volumes
    record(volume("uint8", (48, 40, 36), 30), connectivity=26, delta=3)
    record(np.asfortranarray(volume("float32", (40, 44, 33), 4.0)), connectivity=18, delta=0.75)
    record(volume("uint16", (160, 150), 200), connectivity=8, delta=20)
    record(volume("int32", (170, 140), 50), connectivity=4, delta=6)
    # a delta equal to the dtype's maximum makes the image binary
    record(volume("int8", (17, 15), 100), connectivity=8, delta=127)
    record(volume("uint8", (9, 8, 7), 100), connectivity=26, delta=255)
    # argument errors
    record(volume("uint8", (10, 10), 9), connectivity=8, delta=-1)
    record(volume("uint8", (10, 10), 9), connectivity=8, delta=256)
    record(volume("int16", (6, 6, 6), 9), connectivity=6, delta=70000)
    record(volume("float32", (10, 10), 2.0).astype(np.float16), connectivity=4, delta=1.0)
    record(volume("uint8", (10, 10), 9), connectivity=4, delta=2, periodic_boundary=True)
    np.savez_compressed(os.path.join(HERE, "cc3d_continuous.npz"), **arrays)
    with open(os.path.join(HERE, "cc3d_continuous.json"), "w") as f:
        json.dump(meta, f, indent=0)
    print(len(meta), "cases,", sum("error" in m for m in meta), "errors")


if __name__ == "__main__":
    main()
