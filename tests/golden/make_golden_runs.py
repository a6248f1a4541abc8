"""Golden fixtures for runs, draw and each, made by the reference itself.

Run where make_golden.py has built the reference out of tree:

    python tests/golden/make_golden_runs.py [--ref-build /tmp/cc3d_golden_ref]

Writes cc3d_runs.npz (inputs; each case's runs flattened as parallel uint64
arrays of label, start and end in the reference's dictionary order, and the
list of labels each() yields) and cc3d_runs.json (dtypes, shapes, orders).
An input the reference rejects records the exception's type instead.  Every
input is built here from a seed.
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
    from cc3d import fastcc3d as F

    rng = np.random.default_rng(11)
    meta, arrays = [], {}

    def record(data):
        i = len(meta)
        arrays[f"in{i}"] = data
        order = "F" if data.flags.f_contiguous and not data.flags.c_contiguous else "C"
        try:
            res = F.runs(data)
        except Exception as e:  # the reference's own error for this input
            meta.append({"dtype": str(data.dtype), "shape": list(data.shape), "order": order,
                         "error": type(e).__name__})
            return
        labs, starts, ends = [], [], []
        for key, rns in res.items():
            for a, b in rns:
                labs.append(key)
                starts.append(a)
                ends.append(b)
        arrays[f"lab{i}"] = np.array(labs, dtype=np.uint64)
        arrays[f"start{i}"] = np.array(starts, dtype=np.uint64)
        arrays[f"end{i}"] = np.array(ends, dtype=np.uint64)
        arrays[f"each{i}"] = np.array([k for k, _ in R.each(data)], dtype=np.uint64)
        meta.append({"dtype": str(data.dtype), "shape": list(data.shape), "order": order,
                     "keys": len(res)})

    for dtype in ("uint8", "uint16", "uint32", "uint64", "bool"):
        for shape in ((128,), (37, 29), (19, 13, 11), (1, 1, 1), (1,), (0,), (2,), (5, 1, 7)):
            for order in ("C", "F"):
                if dtype == "bool":
                    a = rng.random(shape) < 0.5
                else:
                    hi = 3 if rng.random() < 0.5 else 200
                    a = rng.integers(0, hi, shape).astype(dtype)
                a = np.asfortranarray(a) if order == "F" else np.ascontiguousarray(a)
                record(a)
    # long runs, a run spanning the last element, a single nonzero voxel, an all-zero volume
    block = np.kron(rng.integers(0, 6, (5, 4, 3)), np.ones((9, 8, 7), np.int64)).astype(np.uint32)
    record(block)
    record(np.asfortranarray(block))
    one = np.zeros((4, 5, 6), np.uint16)
    one[3, 4, 5] = 9
    record(one)
    record(np.zeros((3, 3), np.uint8))
    record(np.full((6, 6), 7, np.uint64))
    record(np.array([0], np.uint32))
    record(np.array([5], np.uint32))
    # large labels close to the top of each width
    big = rng.choice(np.array([0, 2**63 + 5, 2**64 - 1, 1], np.uint64), (17, 9))
    record(big)
    np.savez_compressed(os.path.join(HERE, "cc3d_runs.npz"), **arrays)
    with open(os.path.join(HERE, "cc3d_runs.json"), "w") as f:
        json.dump(meta, f, indent=0)
    print(len(meta), "cases")


if __name__ == "__main__":
    main()
