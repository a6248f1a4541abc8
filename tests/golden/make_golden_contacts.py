"""Golden fixtures for contacts and region_graph, made by the reference itself.

Run where make_golden.py has built the reference out of tree:

    python tests/golden/make_golden_contacts.py [--ref-build /tmp/cc3d_golden_ref]

Writes cc3d_contacts.npz (inputs; each case's pairs as [n, 2] uint64 and
values as float32) and cc3d_contacts.json (call arguments).  Every input is
built here from a seed.
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

    rng = np.random.default_rng(7)
    meta, arrays = [], {}

    def record(data, **kw):
        i = len(meta)
        arrays[f"in{i}"] = data
        res = R.contacts(data, **kw)
        keys = sorted(res)
        arrays[f"pairs{i}"] = np.array(keys, dtype=np.uint64).reshape(-1, 2)
        arrays[f"vals{i}"] = np.array([res[k] for k in keys], dtype=np.float32)
        meta.append({"dtype": str(data.dtype), "shape": list(data.shape),
                     "kwargs": {k: (list(v) if isinstance(v, tuple) else v) for k, v in kw.items()}})

    for dtype in ("uint8", "uint16", "uint32", "int32", "uint64"):
        for shape in ((23, 17, 11), (40, 33), (1, 30, 20), (31, 1, 9)):
            a = (rng.integers(1, 9, shape) * (rng.random(shape) < 0.8)).astype(dtype)
            if rng.random() < 0.5:
                a = np.asfortranarray(a)
            conns = (4, 8, 6, 18, 26) if len(shape) == 2 else (6, 18, 26)
            for conn in conns:
                record(a, connectivity=conn)
                record(a, connectivity=conn, surface_area=False)
                record(a, connectivity=conn, anisotropy=(4, 4, 40))
    # a blocky segmentation with large contact areas, and non-integer anisotropy
    base = rng.integers(1, 50, (6, 6, 6)).astype(np.uint32)
    blocky = np.kron(base, np.ones((7, 7, 7), np.uint32))
    record(blocky, connectivity=26)
    record(blocky, connectivity=6, anisotropy=(0.3, 1.7, 2.9))
    np.savez_compressed(os.path.join(HERE, "cc3d_contacts.npz"), **arrays)
    with open(os.path.join(HERE, "cc3d_contacts.json"), "w") as f:
        json.dump(meta, f, indent=0)
    print(len(meta), "cases")


if __name__ == "__main__":
    main()
