"""Golden fixtures for dust and largest_k, made by the reference itself.

Run where the reference's Cython extension has been built by make_golden.py
(its out-of-tree build under /tmp/cc3d_golden_ref):

    python tests/golden/make_golden_filters.py [--ref-build /tmp/cc3d_golden_ref]

Writes cc3d_filters.npz (inputs and outputs) and cc3d_filters.json (call
arguments, N, dtypes, memory order).  Every input is built here from a seed.
The reference runs without fastremap, as in this container.  largest_k cases
with k >= 2 are kept only where the k+1 largest component sizes differ, so the
expected output does not depend on argpartition's tie order (which differs
between numpy builds).
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
    import cc3d as R  # the reference, built out of tree

    rng = np.random.default_rng(20241204)
    meta, arrays = [], {}

    def record(kind, data, **kw):
        i = len(meta)
        arrays[f"in{i}"] = data
        entry = {"kind": kind, "dtype": str(data.dtype), "shape": list(data.shape),
                 "order": "F" if data.flags.f_contiguous and not data.flags.c_contiguous else "C",
                 "kwargs": {k: (list(v) if isinstance(v, tuple) else v) for k, v in kw.items()}}
        fn = R.dust if kind == "dust" else R.largest_k
        res = fn(np.copy(data, order="A"), return_N=True, **kw)
        out, N = res if isinstance(res, tuple) else (res, None)
        arrays[f"out{i}"] = out
        entry.update(N=None if N is None else int(N), out_dtype=str(out.dtype),
                     out_order="F" if out.flags.f_contiguous and not out.flags.c_contiguous else "C")
        meta.append(entry)

    def distinct_top(data, k, **kw):
        """True when the k+1 largest component sizes are all different, so that
        the choice and order of largest_k do not depend on how a numpy build
        breaks ties in argpartition."""
        if kw.get("precomputed_ccl"):
            lab = data
        else:
            lab = R.connected_components(data, connectivity=kw.get("connectivity", 26),
                                         binary_image=kw.get("binary_image", False))
        cts = np.sort(R.statistics(lab, no_slice_conversion=True)["voxel_counts"][1:])[::-1]
        top = cts[:k + 1]
        return len(cts) <= k or len(np.unique(top)) == len(top)

    def record_k(data, k, **kw):
        for kk in [k] + [x for x in range(2, 9) if x != k]:
            if distinct_top(data, kk, **kw):
                record("largest_k", data, k=kk, **kw)
                return

    def volume(shape, dtype, k, p, order):
        a = (rng.integers(1, k + 1, shape) * (rng.random(shape) < p)).astype(dtype)
        return np.asfortranarray(a) if order == "F" else a

    for dtype in ("uint8", "int16", "uint32", "int64", "bool"):
        for order in ("C", "F"):
            for shape in ((30, 40), (17, 23, 29)):
                conns = (4, 8) if len(shape) == 2 else (6, 18, 26)
                for conn in conns:
                    k = 1 if dtype == "bool" else int(rng.integers(2, 5))
                    a = volume(shape, dtype, k, float(rng.uniform(0.3, 0.7)), order)
                    record("dust", a, threshold=int(rng.integers(2, 12)), connectivity=conn)
                    record("dust", a, threshold=(3, 20), connectivity=conn, invert=True)
                    record("dust", a, threshold=5, connectivity=conn, binary_image=True)
                    record_k(a, int(rng.integers(2, 6)), connectivity=conn)
                    record("largest_k", a, k=1, connectivity=conn)
                    record("largest_k", a, k=0, connectivity=conn)
                    record("largest_k", a, k=10_000, connectivity=conn)
                    record_k(a, 3, connectivity=conn, binary_image=True)
    # precomputed labels and the "nothing to remove" branches
    for shape in ((25, 31, 19), (64, 48)):
        a = volume(shape, "uint16", 3, 0.5, "C")
        lab = R.connected_components(a, connectivity=26 if len(shape) == 3 else 8)
        record("dust", lab, threshold=4, precomputed_ccl=True)
        record("dust", lab, threshold=0)
        record("dust", lab, threshold=0, invert=True)
        record_k(lab, 4, precomputed_ccl=True)
    np.savez_compressed(os.path.join(HERE, "cc3d_filters.npz"), **arrays)
    with open(os.path.join(HERE, "cc3d_filters.json"), "w") as f:
        json.dump(meta, f, indent=0)
    print(len(meta), "cases")


if __name__ == "__main__":
    main()
