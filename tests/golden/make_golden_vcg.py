"""Golden fixtures for voxel_connectivity_graph and color_connectivity_graph,
made by the reference itself.

Run where make_golden.py has built the reference out of tree:

    python tests/golden/make_golden_vcg.py [--ref-build /tmp/cc3d_golden_ref]

Writes cc3d_vcg.npz (inputs and expected outputs) and cc3d_vcg.json (kind,
call arguments, N for color_connectivity_graph, or the exception type for
arguments the reference rejects).  color_connectivity_graph is fed both the
reference's own graphs of seeded label volumes and seeded random bitfields
(the latter need not be symmetric: the reference follows the later voxel's
bits).  Every input is built here from a seed.
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

    rng = np.random.default_rng(31)
    meta, arrays = [], {}

    def record(kind, data, **kw):
        i = len(meta)
        arrays[f"in{i}"] = data
        m = {"kind": kind, "dtype": str(data.dtype), "shape": list(data.shape),
             "order": "F" if data.flags.f_contiguous and not data.flags.c_contiguous else "C", "kwargs": kw}
        fn = R.voxel_connectivity_graph if kind == "vcg" else R.color_connectivity_graph
        try:
            res = fn(data, **kw)
        except Exception as e:  # the reference's own error for these arguments
            m["error"] = type(e).__name__
        else:
            if kind == "ccg" and kw.get("return_N"):
                res, n = res
                m["N"] = int(n)
            arrays[f"out{i}"] = res
            m["out_dtype"] = str(res.dtype)
        meta.append(m)

    for dtype in ("uint8", "int8", "uint16", "int16", "uint32", "int32", "uint64", "int64", "bool"):
        for shape in ((13, 11, 9), (40, 33), (1, 20, 17), (25,), (9, 1, 6), (33, 40, 3)):
            dims = len(shape)
            conns = (4, 8, 6, 18, 26) if dims == 2 else (6, 18, 26)
            for conn in conns:
                k = int(rng.choice([2, 3, 6]))
                a = rng.integers(0, k, shape).astype(dtype)
                if rng.random() < 0.5:
                    a = np.asfortranarray(a)
                record("vcg", a, connectivity=conn)
    # a larger volume and a blocky one
    record("vcg", np.kron(rng.integers(0, 9, (6, 5, 4)), np.ones((7, 8, 9), np.int64)).astype(np.uint32),
           connectivity=26)
    record("vcg", rng.integers(0, 2, (130, 70, 20)).astype(np.uint8), connectivity=18)
    # color_connectivity_graph on the reference's own graphs
    for shape, vconn, cconn in (((30, 28, 12), 26, 26), ((30, 28, 12), 6, 6), ((64, 50), 8, 8),
                                ((64, 50), 4, 4), ((47, 39), 8, 8), ((17, 23, 5), 26, 26),
                                ((90, 70, 9), 26, 26), ((90, 70, 9), 6, 6)):
        for k in (2, 4):
            a = rng.integers(0, k, shape).astype(np.uint16)
            v = R.voxel_connectivity_graph(a, connectivity=vconn)
            record("ccg", v, connectivity=cconn, return_N=True)
    # random bitfields (asymmetric graphs)
    for shape, dtype, conn in (((21, 19, 7), np.uint32, 26), ((21, 19, 7), np.uint8, 6),
                               ((21, 19, 7), np.uint32, 6), ((33, 29), np.uint8, 8), ((33, 29), np.uint8, 4),
                               ((33, 29), np.uint32, 8), ((33, 29), np.uint32, 4), ((33, 29), np.uint8, 6),
                               ((33, 29), np.uint8, 26), ((5, 1, 4), np.uint32, 26)):
        bits = 26 if dtype == np.uint32 else 8
        for p in (0.3, 0.6, 0.9):
            v = np.zeros(shape, dtype=np.uint64)
            for b in range(bits):
                v |= (rng.random(shape) < p).astype(np.uint64) << np.uint64(b)
            record("ccg", v.astype(dtype), connectivity=conn, return_N=True)
    record("ccg", np.full((6, 7, 5), 0x3ffffff, np.uint32), connectivity=26, return_N=False)
    # argument errors
    record("vcg", np.zeros((4, 4), np.float32), connectivity=8)
    record("vcg", np.zeros((4, 4, 4), np.uint8), connectivity=8)
    record("vcg", np.zeros((2, 2, 2, 2), np.uint8), connectivity=26)
    record("ccg", np.zeros((4, 4, 4), np.uint8), connectivity=26)
    record("ccg", np.zeros((4, 4, 4), np.uint16), connectivity=6)
    record("ccg", np.zeros((4, 4, 4), np.uint32), connectivity=18)
    record("ccg", np.zeros((4, 4), np.uint32), connectivity=18)
    record("ccg", np.zeros((4,), np.uint32), connectivity=6)
    np.savez_compressed(os.path.join(HERE, "cc3d_vcg.npz"), **arrays)
    with open(os.path.join(HERE, "cc3d_vcg.json"), "w") as f:
        json.dump(meta, f, indent=0)
    print(len(meta), "cases,", sum("error" in m for m in meta), "errors")


if __name__ == "__main__":
    main()
