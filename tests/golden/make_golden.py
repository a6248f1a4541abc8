"""Generate the golden fixtures in this folder from the reference itself.

Run in a container that has the reference source tree, Cython and g++:

    python tests/golden/make_golden.py --ref <reference source tree>   (or set CC3D_REFERENCE)

It compiles the reference's Cython extension out of tree (into a scratch
directory under /tmp, never into the reference or this repository), imports it,
runs it on seeded inputs and writes:

    cc3d_golden.npz   inputs and expected outputs (compressed)
    cc3d_golden.json  per-case metadata: call arguments, N, dtypes, exceptions

The cases restate the kinds of inputs the reference's own test-suite exercises
for the labelling path (squares, rectangles, crosses, diagonals, 3D crosses,
empty/degenerate shapes, out_dtype rules, single-row inputs, periodic
boundaries, binary images, statistics), plus seeded random volumes across every
dtype, memory order and connectivity.  No array is copied from the reference's
tests; every input is built here from a seed.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import sysconfig

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

DTYPES = ["int8", "int16", "int32", "int64", "uint8", "uint16", "uint32", "uint64",
          "float16", "float32", "float64", "bool"]


def build_reference(ref: str) -> str:
    work = "/tmp/cc3d_golden_ref"
    so_glob = os.path.join(work, "cc3d")
    if not os.path.exists(os.path.join(work, "built.ok")):
        shutil.rmtree(work, ignore_errors=True)
        shutil.copytree(ref, work)
        src = os.path.join(work, "cc3d")
        subprocess.run(["cython", "-3", "--cplus", "fastcc3d.pyx", "-o", "fastcc3d.cpp"],
                       cwd=src, check=True)
        inc = sysconfig.get_paths()["include"]
        suffix = sysconfig.get_config_var("EXT_SUFFIX")
        subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", f"-I{inc}", "-I.",
                        f"-I{np.get_include()}", "fastcc3d.cpp", "-o", "fastcc3d" + suffix],
                       cwd=src, check=True)
        open(os.path.join(work, "built.ok"), "w").close()
    return so_glob


class Recorder:
    def __init__(self, R):
        self.R = R
        self.meta = []
        self.arrays = {}

    def _store(self, key, arr):
        self.arrays[key] = np.asarray(arr)

    def cc(self, name, data, **kw):
        i = len(self.meta)
        entry = {"name": name, "kind": "cc", "kwargs": {}, "order": "F" if data.flags.f_contiguous and not data.flags.c_contiguous else "C",
                 "dtype": str(data.dtype), "shape": list(data.shape)}
        for k, v in kw.items():
            entry["kwargs"][k] = (np.dtype(v).name if k == "out_dtype" and v is not None else v)
        self._store(f"in{i}", data)
        try:
            out, N = self.R.connected_components(data, return_N=True, **kw)
            entry.update(N=int(N), out_dtype=str(out.dtype), out_shape=list(out.shape))
            self._store(f"out{i}", out)
        except Exception as e:  # the reference's own error is part of the contract
            entry.update(exc=type(e).__name__, msg=str(e))
        self.meta.append(entry)

    def epl(self, name, data):
        i = len(self.meta)
        self._store(f"in{i}", data)
        entry = {"name": name, "kind": "epl", "dtype": str(data.dtype), "shape": list(data.shape),
                 "order": "F" if data.flags.f_contiguous and not data.flags.c_contiguous else "C"}
        try:
            entry["epl"] = [int(v) for v in self.R.estimate_provisional_labels(data)]
        except Exception as e:
            entry.update(exc=type(e).__name__, msg=str(e))
        self.meta.append(entry)

    def stats(self, name, labels, no_slice_conversion=True):
        i = len(self.meta)
        self._store(f"in{i}", labels)
        entry = {"name": name, "kind": "stats", "dtype": str(labels.dtype), "shape": list(labels.shape),
                 "order": "F" if labels.flags.f_contiguous and not labels.flags.c_contiguous else "C",
                 "no_slice_conversion": no_slice_conversion}
        try:
            s = self.R.statistics(labels, no_slice_conversion=no_slice_conversion)
            if s["voxel_counts"] is None:
                entry["empty"] = True
            else:
                self._store(f"counts{i}", s["voxel_counts"])
                self._store(f"cent{i}", s["centroids"])
                if no_slice_conversion:
                    self._store(f"bbox{i}", s["bounding_boxes"])
                else:
                    entry["slices"] = [None if sl is None else [[x.start, x.stop] for x in sl]
                                       for sl in s["bounding_boxes"]]
        except Exception as e:
            entry.update(exc=type(e).__name__, msg=str(e))
        self.meta.append(entry)


def structured_cases(rec: Recorder):
    for dt in DTYPES:
        for order in ("C", "F"):
            for conn in (4, 6, 8, 18, 26):
                sq = np.zeros((16, 16), dtype=dt, order=order)
                if dt == "bool":
                    sq[:8, :8] = True
                    sq[8:, 8:] = True
                else:
                    sq[:8, :8] = 8
                    sq[8:, :8] = 9
                    sq[:8, 8:] = 10
                    sq[8:, 8:] = 11
                rec.cc(f"square_{dt}_{order}_{conn}", sq, connectivity=conn)
                rect = np.zeros((16, 13), dtype=dt, order=order)
                if dt == "bool":
                    rect[:8, :8] = True
                else:
                    rect[:8, :8] = 8
                    rect[8:, :8] = 9
                    rect[:8, 8:] = 10
                    rect[8:, 8:] = 11
                rec.cc(f"rect_{dt}_{order}_{conn}", rect, connectivity=conn)
                cross = np.zeros((17, 17), dtype=dt, order=order)
                cross[:, 8] = 1 if dt == "bool" else 5
                cross[8, :] = 1 if dt == "bool" else 6
                rec.cc(f"cross_{dt}_{order}_{conn}", cross, connectivity=conn)
            for conn in (6, 18, 26):
                c3 = np.zeros((11, 12, 13), dtype=dt, order=order)
                c3[5, :, 6] = 1 if dt == "bool" else 3
                c3[:, 6, 6] = 1 if dt == "bool" else 4
                c3[5, 6, :] = 1 if dt == "bool" else 7
                c3[0, 0, 0] = 1 if dt == "bool" else 2
                c3[1, 1, 1] = 1 if dt == "bool" else 2
                c3[10, 11, 12] = 1
                rec.cc(f"cross3d_{dt}_{order}_{conn}", c3, connectivity=conn)
    # diagonal touching squares and an intruder
    for conn in (4, 8, 6, 18, 26):
        d = np.zeros((10, 10), dtype=np.uint32)
        d[0:3, 0:3] = 1
        d[3:6, 3:6] = 1
        d[6:9, 0:3] = 2
        d[9:, 9:] = 1
        rec.cc(f"diag_{conn}", d, connectivity=conn)
        rec.cc(f"diag_bin_{conn}", d, connectivity=conn, binary_image=True)
        d2 = np.copy(d)
        d2[4, 4] = 7
        rec.cc(f"intruder_{conn}", d2, connectivity=conn)
    # degenerate shapes and edge cases
    rec.cc("empty2d", np.zeros((0, 0), dtype=np.uint32))
    rec.cc("empty3d", np.zeros((0, 0, 0), dtype=np.uint32))
    rec.cc("empty_outdtype", np.zeros((0, 3), dtype=np.uint8), out_dtype=np.uint64)
    rec.cc("one_d", np.array([1, 1, 1, 1]))
    rec.cc("one_d_3d", np.array([[[1, 1, 1, 1]]]))
    for conn in (6, 18, 26):
        rec.cc(f"all_zeros_{conn}", np.zeros((7, 8, 9), dtype=np.uint16), connectivity=conn)
        rec.cc(f"all_fg_{conn}", np.full((7, 8, 9), 3, dtype=np.uint16), connectivity=conn)
        rec.cc(f"all_diff_{conn}", np.arange(1, 7 * 8 * 9 + 1, dtype=np.uint32).reshape(7, 8, 9), connectivity=conn)
        rec.cc(f"single_{conn}", np.pad(np.ones((1, 1, 1), np.uint8), 3), connectivity=conn)
    for conn in (4, 8):
        img = np.zeros((5, 6), dtype=np.uint8)
        img[2, 3] = 9
        rec.cc(f"single2d_{conn}", img, connectivity=conn)
    rec.cc("out_dtype_u16_forced", np.ones((4, 4), np.uint8), out_dtype=np.uint16)
    rec.cc("out_dtype_invalid", np.ones((4, 4), np.uint8), out_dtype=np.int32)
    big = np.arange(1, 300 * 300 + 1, dtype=np.uint32).reshape(300, 300)
    rec.cc("out_dtype_too_small", big, out_dtype=np.uint16)
    rec.cc("out_dtype_auto_u32", big)
    rec.cc("max_labels_ignored", np.ones((5, 5), np.uint8), max_labels=1)
    rec.cc("bad_conn_3d", np.ones((3, 3, 3), np.uint8), connectivity=8)
    rec.cc("bad_conn_2d", np.ones((3, 3), np.uint8), connectivity=5)
    rec.cc("bad_periodic", np.ones((3, 3), np.uint8), connectivity=26, periodic_boundary=True)
    # single-row inputs (the special-cased path)
    for conn in (6, 18, 26):
        r3 = np.zeros((3, 4, 9), dtype=np.uint32)
        r3[1, 2, :] = [1, 1, 0, 2, 2, 2, 0, 3, 1]
        rec.cc(f"row_{conn}", r3, connectivity=conn)
        rec.cc(f"row_F_{conn}", np.asfortranarray(r3), connectivity=conn)
    rf = np.zeros((3, 4, 6), dtype=np.float32)
    rf[1, 2, :] = [1.5, 1.5, 0, 2.0, 2.0, -0.0]
    rec.cc("row_float_trunc", rf)
    rp = np.zeros((4, 5), dtype=np.uint8)
    rp[2, :] = [3, 3, 0, 2, 3]
    for conn in (4, 8):
        rec.cc(f"row_periodic_{conn}", rp, connectivity=conn, periodic_boundary=True)
    ru = np.zeros((2, 2, 3), dtype=np.uint64)
    ru[1, 1, :] = [2**63 + 1, 2**63 + 1, 0]
    rec.cc("row_u64_overflow", ru)
    # periodic boundaries
    for seed in range(6):
        rng = np.random.default_rng(100 + seed)
        for conn in (4, 8):
            img = (rng.random((12, 15)) < 0.45).astype(np.uint8) * rng.integers(1, 3, (12, 15)).astype(np.uint8)
            rec.cc(f"periodic2d_{conn}_{seed}", img, connectivity=conn, periodic_boundary=True)
            rec.cc(f"periodic2d_bin_{conn}_{seed}", img, connectivity=conn, periodic_boundary=True, binary_image=True)
        vol = (rng.random((6, 7, 8)) < 0.45).astype(np.uint16) * rng.integers(1, 3, (6, 7, 8)).astype(np.uint16)
        rec.cc(f"periodic3d_{seed}", vol, connectivity=6, periodic_boundary=True)
        rec.cc(f"periodic3d_bin_{seed}", vol, connectivity=6, periodic_boundary=True, binary_image=True)
    # binary stress (checkerboards and their 3D analogues)
    for size in (4, 5, 9):
        cb = (np.indices((size, size)).sum(0) % 2).astype(np.uint8)
        for conn in (4, 8):
            rec.cc(f"checker2d_{conn}_{size}", cb, connectivity=conn, binary_image=True)
        cb3 = (np.indices((size, size, size)).sum(0) % 2).astype(np.uint8)
        for conn in (6, 18, 26):
            rec.cc(f"checker3d_{conn}_{size}", cb3, connectivity=conn, binary_image=True)
    # binary images with multiple foreground values, degenerate shapes
    rec.cc("bin26_row_overflow", np.array([1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1], np.uint8), binary_image=True)
    rec.cc("bin4_row0_values", np.array([[1, 2, 1], [0, 2, 2], [1, 1, 1]], np.uint8), connectivity=4, binary_image=True)
    # special values
    fv = np.zeros((4, 5, 6), dtype=np.float64)
    fv[1, :, :3] = np.nan
    fv[2, :, 2:] = -0.0
    fv[3, 1:, 1:] = 2.5
    rec.cc("float_nan_negzero", fv)
    h = np.zeros((4, 5, 6), dtype=np.float16)
    h[1, :, :] = -0.0
    h[2, 2:, :] = 1.5
    rec.cc("float16_negzero_is_fg", h)


def random_cases(rec: Recorder, n: int, seed: int):
    rng = np.random.default_rng(seed)
    for it in range(n):
        dims = int(rng.integers(1, 4))
        hi = 48 if dims < 3 else 16
        shape = tuple(int(s) for s in rng.integers(1, hi, dims))
        dt = DTYPES[int(rng.integers(0, len(DTYPES)))]
        k = int(rng.integers(1, 6))
        p = float(rng.uniform(0.15, 0.85))
        a = (rng.integers(1, k + 1, shape) * (rng.random(shape) < p)).astype(dt)
        if rng.random() < 0.5:
            a = np.asfortranarray(a)
        conn = int(rng.choice((4, 8, 6, 18, 26) if dims == 2 else (6, 18, 26)))
        kw = dict(connectivity=conn)
        if rng.random() < 0.4:
            kw["binary_image"] = True
        if conn in (4, 8, 6) and rng.random() < 0.3:
            kw["periodic_boundary"] = True
        if rng.random() < 0.2:
            kw["out_dtype"] = [np.uint32, np.uint64][int(rng.integers(0, 2))]
        rec.cc(f"random_{it}", a, **kw)


def epl_cases(rec: Recorder):
    rng = np.random.default_rng(7)
    for dt in DTYPES:
        if dt == "float16":
            continue
        for order in ("C", "F"):
            a = np.array(rng.integers(0, 3, (5, 6, 7)).astype(dt), order=order)
            rec.epl(f"epl_{dt}_{order}", a)
    rec.epl("epl_zeros", np.zeros((3, 3), np.uint8))
    rec.epl("epl_f16_unsupported", np.zeros((3, 3), np.float16))


def stats_cases(rec: Recorder):
    rng = np.random.default_rng(9)
    for dt in ("uint8", "uint16", "uint32", "uint64", "int32", "int64", "bool"):
        for order in ("C", "F"):
            lab = np.array(rng.integers(0, 7, (9, 10, 11)).astype(dt), order=order)
            lab.reshape(-1)[5] = 0
            rec.stats(f"stats3d_{dt}_{order}", lab)
            lab2 = np.array(rng.integers(0, 5, (13, 12)).astype(dt), order=order)
            rec.stats(f"stats2d_{dt}_{order}", lab2)
    lab = np.zeros((10, 12, 14), dtype=np.uint32)
    lab[2:5, 3:7, 1:2] = 3
    lab[6, 0, 13] = 1
    rec.stats("stats_gap_labels", lab)
    rec.stats("stats_slices3d", lab, no_slice_conversion=False)
    rec.stats("stats_slices2d", lab[:, :, 1].copy(), no_slice_conversion=False)
    wide = np.zeros((2, 70000), dtype=np.uint8)
    wide[1, 69990:] = 2
    wide[0, 3] = 1
    rec.stats("stats_big_dim", wide)
    rec.stats("stats_big_dim_slices", wide, no_slice_conversion=False)
    rec.stats("stats_1d", np.array([0, 1, 1, 2], np.uint16))
    rec.stats("stats_empty", np.zeros((0, 3), np.uint32))
    rec.stats("stats_negative", np.array([[0, -1]], np.int32))
    rec.stats("stats_too_large", np.array([[0, 9]], np.uint32))
    rec.stats("stats_float", np.ones((3, 3), np.float32))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CC3D_REFERENCE"), required="CC3D_REFERENCE" not in os.environ,
                    help="the reference source tree (default: $CC3D_REFERENCE)")
    ap.add_argument("--random", type=int, default=700)
    args = ap.parse_args()
    sys.path.insert(0, build_reference(args.ref))
    import fastcc3d as R  # the reference's compiled Cython module

    rec = Recorder(R)
    structured_cases(rec)
    random_cases(rec, args.random, seed=20261203)
    epl_cases(rec)
    stats_cases(rec)
    np.savez_compressed(os.path.join(HERE, "cc3d_golden.npz"), **rec.arrays)
    with open(os.path.join(HERE, "cc3d_golden.json"), "w") as f:
        json.dump({"source": "cc3d 4.0.0 reference, compiled out of tree", "cases": rec.meta}, f, indent=0)
    print(f"{len(rec.meta)} cases written")


if __name__ == "__main__":
    main()
