"""Host-side checks that need no GPU: the C-ABI library loads and exports every
entry point its header declares, and the front end validates its arguments
before it touches the device."""
import os
import re

import numpy as np
import pytest

import __graft_entry__ as entry

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def cc3d():
    entry.build()
    return entry.package()


def declared_symbols():
    with open(os.path.join(ROOT, "include", "cc3d_gpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(cc3d_gpu_\w+)\s*\(", text)))


def test_library_exports_header_symbols(cc3d):
    lib = cc3d._native.load()
    names = declared_symbols()
    assert len(names) >= 7
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(cc3d._native.EXPORTED)
    assert b"sm_103a" in lib.cc3d_gpu_version()


def test_validation_matches_reference(cc3d):
    with pytest.raises(cc3d.DimensionError):
        cc3d.connected_components(np.zeros((2, 2, 2, 2), np.uint8))
    with pytest.raises(ValueError):
        cc3d.connected_components(np.zeros((3, 3, 3), np.uint8), connectivity=8)
    with pytest.raises(ValueError):
        cc3d.connected_components(np.zeros((3, 3), np.uint8), connectivity=5)
    with pytest.raises(ValueError):
        cc3d.connected_components(np.zeros((3, 3), np.uint8), connectivity=26, periodic_boundary=True)
    with pytest.raises(ValueError):
        cc3d.connected_components(np.zeros((3, 3), np.uint8), connectivity=4, periodic_boundary=True, delta=1)


def test_empty_inputs_need_no_device(cc3d):
    out = cc3d.connected_components(np.zeros((0, 0), np.uint32))
    assert out.size == 0 and out.dtype == np.uint32
    out, N = cc3d.connected_components(np.zeros((0, 4, 0), np.uint8), return_N=True, out_dtype=np.uint64)
    assert N == 0 and out.dtype == np.uint64
    s = cc3d.statistics(np.zeros((0, 3), np.uint32))
    assert s == {"voxel_counts": None, "bounding_boxes": None, "centroids": None}


def test_contiguity_rules_match_numpy(cc3d):
    from cc3d_gb300.api import _contig_flags
    rng = np.random.default_rng(0)
    for _ in range(200):
        shape = tuple(int(v) for v in rng.integers(1, 4, int(rng.integers(1, 4))))
        a = np.zeros(shape, np.uint8, order="C" if rng.random() < 0.5 else "F")
        if a.ndim > 1 and rng.random() < 0.3:
            a = a[::2]
        if a.ndim > 1 and rng.random() < 0.3:
            a = a.transpose()
        st = tuple(s // a.itemsize for s in a.strides)
        assert _contig_flags(a.shape, st) == (a.flags.c_contiguous, a.flags.f_contiguous), (a.shape, a.strides)


def test_widened_functions_validate_before_the_device(cc3d):
    """The argument errors of the reference's other functions, raised by the
    front end before any device call (cases from the golden fixtures)."""
    import json
    here = os.path.join(ROOT, "tests", "golden")
    errors = {"OverflowError": OverflowError, "TypeError": TypeError, "ValueError": ValueError}
    for name, fn_of in (("cc3d_continuous", lambda m: cc3d.connected_components),
                        ("cc3d_vcg", lambda m: (cc3d.voxel_connectivity_graph if m["kind"] == "vcg"
                                                else cc3d.color_connectivity_graph))):
        with open(os.path.join(here, name + ".json")) as f:
            meta = json.load(f)
        arrays = np.load(os.path.join(here, name + ".npz"))
        n = 0
        for i, m in enumerate(meta):
            if "error" not in m:
                continue
            data = arrays[f"in{i}"]
            exc = cc3d.DimensionError if m["error"] == "DimensionError" else errors[m["error"]]
            with pytest.raises(exc):
                fn_of(m)(data, **m["kwargs"])
            n += 1
        assert n >= 5, name
    with pytest.raises(ValueError):
        cc3d.connected_components_stack([np.ones((2, 2, 2), np.uint8)], connectivity=18)
