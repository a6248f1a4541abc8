"""voxel_connectivity_graph and color_connectivity_graph
(cc3d/fastcc3d.pyx:941-1178): the oracle's restatements on CPU and the GPU
path, against golden outputs of the reference
(tests/golden/make_golden_vcg.py), plus larger seeded volumes against the
oracle."""
import json
import os

import numpy as np
import pytest

import oracle

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _errors():
    return {"TypeError": TypeError, "ValueError": ValueError, "DimensionError": Exception}


def _cases():
    with open(os.path.join(HERE, "cc3d_vcg.json")) as f:
        meta = json.load(f)
    arrays = np.load(os.path.join(HERE, "cc3d_vcg.npz"))
    for i, m in enumerate(meta):
        data = arrays[f"in{i}"]
        data = np.asfortranarray(data) if m["order"] == "F" else np.ascontiguousarray(data)
        yield i, m, data, (arrays[f"out{i}"] if f"out{i}" in arrays.files else None)


def _check(mod, i, m, data, exp):
    fn = mod.voxel_connectivity_graph if m["kind"] == "vcg" else mod.color_connectivity_graph
    kw = dict(m["kwargs"])
    if "error" in m:
        with pytest.raises(_errors()[m["error"]]) as ei:
            fn(data, **kw)
        if m["error"] == "DimensionError":
            assert type(ei.value).__name__ == "DimensionError"
        return
    res = fn(data, **kw)
    if m["kind"] == "ccg" and kw.get("return_N"):
        res, n = res
        assert int(n) == m["N"], (i, m, n)
    got = res.cpu().numpy() if hasattr(res, "cpu") else np.asarray(res)
    assert str(got.dtype) == m["out_dtype"] and got.shape == exp.shape, (i, m, got.dtype, got.shape)
    assert np.array_equal(got, exp), (i, m)


def test_oracle_graphs_match_reference():
    n = 0
    for i, m, data, exp in _cases():
        _check(oracle, i, m, data, exp)
        n += 1
    assert n >= 230


@pytest.fixture(scope="module")
def cc3d():
    import __graft_entry__ as entry
    entry.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return entry.package()


@pytest.mark.gpu
def test_gpu_graphs_match_reference(cc3d):
    for i, m, data, exp in _cases():
        _check(cc3d, i, m, data, exp)


@pytest.mark.gpu
def test_gpu_graphs_device_tensors(cc3d):
    import torch
    rng = np.random.default_rng(5)
    a = rng.integers(0, 3, (70, 45, 33)).astype(np.uint16)
    for conn in (26, 18, 6):
        exp = oracle.voxel_connectivity_graph(a, connectivity=conn)
        got = cc3d.voxel_connectivity_graph(torch.from_numpy(a).cuda(), connectivity=conn)
        assert got.is_cuda and tuple(got.shape) == exp.shape and np.array_equal(got.cpu().numpy(), exp)
    v = oracle.voxel_connectivity_graph(a, connectivity=26)
    exp, en = oracle.color_connectivity_graph(v, connectivity=26, return_N=True)
    got, n = cc3d.color_connectivity_graph(torch.from_numpy(v).cuda(), connectivity=26, return_N=True)
    assert got.is_cuda and n == en and np.array_equal(got.cpu().numpy(), exp)


@pytest.mark.gpu
@pytest.mark.parametrize("shape,conn,dtype,p", [
    ((160, 150, 40), 26, np.uint32, 0.55), ((160, 150, 40), 6, np.uint8, 0.6), ((700, 600), 8, np.uint8, 0.5),
    ((700, 600), 4, np.uint32, 0.6), ((96, 100, 70), 26, np.uint32, 0.85)])
def test_gpu_color_graph_random_bits(cc3d, shape, conn, dtype, p):
    """Random (asymmetric) bitfields spanning many tiles."""
    rng = np.random.default_rng(sum(shape) + conn)
    bits = 26 if dtype == np.uint32 else 8
    v = np.zeros(shape, np.uint64)
    for b in range(bits):
        v |= (rng.random(shape) < p).astype(np.uint64) << np.uint64(b)
    v = v.astype(dtype)
    exp, en = oracle.color_connectivity_graph(v, connectivity=conn, return_N=True)
    got, n = cc3d.color_connectivity_graph(v, connectivity=conn, return_N=True)
    assert n == en and np.array_equal(got, exp)


@pytest.mark.gpu
def test_gpu_vcg_round_trip_equals_labelling(cc3d):
    """Colouring the graph of a labelled volume joins exactly the voxels that
    share a label and touch: its partition is that of connected_components
    with every value (0 included) a label."""
    rng = np.random.default_rng(9)
    a = (rng.integers(1, 4, (120, 90, 50))).astype(np.uint32)
    v = cc3d.voxel_connectivity_graph(a, connectivity=26)
    col, n = cc3d.color_connectivity_graph(v, connectivity=26, return_N=True)
    lab, N = cc3d.connected_components(np.asfortranarray(a), connectivity=26, return_N=True)
    assert n == N and np.array_equal(col, lab)
