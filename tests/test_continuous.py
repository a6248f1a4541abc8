"""Continuous-value labelling (delta != 0; cc3d/cc3d_continuous.hpp:90-392):
the oracle's restatement on CPU and the GPU path, against golden outputs of
the reference (tests/golden/make_golden_continuous.py), plus larger seeded
volumes against the oracle."""
import json
import os

import numpy as np
import pytest

import oracle

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_ERRORS = {"OverflowError": OverflowError, "TypeError": TypeError, "ValueError": ValueError}


def _cases():
    with open(os.path.join(HERE, "cc3d_continuous.json")) as f:
        meta = json.load(f)
    arrays = np.load(os.path.join(HERE, "cc3d_continuous.npz"))
    for i, m in enumerate(meta):
        data = arrays[f"in{i}"]
        data = np.asfortranarray(data) if m["order"] == "F" else np.ascontiguousarray(data)
        yield i, m, data, (arrays[f"out{i}"] if "out" + str(i) in arrays.files else None)


def _check(fn, i, m, data, exp):
    kw = dict(m["kwargs"])
    if "error" in m:
        with pytest.raises(_ERRORS[m["error"]]):
            fn(data, **kw)
        return
    out, N = fn(data, return_N=True, **kw)
    out = out.cpu().numpy() if hasattr(out, "cpu") else np.asarray(out)
    assert str(out.dtype) == m["out_dtype"], (i, m)
    assert int(N) == m["N"], (i, m, int(N))
    assert out.shape == exp.shape and np.array_equal(out, exp), (i, m)


def test_oracle_matches_reference_continuous():
    oracle.build()
    n = 0
    for i, m, data, exp in _cases():
        _check(lambda d, **kw: oracle.connected_components(d, **kw), i, m, data, exp)
        n += 1
    assert n >= 160


@pytest.mark.skipif(not oracle.have_reference(), reason="reference sources not present")
def test_reference_build_matches_reference_continuous():
    oracle.build()
    for i, m, data, exp in _cases():
        _check(lambda d, **kw: oracle.connected_components(d, backend="reference", **kw), i, m, data, exp)


@pytest.fixture(scope="module")
def cc3d():
    import __graft_entry__ as entry
    entry.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return entry.package()


@pytest.mark.gpu
def test_gpu_continuous_golden_host(cc3d):
    for i, m, data, exp in _cases():
        _check(cc3d.connected_components, i, m, data, exp)


@pytest.mark.gpu
def test_gpu_continuous_golden_device(cc3d):
    import torch
    for i, m, data, exp in _cases():
        if data.dtype in (np.float16,) or "error" in m:
            continue
        src = np.ascontiguousarray(data)
        out, N = cc3d.connected_components(torch.from_numpy(src).cuda(), return_N=True, **m["kwargs"])
        assert out.is_cuda
        # a C-ordered copy of an F-ordered case is labelled in its own memory
        # order (the 2D 8-connected decision tree even partitions differently)
        e, Ne = (exp, m["N"]) if m["order"] == "C" else oracle.connected_components(
            src, return_N=True, **m["kwargs"])
        assert int(N) == Ne and np.array_equal(out.cpu().numpy(), e), (i, m)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,shape,conn,delta", [
    ("uint16", (96, 110, 120), 26, 3),
    ("float32", (100, 90, 130), 18, 0.5),
    ("uint8", (120, 100, 90), 6, 2),
    ("float64", (70, 80, 90), 26, 1.25),
    ("uint32", (1, 700, 900), 26, 5),
    ("uint16", (1500, 1300), 8, 40),
    ("float32", (1100, 1250), 8, 0.8),
    ("int16", (1200, 1000), 4, 3),
    ("uint16", (700, 650), 8, 9),
    ("uint8", (640, 900), 8, 25),
    ("float32", (500, 700), 8, 9.5),
])
def test_gpu_continuous_random_vs_oracle(cc3d, dtype, shape, conn, delta):
    rng = np.random.default_rng(sum(shape) * 131 + conn)
    if conn == 8 and delta in (9, 25, 9.5):
        # a few levels 10 apart: the 2D 8-connected image-span shortcut fires often
        a = (rng.integers(0, 4, shape) * 10).astype(dtype)
    elif np.dtype(dtype).kind == "f":
        # smooth field + noise: long chains of matching neighbours
        base = rng.normal(0, 1, [(s + 7) // 8 for s in shape])
        a = np.kron(base, np.ones([8] * len(shape)))[tuple(slice(0, s) for s in shape)]
        a = (a * 4 + rng.normal(0, 0.3, shape)) * (rng.random(shape) < 0.9)
        a = a.astype(dtype)
    else:
        a = rng.integers(0, 60, shape).astype(dtype)
    if rng.random() < 0.5:
        a = np.asfortranarray(a)
    exp, N = oracle.connected_components(a, connectivity=conn, delta=delta, return_N=True)
    got, Ng = cc3d.connected_components(a, connectivity=conn, delta=delta, return_N=True)
    assert Ng == N and got.dtype == exp.dtype and np.array_equal(got, exp)
