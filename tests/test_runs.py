"""runs, draw and each (cc3d/fastcc3d.pyx:1258-1372): the oracle's
restatement and the GPU path against golden outputs of the reference
(tests/golden/make_golden_runs.py), plus the reference's own each() property
(automated_test.py test_each) on the GPU."""
import json
import os

import numpy as np
import pytest

import oracle

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _cases():
    with open(os.path.join(HERE, "cc3d_runs.json")) as f:
        meta = json.load(f)
    arrays = np.load(os.path.join(HERE, "cc3d_runs.npz"))
    for i, m in enumerate(meta):
        data = arrays[f"in{i}"]
        data = np.asfortranarray(data) if m["order"] == "F" else np.ascontiguousarray(data)
        if "error" in m:
            yield i, m, data, None, None
            continue
        exp = {}
        for lab, a, b in zip(arrays[f"lab{i}"].tolist(), arrays[f"start{i}"].tolist(),
                             arrays[f"end{i}"].tolist()):
            exp.setdefault(int(lab), []).append((a, b))
        yield i, m, data, exp, arrays[f"each{i}"].tolist()


def _check(fn, i, m, data, exp):
    if exp is None:
        with pytest.raises(IndexError):
            fn(data)
        return
    got = fn(data)
    assert list(got.keys()) == list(exp.keys()), (i, m)
    for k in exp:
        assert [tuple(map(int, r)) for r in got[k]] == exp[k], (i, m, k)


def test_oracle_runs_match_reference():
    n = 0
    for i, m, data, exp, _ in _cases():
        if exp is None:
            with pytest.raises(IndexError):
                oracle.runs(data)
        else:
            _check(oracle.runs, i, m, data, exp)
        n += 1
    assert n >= 80


def test_draw_matches_reference_rules():
    import cc3d_gb300.graphs as G
    img = np.zeros((4, 5), np.uint16, order="F")
    G.draw(7, [(0, 3), (10, 12)], img)
    flat = img.reshape(-1, order="F")
    assert flat[:3].tolist() == [7, 7, 7] and flat[10:12].tolist() == [7, 7] and int(flat.sum()) == 35
    with pytest.raises(RuntimeError):
        G.draw(1, [(5, 25)], img)
    with pytest.raises(RuntimeError):
        G.draw(1, [(3, 3)], img)
    with pytest.raises(TypeError):
        G.draw(1, [(0, 1)], np.zeros(4, np.int32))
    b = np.zeros(6, bool)
    G.draw(5, [(1, 3)], b)
    assert b.tolist() == [False, True, True, False, False, False]
    strided = np.zeros((6, 6), np.uint8)[::2]
    G.draw(3, [(0, 4)], strided)  # written through a copy, as in the reference
    assert int(strided.sum()) == 0


@pytest.fixture(scope="module")
def cc3d():
    import __graft_entry__ as entry
    entry.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return entry.package()


@pytest.mark.gpu
def test_gpu_runs_and_each_match_reference(cc3d):
    n = 0
    for i, m, data, exp, each_keys in _cases():
        if exp is None:
            with pytest.raises(IndexError):
                cc3d.runs(data)
            continue
        _check(cc3d.runs, i, m, data, exp)
        assert [k for k, _ in cc3d.each(data)] == each_keys, (i, m)
        n += 1
    assert n >= 70


@pytest.mark.gpu
def test_gpu_runs_torch_input(cc3d):
    import torch
    rng = np.random.default_rng(3)
    a = rng.integers(0, 5, (33, 20, 9)).astype(np.uint32)
    got = cc3d.runs(torch.from_numpy(a).cuda())
    exp = oracle.runs(a)
    assert list(got.keys()) == list(exp.keys())
    assert all(got[k] == exp[k] for k in exp)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", (np.uint8, np.uint16, np.uint32, np.uint64))
@pytest.mark.parametrize("order", ("C", "F"))
@pytest.mark.parametrize("in_place", (True, False))
@pytest.mark.parametrize("dims", (1, 2, 3))
def test_gpu_each(cc3d, dtype, order, in_place, dims):
    rng = np.random.default_rng(dims * 10 + (order == "F"))
    labels = rng.integers(0, 3, [128] * dims).astype(dtype)
    labels = np.asfortranarray(labels) if order == "F" else labels
    seen = []
    for label, img in cc3d.each(labels, binary=False, in_place=in_place):
        assert np.all(img == (label * (labels == label)))
        seen.append(label)
    assert seen == [1, 2]
    for label, img in cc3d.each(labels, binary=True, in_place=in_place):
        assert np.all(img == (labels == label))
