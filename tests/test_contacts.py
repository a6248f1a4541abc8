"""contacts and region_graph (cc3d/fastcc3d.pyx:1180-1256) on the GPU against
golden outputs of the reference (tests/golden/make_golden_contacts.py)."""
import json
import os

import numpy as np
import pytest

import __graft_entry__ as entry

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def cc3d():
    entry.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return entry.package()


def _cases():
    with open(os.path.join(HERE, "cc3d_contacts.json")) as f:
        meta = json.load(f)
    arrays = np.load(os.path.join(HERE, "cc3d_contacts.npz"))
    for i, m in enumerate(meta):
        kw = dict(m["kwargs"])
        if "anisotropy" in kw:
            kw["anisotropy"] = tuple(kw["anisotropy"])
        pairs = [tuple(int(v) for v in p) for p in arrays[f"pairs{i}"]]
        exp = dict(zip(pairs, arrays[f"vals{i}"].tolist()))
        yield i, m, arrays[f"in{i}"], exp, kw


def test_contacts_match_reference(cc3d):
    import torch
    n = 0
    for i, m, data, exp, kw in _cases():
        got = cc3d.contacts(data, **kw)
        assert set(got) == set(exp), (i, m)
        aniso = kw.get("anisotropy", (1, 1, 1))
        exact = all(float(a).is_integer() for a in aniso)
        for k, v in exp.items():
            if exact:
                assert got[k] == v, (i, m, k, got[k], v)
            else:  # float32 sums taken in another order
                assert got[k] == pytest.approx(v, rel=1e-5, abs=1e-6), (i, m, k)
        if i % 5 == 0:  # the same on a CUDA tensor
            t = torch.from_numpy(np.ascontiguousarray(data).view(
                {1: np.uint8, 2: np.int16, 4: np.int32, 8: np.int64}[data.dtype.itemsize])).cuda()
            if data.dtype.itemsize > 1:
                assert set(cc3d.contacts(t, **kw)) == set(exp), (i, m)
        n += 1
    assert n >= 200


def test_region_graph(cc3d):
    for i, m, data, exp, kw in _cases():
        if kw.get("surface_area", True) and "anisotropy" not in kw:
            assert cc3d.region_graph(data, connectivity=kw["connectivity"]) == set(exp), (i, m)


def test_errors_match_reference(cc3d):
    with pytest.raises(ValueError):
        cc3d.contacts(np.ones((4, 4, 4), np.uint8), connectivity=10)
    with pytest.raises(RuntimeError):
        cc3d.contacts(np.ones((4, 4, 2), np.uint8), connectivity=8)
