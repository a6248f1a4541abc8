"""dust and largest_k (cc3d/__init__.py:71-155, 199-279) on the GPU against
golden outputs of the reference (tests/golden/make_golden_filters.py), for
numpy inputs (host path) and CUDA tensors (device path)."""
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
    with open(os.path.join(HERE, "cc3d_filters.json")) as f:
        meta = json.load(f)
    arrays = np.load(os.path.join(HERE, "cc3d_filters.npz"))
    for i, m in enumerate(meta):
        kw = dict(m["kwargs"])
        if isinstance(kw.get("threshold"), list):
            kw["threshold"] = tuple(kw["threshold"])
        yield i, m, arrays[f"in{i}"], arrays[f"out{i}"], kw


def _call(cc3d, kind, data, kw):
    fn = cc3d.dust if kind == "dust" else cc3d.largest_k
    res = fn(data, return_N=True, **kw)
    return res if isinstance(res, tuple) else (res, None)


def test_filters_host_match_reference(cc3d):
    n = 0
    for i, m, data, exp, kw in _cases():
        out, N = _call(cc3d, m["kind"], np.copy(data, order="A"), kw)
        assert isinstance(out, np.ndarray), (i, m)
        assert str(out.dtype) == m["out_dtype"], (i, m, out.dtype)
        assert out.shape == exp.shape and np.array_equal(out, exp), (i, m)
        assert (N if N is None else int(N)) == m["N"], (i, m, N)
        n += 1
    assert n >= 380


def test_filters_device_match_reference(cc3d):
    import torch
    for i, m, data, exp, kw in _cases():
        # the same memory layout as the host input: the binary 4-connected
        # relation of the reference depends on which axis is fastest in memory
        t = torch.from_numpy(data).cuda()
        assert t.stride() == torch.from_numpy(data).stride()
        out, N = _call(cc3d, m["kind"], t, kw)
        assert out.is_cuda, (i, m)
        got = out.cpu().numpy()
        assert str(got.dtype) == m["out_dtype"], (i, m, got.dtype)
        assert np.array_equal(got, exp), (i, m)
        assert (N if N is None else int(N)) == m["N"], (i, m, N)
