"""Host logic of dust and largest_k (cc3d_gb300/filters.py) against the
reference's golden outputs, without a GPU: the labelling and statistics are
the oracle's and the two voxel-wise rewrites are numpy stand-ins, so what is
checked is the per-label decision logic, dtypes, return forms and memory
order.  The GPU path itself is checked in test_filters.py."""
import json
import os

import numpy as np
import pytest

import oracle

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture()
def filters(monkeypatch):
    oracle.build()
    import cc3d_gb300.filters as F

    def remap(cc_labels, table, out_dtype, order="C"):
        out = table[np.asarray(cc_labels).astype(np.int64)]
        if out_dtype == np.bool_:
            out = out.astype(np.bool_)
        return np.asfortranarray(out) if order == "F" else np.ascontiguousarray(out)

    def zero_labels(img, cc_labels, zero):
        img[zero[np.asarray(cc_labels).astype(np.int64)].astype(bool)] = 0

    monkeypatch.setattr(F, "connected_components", lambda img, **kw: oracle.connected_components(img, **kw))
    monkeypatch.setattr(F, "statistics", lambda lab, no_slice_conversion=False:
                        oracle.statistics(lab, no_slice_conversion=no_slice_conversion))
    monkeypatch.setattr(F, "_remap", remap)
    monkeypatch.setattr(F, "_zero_labels", zero_labels)
    return F


def test_filter_logic_matches_reference(filters):
    with open(os.path.join(HERE, "cc3d_filters.json")) as f:
        meta = json.load(f)
    arrays = np.load(os.path.join(HERE, "cc3d_filters.npz"))
    for i, m in enumerate(meta):
        kw = dict(m["kwargs"])
        if isinstance(kw.get("threshold"), list):
            kw["threshold"] = tuple(kw["threshold"])
        fn = filters.dust if m["kind"] == "dust" else filters.largest_k
        res = fn(np.copy(arrays[f"in{i}"], order="A"), return_N=True, **kw)
        out, N = res if isinstance(res, tuple) else (res, None)
        exp = arrays[f"out{i}"]
        assert str(out.dtype) == m["out_dtype"], (i, m)
        assert np.array_equal(out, exp), (i, m)
        assert (N if N is None else int(N)) == m["N"], (i, m)
        order = "F" if out.flags.f_contiguous and not out.flags.c_contiguous else "C"
        if out.ndim > 1 and min(out.shape) > 1:
            assert order == m["out_order"], (i, m, order)
