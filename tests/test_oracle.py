"""The CPU oracle against the reference's golden vectors (and the compiled
reference itself where it is available).  No GPU needed."""
import numpy as np
import pytest

import golden_cases as G
import oracle


@pytest.fixture(scope="module", autouse=True)
def _built():
    oracle.build()


def test_golden_connected_components():
    tally = {"ok": 0, "bg-defect": 0}
    for i, m in G.cases("cc"):
        tally[G.check_cc(i, m, oracle.connected_components)] += 1
    assert tally["ok"] > 1000
    # the documented binary-8 background difference stays rare
    assert tally["bg-defect"] <= 0.05 * (tally["ok"] + tally["bg-defect"])


def test_golden_epl():
    for i, m in G.cases("epl"):
        data = G.input_of(i, m)
        if "exc" in m:
            with pytest.raises(Exception) as ei:
                oracle.estimate_provisional_labels(data)
            assert type(ei.value).__name__ == m["exc"]
        else:
            assert list(oracle.estimate_provisional_labels(data)) == m["epl"], m["name"]


def test_golden_statistics():
    for i, m in G.cases("stats"):
        G.check_stats(i, m, oracle.statistics)


@pytest.mark.skipif(not oracle.have_reference(), reason="reference not compiled here")
@pytest.mark.parametrize("seed", range(4))
def test_port_matches_reference_random(seed):
    rng = np.random.default_rng(seed)
    for _ in range(60):
        dims = int(rng.integers(2, 4))
        shape = tuple(int(s) for s in rng.integers(1, 30 if dims == 2 else 12, dims))
        a = (rng.integers(1, 4, shape) * (rng.random(shape) < rng.uniform(0.2, 0.8))).astype(np.uint16)
        conn = int(rng.choice((4, 8, 6, 18, 26) if dims == 2 else (6, 18, 26)))
        kw = dict(connectivity=conn, binary_image=bool(rng.random() < 0.3),
                  periodic_boundary=bool(conn in (4, 8, 6) and rng.random() < 0.3))
        try:
            r = oracle.connected_components(a, return_N=True, backend="reference", **kw)
        except RuntimeError:
            with pytest.raises(RuntimeError):
                oracle.connected_components(a, return_N=True, **kw)
            continue
        o = oracle.connected_components(a, return_N=True, **kw)
        assert o[1] == r[1]
        if kw["binary_image"] and conn == 8:
            fg = a != 0
            assert np.array_equal(o[0][fg], r[0][fg])
        else:
            assert np.array_equal(o[0], r[0])


@pytest.mark.skipif(not oracle.have_reference(), reason="reference not compiled here")
@pytest.mark.parametrize("conn", [26, 18, 6])
def test_port_matches_reference_voronoi(conn):
    """Cell-like volumes (Voronoi with salt), where most voxels repeat the one
    below, behind or to the left: the 26-connected shortcuts of the port."""
    from cc3d_gb300 import synth
    for it, dt in enumerate((np.uint16, np.uint32, np.float32)):
        vol = synth.voronoi_volume((37, 45, 70), 30 + 40 * it, 60000, seed=conn + it, dtype=dt, salt=0.03)
        if it == 1:
            vol = np.asfortranarray(vol)
        for binary in (False, True):
            o = oracle.connected_components(vol, connectivity=conn, binary_image=binary, return_N=True)
            r = oracle.connected_components(vol, connectivity=conn, binary_image=binary, return_N=True,
                                            backend="reference")
            assert o[1] == r[1] and o[0].dtype == r[0].dtype and np.array_equal(o[0], r[0]), (dt, binary)


def _numpy_statistics(labels):
    """Independent numpy tables for statistics: exact integer reductions."""
    a = labels if labels.ndim >= 2 else labels[:, None]
    N = int(a.max())
    lab = a.astype(np.int64).reshape(-1)
    coords = [c.reshape(-1) for c in np.indices(a.shape, dtype=np.int64)]
    counts = np.bincount(lab, minlength=N + 1)
    bdt = np.uint32 if any(s > 65535 for s in a.shape) else np.uint16
    bb = np.zeros((N + 1, 2 * a.ndim), dtype=bdt)
    cent = np.full((N + 1, a.ndim), np.nan)
    for ax in range(a.ndim):
        mins = np.full(N + 1, np.iinfo(bdt).max, np.int64)
        maxs = np.zeros(N + 1, np.int64)
        np.minimum.at(mins, lab, coords[ax])
        np.maximum.at(maxs, lab, coords[ax])
        bb[:, 2 * ax], bb[:, 2 * ax + 1] = mins, maxs
        sums = np.zeros(N + 1, np.int64)
        np.add.at(sums, lab, coords[ax])
        present = counts > 0
        cent[present, ax] = sums[present].astype(np.float64) / counts[present]
    return counts.astype(np.uint32), bb, cent


@pytest.mark.parametrize("seed", range(3))
def test_statistics_pass_matches_numpy(seed):
    rng = np.random.default_rng(50 + seed)
    for it in range(40):
        dims = int(rng.integers(1, 4))
        shape = tuple(int(s) for s in rng.integers(1, 20 if dims == 3 else 60, dims))
        if it == 0:
            shape = (70000,)  # an axis longer than 65535: uint32 boxes
        dt = (np.uint8, np.uint16, np.uint32, np.uint64, np.int32)[it % 5]
        strided = dims == 3 and rng.random() < 0.3
        final = int(np.prod(shape)) if not strided else shape[0] * ((shape[1] + 1) // 2) * shape[2]
        a = rng.integers(0, max(1, min(final, 40)), shape).astype(dt)
        if dims > 1 and rng.random() < 0.5:
            a = np.asfortranarray(a)
        if strided:
            a = a[:, ::2, :]  # neither C nor Fortran contiguous
        got = oracle.statistics(a, no_slice_conversion=True)
        counts, bb, cent = _numpy_statistics(np.asarray(a))
        assert np.array_equal(got["voxel_counts"], counts), (shape, dt)
        assert got["bounding_boxes"].dtype == bb.dtype and np.array_equal(got["bounding_boxes"], bb), (shape, dt)
        assert np.array_equal(got["centroids"], cent, equal_nan=True), (shape, dt)
