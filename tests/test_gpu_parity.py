"""Parity of the GPU path with the reference (golden vectors) and with the
oracle (seeded volumes), through the public API and therefore the C ABI.
Labels, N and dtypes must match bit for bit."""
import numpy as np
import pytest

import golden_cases as G
import oracle
import __graft_entry__ as entry

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["list/8x8", "runs/8x8", "list/4x16", "runs/4x16", "list/16x4",
                                        "runs/16x4", "list/8x8/plain", "runs/16x4/plain"])
def cc3d(request):
    """The package with one tile-pass configuration selected: every parity
    test runs once per configuration."""
    entry.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    pkg = entry.package()
    prev = pkg.set_tile_pass(request.param)
    yield pkg
    pkg.set_tile_pass(prev)


def _on_device(fn):
    import torch

    def run(data, **kw):
        t = torch.from_numpy(np.asarray(data)).cuda()
        res = fn(t, **kw)
        if isinstance(res, tuple):
            out, N = res
            assert out.is_cuda
            return out.cpu().numpy(), N
        return res
    return run


def test_golden_connected_components_host(cc3d):
    tally = {"ok": 0, "bg-defect": 0}
    for i, m in G.cases("cc"):
        tally[G.check_cc(i, m, cc3d.connected_components)] += 1
    assert tally["ok"] > 1000


def test_golden_connected_components_device(cc3d):
    fn = _on_device(cc3d.connected_components)
    for i, m in G.cases("cc"):
        G.check_cc(i, m, fn)


def test_golden_epl(cc3d):
    for i, m in G.cases("epl"):
        data = G.input_of(i, m)
        if "exc" in m:
            with pytest.raises(Exception) as ei:
                cc3d.estimate_provisional_labels(data)
            assert type(ei.value).__name__ == m["exc"]
        else:
            assert list(cc3d.estimate_provisional_labels(data)) == m["epl"], m["name"]


def test_golden_statistics(cc3d):
    for i, m in G.cases("stats"):
        G.check_stats(i, m, cc3d.statistics)


def test_golden_statistics_device(cc3d):
    import torch
    for i, m in G.cases("stats"):
        data = G.input_of(i, m)
        if "exc" in m or m.get("empty") or not m["no_slice_conversion"] or data.dtype == np.float32:
            continue
        s = cc3d.statistics(torch.from_numpy(data).cuda(), no_slice_conversion=True)
        e = oracle.statistics(data, no_slice_conversion=True)
        assert np.array_equal(s["voxel_counts"].cpu().numpy(), e["voxel_counts"]), m["name"]
        assert np.array_equal(s["bounding_boxes"].cpu().numpy(), e["bounding_boxes"]), m["name"]
        assert np.array_equal(s["centroids"].cpu().numpy(), e["centroids"], equal_nan=True), m["name"]


DTYPES = [np.uint8, np.int8, np.uint16, np.int16, np.uint32, np.int32, np.uint64, np.int64,
          np.float16, np.float32, np.float64, np.bool_]


def _random_case(rng, maxdim):
    dims = int(rng.integers(2, 4))
    shape = tuple(int(s) for s in rng.integers(1, maxdim, dims))
    dt = DTYPES[int(rng.integers(0, len(DTYPES)))]
    k = int(rng.integers(1, 5))
    a = (rng.integers(1, k + 1, shape) * (rng.random(shape) < rng.uniform(0.2, 0.9))).astype(dt)
    if rng.random() < 0.4:
        a = np.asfortranarray(a)
    conn = int(rng.choice((4, 8, 6, 18, 26) if dims == 2 else (6, 18, 26)))
    kw = dict(connectivity=conn, binary_image=bool(rng.random() < 0.35),
              periodic_boundary=bool(conn in (4, 8, 6) and rng.random() < 0.35))
    return a, kw


def _compare(cc3d_fn, a, kw):
    try:
        exp = oracle.connected_components(a, return_N=True, **kw)
    except RuntimeError:
        with pytest.raises(RuntimeError):
            cc3d_fn(a, return_N=True, **kw)
        return
    got = cc3d_fn(a, return_N=True, **kw)
    assert got[1] == exp[1], (a.shape, a.dtype, kw, got[1], exp[1])
    g = np.asarray(got[0])
    assert g.dtype == exp[0].dtype and g.shape == exp[0].shape
    assert np.array_equal(g, exp[0]), (a.shape, a.dtype, kw)


@pytest.mark.parametrize("seed", range(6))
def test_random_small_vs_oracle(cc3d, seed):
    rng = np.random.default_rng(1000 + seed)
    for _ in range(50):
        a, kw = _random_case(rng, 40)
        _compare(cc3d.connected_components, a, kw)


@pytest.mark.parametrize("seed", range(3))
def test_random_multitile_vs_oracle(cc3d, seed):
    """Volumes spanning several tiles in every axis, dense small label sets so
    that many components cross tile faces."""
    rng = np.random.default_rng(2000 + seed)
    fn_dev = _on_device(cc3d.connected_components)
    for it in range(12):
        a, kw = _random_case(rng, 140)
        _compare(cc3d.connected_components if it % 2 else fn_dev, a, kw)


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 1, 257), (257, 1, 1), (1, 257, 1), (3, 70, 33),
                                   (17, 9, 65), (9, 8, 32), (8, 8, 31), (16, 16, 64), (2, 130, 2)])
@pytest.mark.parametrize("conn", [6, 18, 26])
def test_tile_edges(cc3d, shape, conn):
    rng = np.random.default_rng(sum(shape) * conn)
    for p in (0.5, 0.9, 1.0):
        a = (rng.random(shape) < p).astype(np.uint16) * rng.integers(1, 3, shape).astype(np.uint16)
        _compare(cc3d.connected_components, a, dict(connectivity=conn))
        _compare(cc3d.connected_components, a, dict(connectivity=conn, binary_image=True))
        if conn == 6:
            _compare(cc3d.connected_components, a, dict(connectivity=6, periodic_boundary=True))


def test_single_giant_component(cc3d):
    """One component crossing every tile (deep global union chains)."""
    a = np.ones((96, 200, 300), dtype=np.uint8)
    a[::2, ::3, 5] = 0
    out, N = cc3d.connected_components(a, return_N=True)
    assert N == 1 and out.dtype == np.uint16 and np.all(out[a != 0] == 1)
    spiral = np.zeros((1, 301, 301), np.uint8)
    spiral[0, ::4, :] = 1
    spiral[0, :, 0] = 1
    spiral[0, :, -1] = 1
    _compare(cc3d.connected_components, spiral[0], dict(connectivity=4))


def test_voronoi_128_config(cc3d):
    from cc3d_gb300 import synth
    vol = synth.voronoi_volume((128, 128, 128), n_seeds=256, label_max=1 << 20, seed=0)
    for conn in (26, 18, 6):
        _compare(cc3d.connected_components, vol, dict(connectivity=conn))
        _compare(_on_device(cc3d.connected_components), vol, dict(connectivity=conn))


def test_repeatable_under_concurrency(cc3d):
    """The same volume labelled many times gives identical labels (a check on
    the lock-free union-finds), and equals the oracle."""
    import torch
    from cc3d_gb300 import synth
    vol = synth.voronoi_volume((160, 192, 224), n_seeds=600, label_max=1 << 20, seed=11)
    exp, eN = oracle.connected_components(vol, connectivity=26, return_N=True)
    dev = torch.from_numpy(vol).cuda()
    for _ in range(12):
        out, N = cc3d.connected_components(dev, connectivity=26, return_N=True)
        assert N == eN
        assert np.array_equal(out.cpu().numpy(), exp)
    b = synth.bernoulli_volume((128, 160, 192), 0.3116, seed=5)
    expb = oracle.connected_components(b, connectivity=6, binary_image=True, return_N=True)
    devb = torch.from_numpy(b).cuda()
    for _ in range(6):
        out, N = cc3d.connected_components(devb, connectivity=6, binary_image=True, return_N=True)
        assert N == expb[1]
        assert np.array_equal(out.cpu().numpy(), expb[0])


TMA_DTYPES = [np.uint8, np.uint16, np.uint32, np.uint64, np.float32, np.float64]


@pytest.mark.parametrize("dtype", TMA_DTYPES)
def test_tma_box_edges(cc3d, dtype):
    """Rows whose byte length is a multiple of 16 take the TMA box copy: x
    extents that end inside a tile, volumes narrower than the box padding,
    single planes and rows; each against the oracle, plus the same volume at a
    base address that is not 16-byte aligned (plain loads)."""
    import torch
    per16 = 16 // np.dtype(dtype).itemsize
    rng = np.random.default_rng(per16 * 7 + np.dtype(dtype).itemsize)
    shapes = [(5, 9, per16), (3, 11, 3 * per16), (4, 17, 2 * 32 + per16), (2, 3, 32), (1, 70, 5 * per16),
              (9, 1, 32 + per16), (1, 1, 64)]
    for shape in shapes:
        for conn in (26, 18, 6):
            a = (rng.integers(1, 4, shape) * (rng.random(shape) < 0.7)).astype(dtype)
            _compare(cc3d.connected_components, a, dict(connectivity=conn))
            _compare(cc3d.connected_components, a, dict(connectivity=conn, binary_image=True))
            _compare(cc3d.connected_components, a, dict(connectivity=conn, delta=1))
        plane = a[0]
        for conn in (8, 4):
            _compare(cc3d.connected_components, plane, dict(connectivity=conn))
            _compare(cc3d.connected_components, plane, dict(connectivity=conn, delta=1))
            _compare(cc3d.connected_components, plane, dict(connectivity=conn, periodic_boundary=True))
        # the same volume on the device at a base 1 element past an aligned one
        flat = torch.zeros(a.size + 1, dtype=getattr(torch, np.dtype(dtype).name), device="cuda")
        flat[1:] = torch.from_numpy(a.reshape(-1)).cuda()
        t = flat[1:].view(a.shape)
        assert t.data_ptr() % 16 != 0
        got, n = cc3d.connected_components(t, connectivity=26, return_N=True)
        exp, en = oracle.connected_components(a, connectivity=26, return_N=True)
        assert n == en and np.array_equal(got.cpu().numpy(), exp)
