"""Batches (cc3d_gpu_label_batch): every volume of a batch gets exactly what
the single-volume path gives it -- labels, N and output dtype -- and the
oracle agrees, in both batch modes (one persistent launch; one launch per
stage).  A repeated list of shapes replays the captured graph with new
buffers and data; the persistent launch replays its graph for any list."""
import numpy as np
import pytest

import oracle
import __graft_entry__ as entry

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=["persistent", "staged"])
def cc3d(request):
    entry.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    pkg = entry.package()
    prev = pkg.set_batch_mode(request.param)
    yield pkg
    pkg.set_batch_mode(prev)


def _shapes(rng, n, lo, hi, dims=3):
    return [tuple(int(round(np.exp(rng.uniform(np.log(lo), np.log(hi))))) for _ in range(dims)) for _ in range(n)]


def _voronoi_batch(shapes, seed, dtype=np.uint16):
    from cc3d_gb300 import synth
    out = []
    for i, s in enumerate(shapes):
        n_seeds = max(1, int(np.prod(s)) // 4096)
        out.append(synth.voronoi_volume(s, n_seeds, 65535 if dtype == np.uint16 else 1 << 20,
                                        seed=seed * 1000 + i, dtype=dtype, salt=0.0))
    return out


def _check_batch(cc3d, vols, conn, n_oracle=4):
    import torch
    got = cc3d.connected_components_batch(vols, connectivity=conn, return_N=True)
    assert len(got) == len(vols)
    for i, (v, (lab, N)) in enumerate(zip(vols, got)):
        exp, eN = cc3d.connected_components(torch.from_numpy(v).cuda(), connectivity=conn, return_N=True)
        assert N == eN, (i, v.shape, N, eN)
        assert lab.dtype == exp.dtype, (i, lab.dtype, exp.dtype)
        assert np.array_equal(lab.cpu().numpy(), exp.cpu().numpy()), (i, v.shape)
        if i < n_oracle:
            o, oN = oracle.connected_components(v, connectivity=conn, return_N=True)
            assert oN == N and o.dtype == lab.cpu().numpy().dtype
            assert np.array_equal(o, lab.cpu().numpy()), (i, v.shape)


def test_batch_matches_single_volume_path(cc3d):
    rng = np.random.default_rng(7)
    shapes = _shapes(rng, 48, 16, 96)
    vols = _voronoi_batch(shapes, seed=1)
    vols[3] = np.zeros_like(vols[3])            # all background
    vols.append(np.zeros((0, 5, 7), np.uint16))  # empty
    for conn in (26, 18, 6):
        _check_batch(cc3d, vols, conn)


def test_graph_replay_with_new_buffers(cc3d):
    rng = np.random.default_rng(8)
    shapes = _shapes(rng, 24, 16, 80)
    for seed in (2, 3, 4):  # same layout: the second and third calls replay the graph
        _check_batch(cc3d, _voronoi_batch(shapes, seed=seed), 26, n_oracle=2)


def test_batch_2d_and_uint8(cc3d):
    rng = np.random.default_rng(9)
    imgs = [(rng.random(s) < 0.6).astype(np.uint8) * rng.integers(1, 4, s).astype(np.uint8)
            for s in _shapes(rng, 20, 16, 300, dims=2)]
    for conn in (8, 4):
        _check_batch(cc3d, imgs, conn)
    vols = [(rng.random(s) < 0.4).astype(np.uint8) for s in _shapes(rng, 12, 16, 64)]
    _check_batch(cc3d, vols, 6)


def test_batch_rejects_what_it_does_not_take(cc3d):
    with pytest.raises(TypeError):
        cc3d.connected_components_batch([np.zeros((4, 4, 4), np.float32)])
    with pytest.raises(RuntimeError):
        cc3d.connected_components_batch([np.ones((2, 4, 4), np.uint8)], connectivity=8)


def test_autotune_batch_records_a_choice(cc3d):
    rng = np.random.default_rng(10)
    vols = _voronoi_batch(_shapes(rng, 16, 16, 64), seed=5)
    from cc3d_gb300.tuning import CONFIGS
    res = cc3d.autotune_batch(vols, connectivity=26)
    # (batches read their boxes with plain loads: the load-path variants are not timed)
    timed = {c for c in CONFIGS if not c.endswith("/plain")}
    assert res["best"] in timed and set(res["ms"]) == timed
    assert all(v > 0 for v in res["ms"].values())
    _check_batch(cc3d, vols, 26, n_oracle=1)


def test_persistent_replays_for_new_layouts(cc3d):
    # every call a different list of shapes (new layout): the persistent mode
    # keeps one graph, the staged mode captures a new one each time
    rng = np.random.default_rng(11)
    for seed in (6, 7, 8):
        vols = _voronoi_batch(_shapes(rng, 10 + seed, 16, 72), seed=seed)
        _check_batch(cc3d, vols, 26, n_oracle=1)


def test_both_modes_agree_on_a_mixed_stream():
    entry.build()
    pkg = entry.package()
    rng = np.random.default_rng(12)
    vols = _voronoi_batch(_shapes(rng, 64, 16, 128), seed=9)
    prev = pkg.set_batch_mode("persistent")
    try:
        a = pkg.connected_components_batch(vols, connectivity=26, return_N=True)
        pkg.set_batch_mode("staged")
        b = pkg.connected_components_batch(vols, connectivity=26, return_N=True)
    finally:
        pkg.set_batch_mode(prev)
    for (la, na), (lb, nb) in zip(a, b):
        assert na == nb and la.dtype == lb.dtype and np.array_equal(la.cpu().numpy(), lb.cpu().numpy())
