"""Parity at the full sizes of the benchmarked workloads, against the oracle
(which labels each of these volumes in seconds on the host):

* 512^3 uint32 Voronoi (4096 seeds, labels in [1, 2^20], 1-voxel membrane,
  2% salt) at connectivity 26, 18 and 6, and statistics on the 26 output;
* 768^3 uint64 Voronoi (labels in [1, 2^48]) at 26 with out_dtype=uint64;
* 512^3 uint8 Bernoulli(p) for p in {0.2, 0.3116, 0.5}, binary, at 6, 18, 26,
  and at 6 with periodic boundaries;
* 8192^2 uint8 Bernoulli(0.5) at 8 and 4, binary and multilabel.

Every case runs under every tile-pass configuration; labels, N and dtypes must be
identical to the oracle's."""
import numpy as np
import pytest

import oracle
import __graft_entry__ as entry

pytestmark = pytest.mark.gpu

VARIANTS = ("list/8x8", "runs/8x8", "list/4x16", "runs/4x16", "list/16x4", "runs/16x4", "list/16x4/plain",
            "runs/8x8/plain")


@pytest.fixture(scope="module")
def cc3d():
    entry.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    pkg = entry.package()
    yield pkg
    pkg.set_tile_pass("auto")


def _check(cc3d, vol, **kw):
    import torch
    exp, eN = oracle.connected_components(vol, return_N=True, **kw)
    dev = torch.from_numpy(vol).cuda()
    for v in VARIANTS:
        cc3d.set_tile_pass(v)
        out, N = cc3d.connected_components(dev, return_N=True, **kw)
        assert N == eN, (v, kw, N, eN)
        assert out.dtype == getattr(torch, exp.dtype.name), (v, kw)
        assert torch.equal(out, torch.from_numpy(exp).cuda()), (v, kw)
    cc3d.set_tile_pass("auto")
    # host buffers: the input and the labels cross in chunks overlapped with the kernels
    out, N = cc3d.connected_components(vol, return_N=True, **kw)
    assert N == eN and out.dtype == exp.dtype and np.array_equal(out, exp), ("host", kw)
    return exp


def test_voronoi_512_u32(cc3d):
    import torch
    from cc3d_gb300 import synth
    vol = synth.voronoi_volume((512, 512, 512), 4096, 1 << 20, seed=1, dtype=np.uint32)
    for conn in (26, 18, 6):
        labels = _check(cc3d, vol, connectivity=conn)
        if conn == 26:
            s = cc3d.statistics(torch.from_numpy(labels).cuda(), no_slice_conversion=True)
            e = oracle.statistics(labels, no_slice_conversion=True)
            assert np.array_equal(s["voxel_counts"].cpu().numpy(), e["voxel_counts"])
            assert np.array_equal(s["bounding_boxes"].cpu().numpy(), e["bounding_boxes"])
            # integer coordinate sums divided in float64: bit-identical (tolerance 0)
            assert np.array_equal(s["centroids"].cpu().numpy(), e["centroids"], equal_nan=True)


def test_voronoi_768_u64(cc3d):
    from cc3d_gb300 import synth
    vol = synth.voronoi_volume((768, 768, 768), 4096, 1 << 48, seed=2, dtype=np.uint64)
    _check(cc3d, vol, connectivity=26, out_dtype=np.uint64)


@pytest.mark.parametrize("p", [0.2, 0.3116, 0.5])
def test_bernoulli_512_u8_binary(cc3d, p):
    from cc3d_gb300 import synth
    vol = synth.bernoulli_volume((512, 512, 512), p, seed=int(p * 1e4))
    for conn in (6, 18, 26):
        _check(cc3d, vol, connectivity=conn, binary_image=True)
    _check(cc3d, vol, connectivity=6, binary_image=True, periodic_boundary=True)


def test_bernoulli_8192_2d(cc3d):
    from cc3d_gb300 import synth
    img = synth.bernoulli_volume((8192, 8192), 0.5, seed=8192)
    for conn in (8, 4):
        for binary in (True, False):
            _check(cc3d, img, connectivity=conn, binary_image=binary)
