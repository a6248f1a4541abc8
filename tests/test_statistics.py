"""statistics on the GPU against the oracle, on the cases that exercise how
the kernel accumulates: labels frequent enough to be kept in each block's
shared-memory slots (the background, a giant component), many labels that
contend for the same slots, Fortran-ordered device tensors, and an axis of
2^27 or more voxels (coordinate sums reduced in 64 bits).  Counts, boxes and
centroids must be identical (centroids bit for bit, tolerance 0)."""
import numpy as np
import pytest

import oracle
import __graft_entry__ as entry

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cc3d():
    entry.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return entry.package()


def _same(got, exp, what):
    for k in ("voxel_counts", "bounding_boxes", "centroids"):
        g = got[k].cpu().numpy() if hasattr(got[k], "cpu") else got[k]
        assert g.dtype == exp[k].dtype, (what, k)
        assert np.array_equal(g, exp[k], equal_nan=(k == "centroids")), (what, k)


@pytest.mark.parametrize("p", [0.2, 0.5, 0.8])
def test_dense_binary_giant_component(cc3d, p):
    """Bernoulli foreground labelled at 26: the background and one giant
    component lie in almost every warp; thousands of small components
    collide in the hashed slots."""
    import torch
    from cc3d_gb300 import synth
    vol = synth.bernoulli_volume((96, 112, 130), p, seed=int(p * 100))
    labels = oracle.connected_components(vol, connectivity=26, binary_image=True)
    exp = oracle.statistics(labels, no_slice_conversion=True)
    _same(cc3d.statistics(torch.from_numpy(labels).cuda(), no_slice_conversion=True), exp, ("device", p))
    _same(cc3d.statistics(labels, no_slice_conversion=True), exp, ("host", p))


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.uint32, np.uint64])
def test_fortran_order_and_2d(cc3d, dtype):
    import torch
    from cc3d_gb300 import synth
    vol = synth.voronoi_volume((70, 90, 45), 60, 1 << 12, seed=9, dtype=np.uint32)
    labels = oracle.connected_components(vol, connectivity=6).astype(dtype)  # uint8 wraps: still labels
    for arr in (labels, np.asfortranarray(labels), labels[:, :, 17], np.asfortranarray(labels[5])):
        exp = oracle.statistics(arr, no_slice_conversion=True)
        if arr.flags.c_contiguous:
            t = torch.from_numpy(arr).cuda()
        else:  # a Fortran-ordered device tensor with the same values
            t = torch.from_numpy(arr.T.copy()).cuda().permute(*reversed(range(arr.ndim)))
        _same(cc3d.statistics(t, no_slice_conversion=True), exp, (np.dtype(dtype).name, arr.shape))


def test_axis_of_2_27_voxels(cc3d):
    """A 1D array longer than 2^27: its coordinate sums do not fit 32 bits per
    warp and take the 64-bit reduction.  Expected tables from exact numpy
    reductions (every partial sum is an integer below 2^53)."""
    import torch
    n = (1 << 27) + 37
    idx = np.arange(n, dtype=np.int64)
    labels = ((idx // 997) % 7).astype(np.uint8)
    labels[-1] = 9  # label 8 absent: count 0, NaN centroid, boxes at their initial values
    got = cc3d.statistics(torch.from_numpy(labels).cuda(), no_slice_conversion=True)
    counts = np.bincount(labels, minlength=10)
    sums = np.bincount(labels, weights=idx.astype(np.float64), minlength=10)
    assert np.array_equal(got["voxel_counts"].cpu().numpy(), counts.astype(np.uint32))
    cent = got["centroids"].cpu().numpy()
    assert cent.shape == (10, 2)
    with np.errstate(invalid="ignore", divide="ignore"):
        exp_x = np.where(counts == 0, np.nan, sums / np.where(counts == 0, 1, counts))
    assert np.array_equal(cent[:, 0], exp_x, equal_nan=True)
    assert np.array_equal(cent[:, 1], np.where(counts == 0, np.nan, 0.0), equal_nan=True)
    bb = got["bounding_boxes"].cpu().numpy()
    assert bb.dtype == np.uint32  # an axis longer than 65535
    for k in range(10):
        pos = np.flatnonzero(labels == k)
        if pos.size:
            assert (bb[k, 0], bb[k, 1], bb[k, 2], bb[k, 3]) == (pos[0], pos[-1], 0, 0), k
        else:
            assert (bb[k, 0], bb[k, 1], bb[k, 2], bb[k, 3]) == (np.iinfo(np.uint32).max, 0,
                                                                np.iinfo(np.uint32).max, 0), k
