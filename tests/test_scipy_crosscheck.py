"""Cross-checks that need no reference build: scipy.ndimage.label numbers the
components of a binary volume in C raster order of their first voxel, which is
cc3d's numbering, so labels must be identical (the reference's own
test_compare_scipy_26/18/6 check the same at 128^3 and 256^3).  The oracle is
checked on CPU, the GPU path on the GPU.  Also on the GPU: a 512^3 uint64
volume whose voxels all differ, so every tile holds the maximum number of
components (the reference's 512^3 all-distinct stress case)."""
import numpy as np
import pytest

import oracle


def _structure(conn):
    from scipy import ndimage
    if conn == 26:
        return np.ones((3, 3, 3), bool)
    return ndimage.generate_binary_structure(3, 2 if conn == 18 else 1)


def _random_bool(shape, seed, p=0.5):
    return np.random.default_rng(seed).random(shape) < p


def _scipy_labels(vol, conn):
    from scipy import ndimage
    lab, n = ndimage.label(vol, structure=_structure(conn))
    return lab, int(n)


@pytest.mark.parametrize("conn", [26, 18, 6])
def test_oracle_matches_scipy(conn):
    pytest.importorskip("scipy")
    for seed, p in ((1, 0.5), (2, 0.3116), (3, 0.2)):
        vol = _random_bool((48, 56, 64), seed + conn, p)
        exp, en = _scipy_labels(vol, conn)
        got, n = oracle.connected_components(vol, connectivity=conn, return_N=True)
        assert n == en and np.array_equal(got, exp), (conn, seed)


@pytest.fixture(scope="module")
def cc3d():
    import __graft_entry__ as entry
    entry.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return entry.package()


@pytest.mark.gpu
@pytest.mark.parametrize("conn,edge", [(26, 128), (18, 256), (6, 256)])
def test_gpu_matches_scipy(cc3d, conn, edge):
    pytest.importorskip("scipy")
    import torch
    vol = _random_bool((edge, edge, edge), 1000 + conn)
    exp, en = _scipy_labels(vol, conn)
    out, n = cc3d.connected_components(torch.from_numpy(vol).cuda(), connectivity=conn, return_N=True)
    assert n == en and out.is_cuda
    assert np.array_equal(out.cpu().numpy(), exp)
    host, hn = cc3d.connected_components(vol, connectivity=conn, return_N=True)
    assert hn == en and np.array_equal(host, exp)


@pytest.mark.gpu
def test_gpu_512_cube_all_distinct(cc3d):
    """Voxel i holds the value i: voxel 0 is background and every other voxel
    is its own component, numbered by raster order, so the labels are
    0, 1, ..., 512^3 - 1 in uint32 (the estimate is 512^3 - 1)."""
    import torch
    n = 512 ** 3
    vol = np.arange(n, dtype=np.uint64).reshape(512, 512, 512)
    out, N = cc3d.connected_components(torch.from_numpy(vol).cuda(), connectivity=26, return_N=True)
    assert N == n - 1
    got = out.cpu().numpy()
    assert got.dtype == np.uint32 and np.array_equal(got.reshape(-1), np.arange(n, dtype=np.uint32))
