"""connected_components_stack (cc3d/__init__.py:324-501): the reference's own
test of it (automated_test.py test_connected_components_stack) restated on
seeded inputs, run on the oracle's CPU restatement and on the device path,
and the device path's labels compared exactly with the oracle's on random
stacks (C and Fortran order, several dtypes, binary and multilabel)."""
import numpy as np
import pytest

import oracle


def _same_partition(a, b):
    fa = np.asarray(a).reshape(-1, order="F")
    fb = np.asarray(b).reshape(-1, order="F")
    return np.array_equal(_canonical_flat(fa), _canonical_flat(fb))


def _canonical_flat(flat):
    _, first, inv = np.unique(flat, return_index=True, return_inverse=True)
    rank = np.empty(len(first), np.int64)
    rank[np.argsort(first)] = np.arange(len(first))
    return rank[inv]


def _stack_cases(rng):
    image = rng.integers(0, 100, size=[60, 50, 11]).astype(np.uint8)
    return image, [image[:, :, :2], image[:, :, 2:6], image[:, :, 6:9], image[:, :, 9:11]]


def _oracle_stack(slabs, connectivity=26, return_N=False, binary_image=False):
    out, n, _ = oracle.connected_components_stack(slabs, connectivity=connectivity, return_N=True,
                                                  binary_image=binary_image)
    return (out, n) if return_N else out


def _run_reference_test(stack_fn, connectivity, binary_image, full_api=True):
    stack = [np.ones([40, 30, 20], dtype=np.uint32) for _ in range(4)]
    stack += [np.zeros([40, 30, 1], dtype=np.uint32)]
    stack += [np.ones([40, 30, 20], dtype=np.uint32) for _ in range(2)]
    arr = stack_fn(stack, connectivity=connectivity, binary_image=binary_image)
    ans = np.ones([40, 30, 121], dtype=np.uint32)
    ans[:, :, 80] = 0
    ans[:, :, 81:] = 2
    assert np.all(np.unique(arr[:]) == [0, 1, 2])
    assert np.all(arr[:] == ans)
    if full_api:
        assert arr.num_labels() == 3 and arr.decompress().shape == ans.shape
    rng = np.random.default_rng(connectivity + binary_image)
    image, slabs = _stack_cases(rng)
    ans = oracle.connected_components(image, connectivity=connectivity, binary_image=binary_image)
    res, N = stack_fn(slabs, connectivity=connectivity, binary_image=binary_image, return_N=True)
    assert _same_partition(res[:], ans)
    assert N == int(np.max(ans))
    # Fortran-ordered slabs: the stacked numbering is the volume's raster numbering
    fslabs = [np.asfortranarray(s) for s in slabs]
    res = stack_fn(fslabs, connectivity=connectivity, binary_image=binary_image)
    exp = oracle.connected_components(np.asfortranarray(image), connectivity=connectivity,
                                      binary_image=binary_image)
    assert np.array_equal(res[:], exp)


@pytest.mark.parametrize("connectivity", [6, 26])
@pytest.mark.parametrize("binary_image", [False, True])
def test_oracle_stack(connectivity, binary_image):
    oracle.build()
    _run_reference_test(_oracle_stack, connectivity, binary_image, full_api=False)


def test_oracle_stack_rejects_other_connectivities():
    with pytest.raises(ValueError):
        oracle.connected_components_stack([np.ones((3, 3, 3), np.uint8)], connectivity=18)


@pytest.fixture(scope="module")
def cc3d():
    import __graft_entry__ as entry
    entry.build()
    return entry.package()


@pytest.mark.gpu
@pytest.mark.parametrize("connectivity", [6, 26])
@pytest.mark.parametrize("binary_image", [False, True])
def test_stack_gpu(cc3d, connectivity, binary_image):
    _run_reference_test(cc3d.connected_components_stack, connectivity, binary_image)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.uint8, np.int16, np.uint32, np.uint64, np.float32, np.float16, np.bool_])
@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("connectivity", [6, 26])
def test_stack_gpu_matches_oracle(cc3d, dtype, order, connectivity):
    rng = np.random.default_rng(hash((np.dtype(dtype).name, order, connectivity)) % 2**32)
    for binary in (False, True):
        depths = rng.integers(1, 6, size=5)
        vol = rng.integers(0, 4, size=(37, 45, int(depths.sum())))
        vol = (vol != 0) if dtype == np.bool_ else vol.astype(dtype)
        z = np.concatenate([[0], np.cumsum(depths)])
        slabs = [np.asarray(vol[:, :, z[k]:z[k + 1]], order=order) for k in range(len(depths))]
        res, N = cc3d.connected_components_stack(slabs, connectivity=connectivity, return_N=True,
                                                 binary_image=binary)
        exp, eN, bg = oracle.connected_components_stack(slabs, connectivity=connectivity, return_N=True,
                                                        binary_image=binary)
        assert N == eN
        assert res.dtype == exp.dtype
        assert np.array_equal(np.asarray(res[:]), exp)
        assert res.num_labels() == eN + (1 if bg else 0)


@pytest.mark.gpu
def test_stack_gpu_device_slabs(cc3d):
    import torch
    rng = np.random.default_rng(5)
    vol = rng.integers(0, 3, size=(33, 20, 12)).astype(np.uint16)
    slabs = [vol[:, :, :5], vol[:, :, 5:6], vol[:, :, 6:]]
    res, N = cc3d.connected_components_stack([torch.from_numpy(np.ascontiguousarray(s)).cuda() for s in slabs],
                                             return_N=True)
    exp, eN, _ = oracle.connected_components_stack(slabs, return_N=True)
    assert res[:].is_cuda
    assert N == eN
    assert np.array_equal(res[:].cpu().numpy(), exp)


@pytest.mark.gpu
def test_stack_gpu_rejects_other_connectivities(cc3d):
    with pytest.raises(ValueError):
        cc3d.connected_components_stack([np.ones((3, 3, 3), np.uint8)], connectivity=18)
