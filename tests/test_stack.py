"""connected_components_stack (cc3d/__init__.py:324-501): the reference's own
test of it (automated_test.py test_connected_components_stack) restated on
seeded inputs, and exact numbering against the oracle for Fortran-ordered
slabs, where the stacked numbering is the whole volume's raster numbering.
The host logic (seam pairs, grouping, renumbering) also runs on CPU with the
oracle standing in for the device labelling."""
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


def _run_reference_test(stack_fn, cc_fn, connectivity, binary_image):
    stack = [np.ones([40, 30, 20], dtype=np.uint32) for _ in range(4)]
    stack += [np.zeros([40, 30, 1], dtype=np.uint32)]
    stack += [np.ones([40, 30, 20], dtype=np.uint32) for _ in range(2)]
    arr = stack_fn(stack, connectivity=connectivity, binary_image=binary_image)
    ans = np.ones([40, 30, 121], dtype=np.uint32)
    ans[:, :, 80] = 0
    ans[:, :, 81:] = 2
    assert np.all(np.unique(arr[:]) == [0, 1, 2])
    assert np.all(arr[:] == ans)
    assert arr.num_labels() == 3 and arr.decompress().shape == ans.shape
    rng = np.random.default_rng(connectivity + binary_image)
    image, slabs = _stack_cases(rng)
    ans = cc_fn(image, connectivity=connectivity, binary_image=binary_image)
    res, N = stack_fn(slabs, connectivity=connectivity, binary_image=binary_image, return_N=True)
    assert _same_partition(res[:], ans)
    assert N == int(np.max(ans))
    # Fortran-ordered slabs: the stacked numbering is the volume's raster numbering
    fslabs = [np.asfortranarray(s) for s in slabs]
    res = stack_fn(fslabs, connectivity=connectivity, binary_image=binary_image)
    exp = cc_fn(np.asfortranarray(image), connectivity=connectivity, binary_image=binary_image)
    assert np.array_equal(res[:], exp)


@pytest.fixture()
def host_stack(monkeypatch):
    oracle.build()
    import cc3d_gb300.stack as S

    def remap(cc_labels, table, out_dtype, order="C"):
        out = table[np.asarray(cc_labels).astype(np.int64)]
        return np.asfortranarray(out) if order == "F" else out

    monkeypatch.setattr(S, "connected_components", lambda img, **kw: oracle.connected_components(img, **kw))
    monkeypatch.setattr(S, "_remap", remap)
    return S


@pytest.mark.parametrize("connectivity", [6, 26])
@pytest.mark.parametrize("binary_image", [False, True])
def test_stack_host_logic(host_stack, connectivity, binary_image):
    _run_reference_test(host_stack.connected_components_stack,
                        lambda img, **kw: oracle.connected_components(img, **kw), connectivity, binary_image)


def test_stack_rejects_other_connectivities(host_stack):
    with pytest.raises(ValueError):
        host_stack.connected_components_stack([np.ones((3, 3, 3), np.uint8)], connectivity=18)


@pytest.mark.gpu
@pytest.mark.parametrize("connectivity", [6, 26])
@pytest.mark.parametrize("binary_image", [False, True])
def test_stack_gpu(connectivity, binary_image):
    import __graft_entry__ as entry
    entry.build()
    cc3d = entry.package()
    _run_reference_test(cc3d.connected_components_stack,
                        lambda img, **kw: oracle.connected_components(img, **kw), connectivity, binary_image)
