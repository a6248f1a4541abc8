"""CPU torch tensors through every function: they are moved to the device
(never handed to a kernel as host addresses) and come back as CPU tensors,
with the same results as numpy inputs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cc3d():
    import __graft_entry__ as entry
    entry.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return entry.package()


def test_cpu_tensors_everywhere(cc3d):
    import torch
    rng = np.random.default_rng(2)
    a = rng.integers(0, 4, (40, 30, 20)).astype(np.uint32)
    t = torch.from_numpy(a.copy())

    def same(x, y):
        x = x.numpy() if isinstance(x, torch.Tensor) else np.asarray(x)
        return np.array_equal(x, np.asarray(y))

    out = cc3d.connected_components(t, connectivity=26)
    assert isinstance(out, torch.Tensor) and not out.is_cuda
    assert same(out, cc3d.connected_components(a, connectivity=26))
    d = cc3d.dust(t.clone(), 20)
    assert isinstance(d, torch.Tensor) and not d.is_cuda and same(d, cc3d.dust(a.copy(), 20))
    k = cc3d.largest_k(t.clone(), 3)
    assert isinstance(k, torch.Tensor) and not k.is_cuda and same(k, cc3d.largest_k(a.copy(), 3))
    assert cc3d.contacts(t) == cc3d.contacts(a)
    r1, r2 = cc3d.runs(t), cc3d.runs(a)
    assert list(r1) == list(r2) and all(r1[key] == r2[key] for key in r2)
    v = cc3d.voxel_connectivity_graph(t, connectivity=26)
    assert isinstance(v, torch.Tensor) and not v.is_cuda and same(v, cc3d.voxel_connectivity_graph(a, 26))
    c = cc3d.color_connectivity_graph(v, connectivity=26)
    assert isinstance(c, torch.Tensor) and not c.is_cuda
    assert same(c, cc3d.color_connectivity_graph(cc3d.voxel_connectivity_graph(a, 26), connectivity=26))
    s1 = cc3d.statistics(out, no_slice_conversion=True)
    s2 = cc3d.statistics(cc3d.connected_components(a, connectivity=26), no_slice_conversion=True)
    assert np.array_equal(np.asarray(s1["voxel_counts"]), np.asarray(s2["voxel_counts"]))
