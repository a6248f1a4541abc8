"""Entry points that take device buffers refuse host addresses with an error
code instead of handing them to a kernel (checked with pinned host memory,
which a kernel could even read, so the check itself is what is tested)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import __graft_entry__ as entry
    entry.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    cc3d = entry.package()
    return cc3d, cc3d._native, cc3d._native.load(), torch


def test_host_addresses_are_refused(env):
    cc3d, nat, lib, torch = env
    host = torch.ones(4096, dtype=torch.uint32).pin_memory()
    dev = torch.ones(4096, dtype=torch.uint32, device="cuda")
    out = torch.empty(4096, dtype=torch.uint32, device="cuda")
    info = nat.Prepared()
    rc = lib.cc3d_gpu_label_prepare(host.data_ptr(), nat.U32, 16, 16, 16, 26, 0, 0, nat.IN_DEVICE, None,
                                    ctypes.byref(info))
    assert rc == -1 and b"device memory" in lib.cc3d_gpu_last_error()
    # the same call with the device copy works, and then a host output is refused
    assert lib.cc3d_gpu_label_prepare(dev.data_ptr(), nat.U32, 16, 16, 16, 26, 0, 0, nat.IN_DEVICE, None,
                                      ctypes.byref(info)) == 0
    n = ctypes.c_uint64(0)
    rc = lib.cc3d_gpu_label_finish(info.token, 4096, host.data_ptr(), nat.U32, ctypes.byref(n), nat.OUT_DEVICE, None)
    assert rc == -1
    assert lib.cc3d_gpu_voxel_connectivity_graph(host.data_ptr(), 4, 16, 16, 16, 26, 0, out.data_ptr(), None) == -1
    assert lib.cc3d_gpu_run_starts(host.data_ptr(), 4, 4096, ctypes.byref(n), None) == -1
    table = torch.zeros(2, dtype=torch.uint32, device="cuda")
    assert lib.cc3d_gpu_remap_labels(host.data_ptr(), 4, 4096, table.data_ptr(), 4, 2, out.data_ptr(), None) == -1
    # and the checked Python layer still labels the device volume
    lab, N = cc3d.connected_components(dev.view(16, 16, 16), return_N=True)
    assert N == 1


def test_statistics_rejects_labels_above_n(env):
    """statistics takes N from the caller: a label above it must not index past
    the tables.  Its voxels are skipped and the call reports a device error;
    the next call with the right N is exact."""
    cc3d, nat, lib, torch = env
    lab = torch.arange(64, dtype=torch.int32).to(torch.uint32).cuda().view(4, 4, 4)
    N = 10  # the real maximum is 63
    counts = torch.zeros(N + 1, dtype=torch.uint32, device="cuda")
    bbox = torch.zeros((N + 1) * 6, dtype=torch.uint16, device="cuda")
    cent = torch.zeros((N + 1) * 3, dtype=torch.float64, device="cuda")
    rc = lib.cc3d_gpu_statistics(lab.data_ptr(), nat.U32, 4, 4, 4, 3, 1, N, counts.data_ptr(), bbox.data_ptr(),
                                 nat.U16, cent.data_ptr(), nat.IN_DEVICE | nat.OUT_DEVICE, None)
    assert rc == nat.ERR_DEVICE and b"exceeds N" in lib.cc3d_gpu_last_error()
    assert int(counts.cpu().numpy().astype(np.int64).sum()) == N + 1  # only labels 0..N were counted
    s = cc3d.statistics(lab, no_slice_conversion=True)
    assert s["voxel_counts"].cpu().tolist() == [1] * 64
