"""The give-up path of the bounded union-find loops: with the iteration
budget lowered to 1 (cc3d_gpu_set_union_budget), labelling a volume whose
union-find trees need more than one step must stop, report CC3D_ERR_DEVICE
and leave the GPU usable; with the budget restored the next call is exact.
No kernel is made to fault or hang: every loop simply runs out of budget.
(The reference has no device loops; its DisjointSet throws when its label
array is full, cc3d/cc3d.hpp:107-111.)"""
import ctypes

import numpy as np
import pytest

import __graft_entry__ as entry
import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    entry.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    cc3d = entry.package()
    lib = cc3d._native.load()
    yield cc3d, cc3d._native, lib, torch
    lib.cc3d_gpu_set_union_budget(0)


def _label(nat, lib, torch, dev, conn, binary):
    sz, sy, sx = dev.shape
    out = torch.zeros(dev.shape, dtype=torch.uint32, device="cuda")
    N = ctypes.c_uint64(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.cc3d_gpu_connected_components3d(dev.data_ptr(), nat.U8, sx, sy, sz, int(dev.numel()), conn, 0.0,
                                             out.data_ptr(), nat.U32, ctypes.byref(N), 0, int(binary),
                                             nat.IN_DEVICE | nat.OUT_DEVICE, stream)
    torch.cuda.synchronize()
    return rc, out, N.value


@pytest.mark.parametrize("variant", ["list", "runs"])
def test_budget_one_gives_up_and_recovers(env, variant):
    cc3d, nat, lib, torch = env
    from cc3d_gb300 import synth
    # near the percolation threshold: long union-find chains at 6-connectivity
    vol = synth.bernoulli_volume((96, 128, 160), 0.3116, seed=11)
    dev = torch.from_numpy(vol).cuda()
    prev = cc3d.set_tile_pass(variant)
    try:
        assert lib.cc3d_gpu_set_union_budget(-1) == nat.ERR_INVALID
        assert lib.cc3d_gpu_set_union_budget(1) == 0
        rc, _, _ = _label(nat, lib, torch, dev, 6, True)
        assert rc == nat.ERR_DEVICE, (rc, lib.cc3d_gpu_last_error())
        assert b"budget" in lib.cc3d_gpu_last_error()
        assert lib.cc3d_gpu_set_union_budget(0) == 1
        rc, out, N = _label(nat, lib, torch, dev, 6, True)
        assert rc == 0, lib.cc3d_gpu_last_error()
        exp, eN = oracle.connected_components(vol, connectivity=6, return_N=True, binary_image=True,
                                              out_dtype=np.uint32)
        assert N == eN
        assert np.array_equal(out.cpu().numpy(), exp)
    finally:
        lib.cc3d_gpu_set_union_budget(0)
        cc3d.set_tile_pass(prev)
