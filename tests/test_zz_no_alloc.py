"""The no-allocation entry point (cc3d_gpu_connected_components3d_noalloc)
against the workspace entry point (cc3d_gpu_connected_components3d), both
called through the C ABI on device buffers, and against the oracle.  Several
calls in a row share the fixed scratch array, so a call that read what the
previous one left behind would show up as a mismatch.  The calls must also
leave the device's free memory unchanged: that is what the entry point is
for.  Collected last, and written to pass alone in a fresh process too."""
import ctypes

import numpy as np
import pytest

import __graft_entry__ as entry
import oracle

pytestmark = pytest.mark.gpu

CODES = {np.dtype(np.uint8): 1, np.dtype(np.uint16): 2, np.dtype(np.uint32): 3, np.dtype(np.uint64): 4}
OUT = {2: np.uint16, 3: np.uint32, 4: np.uint64}
IN_DEVICE, OUT_DEVICE = 1, 2


@pytest.fixture(scope="module")
def lib():
    entry.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    torch.cuda.init()
    return entry.package()._native.load()


def _label(lib, fn_name, vol, conn, binary, out_code, periodic=False):
    """Label `vol` (numpy, C order) on the device through one entry point."""
    import torch

    dev = torch.from_numpy(np.ascontiguousarray(vol)).cuda()
    out = torch.full(vol.shape, 7, dtype=getattr(torch, np.dtype(OUT[out_code]).name), device="cuda")
    sz, sy, sx = (1,) * (3 - vol.ndim) + tuple(vol.shape)
    N = ctypes.c_uint64(0)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    max_labels = int(vol.size)
    code = CODES[vol.dtype]
    if fn_name == "noalloc":
        rc = lib.cc3d_gpu_connected_components3d_noalloc(
            ctypes.c_void_p(dev.data_ptr()), code, sx, sy, sz, max_labels, conn,
            ctypes.c_void_p(out.data_ptr()), out_code, ctypes.byref(N), int(periodic), int(binary), stream)
    else:
        rc = lib.cc3d_gpu_connected_components3d(
            ctypes.c_void_p(dev.data_ptr()), code, sx, sy, sz, max_labels, conn, 0.0,
            ctypes.c_void_p(out.data_ptr()), out_code, ctypes.byref(N), int(periodic), int(binary),
            IN_DEVICE | OUT_DEVICE, stream)
    assert rc == 0, (fn_name, rc, lib.cc3d_gpu_last_error())
    torch.cuda.synchronize()
    return out.cpu().numpy(), N.value


def _cases():
    from cc3d_gb300 import synth
    vor = synth.voronoi_volume((128, 128, 128), 256, 2 ** 20, seed=3, dtype=np.uint32)
    vor2 = synth.voronoi_volume((40, 72, 96), 64, 2 ** 16 - 1, seed=4, dtype=np.uint16)
    img = synth.bernoulli_volume((300, 260), 0.5, seed=5)
    sparse = synth.bernoulli_volume((48, 64, 80), 0.3116, seed=6)
    return [
        ("voronoi 128^3 u32, 26", vor, 26, False, 3, False),
        ("voronoi u16, 18", vor2, 18, False, 2, False),
        ("binary 2D, 8 (2x2-block numbering)", img, 8, True, 3, False),
        ("binary 3D, 6 periodic", sparse, 6, True, 4, True),
        ("voronoi 128^3 u32, 26 again", vor, 26, False, 3, False),
    ]


def test_noalloc_matches_workspace_path_on_calls_in_a_row(lib):
    for name, vol, conn, binary, out_code, periodic in _cases():
        ref, n_ref = _label(lib, "workspace", vol, conn, binary, out_code, periodic)
        got, n_got = _label(lib, "noalloc", vol, conn, binary, out_code, periodic)
        assert n_got == n_ref, name
        assert got.dtype == ref.dtype and np.array_equal(got, ref), name
        assert n_ref > 0, name
        exp, n_exp = oracle.connected_components(vol, connectivity=conn, return_N=True, binary_image=binary,
                                                 periodic_boundary=periodic, out_dtype=OUT[out_code])
        assert n_got == n_exp, name
        assert np.array_equal(got, exp), name


def test_noalloc_leaves_device_memory_unchanged(lib):
    """After one warm-up call (the module and its scratch array are resident
    from then on), labelling allocates nothing: every input and output is made
    first, and the device's free memory is the same after the calls."""
    import torch

    cases = _cases()
    bufs = []
    for name, vol, conn, binary, out_code, periodic in cases:
        dev = torch.from_numpy(np.ascontiguousarray(vol)).cuda()
        out = torch.zeros(vol.shape, dtype=getattr(torch, np.dtype(OUT[out_code]).name), device="cuda")
        bufs.append((dev, out))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def run_all():
        for (name, vol, conn, binary, out_code, periodic), (dev, out) in zip(cases, bufs):
            sz, sy, sx = (1,) * (3 - vol.ndim) + tuple(vol.shape)
            N = ctypes.c_uint64(0)
            rc = lib.cc3d_gpu_connected_components3d_noalloc(
                ctypes.c_void_p(dev.data_ptr()), CODES[vol.dtype], sx, sy, sz, int(vol.size), conn,
                ctypes.c_void_p(out.data_ptr()), out_code, ctypes.byref(N), int(periodic), int(binary), stream)
            assert rc == 0, (name, lib.cc3d_gpu_last_error())

    run_all()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    run_all()
    run_all()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_volumes_beyond_its_scratch(lib):
    import torch

    vin = torch.zeros(8, dtype=torch.uint32, device="cuda")
    vout = torch.zeros(8, dtype=torch.uint32, device="cuda")
    N = ctypes.c_uint64(0)
    for shape in ((256, 256, 256), (160, 128, 128), (1, 1, 1 << 22)):
        sz, sy, sx = shape
        rc = lib.cc3d_gpu_connected_components3d_noalloc(
            ctypes.c_void_p(vin.data_ptr()), 3, sx, sy, sz, sx * sy * sz, 26,
            ctypes.c_void_p(vout.data_ptr()), 3, ctypes.byref(N), 0, 0, None)
        assert rc == -1, shape
        msg = lib.cc3d_gpu_last_error().decode()
        assert "no-allocation" in msg and "scratch" in msg, msg
