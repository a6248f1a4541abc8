"""Tile-pass variants and the autotuner (cc3d_gpu_set_tile_pass,
cc3d_gpu_tile_pass_choice, cc3d_gpu_autotune).  The choice itself needs no GPU;
timing the variants does."""
import numpy as np
import pytest

import __graft_entry__ as entry


@pytest.fixture(scope="module")
def cc3d():
    entry.build()
    pkg = entry.package()
    yield pkg
    pkg.set_tile_pass("auto")
    pkg.autotune_reset()


def test_choice_follows_the_thread_setting(cc3d):
    vol = np.zeros((40, 50, 60), np.uint32)
    assert cc3d.set_tile_pass("runs") == "auto"
    assert cc3d.tile_pass_choice(vol) == "runs/8x8"
    assert cc3d.set_tile_pass("list/4x16") == "runs/8x8"
    assert cc3d.tile_pass_choice(vol) == "list/4x16"
    cc3d.set_tile_pass("runs/16x4")
    assert cc3d.tile_pass_choice(vol) == "runs/16x4"
    # 2D images have one tile shape
    assert cc3d.tile_pass_choice(np.zeros((64, 64), np.uint32), connectivity=4) == "runs/8x8"
    cc3d.set_tile_pass("auto")
    cc3d.autotune_reset()
    # the default without tuning data: the list pass on 32x8x8 tiles, box by TMA
    assert cc3d.tile_pass_choice(vol) == "list/8x8"
    big = np.zeros((256, 256, 256), np.uint8)
    assert cc3d.tile_pass_choice(big) == "list/8x8"
    assert cc3d.tile_pass_choice(big, connectivity=6) == "list/8x8"
    # the load-path bit survives for 2D images, the shape does not
    cc3d.set_tile_pass("list/16x4/plain")
    assert cc3d.tile_pass_choice(vol) == "list/16x4/plain"
    assert cc3d.tile_pass_choice(np.zeros((64, 64), np.uint32), connectivity=8) == "list/8x8/plain"
    # binary 8-connected images always take the run-union pass (2x2-block numbering)
    cc3d.set_tile_pass("list")
    assert cc3d.tile_pass_choice(np.zeros((64, 64), np.uint8), connectivity=8, binary_image=True) == "runs/8x8"
    cc3d.set_tile_pass("auto")
    from cc3d_gb300.tuning import CONFIGS, config_code
    lib = cc3d._native.load()
    assert [lib.cc3d_gpu_tile_config(i) for i in range(len(CONFIGS))] == [config_code(c) for c in CONFIGS]
    assert lib.cc3d_gpu_tile_config(len(CONFIGS)) == -1


def test_unknown_variant_is_rejected(cc3d):
    lib = cc3d._native.load()
    assert lib.cc3d_gpu_set_tile_pass(7) == -1
    assert lib.cc3d_gpu_set_tile_pass(0x31) == -1
    assert lib.cc3d_gpu_set_tile_pass(0x202) == -1
    with pytest.raises(KeyError):
        cc3d.set_tile_pass("list/8x8/tma")
    with pytest.raises(KeyError):
        cc3d.set_tile_pass("fastest")


@pytest.mark.gpu
def test_autotune_records_the_fastest_configuration(cc3d):
    import torch
    from cc3d_gb300 import synth
    from cc3d_gb300.tuning import CONFIGS
    vol = synth.voronoi_volume((96, 128, 160), 200, 1 << 20, seed=21)
    cc3d.autotune_reset()
    for data in (vol, torch.from_numpy(vol).cuda()):
        res = cc3d.autotune(data, connectivity=26)
        assert set(res["ms"]) == set(CONFIGS) and res["best"] in CONFIGS
        assert all(ms > 0 for ms in res["ms"].values())
        assert res["best"] == min(res["ms"], key=res["ms"].get)
        assert cc3d.tile_pass_choice(vol, connectivity=26) == res["best"]
        # the labels do not depend on the choice
        out, N = cc3d.connected_components(data, connectivity=26, return_N=True)
        for other in CONFIGS:
            cc3d.set_tile_pass(other)
            out2, N2 = cc3d.connected_components(data, connectivity=26, return_N=True)
            assert N == N2
            assert np.array_equal(np.asarray(out.cpu() if hasattr(out, "cpu") else out),
                                  np.asarray(out2.cpu() if hasattr(out2, "cpu") else out2))
        cc3d.set_tile_pass("auto")
    img = synth.bernoulli_volume((300, 400), 0.5, seed=3)
    res = cc3d.autotune(img, connectivity=4)
    assert set(res["ms"]) == {"list/8x8", "list/8x8/plain", "runs/8x8", "runs/8x8/plain"}
