"""The learned cost model: device features, training and inference kernels,
the confidence fallback, and the "model" dispatch policy (labels unchanged)."""
import math

import numpy as np
import pytest

import __graft_entry__ as entry

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cc3d():
    entry.build()
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    pkg = entry.package()
    yield pkg
    pkg.set_tile_pass("auto")
    pkg.autotune_reset()


def test_features_match_a_host_count(cc3d):
    import torch
    cm = cc3d.costmodel
    rng = np.random.default_rng(1)
    vol = (rng.random((40, 64, 96)) < 0.3).astype(np.uint16) * 7
    f = cm.features(torch.from_numpy(vol.view(np.int16)).cuda(), connectivity=18, binary_image=False)
    assert f.shape == (16,) and np.all(np.isfinite(f))
    assert f[0] == pytest.approx(math.log2(96)) and f[1] == pytest.approx(math.log2(64))
    assert f[2] == pytest.approx(math.log2(40)) and f[3] == pytest.approx(math.log2(96 * 64 * 40))
    assert f[4] == pytest.approx(2 / 8) and f[5] == pytest.approx(18 / 26) and f[6] == 0
    assert f[7] == pytest.approx(0.3, abs=0.02)                 # sampled foreground fraction
    assert f[8] == pytest.approx(math.log2(3) / 12, abs=1e-6)   # values {0, 7}
    assert f[9] == pytest.approx(0.3, abs=0.03)                 # P(x+1 also foreground)
    assert f[12] == pytest.approx(0.0) and f[13] == pytest.approx(0.0) and f[14] == pytest.approx(0.0)


def test_train_predict_choose(cc3d):
    import torch
    cm = cc3d.costmodel
    X, Y, desc = cm.collect(24, seed=3, lo=24, hi=72)
    assert X.shape == (24, 16) and Y.shape == (24, 12)
    assert np.isfinite(Y).sum() >= 24 * 2
    loss = cm.train(X, Y, epochs=60, batch=8, lr=3e-3, seed=1)
    assert np.isfinite(loss)
    P = cm.predict(X)
    assert P.shape == (24, 12) and np.all(np.isfinite(P))
    # fitting the training set beats predicting the mean
    m = np.isfinite(Y)
    mean = np.nanmean(Y, axis=0)
    assert ((P - Y)[m] ** 2).mean() < ((mean - Y)[m] ** 2).mean()
    p = cm.get_params()
    assert p.shape == (6084,)
    cm.set_params(p)
    assert np.array_equal(cm.predict(X), P)
    r = cm.regret(Y, P)
    assert 0.0 <= r["mean_regret"] and 0.0 <= r["top1"] <= 1.0
    vol = torch.from_numpy(np.random.default_rng(4).integers(0, 3, (50, 60, 70)).astype(np.uint8)).cuda()
    name, confident = cm.choose(vol, connectivity=26)
    assert name in cc3d.tuning.CONFIGS
    name, confident = cm.choose(vol, connectivity=26, min_margin=1e9)  # never confident: autotuner decides
    assert not confident and name in cc3d.tuning.CONFIGS


def test_model_policy_keeps_labels(cc3d):
    import torch
    from cc3d_gb300 import synth
    vol = synth.voronoi_volume((64, 80, 96), 100, 1 << 20, seed=5)
    dev = torch.from_numpy(vol).cuda()
    cc3d.set_tile_pass("auto")
    ref, n = cc3d.connected_components(dev, connectivity=26, return_N=True)
    cc3d.set_tile_pass("model")
    got, n2 = cc3d.connected_components(dev, connectivity=26, return_N=True)
    cc3d.set_tile_pass("auto")
    assert n == n2 and torch.equal(ref.to(torch.int64), got.to(torch.int64))
