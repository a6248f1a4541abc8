"""The learned cost model (include/cc3d_gpu.h: cc3d_gpu_volume_features,
cc3d_gpu_cost_model_*): an FP32 MLP 16 -> 64 -> 64 -> 12 that predicts the log
milliseconds of every tile-pass configuration from features sampled on the
device, trained on the autotuner's own timings.  Training and inference run in
the library's CUDA kernels; this module generates the timing data, drives the
training, measures the model's regret against the exhaustive autotuner and
saves/loads the parameters.

The reference has no counterpart: it runs one CPU algorithm per connectivity.
"""
from __future__ import annotations

import ctypes
import math
import os
from typing import Any, Dict, List, Sequence, Tuple

import numpy as np

from . import _native as nat
from .tuning import CONFIGS, _volume, config_name

N_FEATURES = 16
N_OUTPUTS = len(CONFIGS)
N_PARAMS = 6084
DEFAULT_PARAMS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "costmodel_params.npy")


# ------------------------------------------------------------ features / model
def features(volume: Any, connectivity: int = 26, binary_image: bool = False) -> np.ndarray:
    """The 16 features of a CUDA volume (see cc3d_gpu_volume_features)."""
    ptr, code, sx, sy, sz, mem, stream, keep = _volume(volume)
    if not mem:
        raise ValueError("features are sampled from a CUDA tensor")
    out = (ctypes.c_float * N_FEATURES)()
    nat.check(nat.load().cc3d_gpu_volume_features(ptr, code, sx, sy, sz, int(connectivity),
                                                  int(bool(binary_image)), mem, stream, out))
    return np.frombuffer(out, dtype=np.float32).copy()


def train(X: np.ndarray, Y: np.ndarray, epochs: int = 300, batch: int = 256, lr: float = 1e-3,
          seed: int = 0) -> float:
    """Train the process's model on X[n, 16] and Y[n, 6] (log-ms, NaN where not
    measured); returns the last epoch's mean squared error (normalised units)."""
    X = np.ascontiguousarray(X, dtype=np.float32)
    Y = np.ascontiguousarray(Y, dtype=np.float32)
    loss = ctypes.c_float(0)
    nat.check(nat.load().cc3d_gpu_cost_model_train(
        X.ctypes.data, Y.ctypes.data, int(X.shape[0]), int(epochs), int(batch), float(lr), int(seed),
        ctypes.byref(loss)))
    return float(loss.value)


def predict(X: np.ndarray) -> np.ndarray:
    X = np.ascontiguousarray(np.atleast_2d(X), dtype=np.float32)
    Y = np.empty((X.shape[0], N_OUTPUTS), np.float32)
    nat.check(nat.load().cc3d_gpu_cost_model_predict(X.ctypes.data, int(X.shape[0]), Y.ctypes.data))
    return Y


def get_params() -> np.ndarray:
    p = np.empty(N_PARAMS, np.float32)
    nat.check(nat.load().cc3d_gpu_cost_model_get(p.ctypes.data, N_PARAMS))
    return p


def set_params(p: np.ndarray) -> None:
    p = np.ascontiguousarray(p, dtype=np.float32)
    nat.check(nat.load().cc3d_gpu_cost_model_set(p.ctypes.data, int(p.size)))


def save(path: str = DEFAULT_PARAMS) -> None:
    np.save(path, get_params())


def load(path: str = DEFAULT_PARAMS) -> bool:
    """Load parameters (the ones shipped with the package by default); False if absent."""
    if not os.path.exists(path):
        return False
    p = np.load(path)
    if p.size != N_PARAMS:  # parameters of another model shape
        return False
    set_params(p)
    return True


def choose(volume: Any, connectivity: int = 26, binary_image: bool = False,
           min_margin: float = 0.05) -> Tuple[str, bool]:
    """(configuration, confident): the model's choice, or the exhaustive
    autotuner's when the predicted runner-up is within min_margin."""
    ptr, code, sx, sy, sz, mem, stream, keep = _volume(volume)
    choice, conf = ctypes.c_int(0), ctypes.c_int(0)
    nat.check(nat.load().cc3d_gpu_cost_model_choose(ptr, code, sx, sy, sz, int(connectivity),
                                                    int(bool(binary_image)), mem, stream,
                                                    float(min_margin), ctypes.byref(choice), ctypes.byref(conf)))
    return config_name(choice.value), bool(conf.value)


# ------------------------------------------------------------ training data
def voronoi_gpu(shape: Sequence[int], cell: float, label_max: int, seed: int, dtype=np.uint32,
                membrane: float = 1.0, salt: float = 0.0):
    """A Voronoi partition on the GPU: one seed jittered inside every cube of
    edge `cell` (so about prod(shape)/cell^3 seeds), each cell a uniform label
    in [1, label_max], voxels whose two nearest seeds are closer than
    `membrane` in distance difference set to 0, then `salt` of the voxels
    given random labels.  For cost-model training data (fast, seeded)."""
    import torch
    dev = torch.device("cuda")
    g = torch.Generator(device=dev)
    g.manual_seed(int(seed))
    Z, Y, X = (int(s) for s in shape)
    gz, gy, gx = (max(1, math.ceil(s / cell)) for s in (Z, Y, X))
    jit = torch.rand((gz, gy, gx, 3), generator=g, device=dev) * cell
    lab = torch.randint(1, int(label_max) + 1, (gz, gy, gx), generator=g, device=dev, dtype=torch.int64)
    out = torch.empty((Z, Y, X), dtype=torch.int64, device=dev)
    yy, xx = torch.meshgrid(torch.arange(Y, device=dev, dtype=torch.float32) + 0.5,
                            torch.arange(X, device=dev, dtype=torch.float32) + 0.5, indexing="ij")
    cy0, cx0 = (yy / cell).floor().long(), (xx / cell).floor().long()
    slab = max(1, (1 << 23) // max(1, Y * X))
    for z0 in range(0, Z, slab):
        z1 = min(Z, z0 + slab)
        zz = torch.arange(z0, z1, device=dev, dtype=torch.float32).view(-1, 1, 1) + 0.5
        cz0 = (zz / cell).floor().long()
        d1 = torch.full((z1 - z0, Y, X), float("inf"), device=dev)
        d2 = d1.clone()
        best = torch.zeros((z1 - z0, Y, X), dtype=torch.int64, device=dev)
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    cz, cy, cx = cz0 + dz, cy0 + dy, cx0 + dx
                    ok = (cz >= 0) & (cz < gz) & (cy >= 0) & (cy < gy) & (cx >= 0) & (cx < gx)
                    czc, cyc, cxc = cz.clamp(0, gz - 1), cy.clamp(0, gy - 1), cx.clamp(0, gx - 1)
                    czb, cyb, cxb = torch.broadcast_tensors(czc, cyc, cxc)
                    j = jit[czb, cyb, cxb]
                    pz = czb.float() * cell + j[..., 0]
                    py = cyb.float() * cell + j[..., 1]
                    px = cxb.float() * cell + j[..., 2]
                    d = ((zz - pz) ** 2 + (yy - py) ** 2 + (xx - px) ** 2).sqrt()
                    d = torch.where(ok.expand_as(d), d, torch.full_like(d, float("inf")))
                    closer = d < d1
                    d2 = torch.where(closer, d1, torch.minimum(d2, d))
                    best = torch.where(closer, lab[czb, cyb, cxb], best)
                    d1 = torch.where(closer, d, d1)
        best[(d2 - d1) < membrane] = 0
        out[z0:z1] = best
    if salt > 0:
        m = torch.rand(out.shape, generator=g, device=dev) < salt
        out[m] = torch.randint(1, int(label_max) + 1, (int(m.sum()),), generator=g, device=dev)
    return _to_dtype(out, dtype)


def _to_dtype(t, dtype):
    """Cast to the signed type of the dtype's width (the library views it as unsigned)."""
    import torch
    return t.to({np.uint8: torch.uint8, np.uint16: torch.int16, np.uint32: torch.int32,
                 np.uint64: torch.int64}[dtype])


def random_volume(rng: np.random.Generator, lo: int = 64, hi: int = 320):
    """One volume of the training distribution: Voronoi (1 to ~1e6 seeds),
    binary Bernoulli (p in 0.05-0.95) or multilabel Bernoulli (K in 2-1000),
    as uint8/16/32/64, edges log-uniform in [lo, hi].  Returns (tensor,
    connectivity, binary_image, description)."""
    import torch
    shape = tuple(int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))))) for _ in range(3))
    dtype = [np.uint8, np.uint16, np.uint32, np.uint64][int(rng.integers(0, 4))]
    kind = int(rng.integers(0, 3))
    conn = int(rng.choice([26, 18, 6]))
    seed = int(rng.integers(0, 2 ** 31))
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    if kind == 0:
        cell = float(math.exp(rng.uniform(math.log(2.5), math.log(max(shape) * 1.5))))
        lmax = {np.uint8: 255, np.uint16: 65535}.get(dtype, 1 << 20)
        vol = voronoi_gpu(shape, cell, lmax, seed, dtype, salt=float(rng.choice([0.0, 0.02])))
        return vol, conn, False, f"voronoi cell={cell:.1f}"
    if kind == 1:
        p = float(rng.uniform(0.05, 0.95))
        vol = (torch.rand(shape, generator=g, device="cuda") < p).to(torch.uint8)
        return _to_dtype(vol.to(torch.int64), dtype), conn, True, f"bernoulli p={p:.2f}"
    K = int(rng.integers(2, 1001))
    p = float(rng.uniform(0.2, 1.0))
    kmax = min(K, 255) if dtype == np.uint8 else K
    v = torch.randint(1, kmax + 1, shape, generator=g, device="cuda")
    v = v * (torch.rand(shape, generator=g, device="cuda") < p)
    return _to_dtype(v, dtype), conn, False, f"multilabel K={kmax} p={p:.2f}"


def collect(n_volumes: int, seed: int, lo: int = 64, hi: int = 320,
            repeats: int = 1) -> Tuple[np.ndarray, np.ndarray, List[str]]:
    """Features and autotuner timings (log-ms of every configuration) of
    n_volumes volumes drawn from random_volume with the given seed."""
    from .tuning import autotune, autotune_reset
    rng = np.random.default_rng(seed)
    X, Y, desc = [], [], []
    for _ in range(n_volumes):
        vol, conn, binary, d = random_volume(rng, lo, hi)
        f = features(vol, conn, binary)
        res = autotune(vol, connectivity=conn, binary_image=binary, repeats=repeats)
        y = np.full(N_OUTPUTS, np.nan, np.float32)
        for i, c in enumerate(CONFIGS):
            if c in res["ms"]:
                y[i] = math.log(res["ms"][c])
        X.append(f)
        Y.append(y)
        desc.append(d)
    autotune_reset()
    return np.stack(X), np.stack(Y), desc


def regret(Y_true: np.ndarray, Y_pred: np.ndarray, min_margin: float = 0.05) -> Dict[str, float]:
    """How much slower the model's picks are than the measured best, over
    volumes (Y in log-ms; NaN = not timed).  "fallback" figures let the
    exhaustive autotuner decide where the predicted runner-up is within
    min_margin (as cc3d_gpu_cost_model_choose does)."""
    true = np.where(np.isnan(Y_true), np.inf, Y_true)
    pred = np.where(np.isnan(Y_true), np.inf, Y_pred)
    pick = pred.argmin(axis=1)
    best = true.min(axis=1)
    picked = true[np.arange(len(true)), pick]
    r = np.exp(picked - best) - 1.0
    srt = np.sort(pred, axis=1)
    unsure = (srt[:, 1] - srt[:, 0]) < np.log1p(min_margin)
    picked_fb = np.where(unsure, best, picked)
    r_fb = np.exp(picked_fb - best) - 1.0
    plain = true[:, 0]  # list/8x8: the single default configuration
    return {"mean_regret": float(r.mean()), "p95_regret": float(np.percentile(r, 95)),
            "top1": float((pick == true.argmin(axis=1)).mean()),
            "time_vs_best": float(np.exp(picked).sum() / np.exp(best).sum()),
            "time_vs_plain": float(np.exp(picked).sum() / np.exp(plain).sum()),
            "fallback_fraction": float(unsure.mean()),
            "fallback_mean_regret": float(r_fb.mean()),
            "fallback_time_vs_plain": float(np.exp(picked_fb).sum() / np.exp(plain).sum())}
