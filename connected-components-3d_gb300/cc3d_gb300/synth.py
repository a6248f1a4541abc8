"""Seeded synthetic volumes with the shapes and value distributions of the
benchmark workloads (no external dataset is used).

* voronoi_volume: a Voronoi partition of uniform random seed points, one
  random label per cell, a one-voxel background membrane where the nearest and
  second-nearest seed distances (from voxel centres) differ by less than 1.0,
  then a fraction of voxels reassigned to uniform random labels ("salt").
* bernoulli_volume: i.i.d. Bernoulli(p) foreground (values 0/1).
* batch_shapes: the mixed-size stream (each dimension log-uniform).

Arrays are C ordered: shape (z, y, x), x fastest.
"""
from __future__ import annotations

import numpy as np


def voronoi_volume(shape, n_seeds: int, label_max: int, seed: int, dtype=np.uint32,
                   salt: float = 0.02, membrane: float = 1.0, workers: int = -1) -> np.ndarray:
    from scipy.spatial import cKDTree

    shape = tuple(int(s) for s in shape)
    rng = np.random.default_rng(seed)
    pts = rng.uniform(0.0, 1.0, size=(n_seeds, 3)) * np.array(shape, dtype=np.float64)
    cell_labels = rng.integers(1, label_max + 1, size=n_seeds, dtype=np.uint64)
    tree = cKDTree(pts)
    out = np.empty(shape, dtype=dtype)
    nz, ny, nx = shape
    yy, xx = np.meshgrid(np.arange(ny) + 0.5, np.arange(nx) + 0.5, indexing="ij")
    plane = np.stack([np.zeros_like(yy), yy, xx], axis=-1).reshape(-1, 3)
    step = max(1, (1 << 22) // max(1, ny * nx))
    k = 2 if n_seeds >= 2 else 1
    for z0 in range(0, nz, step):
        z1 = min(nz, z0 + step)
        q = np.concatenate([plane + np.array([z + 0.5, 0.0, 0.0]) for z in range(z0, z1)])
        d, idx = tree.query(q, k=k, workers=workers)
        if k == 2:
            lab = cell_labels[idx[:, 0]]
            lab[(d[:, 1] - d[:, 0]) < membrane] = 0
        else:
            lab = cell_labels[np.asarray(idx).reshape(-1)]
        out[z0:z1] = lab.reshape(z1 - z0, ny, nx).astype(dtype)
    if salt > 0:
        flat = out.reshape(-1)
        m = rng.random(flat.size, dtype=np.float32) < salt
        flat[m] = rng.integers(1, label_max + 1, size=int(m.sum()), dtype=np.uint64).astype(dtype)
    return out


def bernoulli_volume(shape, p: float, seed: int, dtype=np.uint8) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return (rng.random(tuple(shape), dtype=np.float32) < p).astype(dtype)


def batch_shapes(n: int, lo: int, hi: int, seed: int):
    rng = np.random.default_rng(seed)
    dims = np.exp(rng.uniform(np.log(lo), np.log(hi), size=(n, 3)))
    return [tuple(int(round(v)) for v in row) for row in dims]
