"""cc3d.connected_components_stack on the GPU (cc3d/__init__.py:324-501).

Connected components of a volume that arrives as a sequence of slabs along
its third axis (numpy axis 2), each of the same width and height.  Every slab
is labelled on the device as it arrives (connected_components with uint64
labels, offset by the labels of the slabs before it); the pairs of labels
that touch across each seam (the previous slab's last plane against the new
slab's first plane, 6- or 26-connected, equal values or both foreground for
binary images) are collected; at the end each label is mapped to the
smallest label of its group, as the reference's disjoint set does, and the
groups are numbered 1..N in increasing order of that label, which is how a
sorted label table renumbers.  The relabel runs on the device
(cc3d_gpu_remap_labels), slab by slab.

The reference compresses the result into a crackle array, which needs the
crackle package; here the result is a LabelStack holding a numpy array in
Fortran order (slabs contiguous) with the few methods of the crackle array
that callers use (indexing, decompress, num_labels).  Its dtype is the
smallest unsigned type that holds N.
"""
from __future__ import annotations

from typing import Any, Iterable

import numpy as np

from .api import connected_components
from .filters import _remap


class LabelStack:
    """Labels of a stacked volume: a numpy array behind the interface of the
    reference's crackle array (``arr[...]``, ``decompress()``,
    ``num_labels()``, ``shape``, ``dtype``)."""

    def __init__(self, labels: np.ndarray, n: int, has_background: bool):
        self._labels = labels
        self._n = n
        self._bg = has_background

    @property
    def shape(self):
        return self._labels.shape

    @property
    def dtype(self):
        return self._labels.dtype

    def __getitem__(self, item):
        return self._labels[item]

    def __array__(self, dtype=None, copy=None):
        return self._labels if dtype is None else self._labels.astype(dtype)

    def decompress(self) -> np.ndarray:
        return self._labels

    def numpy(self) -> np.ndarray:
        return self._labels

    def num_labels(self) -> int:
        """Distinct values, background included (as a crackle array counts them)."""
        return self._n + (1 if self._bg else 0)


def _seam_pairs(bottom_img, bottom_lab, top_img, top_lab, connectivity: int, binary_image: bool):
    """(bottom label, top label) pairs joined across one seam: the reference's
    loops (cc3d/__init__.py:425-463) as array operations.  For 26 the
    reference skips a voxel's diagonals once the voxel straight above joins;
    those diagonals join top voxels already joined to that one, so every
    offset can be taken."""
    sx, sy = bottom_img.shape
    offs = [(0, 0)] if connectivity == 6 else [(dx, dy) for dx in (-1, 0, 1) for dy in (-1, 0, 1)]
    pairs = []
    for dx, dy in offs:
        bx = slice(max(0, -dx), sx - max(0, dx))
        by = slice(max(0, -dy), sy - max(0, dy))
        tx = slice(max(0, dx), sx + min(0, dx))
        ty = slice(max(0, dy), sy + min(0, dy))
        bl, tl = bottom_lab[bx, by], top_lab[tx, ty]
        bi, ti = bottom_img[bx, by], top_img[tx, ty]
        rel = (bi != 0) & (ti != 0) if binary_image else (bi == ti)
        m = (bl != 0) & (tl != 0) & rel
        if m.any():
            pairs.append(np.stack([bl[m], tl[m]], axis=1))
    return np.concatenate(pairs) if pairs else np.zeros((0, 2), np.uint64)


def connected_components_stack(stacked_images: Iterable[Any], connectivity: int = 26, return_N: bool = False,
                               binary_image: bool = False):
    """Connected components of the volume the slabs form along axis 2
    (cc3d/__init__.py:324-501); returns a LabelStack (and N)."""
    if connectivity not in (6, 26):
        raise ValueError(f"Connectivity must be 6 or 26. Got: {connectivity}")
    slabs, pairs = [], []
    offset = 0
    prev_img = prev_lab = None
    xy = None
    for image in stacked_images:
        image = image.cpu().numpy() if hasattr(image, "cpu") else np.asarray(image)
        if image.ndim != 3:
            raise ValueError(f"stacked images must be 3D. Got: {image.ndim}D")
        if xy is None:
            xy = image.shape[:2]
        elif image.shape[:2] != xy:
            raise ValueError(f"every image needs the same width and height: {image.shape[:2]} != {xy}")
        cc, n = connected_components(image, connectivity=connectivity, return_N=True, out_dtype=np.uint64,
                                     binary_image=bool(binary_image))
        cc = np.asarray(cc)
        if offset:
            np.add(cc, np.uint64(offset), out=cc, where=(cc != 0))
        if prev_img is not None:
            pairs.append(_seam_pairs(prev_img, prev_lab, image[:, :, 0], cc[:, :, 0], connectivity,
                                     bool(binary_image)))
        offset += int(n)
        slabs.append(cc)
        prev_img, prev_lab = image[:, :, -1], cc[:, :, -1]
    if not slabs:
        raise ValueError("no images to stack")

    # every label -> the smallest label of its group -> its rank among those
    rep = np.arange(offset + 1, dtype=np.uint64)
    allp = np.concatenate(pairs) if pairs else np.zeros((0, 2), np.uint64)
    if len(allp):
        import scipy.sparse as sp
        from scipy.sparse.csgraph import connected_components as graph_components
        nodes, inv = np.unique(allp.reshape(-1), return_inverse=True)
        inv = inv.reshape(-1, 2)
        g = sp.coo_matrix((np.ones(len(inv), np.int8), (inv[:, 0], inv[:, 1])), shape=(len(nodes), len(nodes)))
        ncomp, comp = graph_components(g, directed=False)
        smallest = np.full(ncomp, np.iinfo(np.uint64).max, dtype=np.uint64)
        np.minimum.at(smallest, comp, nodes)
        rep[nodes.astype(np.int64)] = smallest[comp]
    uniq = np.unique(rep[1:])
    N = int(len(uniq))
    table = np.zeros(offset + 1, dtype=np.uint64)
    table[1:] = np.searchsorted(uniq, rep[1:]) + 1
    out_dtype = next(np.dtype(t) for t in (np.uint8, np.uint16, np.uint32, np.uint64)
                     if N <= np.iinfo(t).max)
    table = table.astype(out_dtype)
    depth = sum(s.shape[2] for s in slabs)
    out = np.empty(xy + (depth,), dtype=out_dtype, order="F")
    z = 0
    has_bg = False
    for cc in slabs:
        d = cc.shape[2]
        out[:, :, z:z + d] = _remap(cc, table, out_dtype, "F")
        has_bg = has_bg or bool((cc == 0).any())
        z += d
    arr = LabelStack(out, N, has_bg)
    return (arr, N) if return_N else arr
