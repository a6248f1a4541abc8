"""cc3d_gb300 -- GB300 (sm_103a) implementation of cc3d's labelling path.

Drop-in for ``cc3d.connected_components``, ``cc3d.statistics`` and
``cc3d.estimate_provisional_labels``; the work runs in hand-written CUDA
kernels behind the C ABI of include/cc3d_gpu.h (libcc3d_gpu.so).
"""
from ._build import build  # noqa: F401
from .api import (  # noqa: F401
    DimensionError,
    connected_components,
    estimate_provisional_labels,
    statistics,
)
from . import _native  # noqa: F401
from .tuning import autotune, autotune_reset, set_tile_pass, tile_pass_choice  # noqa: F401
from .batch import autotune_batch, connected_components_batch, set_batch_mode  # noqa: F401
from . import costmodel, tuning  # noqa: F401
from .filters import dust, largest_k  # noqa: F401
from .stack import LabelStack, connected_components_stack  # noqa: F401
from .graphs import (  # noqa: F401
    color_connectivity_graph, contacts, draw, each, region_graph, runs, voxel_connectivity_graph)

__all__ = [
    "build",
    "connected_components",
    "estimate_provisional_labels",
    "statistics",
    "DimensionError",
    "connected_components_batch",
    "set_batch_mode",
    "dust",
    "largest_k",
    "contacts",
    "region_graph",
    "runs",
    "draw",
    "each",
    "autotune_batch",
    "autotune",
    "autotune_reset",
    "set_tile_pass",
    "tile_pass_choice",
    "voxel_connectivity_graph",
    "color_connectivity_graph",
    "connected_components_stack",
    "LabelStack",
]
