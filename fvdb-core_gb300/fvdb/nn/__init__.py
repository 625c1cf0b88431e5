"""Neural-network layers of the sparse-convolution path."""

from .modules import RecomputeSequential, ReLU, Sequential, SparseConv3d
from .vdbtensor import VDBTensor

__all__ = ["SparseConv3d", "ReLU", "Sequential", "RecomputeSequential", "VDBTensor"]
