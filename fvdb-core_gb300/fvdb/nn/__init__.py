"""Neural-network layers of the sparse-convolution path."""

from .modules import ReLU, SparseConv3d
from .vdbtensor import VDBTensor

__all__ = ["SparseConv3d", "ReLU", "VDBTensor"]
