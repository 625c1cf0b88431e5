"""Neural-network layers of the sparse-convolution path."""

from .modules import AvgPool, BatchNorm, GroupNorm, MaxPool, RecomputeSequential, ReLU, Sequential, SparseConv3d, UpsamplingNearest
from .vdbtensor import VDBTensor

__all__ = ["SparseConv3d", "ReLU", "Sequential", "RecomputeSequential", "VDBTensor", "MaxPool", "AvgPool",
           "UpsamplingNearest", "BatchNorm", "GroupNorm"]
