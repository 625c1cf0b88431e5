"""Neural-network layers of the sparse-convolution path."""

from .modules import (
    CELU,
    ELU,
    GELU,
    SELU,
    AvgPool,
    BatchNorm,
    Dropout,
    FillFromGrid,
    GroupNorm,
    LeakyReLU,
    Linear,
    MaxPool,
    RecomputeSequential,
    ReLU,
    Sequential,
    Sigmoid,
    SiLU,
    SparseConv3d,
    SyncBatchNorm,
    Tanh,
    UpsamplingNearest,
)
from .vdbtensor import VDBTensor, vdbtensor_from_dense

__all__ = ["VDBTensor", "vdbtensor_from_dense", "MaxPool", "AvgPool", "UpsamplingNearest", "FillFromGrid", "SparseConv3d", "GroupNorm",
           "BatchNorm", "SyncBatchNorm", "Linear", "ReLU", "LeakyReLU", "ELU", "CELU", "GELU", "SELU", "SiLU", "Tanh",
           "Sigmoid", "Dropout", "Sequential", "RecomputeSequential"]
