"""VDBTensor: a GridBatch plus its per-voxel features (and an optional cached kernel map).

Mirrors fvdb/nn/vdbtensor.py:21-55 of the reference: the stride-1 kernel map of the grid is
carried between layers so consecutive same-grid convolutions do not rebuild it.
"""

from __future__ import annotations

from dataclasses import dataclass

import torch

from ..grid_batch import GridBatch
from ..jagged_tensor import JaggedTensor
from ..sparse_conv_pack_info import SparseConvPackInfo


@dataclass
class VDBTensor:
    grid: GridBatch
    data: JaggedTensor
    kmap: SparseConvPackInfo | None = None

    def __post_init__(self):
        if not isinstance(self.grid, GridBatch):
            raise TypeError("grid should be of type GridBatch")
        if isinstance(self.data, torch.Tensor):
            self.data = self.grid.jagged_like(self.data)
        if not isinstance(self.data, JaggedTensor):
            raise TypeError("data must be a JaggedTensor or a torch.Tensor")
        if self.grid.grid_count != len(self.data):
            raise ValueError("grid and feature should have the same batch size")
        if self.grid.total_voxels != self.data.jdata.size(0):
            raise ValueError("grid and feature should have the same total voxel count")
        if self.kmap is not None:
            if not isinstance(self.kmap, SparseConvPackInfo):
                raise TypeError("kmap should be of type SparseConvPackInfo")
            if not (
                self.grid.is_same(self.kmap.source_grid)
                and self.grid.is_same(self.kmap.target_grid)
                and self.kmap.stride == (1, 1, 1)
            ):
                raise ValueError("kmap should operate on the same grid as this tensor")

    def __len__(self):
        return self.grid.grid_count

    @property
    def jdata(self) -> torch.Tensor:
        return self.data.jdata

    @property
    def device(self) -> torch.device:
        return self.grid.device

    @property
    def dtype(self) -> torch.dtype:
        return self.data.dtype

    def is_same(self, other) -> bool:
        g = other.grid if isinstance(other, VDBTensor) else other
        return self.grid.is_same(g)
