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


@dataclass(eq=False)
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

    def __getitem__(self, idx: int) -> "VDBTensor":
        """Grid `idx` of the batch with its features (no kernel map)."""
        return VDBTensor(self.grid[idx], self.data[idx])

    def to_dense(self) -> torch.Tensor:
        """[B, X, Y, Z, C] dense features over the batch's bounding box (zeros off the grid)."""
        return self.grid.write_to_dense_xyzc(self.data)

    def clear_cache(self) -> None:
        self.kmap = None

    # ------------------------------------------------------------ arithmetic on the features
    # Elementwise operators act on the feature rows and keep grid and kernel map (reference:
    # fvdb/nn/vdbtensor.py:80-214); a VDBTensor operand must have one row per voxel of this grid.
    def _other(self, other):
        if isinstance(other, VDBTensor):
            if other.grid.total_voxels != self.grid.total_voxels or other.grid.grid_count != self.grid.grid_count:
                raise ValueError("VDBTensor operands must live on grids with the same voxel counts")
            return other.data.jdata
        if isinstance(other, JaggedTensor):
            return other.jdata
        return other

    def _wrap(self, t: torch.Tensor) -> "VDBTensor":
        return VDBTensor(self.grid, self.grid.jagged_like(t), self.kmap)

    def _binop(self, other, op) -> "VDBTensor":
        return self._wrap(op(self.data.jdata, self._other(other)))

    def _binop_(self, other, op) -> "VDBTensor":
        op(self.data.jdata, self._other(other))
        return self

    def __add__(self, other):
        return self._binop(other, torch.add)

    def __radd__(self, other):
        return self._binop(other, torch.add)

    def __sub__(self, other):
        return self._binop(other, torch.sub)

    def __mul__(self, other):
        return self._binop(other, torch.mul)

    def __rmul__(self, other):
        return self._binop(other, torch.mul)

    def __pow__(self, other):
        return self._binop(other, torch.pow)

    def __truediv__(self, other):
        return self._binop(other, torch.true_divide)

    def __floordiv__(self, other):
        return self._binop(other, torch.floor_divide)

    def __mod__(self, other):
        return self._binop(other, torch.remainder)

    def __neg__(self):
        return self._wrap(-self.data.jdata)

    def __gt__(self, other):
        return self._binop(other, torch.gt)

    def __lt__(self, other):
        return self._binop(other, torch.lt)

    def __ge__(self, other):
        return self._binop(other, torch.ge)

    def __le__(self, other):
        return self._binop(other, torch.le)

    def __eq__(self, other):
        return self._binop(other, torch.eq)

    def __ne__(self, other):
        return self._binop(other, torch.ne)

    __hash__ = object.__hash__

    def __iadd__(self, other):
        return self._binop_(other, lambda a, b: a.add_(b))

    def __isub__(self, other):
        return self._binop_(other, lambda a, b: a.sub_(b))

    def __imul__(self, other):
        return self._binop_(other, lambda a, b: a.mul_(b))

    def __ipow__(self, other):
        return self._binop_(other, lambda a, b: a.pow_(b))

    def __itruediv__(self, other):
        return self._binop_(other, lambda a, b: a.div_(b))

    def __ifloordiv__(self, other):
        return self._binop_(other, lambda a, b: a.floor_divide_(b))

    def __imod__(self, other):
        return self._binop_(other, lambda a, b: a.remainder_(b))

    def sqrt(self):
        return self._wrap(self.data.jdata.sqrt())

    def abs(self):
        return self._wrap(self.data.jdata.abs())

    def round(self):
        return self._wrap(self.data.jdata.round())

    def floor(self):
        return self._wrap(self.data.jdata.floor())

    def ceil(self):
        return self._wrap(self.data.jdata.ceil())

    def sqrt_(self):
        self.data.jdata.sqrt_()
        return self

    def abs_(self):
        self.data.jdata.abs_()
        return self

    def round_(self):
        self.data.jdata.round_()
        return self

    def floor_(self):
        self.data.jdata.floor_()
        return self

    def ceil_(self):
        self.data.jdata.ceil_()
        return self

    def detach(self) -> "VDBTensor":
        return self._wrap(self.data.jdata.detach())

    def clone(self) -> "VDBTensor":
        return self._wrap(self.data.jdata.clone())

    def type(self, dtype: torch.dtype) -> "VDBTensor":
        return VDBTensor(self.grid, self.grid.jagged_like(self.data.jdata.type(dtype)))

    def to(self, device_or_dtype) -> "VDBTensor":
        """A dtype converts the features; a device must be the grid's own (grids live on one
        CUDA device)."""
        if isinstance(device_or_dtype, torch.dtype):
            return self._wrap(self.data.jdata.to(device_or_dtype))
        return VDBTensor(self.grid.to(device_or_dtype), self.data.to(device_or_dtype), self.kmap)

    def requires_grad_(self, requires_grad: bool = True) -> "VDBTensor":
        self.data.jdata.requires_grad_(requires_grad)
        return self

    @property
    def requires_grad(self) -> bool:
        return self.data.jdata.requires_grad

    @property
    def jidx(self) -> torch.Tensor:
        return self.data.jidx

    @property
    def joffsets(self) -> torch.Tensor:
        return self.data.joffsets

    @property
    def eshape(self):
        return self.data.eshape

    @property
    def lshape(self):
        return self.data.lshape

    @property
    def is_cuda(self) -> bool:
        return self.data.jdata.is_cuda

    @property
    def grid_count(self) -> int:
        return self.grid.grid_count

    @property
    def total_voxels(self) -> int:
        return self.grid.total_voxels

    @property
    def num_voxels(self) -> torch.Tensor:
        return self.grid.num_voxels

    @property
    def cum_voxels(self) -> torch.Tensor:
        return self.grid.cum_voxels

    @property
    def ijk(self) -> JaggedTensor:
        return self.grid.ijk

    @property
    def voxel_sizes(self) -> torch.Tensor:
        return self.grid.voxel_sizes

    @property
    def origins(self) -> torch.Tensor:
        return self.grid.origins

    @property
    def total_leaf_nodes(self) -> int:
        return self.grid.total_leaf_nodes

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


def vdbtensor_from_dense(dense_data: torch.Tensor, ijk_min=0, voxel_sizes=1, origins=0) -> VDBTensor:
    """A VDBTensor holding every voxel of a dense [B, X, Y, Z, C...] block: dense_data[b, 0, 0, 0]
    lands on voxel ijk_min of grid b (reference: fvdb/nn/vdbtensor.py:372-391)."""
    grid = GridBatch.from_dense(dense_data.size(0), list(dense_data.shape[1:4]), ijk_min=ijk_min,
                                voxel_sizes=voxel_sizes, origins=origins, device=dense_data.device)
    return VDBTensor(grid, grid.read_from_dense_xyzc(dense_data.contiguous(), dense_origins=ijk_min))
