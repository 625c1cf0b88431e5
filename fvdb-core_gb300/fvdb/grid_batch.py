"""GridBatch: a jagged batch of sparse voxel grids on one CUDA device.

Conv-path subset of the reference's ``fvdb.GridBatch`` (fvdb/grid_batch.py): the same
constructors, ``conv_grid`` / ``sparse_conv_kernel_map``, ``ijk`` / ``jidx`` / ``joffsets``,
voxel counts, dense read/write and ``ijk_to_index`` used by the convolution tests.
Voxels are numbered in NanoVDB OnIndex order per grid, offset by the voxels of the
preceding grids, so index tensors agree with the reference's.
"""

from __future__ import annotations

from typing import Sequence, Union

import torch

from . import _lib
from .jagged_tensor import JaggedTensor

Numeric = Union[int, float, Sequence, torch.Tensor]


def _device(device, inherit=None) -> torch.device:
    if device is None:
        if inherit is not None and isinstance(inherit, (torch.Tensor, JaggedTensor)):
            device = inherit.device
        else:
            device = "cuda"
    device = torch.device(device)
    if device.type != "cuda":
        raise ValueError("fvdb_gb300 grids live on CUDA devices; got device " + str(device))
    if device.index is None:
        device = torch.device("cuda", torch.cuda.current_device())
    return device


def _vec3i(v, name: str, positive: bool = False, nonneg: bool = False) -> list[int]:
    if isinstance(v, torch.Tensor):
        v = v.tolist()
    if isinstance(v, (int,)) or (hasattr(v, "__int__") and not isinstance(v, (list, tuple))):
        out = [int(v)] * 3
    else:
        v = list(v)
        if len(v) == 1:
            v = v * 3
        if len(v) != 3:
            raise ValueError(f"{name} must be a scalar or have 3 entries")
        for x in v:
            if isinstance(x, float) and not float(x).is_integer():
                raise TypeError(f"{name} must hold integers")
        out = [int(x) for x in v]
    if positive and any(x <= 0 for x in out):
        raise ValueError(f"{name} must be positive")
    if nonneg and any(x < 0 for x in out):
        raise ValueError(f"{name} must be non-negative")
    return out


def _per_grid(v, n: int) -> torch.Tensor:
    t = torch.as_tensor(v, dtype=torch.float64).cpu()
    if t.dim() == 0:
        t = t.reshape(1, 1).expand(n, 3)
    elif t.dim() == 1:
        t = t.reshape(1, -1).expand(n, 3) if t.numel() in (1, 3) else t
    if t.dim() != 2 or t.shape[0] != n or t.shape[1] != 3:
        raise ValueError(f"expected a value broadcastable to ({n}, 3)")
    return t.contiguous()


def _as_jagged(data) -> JaggedTensor:
    if isinstance(data, torch.Tensor):
        return JaggedTensor(data)
    if not isinstance(data, JaggedTensor):
        raise TypeError("data must be a JaggedTensor or a torch.Tensor")
    return data


def _mask_data(mask, grid) -> torch.Tensor | None:
    if mask is None:
        return None
    m = mask.jdata if isinstance(mask, JaggedTensor) else mask
    if m.dim() != 1 or m.shape[0] != grid.total_voxels:
        raise ValueError("subdivision mask must be either empty tensor or have one entry per voxel")
    if m.dtype != torch.bool:
        raise ValueError("subdivision mask must be a boolean tensor")
    return m


class GridBatch:
    def __init__(self, *, impl):
        self._impl = impl

    # ---------------------------------------------------------------- constructors -------
    @classmethod
    def from_ijk(cls, ijk, voxel_sizes: Numeric = 1, origins: Numeric = 0, device=None) -> "GridBatch":
        if isinstance(ijk, torch.Tensor):
            ijk = JaggedTensor(ijk)
        if not isinstance(ijk, JaggedTensor):
            raise TypeError("ijk must be a JaggedTensor or a torch.Tensor")
        dev = _device(device, ijk)
        jd = ijk.jdata
        if jd.is_floating_point():
            raise TypeError("ijk must have an integer dtype")
        C = _lib.load()
        B = ijk.num_outer_lists()
        impl = C.GridImpl.from_ijk(jd.to(dev), ijk.joffsets.to(dev), _per_grid(voxel_sizes, B), _per_grid(origins, B))
        return cls(impl=impl)

    @classmethod
    def from_points(cls, points, voxel_sizes: Numeric = 1, origins: Numeric = 0, device=None) -> "GridBatch":
        if isinstance(points, torch.Tensor):
            points = JaggedTensor(points)
        if not isinstance(points, JaggedTensor):
            raise TypeError("points must be a JaggedTensor or a torch.Tensor")
        dev = _device(device, points)
        C = _lib.load()
        B = points.num_outer_lists()
        impl = C.GridImpl.from_points(
            points.jdata.to(dev), points.joffsets.to(dev), _per_grid(voxel_sizes, B), _per_grid(origins, B)
        )
        return cls(impl=impl)

    @classmethod
    def from_dense(
        cls,
        num_grids: int,
        dense_dims: Numeric,
        ijk_min: Numeric = 0,
        voxel_sizes: Numeric = 1,
        origins: Numeric = 0,
        mask: torch.Tensor | None = None,
        device=None,
    ) -> "GridBatch":
        dims = _vec3i(dense_dims, "dense_dims", positive=True)
        mn = _vec3i(ijk_min, "ijk_min")
        dev = _device(device, mask)
        ax = [torch.arange(d, device=dev, dtype=torch.int32) + m for d, m in zip(dims, mn)]
        gi, gj, gk = torch.meshgrid(*ax, indexing="ij")
        ijk = torch.stack([gi, gj, gk], -1).reshape(-1, 3)
        if mask is not None:
            m = mask.to(dev).reshape(-1).bool()
            if m.numel() != ijk.shape[0]:
                raise ValueError("mask must have dense_dims entries")
            ijk = ijk[m]
        ijk = ijk.repeat(num_grids, 1)
        off = torch.arange(num_grids + 1, dtype=torch.int64, device=dev) * (ijk.shape[0] // max(num_grids, 1))
        return cls.from_ijk(JaggedTensor.from_data_and_offsets(ijk, off), voxel_sizes, origins, device=dev)

    # ---------------------------------------------------------------- convolution -------
    def conv_grid(self, kernel_size: Numeric, stride: Numeric = 0) -> "GridBatch":
        ks = _vec3i(kernel_size, "kernel_size", positive=True)
        st = _vec3i(stride, "stride", nonneg=True)
        return GridBatch(impl=self._impl.conv_grid(ks, st))

    def sparse_conv_kernel_map(self, kernel_size: Numeric, stride: Numeric, target_grid: "GridBatch | None" = None):
        from .sparse_conv_pack_info import SparseConvPackInfo

        ks = _vec3i(kernel_size, "kernel_size", positive=True)
        st = _vec3i(stride, "stride", nonneg=True)
        st = [s if s > 0 else 1 for s in st]
        tgt = target_grid._impl if target_grid is not None else None
        C = _lib.load()
        impl = C.PackInfoImpl(ks, st, self._impl, tgt)
        return SparseConvPackInfo(impl=impl), GridBatch(impl=impl.target_grid)

    def sparse_conv_halo(self, input: JaggedTensor, weight: torch.Tensor, variant: int = 8) -> JaggedTensor:
        """Stride-1 3x3x3 convolution of `input` (one feature row per voxel) over this grid, with
        the reference's arguments, checks and error types (GridBatch.cpp:776-793,
        autograd/SparseConvolutionHalo.cpp:17-86).  Computed without a kernel map: a CTA per
        leaf stages the leaf's 10^3 halo (through the leaf hash) in shared memory and convolves
        its active voxels; x, y, z offsets meet weight dims 4, 3, 2 (K2, K1, K0), the kernel
        map's convention, so the result equals sparse_conv_3d over the grid's stride-1 3^3 map
        up to summation order.  `variant` picks one of the reference's halo kernels and is
        accepted for compatibility (there is one implementation)."""
        if not isinstance(input, JaggedTensor):
            raise TypeError("input must be a JaggedTensor")
        data = input.jdata
        if not data.is_floating_point():
            raise TypeError("input must have a floating point type")
        if data.shape[0] != self.total_voxels:
            raise ValueError("Value count not match!")
        if input.num_outer_lists() != self.grid_count:
            raise ValueError("Batch size not match!")
        if not weight.is_floating_point():
            raise TypeError("kernels must have a floating point type")
        if weight.dim() != 5:
            raise ValueError(
                f"Expected kernels to have 5 dimensions (shape (out_ch, in_ch, d, h, w)) but got {weight.dim()} dimensions")
        if not (weight.shape[2] == weight.shape[3] == weight.shape[4] == 3):
            raise NotImplementedError("sparse_conv_halo only supports kernels of size 3x3x3")
        if not data.is_contiguous():
            raise ValueError("features must be contiguous")
        if data.dim() != 2:
            raise ValueError(f"Expected features to have 2 dimensions (shape (n, nF)) but got {data.dim()} dimensions")
        if weight.shape[1] != data.shape[1]:
            raise ValueError(f"Expected input channels of kernels ({weight.shape[1]}) to equal input channels of "
                             f"features: {data.shape[1]}")
        from ._halo import HaloConvFunction

        return input.jagged_like(HaloConvFunction.apply(self._impl, data, weight))

    # ---------------------------------------------------------------- pooling -----------
    def coarsened_grid(self, coarsening_factor: Numeric) -> "GridBatch":
        """Voxels floor(ijk / factor) (fvdb/grid_batch.py:487-501), voxel size factor * w and
        origin o + (factor - 1) * w / 2."""
        f = _vec3i(coarsening_factor, "coarsening_factor", positive=True)
        return GridBatch(impl=self._impl.coarsened_grid(f))

    def subdivided_grid(self, subdiv_factor: Numeric, mask: JaggedTensor | torch.Tensor | None = None) -> "GridBatch":
        """Every voxel (where `mask` is true) split into factor^3 children (fvdb/grid_batch.py,
        GridBatch.cpp:645-650), voxel size w / factor and origin o - (factor - 1) * w / (2 factor)."""
        f = _vec3i(subdiv_factor, "subdiv_factor", positive=True)
        m = _mask_data(mask, self)
        return GridBatch(impl=self._impl.subdivided_grid(f, m))

    def max_pool(self, pool_factor: Numeric, data: JaggedTensor, stride: Numeric = 0,
                 coarse_grid: "GridBatch | None" = None) -> tuple[JaggedTensor, "GridBatch"]:
        """Max pooling onto `coarse_grid` (default: coarsened_grid(stride)); windows start at
        coarse ijk * stride and span pool_factor voxels per axis; an empty window is -inf
        (fvdb/grid_batch.py:1059-1095, GridBatch.cpp:241-274)."""
        return self._pool(_lib.load().POOL_MAX, pool_factor, data, stride, coarse_grid)

    def avg_pool(self, pool_factor: Numeric, data: JaggedTensor, stride: Numeric = 0,
                 coarse_grid: "GridBatch | None" = None) -> tuple[JaggedTensor, "GridBatch"]:
        """Average pooling: the window's sum over its active voxels divided by the window volume
        (fvdb/grid_batch.py:384-419, GridBatch.cpp:276-310)."""
        return self._pool(_lib.load().POOL_AVG, pool_factor, data, stride, coarse_grid)

    def _pool(self, mode, pool_factor, data, stride, coarse_grid):
        from ._pool import PoolFunction

        pf = _vec3i(pool_factor, "pool_factor", positive=True)
        st = _vec3i(stride, "stride", nonneg=True)
        st = [s if s > 0 else p for s, p in zip(st, pf)]
        data = _as_jagged(data)
        if coarse_grid is None:
            coarse_grid = self.coarsened_grid(st)
        out = PoolFunction.apply(mode, self._impl, coarse_grid._impl, pf, st, data.jdata)
        return coarse_grid.jagged_like(out), coarse_grid

    def subdivide(self, subdiv_factor: Numeric, data: JaggedTensor, mask: JaggedTensor | torch.Tensor | None = None,
                  fine_grid: "GridBatch | None" = None) -> tuple[JaggedTensor, "GridBatch"]:
        """Nearest upsampling onto `fine_grid` (default: subdivided_grid(factor, mask)): a fine
        voxel takes the features of its coarse parent floor(ijk / factor) (fvdb/grid_batch.py:1465-1500,
        GridBatch.cpp:313-345)."""
        from ._pool import UpsampleFunction

        f = _vec3i(subdiv_factor, "subdiv_factor", positive=True)
        data = _as_jagged(data)
        if fine_grid is None:
            fine_grid = self.subdivided_grid(f, mask)
        out = UpsampleFunction.apply(self._impl, fine_grid._impl, f, data.jdata)
        return fine_grid.jagged_like(out), fine_grid

    # ---------------------------------------------------------------- properties --------
    @property
    def grid_count(self) -> int:
        return int(self._impl.grid_count)

    def __len__(self) -> int:
        return self.grid_count

    @property
    def total_voxels(self) -> int:
        return int(self._impl.total_voxels)

    @property
    def total_leaf_nodes(self) -> int:
        return int(self._impl.total_leaf_nodes)

    @property
    def joffsets(self) -> torch.Tensor:
        return self._impl.joffsets

    @property
    def num_voxels(self) -> torch.Tensor:
        h = self._impl.joffsets_host
        return (h[1:] - h[:-1]).to(self.device)

    def num_voxels_at(self, bi: int) -> int:
        h = self._impl.joffsets_host
        return int(h[bi + 1] - h[bi])

    def cum_voxels_at(self, bi: int) -> int:
        return int(self._impl.joffsets_host[bi])

    @property
    def cum_voxels(self) -> torch.Tensor:
        return self._impl.joffsets_host[:-1].to(self.device)

    @property
    def ijk(self) -> JaggedTensor:
        return JaggedTensor.from_data_and_offsets(self._impl.ijk, self._impl.joffsets)

    @property
    def jidx(self) -> torch.Tensor:
        return self._impl.jidx()

    @property
    def device(self) -> torch.device:
        return self._impl.device

    @property
    def voxel_sizes(self) -> torch.Tensor:
        return self._impl.voxel_sizes.to(self.device)

    @property
    def origins(self) -> torch.Tensor:
        return self._impl.origins.to(self.device)

    def jagged_like(self, data: torch.Tensor) -> JaggedTensor:
        if data.shape[0] != self.total_voxels:
            raise ValueError("data must have one row per voxel")
        return JaggedTensor.from_data_and_offsets(data, self._impl.joffsets)

    def is_same(self, other: "GridBatch") -> bool:
        return isinstance(other, GridBatch) and other._impl is self._impl

    def __getitem__(self, bi: int) -> "GridBatch":
        if not isinstance(bi, int):
            raise TypeError("only integer indexing is supported")
        n = self.grid_count
        if bi < 0:
            bi += n
        if not 0 <= bi < n:
            raise IndexError("grid index out of range")
        s, e = self.cum_voxels_at(bi), self.cum_voxels_at(bi) + self.num_voxels_at(bi)
        ijk = self._impl.ijk[s:e]
        return GridBatch.from_ijk(ijk, self._impl.voxel_sizes[bi], self._impl.origins[bi], device=self.device)

    def __iter__(self):
        for b in range(self.grid_count):
            yield self[b]

    # ---------------------------------------------------------------- dense I/O ---------
    def _bbox(self):
        ijk = self._impl.ijk
        if ijk.shape[0] == 0:
            z = torch.zeros(3, dtype=torch.int64)
            return z, z - 1
        return ijk.min(0).values.to(torch.int64).cpu(), ijk.max(0).values.to(torch.int64).cpu()

    def write_to_dense_xyzc(self, sparse_data, min_coord=None, grid_size=None) -> torch.Tensor:
        """Dense [B, X, Y, Z, C] tensor (zeros where no voxel); default box = total bbox."""
        data = sparse_data.jdata if isinstance(sparse_data, JaggedTensor) else sparse_data
        if data.shape[0] != self.total_voxels:
            raise ValueError("sparse_data must have one row per voxel")
        lo, hi = self._bbox()
        B = self.grid_count
        mn = torch.as_tensor(min_coord, dtype=torch.int64).reshape(-1, 3).expand(B, 3) if min_coord is not None else lo.reshape(1, 3).expand(B, 3)
        size = _vec3i(grid_size, "grid_size", nonneg=True) if grid_size is not None else (hi - lo + 1).tolist()
        flat = data.reshape(data.shape[0], -1)
        out = torch.zeros((B, size[0], size[1], size[2], flat.shape[1]), dtype=data.dtype, device=data.device)
        ijk = self._impl.ijk.to(torch.int64)
        jidx = self.jidx.to(torch.int64)
        rel = ijk - mn.to(ijk.device)[jidx]
        ok = ((rel >= 0) & (rel < torch.tensor(size, device=rel.device))).all(1)
        idx = torch.nonzero(ok).squeeze(1)
        out = out.index_put((jidx[idx], rel[idx, 0], rel[idx, 1], rel[idx, 2]), flat[idx])
        return out.reshape((B, size[0], size[1], size[2]) + tuple(data.shape[1:]))

    def write_to_dense_czyx(self, sparse_data, min_coord=None, grid_size=None) -> torch.Tensor:
        d = self.write_to_dense_xyzc(sparse_data, min_coord, grid_size)
        d = d.reshape(d.shape[:4] + (-1,))
        return d.permute(0, 4, 3, 2, 1)

    def read_from_dense_xyzc(self, dense_data: torch.Tensor, dense_origins=0) -> JaggedTensor:
        B = self.grid_count
        org = torch.as_tensor(dense_origins, dtype=torch.int64).reshape(-1, 3).expand(B, 3).to(self.device)
        ijk = self._impl.ijk.to(torch.int64)
        jidx = self.jidx.to(torch.int64)
        rel = ijk - org[jidx]
        size = torch.tensor(dense_data.shape[1:4], device=rel.device)
        ok = ((rel >= 0) & (rel < size)).all(1)
        out = torch.zeros((ijk.shape[0],) + tuple(dense_data.shape[4:]), dtype=dense_data.dtype, device=dense_data.device)
        idx = torch.nonzero(ok).squeeze(1)
        out[idx] = dense_data[jidx[idx], rel[idx, 0], rel[idx, 1], rel[idx, 2]]
        return self.jagged_like(out)

    def read_from_dense_czyx(self, dense_data: torch.Tensor, dense_origins=0) -> JaggedTensor:
        return self.read_from_dense_xyzc(dense_data.permute(0, 4, 3, 2, 1), dense_origins)

    def ijk_to_index(self, ijk, cumulative: bool = False) -> JaggedTensor:
        """Index of each queried coordinate in its grid (-1 where absent); one leaf-hash probe each."""
        if isinstance(ijk, torch.Tensor):
            ijk = JaggedTensor(ijk)
        if ijk.num_outer_lists() != self.grid_count:
            raise ValueError("ijk must have one list per grid")
        idx = self._impl.ijk_to_index(ijk.jdata, ijk.joffsets, bool(cumulative))
        return ijk.jagged_like(idx)

    def inject_from(self, src_grid: "GridBatch", src: JaggedTensor, dst: JaggedTensor | None = None,
                    default_value: float | int | bool = 0) -> JaggedTensor:
        """Copy per-voxel data of `src_grid` onto the voxels of this grid that `src_grid` also holds
        (index space, grid by grid; reference: fvdb/grid_batch.py:748-789).  `dst` (optional) is
        modified in place; without it the result starts filled with `default_value`.  One
        leaf-hash probe per voxel of this grid (ijk_to_index), then one gather."""
        if not isinstance(src_grid, GridBatch):
            raise TypeError("src_grid must be a GridBatch")
        if src_grid.grid_count != self.grid_count:
            raise ValueError("src_grid must have the same number of grids as this grid")
        if isinstance(src, torch.Tensor):
            src = src_grid.jagged_like(src)
        if src.jdata.shape[0] != src_grid.total_voxels:
            raise ValueError("src must have one row per voxel of src_grid")
        if dst is None:
            dst = self.jagged_like(torch.full([self.total_voxels] + list(src.eshape), default_value,
                                              dtype=src.dtype, device=src.device))
        elif isinstance(dst, torch.Tensor):
            dst = self.jagged_like(dst)
        if list(dst.eshape) != list(src.eshape):
            raise ValueError(f"src and dst must have the same element shape, but got src: {src.eshape}, "
                             f"dst: {dst.eshape}")
        idx = src_grid.ijk_to_index(self.ijk, cumulative=True).jdata.long()
        hit = torch.nonzero(idx >= 0).squeeze(1)
        dst.jdata[hit] = src.jdata[idx[hit]].to(dst.dtype)
        return dst

    def to(self, device) -> "GridBatch":
        device = _device(device)
        if device == self.device:
            return self
        raise ValueError("fvdb_gb300 grids are built on one CUDA device; rebuild with from_ijk on the target device")

    def cuda(self) -> "GridBatch":
        return self

    def __repr__(self) -> str:
        return f"GridBatch(grid_count={self.grid_count}, total_voxels={self.total_voxels}, device={self.device})"
