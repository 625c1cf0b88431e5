"""JaggedTensor: a batch of variable-length lists of rows stored as one flat tensor.

Layout as in the reference (src/fvdb/JaggedTensor.h:16-22): ``jdata`` [N, ...] holds the
rows of all lists back to back, ``joffsets`` int64 [B+1] delimits list b as
``jdata[joffsets[b]:joffsets[b+1]]`` and ``jidx`` int32 [N] names the list of each row.
One list dimension (a batch of lists of rows), with the reference's constructors, elementwise
arithmetic on the rows, per-list reductions (jsum / jmin / jmax), row masks, list reshapes and
concatenation (jcat).
"""

from __future__ import annotations

from typing import Sequence

import torch


class JaggedTensor:
    def __init__(self, data: "torch.Tensor | Sequence[torch.Tensor] | None" = None, *, _jdata=None, _joffsets=None):
        if _jdata is not None:
            self._jdata = _jdata
            self._joffsets = _joffsets
        elif isinstance(data, torch.Tensor):
            self._jdata = data
            self._joffsets = torch.tensor([0, data.shape[0]], dtype=torch.int64, device=data.device)
        elif isinstance(data, (list, tuple)):
            if len(data) == 0:
                raise ValueError("JaggedTensor needs at least one list")
            for t in data:
                if not isinstance(t, torch.Tensor):
                    raise TypeError("JaggedTensor lists must be torch.Tensors")
            counts = [int(t.shape[0]) for t in data]
            self._jdata = torch.cat(list(data), 0)
            off = [0]
            for c in counts:
                off.append(off[-1] + c)
            self._joffsets = torch.tensor(off, dtype=torch.int64, device=self._jdata.device)
        else:
            raise TypeError("JaggedTensor expects a tensor or a list of tensors")
        self._jidx = None

    # -- construction helpers ----------------------------------------------------------------
    @classmethod
    def from_data_and_offsets(cls, data: torch.Tensor, offsets: torch.Tensor) -> "JaggedTensor":
        offsets = offsets.to(device=data.device, dtype=torch.int64)
        if offsets.dim() != 1 or offsets.numel() < 2:
            raise ValueError("offsets must be a 1-D tensor with at least two entries")
        return cls(_jdata=data, _joffsets=offsets)

    from_data_offsets_and_list_ids = from_data_and_offsets

    @classmethod
    def from_data_and_indices(cls, data: torch.Tensor, indices: torch.Tensor, num_tensors: int) -> "JaggedTensor":
        """Rows grouped by list: `indices` [N] names the list of each row, in non-decreasing
        order (the jidx layout)."""
        idx = indices.to(device=data.device, dtype=torch.int64).reshape(-1)
        if idx.numel() != data.shape[0]:
            raise ValueError("indices must have one entry per row of data")
        if idx.numel() and (bool((idx[1:] < idx[:-1]).any()) or int(idx.min()) < 0 or int(idx.max()) >= num_tensors):
            raise ValueError("indices must be sorted and lie in [0, num_tensors)")
        counts = torch.bincount(idx, minlength=num_tensors)
        offsets = torch.zeros(num_tensors + 1, dtype=torch.int64, device=data.device)
        offsets[1:] = torch.cumsum(counts, 0)
        return cls(_jdata=data, _joffsets=offsets)

    from_data_indices_and_list_ids = from_data_and_indices

    def jagged_like(self, data: torch.Tensor) -> "JaggedTensor":
        if data.shape[0] != self._jdata.shape[0]:
            raise ValueError("data must have the same number of rows as this JaggedTensor")
        return JaggedTensor(_jdata=data, _joffsets=self._joffsets)

    # -- properties ----------------------------------------------------------------------------
    @property
    def jdata(self) -> torch.Tensor:
        return self._jdata

    @jdata.setter
    def jdata(self, value: torch.Tensor) -> None:
        if value.shape[0] != self._jdata.shape[0]:
            raise ValueError("jdata must keep the same number of rows")
        self._jdata = value

    @property
    def joffsets(self) -> torch.Tensor:
        return self._joffsets

    @property
    def jidx(self) -> torch.Tensor:
        if self._jidx is None:
            counts = (self._joffsets[1:] - self._joffsets[:-1]).to(torch.int64)
            self._jidx = torch.repeat_interleave(
                torch.arange(counts.numel(), device=self._jdata.device, dtype=torch.int32), counts
            )
        return self._jidx

    @property
    def lshape(self) -> list[int]:
        return (self._joffsets[1:] - self._joffsets[:-1]).tolist()

    @property
    def device(self) -> torch.device:
        return self._jdata.device

    @property
    def dtype(self) -> torch.dtype:
        return self._jdata.dtype

    @property
    def eshape(self) -> list[int]:
        return list(self._jdata.shape[1:])

    @property
    def requires_grad(self) -> bool:
        return self._jdata.requires_grad

    @property
    def num_tensors(self) -> int:
        return self.num_outer_lists()

    @property
    def ldim(self) -> int:
        return 1

    @property
    def edim(self) -> int:
        return self._jdata.dim() - 1

    @property
    def rshape(self) -> tuple:
        return tuple(self._jdata.shape)

    @property
    def is_cuda(self) -> bool:
        return self._jdata.is_cuda

    @property
    def is_cpu(self) -> bool:
        return self._jdata.is_cpu

    def num_outer_lists(self) -> int:
        return int(self._joffsets.numel() - 1)

    def element_count(self) -> int:
        return int(self._jdata.shape[0])

    def __len__(self) -> int:
        return self.num_outer_lists()

    def __getitem__(self, i) -> "JaggedTensor":
        """List `i` (an int) or the lists of a step-1 slice, as a JaggedTensor."""
        n = self.num_outer_lists()
        off = self._joffsets.cpu()
        if isinstance(i, slice):
            a, b, step = i.indices(n)
            if step != 1:
                raise ValueError("only step-1 slices of lists are supported")
            b = max(a, b)
            return JaggedTensor(_jdata=self._jdata[int(off[a]):int(off[b])],
                                _joffsets=(self._joffsets[a:b + 1] - self._joffsets[a]).clone())
        if not isinstance(i, int):
            raise TypeError("only integer and slice indexing is supported")
        if i < 0:
            i += n
        if not 0 <= i < n:
            raise IndexError("list index out of range")
        s, e = int(off[i]), int(off[i + 1])
        return JaggedTensor(self._jdata[s:e])

    def __iter__(self):
        for i in range(self.num_outer_lists()):
            yield self[i]

    def unbind(self) -> list[torch.Tensor]:
        off = self._joffsets.cpu().tolist()
        return [self._jdata[off[b] : off[b + 1]] for b in range(len(off) - 1)]

    # -- device / dtype ------------------------------------------------------------------------
    def to(self, *args, **kwargs) -> "JaggedTensor":
        d = self._jdata.to(*args, **kwargs)
        return JaggedTensor(_jdata=d, _joffsets=self._joffsets.to(d.device))

    def cuda(self) -> "JaggedTensor":
        return self.to("cuda")

    def cpu(self) -> "JaggedTensor":
        return self.to("cpu")

    def detach(self) -> "JaggedTensor":
        return self.jagged_like(self._jdata.detach())

    def clone(self) -> "JaggedTensor":
        return self.jagged_like(self._jdata.clone())

    def requires_grad_(self, requires_grad: bool = True) -> "JaggedTensor":
        self._jdata.requires_grad_(requires_grad)
        return self

    def type(self, dtype: torch.dtype) -> "JaggedTensor":
        return self.jagged_like(self._jdata.type(dtype))

    def type_as(self, other) -> "JaggedTensor":
        return self.type(other.dtype)

    def float(self) -> "JaggedTensor":
        return self.type(torch.float32)

    def double(self) -> "JaggedTensor":
        return self.type(torch.float64)

    def int(self) -> "JaggedTensor":
        return self.type(torch.int32)

    def long(self) -> "JaggedTensor":
        return self.type(torch.int64)

    # -- elementwise arithmetic on the rows ----------------------------------------------------
    # A JaggedTensor operand contributes its rows (same row count); tensors and scalars broadcast
    # against jdata.  The result keeps this tensor's lists.
    def _rows_of(self, other):
        if isinstance(other, JaggedTensor):
            if other._jdata.shape[0] != self._jdata.shape[0]:
                raise ValueError("JaggedTensor operands must have the same number of rows")
            return other._jdata
        return other

    def _op(self, other, fn) -> "JaggedTensor":
        return self.jagged_like(fn(self._jdata, self._rows_of(other)))

    def _iop(self, other, fn) -> "JaggedTensor":
        fn(self._jdata, self._rows_of(other))
        return self

    def __add__(self, o):
        return self._op(o, torch.add)

    def __radd__(self, o):
        return self._op(o, lambda a, b: b + a)

    def __sub__(self, o):
        return self._op(o, torch.sub)

    def __rsub__(self, o):
        return self._op(o, lambda a, b: b - a)

    def __mul__(self, o):
        return self._op(o, torch.mul)

    def __rmul__(self, o):
        return self._op(o, lambda a, b: b * a)

    def __truediv__(self, o):
        return self._op(o, torch.true_divide)

    def __rtruediv__(self, o):
        return self._op(o, lambda a, b: b / a)

    def __floordiv__(self, o):
        return self._op(o, torch.floor_divide)

    def __mod__(self, o):
        return self._op(o, torch.remainder)

    def __pow__(self, o):
        return self._op(o, torch.pow)

    def __neg__(self):
        return self.jagged_like(-self._jdata)

    def __eq__(self, o):
        return self._op(o, torch.eq)

    def __ne__(self, o):
        return self._op(o, torch.ne)

    def __lt__(self, o):
        return self._op(o, torch.lt)

    def __le__(self, o):
        return self._op(o, torch.le)

    def __gt__(self, o):
        return self._op(o, torch.gt)

    def __ge__(self, o):
        return self._op(o, torch.ge)

    __hash__ = object.__hash__

    def __iadd__(self, o):
        return self._iop(o, lambda a, b: a.add_(b))

    def __isub__(self, o):
        return self._iop(o, lambda a, b: a.sub_(b))

    def __imul__(self, o):
        return self._iop(o, lambda a, b: a.mul_(b))

    def __itruediv__(self, o):
        return self._iop(o, lambda a, b: a.div_(b))

    def __ifloordiv__(self, o):
        return self._iop(o, lambda a, b: a.floor_divide_(b))

    def __imod__(self, o):
        return self._iop(o, lambda a, b: a.remainder_(b))

    def __ipow__(self, o):
        return self._iop(o, lambda a, b: a.pow_(b))

    def abs(self):
        return self.jagged_like(self._jdata.abs())

    def abs_(self):
        self._jdata.abs_()
        return self

    def ceil(self):
        return self.jagged_like(self._jdata.ceil())

    def ceil_(self):
        self._jdata.ceil_()
        return self

    def floor(self):
        return self.jagged_like(self._jdata.floor())

    def floor_(self):
        self._jdata.floor_()
        return self

    def round(self, decimals: int = 0):
        return self.jagged_like(self._jdata.round(decimals=decimals))

    def round_(self, decimals: int = 0):
        self._jdata.round_(decimals=decimals)
        return self

    def sqrt(self):
        return self.jagged_like(self._jdata.sqrt())

    def sqrt_(self):
        self._jdata.sqrt_()
        return self

    # -- per-list operations -------------------------------------------------------------------
    def rmask(self, mask: torch.Tensor) -> "JaggedTensor":
        """The rows where `mask` [N] (bool) is true, each list keeping its own."""
        if mask.dim() != 1 or mask.shape[0] != self._jdata.shape[0]:
            raise ValueError("mask must have one entry per row")
        m = mask.to(device=self._jdata.device, dtype=torch.bool)
        counts = torch.zeros(self.num_outer_lists(), dtype=torch.int64, device=self._jdata.device)
        counts.index_add_(0, self.jidx.long(), m.long())
        offsets = torch.zeros_like(self._joffsets)
        offsets[1:] = torch.cumsum(counts, 0)
        return JaggedTensor(_jdata=self._jdata[m], _joffsets=offsets)

    def _reduce_dim(self, dim: int) -> int:
        e = self.edim
        if not -e <= dim <= e:
            raise IndexError(f"dim {dim} out of range for a JaggedTensor with {e} element dimension(s)")
        return dim + e + 1 if dim < 0 else dim

    def _per_list(self, out: torch.Tensor) -> "JaggedTensor":
        n = out.shape[0]
        return JaggedTensor(_jdata=out, _joffsets=torch.arange(n + 1, dtype=torch.int64, device=out.device))

    def jsum(self, dim: int = 0, keepdim: bool = False) -> "JaggedTensor":
        """dim 0: the sum of each list's rows (one row per list; empty lists give 0); an element
        dimension: jdata.sum(dim) with the lists kept."""
        d = self._reduce_dim(dim)
        if d > 0:
            return self.jagged_like(self._jdata.sum(dim=d, keepdim=keepdim))
        out = torch.zeros((self.num_outer_lists(),) + tuple(self._jdata.shape[1:]), dtype=self._jdata.dtype,
                          device=self._jdata.device)
        return self._per_list(out.index_add(0, self.jidx.long(), self._jdata))

    def _jextreme(self, dim: int, keepdim: bool, largest: bool):
        d = self._reduce_dim(dim)
        if d > 0:
            v, i = (self._jdata.max if largest else self._jdata.min)(dim=d, keepdim=keepdim)
            return [self.jagged_like(v), self.jagged_like(i)]
        B, x = self.num_outer_lists(), self._jdata
        idx = self.jidx.long().reshape((-1,) + (1,) * (x.dim() - 1)).expand_as(x)
        base = torch.zeros((B,) + tuple(x.shape[1:]), dtype=x.dtype, device=x.device)
        v = base.scatter_reduce(0, idx, x, reduce="amax" if largest else "amin", include_self=False)
        rows = torch.arange(x.shape[0], device=x.device).reshape((-1,) + (1,) * (x.dim() - 1)).expand_as(x)
        hit = x == v.detach()[self.jidx.long()]
        big = torch.full_like(rows, x.shape[0])
        first = torch.full((B,) + tuple(x.shape[1:]), x.shape[0], dtype=torch.int64, device=x.device)
        first = first.scatter_reduce(0, idx, torch.where(hit, rows, big), reduce="amin", include_self=True)
        first = torch.where(first == x.shape[0], torch.zeros_like(first), first)
        return [self._per_list(v), self._per_list(first)]

    def jmax(self, dim: int = 0, keepdim: bool = False):
        """[values, indices]: dim 0 gives each list's maximum row-wise (empty lists give 0) and
        the global row of its first occurrence; an element dimension is torch.max over jdata."""
        return self._jextreme(dim, keepdim, True)

    def jmin(self, dim: int = 0, keepdim: bool = False):
        """[values, indices] as jmax, for the minimum."""
        return self._jextreme(dim, keepdim, False)

    def jreshape(self, lshape) -> "JaggedTensor":
        """The same rows split into lists of the given sizes (they must add up to the rows)."""
        sizes = [int(v) for v in lshape]
        if sum(sizes) != self._jdata.shape[0] or any(v < 0 for v in sizes):
            raise ValueError("lshape must be non-negative sizes adding up to the number of rows")
        off = [0]
        for v in sizes:
            off.append(off[-1] + v)
        return JaggedTensor(_jdata=self._jdata, _joffsets=torch.tensor(off, dtype=torch.int64, device=self.device))

    def jreshape_as(self, other) -> "JaggedTensor":
        if isinstance(other, JaggedTensor):
            return self.jreshape(other.lshape)
        return self.jreshape([other.shape[0]])

    def jflatten(self, dim: int = 0) -> "JaggedTensor":
        """dim 0: all rows as one list."""
        if dim != 0:
            raise ValueError("a JaggedTensor with one list dimension flattens along dim 0 only")
        return JaggedTensor(self._jdata)

    def __repr__(self) -> str:
        return f"JaggedTensor(lists={self.num_outer_lists()}, jdata={tuple(self._jdata.shape)}, dtype={self.dtype})"


def jcat(things, dim=None):
    """Concatenation (reference: fvdb/__init__.py jcat).  JaggedTensors: dim None appends the
    lists; dim 0 concatenates list b of every operand into list b; an element dimension
    concatenates the rows' elements (same lists).  GridBatches (dim None): one batch holding
    every grid.  VDBTensors: dim None concatenates grids and features; an element dimension
    concatenates the features of tensors on the same grid (a UNet skip connection)."""
    if len(things) == 0:
        raise ValueError("Cannot concatenate empty list")
    from .grid_batch import GridBatch
    from .nn.vdbtensor import VDBTensor

    first = things[0]
    if isinstance(first, GridBatch):
        if dim is not None:
            raise ValueError("GridBatch concatenation does not support dim argument")
        return GridBatch.from_ijk(jcat([g.ijk for g in things]),
                                  torch.cat([g.voxel_sizes.reshape(-1, 3).cpu() for g in things]),
                                  torch.cat([g.origins.reshape(-1, 3).cpu() for g in things]), device=first.device)
    if isinstance(first, VDBTensor):
        if dim == 0:
            raise ValueError("VDBTensor concatenation does not support dim=0")
        if dim is None:
            grid = jcat([t.grid for t in things])
            return VDBTensor(grid, grid.jagged_like(jcat([t.data for t in things]).jdata))
        for t in things[1:]:
            if t.grid.total_voxels != first.grid.total_voxels or t.grid.grid_count != first.grid.grid_count:
                raise ValueError("VDBTensors concatenated along a feature dimension must share their grid")
        return VDBTensor(first.grid, jcat([t.data for t in things], dim), first.kmap)
    if not all(isinstance(t, JaggedTensor) for t in things):
        raise TypeError("jcat() can only cat GridBatch, JaggedTensor, or VDBTensor")
    if dim is None:
        data = torch.cat([t.jdata for t in things], 0)
        offs, base = [torch.zeros(1, dtype=torch.int64, device=data.device)], 0
        for t in things:
            offs.append((t.joffsets[1:] - t.joffsets[0]).to(data.device) + base)
            base += t.jdata.shape[0]
        return JaggedTensor(_jdata=data, _joffsets=torch.cat(offs))
    n = first.num_outer_lists()
    if any(t.num_outer_lists() != n for t in things):
        raise ValueError("jcat along a dimension needs the same number of lists in every operand")
    if dim == 0:
        parts = [t.unbind() for t in things]
        return JaggedTensor([torch.cat([p[b] for p in parts], 0) for b in range(n)])
    if any(t.lshape != first.lshape for t in things):
        raise ValueError("jcat along an element dimension needs the same list sizes in every operand")
    e = first.jdata.dim() - 1
    d = dim + e + 1 if dim < 0 else dim
    if not 1 <= d <= e:
        raise IndexError(f"dim {dim} out of range for element dimension(s) {e}")
    return first.jagged_like(torch.cat([t.jdata for t in things], d))
