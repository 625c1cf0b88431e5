"""JaggedTensor: a batch of variable-length lists of rows stored as one flat tensor.

Layout as in the reference (src/fvdb/JaggedTensor.h:16-22): ``jdata`` [N, ...] holds the
rows of all lists back to back, ``joffsets`` int64 [B+1] delimits list b as
``jdata[joffsets[b]:joffsets[b+1]]`` and ``jidx`` int32 [N] names the list of each row.
This is the subset the sparse-convolution path needs (single list dimension).
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

    def num_outer_lists(self) -> int:
        return int(self._joffsets.numel() - 1)

    def element_count(self) -> int:
        return int(self._jdata.shape[0])

    def __len__(self) -> int:
        return self.num_outer_lists()

    def __getitem__(self, i: int) -> "JaggedTensor":
        if not isinstance(i, int):
            raise TypeError("only integer indexing is supported")
        n = self.num_outer_lists()
        if i < 0:
            i += n
        if not 0 <= i < n:
            raise IndexError("list index out of range")
        off = self._joffsets.cpu()
        s, e = int(off[i]), int(off[i + 1])
        return JaggedTensor(self._jdata[s:e])

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

    def __repr__(self) -> str:
        return f"JaggedTensor(lists={self.num_outer_lists()}, jdata={tuple(self._jdata.shape)}, dtype={self.dtype})"
