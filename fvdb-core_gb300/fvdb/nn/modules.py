"""fvdb.nn.SparseConv3d on the GB300 kernels (reference: fvdb/nn/modules.py:156-404).

The module keeps the reference's constructor, weight layout ((Do, Di, K0, K1, K2) with
(K2, K1, K0, Di, Do) memory), initialisation, kernel-map caching through VDBTensor, 1x1x1
shortcut and bias.  ``backend`` and ``allow_tf32`` stay as accepted class attributes; every
value runs the same implementation.  ``precision`` selects the arithmetic of the
contraction for floating-point features: "native" (the features' dtype), "bf16" or "fp8"
(E4M3 with per-channel scales); accumulation is always FP32 or wider.
"""

from __future__ import annotations

import math
from typing import Optional, Sequence, Union

import torch
import torch.nn as nn

from ..grid_batch import GridBatch
from ..sparse_conv_pack_info import ConvPackBackend, SparseConvPackInfo
from .vdbtensor import VDBTensor


class SparseConv3d(nn.Module):
    backend: str = "default"
    allow_tf32: bool = True
    precision: str = "native"

    def __init__(
        self,
        in_channels: int,
        out_channels: int,
        kernel_size: Union[int, Sequence] = 3,
        stride: Union[int, Sequence] = 1,
        bias: bool = True,
        transposed: bool = False,
    ) -> None:
        super().__init__()
        self.in_channels = in_channels
        self.out_channels = out_channels
        if isinstance(kernel_size, int):
            kernel_size = (kernel_size,) * 3
        if isinstance(stride, int):
            stride = (stride,) * 3
        kernel_size = tuple(kernel_size)
        stride = tuple(stride)
        assert len(kernel_size) == 3 and len(stride) == 3
        self.kernel_size = kernel_size
        self.stride = stride
        self.transposed = transposed
        if self.transposed:
            out_channels, in_channels = in_channels, out_channels
        self.kernel_volume = math.prod(self.kernel_size)
        if self.kernel_volume > 1:
            weight_shape = [out_channels, in_channels] + list(self.kernel_size)
            weight = torch.zeros(*weight_shape[::-1]).permute(4, 3, 2, 1, 0)
            self.weight = nn.Parameter(weight)
        else:
            self.weight = nn.Parameter(torch.zeros(out_channels, in_channels))
        if bias:
            self.bias = nn.Parameter(torch.empty(self.out_channels))
        else:
            self.register_parameter("bias", None)
        self.reset_parameters()

    def extra_repr(self) -> str:
        s = "{in_channels}, {out_channels}, kernel_size={kernel_size}"
        if self.stride != (1, 1, 1):
            s += ", stride={stride}"
        if self.bias is None:
            s += ", bias=False"
        if self.transposed:
            s += ", transposed=True"
        return s.format(**self.__dict__)

    def reset_parameters(self) -> None:
        std = 1 / math.sqrt((self.out_channels if self.transposed else self.in_channels) * self.kernel_volume)
        self.weight.data.uniform_(-std, std)
        if self.bias is not None:
            self.bias.data.uniform_(-std, std)

    def _dispatch_conv(self, in_feature, in_grid: GridBatch, in_kmap, out_grid, relu: bool = False, scale=None,
                       shift=None):
        can_cache = self.stride == (1, 1, 1) and (out_grid is None or out_grid.is_same(in_grid))
        if in_kmap is not None and in_kmap.kernel_size == self.kernel_size and can_cache:
            kmap, out_grid = in_kmap, in_grid
        elif self.transposed:
            if out_grid is None:
                raise ValueError("a transposed SparseConv3d needs out_grid")
            kmap, _ = out_grid.sparse_conv_kernel_map(self.kernel_size, self.stride, in_grid)
        else:
            kmap, out_grid = in_grid.sparse_conv_kernel_map(self.kernel_size, self.stride, out_grid)
        out_kmap = kmap if can_cache else None
        if self.training:
            kmap.build_implicit_gemm(sorted=False, training=False)
        prec = None if self.precision == "native" else self.precision
        # the bias is added in the contraction's epilogue (the reference adds it in a second pass)
        bias = self.bias if scale is None else shift
        out_feature = kmap._conv_with_bias(in_feature, self.weight, bias, self.transposed, prec, relu, scale)
        return out_grid, out_feature, out_kmap

    def _folded(self, out_affine):
        """(scale, shift) of conv * scale + shift with a following per-channel affine map
        (s, t) folded in: scale = s, shift = bias * s + t (FP32)."""
        s, t = (v.detach().float() for v in out_affine)
        return s, (t if self.bias is None else self.bias.detach().float() * s + t)

    def forward(self, input: VDBTensor, out_grid: Optional[GridBatch] = None, *, relu: bool = False,
                out_affine=None) -> VDBTensor:
        """`relu` (extension): return max(conv(input) + bias, 0), the clamp fused into the
        contraction's epilogue (nn.Sequential passes it for a SparseConv3d followed by a ReLU).
        `out_affine` (extension, inference only): a pair (s, t) of [C_out] tensors; the output is
        (conv(input) + bias) * s + t, applied in FP32 in the epilogue with the features' dtype
        kept (nn.Sequential passes it to fold an eval-mode BatchNorm into the convolution)."""
        in_feature, in_grid, in_kmap = input.data, input.grid, input.kmap
        scale = shift = None
        if out_affine is not None:
            if torch.is_grad_enabled() and (self.weight.requires_grad or in_feature.jdata.requires_grad):
                raise RuntimeError("out_affine (a folded batch norm) is inference-only")
            scale, shift = self._folded(out_affine)
        if self.kernel_size == (1, 1, 1) and self.stride == (1, 1, 1):
            y = in_feature.jdata.matmul(self.weight.transpose(0, 1))
            if scale is not None:
                y = (y.float() * scale + shift).to(y.dtype)
            elif self.bias is not None:
                y = y + self.bias
            out_feature = in_feature.jagged_like(torch.relu(y) if relu else y)
            out_grid, out_kmap = in_grid, in_kmap
        else:
            out_grid, out_feature, out_kmap = self._dispatch_conv(in_feature, in_grid, in_kmap, out_grid, relu, scale,
                                                                  shift)
        if out_grid is None:
            raise ValueError("Failed to compute output grid. This is a bug in the implementation.")
        return VDBTensor(out_grid, out_feature, out_kmap)


class _OnFeatures:
    """Runs the torch layer it is mixed into on a VDBTensor's [N, C] features; grid and kernel
    map pass through (reference: fvdb/nn/modules.py:529-620)."""

    def forward(self, input: VDBTensor) -> VDBTensor:
        if not isinstance(input, VDBTensor):
            raise TypeError("Input should have type VDBTensor")
        return VDBTensor(input.grid, input.data.jagged_like(super().forward(input.data.jdata)), input.kmap)


class ReLU(_OnFeatures, nn.ReLU):
    """max(x, 0) on the features."""


class LeakyReLU(_OnFeatures, nn.LeakyReLU):
    """max(0, x) + negative_slope * min(0, x) on the features."""


class ELU(_OnFeatures, nn.ELU):
    """x for x > 0, alpha * (exp(x) - 1) otherwise, on the features."""


class CELU(_OnFeatures, nn.CELU):
    """max(0, x) + min(0, alpha * (exp(x / alpha) - 1)) on the features."""


class GELU(_OnFeatures, nn.GELU):
    """x * Phi(x) on the features."""


class SELU(_OnFeatures, nn.SELU):
    """scale * (max(0, x) + min(0, alpha * (exp(x) - 1))) on the features."""


class SiLU(_OnFeatures, nn.SiLU):
    """x * sigmoid(x) on the features."""


class Tanh(_OnFeatures, nn.Tanh):
    """tanh(x) on the features."""


class Sigmoid(_OnFeatures, nn.Sigmoid):
    """1 / (1 + exp(-x)) on the features."""


class Linear(_OnFeatures, nn.Linear):
    """x A^T + b on each voxel's feature row."""


class Dropout(_OnFeatures, nn.Dropout):
    """Bernoulli dropout of the features in training mode."""


class BatchNorm(nn.BatchNorm1d):
    """Batch normalisation of a VDBTensor's features over all voxels of the batch (reference:
    fvdb/nn/modules.py:435-444): torch's BatchNorm1d on the [N, C] feature matrix."""

    def forward(self, input: VDBTensor) -> VDBTensor:
        if input.data.jdata.size(1) != self.num_features:
            raise ValueError("Input feature should have the same number of channels as BatchNorm")
        return VDBTensor(input.grid, input.grid.jagged_like(super().forward(input.data.jdata)), input.kmap)

    def folded_affine(self):
        """(s, t), FP32 [C]: the eval-mode map x -> x * s + t this layer applies with its
        running statistics, or None when it normalises with batch statistics."""
        if self.training or self.running_mean is None or self.running_var is None:
            return None
        s = torch.rsqrt(self.running_var.detach().float() + self.eps)
        if self.weight is not None:
            s = s * self.weight.detach().float()
        t = -self.running_mean.detach().float() * s
        if self.bias is not None:
            t = t + self.bias.detach().float()
        return s, t


class SyncBatchNorm(nn.SyncBatchNorm):
    """Batch normalisation of a VDBTensor's features with statistics over all ranks of the
    process group (reference: fvdb/nn/modules.py:447-526): torch's SyncBatchNorm on the [N, C]
    feature matrix."""

    def forward(self, input: VDBTensor) -> VDBTensor:
        if input.data.jdata.size(1) != self.num_features:
            raise ValueError("Input feature should have the same number of channels as BatchNorm")
        return VDBTensor(input.grid, input.grid.jagged_like(super().forward(input.data.jdata)), input.kmap)

    @classmethod
    def convert_sync_batchnorm(cls, module: nn.Module, process_group=None) -> nn.Module:
        """A copy of `module` with every fvdb.nn.BatchNorm replaced by a SyncBatchNorm that holds
        the same parameters, buffers and mode."""
        out = module
        if isinstance(module, BatchNorm):
            out = cls(module.num_features, module.eps, module.momentum, module.affine, module.track_running_stats,
                      process_group)
            if module.affine:
                with torch.no_grad():
                    out.weight = module.weight
                    out.bias = module.bias
            out.running_mean = module.running_mean
            out.running_var = module.running_var
            out.num_batches_tracked = module.num_batches_tracked
            out.train(module.training)
            if hasattr(module, "qconfig"):
                out.qconfig = module.qconfig
        for name, child in module.named_children():
            out.add_module(name, cls.convert_sync_batchnorm(child, process_group))
        return out


class GroupNorm(nn.GroupNorm):
    """Group normalisation of a VDBTensor's features, per grid of the batch (reference:
    fvdb/nn/modules.py:408-432, which loops over the grids): each (grid, group) is normalised
    over its voxels and the group's channels, with the biased variance and eps of
    torch.nn.GroupNorm.  One vectorised pass over all grids: the per-(grid, group) sums are
    segment sums keyed by the voxels' grid index, the variance is taken about the mean (two
    passes, FP32 or wider), and empty grids contribute nothing.  The segment sums accumulate with
    atomics on CUDA, so results agree with the per-grid loop to rounding but are not bitwise
    reproducible from run to run."""

    def forward(self, input: VDBTensor) -> VDBTensor:
        x = input.data.jdata
        n, c = x.shape[0], x.shape[1] if x.dim() == 2 else -1
        if x.dim() != 2 or c != self.num_channels:
            raise ValueError("Input feature should have the same number of channels as GroupNorm")
        g, b = self.num_groups, input.grid.grid_count
        acc = torch.float64 if x.dtype == torch.float64 else torch.float32
        jidx = input.data.jidx.long()
        xg = x.to(acc).reshape(n, g, c // g)
        counts = torch.bincount(jidx, minlength=b).to(acc) * (c // g)
        denom = counts.clamp(min=1)[:, None]
        mean = torch.zeros(b, g, dtype=acc, device=x.device).index_add_(0, jidx, xg.sum(2)) / denom
        d = xg - mean[jidx][:, :, None]
        var = torch.zeros(b, g, dtype=acc, device=x.device).index_add_(0, jidx, (d * d).sum(2)) / denom
        y = (d * torch.rsqrt(var + self.eps)[jidx][:, :, None]).reshape(n, c)
        if self.affine:
            y = y * self.weight.to(acc) + self.bias.to(acc)
        return VDBTensor(input.grid, input.grid.jagged_like(y.to(x.dtype)), input.kmap)


class Sequential(nn.Sequential):
    """nn.Sequential over VDBTensor-to-VDBTensor layers.  A SparseConv3d directly followed by a
    ReLU runs as one convolution with the ReLU fused into its epilogue: the same values (rounding
    to the output type keeps signs) and gradients, one pass over the output instead of two.
    Without autograd (inference), a SparseConv3d followed by an eval-mode BatchNorm (and
    optionally a ReLU) runs as one convolution with the batch norm's affine map folded into the
    epilogue's per-channel scale and shift: the values of the three layers within the rounding
    of one output type, one pass over the output instead of three."""

    def forward(self, input):
        mods = list(self)
        i = 0
        while i < len(mods):
            m = mods[i]
            nxt = mods[i + 1] if i + 1 < len(mods) else None
            # folded only where the layers' own output dtype is the features' (a bias of a wider
            # dtype would promote the unfused result)
            if (isinstance(m, SparseConv3d) and type(nxt) is BatchNorm and not torch.is_grad_enabled()
                    and m.precision == "native" and isinstance(input, VDBTensor)
                    and (m.bias is None or m.bias.dtype == input.data.jdata.dtype)):
                aff = nxt.folded_affine()
                if aff is not None and aff[0].device == m.weight.device:
                    after = mods[i + 2] if i + 2 < len(mods) else None
                    relu = type(after) is ReLU
                    input = m(input, relu=relu, out_affine=aff)
                    i += 3 if relu else 2
                    continue
            if isinstance(m, SparseConv3d) and type(nxt) is ReLU and not nxt.inplace:
                input = m(input, relu=True)
                i += 2
                continue
            input = m(input)
            i += 1
        return input


class RecomputeSequential(nn.Sequential):
    """Sequential stack whose intermediate activations are not kept for backward: the forward
    runs under torch.utils.checkpoint (non-reentrant) and is re-run during backward.  Kernel
    maps are cached in the VDBTensors, so the re-run repeats only the contractions; only the
    stack's input features stay alive between forward and backward."""

    def forward(self, input: VDBTensor) -> VDBTensor:
        from torch.utils.checkpoint import checkpoint

        box: dict = {}

        def run(x: torch.Tensor) -> torch.Tensor:
            kmap = box.get("in_kmap", input.kmap)
            out = nn.Sequential.forward(self, VDBTensor(input.grid, input.grid.jagged_like(x), kmap))
            box.setdefault("out", out)
            if "in_kmap" not in box and out.kmap is not None and out.grid.is_same(input.grid):
                box["in_kmap"] = out.kmap  # reused by the re-run in backward
            return out.data.jdata

        y = checkpoint(run, input.data.jdata, use_reentrant=False)
        out = box["out"]
        return VDBTensor(out.grid, out.grid.jagged_like(y), out.kmap)


GridOrVDBTensor = Union[GridBatch, VDBTensor]


class MaxPool(nn.Module):
    """3-D max pooling of a VDBTensor onto a coarser grid (reference: fvdb/nn/modules.py:33-72).
    Coarse voxels whose window holds no active voxel get 0 (the pooled -inf values are zeroed,
    as the reference does)."""

    def __init__(self, kernel_size, stride=None):
        super().__init__()
        self.kernel_size = kernel_size
        self.stride = stride or self.kernel_size

    def forward(self, input: VDBTensor, ref_coarse_data: Optional[GridOrVDBTensor] = None) -> VDBTensor:
        coarse_grid, coarse_kmap = _ref_grid(ref_coarse_data)
        feat, grid = input.grid.max_pool(self.kernel_size, input.data, stride=self.stride, coarse_grid=coarse_grid)
        feat.jdata[torch.isinf(feat.jdata)] = 0.0
        return VDBTensor(grid, feat, kmap=coarse_kmap)

    def extra_repr(self) -> str:
        return "kernel_size={kernel_size}, stride={stride}".format(kernel_size=self.kernel_size, stride=self.stride)


class AvgPool(nn.Module):
    """3-D average pooling of a VDBTensor onto a coarser grid (reference: fvdb/nn/modules.py:75-106)."""

    def __init__(self, kernel_size, stride=None):
        super().__init__()
        self.kernel_size = kernel_size
        self.stride = stride or self.kernel_size

    def forward(self, input: VDBTensor, ref_coarse_data: Optional[GridOrVDBTensor] = None) -> VDBTensor:
        coarse_grid, coarse_kmap = _ref_grid(ref_coarse_data)
        feat, grid = input.grid.avg_pool(self.kernel_size, input.data, stride=self.stride, coarse_grid=coarse_grid)
        return VDBTensor(grid, feat, kmap=coarse_kmap)

    def extra_repr(self) -> str:
        return "kernel_size={kernel_size}, stride={stride}".format(kernel_size=self.kernel_size, stride=self.stride)


class FillFromGrid(nn.Module):
    """Moves a VDBTensor's features onto another grid: voxels the input's grid also holds take
    its features, the rest `default_value` (reference: fvdb/nn/modules.py:132-154, through
    GridBatch.inject_from).  Without a target the input is returned."""

    def __init__(self, default_value: float = 0.0) -> None:
        super().__init__()
        self.default_value = default_value

    def forward(self, input: VDBTensor, other_data: Optional[GridOrVDBTensor] = None) -> VDBTensor:
        if isinstance(other_data, VDBTensor):
            other_grid, other_kmap = other_data.grid, other_data.kmap
        elif isinstance(other_data, GridBatch):
            other_grid, other_kmap = other_data, None
        else:
            return input
        feats = other_grid.inject_from(input.grid, input.data, default_value=self.default_value)
        return VDBTensor(other_grid, feats, kmap=other_kmap)

    def extra_repr(self) -> str:
        return f"default_value={self.default_value}"


class UpsamplingNearest(nn.Module):
    """Nearest upsampling of a VDBTensor onto a finer grid (reference: fvdb/nn/modules.py:109-130)."""

    def __init__(self, scale_factor):
        super().__init__()
        self.scale_factor = scale_factor

    def forward(self, input: VDBTensor, mask=None, ref_fine_data: Optional[GridOrVDBTensor] = None) -> VDBTensor:
        fine_grid, fine_kmap = _ref_grid(ref_fine_data)
        feat, grid = input.grid.subdivide(self.scale_factor, input.data, mask, fine_grid=fine_grid)
        return VDBTensor(grid, feat, kmap=fine_kmap)

    def extra_repr(self) -> str:
        return "scale_factor={scale_factor}".format(scale_factor=self.scale_factor)


def _ref_grid(ref):
    if isinstance(ref, VDBTensor):
        return ref.grid, ref.kmap
    if isinstance(ref, GridBatch):
        return ref, None
    return None, None
