"""SparseConvPackInfo: kernel maps of one (kernel_size, stride, source, target) and the
convolutions that use them.

Same surface as the reference's wrapper (fvdb/sparse_conv_pack_info.py:33-374, bound in
src/python/Bindings.cpp:381-458).  Every ``build_*`` call and every ``backend`` value is
accepted and routes to the one GB300 implementation: the kernel map (``out_in_map``,
reference-identical integers) feeds the fused gather-GEMM kernels.  The gather-scatter
tensors (``neighborhood_map``/``neighborhood_sizes``) and the sorted implicit-GEMM tensors
are produced when the matching ``build_*`` is called, for callers that read them.
"""

from __future__ import annotations

import enum

import torch

from . import _lib
from ._conv import sparse_conv
from .jagged_tensor import JaggedTensor


class ConvPackBackend(enum.Enum):
    """Backend selector kept for drop-in compatibility (src/python/Bindings.cpp:374-379)."""

    GATHER_SCATTER = 0
    IGEMM = 1
    CUTLASS = 2
    LGGS = 3


def _is_vec3i(v) -> bool:
    if isinstance(v, bool):
        return False
    if isinstance(v, int):
        return True
    if isinstance(v, torch.Tensor):
        return not v.is_floating_point() and v.numel() in (1, 3)
    if isinstance(v, (list, tuple)):
        return len(v) in (1, 3) and all(isinstance(x, int) and not isinstance(x, bool) for x in v)
    return False


def _vec(v) -> list[int]:
    if isinstance(v, torch.Tensor):
        v = v.tolist()
    if isinstance(v, int):
        return [v] * 3
    v = list(v)
    return v * 3 if len(v) == 1 else v


def _apply(data: torch.Tensor, weights: torch.Tensor, impl, transposed: bool, precision: str | None,
           bias: torch.Tensor | None = None, relu: bool = False, scale: torch.Tensor | None = None) -> torch.Tensor:
    """One convolution in the requested arithmetic.  The result has the dtype that the
    reference's `conv(x) + bias` has (torch type promotion of the contraction's output and the
    bias): the bias is fused into the contraction's epilogue when that dtype is the output's
    own, and added afterwards (promoting) otherwise.  `relu` applies max(., 0) last, fused into
    the epilogue with the bias.  `scale` (inference only) multiplies the contraction before the
    bias: the bias is then an FP32 shift and the output keeps the features' dtype."""
    if scale is not None and precision == "fp8":
        # the FP8 epilogue's scale dequantises: a folded batch norm is applied after it
        y = _apply(data, weights, impl, transposed, precision)
        y = y * scale.to(y.dtype) + (bias.to(y.dtype) if bias is not None else 0)
        return torch.relu(y) if relu else y
    if precision in (None, "native"):
        x, w = data, weights
    elif precision == "bf16":
        x, w = data.to(torch.bfloat16), weights.to(torch.bfloat16)
    elif precision == "fp8":
        if torch.is_grad_enabled() and (data.requires_grad or weights.requires_grad or
                                        (bias is not None and bias.requires_grad)):
            raise RuntimeError("the FP8 convolution is forward-only; use precision='bf16' for training")
        fuse = bias is None
        y, _, _ = _lib.load().conv_forward_fp8(data, weights, impl, transposed, relu and fuse)
        if bias is not None:
            y = y + bias
            if relu:
                y = torch.relu(y)
        return y
    else:
        raise ValueError(f"precision must be one of None, 'native', 'bf16', 'fp8' (got {precision!r})")
    if bias is not None and scale is None and torch.result_type(x, bias) != x.dtype:
        y = sparse_conv(x, w, impl, transposed, None) + bias
        return torch.relu(y) if relu else y
    # with a folded batch norm (scale) the output keeps the features' dtype, as the batch norm's
    # output does; scale and shift are applied in FP32 in the epilogue
    return sparse_conv(x, w, impl, transposed, bias, relu, scale)


class SparseConvPackInfo:
    def __init__(self, kernel_size=None, stride=None, source_grid=None, target_grid=None, impl=None):
        if impl is not None:
            if not (kernel_size is None and stride is None and source_grid is None and target_grid is None):
                raise ValueError("kernel_size, stride, source_grid, and target_grid must be None when impl is provided")
            self._impl = impl
            return
        if kernel_size is None or stride is None or source_grid is None:
            raise ValueError("kernel_size, stride, and source_grid must be provided when impl is None")
        from .grid_batch import GridBatch

        if not isinstance(source_grid, GridBatch):
            raise TypeError("source_grid must be a GridBatch")
        if target_grid is not None and not isinstance(target_grid, GridBatch):
            raise TypeError("target_grid must be a GridBatch")
        if not _is_vec3i(kernel_size) or not _is_vec3i(stride):
            raise TypeError(
                f"kernel_size and stride must be of type Vec3iOrScalar, but got {type(kernel_size)} and {type(stride)}"
            )
        C = _lib.load()
        self._impl = C.PackInfoImpl(
            _vec(kernel_size), _vec(stride), source_grid._impl, target_grid._impl if target_grid is not None else None
        )

    # ---------------------------------------------------------------- builders ----------
    def build_gather_scatter(self, use_me: bool = False) -> None:
        self._impl.build_gather_scatter(bool(use_me))

    def build_implicit_gemm(
        self,
        sorted: bool = False,
        split_mask_num: int = 1,
        training: bool = False,
        split_mask_num_bwd: int = 1,
        use_tf32: bool = False,
    ) -> None:
        self._impl.build_implicit_gemm(bool(sorted), int(split_mask_num), bool(training), int(split_mask_num_bwd), bool(use_tf32))

    def build_cutlass(self, benchmark: bool = False) -> None:
        # The brick backend's buffers are not needed: the one implementation uses the kernel map.
        self._impl.kmap()

    def build_lggs(self) -> None:
        if tuple(self.kernel_size) != (3, 3, 3):
            raise RuntimeError("LGGS only supports 3x3x3 kernel size")
        self._impl.kmap()

    # ---------------------------------------------------------------- convolutions ------
    def _features(self, input, grid_count: int, total: int) -> torch.Tensor:
        if isinstance(input, JaggedTensor):
            if input.num_outer_lists() != grid_count:
                raise ValueError("Input batch size must match target grid batch size")
            data = input.jdata
        elif isinstance(input, torch.Tensor):
            data = input
        else:
            raise TypeError("input must be a JaggedTensor or a torch.Tensor")
        if data.dim() == 0 or data.shape[0] != total:
            raise ValueError("Input element count must match target grid total voxels")
        return data

    def sparse_conv_3d(
        self,
        input,
        weights: torch.Tensor,
        backend: ConvPackBackend = ConvPackBackend.GATHER_SCATTER,
        *,
        precision: str | None = None,
    ):
        """out[t] = sum_k in[kmap[t,k]] . W[:, :, k]  on the target grid (weights (Do, Di, K0, K1, K2)).

        ``precision`` (extension, default: the features' dtype): "bf16" casts features and
        weights to BF16 (tcgen05, FP32 accumulate); "fp8" quantises them to E4M3 with
        per-channel scales (forward only, BF16 output)."""
        src = self._impl.source_grid
        data = self._features(input, src.grid_count, src.total_voxels)
        out = _apply(data, weights, self._impl, False, precision)
        return JaggedTensor.from_data_and_offsets(out, self._impl.target_grid.joffsets)

    def sparse_transpose_conv_3d(
        self,
        input,
        weights: torch.Tensor,
        backend: ConvPackBackend = ConvPackBackend.GATHER_SCATTER,
        *,
        precision: str | None = None,
    ):
        """Transposed convolution from the target grid back onto the source grid (weights (Di, Do, K0, K1, K2))."""
        tgt = self._impl.target_grid
        data = self._features(input, tgt.grid_count, tgt.total_voxels)
        out = _apply(data, weights, self._impl, True, precision)
        return JaggedTensor.from_data_and_offsets(out, self._impl.source_grid.joffsets)

    def _conv_with_bias(self, input, weights: torch.Tensor, bias: torch.Tensor | None, transposed: bool,
                        precision: str | None = None, relu: bool = False,
                        scale: torch.Tensor | None = None) -> JaggedTensor:
        """sparse_conv_3d / sparse_transpose_conv_3d times a per-output-channel scale (optional,
        inference only), plus a per-output-channel bias (and, with `relu`, max(., 0)), applied in
        the contraction's epilogue (used by nn.SparseConv3d and nn.Sequential's conv -> ReLU and
        conv -> BatchNorm (eval) -> ReLU fusions)."""
        src, tgt = self._impl.source_grid, self._impl.target_grid
        inp, out = (tgt, src) if transposed else (src, tgt)
        data = self._features(input, inp.grid_count, inp.total_voxels)
        y = _apply(data, weights, self._impl, transposed, precision, bias, relu, scale)
        return JaggedTensor.from_data_and_offsets(y, out.joffsets)

    # ---------------------------------------------------------------- devices -----------
    def to(self, to_device) -> "SparseConvPackInfo":
        d = torch.device(to_device)
        if d.type != "cuda":
            raise ValueError("fvdb_gb300 kernel maps live on CUDA devices")
        return self

    def cuda(self) -> "SparseConvPackInfo":
        return self

    def cpu(self) -> "SparseConvPackInfo":
        raise ValueError("fvdb_gb300 kernel maps live on CUDA devices")

    # ---------------------------------------------------------------- properties --------
    @property
    def source_grid(self):
        from .grid_batch import GridBatch

        return GridBatch(impl=self._impl.source_grid)

    @property
    def target_grid(self):
        from .grid_batch import GridBatch

        return GridBatch(impl=self._impl.target_grid)

    @property
    def kernel_size(self) -> tuple:
        return tuple(self._impl.kernel_size)

    @property
    def stride(self) -> tuple:
        return tuple(self._impl.stride)

    @property
    def out_in_map(self):
        return self._impl.out_in_map

    @property
    def out_in_map_bwd(self):
        return self._impl.out_in_map_bwd

    @property
    def neighborhood_map(self):
        return self._impl.neighborhood_map

    @property
    def neighborhood_sizes(self):
        return self._impl.neighborhood_sizes

    @property
    def reorder_loc(self):
        return self._impl.reorder_loc

    @property
    def sorted_mask(self):
        return self._impl.sorted_mask

    @property
    def reorder_out_in_map(self):
        return self._impl.reorder_out_in_map

    @property
    def reduced_sorted_mask(self):
        return self._impl.reduced_sorted_mask

    @property
    def reorder_loc_bwd(self):
        return self._impl.reorder_loc_bwd

    @property
    def reorder_out_in_map_bwd(self):
        return self._impl.reorder_out_in_map_bwd

    @property
    def sorted_mask_bwd_w(self):
        return self._impl.sorted_mask_bwd_w

    @property
    def sorted_mask_bwd_d(self):
        return self._impl.sorted_mask_bwd_d

    @property
    def use_me(self) -> bool:
        return self._impl.use_me

    @property
    def use_tf32(self) -> bool:
        return self._impl.use_tf32

    # brick / LGGS buffers of the reference's alternate backends: not built here
    block_kernel_in_idx = None
    block_kernel_ranges = None
    block_kernel_rel_out_idx = None
    halo_index_buffer = None
    output_index_buffer = None
