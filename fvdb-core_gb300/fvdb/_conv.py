"""The torch.autograd.Function of one sparse convolution.

Forward and backward bodies run in the C++ extension (conv_forward / conv_backward), which
launches the hand-written kernels through the C ABI: forward = fused gather-GEMM over the
kernel map; dgrad = the same contraction over the transposed map with W^T; wgrad = the
per-offset reduction with an FP64 cross-CTA sum.  Semantics follow
src/fvdb/detail/autograd/SparseConvolutionKernelMap.cpp:18-191 (weight permutes, checks,
gradient layout).
"""

from __future__ import annotations

import torch

from . import _lib


class SparseConvFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, features: torch.Tensor, weights: torch.Tensor, pack_impl, transposed: bool, bias=None,
                relu: bool = False, scale=None):
        C = _lib.load()
        y, wkio = C.conv_forward(features, weights, pack_impl, transposed, bias, relu, scale)
        ctx.scaled = scale is not None
        if relu:
            ctx.save_for_backward(features, wkio, y)
        else:
            ctx.save_for_backward(features, wkio)
        ctx.pack_impl = pack_impl
        ctx.transposed = transposed
        ctx.relu = relu
        ctx.bias_dtype = bias.dtype if bias is not None else None
        return y

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        C = _lib.load()
        features, wkio = ctx.saved_tensors[:2]
        need_dx, need_dw, need_db = ctx.needs_input_grad[0], ctx.needs_input_grad[1], ctx.needs_input_grad[4]
        if grad_out is None or not (need_dx or need_dw or need_db):
            return None, None, None, None, None, None, None
        if ctx.scaled:
            raise RuntimeError("a convolution with a folded batch norm (out_scale) is inference-only")
        if ctx.relu:
            # fused ReLU: the gradient passes where the output is positive (torch.relu's rule)
            grad_out = grad_out * (ctx.saved_tensors[2] > 0)
        dx = dw = None
        if need_dx or need_dw:
            dx, dw = C.conv_backward(grad_out, features, wkio, ctx.pack_impl, ctx.transposed, need_dx, need_dw)
        # bias gradient = column sum of dy, accumulated in at least FP32 (FP64 stays FP64)
        db = None
        if need_db:
            acc = torch.promote_types(grad_out.dtype, torch.float32)
            db = grad_out.sum(0, dtype=acc).to(ctx.bias_dtype)
        return (dx if need_dx else None), (dw if need_dw else None), None, None, db, None, None


def sparse_conv(features: torch.Tensor, weights: torch.Tensor, pack_impl, transposed: bool, bias=None,
                relu: bool = False, scale=None) -> torch.Tensor:
    """One sparse convolution with autograd; `bias` ([C_out], optional) is added, and with `relu`
    the output clamped at zero, in the contraction's epilogue on the tensor-core path (one pass
    over the output instead of two or three).  `scale` ([C_out], optional, inference only)
    multiplies the contraction before the bias: an eval-mode batch norm folded into the layer."""
    return SparseConvFunction.apply(features, weights, pack_impl, transposed, bias, relu, scale)
