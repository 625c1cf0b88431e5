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
    def forward(ctx, features: torch.Tensor, weights: torch.Tensor, pack_impl, transposed: bool):
        C = _lib.load()
        y, wkio = C.conv_forward(features, weights, pack_impl, transposed)
        ctx.save_for_backward(features, wkio)
        ctx.pack_impl = pack_impl
        ctx.transposed = transposed
        return y

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        C = _lib.load()
        features, wkio = ctx.saved_tensors
        need_dx, need_dw = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        if grad_out is None or not (need_dx or need_dw):
            return None, None, None, None
        dx, dw = C.conv_backward(grad_out, features, wkio, ctx.pack_impl, ctx.transposed, need_dx, need_dw)
        return (dx if need_dx else None), (dw if need_dw else None), None, None


def sparse_conv(features: torch.Tensor, weights: torch.Tensor, pack_impl, transposed: bool) -> torch.Tensor:
    return SparseConvFunction.apply(features, weights, pack_impl, transposed)
