"""Autograd Functions of pooling and nearest upsampling between a fine and a coarse grid.

Forward and backward run in the C++ extension (pool_forward / pool_backward /
upsample_forward / upsample_backward) on the CUDA kernels of csrc/pool.cu.  Semantics follow
the reference's autograd bodies (src/fvdb/detail/autograd/MaxPoolGrid.cpp,
AvgPoolGrid.cpp, UpsampleGrid.cpp): the gradient of max pooling goes to each window's first
strict maximum, of average pooling to every voxel of the window (times 1 / pool volume), of
nearest upsampling to the parent (summed over its children).
"""

from __future__ import annotations

import torch

from . import _lib


class PoolFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, mode: int, fine_impl, coarse_impl, pool, stride, data: torch.Tensor):
        C = _lib.load()
        y = C.pool_forward(mode, fine_impl, coarse_impl, pool, stride, data)
        ctx.save_for_backward(data)
        ctx.args = (mode, fine_impl, coarse_impl, pool, stride)
        return y

    @staticmethod
    def backward(ctx, grad_out):
        (data,) = ctx.saved_tensors
        mode, fine_impl, coarse_impl, pool, stride = ctx.args
        dx = None
        if ctx.needs_input_grad[5]:
            dx = _lib.load().pool_backward(mode, fine_impl, coarse_impl, pool, stride, data, grad_out.contiguous())
        return None, None, None, None, None, dx


class UpsampleFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, coarse_impl, fine_impl, factor, data: torch.Tensor):
        y = _lib.load().upsample_forward(coarse_impl, fine_impl, factor, data)
        ctx.save_for_backward(data)
        ctx.args = (coarse_impl, fine_impl, factor)
        return y

    @staticmethod
    def backward(ctx, grad_out):
        (data,) = ctx.saved_tensors
        coarse_impl, fine_impl, factor = ctx.args
        dx = None
        if ctx.needs_input_grad[3]:
            dx = _lib.load().upsample_backward(coarse_impl, fine_impl, factor, grad_out.contiguous(), data)
        return None, None, None, dx
