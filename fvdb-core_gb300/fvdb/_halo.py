"""Autograd Function of the leaf-halo convolution (GridBatch.sparse_conv_halo).

Forward, data gradient and weight gradient run in the C++ extension (halo_conv /
halo_wgrad) on the CUDA kernels of csrc/halo.cu, with no kernel map.  The weight layout and the
backward follow the reference's autograd body
(src/fvdb/detail/autograd/SparseConvolutionHalo.cpp:17-86): weights [O, I, 3, 3, 3] become
[3, 3, 3, I, O] (offset k = 9 K2 + 3 K1 + K0, K2 on ijk axis 0); the data gradient is the same
convolution of the output gradient with the mirrored, transposed weights; the weight gradient
comes back as [O, I, 3, 3, 3].
"""

from __future__ import annotations

import torch

from . import _lib


def halo_weights(weight: torch.Tensor, dtype: torch.dtype) -> torch.Tensor:
    """[O, I, 3, 3, 3] -> [27, I, O] in the features' dtype."""
    return weight.permute(4, 3, 2, 1, 0).reshape(27, weight.shape[1], weight.shape[0]).to(dtype).contiguous()


class HaloConvFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, grid_impl, data: torch.Tensor, weight: torch.Tensor):
        w = halo_weights(weight, data.dtype)
        y = _lib.load().halo_conv(grid_impl, data, w, False)
        ctx.save_for_backward(data, w)
        ctx.grid_impl = grid_impl
        ctx.weight_meta = (weight.shape, weight.dtype)
        return y

    @staticmethod
    def backward(ctx, grad_out):
        data, w = ctx.saved_tensors
        C = _lib.load()
        dy = grad_out.to(data.dtype).contiguous()
        dx = dw = None
        if ctx.needs_input_grad[1]:
            dx = C.halo_conv(ctx.grid_impl, dy, w, True)
        if ctx.needs_input_grad[2]:
            shape, wdtype = ctx.weight_meta
            dw = C.halo_wgrad(ctx.grid_impl, data, dy)  # [27, I, O]
            dw = dw.reshape(3, 3, 3, shape[1], shape[0]).permute(4, 3, 2, 1, 0).to(wdtype).contiguous()
        return None, dx, dw
