"""Host-side algebra of the batch-norm folding: BatchNorm.folded_affine's (s, t) reproduce the
eval-mode BatchNorm1d map x -> x * s + t, with and without the affine parameters, and a
training-mode layer (batch statistics) folds to nothing."""

import pytest
import torch


@pytest.mark.parametrize("affine", [True, False])
def test_folded_affine_matches_eval_batch_norm(affine):
    import fvdb.nn as fvnn

    g = torch.Generator().manual_seed(2)
    bn = fvnn.BatchNorm(12, affine=affine, eps=1e-3).eval()
    with torch.no_grad():
        bn.running_mean.copy_(torch.randn(12, generator=g))
        bn.running_var.copy_(torch.rand(12, generator=g) + 0.1)
        if affine:
            bn.weight.copy_(torch.randn(12, generator=g))
            bn.bias.copy_(torch.randn(12, generator=g))
    x = torch.randn(50, 12, generator=g)
    s, t = bn.folded_affine()
    ref = torch.nn.BatchNorm1d.forward(bn, x)
    assert torch.allclose(x * s + t, ref, rtol=1e-5, atol=1e-6)
    bn.train()
    assert bn.folded_affine() is None


def test_conv_folds_bias_into_shift():
    import fvdb.nn as fvnn

    conv = fvnn.SparseConv3d(4, 6, 3, bias=True)
    s, t = torch.rand(6) + 0.5, torch.randn(6)
    scale, shift = conv._folded((s, t))
    assert torch.equal(scale, s)
    assert torch.allclose(shift, conv.bias.detach() * s + t)
    conv_nb = fvnn.SparseConv3d(4, 6, 3, bias=False)
    assert torch.equal(conv_nb._folded((s, t))[1], t)


def test_convert_sync_batchnorm_keeps_state():
    import fvdb.nn as fvnn

    net = torch.nn.Sequential(fvnn.SparseConv3d(4, 8, 3), fvnn.BatchNorm(8), fvnn.ReLU(),
                              torch.nn.Sequential(fvnn.BatchNorm(8, affine=False)))
    with torch.no_grad():
        net[1].running_mean.fill_(0.25)
        net[1].weight.fill_(3.0)
    net[3][0].eval()
    out = fvnn.SyncBatchNorm.convert_sync_batchnorm(net)
    assert type(out[1]) is fvnn.SyncBatchNorm and type(out[3][0]) is fvnn.SyncBatchNorm
    assert out[1].weight is net[1].weight and torch.equal(out[1].running_mean, torch.full((8,), 0.25))
    assert out[3][0].weight is None and not out[3][0].training
    assert type(out[0]) is fvnn.SparseConv3d and type(out[2]) is fvnn.ReLU


def test_sequential_does_not_fold_across_dtype_promotion(monkeypatch):
    """A wider bias than the features would promote the unfused output, so the fold is skipped."""
    import fvdb.nn as fvnn
    from fvdb.nn import modules

    conv, bn = fvnn.SparseConv3d(4, 6, 3), fvnn.BatchNorm(6).eval()
    seq = fvnn.Sequential(conv, bn)
    calls = []
    monkeypatch.setattr(modules.SparseConv3d, "forward", lambda self, x, **k: calls.append(k) or x)
    monkeypatch.setattr(modules.BatchNorm, "forward", lambda self, x: x)

    class Feats:
        jdata = torch.zeros(3, 4, dtype=torch.bfloat16)

    x = object.__new__(fvnn.VDBTensor)
    x.data = Feats()
    with torch.no_grad():
        seq(x)
    assert calls == [{}]  # conv bias is FP32, features BF16: layers run one by one
    calls.clear()
    Feats.jdata = torch.zeros(3, 4)
    with torch.no_grad():
        seq(x)
    assert len(calls) == 1 and "out_affine" in calls[0]
