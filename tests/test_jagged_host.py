"""JaggedTensor on the host: per-list reductions, row masks, arithmetic, list reshapes, slicing and
jcat, each against a plain loop over the lists (the reference's tests/unit/test_jagged_tensor.py
checks the same relations against torch_scatter and per-list torch ops)."""

import pytest
import torch


def _lists(seed, n=6, rows=(0, 40), eshape=(3, 4), dtype=torch.float64):
    g = torch.Generator().manual_seed(seed)
    sizes = torch.randint(rows[0], rows[1], (n,), generator=g).tolist()
    sizes[1] = 0  # an empty list
    return [torch.randn((s,) + eshape, generator=g, dtype=dtype) for s in sizes]


@pytest.mark.parametrize("dim", [-2, -1, 0, 1, 2])
@pytest.mark.parametrize("keepdim", [False, True])
def test_jsum(dim, keepdim):
    from fvdb import JaggedTensor

    ls = _lists(1)
    jt = JaggedTensor([t.clone() for t in ls]).requires_grad_(True)
    out = jt.jsum(dim=dim, keepdim=keepdim)
    ref = [t.sum(dim=dim, keepdim=True if dim == 0 else keepdim) for t in ls]
    assert out.lshape == [r.shape[0] for r in ref]
    assert torch.allclose(out.jdata, torch.cat(ref), atol=1e-12)
    go = torch.rand_like(out.jdata)
    out.jdata.backward(go)
    xs = [t.clone().requires_grad_(True) for t in ls]
    torch.cat([x.sum(dim=dim, keepdim=True if dim == 0 else keepdim) for x in xs]).backward(go)
    assert torch.allclose(jt.jdata.grad, torch.cat([x.grad for x in xs]))
    for bad in (-3, 3, 4, -4):
        with pytest.raises(IndexError):
            jt.jsum(dim=bad)


@pytest.mark.parametrize("largest", [True, False])
@pytest.mark.parametrize("dim", [-1, 0, 1])
def test_jmax_jmin(largest, dim):
    from fvdb import JaggedTensor

    ls = _lists(2)
    jt = JaggedTensor([t.clone() for t in ls]).requires_grad_(True)
    vals, idx = (jt.jmax if largest else jt.jmin)(dim=dim)
    fn = torch.max if largest else torch.min
    if dim == 0:
        ref = torch.stack([fn(t, 0)[0] if t.shape[0] else torch.zeros(t.shape[1:], dtype=t.dtype) for t in ls])
        assert vals.lshape == [1] * len(ls)
        base = 0
        for b, t in enumerate(ls):
            if t.shape[0]:
                loc = fn(t, 0)[1]
                assert torch.equal(idx.jdata[b], loc + base)
            base += t.shape[0]
    else:
        ref = torch.cat([fn(t, dim)[0] for t in ls])
    assert torch.equal(vals.jdata, ref)
    vals.jdata.sum().backward()
    assert float(jt.jdata.grad.sum()) == pytest.approx(float(vals.jdata.numel() - (ls[1].shape[1:].numel() if dim == 0 else 0)))


def test_rmask_and_reshape_and_slices():
    from fvdb import JaggedTensor

    ls = _lists(3, eshape=(2,))
    jt = JaggedTensor(ls)
    m = torch.rand(jt.jdata.shape[0], generator=torch.Generator().manual_seed(4)) < 0.5
    r = jt.rmask(m)
    off = jt.joffsets.tolist()
    for b, t in enumerate(ls):
        assert torch.equal(r[b].jdata, t[m[off[b]:off[b + 1]]])
    assert r.jdata.shape[0] == int(m.sum())
    sizes = jt.lshape[::-1]
    rs = jt.jreshape(sizes)
    assert rs.lshape == sizes and rs.jdata is jt.jdata
    with pytest.raises(ValueError):
        jt.jreshape([1, 2])
    sl = jt[2:5]
    assert sl.lshape == jt.lshape[2:5] and torch.equal(sl.jdata, torch.cat(ls[2:5]))
    assert [t.jdata.shape[0] for t in jt] == jt.lshape
    fi = JaggedTensor.from_data_and_indices(jt.jdata, jt.jidx, len(ls))
    assert torch.equal(fi.joffsets, jt.joffsets)
    with pytest.raises(ValueError):
        JaggedTensor.from_data_and_indices(jt.jdata, jt.jidx.flip(0), len(ls))


def test_arithmetic():
    from fvdb import JaggedTensor

    ls = _lists(5, eshape=(3,))
    a = JaggedTensor(ls)
    b = JaggedTensor([t.abs() + 1 for t in ls])
    A, B = a.jdata, b.jdata
    for got, want in [(a + b, A + B), (a - 2, A - 2), (2 - a, 2 - A), (3 * a, 3 * A), (a / b, A / B), (1 / b, 1 / B),
                      (a // b, A // B), (a % b, A % B), (b ** 2, B ** 2), (-a, -A), (a > b, A > B), (a == a, A == A),
                      (a.abs(), A.abs()), (b.sqrt(), B.sqrt()), (a.round(1), A.round(decimals=1))]:
        assert got.lshape == a.lshape and torch.equal(got.jdata, want)
    c = a.clone()
    c += b
    c *= 2
    assert torch.equal(c.jdata, (A + B) * 2) and torch.equal(a.jdata, A)
    with pytest.raises(ValueError):
        a + JaggedTensor([torch.zeros(3, 3)])
    assert a.float().dtype == torch.float32 and a.long().dtype == torch.int64


def test_jcat():
    from fvdb import JaggedTensor, jcat

    l1, l2 = _lists(6, eshape=(3,)), _lists(7, eshape=(3,))
    a, b = JaggedTensor(l1), JaggedTensor(l2)
    c = jcat([a, b])
    assert c.lshape == a.lshape + b.lshape and torch.equal(c.jdata, torch.cat([a.jdata, b.jdata]))
    d = jcat([a, b], dim=0)
    assert d.lshape == [x + y for x, y in zip(a.lshape, b.lshape)]
    for i in range(len(l1)):
        assert torch.equal(d[i].jdata, torch.cat([l1[i], l2[i]]))
    a2 = JaggedTensor([t * 2 for t in l1])
    for dim in (1, -1):
        e = jcat([a, a2], dim=dim)
        assert e.lshape == a.lshape and torch.equal(e.jdata, torch.cat([a.jdata, a2.jdata], 1))
    with pytest.raises(ValueError):
        jcat([a, b], dim=1)  # different list sizes
    with pytest.raises(ValueError):
        jcat([])
    with pytest.raises(ValueError):
        jcat([a, JaggedTensor(l1[:3])], dim=0)
