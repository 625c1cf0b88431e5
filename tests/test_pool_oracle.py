"""Pins the oracle's pooling and nearest upsampling (no GPU).

The reference pins these ops by equivalence with torch's dense pooling on a fully active box
(tests/unit/test_basic_ops.py:900-1230: MaxPool3d / AvgPool3d with ceil_mode, nn.Upsample);
the same equivalences are re-hosted here against the oracle, forward and backward.
"""

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import dense_ijk

N = 12


def _dense_case(seed, dtype=np.float64):
    ijk = dense_ijk((N, N, N))
    g, off = orc.grid_from_ijk(ijk, np.array([0, ijk.shape[0]]))
    x = np.random.default_rng(seed).standard_normal((g.shape[0], 3)).astype(dtype)
    return g, off, x


def _to_dense(g, x):
    d = torch.zeros(x.shape[1], N, N, N, dtype=torch.float64)
    d[:, g[:, 0], g[:, 1], g[:, 2]] = torch.from_numpy(x.astype(np.float64)).T
    return d


@pytest.mark.parametrize("pool,stride", [((2, 3, 1), 0), (2, 0), (3, 0), (5, 0), (7, 0), (2, 3), (3, 4), ((2, 3, 4), (3, 4, 5))])
def test_max_pool_matches_dense(pool, stride):
    g, off, x = _dense_case(1)
    st = stride if stride else pool
    c, coff = orc.coarsened_grid(g, off, st)
    y = orc.pool_forward(g, off, c, coff, x, pool, stride, "max")
    ref = torch.nn.functional.max_pool3d(_to_dense(g, x)[None], pool, stride=st, ceil_mode=True)[0]
    inside = np.all(c * np.asarray(orc._vec3(st)) < N, axis=1)  # windows that start inside the box
    want = ref[:, c[inside, 0], c[inside, 1], c[inside, 2]].T.numpy()
    assert np.array_equal(y[inside], want)


@pytest.mark.parametrize("pool", [2, 3, 4, (2, 3, 1), (3, 2, 4)])
def test_avg_pool_matches_dense(pool):
    g, off, x = _dense_case(2)
    c, coff = orc.coarsened_grid(g, off, pool)
    y = orc.pool_forward(g, off, c, coff, x, pool, 0, "avg")
    ref = torch.nn.functional.avg_pool3d(_to_dense(g, x)[None], pool, ceil_mode=True)[0]
    want = ref[:, c[:, 0], c[:, 1], c[:, 2]].T.numpy()
    np.testing.assert_allclose(y, want, rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("mode", ["max", "avg"])
def test_pool_gradients_match_dense_autograd(mode):
    g, off, x = _dense_case(3)
    pool = 2
    c, coff = orc.coarsened_grid(g, off, pool)
    dy = np.random.default_rng(4).standard_normal((c.shape[0], 3))
    dx = orc.pool_backward(g, off, c, coff, x, dy, pool, 0, mode)
    d = _to_dense(g, x).requires_grad_(True)
    f = torch.nn.functional.max_pool3d if mode == "max" else torch.nn.functional.avg_pool3d
    out = f(d[None], pool)[0]
    gd = torch.zeros_like(out)
    gd[:, c[:, 0], c[:, 1], c[:, 2]] = torch.from_numpy(dy).T
    out.backward(gd)
    want = d.grad[:, g[:, 0], g[:, 1], g[:, 2]].T.numpy()
    np.testing.assert_allclose(dx, want, rtol=1e-12, atol=1e-12)


def test_upsample_matches_dense():
    ijk = dense_ijk((4, 4, 4))
    c, coff = orc.grid_from_ijk(ijk, np.array([0, 64]))
    f, foff = orc.subdivided_grid(c, coff, 2)
    assert f.shape[0] == 512
    x = np.random.default_rng(5).standard_normal((64, 3))
    y = orc.upsample_forward(c, coff, f, foff, x, 2)
    d = torch.zeros(3, 4, 4, 4, dtype=torch.float64)
    d[:, c[:, 0], c[:, 1], c[:, 2]] = torch.from_numpy(x).T
    d.requires_grad_(True)
    up = torch.nn.functional.interpolate(d[None], scale_factor=2, mode="nearest")[0]
    np.testing.assert_array_equal(y, up[:, f[:, 0], f[:, 1], f[:, 2]].T.detach().numpy())
    dy = np.random.default_rng(6).standard_normal((512, 3))
    dx = orc.upsample_backward(c, coff, f, foff, dy, 2)
    gd = torch.zeros_like(up)
    gd[:, f[:, 0], f[:, 1], f[:, 2]] = torch.from_numpy(dy).T
    up.backward(gd)
    np.testing.assert_allclose(dx, d.grad[:, c[:, 0], c[:, 1], c[:, 2]].T.numpy(), rtol=1e-12, atol=1e-12)


def test_subdivide_mask_and_coarsen_negative():
    ijk = np.array([[-3, 0, 5], [-4, 1, 5], [7, -9, 2]], dtype=np.int32)
    g, off = orc.grid_from_ijk(ijk, np.array([0, 3]))
    c, _ = orc.coarsened_grid(g, off, 2)
    assert {tuple(r) for r in c.tolist()} == {(-2, 0, 2), (3, -5, 1)}
    mask = np.array([True, False, True])
    f, _ = orc.subdivided_grid(g, off, (1, 2, 1), mask)
    kept = {tuple(r) for r in g[mask].tolist()}
    assert {tuple(r) for r in f.tolist()} == {(x, 2 * y + j, z) for (x, y, z) in kept for j in (0, 1)}
