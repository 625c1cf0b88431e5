"""The oracle against the committed golden fixtures (no GPU).

Fixtures (tests/golden/make_golden.py) hold torch dense-conv float64 outputs and
coordinate-form neighbour relations; see that script for how they were made."""

import numpy as np
import pytest

from oracle import oracle as orc
from tests.helpers import golden_cases, kmap_to_coords, load_golden, rows_by_coord


@pytest.mark.parametrize("name", golden_cases("sparse_"))
def test_oracle_matches_golden(name):
    g = load_golden(name)
    ks, st = tuple(g["kernel_size"].tolist()), tuple(g["stride"].tolist())
    src, soff = orc.grid_from_ijk(g["ijk"], np.array([0, g["ijk"].shape[0]]))
    tgt, toff = (src, soff) if st == (1, 1, 1) else orc.conv_grid(src, soff, ks, st)
    assert set(map(tuple, tgt.tolist())) == set(map(tuple, g["target_ijk"].tolist()))
    kmap = orc.kernel_map(src, soff, tgt, toff, ks, st)
    order = [rows_by_coord(tgt)[tuple(r)] for r in g["target_ijk"].tolist()]
    assert np.array_equal(kmap_to_coords(kmap, src)[order], g["neighbours"])
    perm = [rows_by_coord(g["ijk"])[tuple(r)] for r in src.tolist()]
    out = orc.conv_forward_f64(g["features"][perm], g["weights"], kmap)
    np.testing.assert_allclose(out[order], g["expected"], rtol=1e-10, atol=1e-10)


@pytest.mark.parametrize("name", golden_cases("dense_transposed"))
def test_oracle_transposed_matches_golden(name):
    g = load_golden(name)
    ks = tuple(g["kernel_size"].tolist())
    src, soff = orc.grid_from_ijk(g["ijk"], np.array([0, g["ijk"].shape[0]]))
    kmap = orc.kernel_map(src, soff, src, soff, ks, (1, 1, 1))
    perm = [rows_by_coord(g["ijk"])[tuple(r)] for r in src.tolist()]
    out = orc.conv_forward_f64(g["features"][perm], g["weights"], kmap, transposed=True, n_src=src.shape[0])
    np.testing.assert_allclose(out, g["expected"][perm], rtol=1e-10, atol=1e-10)


@pytest.mark.parametrize("name", golden_cases("strided_transposed"))
def test_oracle_strided_transposed_matches_golden(name):
    """Coarse features onto the fine grid through the fine -> coarse forward map."""
    g = load_golden(name)
    ks, st = tuple(g["kernel_size"].tolist()), tuple(g["stride"].tolist())
    src, soff = orc.grid_from_ijk(g["ijk"], np.array([0, g["ijk"].shape[0]]))
    tgt, toff = orc.conv_grid(src, soff, ks, st)
    assert set(map(tuple, tgt.tolist())) == set(map(tuple, g["target_ijk"].tolist()))
    kmap = orc.kernel_map(src, soff, tgt, toff, ks, st)
    xt = g["features"][[rows_by_coord(g["target_ijk"])[tuple(r)] for r in tgt.tolist()]]
    out = orc.conv_forward_f64(xt, g["weights"], kmap, transposed=True, n_src=src.shape[0])
    perm = [rows_by_coord(g["ijk"])[tuple(r)] for r in src.tolist()]
    np.testing.assert_allclose(out, g["expected"][perm], rtol=1e-10, atol=1e-10)
