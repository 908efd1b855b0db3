"""The scipy observation operator ``Obsop_interp_l3`` (obsop.py:161-373):
neighbour rules (excluded ring and mask points, obsop.py:118-134 and
197-219) of the host construction against the oracle's restatement of the
reference's per-observation loop."""
import numpy as np
import pytest

from oracle import obsop as ref
from vardyn_gb300.obsop import interp_rows, l3_exclusion

GRID = (20, 26, 4.0e3, 6.0e3)


def _mask(ny, nx):
    m = np.zeros((ny, nx), dtype=bool)
    m[8:12, 10:15] = True       # island
    m[15:, 3] = True            # strip down to row 0's column 3 at the far edge
    return m


@pytest.mark.parametrize("borders", [False, True])
@pytest.mark.parametrize("with_mask", [False, True])
def test_exclusion_table_matches_reference_sets(borders, with_mask):
    ny, nx, dx, dy = GRID
    mask = _mask(ny, nx) if with_mask else None
    got = set(np.flatnonzero(l3_exclusion(ny, nx, mask, borders)).tolist())
    assert got == ref.l3_excluded(ny, nx, dx, dy, mask, borders)


def test_mask_rule_is_the_references_column_rule():
    ny, nx, _, _ = GRID
    ex = l3_exclusion(ny, nx, _mask(ny, nx), False).reshape(ny, nx)
    # the masked points themselves are not excluded; row 0 at their columns is
    assert ex[8:12, 10:15].sum() == 0
    assert set(np.flatnonzero(ex[0]).tolist()) == {3, 10, 11, 12, 13, 14}
    assert ex[1:].sum() == 0


def _dense(data, rows, cols, n, size):
    h = np.zeros((n, size))
    np.add.at(h, (rows, cols), data)
    return h


@pytest.mark.parametrize("npix", [1, 2, 4])
@pytest.mark.parametrize("borders", [False, True])
def test_host_rows_match_reference_loop(npix, borders):
    ny, nx, dx, dy = GRID
    rng = np.random.default_rng(10 * npix + borders)
    n = 300
    x = rng.uniform(-20.0, nx * dx / 1e3 + 20.0, n)
    y = rng.uniform(-20.0, ny * dy / 1e3 + 20.0, n)
    ex = l3_exclusion(ny, nx, _mask(ny, nx), borders)
    idx, w = interp_rows(x, y, ny, nx, dx, dy, npix, exclude=ex)
    r = np.repeat(np.arange(n), npix).reshape(n, npix)
    keep = idx >= 0
    h = _dense(w[keep], r[keep], idx[keep], n, ny * nx)
    d, rr, cc = ref.sparse_op_l3(x, y, ny, nx, dx, dy, npix, ref.l3_excluded(ny, nx, dx, dy, _mask(ny, nx), borders))
    h_ref = _dense(d, rr, cc, n, ny * nx)
    assert np.abs(h - h_ref).max() <= 1e-15
    # some observations lost a neighbour to the rule, none kept an excluded one
    assert np.all(ex[idx[keep]] == 0)
    assert keep.sum() < _dense(*ref.sparse_op_l3(x, y, ny, nx, dx, dy, npix), n, ny * nx).astype(bool).sum()


def test_empty_exclusion_is_the_jax_operator():
    ny, nx, dx, dy = GRID
    rng = np.random.default_rng(3)
    x = rng.uniform(0, nx * dx / 1e3, 200)
    y = rng.uniform(0, ny * dy / 1e3, 200)
    a = interp_rows(x, y, ny, nx, dx, dy, 4)
    b = interp_rows(x, y, ny, nx, dx, dy, 4, exclude=np.zeros(ny * nx, np.uint8))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
