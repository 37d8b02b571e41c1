"""CPU checks of the differentiable float reconstruction's oracle: the provenance map names
a source of each output value inside its own plateau (checked against plateaus found by
scipy's graph components), and the fixed-point gradient agrees with float64 central finite
differences."""
import numpy as np
import pytest

INT_MIN = np.iinfo(np.int32).min


def _plateaus(R, conn):
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components

    H, W = R.shape
    idx = np.arange(H * W).reshape(H, W)
    rows, cols = [], []
    offs = [(0, 1), (1, 0)] + ([(1, 1), (1, -1)] if conn == 8 else [])
    for dy, dx in offs:
        ys = slice(0, H - dy)
        xs = slice(max(0, -dx), W - max(0, dx))
        ys2 = slice(dy, H)
        xs2 = slice(max(0, dx), W - max(0, -dx) if dx < 0 else W)
        a, b = R[ys, xs], R[ys2, xs2]
        eq = a == b
        rows.append(idx[ys, xs][eq])
        cols.append(idx[ys2, xs2][eq])
    r, c = np.concatenate(rows), np.concatenate(cols)
    g = coo_matrix((np.ones(len(r)), (r, c)), shape=(H * W, H * W))
    return connected_components(g, directed=False)[1].reshape(H, W)


def _inputs(kind, H=72, W=90, seed=0):
    rng = np.random.default_rng(seed)
    mask = rng.random((H, W), dtype=np.float32)
    if kind == "ties":
        mask = np.floor(mask * 8) / 8
    marker = (mask * rng.uniform(0.5, 1.0, (H, W))).astype(np.float32)
    if kind == "ties":
        marker = np.floor(marker * 8) / 8
    if kind == "negative":
        # mostly negative marker: the zero ring wins on the border and spreads inward
        marker = (marker - 1.0).astype(np.float32)
        mask = (mask - 0.2).astype(np.float32)
    return marker.astype(np.float32), mask.astype(np.float32)


@pytest.mark.parametrize("kind", ["tie_free", "ties", "negative"])
@pytest.mark.parametrize("conn", [4, 8])
def test_provenance_names_a_source_in_the_plateau(oracle, kind, conn):
    marker, mask = _inputs(kind)
    R, prov = oracle.recon_f32_prov(marker, mask, conn)
    assert np.array_equal(R, oracle.imreconstruct(marker, mask, conn))
    H, W = R.shape
    n = H * W
    q = np.where(prov >= 0, prov, np.where(prov == INT_MIN, -1, ~prov))
    val = np.where(prov == INT_MIN, np.float32(0),
                   np.where(prov >= 0, marker.ravel()[np.clip(q, 0, n - 1)].reshape(H, W),
                            mask.ravel()[np.clip(q, 0, n - 1)].reshape(H, W)))
    assert np.array_equal(val, R)
    lab = _plateaus(R, conn)
    # one provenance per plateau, and the source pixel lies in it
    for l in np.unique(lab):
        sel = lab == l
        assert len(np.unique(prov[sel])) == 1
        p = prov[sel][0]
        if p != INT_MIN:
            src = p if p >= 0 else ~p
            assert lab.ravel()[src] == l
        else:
            ys, xs = np.nonzero(sel)
            assert ((ys == 0) | (ys == H - 1) | (xs == 0) | (xs == W - 1)).any()
    if kind == "negative":
        assert (prov == INT_MIN).any()


@pytest.mark.parametrize("conn", [4, 8])
def test_gradient_matches_finite_differences(oracle, conn):
    from nsgb import synth

    mask, marker = synth.float_pair((48, 64), 11)
    R, prov = oracle.recon_f32_prov(marker, mask, conn)
    g = np.random.default_rng(5).standard_normal(R.shape).astype(np.float32)
    dm, dk = oracle.recon_f32_grad(g, prov)
    idx = np.arange(R.size)
    fm, fk, vm, vk = oracle.recon_fd(marker, mask, g, conn, idx, h=1e-4)
    assert (~vm).sum() + (~vk).sum() < 0.01 * 2 * R.size
    # the adjoint is the exact sum rounded once to float32, so it lies within half an ulp of the
    # float64 differences, whose own error is below 1e-10 here (2h = 2e-4 with x ~ 1 in float64)
    for fd, d, v in ((fm, dm.ravel(), vm), (fk, dk.ravel(), vk)):
        assert np.all((np.abs(fd - d) <= half_ulp(d) + 1e-10)[v])
    # every output pixel's gradient lands somewhere: the totals agree
    assert abs(float(dm.sum() + dk.sum()) - float(g[prov != INT_MIN].sum())) < 1e-3


def half_ulp(d):
    d = np.abs(np.asarray(d, np.float32))
    return (np.nextafter(d, np.float32(np.inf)) - d).astype(np.float64) / 2


def exact_float32_sum(vals):
    """The exact sum of float32 values, rounded once to float32 (nearest, ties to even)."""
    import math
    from fractions import Fraction

    exact = sum(Fraction(float(v)) for v in vals)
    d = math.fsum(float(v) for v in vals)
    assert Fraction(d) == exact  # representable in float64, so one rounding to float32 follows
    return np.float32(d)


def test_gradient_sum_is_exact_and_order_free(oracle):
    # all pixels of one plateau feed one source: the sum is the exact sum, rounded once
    g = np.random.default_rng(1).standard_normal((16, 16)).astype(np.float32)
    prov = np.full((16, 16), 5, np.int32)
    dm, dk = oracle.recon_f32_grad(g, prov)
    assert dm.ravel()[5] == exact_float32_sum(g.ravel()) and np.count_nonzero(dm) == 1 and not dk.any()
    perm = np.random.default_rng(2).permutation(g.size)
    dm2, _ = oracle.recon_f32_grad(g.ravel()[perm].reshape(g.shape), prov)
    assert dm2.ravel()[5] == dm.ravel()[5]


def test_gradient_sum_cancellation_and_small_values(oracle):
    """Cancellation leaves the small terms exact (a 2^-32 fixed point would lose them), values
    down to 2^-73 are exact, and a sum that ends between two floats rounds to nearest even."""
    g = np.zeros((1, 8), np.float32)
    g[0, :4] = [2.0**30, -(2.0**30), 2.0**-70, 3.0 * 2.0**-60]
    g[0, 4:] = [1.0, 2.0**-24, 2.0**-24, 0.0]  # 1 + 2^-23: exactly representable
    prov = np.array([[3, 3, 3, 3, ~1, ~1, ~1, ~1]], np.int32)
    dm, dk = oracle.recon_f32_grad(g, prov)
    assert dm[0, 3] == np.float32(2.0**-70 + 3.0 * 2.0**-60)
    assert dk[0, 1] == np.float32(1.0 + 2.0**-23)
    g2 = np.array([[1.0, 2.0**-24, 0.0, 0.0]], np.float32)  # 1 + 2^-24: a tie, rounds to even (1.0)
    dm2, _ = oracle.recon_f32_grad(g2, np.array([[0, 0, 2, 2]], np.int32))
    assert dm2[0, 0] == np.float32(1.0)
    with pytest.raises(ValueError):
        oracle.recon_f32_grad(np.full((1, 2), 2.0**31, np.float32), np.zeros((1, 2), np.int32))
