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
    tol = 4e-7 * np.maximum(1.0, np.abs(dm.ravel()))
    assert np.all(np.abs(fm - dm.ravel())[vm] <= tol[vm])
    tol = 4e-7 * np.maximum(1.0, np.abs(dk.ravel()))
    assert np.all(np.abs(fk - dk.ravel())[vk] <= tol[vk])
    # every output pixel's gradient lands somewhere: the totals agree
    assert abs(float(dm.sum() + dk.sum()) - float(g[prov != INT_MIN].sum())) < 1e-3


def test_fixed_point_sum_is_order_free(oracle):
    # all pixels of one plateau feed one source: the sum is the exact integer sum
    g = np.random.default_rng(1).standard_normal((16, 16)).astype(np.float32)
    prov = np.full((16, 16), 5, np.int32)
    dm, dk = oracle.recon_f32_grad(g, prov)
    exp = np.float32(np.sum(np.rint(g.astype(np.float64) * 2.0**32).astype(np.int64)) * 2.0**-32)
    assert dm.ravel()[5] == exp and np.count_nonzero(dm) == 1 and not dk.any()
