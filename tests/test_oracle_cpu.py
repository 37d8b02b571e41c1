"""Pins the CPU oracle (oracle/) before it is trusted as the checker of the GPU path.

* union-find labelling: exact match with the reference's own ConnComponents.cpp, through the
  committed fixtures (tests/golden/ref_ccl_cases.npz) and, where oracle/_ref was built, live;
* bounding boxes: the same for ConnComponents::boundingBox (tests/golden/ref_bbox_cases.npz),
  plus an independent numpy formulation;
* reconstruction: the reference's inline 32x32 queue fixture, and an independent numpy
  fixed-point definition (Jacobi iteration to convergence) on random small images, including
  the 0-valued padding ring and odd / non-square sizes;
* hole filling, bwselect, binary reconstruction, h-minima: independent scipy / numpy
  formulations.
"""
import os

import numpy as np
import pytest
import scipy.ndimage as ndi

from conftest import ROOT  # noqa: F401


# ---------------------------------------------------------------------------------------
# Independent definitions (numpy), small sizes only.
def struct(conn):
    return ndi.generate_binary_structure(2, 1 if conn == 4 else 2)


def np_recon(marker, mask, conn, erode=False, ring=True):
    """Fixed point of R = max(R, min(nbr_max(R), mask)) over the image padded with a fixed
    0 ring (the reference's copyMakeBorder(..., 0)); erode = the dual without a ring."""
    if erode:
        if np.issubdtype(mask.dtype, np.floating):
            return -np_recon(-marker, -mask, conn, False, ring)
        if np.issubdtype(mask.dtype, np.signedinteger):
            return ~np_recon(~marker, ~mask, conn, False, ring)
        mx = np.iinfo(mask.dtype).max
        return (mx - np_recon((mx - marker).astype(mask.dtype), (mx - mask).astype(mask.dtype), conn, False,
                              ring)).astype(mask.dtype)
    H, W = mask.shape
    low = np.finfo(mask.dtype).min if np.issubdtype(mask.dtype, np.floating) else np.iinfo(mask.dtype).min
    pad_v = 0 if ring else low
    K = np.full((H + 2, W + 2), pad_v, mask.dtype)
    K[1:-1, 1:-1] = mask
    R = np.full((H + 2, W + 2), pad_v, mask.dtype)
    R[1:-1, 1:-1] = np.minimum(marker, mask)
    fp = struct(conn)
    while True:
        D = ndi.grey_dilation(R, footprint=fp, mode="constant", cval=low)
        N = R.copy()
        N[1:-1, 1:-1] = np.maximum(R[1:-1, 1:-1], np.minimum(D[1:-1, 1:-1], K[1:-1, 1:-1]))
        if np.array_equal(N, R):
            return R[1:-1, 1:-1]
        R = N


def np_binary_recon(marker, mask, conn):
    lab, _ = ndi.label(mask != 0, structure=struct(conn))
    seeded = np.unique(lab[(marker != 0) & (mask != 0)])
    seeded = seeded[seeded > 0]
    filled = np.isin(lab, seeded) & (mask != 0) & (marker == 0)
    out = marker.copy()
    out[filled] = np.iinfo(mask.dtype).max
    return out


def np_fill_binary(img, conn):
    mx = np.iinfo(img.dtype).max
    cls = img != mx
    lab, _ = ndi.label(cls, structure=struct(conn))
    border = np.unique(np.concatenate([lab[0], lab[-1], lab[:, 0], lab[:, -1]]))
    border = border[border > 0]
    reach = np.isin(lab, border)
    return np.where(reach, 0, mx).astype(img.dtype)


def rand_gray(rng, h, w, dtype, levels=6):
    if dtype == np.float32:
        return rng.random((h, w)).astype(np.float32)
    base = rng.integers(0, levels, (h, w))
    if dtype == np.uint8:
        return (base * 40).astype(np.uint8)
    if dtype == np.uint16:
        return (base * 10000).astype(np.uint16)
    return (base * 1000 - 1500).astype(np.int32)  # includes negatives: exercises the ring


SHAPES = [(1, 1), (1, 9), (9, 1), (5, 7), (13, 31), (33, 17), (40, 40)]


# ---------------------------------------------------------------------------------------
def test_labels_match_reference_fixtures(oracle, golden_dir):
    d = np.load(os.path.join(golden_dir, "ref_ccl_cases.npz"))
    k = 0
    while f"img{k}" in d:
        img = d[f"img{k}"]
        for conn in (4, 8):
            lab, _ = oracle.bwlabel2(img, conn, relab=False)
            rel, n = oracle.bwlabel2(img, conn, relab=True)
            assert np.array_equal(lab, d[f"lab{k}_{conn}"]), (k, conn)
            assert np.array_equal(rel, d[f"rel{k}_{conn}"]), (k, conn)
            assert n == int(d[f"n{k}_{conn}"])
            kept, nk = oracle.bwareaopen2(lab, True, False, 3, 40, conn)
            assert np.array_equal(kept, d[f"kept{k}_{conn}"]) and nk == int(d[f"nk{k}_{conn}"])
        k += 1
    assert k >= 30


def test_labels_match_reference_live(oracle):
    if not oracle.ref_available():
        pytest.skip("reference ConnComponents not built here (oracle/_ref)")
    rng = np.random.default_rng(7)
    for trial in range(40):
        h, w = rng.integers(1, 90, 2)
        img = (rng.integers(0, 3, (h, w)) * 100).astype(np.uint8)
        for conn in (4, 8):
            a, n = oracle.bwlabel2(img, conn, True)
            b, m = oracle.ref_label(img, conn, True)
            assert n == m and np.array_equal(a, b)


def _bbox_numpy(labels, bg):
    """Independent formulation: the scan ends at the first -1 / 0 pixel that is not bg;
    entries in order of first appearance."""
    flat = labels.ravel()
    bad = np.flatnonzero(((flat == -1) | (flat == 0)) & (flat != bg))
    end = bad[0] if bad.size else flat.size
    idx = np.flatnonzero(flat[:end] != bg)
    if idx.size == 0:
        return np.zeros((5, 0), np.int32)
    labs, first = np.unique(flat[idx], return_index=True)
    order = np.argsort(idx[first])
    W = labels.shape[1]
    out = []
    for l in labs[order]:
        p = idx[flat[idx] == l]
        x, y = p % W, p // W
        out.append([l, x.min(), x.max(), y.min(), y.max()])
    return np.array(out, np.int32).T


def test_bbox_matches_reference_fixtures(oracle, golden_dir):
    d = np.load(os.path.join(golden_dir, "ref_bbox_cases.npz"))
    k = 0
    while f"lab{k}" in d:
        lab, bg = d[f"lab{k}"], int(d[f"bg{k}"])
        got = oracle.bounding_box(lab, bg)
        assert np.array_equal(got, d[f"box{k}"]), k
        assert np.array_equal(got, _bbox_numpy(lab, bg)), k
        k += 1
    assert k >= 150


def test_bbox_matches_reference_live(oracle):
    if not oracle.ref_available():
        pytest.skip("reference ConnComponents not built here (oracle/_ref)")
    rng = np.random.default_rng(11)
    for trial in range(60):
        h, w = rng.integers(1, 60, 2)
        lab = rng.integers(-1, 9, (h, w)).astype(np.int32)
        bg = int(rng.choice([-1, 0, 4]))
        assert np.array_equal(oracle.bounding_box(lab, bg), oracle.ref_bounding_box(lab, bg))


def test_recon_reference_queue_fixture(oracle, golden_dir):
    d = np.load(os.path.join(golden_dir, "ref_fixture_32.npz"))
    image = d["image"].astype(np.int32)
    seeds = d["seeds"].astype(np.int32)
    assert sorted(int(v) for v in d["seed_list"]) == sorted(int(v) for v in np.flatnonzero(seeds))
    for conn in (4, 8):
        out = oracle.imreconstruct(seeds, image, conn)
        assert np.array_equal(out, d[f"expected{conn}"])


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.int32, np.float32])
@pytest.mark.parametrize("conn", [4, 8])
def test_recon_matches_fixed_point_definition(oracle, dtype, conn):
    rng = np.random.default_rng(11 + conn)
    for (h, w) in SHAPES:
        mask = rand_gray(rng, h, w, dtype)
        marker = rand_gray(rng, h, w, dtype)  # not <= mask: exercises min(marker, mask)
        got = oracle.imreconstruct(marker, mask, conn)
        exp = np_recon(marker, mask, conn)
        assert np.array_equal(got, exp), (h, w)
        assert (got <= mask).all() and (got >= np.minimum(marker, mask)).all()
        assert np.array_equal(oracle.imreconstruct(got, mask, conn), got)  # idempotent


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.int32])
@pytest.mark.parametrize("conn", [4, 8])
def test_binary_recon_and_bwselect(oracle, dtype, conn):
    rng = np.random.default_rng(5)
    mx = np.iinfo(dtype).max
    for (h, w) in SHAPES:
        mask = (rng.random((h, w)) < 0.55).astype(dtype) * mx
        marker = (rng.random((h, w)) < 0.08).astype(dtype) * 7
        assert np.array_equal(oracle.imreconstruct_binary(marker, mask, conn), np_binary_recon(marker, mask, conn))
        seeds = (rng.random((h, w)) < 0.1).astype(dtype)
        sel = oracle.bwselect(mask, seeds, conn)
        exp = np_binary_recon(np.where(seeds != 0, mask, 0).astype(dtype), mask, conn) & mask
        assert np.array_equal(sel, exp)


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16])
@pytest.mark.parametrize("conn", [4, 8])
def test_fill_holes_binary(oracle, dtype, conn):
    rng = np.random.default_rng(3)
    mx = np.iinfo(dtype).max
    for (h, w) in SHAPES:
        img = (rng.random((h, w)) < 0.5).astype(dtype) * mx
        got = oracle.imfill_holes(img, True, conn)
        assert np.array_equal(got, np_fill_binary(img, conn))
        # 0/max input: the usual scipy hole filling (background connectivity = conn)
        exp = ndi.binary_fill_holes(img != 0, structure=struct(conn)).astype(dtype) * mx
        assert np.array_equal(got, exp)


def test_fill_holes_binary_int32_is_constant(oracle):
    img = (np.random.default_rng(0).random((9, 11)) < 0.5).astype(np.int32) * 255
    got = oracle.imfill_holes(img, True, 4)
    assert (got == np.iinfo(np.int32).max).all()


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.int32, np.float32])
@pytest.mark.parametrize("conn", [4, 8])
def test_fill_holes_gray_is_border_erosion(oracle, dtype, conn):
    rng = np.random.default_rng(9)
    for (h, w) in SHAPES:
        img = rand_gray(rng, h, w, dtype)
        if dtype == np.int32:
            img = np.abs(img).astype(np.int32)
        got = oracle.imfill_holes(img, False, conn)
        top = np.finfo(dtype).max if dtype == np.float32 else np.iinfo(dtype).max
        marker = np.full_like(img, top)
        marker[0], marker[-1], marker[:, 0], marker[:, -1] = img[0], img[-1], img[:, 0], img[:, -1]
        exp = np_recon(marker, img, conn, erode=True, ring=False)
        assert np.array_equal(got, exp), (h, w)


@pytest.mark.parametrize("dtype", [np.uint8, np.float32])
def test_hmin(oracle, dtype):
    rng = np.random.default_rng(4)
    for (h, w) in SHAPES:
        img = rand_gray(rng, h, w, dtype)
        hv = 30 if dtype == np.uint8 else 0.25
        got = oracle.imhmin(img, hv, 8)
        if dtype == np.uint8:
            inv = (255 - img).astype(np.uint8)
            mk = np.maximum(inv.astype(int) - hv, 0).astype(np.uint8)
            exp = (255 - np_recon(mk, inv, 8)).astype(np.uint8)
        else:
            exp = -np_recon((-img - np.float32(hv)).astype(np.float32), -img, 8)
        assert np.array_equal(got, exp)


def test_chain_small(oracle):
    from nsgb import synth

    mask, marker = synth.tile_u8(96, 80, 12, 1)
    r = oracle.chain(marker, mask)
    assert np.array_equal(r["recon"], oracle.imreconstruct(marker, mask, 8))
    assert np.array_equal(r["thr"], np.where(r["recon"] > 128, 255, 0))
    assert np.array_equal(r["fill"], oracle.imfill_holes(r["thr"], True, 4))
    lab, n = oracle.bwlabel2(r["fill"], 8, True)
    assert np.array_equal(r["labels"], lab) and n == r["n_labels"]
    a, k = oracle.bwareaopen2(r["fill"], False, True, 11, 1000, 8)
    assert np.array_equal(r["area"], a) and k == r["n_kept"]


def np_candidates(rc, rc_open, rbc, g1=80, g2=45, lo=11, hi=1000):
    """Independent statement of HistologicalEntities.cpp:195-275: numpy reconstruction, scipy
    hole filling (4-connected background), 8-connected areas and component selection."""
    rec = np_recon(rc_open, rc, 8)
    diff = np.where(rc > rec, rc.astype(np.int16) - rec, 0)
    bw1 = np_fill_binary(np.where(diff > g1, 255, 0).astype(np.uint8), 4) != 0
    lab, _ = ndi.label(bw1, structure=struct(8))
    areas = np.bincount(lab.ravel())
    keep = (areas >= lo) & (areas < hi)
    keep[0] = False
    bw1_t = keep[lab]
    bw2 = diff > g2
    lab2, _ = ndi.label(bw2, structure=struct(8))
    sel = np.unique(lab2[bw1_t & bw2])
    sel = sel[sel > 0]
    seg = np.isin(lab2, sel) & bw2 & (rbc == 0)
    return np.where(seg, 255, 0).astype(np.uint8), int(keep.sum())


@pytest.mark.parametrize("case", ["tile", "noise", "small", "row", "col"])
def test_nucleus_candidates_composition(oracle, case):
    import candidates_inputs as ci

    rng = np.random.default_rng(11)
    if case == "tile":
        rc, rc_open, rbc = ci.tile(128, 96, 14, 3)
    elif case == "noise":
        rc, rc_open, rbc = ci.noise(rng, 40, 52)
    elif case == "small":
        rc, rc_open, rbc = ci.tile(9, 13, 2, 5, drop=120)
    elif case == "row":
        rc, rc_open, rbc = ci.noise(rng, 1, 90)
    else:
        rc, rc_open, rbc = ci.noise(rng, 90, 1)
    seg, n = oracle.nucleus_candidates(rc, rc_open, rbc)
    exp, n_exp = np_candidates(rc, rc_open, rbc)
    assert n == n_exp
    assert np.array_equal(seg, exp)
    if case == "tile":
        assert n > 0 and seg.any()


def test_nucleus_candidates_thresholds(oracle):
    import candidates_inputs as ci

    rc, rc_open, rbc = ci.tile(120, 120, 20, 7)
    for g1, g2, lo, hi in [(80, 45, 11, 1000), (40, 60, 1, 10 ** 6), (255, 45, 11, 1000), (80.5, 44.9, 30, 200)]:
        seg, n = oracle.nucleus_candidates(rc, rc_open, rbc, g1, g2, lo, hi)
        exp, n_exp = np_candidates(rc, rc_open, rbc, g1, g2, lo, hi)
        assert n == n_exp and np.array_equal(seg, exp), (g1, g2, lo, hi)
    # nothing above g1 = 255: no component survives, nothing is selected
    seg, n = oracle.nucleus_candidates(rc, rc_open, rbc, 255, 45)
    assert n == 0 and not seg.any()


def np_morph_open(img, kern):
    """OpenCV's erode / dilate convention written out in numpy: min / max of
    src(y + i - c, x + j - c) over the element, outside the image 255 for the erosion and 0 for
    the dilation (morphOpen's borders, MorphologicOperations.cpp:2472-2481)."""
    k = kern.shape[0]
    c = (k - 1) // 2
    H, W = img.shape

    def pass_(src, pad, op):
        P = np.full((H + 2 * c, W + 2 * c), pad, np.uint8)
        P[c:c + H, c:c + W] = src
        acc = np.full((H, W), pad, np.uint8)  # the identity of the fold
        for i in range(k):
            for j in range(k):
                if kern[i, j]:
                    acc = op(acc, P[i:i + H, j:j + W])
        return acc

    return pass_(pass_(img, 255, np.minimum), 0, np.maximum)


@pytest.mark.parametrize("shape", [(1, 1), (1, 40), (40, 1), (23, 37), (70, 90)])
def test_morph_open(oracle, shape):
    from nsgb import disk19, ellipse3

    rng = np.random.default_rng(shape[0] * 100 + shape[1])
    img = rng.integers(0, 256, shape).astype(np.uint8)
    asym = (rng.random((5, 5)) < 0.4).astype(np.uint8)
    asym[0, 4] = 1
    y, x = np.mgrid[-31:32, -31:32]
    disk63 = (x * x + y * y <= 31 * 31).astype(np.uint8)
    kerns = (disk19(), ellipse3(), np.ones((3, 3), np.uint8), asym) + ((disk63,) if shape[0] * shape[1] < 1000 else ())
    for kern in kerns:
        got = oracle.morph_open(img, kern)
        assert np.array_equal(got, np_morph_open(img, kern))
        if np.array_equal(kern, kern[::-1, ::-1]):  # symmetric: scipy's footprint convention agrees
            e = ndi.grey_erosion(img, footprint=kern != 0, mode="constant", cval=255)
            assert np.array_equal(got, ndi.grey_dilation(e, footprint=kern != 0, mode="constant", cval=0))


def test_disk19_matches_reference_shape():
    from nsgb import disk19

    d = disk19()
    assert d.shape == (19, 19) and int(d.sum()) == 321
    assert np.array_equal(d, d[::-1]) and np.array_equal(d, d[:, ::-1]) and np.array_equal(d, d.T)
    assert [int(r.sum()) for r in d[:5]] == [11, 13, 15, 17, 19]


def _blob_mask(rng, h, w, n):
    m = np.zeros((h, w), np.uint8)
    yy, xx = np.mgrid[0:h, 0:w]
    for _ in range(n):
        cy, cx, r = rng.integers(0, h), rng.integers(0, w), rng.integers(2, 15)
        m[(yy - cy) ** 2 + (xx - cx) ** 2 <= r * r] = 255
    return m


@pytest.mark.parametrize("case", ["blobs", "noise", "one_zero", "row", "col", "dense", "band", "far"])
def test_distance_transform_exact(oracle, case):
    """The oracle's distance map equals scipy's exact EDT (float64 sqrt of the integer squared
    distance, rounded to float32), and the basins follow HistologicalEntities.cpp:347-356."""
    rng = np.random.default_rng(len(case))
    if case == "blobs":
        m = _blob_mask(rng, 120, 150, 25)
    elif case == "noise":
        m = np.where(rng.random((60, 70)) < 0.8, 255, 0).astype(np.uint8)
    elif case == "one_zero":
        m = np.full((50, 90), 255, np.uint8)
        m[49, 0] = 0
    elif case == "row":
        m = np.where(rng.random((1, 200)) < 0.9, 7, 0).astype(np.uint8)
    elif case == "col":
        m = np.where(rng.random((200, 1)) < 0.9, 7, 0).astype(np.uint8)
    elif case == "dense":
        m = np.where(rng.random((80, 80)) < 0.995, 1, 0).astype(np.uint8)
        m[0, 0] = 0
    elif case == "band":  # zeros in a few rows and columns only: columns without any zero
        m = np.full((300, 200), 9, np.uint8)
        m[130:140:3, ::37] = 0
    else:  # one zero row with a gap: distances grow down the image
        m = np.full((400, 150), 255, np.uint8)
        m[0, :] = 0
        m[0, 75] = 255
    d = oracle.distance_transform(m)
    exp = ndi.distance_transform_edt(m != 0).astype(np.float32)
    assert np.array_equal(d, exp)
    b = oracle.distance_transform(m, basins=True)
    assert np.array_equal(b, np.where(m != 0, -exp, -np.finfo(np.float32).max).astype(np.float32))


def test_distance_transform_without_zero(oracle):
    d = oracle.distance_transform(np.full((5, 7), 3, np.uint8))
    assert np.isinf(d).all() and (d > 0).all()


def test_distance_queue_never_below_exact(oracle):
    """The reference's queue propagation settles on a real zero pixel, so it is never closer than
    the exact distance; on blob masks it agrees almost everywhere."""
    rng = np.random.default_rng(3)
    m = _blob_mask(rng, 200, 260, 60)
    exact = oracle.distance_transform(m)
    queue = oracle.distance_queue(m)
    assert (queue >= exact).all()
    assert (queue == exact).mean() > 0.99
    assert (queue[m == 0] == 0).all()
