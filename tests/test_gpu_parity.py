"""GPU parity: every operation of the device library against the CPU oracle, bit-exact.

Integer / byte / index work must match exactly; the float reconstruction only selects among
input values (min / max), so it must match exactly too.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (1, 100), (100, 1), (3, 5), (31, 33), (32, 64), (33, 65), (65, 130), (100, 257), (257, 100),
          (96, 200)]
DTYPES = [np.uint8, np.uint16, np.int32, np.float32]


def to_dev(a):
    import torch

    t = torch.from_numpy(np.ascontiguousarray(a))
    return t.cuda()


def to_np(t):
    return t.cpu().numpy()


def rand_gray(rng, h, w, dtype, levels=7, negative=False):
    if dtype == np.float32:
        a = rng.random((h, w)).astype(np.float32)
        return (a - 0.5).astype(np.float32) if negative else a
    base = rng.integers(0, levels, (h, w))
    if dtype == np.uint8:
        return (base * 37).astype(np.uint8)
    if dtype == np.uint16:
        return (base * 9001).astype(np.uint16)
    return (base * 1000 - (3000 if negative else 0)).astype(np.int32)


def smooth_gray(rng, h, w, dtype):
    """Larger plateaus, long propagation paths."""
    import scipy.ndimage as ndi

    a = ndi.gaussian_filter(rng.random((h, w)), 3)
    a = (a - a.min()) / max(a.max() - a.min(), 1e-9)
    if dtype == np.float32:
        return a.astype(np.float32)
    if dtype == np.uint8:
        return (a * 255).astype(np.uint8)
    if dtype == np.uint16:
        return (a * 65535).astype(np.uint16)
    return (a * 1e6).astype(np.int32)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("conn", [4, 8])
def test_recon_random(nsgb, oracle, dtype, conn):
    rng = np.random.default_rng(100 + conn)
    for (h, w) in SHAPES:
        for kind in range(3):
            if kind == 0:
                mask = rand_gray(rng, h, w, dtype, negative=True)
                marker = rand_gray(rng, h, w, dtype, negative=True)
            elif kind == 1:
                mask = smooth_gray(rng, h, w, dtype)
                marker = np.zeros_like(mask)
                marker[rng.integers(0, h), rng.integers(0, w)] = mask.max()
            else:
                mask = smooth_gray(rng, h, w, dtype)
                marker = rand_gray(rng, h, w, dtype)
            got = to_np(nsgb.imreconstruct(to_dev(marker), to_dev(mask), conn))
            exp = oracle.imreconstruct(marker, mask, conn)
            assert np.array_equal(got, exp), (dtype, conn, h, w, kind, int((got != exp).sum()))


def _np_erode_dual(marker, mask, conn):
    # Erosion reconstruction without a padding ring, as the order-reversed dilation.
    if mask.dtype == np.float32:
        flip = lambda a: (-a).astype(np.float32)  # noqa: E731
    elif mask.dtype == np.int32:
        flip = lambda a: ~a  # noqa: E731
    else:
        mx = np.iinfo(mask.dtype).max
        flip = lambda a: (mx - a).astype(mask.dtype)  # noqa: E731
    from test_oracle_cpu import np_recon

    return flip(np_recon(flip(marker), flip(mask), conn, ring=False))


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("conn", [4, 8])
def test_recon_erode(nsgb, dtype, conn):
    rng = np.random.default_rng(7)
    for (h, w) in [(1, 7), (9, 5), (31, 33), (40, 70)]:
        mask = rand_gray(rng, h, w, dtype, negative=True)
        marker = rand_gray(rng, h, w, dtype, negative=True)
        got = to_np(nsgb.imreconstruct(to_dev(marker), to_dev(mask), conn, erode=True))
        assert np.array_equal(got, _np_erode_dual(marker, mask, conn)), (dtype, conn, h, w)


def test_recon_reference_fixture(nsgb, golden_dir):
    d = np.load(os.path.join(golden_dir, "ref_fixture_32.npz"))
    image = d["image"].astype(np.int32)
    seeds = d["seeds"].astype(np.int32)
    for conn in (4, 8):
        got = to_np(nsgb.imreconstruct(to_dev(seeds), to_dev(image), conn))
        assert np.array_equal(got, d[f"expected{conn}"])


def test_recon_pitched_and_inplace(nsgb, oracle):
    import ctypes as C

    import torch
    from nsgb import _ffi

    rng = np.random.default_rng(1)
    h, w = 77, 150
    mask = smooth_gray(rng, h, w, np.uint8)
    marker = rand_gray(rng, h, w, np.uint8)
    exp = oracle.imreconstruct(marker, mask, 8)
    big_m = torch.zeros((h, w + 13), dtype=torch.uint8, device="cuda")
    big_k = torch.zeros((h, w + 13), dtype=torch.uint8, device="cuda")
    big_m[:, :w] = to_dev(mask)
    big_k[:, :w] = to_dev(marker)
    m, k = big_m[:, :w], big_k[:, :w]
    ws = torch.empty(_ffi.lib.nsgb_workspace_size(0, 0, h, w) + 256, dtype=torch.uint8, device="cuda")
    wsp = (ws.data_ptr() + 255) & ~255
    st = _ffi.lib.nsgb_imreconstruct(0, k.data_ptr(), m.data_ptr(), h, w, (w + 13), 8, 0, wsp, ws.numel() - 256,
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream), None)
    assert st == 0
    assert np.array_equal(to_np(k), exp)
    assert (to_np(big_k[:, w:]) == 0).all()


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.int32])
def test_synthetic_tiles(nsgb, oracle, dtype):
    from nsgb import synth

    for (H, W, n, seed) in [(1024, 1024, 400, 0), (300, 517, 55, 3), (257, 4096, 376, 9)]:
        m8, k8 = synth.tile_u8(H, W, n, seed)
        if dtype == np.uint8:
            mask, marker = m8, k8
        else:
            mask, marker = synth.scale(m8, "u16" if dtype == np.uint16 else "i32")
        for conn in (4, 8):
            got = to_np(nsgb.imreconstruct(to_dev(marker), to_dev(mask), conn))
            assert np.array_equal(got, oracle.imreconstruct(marker, mask, conn)), (H, W, conn)


def test_synthetic_4096(nsgb, oracle):
    from nsgb import synth

    mask, marker = synth.tile_u8(4096, 4096, 6000, 0)
    got = to_np(nsgb.imreconstruct(to_dev(marker), to_dev(mask), 8))
    assert np.array_equal(got, oracle.imreconstruct(marker, mask, 8))


def test_float_recon_tie_free(nsgb, oracle):
    from nsgb import synth

    mask, marker = synth.float_pair((512, 384), 0)
    for conn in (4, 8):
        got = to_np(nsgb.imreconstruct(to_dev(marker), to_dev(mask), conn))
        assert np.array_equal(got, oracle.imreconstruct(marker, mask, conn))


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.int32])
@pytest.mark.parametrize("conn", [4, 8])
def test_binary_recon_bwselect(nsgb, oracle, dtype, conn):
    rng = np.random.default_rng(3)
    mx = np.iinfo(dtype).max
    for (h, w) in SHAPES + [(300, 301)]:
        mask = (rng.random((h, w)) < 0.55).astype(dtype) * mx
        marker = (rng.random((h, w)) < 0.05).astype(dtype) * 5
        got = to_np(nsgb.imreconstructBinary(to_dev(marker), to_dev(mask), conn))
        assert np.array_equal(got, oracle.imreconstruct_binary(marker, mask, conn)), (h, w)
        seeds = (rng.random((h, w)) < 0.02).astype(dtype)
        got = to_np(nsgb.bwselect(to_dev(mask), to_dev(seeds), conn))
        assert np.array_equal(got, oracle.bwselect(mask, seeds, conn)), (h, w)


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.int32, np.float32])
@pytest.mark.parametrize("conn", [4, 8])
def test_fill_holes(nsgb, oracle, dtype, conn):
    rng = np.random.default_rng(5)
    for (h, w) in SHAPES + [(200, 333)]:
        if dtype != np.float32:
            mx = np.iinfo(dtype).max
            img = (rng.random((h, w)) < 0.5).astype(dtype) * mx
            got = to_np(nsgb.imfillHoles(to_dev(img), True, conn))
            assert np.array_equal(got, oracle.imfill_holes(img, True, conn)), ("bin", h, w)
        img = smooth_gray(rng, h, w, dtype)
        got = to_np(nsgb.imfillHoles(to_dev(img), False, conn))
        assert np.array_equal(got, oracle.imfill_holes(img, False, conn)), ("gray", h, w)


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.float32])
def test_hmin(nsgb, oracle, dtype):
    rng = np.random.default_rng(8)
    for (h, w) in SHAPES:
        img = smooth_gray(rng, h, w, dtype)
        hv = {np.uint8: 20, np.uint16: 3000, np.float32: 0.1}[dtype]
        for conn in (4, 8):
            got = to_np(nsgb.imhmin(to_dev(img), hv, conn))
            assert np.array_equal(got, oracle.imhmin(img, hv, conn)), (h, w, conn)


@pytest.mark.parametrize("conn", [4, 8])
def test_bwlabel_matches_reference_fixtures(nsgb, golden_dir, conn):
    d = np.load(os.path.join(golden_dir, "ref_ccl_cases.npz"))
    k = 0
    while f"img{k}" in d:
        img = d[f"img{k}"]
        lab = to_np(nsgb.bwlabel2(to_dev(img), conn, False))
        assert np.array_equal(lab, d[f"lab{k}_{conn}"]), k
        rel, n = nsgb.bwlabel2_count(to_dev(img), conn)
        assert np.array_equal(to_np(rel), d[f"rel{k}_{conn}"]) and n == int(d[f"n{k}_{conn}"]), k
        kept, nk = nsgb.bwareaopen2(to_dev(d[f"lab{k}_{conn}"]), True, False, 3, 40, conn)
        assert np.array_equal(to_np(kept), d[f"kept{k}_{conn}"]) and nk == int(d[f"nk{k}_{conn}"]), k
        k += 1


@pytest.mark.parametrize("conn", [4, 8])
def test_bwlabel_bwareaopen_random(nsgb, oracle, conn):
    rng = np.random.default_rng(2)
    for (h, w) in SHAPES + [(513, 1000), (1024, 1024)]:
        for p in (0.3, 0.6):
            img = ((rng.random((h, w)) < p) * rng.integers(1, 3, (h, w)) * 100).astype(np.uint8)
            got, n = nsgb.bwlabel2_count(to_dev(img), conn)
            exp, m = oracle.bwlabel2(img, conn, True)
            assert n == m and np.array_equal(to_np(got), exp), (h, w, p)
            got = to_np(nsgb.bwlabel2(to_dev(img), conn, False))
            assert np.array_equal(got, oracle.bwlabel2(img, conn, False)[0])
            for flatten in (True, False):
                got, c = nsgb.bwareaopen2(to_dev(img), False, flatten, 3, 50, conn)
                exp, ce = oracle.bwareaopen2(img, False, flatten, 3, 50, conn)
                assert c == ce and np.array_equal(to_np(got), exp), (h, w, p, flatten)


def test_bounding_boxes_reference_fixtures(nsgb, golden_dir):
    """ConnComponents::boundingBox of the reference itself (raw root labels, raster labels, and
    raster labels with a stray -1 that ends the reference's scan)."""
    d = np.load(os.path.join(golden_dir, "ref_bbox_cases.npz"))
    k = 0
    while f"lab{k}" in d:
        got = to_np(nsgb.bounding_boxes(to_dev(d[f"lab{k}"]), int(d[f"bg{k}"])))
        assert np.array_equal(got, d[f"box{k}"]), k
        k += 1
    assert k >= 150


def test_bounding_boxes_random(nsgb, oracle):
    rng = np.random.default_rng(3)
    for (h, w) in SHAPES + [(513, 1000), (1024, 1024)]:
        for p in (0.2, 0.55, 0.9):
            img = ((rng.random((h, w)) < p) * 255).astype(np.uint8)
            rel, _ = oracle.bwlabel2(img, 8, True)
            assert np.array_equal(to_np(nsgb.bounding_boxes(to_dev(rel), 0)), oracle.bounding_box(rel, 0)), (h, w, p)
            raw, _ = oracle.bwlabel2(img, 4, False)
            assert np.array_equal(to_np(nsgb.bounding_boxes(to_dev(raw), -1)), oracle.bounding_box(raw, -1)), (h, w)
    # arbitrary label values in [1, n), repeated in separate places, and a background of 7
    lab = rng.integers(1, 60, (300, 200)).astype(np.int32)
    lab[rng.random(lab.shape) < 0.4] = 7
    assert np.array_equal(to_np(nsgb.bounding_boxes(to_dev(lab), 7)), oracle.bounding_box(lab, 7))


def test_bounding_boxes_capacity_retry(nsgb, oracle):
    """An output sized below the number of labels is redone at the reported count."""
    rng = np.random.default_rng(5)
    img = ((rng.random((300, 400)) < 0.3) * 255).astype(np.uint8)
    rel, n = oracle.bwlabel2(img, 8, True)
    assert n > 100
    exp = oracle.bounding_box(rel, 0)
    for cap in (1, 17, n - 1, n, n + 5):
        assert np.array_equal(to_np(nsgb.bounding_boxes(to_dev(rel), 0, capacity=cap)), exp), cap


def test_bounding_boxes_chain_labels(nsgb, oracle):
    """The boxes of the chain's labelled output (HistologicalEntities.cpp:573 takes them after
    bwlabel2), on the inverted workload with thousands of components."""
    from nsgb import synth

    mask, marker = synth.tile_u8(2048, 2048, 1500, 4)
    inv_mask = (255 - mask).astype(np.uint8)
    inv_marker = np.maximum(inv_mask.astype(int) - 10, 0).astype(np.uint8)
    got = nsgb.chain(to_dev(inv_marker), to_dev(inv_mask), thr=128)
    labels = got["labels"]
    box = to_np(nsgb.bounding_boxes(labels, 0))
    exp = oracle.bounding_box(to_np(labels), 0)
    assert box.shape[1] == got["n_labels"] > 100
    assert np.array_equal(box, exp)


def test_bounding_boxes_bad_labels(nsgb):
    lab = np.zeros((16, 16), np.int32)
    lab[3, 4] = 16 * 16 + 1  # outside [-1, rows*cols]
    with pytest.raises(nsgb.NsgbError):
        nsgb.bounding_boxes(to_dev(lab), 0)
    lab[3, 4] = -5
    with pytest.raises(nsgb.NsgbError):
        nsgb.bounding_boxes(to_dev(lab), 0)


def test_threshold_invert(nsgb, oracle):
    rng = np.random.default_rng(0)
    for dtype in DTYPES:
        img = rand_gray(rng, 37, 53, dtype, negative=True)
        for thr in (-1.0, 0.0, 74.0, 0.25, 128.5):
            got = to_np(nsgb.threshold(to_dev(img), thr))
            assert np.array_equal(got, oracle.threshold_gt(img, thr)), (dtype, thr)
        inv = to_np(nsgb.invert(to_dev(img)))
        if dtype == np.float32:
            assert np.array_equal(inv, -img)
        elif dtype == np.int32:
            assert np.array_equal(inv, -img)
        else:
            assert np.array_equal(inv, np.iinfo(dtype).max - img)


@pytest.mark.parametrize("size,n", [(1024, 400), (4096, 6000)])
def test_chain(nsgb, oracle, size, n):
    from nsgb import synth

    mask, marker = synth.tile_u8(size, size, n, 0)
    got = nsgb.chain(to_dev(marker), to_dev(mask))
    exp = oracle.chain(marker, mask)
    assert np.array_equal(to_np(got["recon"]), exp["recon"])
    assert np.array_equal(to_np(got["fill"]), exp["fill"])
    assert np.array_equal(to_np(got["labels"]), exp["labels"])
    assert got["n_labels"] == exp["n_labels"]
    assert np.array_equal(to_np(got["area"]), exp["area"])
    assert got["n_kept"] == exp["n_kept"]


def test_chain_in_cuda_graph_with_timing_events(nsgb, oracle):
    """nsgb_chain captured into a CUDA graph and replayed: the results match the oracle on every
    replay, and the reconstruction's timing events (recorded by event-record nodes of the
    graph) give a positive time on each replay."""
    import ctypes as C

    import torch
    from nsgb import _ffi, synth

    lib = _ffi.lib
    H, W = 300, 500
    mask_h, marker_h = synth.tile_u8(H, W, 60, 3)
    exp = oracle.chain(marker_h, mask_h)
    mask, marker0 = to_dev(mask_h), to_dev(marker_h)
    work = marker0.clone()
    fill = torch.empty_like(mask)
    labels = torch.empty((H, W), dtype=torch.int32, device="cuda")
    area = torch.empty_like(mask)
    nb = lib.nsgb_workspace_size(_ffi.OP_CHAIN, _ffi.U8, H, W)
    wst = torch.empty(nb + 256, dtype=torch.uint8, device="cuda")
    ws = (wst.data_ptr() + 255) & ~255
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    ev1.record()
    opts = _ffi.Opts(0, 0, 0)
    opts.recon_event_begin = C.c_void_p(ev0.cuda_event)
    opts.recon_event_end = C.c_void_p(ev1.cuda_event)
    cs = torch.cuda.Stream()

    def call(stream):
        st = lib.nsgb_chain(_ffi.U8, work.data_ptr(), mask.data_ptr(), H, W, W, 8, 128.0, 4, 8, 11, 1000,
                            fill.data_ptr(), labels.data_ptr(), area.data_ptr(), None, None, ws, nb,
                            C.c_void_p(stream.cuda_stream), C.byref(opts))
        assert st == 0

    torch.cuda.synchronize()
    with torch.cuda.stream(cs):
        call(cs)  # warm-up outside the capture (first-call set-up)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=cs):
        call(cs)
    for _ in range(3):
        work.copy_(marker0)
        g.replay()
        torch.cuda.synchronize()
        assert ev0.elapsed_time(ev1) > 0
        assert np.array_equal(to_np(work), exp["recon"])
        assert np.array_equal(to_np(fill), exp["fill"])
        assert np.array_equal(to_np(labels), exp["labels"])
        assert np.array_equal(to_np(area), exp["area"])
    assert lib.nsgb_device_status(C.c_void_p(ws), None) == 0


@pytest.mark.parametrize("fill_conn,label_conn", [(4, 8), (8, 4)])
def test_chain_pitched_inputs(nsgb, oracle, fill_conn, label_conn):
    """nsgb_chain through the C ABI on marker and mask rows with padding (pitch > cols, odd
    sizes), the one-labelling fill of both dual connectivity pairs, against the oracle; the
    padding bytes stay untouched and the counts come back through the host pointers."""
    import ctypes as C

    import torch
    from nsgb import _ffi, synth

    lib = _ffi.lib
    H, W, pad = 157, 301, 19
    mask_h, marker_h = synth.tile_u8(H, W, 25, 5)
    exp = oracle.chain(marker_h, mask_h, fill_conn=fill_conn, label_conn=label_conn)
    big_k = torch.full((H, W + pad), 7, dtype=torch.uint8, device="cuda")
    big_m = torch.full((H, W + pad), 9, dtype=torch.uint8, device="cuda")
    big_k[:, :W] = to_dev(marker_h)
    big_m[:, :W] = to_dev(mask_h)
    fill = torch.empty((H, W), dtype=torch.uint8, device="cuda")
    labels = torch.empty((H, W), dtype=torch.int32, device="cuda")
    area = torch.empty((H, W), dtype=torch.uint8, device="cuda")
    nb = lib.nsgb_workspace_size(_ffi.OP_CHAIN, _ffi.U8, H, W)
    wst = torch.empty(nb + 256, dtype=torch.uint8, device="cuda")
    ws = (wst.data_ptr() + 255) & ~255
    nl, nk = C.c_int32(-1), C.c_int32(-1)
    st = lib.nsgb_chain(_ffi.U8, big_k.data_ptr(), big_m.data_ptr(), H, W, W + pad, 8, 128.0, fill_conn, label_conn,
                        11, 1000, fill.data_ptr(), labels.data_ptr(), area.data_ptr(), C.byref(nl), C.byref(nk), ws,
                        nb, C.c_void_p(torch.cuda.current_stream().cuda_stream), None)
    assert st == 0
    assert np.array_equal(to_np(big_k[:, :W]), exp["recon"])
    assert np.array_equal(to_np(fill), exp["fill"])
    assert np.array_equal(to_np(labels), exp["labels"])
    assert np.array_equal(to_np(area), exp["area"])
    assert nl.value == exp["n_labels"] and nk.value == exp["n_kept"]
    assert (to_np(big_k[:, W:]) == 7).all() and (to_np(big_m[:, W:]) == 9).all()


def _nested_rings(H, W, seed):
    """Concentric rectangular rings of alternating brightness around random centres, with random
    gaps cut into some rings: components enclosed by components several levels deep."""
    rng = np.random.default_rng(seed)
    img = np.full((H, W), 200, np.uint8)
    yy, xx = np.mgrid[0:H, 0:W]
    for _ in range(max(1, H * W // 600)):
        cy, cx = rng.integers(0, H), rng.integers(0, W)
        d = np.maximum(np.abs(yy - cy), np.abs(xx - cx))
        for r in range(int(rng.integers(2, 14)), 0, -1):
            ring = d == r
            if rng.random() < 0.3:  # a gap
                ring &= ~((yy == cy) & (xx > cx))
            img[ring] = 40 if r % 2 else 220
    return img


@pytest.mark.parametrize("fill_conn,label_conn", [(4, 8), (8, 4), (4, 4), (8, 8)])
def test_chain_hole_fill_and_labels_nested(nsgb, oracle, fill_conn, label_conn):
    """The single-image chain's hole fill and labelling on inputs built to stress the enclosure
    tree (nested rings with gaps, salt-and-pepper noise around the threshold), widths and heights
    around the 32-pixel labelling tiles, one-pixel images, three dtypes and every pair of fill /
    label connectivities, against the oracle.  The marker equals the mask, so the
    reconstruction is the image itself and the threshold splits it directly."""
    rng = np.random.default_rng(11)
    sizes = [(1, 1), (1, 40), (40, 1), (2, 2), (31, 33), (33, 31), (64, 64), (65, 97), (200, 300), (257, 1100)]
    for i, (h, w) in enumerate(sizes):
        base = _nested_rings(h, w, i)
        noise = np.where(rng.random((h, w)) < 0.5, 60, 190).astype(np.uint8)
        for img8 in (base, noise, (255 - base).astype(np.uint8)):
            for dt, scale in ((np.uint8, 1), (np.uint16, 257), (np.int32, -1000)):
                img = img8.astype(np.int64) * scale
                img = img.astype(dt)
                thr = 128 * scale if scale > 0 else -128000.5
                got = nsgb.chain(to_dev(img), to_dev(img), thr=thr, fill_conn=fill_conn, label_conn=label_conn)
                exp = oracle.chain(img, img, thr=thr, fill_conn=fill_conn, label_conn=label_conn)
                ctx = (h, w, dt.__name__, fill_conn, label_conn)
                assert np.array_equal(to_np(got["fill"]), exp["fill"]), ctx
                assert np.array_equal(to_np(got["labels"]), exp["labels"]), ctx
                assert np.array_equal(to_np(got["area"]), exp["area"]), ctx
                assert got["n_labels"] == exp["n_labels"] and got["n_kept"] == exp["n_kept"], ctx


def test_chain_inverted_workload(nsgb, oracle):
    """The same chain on the inverted reconstruction: dark nuclei as foreground, thousands of
    components, so labelling and the area filter do real work."""
    from nsgb import synth

    mask, marker = synth.tile_u8(2048, 2048, 1500, 4)
    inv_mask = (255 - mask).astype(np.uint8)
    inv_marker = np.maximum(inv_mask.astype(int) - 10, 0).astype(np.uint8)
    got = nsgb.chain(to_dev(inv_marker), to_dev(inv_mask), thr=128)
    exp = oracle.chain(inv_marker, inv_mask, thr=128)
    assert got["n_labels"] == exp["n_labels"] and exp["n_labels"] > 100
    assert np.array_equal(to_np(got["labels"]), exp["labels"])
    assert np.array_equal(to_np(got["area"]), exp["area"]) and got["n_kept"] == exp["n_kept"]


def test_device_budgets_report_status(nsgb):
    """Failure detection without a fault: a one-visit-per-tile / one-sweep budget on an input
    that needs more returns NOT_CONVERGED through the status word; the context stays usable."""
    from nsgb import synth

    mask, marker = synth.tile_u8(512, 512, 60, 2)
    with pytest.raises(nsgb.NsgbError) as e:
        nsgb.imreconstruct(to_dev(marker), to_dev(mask), 8, max_visits_per_tile=1)
    assert e.value.status == 4
    with pytest.raises(nsgb.NsgbError) as e:
        nsgb.imreconstruct(to_dev(marker), to_dev(mask), 8, max_visit_iters=1)
    assert e.value.status == 4
    out = nsgb.imreconstruct(to_dev(marker), to_dev(mask), 8)  # still works afterwards
    assert out.shape == mask.shape


def test_queue_wait_timeout_reports_status(nsgb, oracle):
    """Failure detection of the queue waits without a fault: with a poll limit of a few polls,
    warps that wait for work on the tile queue (most of the grid, on a 128-tile image) give up
    and the call returns NSGB_ERR_TIMEOUT through the status word; the context stays usable and
    the next call with the default limit is bit-exact."""
    from nsgb import synth

    mask, marker = synth.tile_u8(512, 512, 60, 2)
    with pytest.raises(nsgb.NsgbError) as e:
        nsgb.imreconstruct(to_dev(marker), to_dev(mask), 8, queue_poll_limit=2)
    assert e.value.status == 5
    out = nsgb.imreconstruct(to_dev(marker), to_dev(mask), 8)
    assert np.array_equal(to_np(out), oracle.imreconstruct(marker, mask, 8))
