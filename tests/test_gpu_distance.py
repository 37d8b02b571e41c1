"""GPU parity of the distance transform (nsgb_distance_transform: the exact Euclidean map of
HistologicalEntities.cpp:341 and the watershed basins of :347-356) against the oracle,
bit-exact: blob masks, noise, a single zero pixel (distances across the whole image), masks
whose zeros sit in one 128-row chunk, rows on both sides of the row pass's switch between its
search and its envelope, one-pixel-wide images, a mask without zeros, pitched output, and the
full 4096 x 4096 tile."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def blobs(rng, h, w, n):
    m = np.zeros((h, w), np.uint8)
    yy, xx = np.mgrid[0:h, 0:w]
    for _ in range(n):
        cy, cx, r = rng.integers(0, h), rng.integers(0, w), rng.integers(2, 30)
        m[(yy - cy) ** 2 + (xx - cx) ** 2 <= r * r] = 255
    return m


def masks():
    rng = np.random.default_rng(4)
    out = {"blobs": blobs(rng, 300, 400, 60), "noise": np.where(rng.random((257, 129)) < 0.9, 1, 0).astype(np.uint8)}
    one = np.full((700, 500), 255, np.uint8)
    one[3, 497] = 0
    out["one_zero"] = one
    band = np.full((600, 333), 9, np.uint8)
    band[130:140:3, ::37] = 0  # zeros only inside the second 128-row chunk
    out["band"] = band
    out["row"] = np.where(rng.random((1, 1000)) < 0.97, 255, 0).astype(np.uint8)
    out["col"] = np.where(rng.random((1000, 1)) < 0.97, 255, 0).astype(np.uint8)
    out["pixel"] = np.zeros((1, 1), np.uint8)
    far = np.full((800, 300), 255, np.uint8)
    far[0, :] = 0  # rows near the zero row search along the row, the far ones take the divide and conquer
    far[0, 150] = 255
    out["far"] = far
    return out


@pytest.mark.parametrize("name", ["blobs", "noise", "one_zero", "band", "row", "col", "pixel", "far"])
@pytest.mark.parametrize("basins", [False, True])
def test_distance_parity(nsgb, oracle, name, basins):
    m = masks()[name]
    got = nsgb.distanceTransform(to_dev(m), basins=basins).cpu().numpy()
    assert np.array_equal(got, oracle.distance_transform(m, basins=basins))


def zero_free_masks():
    """Inputs whose rows take the divide and conquer (mean g above the search threshold): large
    objects, columns without any zero pixel, one zero pixel far away, and rows wider than its
    shared tables (the envelope fallback)."""
    rng = np.random.default_rng(21)
    out = {}
    big = np.zeros((1500, 1700), np.uint8)
    yy, xx = np.mgrid[0:1500, 0:1700]
    for cy, cx, r in ((700, 800, 600), (200, 200, 150), (1300, 1500, 180)):
        big[(yy - cy) ** 2 + (xx - cx) ** 2 <= r * r] = 255
    out["large_objects"] = big
    cols = np.full((900, 1100), 200, np.uint8)
    cols[rng.integers(0, 900, 40), rng.integers(0, 550, 40)] = 0  # zeros only in the left half
    out["zero_free_columns"] = cols
    single = np.full((1024, 1024), 1, np.uint8)
    single[1000, 3] = 0
    out["single_zero"] = single
    wide = np.full((40, 13000), 77, np.uint8)
    wide[rng.integers(0, 40, 6), rng.integers(0, 13000, 6)] = 0  # wider than the shared tables
    out["wide"] = wide
    ties = np.full((300, 301), 5, np.uint8)
    ties[::100, ::100] = 0  # equidistant zero pixels: ties between columns
    out["ties"] = ties
    return out


@pytest.mark.parametrize("name", ["large_objects", "zero_free_columns", "single_zero", "wide", "ties"])
def test_distance_zero_free_regions(nsgb, oracle, name):
    m = zero_free_masks()[name]
    for basins in (False, True):
        got = nsgb.distanceTransform(to_dev(m), basins=basins).cpu().numpy()
        assert np.array_equal(got, oracle.distance_transform(m, basins=basins)), basins


def test_distance_all_foreground_4096(nsgb, oracle):
    """An all-foreground 4096 x 4096 mask except one zero pixel: every row is far from the
    zero pixel; timed against the bench's blob tile (within 3x of it)."""
    import torch

    m = np.full((4096, 4096), 255, np.uint8)
    m[2048, 17] = 0
    d = to_dev(m)
    nsgb.distanceTransform(d)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    got = nsgb.distanceTransform(d)
    e1.record()
    torch.cuda.synchronize()
    print(f"all-foreground 4096^2 distance transform: {e0.elapsed_time(e1):.3f} ms")
    assert np.array_equal(got.cpu().numpy(), oracle.distance_transform(m))
    assert e0.elapsed_time(e1) < 0.51


def test_distance_without_zero(nsgb, oracle):
    m = np.full((130, 70), 255, np.uint8)
    d = nsgb.distanceTransform(to_dev(m)).cpu().numpy()
    assert np.array_equal(d, oracle.distance_transform(m)) and np.isinf(d).all()


def test_distance_pitched(nsgb, oracle):
    import torch

    from nsgb import _ffi

    lib = _ffi.lib
    rng = np.random.default_rng(8)
    H, W, PI = 333, 517, 523
    m = blobs(rng, H, W, 40)
    exp = oracle.distance_transform(m)
    src = torch.zeros((H, PI), dtype=torch.uint8, device="cuda")
    src[:, :W] = to_dev(m)
    dst = torch.full((H, W + 3), 7.0, dtype=torch.float32, device="cuda")
    nb = lib.nsgb_workspace_size(_ffi.OP_DISTANCE, _ffi.U8, H, W)
    ws_t = torch.empty(nb + 256, dtype=torch.uint8, device="cuda")
    ws = (ws_t.data_ptr() + 255) & ~255
    st = lib.nsgb_distance_transform(src.data_ptr(), dst.data_ptr(), H, W, PI, (W + 3) * 4, 0, ws, nb,
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream), None)
    assert st == 0
    assert np.array_equal(dst[:, :W].cpu().numpy(), exp)
    assert (dst[:, W:] == 7.0).all()


def test_distance_full_tile(nsgb, oracle):
    from nsgb import synth

    mask, _ = synth.tile_u8(4096, 4096, 6000, 0)
    m = np.where(mask < 128, 255, 0).astype(np.uint8)
    got = nsgb.distanceTransform(to_dev(m)).cpu().numpy()
    assert np.array_equal(got, oracle.distance_transform(m))
