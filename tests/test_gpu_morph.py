"""GPU parity of the opening (nsgb_morph_open, nscale::morphOpen<unsigned char>,
MorphologicOperations.cpp:2459-2493) against the oracle, bit-exact: the reference's two
elements (19 x 19 disk, 3 x 3 ellipse), other centred elements (fast path), off-centre and
ragged elements (direct path), the largest element, pitched and unaligned rows, a column image
taller than one grid's row of tiles, and strips of a full 4096 x 4096 tile."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def to_dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def disk(r):
    y, x = np.mgrid[-r:r + 1, -r:r + 1]
    return (x * x + y * y <= r * r).astype(np.uint8)


def elements():
    from nsgb import disk19, ellipse3

    rng = np.random.default_rng(5)
    ragged = (rng.random((7, 7)) < 0.35).astype(np.uint8)
    ragged[3, 3] = 0
    ragged[0, 6] = 1
    shifted = np.zeros((5, 5), np.uint8)
    shifted[0, 4] = 1  # a single pixel up and to the right: a pure shift
    diamond = (np.abs(np.mgrid[-3:4, -3:4]).sum(0) <= 3).astype(np.uint8)
    return {"disk19": disk19(), "ellipse3": ellipse3(), "rect5": np.ones((5, 5), np.uint8), "diamond7": diamond,
            "ragged7": ragged, "shift5": shifted, "disk63": disk(31), "hline9": np.pad(np.ones((1, 9), np.uint8),
                                                                                        ((4, 4), (0, 0)))}


@pytest.mark.parametrize("name", ["disk19", "ellipse3", "rect5", "diamond7", "ragged7", "shift5", "disk63", "hline9"])
@pytest.mark.parametrize("shape", [(1, 1), (1, 300), (300, 1), (37, 61), (64, 128), (65, 129), (129, 257),
                                   (700, 1100)])
def test_morph_open_elements(nsgb, oracle, name, shape):
    kern = elements()[name]
    if name == "disk63" and shape[0] * shape[1] > 100_000:
        shape = (250, 300)  # the oracle folds 3001 element pixels per pixel
    rng = np.random.default_rng(shape[0] * 1000 + shape[1])
    img = rng.integers(0, 256, shape).astype(np.uint8)
    if shape[0] * shape[1] > 1000:  # smoother content as well: plateaus and ramps
        img = np.where(rng.random(shape) < 0.5, img, (np.add.outer(np.arange(shape[0]), np.arange(shape[1])) % 256))
        img = img.astype(np.uint8)
    got = nsgb.morphOpen(to_dev(img), kern).cpu().numpy()
    assert np.array_equal(got, oracle.morph_open(img, kern))


def test_morph_open_synthetic_tile(nsgb, oracle):
    from nsgb import disk19, synth

    mask, _ = synth.tile_u8(1024, 1536, 540, 3)
    rc = (255 - mask).astype(np.uint8)
    got = nsgb.morphOpen(to_dev(rc), disk19()).cpu().numpy()
    assert np.array_equal(got, oracle.morph_open(rc, disk19()))


def test_morph_open_pitched_unaligned(nsgb, oracle):
    import torch

    from nsgb import _ffi, disk19

    lib = _ffi.lib
    H, W, PI, PO = 333, 517, 521, 530
    rng = np.random.default_rng(9)
    img = rng.integers(0, 256, (H, W)).astype(np.uint8)
    exp = oracle.morph_open(img, disk19())
    src = torch.zeros(H * PI + 3, dtype=torch.uint8, device="cuda")
    dst = torch.zeros(H * PO + 3, dtype=torch.uint8, device="cuda")
    src[1:1 + H * PI].view(H, PI)[:, :W] = to_dev(img)  # rows start at odd addresses
    nb = lib.nsgb_workspace_size(_ffi.OP_MORPH_OPEN, _ffi.U8, H, W)
    ws_t = torch.empty(nb + 256, dtype=torch.uint8, device="cuda")
    ws = (ws_t.data_ptr() + 255) & ~255
    k = np.ascontiguousarray(disk19())
    st = lib.nsgb_morph_open(src.data_ptr() + 1, dst.data_ptr() + 3, H, W, PI, PO, k.ctypes.data_as(C.c_void_p), 19,
                             ws, nb, C.c_void_p(torch.cuda.current_stream().cuda_stream), None)
    assert st == 0
    out = dst[3:3 + H * PO].view(H, PO)
    assert np.array_equal(out[:, :W].cpu().numpy(), exp)
    assert not out[:, W:].any() and not dst[:3].any()


def test_morph_open_tall_column(nsgb, oracle):
    """4.2 M rows: more 64-row tiles than one grid dimension holds, so tiles stride the grid."""
    from nsgb import ellipse3

    rng = np.random.default_rng(2)
    img = rng.integers(0, 256, (4_200_000, 1)).astype(np.uint8)
    got = nsgb.morphOpen(to_dev(img), ellipse3()).cpu().numpy()
    assert np.array_equal(got, oracle.morph_open(img, ellipse3()))


def test_morph_open_full_tile_strips(nsgb, oracle):
    """4096 x 4096 with the 19 x 19 disk: rows away from a strip's cut are exact, so the oracle
    runs on strips (top, middle, bottom) and the rows it fixes are compared."""
    from nsgb import disk19, synth

    mask, _ = synth.tile_u8(4096, 4096, 6000, 0)
    rc = (255 - mask).astype(np.uint8)
    got = nsgb.morphOpen(to_dev(rc), disk19()).cpu().numpy()
    reach = 18  # erosion then dilation, 9 rows each
    for a, b in [(0, 160), (2000, 2200), (3936, 4096)]:
        exp = oracle.morph_open(rc[a:b], disk19())
        lo = 0 if a == 0 else reach
        hi = (b - a) if b == 4096 else (b - a) - reach
        assert np.array_equal(got[a + lo:a + hi], exp[lo:hi]), (a, b)
