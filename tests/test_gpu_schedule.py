"""The reconstruction's schedule knobs change the order of work, never the result: streaming
passes before the work queue (on the tile grid and the half-tile-shifted grid, whose edge tiles
are partial), the initial ring order, and the number of queue CTAs per SM.  Every combination
is compared bit for bit with the oracle (and, for batches, tile by tile), on odd, one-pixel-wide
and pitched shapes, all dtypes, dilation and erosion."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = {np.dtype(np.uint8): 0, np.dtype(np.uint16): 1, np.dtype(np.int32): 2, np.dtype(np.float32): 3}
SCHEDULES = [(-1, 1, 0), (1, 0, 0), (2, 0, 0), (3, 0, 2), (4, 0, 1), (-1, 3, 3), (-1, 2, 1), (5, 0, 0)]


def gray(rng, shape, dtype):
    if dtype == np.float32:
        return (rng.random(shape, dtype=np.float32) - 0.2).astype(np.float32)
    if dtype == np.int32:
        return rng.integers(-5000, 5000, shape).astype(np.int32)
    hi = np.iinfo(dtype).max
    base = rng.integers(hi // 2, hi, shape)
    return np.where(rng.random(shape) < 0.25, rng.integers(0, hi // 3, shape), base).astype(dtype)


def run(marker, mask, conn, erode, sched, pitch_extra=0):
    import torch

    from nsgb import _ffi

    lib = _ffi.lib
    passes, order, ctas = sched
    code = DT[mask.dtype]
    H, W = mask.shape
    esz = mask.itemsize
    pw = W + pitch_extra
    # planes staged as bytes (rows padded to the pitch), so that every dtype is handled alike
    mk = torch.zeros((H, pw * esz), dtype=torch.uint8, device="cuda")
    ms = torch.zeros_like(mk)
    mk[:, :W * esz] = torch.from_numpy(np.ascontiguousarray(marker).view(np.uint8).reshape(H, W * esz)).cuda()
    ms[:, :W * esz] = torch.from_numpy(np.ascontiguousarray(mask).view(np.uint8).reshape(H, W * esz)).cuda()
    nb = lib.nsgb_workspace_size(_ffi.OP_IMRECONSTRUCT, code, H, W)
    ws_t = torch.empty(nb + 256, dtype=torch.uint8, device="cuda")
    ws = (ws_t.data_ptr() + 255) & ~255
    o = _ffi.Opts(1, 0, 0, 0, passes, order, ctas)
    st = lib.nsgb_imreconstruct(code, mk.data_ptr(), ms.data_ptr(), H, W, pw * esz, conn, int(erode), ws, nb,
                                C.c_void_p(torch.cuda.current_stream().cuda_stream), C.byref(o))
    assert st == 0, _ffi.STATUS.get(st, st)
    return np.ascontiguousarray(mk[:, :W * esz].cpu().numpy()).view(mask.dtype).reshape(H, W)


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.int32, np.float32])
@pytest.mark.parametrize("conn", [4, 8])
@pytest.mark.parametrize("shape", [(1, 1), (1, 130), (97, 1), (31, 65), (200, 333), (257, 129)])
def test_schedules_dilation_match_oracle(nsgb, oracle, dtype, conn, shape):
    rng = np.random.default_rng(hash((shape, conn)) % 1000)
    mask = gray(rng, shape, dtype)
    marker = (mask - (rng.random(shape) * 40).astype(mask.dtype)) if dtype != np.float32 else \
        (mask * rng.uniform(0.3, 1.0, shape)).astype(np.float32)
    if dtype in (np.uint8, np.uint16):
        marker = np.minimum(marker, mask)
    exp = oracle.imreconstruct(marker, mask, conn)
    for sched in SCHEDULES:
        got = run(marker, mask, conn, False, sched, pitch_extra=3 if shape[1] > 1 else 0)
        assert got.tobytes() == exp.tobytes(), sched


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.int32])
@pytest.mark.parametrize("conn", [4, 8])
def test_schedules_erosion_match_reference_fill(nsgb, oracle, dtype, conn):
    """Erosion from the border (hole filling) under every schedule equals the grayscale fill."""
    import torch

    from nsgb import synth

    m8, _ = synth.tile_u8(300, 517, 40, 9)
    img = m8 if dtype == np.uint8 else synth.scale(m8, "u16" if dtype == np.uint16 else "i32")[0]
    exp = oracle.imfill_holes(img, False, conn)
    mx = np.iinfo(dtype).max
    marker = np.full_like(img, mx)
    marker[0, :], marker[-1, :], marker[:, 0], marker[:, -1] = img[0, :], img[-1, :], img[:, 0], img[:, -1]
    for sched in SCHEDULES:
        got = run(marker, img, conn, True, sched)
        assert got.tobytes() == exp.tobytes(), sched
    # the library's own fill under a schedule set through the options
    from nsgb import _ffi

    lib = _ffi.lib
    d = torch.from_numpy(img).cuda()
    out = torch.empty_like(d)
    nb = lib.nsgb_workspace_size(_ffi.OP_FILL_HOLES, DT[img.dtype], *img.shape)
    ws_t = torch.empty(nb + 256, dtype=torch.uint8, device="cuda")
    ws = (ws_t.data_ptr() + 255) & ~255
    for sched in SCHEDULES[:4]:
        o = _ffi.Opts(1, 0, 0, 0, *sched)
        st = lib.nsgb_imfill_holes(DT[img.dtype], d.data_ptr(), out.data_ptr(), img.shape[0], img.shape[1],
                                   img.shape[1] * img.itemsize, 0, conn, ws, nb,
                                   C.c_void_p(torch.cuda.current_stream().cuda_stream), C.byref(o))
        assert st == 0 and out.cpu().numpy().tobytes() == exp.tobytes(), sched


@pytest.mark.parametrize("dtype", ["u8", "i32"])
def test_schedules_batch_match_single_tiles(nsgb, oracle, dtype):
    import torch

    from nsgb import _ffi, synth

    sizes = [(256, 300), (33, 65), (1, 97), (97, 1), (300, 256), (129, 31), (2, 2), (200, 700)]
    tiles = []
    for k, (h, w) in enumerate(sizes):
        m8, k8 = synth.tile_u8(h, w, synth.ellipses_for(h, w), 60 + k)
        tiles.append((m8, k8) if dtype == "u8" else synth.scale(m8, dtype))
    exps = [oracle.imreconstruct(k, m, 8) for m, k in tiles]
    code = {"u8": 0, "i32": 2}[dtype]
    lib = _ffi.lib
    for sched in SCHEDULES:
        markers = [torch.from_numpy(k).cuda() for _, k in tiles]
        masks = [torch.from_numpy(m).cuda() for m, _ in tiles]
        desc = (_ffi.Tile * len(tiles))()
        for i, (mk, ms) in enumerate(zip(markers, masks)):
            desc[i] = _ffi.Tile(mk.data_ptr(), ms.data_ptr(), ms.shape[0], ms.shape[1], ms.shape[1] * ms.element_size(),
                                None, None, None)
        nb = lib.nsgb_batch_workspace_size(code, desc, len(tiles))
        ws_t = torch.empty(nb + 256, dtype=torch.uint8, device="cuda")
        ws = (ws_t.data_ptr() + 255) & ~255
        batch = _ffi.Batch()
        assert lib.nsgb_batch_prepare(code, desc, len(tiles), ws, nb, C.byref(batch)) == 0
        o = _ffi.Opts(1, 0, 0, 0, *sched)
        st = lib.nsgb_imreconstruct_batch(C.byref(batch), 8, 0, C.c_void_p(torch.cuda.current_stream().cuda_stream),
                                          C.byref(o))
        assert st == 0, sched
        for mk, e in zip(markers, exps):
            assert mk.cpu().numpy().tobytes() == e.tobytes(), sched


def test_pass_visits_count_towards_the_budget(nsgb):
    """A one-visit-per-tile budget is exhausted by the streaming passes alone."""
    import torch

    from nsgb import _ffi, synth

    mask, marker = synth.tile_u8(512, 512, 60, 2)
    lib = _ffi.lib
    mk = torch.from_numpy(marker).cuda()
    ms = torch.from_numpy(mask).cuda()
    nb = lib.nsgb_workspace_size(0, 0, 512, 512)
    ws_t = torch.empty(nb + 256, dtype=torch.uint8, device="cuda")
    ws = (ws_t.data_ptr() + 255) & ~255
    o = _ffi.Opts(1, 1, 0, 0, 3, 0, 0)
    st = lib.nsgb_imreconstruct(0, mk.data_ptr(), ms.data_ptr(), 512, 512, 512, 8, 0, ws, nb,
                                C.c_void_p(torch.cuda.current_stream().cuda_stream), C.byref(o))
    assert st == 4  # NSGB_ERR_NOT_CONVERGED
