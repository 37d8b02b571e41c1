"""The allocation-free reconstruction entry point (nsgb_imreconstruct_noalloc).

It is for callers that cannot allocate device memory -- a plugin inside a framework that owns
the whole GPU memory pool, a real-time loop that forbids allocation once running, a
foreign-language host that only receives device buffers -- so it takes no workspace and uses
a fixed scratch array inside the library instead.  These tests call it through the C ABI and
compare it with the workspace entry point (nsgb_imreconstruct) on the same inputs, bit for bit
(the tolerance of all integer and min/max work in this library), on consecutive calls.  The
file sorts last so that a run stopping at the first failure has already run everything else.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _both(nsgb, marker, mask, conn, erode=False):
    import torch
    from nsgb import _ffi

    code = {np.dtype(np.uint8): 0, np.dtype(np.uint16): 1, np.dtype(np.int32): 2, np.dtype(np.float32): 3}[mask.dtype]
    m = torch.from_numpy(mask).cuda()
    ref = torch.from_numpy(marker).cuda()
    out = torch.from_numpy(marker).cuda()
    rows, cols = mask.shape
    pitch = cols * mask.itemsize
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    nb = _ffi.lib.nsgb_workspace_size(_ffi.OP_IMRECONSTRUCT, code, rows, cols)
    ws = torch.empty(nb + 256, dtype=torch.uint8, device="cuda")
    wsp = (ws.data_ptr() + 255) & ~255
    st = _ffi.lib.nsgb_imreconstruct(code, ref.data_ptr(), m.data_ptr(), rows, cols, pitch, conn, int(erode), wsp, nb,
                                     stream, None)
    assert st == 0
    st = _ffi.lib.nsgb_imreconstruct_noalloc(code, out.data_ptr(), m.data_ptr(), rows, cols, pitch, conn,
                                             int(erode), stream, None)
    assert st == 0
    return ref.cpu().numpy(), out.cpu().numpy()


def test_noalloc_matches_workspace_entry_point_on_consecutive_calls(nsgb):
    from nsgb import synth

    rng = np.random.default_rng(11)
    mask8, marker8 = synth.tile_u8(1024, 1024, 400, 0)
    cases = [
        (marker8, mask8, 8, False),                                                   # config-0 tile
        (rng.integers(-3000, 3000, (300, 517)).astype(np.int32),
         rng.integers(-3000, 3000, (300, 517)).astype(np.int32), 4, False),          # different size / dtype
        (marker8, mask8, 8, False),                                                   # the first input again
        (rng.random((257, 130)).astype(np.float32), rng.random((257, 130)).astype(np.float32), 8, True),
    ]
    for marker, mask, conn, erode in cases:
        ref, out = _both(nsgb, marker, mask, conn, erode)
        assert np.array_equal(out, ref)


def test_noalloc_refuses_images_beyond_its_scratch(nsgb):
    from nsgb import _ffi

    # 16384 x 16384 u8 needs 131072 tiles, above the built-in scratch: refused before any GPU work.
    assert _ffi.lib.nsgb_workspace_size(_ffi.OP_IMRECONSTRUCT, 0, 16384, 16384) > _ffi.NOALLOC_SCRATCH_BYTES
    st = _ffi.lib.nsgb_imreconstruct_noalloc(0, 256, 256, 16384, 16384, 16384, 8, 0, None, None)
    assert st == 3  # NSGB_ERR_WORKSPACE


def test_noalloc_async_status_is_read_back(nsgb):
    """With opts->sync == 0 the call returns once enqueued; its device status is read from the
    built-in scratch with nsgb_noalloc_device_status.  A one-sweep budget on an input that needs
    more ends NOT_CONVERGED there; the next call, with the default budget, is bit-exact against
    the workspace entry point."""
    import torch
    from nsgb import _ffi, synth

    mask, marker = synth.tile_u8(512, 512, 60, 2)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    out = torch.from_numpy(marker).cuda()
    m = torch.from_numpy(mask).cuda()
    opts = _ffi.Opts(0, 0, 1)  # sync = 0, max_visit_iters = 1
    st = _ffi.lib.nsgb_imreconstruct_noalloc(0, out.data_ptr(), m.data_ptr(), 512, 512, 512, 8, 0, stream,
                                             C.byref(opts))
    assert st == 0
    assert _ffi.lib.nsgb_noalloc_device_status(stream) == 4  # NSGB_ERR_NOT_CONVERGED
    ref, got = _both(nsgb, marker, mask, 8)
    assert np.array_equal(got, ref)
    assert _ffi.lib.nsgb_noalloc_device_status(stream) == 0
