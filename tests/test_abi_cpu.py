"""CPU-only checks of the device library boundary: it loads without a GPU, exports every
entry point declared in include/*.h, and its host-only helpers behave."""
import ctypes
import glob
import os
import re

from conftest import ROOT

LIB = os.path.join(ROOT, "emory-cci-fast-ia-gsoc_gb300", "lib", "libnsgb.so")


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(nsgb_[a-z0-9_]+)\s*\(", txt):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(LIB)
    names = declared_symbols()
    assert len(names) >= 15
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_declares_every_symbol():
    import nsgb._ffi as ffi

    assert declared_symbols() <= set(ffi.EXPORTED) | {"nsgb_stream_t"}


def test_status_strings_and_workspace_sizes():
    import nsgb._ffi as ffi

    lib = ffi.lib
    assert lib.nsgb_status_string(0) == b"ok"
    assert b"workspace" in lib.nsgb_status_string(3)
    for op in range(12):
        for dt in range(4):
            assert lib.nsgb_workspace_size(op, dt, 64, 64) > 0
    assert lib.nsgb_workspace_size(12, 0, 64, 64) == 0
    # distance transform: column distances and the row pass's two stacks, 4 B/px each
    assert lib.nsgb_workspace_size(ffi.OP_DISTANCE, ffi.U8, 100, 130) >= 3 * 4 * 100 * 130
    # opening: the status word and the eroded image with rows padded to 128 bytes
    assert lib.nsgb_workspace_size(ffi.OP_MORPH_OPEN, ffi.U8, 100, 130) >= 256 + 100 * 256
    assert lib.nsgb_workspace_size(-1, 0, 64, 64) == 0
    # nucleus candidates: the chain's u8 workspace whatever dtype is asked for
    for dt in range(4):
        assert lib.nsgb_workspace_size(ffi.OP_NUCLEUS_CANDIDATES, dt, 300, 400) == \
            lib.nsgb_workspace_size(ffi.OP_CHAIN, ffi.U8, 300, 400)
    # bounding boxes: five per-label planes plus the bitmap and rank scratch
    assert lib.nsgb_workspace_size(ffi.OP_BOUNDING_BOX, ffi.I32, 4096, 4096) >= 5 * 4 * 4096 * 4096
    assert lib.nsgb_workspace_size(0, 0, 0, 10) == 0
    big = lib.nsgb_workspace_size(7, 0, 4096, 4096)
    assert big > 3 * 4 * 4096 * 4096


def test_argument_errors_need_no_gpu():
    import nsgb._ffi as ffi

    lib = ffi.lib
    # Invalid dtype / null pointers / bad connectivity are rejected before any CUDA call.
    assert lib.nsgb_imreconstruct(9, 1, 1, 4, 4, 4, 8, 0, 1, 1 << 20, None, None) == 2
    assert lib.nsgb_imreconstruct(0, None, 1, 4, 4, 4, 8, 0, 1, 1 << 20, None, None) == 1
    assert lib.nsgb_imreconstruct(0, 1, 1, 4, 4, 4, 6, 0, 1, 1 << 20, None, None) == 1
    assert lib.nsgb_imreconstruct(0, 1, 1, 4, 4, 3, 8, 0, 1, 1 << 20, None, None) == 1
    assert lib.nsgb_imreconstruct(0, 1, 1, 4, 4, 4, 8, 0, None, 0, None, None) == 3
    assert lib.nsgb_bwlabel(None, 1, 4, 4, 4, 16, 8, 1, None, 1, 1 << 20, None, None) == 1
    # the allocation-free entry point checks arguments like the others: a product of dimensions
    # that wraps in 64 bits, a pitch below the row and a bad connectivity are refused
    assert lib.nsgb_imreconstruct_noalloc(0, 1, 1, 1 << 37, 1 << 27, 1 << 27, 8, 0, None, None) == 1
    assert lib.nsgb_imreconstruct_noalloc(0, 1, 1, 4, 4, 3, 8, 0, None, None) == 1
    assert lib.nsgb_imreconstruct_noalloc(0, 1, 1, 4, 4, 4, 5, 0, None, None) == 1
    assert lib.nsgb_imhmin(2, 1, 2, 4, 4, 16, 1.0, 8, 1, 1 << 20, None, None) == 2
    # bounding boxes: null labels, pitch below the row, capacity without an output buffer
    assert lib.nsgb_bounding_boxes(None, 4, 4, 16, 0, 1, 4, None, None, 1, 1 << 20, None, None) == 1
    assert lib.nsgb_bounding_boxes(1, 4, 4, 8, 0, 1, 4, None, None, 1, 1 << 20, None, None) == 1
    assert lib.nsgb_bounding_boxes(1, 4, 4, 16, 0, None, 4, None, None, 1, 1 << 20, None, None) == 1
    # opening: even / too large / empty element, overlapping output, missing workspace
    k3 = (ctypes.c_uint8 * 9)(0, 1, 0, 1, 1, 1, 0, 1, 0)
    k0 = (ctypes.c_uint8 * 9)()
    k4 = (ctypes.c_uint8 * 16)(*([1] * 16))
    ka = ctypes.addressof
    assert lib.nsgb_morph_open(1, 4096, 4, 4, 4, 4, ka(k4), 4, 1, 1 << 20, None, None) == 1
    assert lib.nsgb_morph_open(1, 4096, 4, 4, 4, 4, ka(k0), 3, 1, 1 << 20, None, None) == 1
    assert lib.nsgb_morph_open(1, 4096, 4, 4, 4, 4, ka(k3), 65, 1, 1 << 20, None, None) == 1
    assert lib.nsgb_morph_open(1, 4096, 4, 4, 4, 4, None, 3, 1, 1 << 20, None, None) == 1
    assert lib.nsgb_morph_open(4096, 4100, 4, 4, 4, 4, ka(k3), 3, 1, 1 << 20, None, None) == 1
    assert lib.nsgb_morph_open(4096, 8192, 4, 4, 4, 4, ka(k3), 3, None, 0, None, None) == 3
    # distance transform: null mask, float pitch not a multiple of 4, too many rows, no workspace
    assert lib.nsgb_distance_transform(None, 1, 4, 4, 4, 16, 0, 1, 1 << 20, None, None) == 1
    assert lib.nsgb_distance_transform(1, 1, 4, 4, 4, 18, 0, 1, 1 << 20, None, None) == 1
    assert lib.nsgb_distance_transform(1, 1, 65535 * 128 + 1, 1, 1, 4, 0, 1, 1 << 30, None, None) == 1
    assert lib.nsgb_distance_transform(1, 1, 4, 4, 4, 16, 0, None, 0, None, None) == 3
    # nucleus candidates: null image, pitch below the row, missing workspace
    assert lib.nsgb_nucleus_candidates(None, 1, 1, 1, 4, 4, 4, 80.0, 45.0, 11, 1000, None, None, 1, 1 << 20,
                                       None, None) == 1
    assert lib.nsgb_nucleus_candidates(1, 1, 1, 1, 4, 4, 3, 80.0, 45.0, 11, 1000, None, None, 1, 1 << 20,
                                       None, None) == 1
    assert lib.nsgb_nucleus_candidates(1, 1, 1, 1, 4, 4, 4, 80.0, 45.0, 11, 1000, None, None, None, 0,
                                       None, None) == 3
