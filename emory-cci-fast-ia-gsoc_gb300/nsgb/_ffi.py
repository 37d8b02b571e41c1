"""ctypes declarations for libnsgb.so (include/nsgb.h).

The library is the only compute path: if it cannot be loaded, importing this module raises.
"""
from __future__ import annotations

import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libnsgb.so")

U8, U16, I32, F32 = 0, 1, 2, 3
OP_IMRECONSTRUCT, OP_IMRECONSTRUCT_BINARY, OP_FILL_HOLES, OP_HMIN = 0, 1, 2, 3
OP_BWSELECT, OP_BWLABEL, OP_BWAREAOPEN, OP_CHAIN = 4, 5, 6, 7
OP_BOUNDING_BOX, OP_NUCLEUS_CANDIDATES, OP_MORPH_OPEN, OP_DISTANCE = 8, 9, 10, 11
NOALLOC_SCRATCH_BYTES = 1 << 20  # NSGB_NOALLOC_SCRATCH_BYTES

STATUS = {
    0: "NSGB_OK",
    1: "NSGB_ERR_BAD_ARG",
    2: "NSGB_ERR_UNSUPPORTED_DTYPE",
    3: "NSGB_ERR_WORKSPACE",
    4: "NSGB_ERR_NOT_CONVERGED",
    5: "NSGB_ERR_TIMEOUT",
    6: "NSGB_ERR_CUDA",
    7: "NSGB_ERR_QUEUE_OVERFLOW",
}


class NsgbError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__(f"{where}: {STATUS.get(status, status)}")


class Opts(C.Structure):
    _fields_ = [("sync", C.c_int), ("max_visits_per_tile", C.c_int), ("max_visit_iters", C.c_int),
                ("queue_poll_limit", C.c_int), ("recon_passes", C.c_int), ("recon_order", C.c_int),
                ("recon_ctas_per_sm", C.c_int), ("reserved", C.c_int * 1),
                ("recon_event_begin", C.c_void_p),
                ("recon_event_end", C.c_void_p)]


class Tile(C.Structure):
    _fields_ = [("marker", C.c_void_p), ("mask", C.c_void_p), ("rows", C.c_int64), ("cols", C.c_int64),
                ("pitch", C.c_int64), ("fill_out", C.c_void_p), ("labels_out", C.c_void_p), ("area_out", C.c_void_p)]


class Batch(C.Structure):
    _fields_ = [("dtype", C.c_int), ("n", C.c_int), ("total_px", C.c_int64), ("recon_tiles", C.c_int),
                ("label_tiles", C.c_int), ("rank_blocks", C.c_int), ("total_rows", C.c_int), ("max_cols", C.c_int),
                ("max_perimeter", C.c_int), ("ws", C.c_void_p), ("ws_bytes", C.c_size_t), ("flood_tiles", C.c_int),
                ("bit_words", C.c_int), ("reserved", C.c_int * 6)]


def _load() -> C.CDLL:
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libnsgb.so is not built ({LIB_PATH}); run __graft_entry__.build()")
    return C.CDLL(LIB_PATH)


lib = _load()

_vp, _i64, _int, _sz, _dbl = C.c_void_p, C.c_int64, C.c_int, C.c_size_t, C.c_double
_i32p = C.POINTER(C.c_int32)
_optp = C.POINTER(Opts)

_SIGS = {
    "nsgb_workspace_size": (_sz, [_int, _int, _i64, _i64]),
    "nsgb_status_string": (C.c_char_p, [_int]),
    "nsgb_device_status": (_int, [_vp, _vp]),
    "nsgb_imreconstruct": (_int, [_int, _vp, _vp, _i64, _i64, _i64, _int, _int, _vp, _sz, _vp, _optp]),
    "nsgb_imreconstruct_noalloc": (_int, [_int, _vp, _vp, _i64, _i64, _i64, _int, _int, _vp, _optp]),
    "nsgb_noalloc_device_status": (_int, [_vp]),
    "nsgb_imreconstruct_binary": (_int, [_int, _vp, _vp, _i64, _i64, _i64, _int, _vp, _sz, _vp, _optp]),
    "nsgb_imfill_holes": (_int, [_int, _vp, _vp, _i64, _i64, _i64, _int, _int, _vp, _sz, _vp, _optp]),
    "nsgb_imhmin": (_int, [_int, _vp, _vp, _i64, _i64, _i64, _dbl, _int, _vp, _sz, _vp, _optp]),
    "nsgb_bwselect": (_int, [_int, _vp, _vp, _vp, _i64, _i64, _i64, _int, _vp, _sz, _vp, _optp]),
    "nsgb_bwlabel": (_int, [_vp, _vp, _i64, _i64, _i64, _i64, _int, _int, _i32p, _vp, _sz, _vp, _optp]),
    "nsgb_bwareaopen": (_int, [_vp, _int, _vp, _vp, _i64, _i64, _i64, _i64, _i64, C.c_int32, C.c_int32, _int,
                               _i32p, _vp, _sz, _vp, _optp]),
    "nsgb_bounding_boxes": (_int, [_vp, _i64, _i64, _i64, C.c_int32, _vp, _i64, _i32p, _vp, _vp, _sz, _vp, _optp]),
    "nsgb_distance_transform": (_int, [_vp, _vp, _i64, _i64, _i64, _i64, _int, _vp, _sz, _vp, _optp]),
    "nsgb_morph_open": (_int, [_vp, _vp, _i64, _i64, _i64, _i64, _vp, _int, _vp, _sz, _vp, _optp]),
    "nsgb_nucleus_candidates": (_int, [_vp, _vp, _vp, _vp, _i64, _i64, _i64, _dbl, _dbl, C.c_int32, C.c_int32, _i32p,
                                       _vp, _vp, _sz, _vp, _optp]),
    "nsgb_threshold": (_int, [_int, _vp, _vp, _i64, _i64, _i64, _i64, _dbl, _vp]),
    "nsgb_invert": (_int, [_int, _vp, _vp, _i64, _i64, _i64, _vp]),
    "nsgb_chain": (_int, [_int, _vp, _vp, _i64, _i64, _i64, _int, _dbl, _int, _int, C.c_int32, C.c_int32,
                          _vp, _vp, _vp, _i32p, _i32p, _vp, _sz, _vp, _optp]),
    "nsgb_batch_workspace_size": (_sz, [_int, C.POINTER(Tile), _int]),
    "nsgb_batch_prepare": (_int, [_int, C.POINTER(Tile), _int, _vp, _sz, C.POINTER(Batch)]),
    "nsgb_chain_batch": (_int, [C.POINTER(Batch), _int, _dbl, _int, _int, C.c_int32, C.c_int32, _i32p, _i32p, _vp,
                                _optp]),
    "nsgb_batch_counts_async": (_int, [C.POINTER(Batch), _vp, _vp]),
    "nsgb_imreconstruct_batch": (_int, [C.POINTER(Batch), _int, _int, _vp, _optp]),
    "nsgb_recon_f32_workspace_size": (_sz, [C.c_int64, C.c_int64, C.c_int64, _int]),
    "nsgb_recon_f32_fwd": (_int, [_vp, _vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int64, _int,
                                  _vp, _sz, _vp, _optp]),
    "nsgb_recon_f32_bwd": (_int, [_vp, _vp, _vp, _vp, C.c_int64, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                  _vp, _sz, _vp, _optp]),
    "nsgb_synth_tile_u8": (_int, [_vp, _vp, _i64, _i64, _i64, _i64, C.c_uint64]),
    "nsgb_synth_scale_u16": (_int, [_vp, _vp, _vp, _i64]),
    "nsgb_synth_scale_i32": (_int, [_vp, _vp, _vp, _i64]),
    "nsgb_synth_float": (_int, [_vp, _vp, _i64, C.c_uint64]),
    "nsgb_synth_tile_sizes": (_int, [_vp, _vp, _i64, C.c_int32, C.c_int32, C.c_uint64]),
}

for _name, (_res, _args) in _SIGS.items():
    _f = getattr(lib, _name)
    _f.restype = _res
    _f.argtypes = _args

EXPORTED = tuple(_SIGS)


def check(status: int, where: str) -> None:
    if status != 0:
        raise NsgbError(status, where)
