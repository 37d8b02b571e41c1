"""Seeded synthetic pathology-like tiles (host side; the definition is in csrc/synth.cpp).

The reference's tests read tiles from a data directory it does not ship; these stand-ins
have the same shapes and value ranges.  All functions return numpy arrays.
"""
from __future__ import annotations

import ctypes as C
from typing import Tuple

import numpy as np

from ._ffi import lib


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def tile_u8(H: int, W: int, n_ellipses: int, seed: int = 0) -> Tuple[np.ndarray, np.ndarray]:
    """(mask, marker) u8: background 185..215, `n_ellipses` dark ellipses (40..90),
    marker = max(mask - 10, 0)."""
    mask = np.empty((H, W), np.uint8)
    marker = np.empty((H, W), np.uint8)
    rc = lib.nsgb_synth_tile_u8(_p(mask), _p(marker), H, W, W, n_ellipses, seed)
    if rc != 0:
        raise ValueError("bad synth arguments")
    return mask, marker


def scale(mask_u8: np.ndarray, dtype: str) -> Tuple[np.ndarray, np.ndarray]:
    """u16 (x257, marker - 2570) or i32 (x1000, marker - 10000) tiles from a u8 tile."""
    src = np.ascontiguousarray(mask_u8)
    if dtype == "u16":
        m = np.empty(src.shape, np.uint16)
        k = np.empty(src.shape, np.uint16)
        rc = lib.nsgb_synth_scale_u16(_p(src), _p(m), _p(k), src.size)
    elif dtype == "i32":
        m = np.empty(src.shape, np.int32)
        k = np.empty(src.shape, np.int32)
        rc = lib.nsgb_synth_scale_i32(_p(src), _p(m), _p(k), src.size)
    else:
        raise ValueError(dtype)
    if rc != 0:
        raise ValueError("bad synth arguments")
    return m, k


def float_pair(shape, seed: int = 0) -> Tuple[np.ndarray, np.ndarray]:
    """(mask, marker) f32: mask uniform in [0,1), marker = mask * u, u uniform in [0.5, 1)."""
    m = np.empty(shape, np.float32)
    k = np.empty(shape, np.float32)
    rc = lib.nsgb_synth_float(_p(m), _p(k), m.size, seed)
    if rc != 0:
        raise ValueError("bad synth arguments")
    return m, k


def tile_sizes(n: int, lo: int = 256, hi: int = 4096, seed: int = 0xC2) -> Tuple[np.ndarray, np.ndarray]:
    h = np.empty(n, np.int32)
    w = np.empty(n, np.int32)
    rc = lib.nsgb_synth_tile_sizes(_p(h), _p(w), n, lo, hi, seed)
    if rc != 0:
        raise ValueError("bad synth arguments")
    return h, w


def ellipses_for(H: int, W: int, px_per_ellipse: int = 2800) -> int:
    return int(round(H * W / px_per_ellipse))
