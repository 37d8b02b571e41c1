"""Seeded inputs of the five workloads, and the digest the reference fixtures are keyed by.

Shared by tests/golden/make_ref_recon.py (which runs the reference's own code on them) and the
tests (which run the oracle or the GPU on the same inputs and compare digests), so that both
sides build byte-identical inputs.  The inputs come from the seeded generator (its outputs
are pinned in synth_digest.json).

  c0  1024 x 1024 u8, 400 ellipses, seed 0; marker = mask - 10
  c1  4096 x 4096 u8, 6000 ellipses, seed 0; the chain (a)-(e); also its inverse (255 - mask)
  c2  256 tiles, H and W uniform in [256, 4096] (sizes seed 0xC2), tile i from seed i with one
      ellipse per 2800 px^2; u8, and u16 / i32 scaled by 257 / 1000 (threshold scaled alike)
  c3  16 x 2048 x 2048 f32, mask uniform in [0, 1), marker = mask * U[0.5, 1), seed 0
  c4  16384 x 16384, one ellipse per 2621 px^2, seed 0; u8 and scaled u16 / i32
"""
from __future__ import annotations

import hashlib

import numpy as np

SCALE = {"u8": 1, "u16": 257, "i32": 1000}


def digest(*arrays) -> str:
    """SHA-256 over each array's dtype (with byte order), shape and bytes, in order."""
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(f"{a.dtype.str}{a.shape}".encode())
        h.update(a.tobytes())
    return h.hexdigest()


def chain_digest(res) -> str:
    """Digest of one chain result (dict with recon, fill, labels, area, n_labels, n_kept; the
    arrays may be numpy arrays or anything with .cpu().numpy())."""
    def np_(a):
        return a if isinstance(a, np.ndarray) else a.cpu().numpy()

    return digest(np_(res["recon"]), np_(res["fill"]), np_(res["labels"]), np_(res["area"]),
                  np.array([res["n_labels"], res["n_kept"]], np.int64))


def c0():
    from nsgb import synth

    mask, marker = synth.tile_u8(1024, 1024, 400, 0)
    return marker, mask


def c1(size=4096, n=6000, seed=0):
    from nsgb import synth

    mask, marker = synth.tile_u8(size, size, n, seed)
    return marker, mask


def inverted(mask):
    """Dark objects as foreground: mask' = 255 - mask, marker' = max(mask' - 10, 0)."""
    inv = (255 - mask).astype(np.uint8)
    return np.maximum(inv.astype(np.int32) - 10, 0).astype(np.uint8), inv


def c2_sizes():
    from nsgb import synth

    return synth.tile_sizes(256, 256, 4096, 0xC2)


def c2_tile(i, dtype, sizes=None):
    """(marker, mask) of tile i."""
    from nsgb import synth

    h, w = sizes if sizes is not None else c2_sizes()
    H, W = int(h[i]), int(w[i])
    m, k = synth.tile_u8(H, W, synth.ellipses_for(H, W), i)
    if dtype == "u8":
        return k, m
    m2, k2 = synth.scale(m, dtype)
    return k2, m2


def c3():
    from nsgb import synth

    mask, marker = synth.float_pair((16, 2048, 2048), 0)
    return marker, mask


C4_SIZE = 16384


def c4(dtype, size=C4_SIZE):
    """The c4 image (the generator's mask plane) in `dtype`."""
    from nsgb import synth

    mask, _ = synth.tile_u8(size, size, int(round(size * size / 2621)), 0)
    return mask if dtype == "u8" else synth.scale(mask, dtype)[0]
