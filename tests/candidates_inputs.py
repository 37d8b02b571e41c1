"""Seeded inputs for the nucleus-candidate stage (HistologicalEntities.cpp:195-275).

rc is the inverted red channel of a synthetic tile (nuclei bright on a dark background);
rc_open stands in for its 19x19 disk opening: rc lowered by `h` (saturating), which keeps
rc_open <= rc as an opening does and leaves valleys rc - recon of up to h on each nucleus;
rbc marks the dark objects of a second tile, so that some candidates overlap it.
"""
import numpy as np

from nsgb import synth


def tile(h: int, w: int, n_ellipses: int, seed: int = 0, drop: int = 90):
    mask, _ = synth.tile_u8(h, w, n_ellipses, seed)
    rc = (255 - mask).astype(np.uint8)
    rc_open = np.where(rc > drop, rc - drop, 0).astype(np.uint8)
    other, _ = synth.tile_u8(h, w, max(n_ellipses // 4, 1), seed + 1)
    rbc = np.where(other < 128, 255, 0).astype(np.uint8)
    return rc, rc_open, rbc


def noise(rng, h: int, w: int):
    """Unstructured case: rc uniform, rc_open = rc minus a random amount, rbc sparse."""
    rc = rng.integers(0, 256, (h, w)).astype(np.uint8)
    rc_open = np.maximum(rc.astype(np.int16) - rng.integers(0, 200, (h, w)), 0).astype(np.uint8)
    rbc = np.where(rng.random((h, w)) < 0.05, 255, 0).astype(np.uint8)
    return rc, rc_open, rbc
