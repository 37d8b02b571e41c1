"""The synthetic input generator is deterministic and matches its committed digests."""
import hashlib
import json
import os

import numpy as np


def test_generator_digests(golden_dir):
    from nsgb import synth

    dig = json.load(open(os.path.join(golden_dir, "synth_digest.json")))
    for (H, W, n, seed) in [(64, 80, 20, 3), (257, 131, 12, 7), (1024, 1024, 400, 0)]:
        m, k = synth.tile_u8(H, W, n, seed)
        assert hashlib.sha256(m.tobytes() + k.tobytes()).hexdigest() == dig[f"u8_{H}x{W}_{n}_{seed}"]
    m, _ = synth.tile_u8(64, 80, 20, 3)
    for dt in ("u16", "i32"):
        a, b = synth.scale(m, dt)
        assert hashlib.sha256(a.tobytes() + b.tobytes()).hexdigest() == dig[f"{dt}_64x80_20_3"]
    a, b = synth.float_pair((33, 47), 5)
    assert hashlib.sha256(a.tobytes() + b.tobytes()).hexdigest() == dig["f32_33x47_5"]
    h, w = synth.tile_sizes(256)
    assert hashlib.sha256(h.tobytes() + w.tobytes()).hexdigest() == dig["sizes_256"]


def test_generator_value_ranges():
    from nsgb import synth

    m, k = synth.tile_u8(512, 384, 300, 1)
    bg = m[m > 100]
    assert bg.min() >= 185 and bg.max() <= 215
    dark = m[m < 100]
    assert dark.min() >= 40 and dark.max() <= 90 and dark.size > 0
    assert np.array_equal(k, np.maximum(m.astype(int) - 10, 0).astype(np.uint8))
    h, w = synth.tile_sizes(256)
    assert h.min() >= 256 and h.max() <= 4096 and w.min() >= 256 and w.max() <= 4096
    f, g = synth.float_pair((64, 64), 0)
    assert f.min() >= 0 and f.max() < 1 and (g <= f).all() and (g >= 0.5 * f - 1e-7).all()
