"""Pins the oracle's reconstruction restatement (oracle/recon_oracle.hpp) to the reference's own
code: nscale::imreconstruct, imreconstructBinary, imfillHoles, imhmin, bwselect, bwlabel2 and
bwareaopen2 from MorphologicOperations.cpp, compiled unmodified over a small OpenCV stand-in
(oracle/build_ref.sh, oracle/ref_morph.cpp, oracle/cv_shim.hpp).

* always: the oracle against the committed reference outputs (tests/golden/ref_recon_cases.npz,
  308 small cases; tests/golden/ref_recon_digests.json for the c0 and c1 workloads);
* where oracle/_ref was built: the oracle against the reference live, on fresh seeded inputs,
  and the two readings of OpenCV's CV_32S arithmetic in imfillHoles<int>.
"""
import json
import os

import numpy as np
import pytest

from conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden")
DT = {"u8": np.uint8, "u16": np.uint16, "i32": np.int32, "f32": np.float32}


def _same(a, b):
    """Bit-exact equality (floats compared by their bits: -0.0 and +0.0 differ)."""
    a, b = np.asarray(a), np.asarray(b)
    return a.dtype == b.dtype and a.shape == b.shape and a.tobytes() == b.tobytes()


def run_case(impl, case, arrays):
    ins = [arrays[k] for k in case["inputs"]]
    op, conn = case["op"], case["conn"]
    if op == "imreconstruct":
        return impl.imreconstruct(ins[0], ins[1], conn)
    if op == "imreconstructBinary":
        return impl.imreconstruct_binary(ins[0], ins[1], conn)
    if op == "imfillHoles":
        return impl.imfill_holes(ins[0], case["binary"], conn)
    if op == "imhmin":
        return impl.imhmin(ins[0], case["h"], conn)
    if op == "bwselect":
        return impl.bwselect(ins[0], ins[1], conn)
    raise ValueError(op)


def load_cases():
    d = np.load(os.path.join(GOLDEN, "ref_recon_cases.npz"))
    return d, json.loads(str(d["meta"]))


def test_oracle_matches_reference_cases(oracle):
    arrays, meta = load_cases()
    assert len(meta) >= 300
    checked = 0
    for k, case in enumerate(meta):
        if case.get("reading") == "wrap":
            continue  # the oracle takes the saturating reading of invert<int>(INT_MIN)
        got = run_case(oracle, case, arrays)
        assert _same(got, arrays[f"out{k}"]), case
        checked += 1
    assert checked > 250


def test_reference_int_fill_wraps_to_int_min(oracle):
    """Under OpenCV's CV_32S arithmetic (no saturation) invert<int>(INT_MIN) = INT_MIN, so the
    reference's imfillHoles<int> returns INT_MIN everywhere, grayscale and binary; the
    fixtures record it, and the saturating reading (the oracle's and the GPU's) differs."""
    arrays, meta = load_cases()
    wrap = [(k, c) for k, c in enumerate(meta) if c.get("reading") == "wrap"]
    assert wrap
    for k, c in wrap:
        out = arrays[f"out{k}"]
        assert (out == np.iinfo(np.int32).min).all(), c


def test_oracle_matches_reference_digests_c0_c1(oracle):
    import workloads as W

    dig = json.load(open(os.path.join(GOLDEN, "ref_recon_digests.json")))
    marker, mask = W.c0()
    for conn in (4, 8):
        assert W.digest(oracle.imreconstruct(marker, mask, conn)) == dig["c0"][f"recon{conn}"]
    runs = {"c1_1024": W.c1(1024, 400, 0), "c1_2048_s4": W.c1(2048, 1500, 4), "c1_4096": W.c1()}
    for name, (mk, ms) in runs.items():
        assert W.chain_digest(oracle.chain(mk, ms)) == dig["c1"][name], name
        imk, ims = W.inverted(ms)
        assert W.chain_digest(oracle.chain(imk, ims)) == dig["c1"][name + "_inverted"], name


def test_oracle_matches_reference_digests_c2_sample(oracle):
    import workloads as W

    dig = json.load(open(os.path.join(GOLDEN, "ref_recon_digests.json")))
    sizes = W.c2_sizes()
    small = np.argsort(sizes[0].astype(np.int64) * sizes[1])[:6]  # the six smallest tiles
    for dtype in ("u8", "u16", "i32"):
        for i in small:
            mk, ms = W.c2_tile(int(i), dtype, sizes)
            res = oracle.chain(mk, ms, thr=128.0 * W.SCALE[dtype])
            assert W.chain_digest(res) == dig["c2"][dtype][int(i)], (dtype, int(i))


# ---- live, where the reference's code was built here ------------------------------------
live = pytest.mark.skipif("not __import__('oracle').ref_morph_available()",
                          reason="oracle/_ref not built (reference sources absent)")


@live
@pytest.mark.parametrize("dtype", ["u8", "u16", "i32", "f32"])
def test_oracle_matches_reference_live(oracle, dtype):
    from make_ref_recon import small_inputs

    rng = np.random.default_rng(7 + len(dtype))
    for shape in [(2, 3), (17, 1), (1, 23), (31, 45), (64, 64), (100, 37)]:
        marker, mask, bmark, bimg = small_inputs(rng, DT[dtype], shape)
        for conn in (4, 8):
            assert _same(oracle.imreconstruct(marker, mask, conn), oracle.ref_imreconstruct(marker, mask, conn))
            sat = dtype == "i32"
            assert _same(oracle.imfill_holes(mask, False, conn),
                         oracle.ref_imfill_holes(mask, False, conn, saturate_32s=sat))
            if dtype != "f32":
                assert _same(oracle.imreconstruct_binary(bmark, bimg, conn),
                             oracle.ref_imreconstruct_binary(bmark, bimg, conn))
                assert _same(oracle.imfill_holes(bimg, True, conn),
                             oracle.ref_imfill_holes(bimg, True, conn, saturate_32s=sat))
                assert _same(oracle.bwselect(bimg, bmark, conn), oracle.ref_bwselect(bimg, bmark, conn))
            if dtype != "i32":
                h = {"u8": 9, "u16": 700, "f32": 0.125}[dtype]
                assert _same(oracle.imhmin(mask, h, conn), oracle.ref_imhmin(mask, h, conn))


@live
def test_oracle_chain_stages_match_reference_live(oracle):
    import workloads as W

    mk, ms = W.c1(768, 230, 11)
    for m, k in ((mk, ms), W.inverted(ms)):
        a, b = oracle.chain(m, k), oracle.ref_chain(m, k)
        for key in ("recon", "thr", "fill", "labels", "area"):
            assert _same(a[key], b[key]), key
        assert (a["n_labels"], a["n_kept"]) == (b["n_labels"], b["n_kept"])
        lab_o, n_o = oracle.bwlabel2(a["fill"], 8, True)
        lab_r, n_r = oracle.ref_bwlabel2(a["fill"], 8, True)
        assert _same(lab_o, lab_r) and n_o == n_r
        for flatten in (True, False):
            o, no = oracle.bwareaopen2(a["fill"], False, flatten, 11, 1000, 8)
            r, nr = oracle.ref_bwareaopen2(a["fill"], False, flatten, 11, 1000, 8)
            assert _same(o, r) and no == nr


@live
def test_reference_int_fill_readings_live(oracle):
    rng = np.random.default_rng(5)
    img = rng.integers(0, 1000, (21, 34)).astype(np.int32)
    for binary in (False, True):
        wrap = oracle.ref_imfill_holes(img, binary, 4)
        assert (wrap == np.iinfo(np.int32).min).all()
        assert _same(oracle.ref_imfill_holes(img, binary, 4, saturate_32s=True), oracle.imfill_holes(img, binary, 4))


@live
@pytest.mark.parametrize("dtype", ["u8", "u16", "i32", "f32"])
def test_threshold_matches_reference(oracle, dtype):
    rng = np.random.default_rng(12)
    if dtype == "f32":
        img = rng.random((40, 50), dtype=np.float32)
        thrs = [0.5, 0.1, 1.0 / 3.0]
    else:
        hi = {"u8": 255, "u16": 65535, "i32": 100000}[dtype]
        img = rng.integers(0, hi, (40, 50)).astype(DT[dtype])
        thrs = [hi / 2, 128.0, 127.5, hi / 3]
    img.flat[:4] = [np.float32(0.1) if dtype == "f32" else 128, 0, 1, 2]
    for t in thrs:
        assert _same(oracle.threshold_gt(img, t), oracle.ref_threshold_gt(img, t)), t
