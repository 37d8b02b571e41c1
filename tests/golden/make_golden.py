"""Writes the golden fixtures under tests/golden/ (run in a container that has the reference).

Sources of truth, both independent of the oracle restatement:
  * ref_fixture_32.npz -- the inline 32x32 binary image and seed image of the reference's
    queue test (test/segment/cuda/globalQueueTest.cu, BOOST_AUTO_TEST_CASE(morphReconstruction)),
    parsed from that file as text.  The reference prints the reconstruction without checking it,
    so the expected result is derived here by an independent 4-connected flood fill
    (scipy.ndimage.label): mask pixels connected to a seed take the seed value.
  * ref_ccl_cases.npz -- seeded u8 images labelled by the reference's own ConnComponents.cpp
    (label, relabel, areaThresholdLabeled), compiled from its sources into oracle/_ref/.
  * ref_bbox_cases.npz -- label images (raw root labels with background -1, raster labels with
    background 0, and raster labels with stray -1 pixels that end the reference's scan) and the
    reference's own ConnComponents::boundingBox output for them.
  * synth_digest.json -- SHA-256 of generator outputs, pinning the synthetic inputs across
    machines (x86-64 here, aarch64 on the GPU hosts).
Usage: python tests/golden/make_golden.py REFERENCE_ROOT [--bbox-only]  (or NSGB_REFERENCE_DIR=...)
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import sys

import numpy as np
import scipy.ndimage as ndi

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "emory-cci-fast-ia-gsoc_gb300"))


def parse_queue_fixture(ref_root: str):
    path = os.path.join(ref_root, "test/segment/cuda/globalQueueTest.cu")
    src = open(path).read()
    body = src[src.index("BOOST_AUTO_TEST_CASE(morphReconstruction)"):]

    def array(name):
        m = re.search(name + r"\[\]\s*=\s*\{(.*?)\};", body, re.S)
        txt = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
        txt = re.sub(r"//[^\n]*", "", txt)
        return np.array([int(v) for v in re.findall(r"-?\d+", txt)])

    image = array("host_image").astype(np.uint8).reshape(32, 32)
    seeds = array("host_seeds").astype(np.int32).reshape(32, 32)
    m = re.search(r"host_input_list\[\]\s*=\s*\{(.*?)\};", body, re.S)
    seed_list = []
    for term in m.group(1).split(","):
        total = 0
        for prod in term.split("+"):
            v = 1
            for f in prod.split("*"):
                v *= int(f.strip())
            total += v
        seed_list.append(total)
    seed_list = np.array(seed_list)
    return image, seeds, seed_list


def flood_expected(image, seeds, conn):
    st = ndi.generate_binary_structure(2, 1 if conn == 4 else 2)
    lab, _ = ndi.label(image != 0, structure=st)
    out = np.zeros_like(seeds)
    for v in np.unique(lab[(seeds != 0) & (image != 0)]):
        comp = lab == v
        out[comp] = np.minimum(seeds[(seeds != 0) & comp].max(), image[comp])
    return out


def ccl_cases(rng):
    cases = []
    shapes = [(1, 1), (1, 57), (63, 1), (7, 9), (32, 32), (33, 31), (64, 100), (97, 65), (128, 128)]
    for (h, w) in shapes:
        for kind in ("binary", "multi", "checker", "dense"):
            if kind == "binary":
                img = (rng.random((h, w)) < 0.45).astype(np.uint8) * 255
            elif kind == "multi":
                img = rng.integers(0, 4, (h, w)).astype(np.uint8) * 60
            elif kind == "checker":
                img = (((np.arange(h)[:, None] + np.arange(w)[None, :]) % 2) * 255).astype(np.uint8)
            else:
                img = (rng.random((h, w)) < 0.7).astype(np.uint8) * 255
            cases.append(img)
    return cases


def bbox_cases(oracle):
    """Label images for ConnComponents::boundingBox, each with the background value it uses."""
    rng = np.random.default_rng(20261204)
    cases = []
    for k, img in enumerate(ccl_cases(np.random.default_rng(20261203))):
        for conn in (4, 8):
            lab, _ = oracle.ref_label(img, conn, relab=False)
            rel, _ = oracle.ref_label(img, conn, relab=True)
            cases.append((lab, -1))
            cases.append((rel, 0))
            if rel.size >= 16 and (rel > 0).any():
                stray = rel.copy()
                fg = np.flatnonzero(stray > 0)
                stray.flat[fg[rng.integers(0, fg.size)]] = -1  # ends the reference's scan there
                cases.append((stray, 0))
    return cases


def write_bbox(oracle):
    arrays = {}
    for k, (lab, bg) in enumerate(bbox_cases(oracle)):
        arrays[f"lab{k}"] = lab
        arrays[f"bg{k}"] = np.array(bg)
        arrays[f"box{k}"] = oracle.ref_bounding_box(lab, bg)
    np.savez_compressed(os.path.join(HERE, "ref_bbox_cases.npz"), **arrays)


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    ref_root = args[0] if args else os.environ.get("NSGB_REFERENCE_DIR", "")
    if not ref_root and "--bbox-only" not in sys.argv:
        raise SystemExit("usage: make_golden.py REFERENCE_ROOT [--bbox-only]  (or set NSGB_REFERENCE_DIR)")
    import oracle  # noqa: E402

    if "--bbox-only" in sys.argv:
        if not oracle.ref_available():
            raise SystemExit("oracle/_ref not built: run oracle/build_ref.sh first")
        write_bbox(oracle)
        print("wrote ref_bbox_cases.npz")
        return

    # 1. reference inline fixture
    image, seeds, seed_list = parse_queue_fixture(ref_root)
    np.savez_compressed(os.path.join(HERE, "ref_fixture_32.npz"), image=image, seeds=seeds, seed_list=seed_list,
                        expected4=flood_expected(image, seeds, 4), expected8=flood_expected(image, seeds, 8))

    # 2. reference ConnComponents on seeded inputs
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref not built: run oracle/build_ref.sh first")
    rng = np.random.default_rng(20261203)
    arrays = {}
    for k, img in enumerate(ccl_cases(rng)):
        arrays[f"img{k}"] = img
        for conn in (4, 8):
            lab, n = oracle.ref_label(img, conn, relab=False)
            rel, nr = oracle.ref_label(img, conn, relab=True)
            kept, nk = oracle.ref_area_threshold_labeled(lab, 3, 40)
            arrays[f"lab{k}_{conn}"] = lab
            arrays[f"rel{k}_{conn}"] = rel
            arrays[f"n{k}_{conn}"] = np.array(nr)
            arrays[f"kept{k}_{conn}"] = kept
            arrays[f"nk{k}_{conn}"] = np.array(nk)
    np.savez_compressed(os.path.join(HERE, "ref_ccl_cases.npz"), **arrays)
    write_bbox(oracle)

    # 3. generator digests
    from nsgb import synth
    dig = {}
    for (H, W, n, seed) in [(64, 80, 20, 3), (257, 131, 12, 7), (1024, 1024, 400, 0)]:
        m, k = synth.tile_u8(H, W, n, seed)
        dig[f"u8_{H}x{W}_{n}_{seed}"] = hashlib.sha256(m.tobytes() + k.tobytes()).hexdigest()
    m, _ = synth.tile_u8(64, 80, 20, 3)
    for dt in ("u16", "i32"):
        a, b = synth.scale(m, dt)
        dig[f"{dt}_64x80_20_3"] = hashlib.sha256(a.tobytes() + b.tobytes()).hexdigest()
    a, b = synth.float_pair((33, 47), 5)
    dig["f32_33x47_5"] = hashlib.sha256(a.tobytes() + b.tobytes()).hexdigest()
    h, w = synth.tile_sizes(256)
    dig["sizes_256"] = hashlib.sha256(h.tobytes() + w.tobytes()).hexdigest()
    with open(os.path.join(HERE, "synth_digest.json"), "w") as f:
        json.dump(dig, f, indent=1, sort_keys=True)
    print("wrote golden fixtures")


if __name__ == "__main__":
    main()
