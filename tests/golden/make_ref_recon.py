"""Writes the reconstruction fixtures from the reference's own code (oracle/_ref/libmorph_ref*.so,
built from the reference's sources by oracle/build_ref.sh).  Run where the reference tree is
readable: python tests/golden/make_ref_recon.py [--no-large]

  ref_recon_cases.npz     seeded small inputs (odd, non-square, 1-pixel-wide shapes; u8, u16,
                          i32, f32; 4- and 8-connected) and the reference's outputs for
                          imreconstruct, imreconstructBinary, imfillHoles (grayscale and
                          binary), imhmin and bwselect.  i32 hole filling is stored under both
                          CV_32S readings ("wrap", OpenCV's, and "sat").
  ref_recon_digests.json  SHA-256 digests (workloads.digest) of the reference's outputs on the
                          five workloads of workloads.py: c0 reconstruction, the c1 chain
                          stages (and the inverted chain), every c2 tile's chain in u8 / u16 /
                          i32, the c3 f32 reconstruction of each image, and the c4 hole fill,
                          threshold and labelling (unless --no-large).
"""
from __future__ import annotations

import json
import os
import sys
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "emory-cci-fast-ia-gsoc_gb300"))

import workloads as W  # noqa: E402

SHAPES = [(1, 1), (1, 37), (29, 1), (7, 9), (33, 31), (40, 50), (65, 33)]
DTYPES = {"u8": np.uint8, "u16": np.uint16, "i32": np.int32, "f32": np.float32}


def small_inputs(rng, dt, shape):
    """marker, mask (grayscale) and binary marker / image for one case."""
    h, w = shape
    if dt == np.float32:
        mask = (rng.random(shape, dtype=np.float32) - 0.25).astype(np.float32)
        marker = (mask * rng.uniform(0.4, 1.3, shape)).astype(np.float32)
        return marker, mask, None, None
    if dt == np.int32:
        mask = rng.integers(-2000, 2000, shape).astype(np.int32)
        marker = (mask - rng.integers(0, 600, shape)).astype(np.int32)
        fg = np.int32(5)
    else:
        hi = np.iinfo(dt).max
        base = rng.integers(hi // 2, hi, shape)
        holes = rng.random(shape) < 0.2
        mask = np.where(holes, rng.integers(0, hi // 3, shape), base).astype(dt)
        marker = np.maximum(mask.astype(np.int64) - rng.integers(0, hi // 8, shape), 0).astype(dt)
        fg = np.iinfo(dt).max
    bimg = np.where(rng.random(shape) < 0.6, fg, 0).astype(dt)
    bmark = np.where(rng.random(shape) < 0.08, fg, 0).astype(dt)
    return marker, mask, bmark, bimg


def write_cases(O):
    rng = np.random.default_rng(20261204)
    arrays, meta = {}, []

    def add(op, dt, conn, out, inputs, **extra):
        k = len(meta)
        meta.append({"op": op, "dtype": dt, "conn": conn, "inputs": inputs, **extra})
        arrays[f"out{k}"] = out

    for dname, dt in DTYPES.items():
        for shape in SHAPES:
            marker, mask, bmark, bimg = small_inputs(rng, dt, shape)
            key = f"{dname}_{shape[0]}x{shape[1]}"
            arrays[f"{key}_marker"], arrays[f"{key}_mask"] = marker, mask
            if bimg is not None:
                arrays[f"{key}_bmark"], arrays[f"{key}_bimg"] = bmark, bimg
            for conn in (4, 8):
                add("imreconstruct", dname, conn, O.ref_imreconstruct(marker, mask, conn), [f"{key}_marker", f"{key}_mask"])
                if dname == "i32":
                    for reading, sat in (("wrap", False), ("sat", True)):
                        add("imfillHoles", dname, conn, O.ref_imfill_holes(mask, False, conn, saturate_32s=sat),
                            [f"{key}_mask"], binary=False, reading=reading)
                        add("imfillHoles", dname, conn, O.ref_imfill_holes(bimg, True, conn, saturate_32s=sat),
                            [f"{key}_bimg"], binary=True, reading=reading)
                else:
                    add("imfillHoles", dname, conn, O.ref_imfill_holes(mask, False, conn), [f"{key}_mask"], binary=False)
                if dname in ("u8", "u16"):
                    add("imfillHoles", dname, conn, O.ref_imfill_holes(bimg, True, conn), [f"{key}_bimg"], binary=True)
                if dname in ("u8", "u16", "f32"):
                    h = {"u8": 23, "u16": 5000, "f32": 0.0625}[dname]
                    add("imhmin", dname, conn, O.ref_imhmin(mask, h, conn), [f"{key}_mask"], h=h)
                if bimg is not None:
                    add("imreconstructBinary", dname, conn, O.ref_imreconstruct_binary(bmark, bimg, conn),
                        [f"{key}_bmark", f"{key}_bimg"])
                    add("bwselect", dname, conn, O.ref_bwselect(bimg, bmark, conn), [f"{key}_bimg", f"{key}_bmark"])
    arrays["meta"] = np.array(json.dumps(meta))
    np.savez_compressed(os.path.join(HERE, "ref_recon_cases.npz"), **arrays)
    print(f"ref_recon_cases.npz: {len(meta)} cases")


def c4_entry(O, dtype, conn):
    img = W.c4(dtype)
    thr = 128.0 * W.SCALE[dtype]
    fill = O.ref_imfill_holes(img, False, conn, saturate_32s=(dtype == "i32"))
    lab, n = O.ref_bwlabel2(O.ref_threshold_gt(fill, thr), 8, True)
    return {"fill": W.digest(fill), "labels": W.digest(lab), "n_labels": n}


def c4_dark(O, dtype):
    img = W.c4(dtype)
    lab, n = O.ref_bwlabel2(255 - O.ref_threshold_gt(img, 128.0 * W.SCALE[dtype]), 8, True)
    return {"labels": W.digest(lab), "n_labels": n}


def write_digests(O, large: bool):
    out = {"reference": "oracle/_ref/libmorph_ref.so (reference sources, see oracle/build_ref.sh); "
                        "i32 hole filling with saturating CV_32S arithmetic"}
    t0 = time.time()
    marker, mask = W.c0()
    out["c0"] = {f"recon{c}": W.digest(O.ref_imreconstruct(marker, mask, c)) for c in (4, 8)}
    chains = {}
    for name, (mk, ms) in {"c1_4096": W.c1(), "c1_1024": W.c1(1024, 400, 0), "c1_2048_s4": W.c1(2048, 1500, 4)}.items():
        chains[name] = W.chain_digest(O.ref_chain(mk, ms))
        imk, ims = W.inverted(ms)
        chains[name + "_inverted"] = W.chain_digest(O.ref_chain(imk, ims))
    out["c1"] = chains
    print(f"c0/c1 {time.time() - t0:.1f} s", flush=True)

    sizes = W.c2_sizes()
    out["c2"] = {}
    for dtype in ("u8", "u16", "i32"):
        t0 = time.time()

        def one(i):
            mk, ms = W.c2_tile(i, dtype, sizes)
            return W.chain_digest(O.ref_chain(mk, ms, thr=128.0 * W.SCALE[dtype]))

        with ThreadPoolExecutor(os.cpu_count()) as ex:
            out["c2"][dtype] = list(ex.map(one, range(256)))
        print(f"c2 {dtype} {time.time() - t0:.1f} s", flush=True)

    t0 = time.time()
    marker, mask = W.c3()
    with ThreadPoolExecutor(os.cpu_count()) as ex:
        out["c3"] = {"recon8": list(ex.map(lambda b: W.digest(O.ref_imreconstruct(marker[b], mask[b], 8)), range(16)))}
    print(f"c3 {time.time() - t0:.1f} s", flush=True)

    if large:
        t0 = time.time()
        out["c4"] = {}
        jobs = [(d, c) for d in ("u8", "u16", "i32") for c in (4, 8)]
        with ThreadPoolExecutor(3) as ex:
            res = list(ex.map(lambda dc: c4_entry(O, *dc), jobs))
            dark = list(ex.map(lambda d: c4_dark(O, d), ("u8", "u16", "i32")))
        for (d, c), r in zip(jobs, res):
            out["c4"][f"{d}_conn{c}"] = r
        for d, r in zip(("u8", "u16", "i32"), dark):
            out["c4"][f"{d}_dark"] = r
        print(f"c4 {time.time() - t0:.1f} s", flush=True)
    else:
        prev = os.path.join(HERE, "ref_recon_digests.json")
        if os.path.exists(prev):
            old = json.load(open(prev))
            if "c4" in old:
                out["c4"] = old["c4"]
    with open(os.path.join(HERE, "ref_recon_digests.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote ref_recon_digests.json")


def main():
    import oracle as O

    if not O.ref_morph_available():
        raise SystemExit("oracle/_ref not built: run oracle/build_ref.sh REFERENCE_ROOT first")
    write_cases(O)
    write_digests(O, large="--no-large" not in sys.argv)


if __name__ == "__main__":
    main()
