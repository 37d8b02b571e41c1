#!/usr/bin/env python3
"""Autotuner for the reconstruction's schedule: sweeps its run-time knobs on the GPU over
seeded synthetic workloads and writes the winners to tuning.json, which build.py compiles into
the library (the defaults of nsgb_imreconstruct, the chain and the batched calls, including
nsgb_batch_prepare / nsgb_chain_batch).

Knobs (no recompilation needed, each a field of nsgb_opts and of the table):
  passes  streaming passes over all tiles before the work queue (0, 2, 3)
  order   initial ring order of the work queue when there are no passes (0 raster,
          1 checkerboard, 2 four colours)
  ctas    CTAs of the work queue per SM (0 = as many as fit, 2, 3): fewer workers waste fewer
          visits where only a front of tiles has work (hole filling)
Keys: dtype (u8 / u16 / i32 / f32), connectivity, direction (dilation, or erosion as in hole
filling), single image or batch, and the image-size bucket (pixels up to 1 M, 8 M, 64 M, more).

Workloads (the generator of nsgb.synth, seeds fixed): single images are the pathology-like
tile at 1024^2 / 2048^2 / 4096^2 / 8192^2 with marker = mask - 10 (scaled with the dtype; f32: the
uniform mask with marker = mask * U[0.5, 1)); erosion is the hole fill (marker = image on the
border, max inside); batches are 48 uneven tiles (256 .. 4096 per side, one ellipse per
2800 px^2).  Each candidate is timed with CUDA events after warm-up, L2 flushed before every
run, median of `--reps`; every candidate's result is checked bit-for-bit against the first.

Usage (on a GPU): python tune.py [--out tuning.json] [--reps 7] [--quick]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

BUCKETS = [(1 << 20, 1024), (8 << 20, 2048), (64 << 20, 4096), (1 << 40, 8192)]  # (max pixels, tuning size)
DTYPES = {"u8": 0, "u16": 1, "i32": 2, "f32": 3}
# (passes, order, ctas); passes -1 = none, order is used when there are no passes
CANDIDATES = [(p, o, c) for c in (0, 2, 3) for (p, o) in ((-1, 0), (-1, 1), (-1, 2), (2, 2), (3, 2))]
SCALE = {"u8": 1, "u16": 257, "i32": 1000}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--out", default=os.path.join(HERE, "tuning.json"))
    p.add_argument("--reps", type=int, default=7)
    p.add_argument("--quick", action="store_true", help="fewer keys (u8 / i32, 8-conn dilation, batches)")
    return p.parse_args()


class Timer:
    def __init__(self, torch):
        self.torch = torch
        self.flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
        self.stream = torch.cuda.current_stream()

    def run(self, prepare, call, reps):
        torch = self.torch
        ts = []
        for r in range(reps + 2):
            prepare()
            self.flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(self.stream)
            call()
            e1.record(self.stream)
            torch.cuda.synchronize()
            if r >= 2:
                ts.append(e0.elapsed_time(e1))
        return statistics.median(ts)


def single_inputs(dtype, size, erode):
    import numpy as np

    from nsgb import synth

    if dtype == "f32":
        mask, marker = synth.float_pair((size, size), 0)
    else:
        m8, k8 = synth.tile_u8(size, size, int(round(size * size / 2796)), 0)
        mask, marker = (m8, k8) if dtype == "u8" else synth.scale(m8, dtype)
    if erode:
        img = mask
        mx = np.finfo(np.float32).max if dtype == "f32" else np.iinfo(img.dtype).max
        marker = np.full_like(img, mx)
        marker[0, :], marker[-1, :], marker[:, 0], marker[:, -1] = img[0, :], img[-1, :], img[:, 0], img[:, -1]
    return marker, mask


def tune_single(torch, T, lib, ffi, dtype, conn, erode, size, reps):
    import numpy as np

    code = DTYPES[dtype]
    marker, mask = single_inputs(dtype, size, erode)
    H, W = mask.shape
    esz = mask.dtype.itemsize
    m = torch.from_numpy(mask).cuda()
    mk0 = torch.from_numpy(marker).cuda()
    mk = mk0.clone()
    nb = lib.nsgb_workspace_size(ffi.OP_IMRECONSTRUCT, code, H, W)
    wst = torch.empty(nb + 256, dtype=torch.uint8, device="cuda")
    ws = (wst.data_ptr() + 255) & ~255
    sp = C.c_void_p(T.stream.cuda_stream)
    results, ref = [], None
    for passes, order, ctas in CANDIDATES:
            o = ffi.Opts(1, 0, 0, 0, passes, order + 1, ctas)

            def call():
                st = lib.nsgb_imreconstruct(code, mk.data_ptr(), m.data_ptr(), H, W, W * esz, conn, int(erode), ws, nb,
                                            sp, C.byref(o))
                if st != 0:
                    raise RuntimeError(f"nsgb_imreconstruct: {st}")

            t = T.run(lambda: mk.copy_(mk0), call, reps)
            out = mk.cpu().numpy()
            if ref is None:
                ref = out
            elif not np.array_equal(out.view(np.uint8), ref.view(np.uint8)):
                raise RuntimeError(f"tuning candidate passes={passes} order={order} changed the result")
            results.append({"passes": max(passes, 0), "order": order, "ctas": ctas, "ms": t})
    return results


def tune_batch(torch, T, lib, ffi, dtype, conn, reps, n_tiles=48):
    import numpy as np

    from nsgb import synth

    code = DTYPES[dtype]
    h, w = synth.tile_sizes(n_tiles, 256, 4096, 0x7E)
    tiles = []
    for i in range(n_tiles):
        m8, k8 = synth.tile_u8(int(h[i]), int(w[i]), synth.ellipses_for(int(h[i]), int(w[i])), 1000 + i)
        tiles.append((m8, k8) if dtype == "u8" else synth.scale(m8, dtype))
    masks = [torch.from_numpy(m).cuda() for m, _ in tiles]
    markers0 = [torch.from_numpy(k).cuda() for _, k in tiles]
    markers = [k.clone() for k in markers0]
    desc = (ffi.Tile * n_tiles)()
    for i, (mk, ms) in enumerate(zip(markers, masks)):
        hh, ww = ms.shape
        desc[i] = ffi.Tile(mk.data_ptr(), ms.data_ptr(), hh, ww, ww * ms.element_size(), None, None, None)
    nb = lib.nsgb_batch_workspace_size(code, desc, n_tiles)
    wst = torch.empty(nb + 256, dtype=torch.uint8, device="cuda")
    ws = (wst.data_ptr() + 255) & ~255
    batch = ffi.Batch()
    ffi.check(lib.nsgb_batch_prepare(code, desc, n_tiles, ws, nb, C.byref(batch)), "batch_prepare")
    sp = C.c_void_p(T.stream.cuda_stream)
    results, ref = [], None

    def restore():
        for a, b in zip(markers, markers0):
            a.copy_(b)

    for passes, order, ctas in CANDIDATES:
            o = ffi.Opts(1, 0, 0, 0, passes, order + 1, ctas)

            def call():
                st = lib.nsgb_imreconstruct_batch(C.byref(batch), conn, 0, sp, C.byref(o))
                if st != 0:
                    raise RuntimeError(f"nsgb_imreconstruct_batch: {st}")

            t = T.run(restore, call, reps)
            out = [k.cpu().numpy() for k in markers]
            if ref is None:
                ref = out
            elif not all(np.array_equal(a, b) for a, b in zip(out, ref)):
                raise RuntimeError(f"tuning candidate passes={passes} order={order} changed a batch result")
            results.append({"passes": max(passes, 0), "order": order, "ctas": ctas, "ms": t})
    return results


def main():
    args = parse()
    import torch

    from nsgb import _ffi as ffi

    lib = ffi.lib
    T = Timer(torch)
    entries, log = [], []
    t0 = time.time()
    dtypes = ("u8", "i32") if args.quick else ("u8", "u16", "i32", "f32")
    for dtype in dtypes:
        for conn in ((8,) if args.quick else (4, 8)):
            for erode in ((False,) if args.quick or dtype == "f32" else (False, True)):
                for max_px, size in BUCKETS:
                    res = tune_single(torch, T, lib, ffi, dtype, conn, erode, size, args.reps)
                    best = min(res, key=lambda r: r["ms"])
                    base = res[0]["ms"]
                    entries.append({"dtype": dtype, "conn": conn, "erode": erode, "batch": False, "max_px": max_px,
                                    "passes": best["passes"], "order": best["order"], "ctas": best["ctas"]})
                    log.append({"key": [dtype, conn, erode, "single", size], "candidates": res})
                    print(f"{dtype} conn{conn} {'erode' if erode else 'dilate'} {size}^2: best passes "
                          f"{best['passes']} order {best['order']} ctas {best['ctas']} {best['ms']:.4f} ms "
                          f"(raster, no passes, all CTAs: {base:.4f} ms)", flush=True)
        if dtype != "f32":
            for conn in ((8,) if args.quick else (4, 8)):
                res = tune_batch(torch, T, lib, ffi, dtype, conn, args.reps)
                best = min(res, key=lambda r: r["ms"])
                entries.append({"dtype": dtype, "conn": conn, "erode": False, "batch": True, "max_px": 1 << 40,
                                "passes": best["passes"], "order": best["order"], "ctas": best["ctas"]})
                log.append({"key": [dtype, conn, False, "batch", 48], "candidates": res})
                print(f"{dtype} conn{conn} batch: best passes {best['passes']} order {best['order']} ctas "
                      f"{best['ctas']} {best['ms']:.3f} ms (raster, no passes, all CTAs: {res[0]['ms']:.3f} ms)",
                      flush=True)
    out = {"generated_by": "emory-cci-fast-ia-gsoc_gb300/tune.py", "device": torch.cuda.get_device_name(0),
           "seconds": round(time.time() - t0, 1), "entries": entries, "measurements": log}
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {args.out} ({len(entries)} entries)")


if __name__ == "__main__":
    main()
