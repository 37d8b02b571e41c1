#!/usr/bin/env python3
"""Benchmark of the reconstruction + labelling hot path on one GB300.

Workload (the single-tile chain): a 4096 x 4096 uint8 synthetic pathology tile with 6000
dark ellipses; (a) reconstruction by dilation of marker = mask - 10 under the mask,
8-connected; (b) threshold `> 128`; (c) binary hole fill, 4-connected; (d) bwlabel,
8-connected, raster-order int32 labels; (e) bwareaopen keeping areas in [11, 1000).

One step = one pass of the chain over the tile.  `value` is the whole-job throughput in
MPix/s with inputs already resident in HBM (marker reset and L2 flushed outside the timed
events before every step; the nsgb_chain call recorded once in a CUDA graph and replayed, the
direct call's time reported beside it); `e2e` is the same chain through the C ABI with host buffers,
host->device copies of marker and mask and device->host copies of labels and the area mask
inside the timed region (steps rotate over four streams with their own buffers, so the
copies of some steps overlap the kernels of another).  `--impl reference` times the reference's
own CPU code for the chain (its MorphologicOperations / ConnComponents functions compiled from
its sources into oracle/_ref/; the oracle's restatement where that was not built) on the full
tile, one tile per host core per step, loading no device library.

Multi-GPU (torchrun, one process per GPU): the path does not shard a single tile, so every
rank processes its own tile (replicas, weak scaling); the max over ranks of the step time
gives the job throughput.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "emory-cci-fast-ia-gsoc_gb300")
sys.path.insert(0, PKG)

METRIC = "imreconstruct+bwlabel MPix/s, uint8 4096², plain vs batched GPU; % of HBM peak"
# One image: recon init + recon, the two-class labelling that fills and labels at once
# (zeroing, local, merge, border walk, parent join, flatten), rank (mark, count, scan, assign),
# label/area/fill output.  A batch: recon init + recon, fill (pack, flood seed, flood
# seed finish, flood), label of the flooded plane (local, merge, flatten), rank (mark, count,
# scan, assign), label/area/fill output.  See csrc/ops.cu chain_impl.  A tuned schedule with
# streaming passes replaces recon init by its passes and two seed kernels (tuned_passes below).
KERNELS_PER_CHAIN = 13
KERNELS_PER_BATCH_CHAIN = 14
E2E_LANES = 4  # streams the end-to-end steps rotate over


def tuned_passes(dtype, conn, batch, px):
    """Streaming passes of the reconstruction's tuned schedule (tuning.json, compiled into the
    library) for a call: 0 when the ring starts with every tile."""
    try:
        with open(os.path.join(PKG, "tuning.json")) as f:
            entries = json.load(f)["entries"]
    except (OSError, ValueError, KeyError):
        return 0
    for e in entries:
        if (e["dtype"] == dtype and int(e["conn"]) == conn and not e["erode"] and bool(e["batch"]) == batch
                and px <= int(e["max_px"])):
            return int(e["passes"])
    return 0


def chain_kernels(dtype, batch, px):
    p = tuned_passes(dtype, 8, batch, px)
    return (KERNELS_PER_BATCH_CHAIN if batch else KERNELS_PER_CHAIN) + (p + 1 if p > 0 else 0)
RECON_BYTES_PER_PX = 3  # marker read + mask read + result write (u8)
CHAIN_BYTES_PER_PX = 17  # recon 3 + threshold 2 + fill 2 + bwlabel 5 + bwareaopen 5


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=None, help="default: 400 (GPU arm), 5 (--impl reference)")
    p.add_argument("--warmup", type=int, default=None, help="default: 10 (GPU arm), 1 (--impl reference)")
    p.add_argument("--impl", default="nsgb", choices=["nsgb", "reference"])
    p.add_argument("--size", type=int, default=4096)
    p.add_argument("--ellipses", type=int, default=6000)
    p.add_argument("--e2e-steps", type=int, default=50)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--batch-tiles", type=int, default=256)
    p.add_argument("--batch-steps", type=int, default=5)
    p.add_argument("--batch-dtypes", default="u8,u16,i32")
    p.add_argument("--no-batch", action="store_true")
    p.add_argument("--batch-only", action="store_true",
                   help="profiling aid: only the batched chain replays (no per-tile loop, no headline); "
                        "prints the batched section alone")
    p.add_argument("--no-grad", action="store_true")
    p.add_argument("--no-large", action="store_true")
    p.add_argument("--no-bbox", action="store_true")
    p.add_argument("--no-candidates", action="store_true")
    p.add_argument("--no-distance", action="store_true")
    p.add_argument("--candidates-only", action="store_true",
                   help="profiling aid: only the segmentation-stage sections (opening + candidates, distance)")
    p.add_argument("--large-size", type=int, default=16384)
    p.add_argument("--large-dtypes", default="u8,u16,i32")
    p.add_argument("--only", default="", choices=["", "batched", "grad", "large", "bbox", "candidates", "distance"],
                   help="profiling aid: run this one section alone (no headline) and print it")
    a = p.parse_args()
    if a.steps is None:
        a.steps = 5 if a.impl == "reference" else 400
    if a.warmup is None:
        a.warmup = 1 if a.impl == "reference" else 10
    return a


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


RECON_SOURCES = ("recon.cu", "tilequeue.cuh", "common.cuh", "batch.cuh")
RECON_PROFILE = os.path.join(ROOT, "profiles", "recon_kernel_u8_4096.md")


def recon_source_sha():
    """SHA-256 over the reconstruction's device sources, in a fixed order."""
    import hashlib

    h = hashlib.sha256()
    for name in RECON_SOURCES:
        with open(os.path.join(PKG, "csrc", name), "rb") as f:
            h.update(name.encode() + b"\0" + f.read())
    return h.hexdigest()


def read_traffic(size):
    """DRAM bytes per reconstruction call (all its launches) from the committed ncu summary, and
    a note.  ncu cannot run inside the bench (it replays kernels), so the capture is taken
    separately; it is used only while the reconstruction's sources hash to the value recorded
    with it, otherwise traffic is null and the note says why."""
    fields = {}
    try:
        for line in open(RECON_PROFILE):
            if ":" in line and line.split(":")[0] in ("traffic_bytes_per_launch_4096", "recon_source_sha256"):
                k, v = line.split(":", 1)
                fields[k.strip()] = v.strip()
    except OSError:
        return None, "no ncu summary committed"
    if size != 4096 or "traffic_bytes_per_launch_4096" not in fields:
        return None, "no ncu capture for this size"
    cur = recon_source_sha()
    if fields.get("recon_source_sha256") != cur:
        return None, f"stale: the reconstruction sources (sha256 {cur[:12]}) changed since the ncu capture"
    return int(fields["traffic_bytes_per_launch_4096"]), (
        f"ncu capture of the same bench command, reconstruction sources sha256 {cur[:12]} (see {os.path.relpath(RECON_PROFILE, ROOT)})")


class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.proc = None
        self.path = None
        try:
            import torch

            bus = getattr(torch.cuda.get_device_properties(device_index), "pci_bus_id", None)
        except Exception:
            bus = None
        ident = f"{bus:02x}" if isinstance(bus, int) else None
        self.ident = ident

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        sel = []
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        if vis and vis.split(",")[0].strip().isdigit():
            sel = ["-i", vis.split(",")[0].strip()]
        cmd = ["nvidia-smi", *sel, f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100"]
        try:
            self.proc = subprocess.Popen(cmd, stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _cpu_chain_timer():
    """(timer, kind, what): the reference's own compiled chain (oracle/_ref, built from the
    reference's sources) where it was built, else the oracle's restatement of it."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    if oracle.ref_morph_available():
        return (oracle.ref_chain_replicas_seconds, "reference",
                "the reference's own imreconstruct<uchar> / imfillHoles<uchar> / bwlabel2 / bwareaopen2 "
                "(MorphologicOperations.cpp, ConnComponents.cpp compiled from its sources, oracle/_ref)")
    return (oracle.chain_replicas_seconds, "port",
            "the oracle's C++ restatement of imreconstruct / imfillHoles / bwlabel2 / bwareaopen2")


def cpu_baseline(marker, mask, budget_s=12.0):
    """The reference's serial chain (a)-(e) on one host core, on the same tile."""
    timer, kind, what = _cpu_chain_timer()
    t = timer(marker, mask, 1, 1)
    reps = max(1, min(20, int(round(budget_s / max(t, 1e-3)))))
    t = timer(marker, mask, 1, reps)
    mpix = reps * mask.size / 1e6
    return {"value": mpix / t, "unit": "MPix/s", "cores": 1, "kind": kind,
            "sample": f"{reps} serial runs of the full {mask.shape[0]}x{mask.shape[1]} u8 chain (a)-(e), "
                      f"{t:.1f} s, one thread; {what}"}


def run_reference(args):
    """The reference's CPU implementation of the chain on all host cores: every step runs the
    full workload tile through the chain once per host thread (independent tiles, one per core),
    so the sample is `threads` tiles of exactly the GPU arm's workload.  Loads only oracle/
    libraries (the generator included), no device library."""
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    timer, kind, what = _cpu_chain_timer()
    threads = os.cpu_count() or 1
    mask, marker = oracle.synth_tile_u8(args.size, args.size, args.ellipses, 0)
    for _ in range(args.warmup):
        timer(marker, mask, threads, 1)
    times = [timer(marker, mask, threads, 1) for _ in range(args.steps)]
    ms = statistics.mean(times) * 1e3
    value = threads * mask.size / 1e6 / (ms / 1e3)
    workload = (f"single-tile chain (a)-(e): u8 {args.size}x{args.size}, {args.ellipses} ellipses, recon 8-conn, "
                f"threshold >128, fillHoles binary 4-conn, bwlabel 8-conn relabel, bwareaopen [11,1000)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "MPix/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": workload, "threads": threads,
                   "step": f"{threads} host threads, each running the full tile through the chain once"},
        "cpu_baseline": {"value": value, "unit": "MPix/s", "cores": threads, "kind": kind,
                         "sample": f"{threads} threads x one {args.size}x{args.size} u8 chain (a)-(e) per step; "
                                   f"{what}"},
        "e2e": {"value": value, "unit": "MPix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_nsgb(args):
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if args.batch_only:
        print(json.dumps({"batched": batched_section(args, torch.device("cuda", local))}))
        return 0
    if args.candidates_only:
        dev = torch.device("cuda", local)
        print(json.dumps({"candidates": candidates_section(args, dev), "distance": distance_section(args, dev)}))
        return 0
    if args.only:
        dev = torch.device("cuda", local)
        fn = {"batched": lambda: batched_section(args, dev), "grad": lambda: grad_section(dev),
              "large": lambda: large_section(args, dev), "bbox": lambda: bbox_section(args, dev),
              "candidates": lambda: candidates_section(args, dev), "distance": lambda: distance_section(args, dev)}
        print(json.dumps({args.only: fn[args.only]()}))
        return 0
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from nsgb import _ffi, synth

    lib = _ffi.lib
    H = W = args.size
    n_px = H * W
    mask_h, marker_h = synth.tile_u8(H, W, args.ellipses, 0)
    dev = torch.device("cuda", local)
    mask = torch.from_numpy(mask_h).to(dev)
    marker_src = torch.from_numpy(marker_h).to(dev)
    work = torch.empty_like(marker_src)
    fill = torch.empty((H, W), dtype=torch.uint8, device=dev)
    labels = torch.empty((H, W), dtype=torch.int32, device=dev)
    area = torch.empty((H, W), dtype=torch.uint8, device=dev)
    ws_bytes = lib.nsgb_workspace_size(_ffi.OP_CHAIN, _ffi.U8, H, W)
    ws_t = torch.empty(ws_bytes + 256, dtype=torch.uint8, device=dev)
    ws = (ws_t.data_ptr() + 255) & ~255
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)

    ev_rb = torch.cuda.Event(enable_timing=True)
    ev_re = torch.cuda.Event(enable_timing=True)
    opts = _ffi.Opts(0, 0, 0)

    def chain_call(o):
        st = lib.nsgb_chain(_ffi.U8, work.data_ptr(), mask.data_ptr(), H, W, W, 8, 128.0, 4, 8, 11, 1000,
                            fill.data_ptr(), labels.data_ptr(), area.data_ptr(), None, None, ws, ws_bytes, sp,
                            C.byref(o))
        if st != 0:
            raise RuntimeError(f"nsgb_chain: {_ffi.STATUS.get(st, st)}")

    def step(ev0, ev1):
        work.copy_(marker_src)
        flush.fill_(1)
        ev0.record(stream)
        chain_call(opts)
        ev1.record(stream)

    def new_events(n):
        # torch creates the CUDA event on first record(); record once so the handle exists
        # before it is handed to the C ABI.
        out = []
        for _ in range(n):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            b.record(stream)
            out.append((a, b))
        return out

    ev_rb.record(stream)
    ev_re.record(stream)
    opts.recon_event_begin = C.c_void_p(ev_rb.cuda_event)
    opts.recon_event_end = C.c_void_p(ev_re.cuda_event)
    w0, w1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(max(args.warmup, 3)):
        step(w0, w1)
    torch.cuda.synchronize()
    st = lib.nsgb_device_status(C.c_void_p(ws), sp)
    if st != 0:
        raise RuntimeError(f"device status after warm-up: {_ffi.STATUS.get(st, st)}")

    # The chain call recorded once in a CUDA graph (as a serving loop records its per-tile call)
    # and replayed every step: the graph removes the launch gaps between the chain's 15 kernels
    # and its memsets.  The recon events are recorded by nodes of the graph; each step is
    # followed by a synchronisation (outside its events) to read them.
    graph = torch.cuda.CUDAGraph()
    cs = torch.cuda.Stream(dev)
    g_rb, g_re = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g_rb.record(stream)
    g_re.record(stream)
    g_opts = _ffi.Opts(0, 0, 0)
    g_opts.recon_event_begin = C.c_void_p(g_rb.cuda_event)
    g_opts.recon_event_end = C.c_void_p(g_re.cuda_event)
    torch.cuda.synchronize()
    cs.wait_stream(stream)
    with torch.cuda.graph(graph, stream=cs):
        st = lib.nsgb_chain(_ffi.U8, work.data_ptr(), mask.data_ptr(), H, W, W, 8, 128.0, 4, 8, 11, 1000,
                            fill.data_ptr(), labels.data_ptr(), area.data_ptr(), None, None, ws, ws_bytes,
                            C.c_void_p(cs.cuda_stream), C.byref(g_opts))
        if st != 0:
            raise RuntimeError(f"nsgb_chain (capture): {_ffi.STATUS.get(st, st)}")
    stream.wait_stream(cs)

    def graph_step(ev0, ev1):
        work.copy_(marker_src)
        flush.fill_(1)
        ev0.record(stream)
        graph.replay()
        ev1.record(stream)

    for _ in range(max(args.warmup, 3)):
        graph_step(w0, w1)
    torch.cuda.synchronize()

    evs = new_events(args.steps)
    recon_ms = []
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in range(args.steps):
        graph_step(*evs[i])
        stream.synchronize()
        recon_ms.append(g_rb.elapsed_time(g_re))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    st = lib.nsgb_device_status(C.c_void_p(ws), sp)
    if st != 0:
        raise RuntimeError(f"device status after timed steps: {_ffi.STATUS.get(st, st)}")

    step_ms = [a.elapsed_time(b) for a, b in evs]
    ms = statistics.mean(step_ms)
    rms = statistics.mean(recon_ms)
    if dist:
        t = torch.tensor([ms, rms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms, rms = float(t[0]), float(t[1])

    # The same chain called directly through the C ABI every step (no graph), for reference.
    dsteps = min(args.steps, 50)
    devs = new_events(dsteps)
    torch.cuda.synchronize()
    for i in range(dsteps):
        step(*devs[i])
    torch.cuda.synchronize()
    direct_ms = statistics.mean(a.elapsed_time(b) for a, b in devs)

    # End to end through the C ABI with host buffers.  Every step copies its marker and mask in
    # from pinned host memory, runs the chain and copies its labels and area mask out.  Steps
    # rotate over E2E_LANES streams, each with its own device buffers and workspace, so the
    # copies of some steps overlap the kernels of another (the way a caller streams tiles).  A
    # step's copies (33.5 MB in, 83.9 MB out at about 200 GB/s each way) take longer than its
    # kernels; two streams left the copy engines the bound (0.67 ms per step), four hide them.
    pin_marker = torch.from_numpy(marker_h).pin_memory()
    pin_mask = torch.from_numpy(mask_h).pin_memory()
    e2e_opts = _ffi.Opts(0, 0, 0)
    lanes = []
    for j in range(E2E_LANES):
        st_j = torch.cuda.Stream(dev)
        ws_j = torch.empty(ws_bytes + 256, dtype=torch.uint8, device=dev)
        lanes.append({
            "stream": st_j, "sp": C.c_void_p(st_j.cuda_stream),
            "work": torch.empty_like(marker_src), "mask": torch.empty_like(mask),
            "fill": torch.empty_like(fill), "labels": torch.empty_like(labels), "area": torch.empty_like(area),
            "ws_t": ws_j, "ws": (ws_j.data_ptr() + 255) & ~255,
            "pin_labels": torch.empty((H, W), dtype=torch.int32).pin_memory(),
            "pin_area": torch.empty((H, W), dtype=torch.uint8).pin_memory(),
        })

    def e2e_step(i):
        ln = lanes[i % E2E_LANES]
        with torch.cuda.stream(ln["stream"]):
            ln["work"].copy_(pin_marker, non_blocking=True)
            ln["mask"].copy_(pin_mask, non_blocking=True)
            st = lib.nsgb_chain(_ffi.U8, ln["work"].data_ptr(), ln["mask"].data_ptr(), H, W, W, 8, 128.0, 4, 8, 11,
                                1000, ln["fill"].data_ptr(), ln["labels"].data_ptr(), ln["area"].data_ptr(), None,
                                None, ln["ws"], ws_bytes, ln["sp"], C.byref(e2e_opts))
            if st != 0:
                raise RuntimeError(f"nsgb_chain: {_ffi.STATUS.get(st, st)}")
            ln["pin_labels"].copy_(ln["labels"], non_blocking=True)
            ln["pin_area"].copy_(ln["area"], non_blocking=True)

    for i in range(4):
        e2e_step(i)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    e0.record(stream)
    for ln in lanes:
        ln["stream"].wait_event(e0)
    for i in range(args.e2e_steps):
        e2e_step(i)
    for ln in lanes:
        stream.wait_stream(ln["stream"])
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.e2e_steps
    if dist:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t[0])
    # the e2e outputs are the chain's results: spot-check them against the device-resident run
    for ln in lanes:
        if not torch.equal(ln["pin_labels"].to(dev), labels) or not torch.equal(ln["pin_area"].to(dev), area):
            raise RuntimeError("e2e outputs differ from the device-resident run")

    link = host_link(dev, 2 * n_px, 5 * n_px, n_px)

    peak, peak_kind = read_peaks()
    achieved = RECON_BYTES_PER_PX * n_px / (rms / 1e3) / 1e9
    traffic, traffic_note = read_traffic(args.size)
    line = {
        "metric": METRIC,
        "value": world * n_px / 1e6 / (ms / 1e3),
        "unit": "MPix/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u8",
        "data": "synthetic",
        "config": {
            "workload": f"single-tile chain (a)-(e): u8 {H}x{W}, {args.ellipses} ellipses, recon 8-conn, "
                        f"threshold >128, fillHoles binary 4-conn, bwlabel 8-conn relabel, bwareaopen [11,1000)",
            "l2": "flushed (512 MB write) before every step, outside the timed events",
            "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
            "execution": "the nsgb_chain call recorded once in a CUDA graph, replayed every step (e2e below calls "
                         "the C ABI directly every step)",
            "chain_ms_per_step": ms,
            "chain_ms_per_direct_call": direct_ms,
            "recon_ms_per_step": rms,
            "chain_algorithmic_GBps": CHAIN_BYTES_PER_PX * n_px / (ms / 1e3) / 1e9,
            "wall_s_timed_loop": wall,
        },
        "roofline": {
            "kernel": "recon_kernel<uint8_t,8> (persistent tile reconstruction)",
            "bound": "hbm",
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": achieved / peak,
            "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})",
            "algorithmic_bytes_per_launch": RECON_BYTES_PER_PX * n_px,
            "traffic": traffic,
            "traffic_source": traffic_note,
        },
        "e2e": {
            "value": world * n_px / 1e6 / (e2e_ms / 1e3),
            "unit": "MPix/s",
            "h2d_bytes_per_step": 2 * n_px,
            "d2h_bytes_per_step": 5 * n_px,
            "ms_per_step": e2e_ms,
            "path": f"nsgb_chain C ABI, pinned host marker/mask in, labels + area mask out; steps rotate over "
                    f"{E2E_LANES} streams with their own buffers, so some steps' copies overlap another's kernels",
            "host_link": dict(link, frac=(world * n_px / 1e6 / (e2e_ms / 1e3)) / (world * link["bound_mpix_s"])),
        },
        "gpu_launches": chain_kernels("u8", False, args.size * args.size) * args.steps,
        "clocks": clk,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(marker_h, mask_h)
    if not args.no_batch:
        line["batched"] = batched_section(args, dev)
    if not args.no_grad:
        line["differentiable"] = grad_section(dev)
    if not args.no_large:
        line["large"] = large_section(args, dev)
    if not args.no_bbox:
        line["bbox"] = bbox_section(args, dev)
    if not args.no_candidates:
        line["candidates"] = candidates_section(args, dev)
    if not args.no_distance:
        line["distance"] = distance_section(args, dev)
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


# -- batched form ---------------------------------------------------------------------------
BATCH_SCALE = {"u8": 1, "u16": 257, "i32": 1000}


def batch_tiles_host(n, seed_sizes=0xC2):
    """n synthetic u8 tiles (mask, marker); H and W i.i.d. uniform in [256, 4096], one ellipse
    per 2800 px^2, tile i generated with seed i.  Generated on all host threads."""
    from concurrent.futures import ThreadPoolExecutor

    from nsgb import synth

    h, w = synth.tile_sizes(n, 256, 4096, seed_sizes)
    with ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        return list(ex.map(lambda i: synth.tile_u8(int(h[i]), int(w[i]), synth.ellipses_for(int(h[i]), int(w[i])), i),
                           range(n)))


class FlatTiles:
    """Tiles of one dtype packed into one device buffer (each tile starts 256-byte aligned), so
    that all markers are restored with one copy."""

    def __init__(self, shapes, torch_dtype, dev):
        import torch
        # zero-filled so that the padding between tiles compares equal across buffers

        esz = torch.empty((), dtype=torch_dtype).element_size()
        self.offsets, off = [], 0
        for hh, ww in shapes:
            self.offsets.append(off)
            off += (hh * ww * esz + 255) // 256 * 256
        self.buf = torch.zeros(off // esz, dtype=torch_dtype, device=dev)
        self.esz = esz
        self.views = [self.buf[o // esz:o // esz + hh * ww].view(hh, ww) for o, (hh, ww) in zip(self.offsets, shapes)]


def run_batched(args, dev, tiles_u8, dtype):
    """Plain per-tile loop (nsgb_chain per tile on one stream) against the batched chain
    (nsgb_chain_batch recorded once in a CUDA graph and replayed) on the same tiles."""
    import torch

    from nsgb import _ffi, synth

    lib = _ffi.lib
    tdt = {"u8": torch.uint8, "u16": torch.int16, "i32": torch.int32}[dtype]
    code = {"u8": _ffi.U8, "u16": _ffi.U16, "i32": _ffi.I32}[dtype]
    thr = 128.0 * BATCH_SCALE[dtype]
    shapes = [m.shape for m, _ in tiles_u8]
    n = len(shapes)
    total_px = sum(hh * ww for hh, ww in shapes)
    mask, marker, work = (FlatTiles(shapes, tdt, dev) for _ in range(3))
    for i, (m8, k8) in enumerate(tiles_u8):
        if dtype == "u8":
            m, k = m8, k8
        else:
            m, k = synth.scale(m8, dtype)
            if dtype == "u16":
                m, k = m.view("int16"), k.view("int16")
        mask.views[i].copy_(torch.from_numpy(m))
        marker.views[i].copy_(torch.from_numpy(k))
    outs = {}
    for arm in ("plain", "batch"):
        outs[arm] = (FlatTiles(shapes, torch.uint8, dev), FlatTiles(shapes, torch.int32, dev),
                     FlatTiles(shapes, torch.uint8, dev))
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)

    # plain loop: one workspace sized for the largest tile
    mh, mw = max(s[0] for s in shapes), max(s[1] for s in shapes)
    ws_bytes = lib.nsgb_workspace_size(_ffi.OP_CHAIN, code, mh, mw)
    ws_t = torch.empty(ws_bytes + 256, dtype=torch.uint8, device=dev)
    ws = (ws_t.data_ptr() + 255) & ~255
    plain_counts = [(C.c_int32(0), C.c_int32(0)) for _ in range(n)]
    sync_opts, async_opts = _ffi.Opts(1, 0, 0), _ffi.Opts(0, 0, 0)
    fo, lo, ao = outs["plain"]

    def plain(with_counts):
        for i, (hh, ww) in enumerate(shapes):
            nl, nk = plain_counts[i]
            st = lib.nsgb_chain(code, work.views[i].data_ptr(), mask.views[i].data_ptr(), hh, ww, ww * work.esz, 8,
                                thr, 4, 8, 11, 1000, fo.views[i].data_ptr(), lo.views[i].data_ptr(),
                                ao.views[i].data_ptr(), C.byref(nl) if with_counts else None,
                                C.byref(nk) if with_counts else None, ws, ws_bytes, sp,
                                C.byref(sync_opts if with_counts else async_opts))
            if st != 0:
                raise RuntimeError(f"nsgb_chain tile {i}: {_ffi.STATUS.get(st, st)}")

    # batch: prepare once, record the chain and the count copy in a CUDA graph
    bf, bl, ba = outs["batch"]
    tarr = (_ffi.Tile * n)()
    for i, (hh, ww) in enumerate(shapes):
        tarr[i] = _ffi.Tile(work.views[i].data_ptr(), mask.views[i].data_ptr(), hh, ww, ww * work.esz,
                            bf.views[i].data_ptr(), bl.views[i].data_ptr(), ba.views[i].data_ptr())
    bws_bytes = lib.nsgb_batch_workspace_size(code, tarr, n)
    if bws_bytes == 0:
        raise RuntimeError("batch too large for one workspace")
    bws_t = torch.empty(bws_bytes + 256, dtype=torch.uint8, device=dev)
    bws = (bws_t.data_ptr() + 255) & ~255
    batch = _ffi.Batch()
    _ffi.check(lib.nsgb_batch_prepare(code, tarr, n, bws, bws_bytes, C.byref(batch)), "batch_prepare")
    counts = torch.zeros(2 * n, dtype=torch.int32).pin_memory()

    def batch_call():
        _ffi.check(lib.nsgb_chain_batch(C.byref(batch), 8, thr, 4, 8, 11, 1000, None, None,
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream), C.byref(async_opts)),
                   "chain_batch")
        _ffi.check(lib.nsgb_batch_counts_async(C.byref(batch), counts.data_ptr(),
                                               C.c_void_p(torch.cuda.current_stream().cuda_stream)),
                   "batch_counts_async")

    work.buf.copy_(marker.buf)
    batch_call()  # warm the launch path outside the capture
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    cs = torch.cuda.Stream()
    cs.wait_stream(stream)
    with torch.cuda.stream(cs):
        graph.capture_begin()
        batch_call()
        graph.capture_end()
    stream.wait_stream(cs)
    torch.cuda.synchronize()

    def timed(fn, steps, warmup):
        res = []
        for k in range(warmup + steps):
            work.buf.copy_(marker.buf)  # marker restore, outside the events
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            if k >= warmup:
                res.append(a.elapsed_time(b))
        return statistics.mean(res)

    steps, warm = args.batch_steps, 3
    mp = total_px / 1e6
    if args.batch_only:
        t_batch = timed(graph.replay, steps, warm)
        return {"batched_graph_mpix_s": mp / (t_batch / 1e3), "batched_ms": t_batch}
    t_plain = timed(lambda: plain(True), steps, warm)
    t_plain_async = timed(lambda: plain(False), steps, warm)
    plain(True)  # leave the plain outputs of an exact run (work restored by the last timed step)
    torch.cuda.synchronize()
    pc = [(a.value, b.value) for a, b in plain_counts]
    work.buf.copy_(marker.buf)
    t_batch = timed(graph.replay, steps, warm)
    torch.cuda.synchronize()
    st = lib.nsgb_device_status(C.c_void_p(bws), sp)
    if st != 0:
        raise RuntimeError(f"batch device status: {_ffi.STATUS.get(st, st)}")
    bc = counts.view(n, 2).tolist()
    same = (all(tuple(x) == y for x, y in zip(bc, pc)) and torch.equal(bf.buf, fo.buf) and torch.equal(bl.buf, lo.buf)
            and torch.equal(ba.buf, ao.buf))
    return {
        "plain_mpix_s": mp / (t_plain / 1e3), "plain_ms": t_plain,
        "plain_async_mpix_s": mp / (t_plain_async / 1e3), "plain_async_ms": t_plain_async,
        "batched_graph_mpix_s": mp / (t_batch / 1e3), "batched_ms": t_batch,
        "speedup_vs_plain": t_plain / t_batch, "speedup_vs_plain_async": t_plain_async / t_batch,
        "batch_equals_single_tile": bool(same),
        "gpu_launches_per_batch": chain_kernels(dtype, True, total_px // max(1, n)),
    }


def cpu_tile_parallel(tiles_u8, budget_tiles):
    """The reference's own CPU chain (oracle/_ref, built from its sources; the oracle's
    restatement where that was not built), one tile per host thread, on the first
    `budget_tiles` tiles."""
    from concurrent.futures import ThreadPoolExecutor

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    ref = oracle.ref_morph_available()
    fn = oracle.ref_chain if ref else oracle.chain
    sample = tiles_u8[:budget_tiles]
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(lambda mk: fn(mk[1], mk[0]), sample))
    dt = time.perf_counter() - t0
    px = sum(m.size for m, _ in sample)
    return {"value": px / 1e6 / dt, "unit": "MPix/s", "cores": threads, "kind": "reference" if ref else "port",
            "sample": f"first {len(sample)} of the u8 tiles, one tile per thread, {dt:.1f} s"}


def combine_batched(r, px):
    """One dtype's batched figures over the ranks: the slowest rank's times, all ranks' pixels."""
    from nsgb.shard import combine

    out = dict(r)
    total = px
    for arm in ("plain", "plain_async", "batched"):
        key = "batched_ms" if arm == "batched" else f"{arm}_ms"
        if key in r:
            out[key], total = combine(r[key], px)
    mp = total / 1e6
    if "plain_ms" in out:
        out["plain_mpix_s"] = mp / (out["plain_ms"] / 1e3)
        out["plain_async_mpix_s"] = mp / (out["plain_async_ms"] / 1e3)
        out["speedup_vs_plain"] = out["plain_ms"] / out["batched_ms"]
        out["speedup_vs_plain_async"] = out["plain_async_ms"] / out["batched_ms"]
    out["batched_graph_mpix_s"] = mp / (out["batched_ms"] / 1e3)
    if "batch_equals_single_tile" in r:
        ok, _ = combine(0.0 if r["batch_equals_single_tile"] else 1.0, 0)  # any rank that differs -> 1
        out["batch_equals_single_tile"] = ok == 0.0
    return out


def batched_section(args, dev):
    rank, world, _ = dist_info()
    tiles = batch_tiles_host(args.batch_tiles)
    all_px = int(sum(m.size for m, _ in tiles))
    if world > 1:
        from nsgb.shard import rank_tiles

        tiles = [tiles[i] for i in rank_tiles([m.size for m, _ in tiles], world, rank)]
    res = {"workload": f"{args.batch_tiles} tiles, H and W i.i.d. uniform in [256,4096], 1 ellipse per 2800 px^2, "
                       "chain (a)-(e) per tile; u16 = u8 x 257, i32 = u8 x 1000 (threshold scaled the same way)",
           "total_px": all_px,
           "sharding": (f"tiles split over {world} ranks by pixel count (largest first onto the least-loaded "
                        f"rank), no exchange; times are the slowest rank's") if world > 1 else "one GPU",
           "plain": "nsgb_chain per tile on one stream, counts read per tile (the reference API returns them)",
           "plain_async": "nsgb_chain per tile on one stream, no count reads",
           "batched": "nsgb_chain_batch + nsgb_batch_counts_async recorded once in a CUDA graph, replayed",
           "l2": "inputs larger than L2; marker restore outside the timed events"}
    my_px = int(sum(m.size for m, _ in tiles))
    for d in [x for x in args.batch_dtypes.split(",") if x]:
        r = run_batched(args, dev, tiles, d)
        res[d] = combine_batched(r, my_px) if world > 1 else r
    if not args.no_cpu_baseline and world == 1:
        res["cpu_tile_parallel"] = cpu_tile_parallel(tiles, 2 * (os.cpu_count() or 1))
    return res


# -- differentiable float32 reconstruction ----------------------------------------------------
def event_ms(fn, steps, warmup, stream):
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(steps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def grad_section(dev, steps=5):
    """16 x 2048 x 2048 float32: forward with provenance, adjoint of an N(0,1) upstream gradient."""
    import numpy as np
    import torch

    from nsgb import _ffi, synth

    lib = _ffi.lib
    B, H, W = 16, 2048, 2048
    mask_h, marker_h = synth.float_pair((B, H, W), 0)
    g_h = np.random.default_rng(0).standard_normal((B, H, W)).astype(np.float32)
    marker, mask, g = (torch.from_numpy(a).to(dev) for a in (marker_h, mask_h, g_h))
    out = torch.empty_like(mask)
    prov = torch.empty((B, H, W), dtype=torch.int32, device=dev)
    dm, dk = torch.empty_like(mask), torch.empty_like(mask)
    wsz = [lib.nsgb_recon_f32_workspace_size(B, H, W, k) for k in (0, 1)]
    wst = [torch.empty(n + 256, dtype=torch.uint8, device=dev) for n in wsz]
    ws = [(t.data_ptr() + 255) & ~255 for t in wst]
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    opts = _ffi.Opts(0, 0, 0)

    def fwd():
        _ffi.check(lib.nsgb_recon_f32_fwd(marker.data_ptr(), mask.data_ptr(), out.data_ptr(), prov.data_ptr(), B, H, W,
                                          W * 4, H * W * 4, 8, ws[0], wsz[0], sp, C.byref(opts)), "recon_f32_fwd")

    def bwd():
        _ffi.check(lib.nsgb_recon_f32_bwd(g.data_ptr(), prov.data_ptr(), dm.data_ptr(), dk.data_ptr(), B, H, W, W * 4,
                                          H * W * 4, ws[1], wsz[1], sp, C.byref(opts)), "recon_f32_bwd")

    t_fwd = event_ms(fwd, steps, 3, stream)
    t_bwd = event_ms(bwd, steps, 3, stream)
    for w in ws:
        st = lib.nsgb_device_status(C.c_void_p(w), sp)
        if st != 0:
            raise RuntimeError(f"recon_f32 device status {_ffi.STATUS.get(st, st)}")
    px = B * H * W
    return {"workload": "16 x 2048 x 2048 float32, mask U[0,1), marker = mask * U[0.5,1), 8-connected; "
                        "upstream gradient N(0,1)",
            "forward_ms": t_fwd, "backward_ms": t_bwd, "backward_over_forward": t_bwd / t_fwd,
            "forward_mpix_s": px / 1e6 / (t_fwd / 1e3), "backward_mpix_s": px / 1e6 / (t_bwd / 1e3),
            "forward_algorithmic_GBps": 16 * px / (t_fwd / 1e3) / 1e9,
            "backward_algorithmic_GBps": 16 * px / (t_bwd / 1e3) / 1e9,
            "bytes_per_px": "16 each way (fwd: marker, mask, out, prov; bwd: g, prov, dmarker, dmask)"}


# -- per-label bounding boxes ---------------------------------------------------------------------
def bbox_section(args, dev, steps=20):
    """ConnComponents::boundingBox after bwlabel (HistologicalEntities.cpp:573) on the dark objects
    of the headline tile (thousands of components): raster labels in, boxes in raster order of
    first appearance out."""
    import torch

    from nsgb import _ffi, synth

    lib = _ffi.lib
    H = W = args.size
    mask_h, _ = synth.tile_u8(H, W, args.ellipses, 0)
    binary = ((torch.from_numpy(mask_h).to(dev) < 128).to(torch.uint8) * 255).contiguous()
    labels = torch.empty((H, W), dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    lws_n = lib.nsgb_workspace_size(_ffi.OP_BWLABEL, _ffi.U8, H, W)
    lws_t = torch.empty(lws_n + 256, dtype=torch.uint8, device=dev)
    lws = (lws_t.data_ptr() + 255) & ~255
    n_lab = C.c_int32(0)
    _ffi.check(lib.nsgb_bwlabel(binary.data_ptr(), labels.data_ptr(), H, W, W, W * 4, 8, 1, C.byref(n_lab), lws,
                                lws_n, sp, None), "bwlabel")
    bws_n = lib.nsgb_workspace_size(_ffi.OP_BOUNDING_BOX, _ffi.I32, H, W)
    bws_t = torch.empty(bws_n + 256, dtype=torch.uint8, device=dev)
    bws = (bws_t.data_ptr() + 255) & ~255
    cap = max(int(n_lab.value), 1)
    boxes = torch.empty((5, cap), dtype=torch.int32, device=dev)
    count_dev = torch.zeros(1, dtype=torch.int32, device=dev)
    opts = _ffi.Opts(0, 0, 0)

    def f_box():
        _ffi.check(lib.nsgb_bounding_boxes(labels.data_ptr(), H, W, W * 4, 0, boxes.data_ptr(), cap, None,
                                           count_dev.data_ptr(), bws, bws_n, sp, C.byref(opts)), "bounding_boxes")

    t = event_ms(f_box, steps, 3, stream)
    st = lib.nsgb_device_status(C.c_void_p(bws), sp)
    if st != 0:
        raise RuntimeError(f"bounding boxes: device status {_ffi.STATUS.get(st, st)}")
    n_box = int(count_dev.item())
    if n_box != int(n_lab.value):
        raise RuntimeError(f"bounding boxes: {n_box} boxes for {n_lab.value} labels")
    return {"workload": f"{H}x{W} raster labels of the dark objects of the headline tile (mask < 128, "
                        f"bwlabel 8-conn relabel), background 0",
            "components": n_box, "ms": t, "mpix_s": H * W / 1e3 / t}


# -- S1 after the colour steps: opening and nucleus-candidate stage ------------------------------
# recon init + recon, bw1 filled and labelled at once (zeroing, local, merge, border walk,
# parent join, flatten) + kept count, bw2 label (local, merge, flatten), seeds, output:
# csrc/ops.cu candidates_impl
CANDIDATE_KERNELS = 14
OPEN_KERNELS = 2  # erosion, dilation (csrc/morph.cu)


def timed_steps(stream, steps, before, call):
    """Mean / median ms of `call` over `steps` runs, each after an untimed `before`."""
    import torch

    for _ in range(3):
        before()
        call()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for a, b in evs:
        before()
        a.record(stream)
        call()
        b.record(stream)
    torch.cuda.synchronize()
    ms = sorted(a.elapsed_time(b) for a, b in evs)
    return sum(ms) / len(ms), ms[len(ms) // 2]


def candidates_section(args, dev, steps=20):
    """S1 of plFindNucleusCandidates after the colour steps (HistologicalEntities.cpp:184-275) on
    the headline tile: rc = the inverted tile (nuclei bright), rc_open = morphOpen(rc, 19 x 19
    disk), then the candidate stage with rbc = dark objects of a second tile.  Timed: the opening
    alone, the candidate stage alone (rc_open restored untimed), and both back to back from rc.
    L2 flushed before every step."""
    import numpy as np
    import torch

    from nsgb import _ffi, disk19, synth

    lib = _ffi.lib
    H = W = args.size
    mask_h, _ = synth.tile_u8(H, W, args.ellipses, 0)
    rc_h = (255 - mask_h).astype(np.uint8)
    other_h, _ = synth.tile_u8(H, W, args.ellipses // 4, 1)
    rbc_h = np.where(other_h < 128, 255, 0).astype(np.uint8)
    rc, rbc = (torch.from_numpy(a).to(dev) for a in (rc_h, rbc_h))
    open_src = torch.empty_like(rc)
    work = torch.empty_like(rc)
    seg = torch.empty_like(rc)
    kern = np.ascontiguousarray(disk19())
    kp = kern.ctypes.data_as(C.c_void_p)
    nb_c = lib.nsgb_workspace_size(_ffi.OP_NUCLEUS_CANDIDATES, _ffi.U8, H, W)
    nb_o = lib.nsgb_workspace_size(_ffi.OP_MORPH_OPEN, _ffi.U8, H, W)
    ws_t = [torch.empty(n + 256, dtype=torch.uint8, device=dev) for n in (nb_c, nb_o)]
    ws_c, ws_o = [(t.data_ptr() + 255) & ~255 for t in ws_t]
    n_dev = torch.zeros(1, dtype=torch.int32, device=dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    opts = _ffi.Opts(0, 0, 0)

    def open_into(dst):
        _ffi.check(lib.nsgb_morph_open(rc.data_ptr(), dst.data_ptr(), H, W, W, W, kp, 19, ws_o, nb_o, sp,
                                       C.byref(opts)), "morph_open")

    def candidates():
        _ffi.check(lib.nsgb_nucleus_candidates(work.data_ptr(), rc.data_ptr(), rbc.data_ptr(), seg.data_ptr(), H, W, W,
                                               80.0, 45.0, 11, 1000, None, n_dev.data_ptr(), ws_c, nb_c, sp,
                                               C.byref(opts)), "nucleus_candidates")

    def restore():
        work.copy_(open_src)
        flush.fill_(1)

    open_into(open_src)
    t_open, t_open_med = timed_steps(stream, steps, lambda: flush.fill_(1), lambda: open_into(work))
    t_cand, t_cand_med = timed_steps(stream, steps, restore, candidates)
    t_s1, t_s1_med = timed_steps(stream, steps, lambda: flush.fill_(1), lambda: (open_into(work), candidates()))
    for w in (ws_c, ws_o):
        st = lib.nsgb_device_status(C.c_void_p(w), sp)
        if st != 0:
            raise RuntimeError(f"S1: device status {_ffi.STATUS.get(st, st)}")
    px = H * W
    res = {"workload": f"{H}x{W} u8: rc = 255 - headline tile, rc_open = morphOpen(rc, 19x19 disk), rbc = mask < 128 "
                       f"of a second tile ({args.ellipses // 4} ellipses); G1 80, G2 45, areas [11, 1000)",
           "kept_components": int(n_dev.item()), "candidate_px": int((seg != 0).sum().item()),
           "open_ms": t_open, "open_mpix_s": px / 1e3 / t_open,
           "open_algorithmic_GBps": 4 * px / (t_open / 1e3) / 1e9,
           "open_bytes_per_px": "4 (erosion: read, write; dilation: read, write)",
           "candidates_ms": t_cand, "candidates_mpix_s": px / 1e3 / t_cand,
           "s1_ms": t_s1, "s1_mpix_s": px / 1e3 / t_s1,
           "medians_ms": {"open": t_open_med, "candidates": t_cand_med, "s1": t_s1_med},
           "gpu_launches_per_s1": OPEN_KERNELS + CANDIDATE_KERNELS,
           "l2": "flushed before every step (512 MB write)"}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        strip = 512
        t0 = time.perf_counter()
        oracle.morph_open(rc_h[:strip], kern)
        t_o = time.perf_counter() - t0
        open_h = open_src.cpu().numpy()
        t0 = time.perf_counter()
        _, n_exp = oracle.nucleus_candidates(rc_h, open_h, rbc_h)
        t_c = time.perf_counter() - t0
        s1_s = t_o * H / strip + t_c
        res["cpu_baseline"] = {"value": px / 1e6 / s1_s, "unit": "MPix/s", "cores": 1, "kind": "port",
                               "sample": f"oracle opening of a {strip}x{W} strip ({t_o:.2f} s, scaled to {H} rows) "
                                         f"plus the candidate stage on the full tile ({t_c:.2f} s), one host core",
                               "same_kept_count": n_exp == res["kept_components"]}
    return res


def distance_section(args, dev, steps=20):
    """The distance map and watershed basins of S2 (HistologicalEntities.cpp:341-356) for the dark
    objects of the headline tile (mask < 128): exact Euclidean distance to the nearest zero pixel,
    -distance on the objects, -FLT_MAX elsewhere.  L2 flushed before every step."""
    import numpy as np
    import torch

    from nsgb import _ffi, synth

    lib = _ffi.lib
    H = W = args.size
    mask_h, _ = synth.tile_u8(H, W, args.ellipses, 0)
    m_h = np.where(mask_h < 128, 255, 0).astype(np.uint8)
    m = torch.from_numpy(m_h).to(dev)
    out = torch.empty((H, W), dtype=torch.float32, device=dev)
    nb = lib.nsgb_workspace_size(_ffi.OP_DISTANCE, _ffi.U8, H, W)
    ws_t = torch.empty(nb + 256, dtype=torch.uint8, device=dev)
    ws = (ws_t.data_ptr() + 255) & ~255
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    opts = _ffi.Opts(0, 0, 0)

    def call():
        _ffi.check(lib.nsgb_distance_transform(m.data_ptr(), out.data_ptr(), H, W, W, W * 4, 1, ws, nb, sp,
                                               C.byref(opts)), "distance_transform")

    t, t_med = timed_steps(stream, steps, lambda: flush.fill_(1), call)
    st = lib.nsgb_device_status(C.c_void_p(ws), sp)
    if st != 0:
        raise RuntimeError(f"distance: device status {_ffi.STATUS.get(st, st)}")
    px = H * W
    res = {"workload": f"{H}x{W} u8 mask (dark objects of the headline tile, mask < 128), basins output",
           "object_px": int(m_h.astype(bool).sum()), "ms": t, "ms_median": t_med, "mpix_s": px / 1e3 / t,
           "gpu_launches_per_call": 3, "l2": "flushed before every step (512 MB write)"}
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        t0 = time.perf_counter()
        oracle.distance_queue(m_h)
        t_q = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": px / 1e6 / t_q, "unit": "MPix/s", "cores": 1, "kind": "port",
                               "sample": f"the reference's queue-based distanceTransform restated, full tile, "
                                         f"{t_q:.2f} s, one host core"}
    return res


# -- large single image -------------------------------------------------------------------------
def large_section(args, dev, steps=3):
    """16384 x 16384 with ~102k ellipses: hole filling (reconstruction by erosion), threshold,
    bwlabel (8-conn), per dtype and fill connectivity; per-stage algorithmic GB/s."""
    import torch

    from nsgb import _ffi, synth

    lib = _ffi.lib
    N = args.large_size
    img8, _ = synth.tile_u8(N, N, int(round(N * N / 2621)), 0)
    stream = torch.cuda.current_stream()
    sp = C.c_void_p(stream.cuda_stream)
    opts = _ffi.Opts(0, 0, 0)
    binary = torch.empty((N, N), dtype=torch.uint8, device=dev)
    labels = torch.empty((N, N), dtype=torch.int32, device=dev)
    lws_n = lib.nsgb_workspace_size(_ffi.OP_BWLABEL, _ffi.U8, N, N)
    lws_t = torch.empty(lws_n + 256, dtype=torch.uint8, device=dev)
    lws = (lws_t.data_ptr() + 255) & ~255
    res = {"workload": f"{N}x{N}, {int(round(N * N / 2621))} ellipses; imfillHoles (grayscale, reconstruction by "
                       f"erosion), threshold > 128 x scale, bwlabel 8-conn relabel; device-resident",
           "bytes_per_px": "fill 2*s (image read, result written), threshold s+1, bwlabel 5"}
    peak, _ = read_peaks()
    for dt in [d for d in args.large_dtypes.split(",") if d]:
        img_h = img8 if dt == "u8" else synth.scale(img8, dt)[0]
        code = {"u8": _ffi.U8, "u16": _ffi.U16, "i32": _ffi.I32}[dt]
        esz = img_h.dtype.itemsize
        img = torch.from_numpy(img_h).to(dev)
        fill = torch.empty_like(img)
        fws_n = lib.nsgb_workspace_size(_ffi.OP_FILL_HOLES, code, N, N)
        fws_t = torch.empty(fws_n + 256, dtype=torch.uint8, device=dev)
        fws = (fws_t.data_ptr() + 255) & ~255
        thr = 128.0 * BATCH_SCALE[dt]
        for conn in (4, 8):
            def f_fill():
                _ffi.check(lib.nsgb_imfill_holes(code, img.data_ptr(), fill.data_ptr(), N, N, N * esz, 0, conn, fws,
                                                 fws_n, sp, C.byref(opts)), "imfill_holes")

            def f_thr():
                _ffi.check(lib.nsgb_threshold(code, fill.data_ptr(), binary.data_ptr(), N, N, N * esz, N, thr, sp),
                           "threshold")

            def f_lab():
                _ffi.check(lib.nsgb_bwlabel(binary.data_ptr(), labels.data_ptr(), N, N, N, N * 4, 8, 1, None, lws,
                                            lws_n, sp, C.byref(opts)), "bwlabel")

            t_fill = event_ms(f_fill, steps, 3, stream)
            t_thr = event_ms(f_thr, steps, 3, stream)
            t_lab = event_ms(f_lab, steps, 3, stream)
            for w in (fws, lws):
                st = lib.nsgb_device_status(C.c_void_p(w), sp)
                if st != 0:
                    raise RuntimeError(f"large {dt}: device status {_ffi.STATUS.get(st, st)}")
            px = N * N
            gbs = {"fill": 2 * esz * px / (t_fill / 1e3) / 1e9, "threshold": (esz + 1) * px / (t_thr / 1e3) / 1e9,
                   "bwlabel": 5 * px / (t_lab / 1e3) / 1e9}
            res[f"{dt}_conn{conn}"] = {
                "fill_ms": t_fill, "threshold_ms": t_thr, "bwlabel_ms": t_lab,
                "chain_mpix_s": px / 1e6 / ((t_fill + t_thr + t_lab) / 1e3),
                "GBps": gbs, "frac_of_hbm": {k: v / peak for k, v in gbs.items()}}
        del img, fill, fws_t
        torch.cuda.empty_cache()
    return res


def link_bound_s(in_bytes, out_bytes, d2h_gbps, h2d_gbps, both_gbps):
    """Seconds a step's copies need on the host link: both directions start together at the
    concurrent rate; once the smaller transfer is done the rest of the larger one runs at its
    direction's solo rate."""
    lo, hi = min(in_bytes, out_bytes), max(in_bytes, out_bytes)
    solo = d2h_gbps if out_bytes >= in_bytes else h2d_gbps
    return lo / (both_gbps * 1e9) + (hi - lo) / (solo * 1e9)


def host_link(dev, in_bytes, out_bytes, px, reps=5):
    """The host link's own bound on an end-to-end step: pinned-memory copy bandwidth measured
    in this process (device -> host alone, host -> device alone, and both directions at once on
    two streams), and the time a step's copies need at those rates when its inputs go in while
    its outputs come out (the directions share the link: the smaller transfer runs at the
    concurrent rate, the rest of the larger one at its solo rate)."""
    import torch

    n = max(in_bytes, out_bytes)
    d_out = torch.empty(n, dtype=torch.uint8, device=dev)
    d_in = torch.empty(n, dtype=torch.uint8, device=dev)
    h_out = torch.empty(n, dtype=torch.uint8).pin_memory()
    h_in = torch.zeros(n, dtype=torch.uint8).pin_memory()
    s1, s2 = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

    def timed(d2h, h2d):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        ev[0].record(s1)
        s2.wait_event(ev[0])
        for _ in range(reps):
            if d2h:
                with torch.cuda.stream(s1):
                    h_out.copy_(d_out, non_blocking=True)
            if h2d:
                with torch.cuda.stream(s2):
                    d_in.copy_(h_in, non_blocking=True)
        s1.wait_stream(s2)
        ev[1].record(s1)
        torch.cuda.synchronize()
        return n * reps / (ev[0].elapsed_time(ev[1]) / 1e3) / 1e9

    timed(True, True)  # warm-up
    d2h, h2d, both = timed(True, False), timed(False, True), timed(True, True)
    bound_s = link_bound_s(in_bytes, out_bytes, d2h, h2d, both)
    return {"d2h_GBps": d2h, "h2d_GBps": h2d, "concurrent_GBps_per_direction": both,
            "bound_ms_per_step": bound_s * 1e3, "bound_mpix_s": px / 1e6 / bound_s,
            "note": "pinned-memory copies timed in this run; frac = e2e value / this bound"}


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_nsgb(args)


if __name__ == "__main__":
    sys.exit(main())
