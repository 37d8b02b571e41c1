"""Builds libnsgb.so (the CUDA kernels + C ABI) for sm_103a, in-tree.

Every .cu file under csrc/ is compiled with nvcc for `-gencode arch=compute_103a,code=sm_103a`
and the host-only .cpp files with g++; the objects are linked into lib/libnsgb.so.  Sources
are compiled in parallel and only when they changed.  No cmake, no torch extension machinery.
The reconstruction's tuned schedule (tuning.json, written by tune.py) is compiled in as a
generated table, _build/tuning.inc.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libnsgb.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

TUNING_JSON = os.path.join(HERE, "tuning.json")
TUNING_INC = os.path.join(OBJ, "tuning.inc")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "--expt-relaxed-constexpr", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-I", OBJ]

_DTYPE = {"u8": 0, "u16": 1, "i32": 2, "f32": 3}


def write_tuning_inc() -> None:
    """tuning.json -> the C table csrc/recon.cu includes (rewritten only when it changes)."""
    import json

    rows = []
    if os.path.exists(TUNING_JSON):
        with open(TUNING_JSON) as f:
            for e in json.load(f)["entries"]:
                rows.append("  {%d, %d, %d, %d, %dll, %d, %d, %d}," % (
                    _DTYPE[e["dtype"]], int(e["conn"]), int(bool(e["erode"])), int(bool(e["batch"])),
                    int(e["max_px"]), int(e["passes"]), int(e["order"]), int(e.get("ctas", 0))))
    rows.append("  {0, 0, 0, 0, 0ll, 0, 0, 0},  // end (max_px 0 never matches)")
    text = ("// Generated by build.py from tuning.json (tune.py); do not edit.\n"
            "// {dtype, conn, erode, batch, max_px, passes, order, queue CTAs per SM}\n"
            "static const TuneEntry kTuning[] = {\n" + "\n".join(rows) + "\n};\n")
    if not os.path.exists(TUNING_INC) or open(TUNING_INC).read() != text:
        with open(TUNING_INC, "w") as f:
            f.write(text)
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I", INCLUDE]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps(src: str) -> list[str]:
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h", ".hpp"))]
    hdrs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return [src, TUNING_INC] + hdrs


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str) -> str:
    base = os.path.splitext(os.path.basename(src))[0]
    out = os.path.join(OBJ, base + ".o")
    if not _stale(out, _deps(src)):
        return out
    if src.endswith(".cu"):
        cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, "-c", src, "-o", out]
    else:
        cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, "-c", src, "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return out


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    write_tuning_inc()
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    if _stale(LIB, objs):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose:
            print("linked", LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
