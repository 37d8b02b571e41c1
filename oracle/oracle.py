"""Python view of the CPU oracle (liboracle.so).  TEST INFRASTRUCTURE ONLY.

Restates the reference's serial algorithms (recon_oracle.hpp cites each one).  Used by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, never by the product.
`ref` (optional) is the reference's own ConnComponents.cpp compiled from its sources into
oracle/_ref/ (oracle/build_ref.sh); it exists only where the reference tree was available.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libconncomp_ref.so")

DT = {np.dtype(np.uint8): 0, np.dtype(np.uint16): 1, np.dtype(np.int32): 2, np.dtype(np.float32): 3}


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    subprocess.run([os.path.join(HERE, "build_ref.sh")], check=True, capture_output=True)


def _load() -> C.CDLL:
    if not os.path.exists(LIB):
        build()
    lib = C.CDLL(LIB)
    vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int32
    lib.orc_imreconstruct.argtypes = [C.c_int, vp, vp, i64, i64, C.c_int, vp]
    lib.orc_imreconstruct_binary.argtypes = [C.c_int, vp, vp, i64, i64, C.c_int, vp]
    lib.orc_imfill_holes.argtypes = [C.c_int, vp, i64, i64, C.c_int, C.c_int, vp]
    lib.orc_imhmin.argtypes = [C.c_int, vp, i64, i64, C.c_double, C.c_int, vp]
    lib.orc_bwselect.argtypes = [C.c_int, vp, vp, i64, i64, C.c_int, vp]
    lib.orc_threshold_gt.argtypes = [C.c_int, vp, i64, C.c_double, vp]
    lib.orc_morph_open_u8.argtypes = [vp, i64, i64, vp, C.c_int, vp]
    lib.orc_edt_exact_u8.argtypes = [vp, i64, i64, C.c_int, vp]
    lib.orc_dist_queue_u8.argtypes = [vp, i64, i64, vp]
    lib.orc_bwlabel2.argtypes = [vp, i64, i64, C.c_int, C.c_int, vp]
    lib.orc_bwlabel2.restype = i32
    lib.orc_bwareaopen2.argtypes = [vp, C.c_int, C.c_int, i32, i32, C.c_int, i64, i64, vp, vp]
    lib.orc_bwareaopen2.restype = i32
    lib.orc_bounding_box.argtypes = [vp, i64, i64, i32, vp, i64]
    lib.orc_bounding_box.restype = i32
    lib.orc_chain.argtypes = [C.c_int, vp, vp, i64, i64, C.c_int, C.c_double, C.c_int, C.c_int, i32, i32,
                              vp, vp, vp, vp, C.POINTER(i32), vp]
    lib.orc_chain.restype = i32
    lib.orc_chain_replicas_seconds.argtypes = [vp, vp, i64, i64, C.c_int, C.c_int]
    lib.orc_chain_replicas_seconds.restype = C.c_double
    lib.orc_recon_f32_prov.argtypes = [vp, vp, i64, i64, i64, C.c_int, vp, vp, C.c_int]
    lib.orc_recon_f32_prov.restype = C.c_int
    lib.orc_recon_f32_grad.argtypes = [vp, vp, i64, i64, i64, vp, vp, C.c_int]
    lib.orc_recon_f32_grad.restype = C.c_int
    lib.orc_recon_fd.argtypes = [vp, vp, vp, i64, i64, C.c_int, vp, i64, C.c_double, vp, vp, C.c_int]
    lib.nsgb_synth_tile_u8.argtypes = [vp, vp, i64, i64, i64, i64, C.c_uint64]
    return lib


lib = _load()


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _c(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a)


def synth_tile_u8(H: int, W: int, n_ellipses: int, seed: int = 0):
    """(mask, marker) of the seeded generator (csrc/synth.cpp, built into liboracle.so), the
    same bytes as nsgb.synth.tile_u8, for CPU-only processes."""
    mask = np.empty((H, W), np.uint8)
    marker = np.empty((H, W), np.uint8)
    if lib.nsgb_synth_tile_u8(_p(mask), _p(marker), H, W, W, n_ellipses, seed) != 0:
        raise ValueError("bad synth arguments")
    return mask, marker


def imreconstruct(seeds: np.ndarray, image: np.ndarray, conn: int) -> np.ndarray:
    seeds, image = _c(seeds), _c(image)
    out = np.empty_like(image)
    assert lib.orc_imreconstruct(DT[image.dtype], _p(seeds), _p(image), image.shape[0], image.shape[1], conn,
                                 _p(out)) == 0
    return out


def imreconstruct_binary(seeds: np.ndarray, image: np.ndarray, conn: int) -> np.ndarray:
    seeds, image = _c(seeds), _c(image)
    out = np.empty_like(image)
    assert lib.orc_imreconstruct_binary(DT[image.dtype], _p(seeds), _p(image), image.shape[0], image.shape[1],
                                        conn, _p(out)) == 0
    return out


def imfill_holes(image: np.ndarray, binary: bool, conn: int) -> np.ndarray:
    image = _c(image)
    out = np.empty_like(image)
    assert lib.orc_imfill_holes(DT[image.dtype], _p(image), image.shape[0], image.shape[1], int(binary), conn,
                                _p(out)) == 0
    return out


def imhmin(image: np.ndarray, h: float, conn: int) -> np.ndarray:
    image = _c(image)
    out = np.empty_like(image)
    assert lib.orc_imhmin(DT[image.dtype], _p(image), image.shape[0], image.shape[1], float(h), conn, _p(out)) == 0
    return out


def bwselect(image: np.ndarray, seeds: np.ndarray, conn: int) -> np.ndarray:
    image, seeds = _c(image), _c(seeds)
    out = np.empty_like(image)
    assert lib.orc_bwselect(DT[image.dtype], _p(image), _p(seeds), image.shape[0], image.shape[1], conn,
                            _p(out)) == 0
    return out


def morph_open(image: np.ndarray, kernel: np.ndarray) -> np.ndarray:
    """morphOpen<unsigned char> (MorphologicOperations.cpp:2459-2493), u8 image, k x k element."""
    image = _c(image).astype(np.uint8, copy=False)
    kernel = _c((np.asarray(kernel) != 0).astype(np.uint8))
    out = np.empty_like(image)
    assert lib.orc_morph_open_u8(_p(image), image.shape[0], image.shape[1], _p(kernel), kernel.shape[0],
                                 _p(out)) == 0
    return out


def distance_transform(mask: np.ndarray, basins: bool = False) -> np.ndarray:
    """Exact distance to the nearest zero pixel, float32 (HistologicalEntities.cpp:341's map);
    basins: -distance on non-zero pixels, -FLT_MAX on zero pixels (347-356)."""
    mask = _c(mask).astype(np.uint8, copy=False)
    out = np.empty(mask.shape, np.float32)
    assert lib.orc_edt_exact_u8(_p(mask), mask.shape[0], mask.shape[1], int(basins), _p(out)) == 0
    return out


def distance_queue(mask: np.ndarray) -> np.ndarray:
    """The reference's queue-based nscale::distanceTransform (MorphologicOperations.cpp:197-275)."""
    mask = _c(mask).astype(np.uint8, copy=False)
    out = np.empty(mask.shape, np.float32)
    assert lib.orc_dist_queue_u8(_p(mask), mask.shape[0], mask.shape[1], _p(out)) == 0
    return out


def threshold_gt(image: np.ndarray, thr: float) -> np.ndarray:
    image = _c(image)
    out = np.empty(image.shape, np.uint8)
    assert lib.orc_threshold_gt(DT[image.dtype], _p(image), image.size, float(thr), _p(out)) == 0
    return out


def bwlabel2(binary: np.ndarray, conn: int, relab: bool):
    binary = _c(binary).astype(np.uint8, copy=False)
    out = np.empty(binary.shape, np.int32)
    n = lib.orc_bwlabel2(_p(binary), binary.shape[0], binary.shape[1], conn, int(relab), _p(out))
    return out, int(n)


def bwareaopen2(image: np.ndarray, labeled: bool, flatten: bool, lo: int, hi: int, conn: int):
    image = _c(image)
    H, W = image.shape
    labels = np.empty((H, W), np.int32)
    flat = np.empty((H, W), np.uint8)
    cnt = lib.orc_bwareaopen2(_p(image), int(labeled), int(flatten), lo, hi, conn, H, W, _p(labels), _p(flat))
    return (flat if flatten else labels), int(cnt)


def bounding_box(labels: np.ndarray, bgval: int = 0) -> np.ndarray:
    """ConnComponents::boundingBox (ConnComponents.cpp:241-284): int32 array (5, count) of
    label, min x, max x, min y, max y per label other than bgval, in order of first appearance
    in raster order."""
    labels = _c(labels).astype(np.int32)
    H, W = labels.shape
    cap = H * W
    out = np.zeros((5, max(cap, 1)), np.int32)
    n = lib.orc_bounding_box(_p(labels), H, W, bgval, _p(out), max(cap, 1))
    return np.ascontiguousarray(out[:, :n])


def chain(marker: np.ndarray, mask: np.ndarray, recon_conn=8, thr=128.0, fill_conn=4, label_conn=8, lo=11,
          hi=1000):
    marker, mask = _c(marker), _c(mask)
    H, W = mask.shape
    rec = np.empty_like(mask)
    b = np.empty((H, W), np.uint8)
    f = np.empty((H, W), np.uint8)
    lab = np.empty((H, W), np.int32)
    a = np.empty((H, W), np.uint8)
    nl = C.c_int32(0)
    kept = lib.orc_chain(DT[mask.dtype], _p(marker), _p(mask), H, W, recon_conn, float(thr), fill_conn, label_conn,
                         lo, hi, _p(rec), _p(b), _p(f), _p(lab), C.byref(nl), _p(a))
    return {"recon": rec, "thr": b, "fill": f, "labels": lab, "n_labels": int(nl.value), "area": a,
            "n_kept": int(kept)}


def nucleus_candidates(rc: np.ndarray, rc_open: np.ndarray, rbc: np.ndarray, g1=80.0, g2=45.0, lo=11, hi=1000):
    """The candidate stage of HistologicalEntities::plFindNucleusCandidates after the opening
    (src/segment/HistologicalEntities.cpp:195-275), composed from the restated steps:
    recon 8-conn (195), diffIm = rc - recon saturating (199), imfillHoles(diffIm > G1, binary, 4)
    (214-219), bwareaopen2(.., false, true, lo, hi, 8) (247), bwselect(diffIm > G2, bw1_t, 8)
    (268) and `& (rbc == 0)` (271).  Returns (seg_norbc, compcount2)."""
    rc, rc_open, rbc = _c(rc), _c(rc_open), _c(rbc)
    rec = imreconstruct(rc_open, rc, 8)
    diff = np.where(rc > rec, rc.astype(np.int16) - rec, 0).astype(np.uint8)
    bw1 = imfill_holes(threshold_gt(diff, g1), True, 4)
    bw1_t, n = bwareaopen2(bw1, False, True, lo, hi, 8)
    seg = bwselect(threshold_gt(diff, g2), bw1_t, 8)
    return np.where(rbc == 0, seg, 0).astype(np.uint8), n


def chain_replicas_seconds(marker: np.ndarray, mask: np.ndarray, threads: int, reps: int) -> float:
    marker, mask = _c(marker), _c(mask)
    return float(lib.orc_chain_replicas_seconds(_p(marker), _p(mask), mask.shape[0], mask.shape[1], threads, reps))


# -- the reference's own ConnComponents (only where it was built) ---------------------------
def ref_available() -> bool:
    return os.path.exists(REF_LIB)


# -- the reference's own serial reconstruction functions (only where they were built) ------
# libmorph_ref.so follows OpenCV's CV_32S arithmetic (wrap-around); libmorph_ref_sat.so is the
# same code with saturating CV_32S arithmetic (the reading the oracle takes for
# invert<int>(INT_MIN)).  See oracle/ref_morph.cpp and oracle/cv_shim.hpp.
REF_MORPH_LIB = os.path.join(HERE, "_ref", "libmorph_ref.so")
REF_MORPH_SAT_LIB = os.path.join(HERE, "_ref", "libmorph_ref_sat.so")


def ref_morph_available() -> bool:
    return os.path.exists(REF_MORPH_LIB) and os.path.exists(REF_MORPH_SAT_LIB)


_ref_morph_libs = {}


def _ref_morph(saturate_32s: bool = False) -> C.CDLL:
    key = bool(saturate_32s)
    if key not in _ref_morph_libs:
        r = C.CDLL(REF_MORPH_SAT_LIB if key else REF_MORPH_LIB)
        vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int32
        r.ref_imreconstruct.argtypes = [C.c_int, vp, vp, i64, i64, C.c_int, vp]
        r.ref_imreconstruct_binary.argtypes = [C.c_int, vp, vp, i64, i64, C.c_int, vp]
        r.ref_imfill_holes.argtypes = [C.c_int, vp, i64, i64, C.c_int, C.c_int, vp]
        r.ref_imhmin.argtypes = [C.c_int, vp, i64, i64, C.c_double, C.c_int, vp]
        r.ref_bwselect.argtypes = [C.c_int, vp, vp, i64, i64, C.c_int, vp]
        r.ref_threshold_gt.argtypes = [C.c_int, vp, i64, i64, C.c_double, vp]
        r.ref_bwlabel2.argtypes = [vp, i64, i64, C.c_int, C.c_int, vp]
        r.ref_bwlabel2.restype = C.c_int
        r.ref_bwareaopen2.argtypes = [vp, C.c_int, C.c_int, i32, i32, C.c_int, i64, i64, vp]
        r.ref_bwareaopen2.restype = C.c_int
        r.ref_chain.argtypes = [C.c_int, vp, vp, i64, i64, C.c_int, C.c_double, C.c_int, C.c_int, i32, i32,
                                vp, vp, vp, vp, C.POINTER(i32), vp]
        r.ref_chain.restype = i32
        r.ref_chain_replicas_seconds.argtypes = [vp, vp, i64, i64, C.c_int, C.c_int]
        r.ref_chain_replicas_seconds.restype = C.c_double
        _ref_morph_libs[key] = r
    return _ref_morph_libs[key]


def ref_imreconstruct(seeds, image, conn, saturate_32s=False):
    seeds, image = _c(seeds), _c(image)
    out = np.empty_like(image)
    rc = _ref_morph(saturate_32s).ref_imreconstruct(DT[image.dtype], _p(seeds), _p(image), *image.shape, conn,
                                                    _p(out))
    assert rc == 0, rc
    return out


def ref_imreconstruct_binary(seeds, image, conn, saturate_32s=False):
    seeds, image = _c(seeds), _c(image)
    out = np.empty_like(image)
    rc = _ref_morph(saturate_32s).ref_imreconstruct_binary(DT[image.dtype], _p(seeds), _p(image), *image.shape,
                                                           conn, _p(out))
    assert rc == 0, rc
    return out


def ref_imfill_holes(image, binary, conn, saturate_32s=False):
    image = _c(image)
    out = np.empty_like(image)
    rc = _ref_morph(saturate_32s).ref_imfill_holes(DT[image.dtype], _p(image), *image.shape, int(binary), conn,
                                                   _p(out))
    assert rc == 0, rc
    return out


def ref_imhmin(image, h, conn, saturate_32s=False):
    image = _c(image)
    out = np.empty_like(image)
    rc = _ref_morph(saturate_32s).ref_imhmin(DT[image.dtype], _p(image), *image.shape, float(h), conn, _p(out))
    assert rc == 0, rc
    return out


def ref_bwselect(image, seeds, conn, saturate_32s=False):
    image, seeds = _c(image), _c(seeds)
    out = np.empty_like(image)
    rc = _ref_morph(saturate_32s).ref_bwselect(DT[image.dtype], _p(image), _p(seeds), *image.shape, conn, _p(out))
    assert rc == 0, rc
    return out


def ref_threshold_gt(image, thr):
    image = _c(image)
    out = np.empty(image.shape, np.uint8)
    assert _ref_morph().ref_threshold_gt(DT[image.dtype], _p(image), *image.shape, float(thr), _p(out)) == 0
    return out


def ref_bwlabel2(binary, conn, relab):
    binary = _c(binary).astype(np.uint8, copy=False)
    out = np.empty(binary.shape, np.int32)
    n = _ref_morph().ref_bwlabel2(_p(binary), *binary.shape, conn, int(relab), _p(out))
    assert n >= 0
    return out, int(n)


def ref_bwareaopen2(image, labeled, flatten, lo, hi, conn):
    image = _c(image)
    out = np.empty(image.shape, np.uint8 if flatten else np.int32)
    n = _ref_morph().ref_bwareaopen2(_p(image), int(labeled), int(flatten), lo, hi, conn, *image.shape, _p(out))
    assert n >= 0
    return out, int(n)


def ref_chain(marker, mask, recon_conn=8, thr=128.0, fill_conn=4, label_conn=8, lo=11, hi=1000):
    marker, mask = _c(marker), _c(mask)
    H, W = mask.shape
    rec = np.empty_like(mask)
    b = np.empty((H, W), np.uint8)
    f = np.empty((H, W), np.uint8)
    lab = np.empty((H, W), np.int32)
    a = np.empty((H, W), np.uint8)
    nl = C.c_int32(0)
    kept = _ref_morph().ref_chain(DT[mask.dtype], _p(marker), _p(mask), H, W, recon_conn, float(thr), fill_conn,
                                  label_conn, lo, hi, _p(rec), _p(b), _p(f), _p(lab), C.byref(nl), _p(a))
    assert kept >= 0
    return {"recon": rec, "thr": b, "fill": f, "labels": lab, "n_labels": int(nl.value), "area": a,
            "n_kept": int(kept)}


def ref_chain_replicas_seconds(marker, mask, threads: int, reps: int) -> float:
    marker, mask = _c(marker), _c(mask)
    t = _ref_morph().ref_chain_replicas_seconds(_p(marker), _p(mask), mask.shape[0], mask.shape[1], threads, reps)
    if t < 0:
        raise RuntimeError("the reference chain failed")
    return float(t)


def _ref() -> C.CDLL:
    r = C.CDLL(REF_LIB)
    r.ref_cc_label.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int]
    r.ref_cc_relabel.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_int]
    r.ref_cc_relabel.restype = C.c_int
    r.ref_cc_area_threshold_labeled.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int]
    r.ref_cc_area_threshold_labeled.restype = C.c_int
    r.ref_cc_bounding_box.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int]
    r.ref_cc_bounding_box.restype = C.c_int
    return r


def ref_label(img: np.ndarray, conn: int, relab: bool):
    r = _ref()
    img = _c(img).astype(np.uint8).copy()
    H, W = img.shape
    out = np.empty((H, W), np.int32)
    r.ref_cc_label(_p(img), W, H, _p(out), -1, conn)
    n = r.ref_cc_relabel(W, H, _p(out), -1) if relab else 0
    return out, int(n)


def ref_area_threshold_labeled(labels: np.ndarray, lo: int, hi: int):
    r = _ref()
    labels = _c(labels).astype(np.int32)
    H, W = labels.shape
    out = np.empty((H, W), np.int32)
    n = r.ref_cc_area_threshold_labeled(_p(labels), W, H, _p(out), -1, lo, hi)
    return out, int(n)


def ref_bounding_box(labels: np.ndarray, bgval: int = 0) -> np.ndarray:
    r = _ref()
    labels = _c(labels).astype(np.int32)
    H, W = labels.shape
    cap = max(H * W, 1)
    out = np.zeros((5, cap), np.int32)
    n = r.ref_cc_bounding_box(_p(labels), W, H, bgval, _p(out), cap)
    return np.ascontiguousarray(out[:, :n])


# -- differentiable float32 reconstruction ------------------------------------------------
def _stack(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a if a.ndim == 3 else a[None]


def recon_f32_prov(marker: np.ndarray, mask: np.ndarray, conn: int, threads: int = 0):
    """(R, prov) for one image or a stack [B, H, W] (prov: ~q mask source, q marker source,
    INT32_MIN the zero ring)."""
    squeeze = np.ndim(mask) == 2
    mk, ms = _stack(marker), _stack(mask)
    B, H, W = ms.shape
    R = np.empty_like(ms)
    prov = np.empty(ms.shape, np.int32)
    rc = lib.orc_recon_f32_prov(_p(mk), _p(ms), B, H, W, conn, _p(R), _p(prov), threads or (os.cpu_count() or 1))
    if rc != 0:
        raise ValueError("a plateau without a source (NaN input?)")
    return (R[0], prov[0]) if squeeze else (R, prov)


def recon_f32_grad(g: np.ndarray, prov: np.ndarray, threads: int = 0):
    """CPU reference gradient (dmarker, dmask): for every source, the exact sum of the upstream
    gradients of the pixels it feeds, rounded once to float32 (nearest, ties to even)."""
    squeeze = np.ndim(g) == 2
    gg = _stack(g)
    pp = np.ascontiguousarray(prov, dtype=np.int32).reshape(gg.shape)
    B, H, W = gg.shape
    dm = np.empty_like(gg)
    dk = np.empty_like(gg)
    if lib.orc_recon_f32_grad(_p(gg), _p(pp), B, H, W, _p(dm), _p(dk), threads or (os.cpu_count() or 1)) != 0:
        raise ValueError("upstream gradient not finite or |g| >= 2^31")
    return (dm[0], dk[0]) if squeeze else (dm, dk)


def recon_fd(marker, mask, g, conn, idx, h=1e-4, threads: int = 0):
    """Central differences in float64 at the listed flat pixel indices.  Returns
    (fd_marker, fd_mask, valid_marker, valid_mask)."""
    mk = np.ascontiguousarray(marker, dtype=np.float32)
    ms = np.ascontiguousarray(mask, dtype=np.float32)
    gg = np.ascontiguousarray(g, dtype=np.float32)
    ix = np.ascontiguousarray(idx, dtype=np.int64)
    H, W = ms.shape
    fd = np.empty(2 * len(ix), np.float64)
    ok = np.empty(2 * len(ix), np.int32)
    lib.orc_recon_fd(_p(mk), _p(ms), _p(gg), H, W, conn, _p(ix), len(ix), h, _p(fd), _p(ok),
                     threads or (os.cpu_count() or 1))
    return fd[0::2], fd[1::2], ok[0::2].astype(bool), ok[1::2].astype(bool)
