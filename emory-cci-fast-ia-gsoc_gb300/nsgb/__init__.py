"""nsgb: GB300-native morphological reconstruction and union-find labelling.

Thin Python mirror of the reference's `nscale::` / `nscale::gpu::` interface
(fastIA-master/src/segment/MorphologicOperations.h:21-190) over the C ABI in libnsgb.so.
Same names, argument order and meaning; images are 2-D CUDA tensors (uint8, uint16, int32,
float32) instead of cv::Mat / cv::gpu::GpuMat, and results are new tensors.  Errors raise
`NsgbError` (the reference raised cv::Exception on bad arguments); there is no CPU fallback:
CPU tensors are rejected.

Every call runs on torch's current CUDA stream and synchronizes it at the end to report the
device-side status, matching the reference's blocking calls.  For asynchronous use call the
C ABI directly (opts.sync = 0).
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, Optional, Tuple

import torch

from . import _ffi
from ._ffi import NsgbError, lib

__all__ = [
    "imreconstruct", "imreconstructBinary", "imfillHoles", "imhmin", "bwselect", "bwlabel", "bwlabel2",
    "bwareaopen2", "bounding_boxes", "threshold", "invert", "chain", "imreconstructQueueThroughput", "chain_batch", "BatchPlan",
    "recon_f32", "recon_f32_backward", "NsgbError", "workspace",
]

_DT = {torch.uint8: _ffi.U8, torch.int32: _ffi.I32, torch.float32: _ffi.F32}
if hasattr(torch, "uint16"):
    _DT[torch.uint16] = _ffi.U16


def _dtype_code(t: torch.Tensor) -> int:
    if t.dtype not in _DT:
        raise NsgbError(2, f"dtype {t.dtype}")
    return _DT[t.dtype]


def _check_image(t: torch.Tensor, name: str) -> None:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise NsgbError(1, f"{name} must be a CUDA tensor (no CPU path)")
    if t.dim() != 2:
        raise NsgbError(1, f"{name} must be 2-D (single channel)")
    if t.stride(1) != 1:
        raise NsgbError(1, f"{name} must have unit column stride")


def _pitch(t: torch.Tensor) -> int:
    return t.stride(0) * t.element_size()


def _stream() -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class _Workspace:
    """Per-device cached workspace (a uint8 tensor grown on demand)."""

    def __init__(self) -> None:
        self._buf: Dict[int, torch.Tensor] = {}

    def get(self, nbytes: int, device: torch.device) -> Tuple[int, int]:
        idx = device.index if device.index is not None else torch.cuda.current_device()
        buf = self._buf.get(idx)
        if buf is None or buf.numel() < nbytes:
            buf = torch.empty(max(nbytes, 1 << 20) + 256, dtype=torch.uint8, device=device)
            self._buf[idx] = buf
        ptr = buf.data_ptr()
        aligned = (ptr + 255) & ~255
        return aligned, buf.numel() - (aligned - ptr)


workspace = _Workspace()


def _ws(op: int, dtype: int, rows: int, cols: int, device: torch.device) -> Tuple[int, int]:
    need = lib.nsgb_workspace_size(op, dtype, rows, cols)
    return workspace.get(need, device)


def _same_shape(a: torch.Tensor, b: torch.Tensor, what: str) -> None:
    if a.shape != b.shape or a.dtype != b.dtype or a.device != b.device:
        raise NsgbError(1, f"{what}: shape/dtype/device mismatch")


def _dense_like(t: torch.Tensor, dtype: Optional[torch.dtype] = None) -> torch.Tensor:
    return torch.empty(t.shape, dtype=dtype or t.dtype, device=t.device)


def _contig(t: torch.Tensor) -> torch.Tensor:
    return t if t.is_contiguous() else t.contiguous()


def imreconstruct(seeds: torch.Tensor, image: torch.Tensor, connectivity: int, erode: bool = False,
                  max_visits_per_tile: int = 0, max_visit_iters: int = 0, queue_poll_limit: int = 0) -> torch.Tensor:
    """nscale::imreconstruct<T>(seeds, image, connectivity) (MorphologicOperations.cpp:665-838) /
    nscale::gpu::imreconstruct<T> (MorphologicOperationsGPU.cpp:172-200): reconstruction by
    dilation of `seeds` under `image`.  `erode=True` gives the dual (reconstruction by erosion).
    The budgets (nsgb_opts) bound the device work: exceeding them raises NsgbError with
    NSGB_ERR_NOT_CONVERGED (visits, sweeps) or NSGB_ERR_TIMEOUT (queue polls)."""
    _check_image(seeds, "seeds")
    _check_image(image, "image")
    _same_shape(seeds, image, "imreconstruct")
    dt = _dtype_code(image)
    out = _contig(seeds).clone()
    mask = _contig(image)
    rows, cols = out.shape
    ws, nb = _ws(_ffi.OP_IMRECONSTRUCT, dt, rows, cols, out.device)
    opts = _ffi.Opts(1, max_visits_per_tile, max_visit_iters, queue_poll_limit)
    st = lib.nsgb_imreconstruct(dt, out.data_ptr(), mask.data_ptr(), rows, cols, _pitch(out), connectivity,
                                1 if erode else 0, ws, nb, _stream(), C.byref(opts))
    _ffi.check(st, "imreconstruct")
    return out


def imreconstructBinary(seeds: torch.Tensor, binaryImage: torch.Tensor, connectivity: int) -> torch.Tensor:
    """nscale::imreconstructBinary<T> (MorphologicOperations.cpp:1688-1829)."""
    _check_image(seeds, "seeds")
    _check_image(binaryImage, "binaryImage")
    _same_shape(seeds, binaryImage, "imreconstructBinary")
    dt = _dtype_code(binaryImage)
    out = _contig(seeds).clone()
    mask = _contig(binaryImage)
    rows, cols = out.shape
    ws, nb = _ws(_ffi.OP_IMRECONSTRUCT_BINARY, dt, rows, cols, out.device)
    st = lib.nsgb_imreconstruct_binary(dt, out.data_ptr(), mask.data_ptr(), rows, cols, _pitch(out), connectivity,
                                       ws, nb, _stream(), None)
    _ffi.check(st, "imreconstructBinary")
    return out


def imfillHoles(image: torch.Tensor, binary: bool, connectivity: int) -> torch.Tensor:
    """nscale::imfillHoles<T>(image, binary, connectivity) (MorphologicOperations.cpp:1859-1926)."""
    _check_image(image, "image")
    dt = _dtype_code(image)
    img = _contig(image)
    out = _dense_like(img)
    rows, cols = img.shape
    ws, nb = _ws(_ffi.OP_FILL_HOLES, dt, rows, cols, img.device)
    st = lib.nsgb_imfill_holes(dt, img.data_ptr(), out.data_ptr(), rows, cols, _pitch(img), 1 if binary else 0,
                               connectivity, ws, nb, _stream(), None)
    _ffi.check(st, "imfillHoles")
    return out


def imhmin(image: torch.Tensor, h: float, connectivity: int) -> torch.Tensor:
    """nscale::imhmin<T>(image, h, connectivity) (MorphologicOperations.cpp:2260-2282)."""
    _check_image(image, "image")
    dt = _dtype_code(image)
    img = _contig(image)
    out = _dense_like(img)
    rows, cols = img.shape
    ws, nb = _ws(_ffi.OP_HMIN, dt, rows, cols, img.device)
    st = lib.nsgb_imhmin(dt, img.data_ptr(), out.data_ptr(), rows, cols, _pitch(img), float(h), connectivity, ws,
                         nb, _stream(), None)
    _ffi.check(st, "imhmin")
    return out


def bwselect(binaryImage: torch.Tensor, seeds: torch.Tensor, connectivity: int) -> torch.Tensor:
    """nscale::bwselect<T>(binaryImage, seeds, connectivity) (MorphologicOperations.cpp:1929-1951)."""
    _check_image(binaryImage, "binaryImage")
    _check_image(seeds, "seeds")
    _same_shape(binaryImage, seeds, "bwselect")
    dt = _dtype_code(binaryImage)
    img = _contig(binaryImage)
    sd = _contig(seeds)
    out = _dense_like(img)
    rows, cols = img.shape
    ws, nb = _ws(_ffi.OP_BWSELECT, dt, rows, cols, img.device)
    st = lib.nsgb_bwselect(dt, img.data_ptr(), sd.data_ptr(), out.data_ptr(), rows, cols, _pitch(img), connectivity,
                           ws, nb, _stream(), None)
    _ffi.check(st, "bwselect")
    return out


def bwlabel2(binaryImage: torch.Tensor, connectivity: int, relab: bool) -> torch.Tensor:
    """nscale::bwlabel2(binaryImage, connectivity, relab) (MorphologicOperations.cpp:2012-2035).
    relab=True: labels 1..n in raster order, background 0; relab=False: smallest raster
    index of the component, background -1."""
    lab, _ = _bwlabel(binaryImage, connectivity, relab)
    return lab


def bwlabel(binaryImage: torch.Tensor, connectivity: int, relab: bool) -> torch.Tensor:
    """nscale::gpu::bwlabel(binaryImage, connectivity, relab) (MorphologicOperationsGPU.cpp:878-900)."""
    return bwlabel2(binaryImage, connectivity, relab)


def _bwlabel(binaryImage: torch.Tensor, connectivity: int, relab: bool) -> Tuple[torch.Tensor, int]:
    _check_image(binaryImage, "binaryImage")
    if binaryImage.dtype != torch.uint8:
        raise NsgbError(2, "bwlabel2 takes a uint8 image")
    img = _contig(binaryImage)
    rows, cols = img.shape
    lab = torch.empty((rows, cols), dtype=torch.int32, device=img.device)
    ws, nb = _ws(_ffi.OP_BWLABEL, _ffi.U8, rows, cols, img.device)
    n = C.c_int32(0)
    st = lib.nsgb_bwlabel(img.data_ptr(), lab.data_ptr(), rows, cols, _pitch(img), _pitch(lab), connectivity,
                          1 if relab else 0, C.byref(n), ws, nb, _stream(), None)
    _ffi.check(st, "bwlabel2")
    return lab, int(n.value)


def bwlabel2_count(binaryImage: torch.Tensor, connectivity: int) -> Tuple[torch.Tensor, int]:
    """bwlabel2 with relabelling, also returning the number of components
    (ConnComponents::relabel's return value)."""
    return _bwlabel(binaryImage, connectivity, True)


def bwareaopen2(image: torch.Tensor, labeled: bool, flatten: bool, minSize: int, maxSize: int,
                connectivity: int) -> Tuple[torch.Tensor, int]:
    """nscale::bwareaopen2(image, labeled, flatten, minSize, maxSize, connectivity, count)
    (MorphologicOperations.cpp:2199-2232).  Returns (result, count): result is uint8 255/0 when
    `flatten`, else int32 kept labels (background -1); count = components kept."""
    _check_image(image, "image")
    if labeled and image.dtype != torch.int32:
        raise NsgbError(2, "labeled input must be int32")
    if not labeled and image.dtype != torch.uint8:
        raise NsgbError(2, "unlabeled input must be uint8")
    img = _contig(image)
    rows, cols = img.shape
    ws, nb = _ws(_ffi.OP_BWAREAOPEN, _ffi.U8, rows, cols, img.device)
    cnt = C.c_int32(0)
    if flatten:
        out = torch.empty((rows, cols), dtype=torch.uint8, device=img.device)
        st = lib.nsgb_bwareaopen(img.data_ptr(), 1 if labeled else 0, None, out.data_ptr(), rows, cols, _pitch(img),
                                 0, _pitch(out), int(minSize), int(maxSize), connectivity, C.byref(cnt), ws, nb,
                                 _stream(), None)
    else:
        out = torch.empty((rows, cols), dtype=torch.int32, device=img.device)
        st = lib.nsgb_bwareaopen(img.data_ptr(), 1 if labeled else 0, out.data_ptr(), None, rows, cols, _pitch(img),
                                 _pitch(out), 0, int(minSize), int(maxSize), connectivity, C.byref(cnt), ws, nb,
                                 _stream(), None)
    _ffi.check(st, "bwareaopen2")
    return out, int(cnt.value)


def bounding_boxes(labels: torch.Tensor, bgval: int = 0, capacity: Optional[int] = None) -> torch.Tensor:
    """ConnComponents::boundingBox (ConnComponents.cpp:241-284) of an int32 label image on the
    device: int32 tensor (5, count) of label, min x, max x, min y, max y per label other than
    `bgval`, in the order of each label's first pixel in raster order.

    `capacity` bounds the labels the output is first sized for (default: 65536, or rows*cols if
    smaller).  The call reports the number of labels; if it exceeds the capacity, the boxes are
    computed again into an output of exactly that size, so the result is always complete."""
    _check_image(labels, "labels")
    if labels.dtype != torch.int32:
        raise NsgbError(2, "labels must be int32")
    lab = _contig(labels)
    rows, cols = lab.shape
    ws, nb = _ws(_ffi.OP_BOUNDING_BOX, _ffi.I32, rows, cols, lab.device)
    cap = min(rows * cols, 65536 if capacity is None else max(1, int(capacity)))
    while True:
        boxes = torch.empty((5, cap), dtype=torch.int32, device=lab.device)
        cnt = C.c_int32(0)
        st = lib.nsgb_bounding_boxes(lab.data_ptr(), rows, cols, _pitch(lab), int(bgval), boxes.data_ptr(), cap,
                                     C.byref(cnt), None, ws, nb, _stream(), None)
        _ffi.check(st, "bounding_boxes")
        if int(cnt.value) <= cap:
            return boxes[:, :int(cnt.value)].contiguous()
        cap = int(cnt.value)


def threshold(image: torch.Tensor, thr: float) -> torch.Tensor:
    """`image > thr` as 255 / 0 uint8 (OpenCV `Mat > k`, HistologicalEntities.cpp:214)."""
    _check_image(image, "image")
    dt = _dtype_code(image)
    img = _contig(image)
    out = _dense_like(img, torch.uint8)
    rows, cols = img.shape
    st = lib.nsgb_threshold(dt, img.data_ptr(), out.data_ptr(), rows, cols, _pitch(img), _pitch(out), float(thr),
                            _stream())
    _ffi.check(st, "threshold")
    return out


def invert(image: torch.Tensor) -> torch.Tensor:
    """nscale::PixelOperations::invert<T> (PixelOperations.cpp:18-39)."""
    _check_image(image, "image")
    dt = _dtype_code(image)
    img = _contig(image)
    out = _dense_like(img)
    rows, cols = img.shape
    st = lib.nsgb_invert(dt, img.data_ptr(), out.data_ptr(), rows, cols, _pitch(img), _stream())
    _ffi.check(st, "invert")
    return out


def chain(marker: torch.Tensor, mask: torch.Tensor, recon_conn: int = 8, thr: float = 128, fill_conn: int = 4,
          label_conn: int = 8, area_min: int = 11, area_max: int = 1000) -> Dict[str, object]:
    """The device-resident segmentation chain of HistologicalEntities.cpp:195-246:
    reconstruction, threshold, binary hole fill, bwlabel2 (relabelled) and bwareaopen2."""
    _check_image(marker, "marker")
    _check_image(mask, "mask")
    _same_shape(marker, mask, "chain")
    dt = _dtype_code(mask)
    rec = _contig(marker).clone()
    msk = _contig(mask)
    rows, cols = rec.shape
    dev = rec.device
    fill = torch.empty((rows, cols), dtype=torch.uint8, device=dev)
    labels = torch.empty((rows, cols), dtype=torch.int32, device=dev)
    area = torch.empty((rows, cols), dtype=torch.uint8, device=dev)
    ws, nb = _ws(_ffi.OP_CHAIN, dt, rows, cols, dev)
    nl, nk = C.c_int32(0), C.c_int32(0)
    st = lib.nsgb_chain(dt, rec.data_ptr(), msk.data_ptr(), rows, cols, _pitch(rec), recon_conn, float(thr),
                        fill_conn, label_conn, int(area_min), int(area_max), fill.data_ptr(), labels.data_ptr(),
                        area.data_ptr(), C.byref(nl), C.byref(nk), ws, nb, _stream(), None)
    _ffi.check(st, "chain")
    return {"recon": rec, "fill": fill, "labels": labels, "area": area, "n_labels": int(nl.value),
            "n_kept": int(nk.value)}


def disk19() -> "np.ndarray":
    """The 19 x 19 disk the reference opens the red channel with (HistologicalEntities.cpp:
    162-185, MATLAB's strel('disk', 10) written out): centred rows of widths 11, 13, 15, 17,
    eleven of 19, then 17, 15, 13, 11."""
    import numpy as np

    widths = [11, 13, 15, 17] + [19] * 11 + [17, 15, 13, 11]
    k = np.zeros((19, 19), np.uint8)
    for i, w in enumerate(widths):
        k[i, 9 - w // 2:9 + w // 2 + 1] = 1
    return k


def ellipse3() -> "np.ndarray":
    """getStructuringElement(MORPH_ELLIPSE, Size(3, 3)) (HistologicalEntities.cpp:309): the cross."""
    import numpy as np

    return np.array([[0, 1, 0], [1, 1, 1], [0, 1, 0]], np.uint8)


def morphOpen(image: torch.Tensor, kernel) -> torch.Tensor:
    """nscale::morphOpen<unsigned char> (MorphologicOperations.cpp:2459-2493): erosion with the
    image surrounded by 255, then dilation surrounded by 0, by the flat element `kernel` (a k x k
    host array, k odd in [3, 63], non-zero = in the element)."""
    import numpy as np

    _check_image(image, "image")
    if image.dtype != torch.uint8:
        raise NsgbError(2, "morphOpen: image must be uint8 (the reference's one instantiation)")
    k = np.ascontiguousarray((np.asarray(kernel) != 0).astype(np.uint8))
    if k.ndim != 2 or k.shape[0] != k.shape[1]:
        raise NsgbError(1, "morphOpen: kernel must be square")
    img = _contig(image)
    rows, cols = img.shape
    out = torch.empty((rows, cols), dtype=torch.uint8, device=img.device)
    ws, nb = _ws(_ffi.OP_MORPH_OPEN, _ffi.U8, rows, cols, img.device)
    st = lib.nsgb_morph_open(img.data_ptr(), out.data_ptr(), rows, cols, _pitch(img), _pitch(out),
                             k.ctypes.data_as(C.c_void_p), int(k.shape[0]), ws, nb, _stream(), None)
    _ffi.check(st, "morphOpen")
    return out


def distanceTransform(mask: torch.Tensor, basins: bool = False) -> torch.Tensor:
    """Distance from every pixel of a uint8 mask to its nearest zero pixel, float32, exact (the
    map of HistologicalEntities.cpp:341; nscale::gpu::distanceTransform's role).  basins=True
    gives the watershed basins of HistologicalEntities.cpp:347-356 instead: -distance on
    non-zero pixels, -FLT_MAX on zero pixels."""
    _check_image(mask, "mask")
    if mask.dtype != torch.uint8:
        raise NsgbError(2, "distanceTransform: mask must be uint8")
    m = _contig(mask)
    rows, cols = m.shape
    out = torch.empty((rows, cols), dtype=torch.float32, device=m.device)
    ws, nb = _ws(_ffi.OP_DISTANCE, _ffi.U8, rows, cols, m.device)
    st = lib.nsgb_distance_transform(m.data_ptr(), out.data_ptr(), rows, cols, _pitch(m), _pitch(out),
                                     1 if basins else 0, ws, nb, _stream(), None)
    _ffi.check(st, "distanceTransform")
    return out


def nucleus_candidates(rc: torch.Tensor, rc_open: torch.Tensor, rbc: torch.Tensor, g1: float = 80, g2: float = 45,
                       area_min: int = 11, area_max: int = 1000) -> Tuple[torch.Tensor, int]:
    """The nucleus-candidate stage after the opening (HistologicalEntities.cpp:195-275) on the
    device, uint8 images of one shape: reconstruction of `rc_open` under `rc`, valleys
    D = rc - recon, bw1 = imfillHoles(D > g1), bw1_t = bwareaopen2(bw1, [area_min, area_max)),
    seg = bwselect(D > g2, bw1_t, 8) & (rbc == 0).  Returns (seg as 255 / 0, number of
    components kept in bw1_t); the reference stops with NO_CANDIDATES_LEFT when that is 0."""
    for t, n in ((rc, "rc"), (rc_open, "rc_open"), (rbc, "rbc")):
        _check_image(t, n)
        if t.dtype != torch.uint8:
            raise NsgbError(2, f"{n} must be uint8")
    _same_shape(rc, rc_open, "nucleus_candidates")
    _same_shape(rc, rbc, "nucleus_candidates")
    rec = _contig(rc_open).clone()
    img, red = _contig(rc), _contig(rbc)
    rows, cols = rec.shape
    seg = torch.empty((rows, cols), dtype=torch.uint8, device=rec.device)
    ws, nb = _ws(_ffi.OP_NUCLEUS_CANDIDATES, _ffi.U8, rows, cols, rec.device)
    nk = C.c_int32(0)
    st = lib.nsgb_nucleus_candidates(rec.data_ptr(), img.data_ptr(), red.data_ptr(), seg.data_ptr(), rows, cols,
                                     _pitch(rec), float(g1), float(g2), int(area_min), int(area_max), C.byref(nk),
                                     None, ws, nb, _stream(), None)
    _ffi.check(st, "nucleus_candidates")
    return seg, int(nk.value)


class BatchPlan:
    """A prepared batch of tiles (nsgb_batch_prepare): the image table lives in a workspace
    owned by this object; `chain()` / `reconstruct()` then launch kernels only."""

    def __init__(self, markers, masks, with_outputs: bool = True) -> None:
        if len(markers) != len(masks) or not markers:
            raise NsgbError(1, "batch: markers and masks must be non-empty lists of equal length")
        dt = _dtype_code(masks[0])
        self.markers = [_contig(m) for m in markers]
        self.masks = [_contig(m) for m in masks]
        self.fill, self.labels, self.area = [], [], []
        tiles = (_ffi.Tile * len(markers))()
        for i, (mk, ms) in enumerate(zip(self.markers, self.masks)):
            _check_image(mk, "marker")
            _check_image(ms, "mask")
            _same_shape(mk, ms, "batch")
            if _dtype_code(ms) != dt:
                raise NsgbError(1, "batch: all tiles must share one dtype")
            rows, cols = ms.shape
            if with_outputs:
                self.fill.append(torch.empty((rows, cols), dtype=torch.uint8, device=ms.device))
                self.labels.append(torch.empty((rows, cols), dtype=torch.int32, device=ms.device))
                self.area.append(torch.empty((rows, cols), dtype=torch.uint8, device=ms.device))
            tiles[i] = _ffi.Tile(mk.data_ptr(), ms.data_ptr(), rows, cols, _pitch(ms),
                                 self.fill[i].data_ptr() if with_outputs else None,
                                 self.labels[i].data_ptr() if with_outputs else None,
                                 self.area[i].data_ptr() if with_outputs else None)
        need = lib.nsgb_batch_workspace_size(dt, tiles, len(markers))
        if need == 0:
            raise NsgbError(1, "batch: bad tiles (or more than 2^31 pixels in total)")
        self._ws = torch.empty(need + 256, dtype=torch.uint8, device=self.masks[0].device)
        ptr = (self._ws.data_ptr() + 255) & ~255
        self.batch = _ffi.Batch()
        _ffi.check(lib.nsgb_batch_prepare(dt, tiles, len(markers), ptr, need, C.byref(self.batch)), "batch_prepare")
        self.n = len(markers)

    def chain(self, recon_conn=8, thr=128.0, fill_conn=4, label_conn=8, area_min=11, area_max=1000,
              counts: bool = True, sync: bool = True):
        nl = (C.c_int32 * self.n)() if counts else None
        nk = (C.c_int32 * self.n)() if counts else None
        opts = _ffi.Opts(1 if sync else 0, 0, 0)
        st = lib.nsgb_chain_batch(C.byref(self.batch), recon_conn, float(thr), fill_conn, label_conn, int(area_min),
                                  int(area_max), nl, nk, _stream(), C.byref(opts))
        _ffi.check(st, "chain_batch")
        if counts:
            return list(nl), list(nk)
        return None

    def counts_async(self, out: torch.Tensor) -> None:
        """Enqueue the per-tile (n_labels, n_kept) of the last chain into `out` (int32, 2*n,
        device or pinned host) without synchronising."""
        if out.dtype != torch.int32 or out.numel() < 2 * self.n or not out.is_contiguous():
            raise NsgbError(1, "counts_async: need a contiguous int32 tensor of 2*n elements")
        _ffi.check(lib.nsgb_batch_counts_async(C.byref(self.batch), out.data_ptr(), _stream()), "batch_counts_async")

    def reconstruct(self, connectivity: int, erode: bool = False, sync: bool = True) -> None:
        opts = _ffi.Opts(1 if sync else 0, 0, 0)
        st = lib.nsgb_imreconstruct_batch(C.byref(self.batch), connectivity, 1 if erode else 0, _stream(),
                                          C.byref(opts))
        _ffi.check(st, "imreconstruct_batch")


def imreconstructQueueThroughput(seeds, images, connectivity: int, nItFirstPass: int = 0):
    """nscale::gpu::imreconstructQueueThroughput<T> (MorphologicOperationsGPU.cpp:447-545):
    reconstruct a list of tiles in one batched launch.  Returns new tensors (nItFirstPass is
    accepted for compatibility and has no meaning here)."""
    outs = [_contig(s).clone() for s in seeds]
    plan = BatchPlan(outs, list(images), with_outputs=False)
    plan.reconstruct(connectivity)
    return outs


def chain_batch(markers, masks, recon_conn=8, thr=128.0, fill_conn=4, label_conn=8, area_min=11, area_max=1000):
    """The segmentation chain on a batch of tiles (one launch per stage for all of them).
    Returns a list of dicts like `chain`."""
    recon = [_contig(m).clone() for m in markers]
    plan = BatchPlan(recon, list(masks))
    nl, nk = plan.chain(recon_conn, thr, fill_conn, label_conn, area_min, area_max)
    return [{"recon": recon[i], "fill": plan.fill[i], "labels": plan.labels[i], "area": plan.area[i],
             "n_labels": nl[i], "n_kept": nk[i]} for i in range(plan.n)]


def _stack3(t: torch.Tensor, name: str) -> torch.Tensor:
    if t.dtype != torch.float32 or not t.is_cuda or t.dim() not in (2, 3):
        raise NsgbError(1, f"{name}: need a float32 CUDA tensor [H, W] or [B, H, W]")
    t = _contig(t)
    return t if t.dim() == 3 else t.unsqueeze(0)


_f32_ws = {}


def _f32_workspace(B, H, W, backward, dev):
    need = lib.nsgb_recon_f32_workspace_size(B, H, W, 1 if backward else 0)
    if need == 0:
        raise NsgbError(1, "recon_f32: image stack too large")
    key = (dev.index, bool(backward))
    buf = _f32_ws.get(key)
    if buf is None or buf.numel() < need + 256:
        buf = torch.empty(need + 256, dtype=torch.uint8, device=dev)
        _f32_ws[key] = buf
    return (buf.data_ptr() + 255) & ~255, need


def recon_f32(marker: torch.Tensor, mask: torch.Tensor, connectivity: int = 8):
    """Float32 reconstruction by dilation with its provenance map (no counterpart in the
    reference).  Returns (out, prov) shaped like the inputs; prov = q (marker q), ~q (mask q)
    or INT32_MIN (the zero ring), q = y * W + x."""
    squeeze = marker.dim() == 2
    mk, ms = _stack3(marker, "marker"), _stack3(mask, "mask")
    _same_shape(mk, ms, "recon_f32")
    B, H, W = ms.shape
    out = torch.empty_like(ms)
    prov = torch.empty(ms.shape, dtype=torch.int32, device=ms.device)
    ws, nb = _f32_workspace(B, H, W, False, ms.device)
    st = lib.nsgb_recon_f32_fwd(mk.data_ptr(), ms.data_ptr(), out.data_ptr(), prov.data_ptr(), B, H, W, W * 4,
                                H * W * 4, connectivity, ws, nb, _stream(), None)
    _ffi.check(st, "recon_f32_fwd")
    return (out[0], prov[0]) if squeeze else (out, prov)


def recon_f32_backward(grad: torch.Tensor, prov: torch.Tensor):
    """Adjoint of recon_f32: (d/dmarker, d/dmask) of sum(grad * out); each source's gradient is
    the exact sum of its contributions rounded once to float32."""
    squeeze = grad.dim() == 2
    g = _stack3(grad, "grad")
    p = _contig(prov).view(g.shape)
    if p.dtype != torch.int32:
        raise NsgbError(1, "recon_f32_backward: prov must be int32")
    B, H, W = g.shape
    dm = torch.empty_like(g)
    dk = torch.empty_like(g)
    ws, nb = _f32_workspace(B, H, W, True, g.device)
    st = lib.nsgb_recon_f32_bwd(g.data_ptr(), p.data_ptr(), dm.data_ptr(), dk.data_ptr(), B, H, W, W * 4,
                                H * W * 4, ws, nb, _stream(), None)
    _ffi.check(st, "recon_f32_bwd")
    return (dm[0], dk[0]) if squeeze else (dm, dk)
