/* nsgb — GB300-native morphological reconstruction and union-find labelling.
 *
 * C ABI of the device library (libnsgb.so).  Every entry point:
 *   - takes DEVICE pointers for images (row pitch in bytes, pitch >= cols * element size,
 *     pitch a multiple of the element size), a caller-provided device workspace of at least
 *     nsgb_workspace_size(op, ...) bytes, and a CUDA stream;
 *   - enqueues its kernels on that stream and never allocates device memory;
 *   - returns an nsgb_status and never throws.  With opts == NULL or opts->sync != 0 the
 *     call synchronizes the stream and also reports errors detected on the device (iteration
 *     budget exhausted, wait timeout); with opts->sync == 0 it returns after enqueueing and
 *     nsgb_device_status() reads the device-side status later.
 *   - calls on different streams with different workspaces are independent (no global state).
 *
 * Semantics follow the reference's serial CPU implementation (nscale::, fastIA-master/src/
 * segment/MorphologicOperations.cpp and ConnComponents.cpp), which is also what its GPU path
 * computes; each function names the reference interface it replaces.
 */
#ifndef NSGB_H_
#define NSGB_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* nsgb_stream_t; /* == cudaStream_t */

typedef enum {
  NSGB_OK = 0,
  NSGB_ERR_BAD_ARG = 1,           /* null pointer, bad size, pitch, connectivity ... */
  NSGB_ERR_UNSUPPORTED_DTYPE = 2, /* dtype not defined for this operation */
  NSGB_ERR_WORKSPACE = 3,         /* workspace missing or smaller than required */
  NSGB_ERR_NOT_CONVERGED = 4,     /* iteration / round budget exhausted on the device */
  NSGB_ERR_TIMEOUT = 5,           /* a bounded device-side wait gave up */
  NSGB_ERR_CUDA = 6,              /* a CUDA runtime call failed */
  NSGB_ERR_QUEUE_OVERFLOW = 7     /* a device work list ran out of capacity */
} nsgb_status;

typedef enum { NSGB_U8 = 0, NSGB_U16 = 1, NSGB_I32 = 2, NSGB_F32 = 3 } nsgb_dtype;

typedef enum {
  NSGB_OP_IMRECONSTRUCT = 0,
  NSGB_OP_IMRECONSTRUCT_BINARY = 1,
  NSGB_OP_FILL_HOLES = 2,
  NSGB_OP_HMIN = 3,
  NSGB_OP_BWSELECT = 4,
  NSGB_OP_BWLABEL = 5,
  NSGB_OP_BWAREAOPEN = 6,
  NSGB_OP_CHAIN = 7,
  NSGB_OP_BOUNDING_BOX = 8,
  NSGB_OP_NUCLEUS_CANDIDATES = 9,
  NSGB_OP_MORPH_OPEN = 10,
  NSGB_OP_DISTANCE = 11
} nsgb_op;

typedef struct {
  int sync;       /* 1: synchronize and return the device status (default when opts == NULL) */
  int max_visits_per_tile; /* reconstruction: cap on tile visits, in units of the number of
                             tiles (0 = default, effectively unbounded) */
  int max_visit_iters; /* reconstruction: cap on row/column sweeps per tile visit (0 = default) */
  int queue_poll_limit; /* reconstruction: polls a warp makes on the tile queue before it gives
                           up with NSGB_ERR_TIMEOUT (0 = default, about 2 s of polling); a small
                           value makes an idle warp's wait run out, for testing that path */
  int recon_passes; /* reconstruction: streaming passes over all tiles before the work queue
                       (> 0 that many, < 0 none, 0 the library's tuned default) */
  int recon_order;  /* reconstruction: initial order of the work queue when it starts with every
                       tile (1 raster, 2 checkerboard, 3 four colours; 0 the tuned default) */
  int recon_ctas_per_sm; /* reconstruction: CTAs of 4 tile workers per SM for the work queue (1 .. 4;
                            0 the tuned default).  Fewer workers waste fewer visits where only a
                            front of tiles has work, as in hole filling */
  int reserved[1];
  /* Optional CUDA events (cudaEvent_t) recorded on the call's stream immediately before and
   * after the reconstruction kernel (nsgb_imreconstruct, nsgb_chain), for timing it alone.  In
   * a call captured into a CUDA graph they become external event-record nodes, recorded at
   * every replay. */
  void* recon_event_begin;
  void* recon_event_end;
} nsgb_opts;

/* Bytes of device workspace needed by `op` on an image of rows x cols of `dtype`. */
size_t nsgb_workspace_size(int op, int dtype, int64_t rows, int64_t cols);

const char* nsgb_status_string(int status);

/* Reads (synchronously) the device-side status word of the last call that used `ws`. */
nsgb_status nsgb_device_status(const void* ws, nsgb_stream_t stream);

/* Grayscale morphological reconstruction, in place on `marker` (read-only `mask`).
 *   erode = 0: reconstruction by dilation of marker under mask -- nscale::imreconstruct<T>
 *              (MorphologicOperations.cpp:665-838; GPU: nscale::gpu::imreconstruct<T>
 *              MorphologicOperationsGPU.cpp:172-200, imreconstructIntCaller<T> /
 *              imreconstructFloatCaller<T> imreconstruct_int_kernel.cuh:7-9,
 *              imreconstruct_float_kernel.cuh, and the queue variants
 *              imreconstructQueueSpeedup<T> MorphologicOperationsGPU.cpp:286-360 /
 *              morphReconSpeedup global_queue.cuh:48-50).  Includes the reference's
 *              0-valued padding ring (visible only for negative signed / float data).
 *   erode = 1: reconstruction by erosion of marker above mask (the dual), with no padding
 *              ring; the hole-filling building block.
 * dtypes: u8, u16, i32, f32.  conn: 4 or 8. */
nsgb_status nsgb_imreconstruct(int dtype, void* marker, const void* mask, int64_t rows, int64_t cols,
                               int64_t pitch, int conn, int erode, void* ws, size_t ws_bytes,
                               nsgb_stream_t stream, const nsgb_opts* opts);

/* Binary reconstruction in place on `marker`: every zero marker pixel whose mask is non-zero
 * and that is connected through non-zero mask pixels to a pixel with marker != 0 and
 * mask != 0 becomes max<T>; other pixels keep their marker value (the marker is not
 * clamped by the mask).  nscale::imreconstructBinary<T> (MorphologicOperations.cpp:1688-
 * 1829); GPU nscale::gpu::imreconstructBinary<T> (MorphologicOperationsGPU.cpp:686-721),
 * imreconstructBinaryCaller<T> (imreconstruct_binary_kernel.cuh).  dtypes: u8, u16, i32. */
nsgb_status nsgb_imreconstruct_binary(int dtype, void* marker, const void* mask, int64_t rows,
                                      int64_t cols, int64_t pitch, int conn, void* ws,
                                      size_t ws_bytes, nsgb_stream_t stream, const nsgb_opts* opts);

/* Hole filling: nscale::imfillHoles<T>(image, binary, conn) (MorphologicOperations.cpp:
 * 1859-1926); GPU nscale::gpu::imfillHoles<T> (MorphologicOperationsGPU.cpp:751-836).
 * binary = 1: u8/u16 -> 0 where the pixel is not max<T> and is connected to the image
 *             border through pixels that are not max<T>, else max<T> (0/max input gives the
 *             usual fill); i32 -> INT_MAX everywhere (the reference's result for int, whose
 *             padding value min<int> is non-zero).
 * binary = 0: grayscale fill, the erosion reconstruction of (image on the border, max<T>
 *             inside) above the image.  dtypes u8, u16, i32, f32.  out must not alias image. */
nsgb_status nsgb_imfill_holes(int dtype, const void* image, void* out, int64_t rows, int64_t cols,
                              int64_t pitch, int binary, int conn, void* ws, size_t ws_bytes,
                              nsgb_stream_t stream, const nsgb_opts* opts);

/* h-minima transform: nscale::imhmin<T>(image, h, conn) (MorphologicOperations.cpp:2260-2282;
 * GPU MorphologicOperationsGPU.cpp:1059-1098) = invert(imreconstruct(invert(I) - h,
 * invert(I))) with saturating subtraction.  dtypes u8, u16, f32. */
nsgb_status nsgb_imhmin(int dtype, const void* image, void* out, int64_t rows, int64_t cols,
                        int64_t pitch, double h, int conn, void* ws, size_t ws_bytes,
                        nsgb_stream_t stream, const nsgb_opts* opts);

/* nscale::bwselect<T>(binaryImage, seeds, conn) (MorphologicOperations.cpp:1929-1951; GPU
 * MorphologicOperationsGPU.cpp:839-868): keeps the image's non-zero pixels whose component
 * (non-zero adjacency) contains a pixel with seeds != 0.  dtypes u8, u16, i32. */
nsgb_status nsgb_bwselect(int dtype, const void* image, const void* seeds, void* out, int64_t rows,
                          int64_t cols, int64_t pitch, int conn, void* ws, size_t ws_bytes,
                          nsgb_stream_t stream, const nsgb_opts* opts);

/* Union-find labelling of a u8 image: equal-valued non-zero neighbours are joined.
 * relabel = 1: labels 1..n in raster order of each component's first pixel, background 0
 *              (nscale::bwlabel2(bin, conn, true), MorphologicOperations.cpp:2012-2035 ->
 *              ConnComponents::label + relabel, ConnComponents.cpp:52-118; GPU
 *              nscale::gpu::bwlabel MorphologicOperationsGPU.cpp:878-900 -> CCL + relabel,
 *              ccl_uf.cuh:11-16).
 * relabel = 0: each pixel gets the smallest raster index (row*cols + col) of its component,
 *              background -1 (bwlabel2(bin, conn, false)).
 * `count` (host pointer, optional) receives n; it forces a stream synchronization. */
nsgb_status nsgb_bwlabel(const uint8_t* bin, int32_t* labels, int64_t rows, int64_t cols,
                         int64_t pitch_in, int64_t pitch_labels, int conn, int relabel,
                         int32_t* count, void* ws, size_t ws_bytes, nsgb_stream_t stream,
                         const nsgb_opts* opts);

/* Area opening: nscale::bwareaopen2(image, labeled, flatten, minSize, maxSize, conn, count)
 * (MorphologicOperations.cpp:2199-2232 -> ConnComponents::areaThresholdLabeled,
 * ConnComponents.cpp:205-239; GPU nscale::gpu::bwareaopen2 MorphologicOperationsGPU.cpp:
 * 1024-1057 -> areaThreshold2 ccl_uf.cuh).  Keeps components whose pixel count is in
 * [min_size, max_size).  labeled = 0: `in` is a u8 image labelled first (conn);
 * labeled = 1: `in` is an int32 label image (background -1).  Outputs (each optional):
 * labels_out = kept label (the input label / smallest raster index), -1 elsewhere;
 * flat_out = 255 where kept, else 0.  `count` (host, optional) = components kept. */
nsgb_status nsgb_bwareaopen(const void* in, int labeled, int32_t* labels_out, uint8_t* flat_out,
                            int64_t rows, int64_t cols, int64_t pitch_in, int64_t pitch_labels,
                            int64_t pitch_flat, int32_t min_size, int32_t max_size, int conn,
                            int32_t* count, void* ws, size_t ws_bytes, nsgb_stream_t stream,
                            const nsgb_opts* opts);

/* Per-label bounding boxes: ConnComponents::boundingBox (src/segment/ConnComponents.cpp:241-284),
 * GPU counterpart nscale::gpu::boundingBox2 (src/segment/cuda/ccl_uf.cuh:16, ccl_uf.cu:847-1107).
 * `labels`: int32 device image (rows x cols, pitch in bytes).  Each pixel holds `bgval` or a label
 * in [1, rows*cols]: the raster labels of nsgb_bwlabel (1..n, background 0) or its root indices
 * (background -1).  As in the reference, a pixel labelled -1 or 0 that is not bgval ends the scan:
 * only the pixels before it in raster order count.  Any other value outside [-1, rows*cols]
 * gives NSGB_ERR_BAD_ARG.
 * `boxes`: device int32, 5 * capacity: entry k is label boxes[k], min x boxes[capacity + k],
 * max x [2 * capacity + k], min y [3 * capacity + k], max y [4 * capacity + k], entries in the
 * order of each label's first pixel in raster order (the reference CPU order; for raster labels
 * that is label order).  Entries past `capacity` are dropped.  The number of labels goes to
 * `count` (host, optional: forces a synchronisation) and / or `count_dev` (device, optional).
 * Workspace: nsgb_workspace_size(NSGB_OP_BOUNDING_BOX, NSGB_I32, rows, cols). */
nsgb_status nsgb_bounding_boxes(const int32_t* labels, int64_t rows, int64_t cols, int64_t pitch, int32_t bgval,
                                int32_t* boxes, int64_t capacity, int32_t* count, int32_t* count_dev, void* ws,
                                size_t ws_bytes, nsgb_stream_t stream, const nsgb_opts* opts);

/* Elementwise helpers of the path: `in > thr` -> 255 / 0 (u8 out; OpenCV `Mat > k` as used at
 * HistologicalEntities.cpp:214; GPU thresholdCaller pixel-ops.cu:349-381), and invert
 * (PixelOperations::invert<T>, PixelOperations.cpp:18-39; GPU invertKernel* pixel-ops.cu:
 * 15-48): unsigned max - x, signed -x (INT_MIN -> INT_MAX), float -x. */
nsgb_status nsgb_threshold(int dtype, const void* in, uint8_t* out, int64_t rows, int64_t cols,
                           int64_t pitch_in, int64_t pitch_out, double thr, nsgb_stream_t stream);
nsgb_status nsgb_invert(int dtype, const void* in, void* out, int64_t rows, int64_t cols,
                        int64_t pitch, nsgb_stream_t stream);

/* The single-tile segmentation chain of HistologicalEntities.cpp:195-246, kept on the
 * device: R = imreconstruct(marker, mask, recon_conn) in place on `marker`;
 * B = R > thr; F = imfillHoles(B, binary, fill_conn); L = bwlabel2(F, label_conn, relabel);
 * A = bwareaopen2(F, unlabeled, flatten, area_min, area_max, label_conn).  Outputs fill,
 * labels, area (each optional).  n_labels / n_kept: host pointers (optional; synchronize).
 * dtypes of marker/mask: u8, u16, i32 (threshold in the same units).  With n_labels = n_kept =
 * NULL and opts->sync == 0 the call only enqueues work, so it can be captured into a CUDA graph;
 * its launches after the reconstruction are programmatic dependents of one another, ordered
 * after everything queued before the call. */
nsgb_status nsgb_chain(int dtype, void* marker, const void* mask, int64_t rows, int64_t cols,
                       int64_t pitch, int recon_conn, double thr, int fill_conn, int label_conn,
                       int32_t area_min, int32_t area_max, uint8_t* fill_out, int32_t* labels_out,
                       uint8_t* area_out, int32_t* n_labels, int32_t* n_kept, void* ws,
                       size_t ws_bytes, nsgb_stream_t stream, const nsgb_opts* opts);

/* Opening of a u8 image by a flat k x k structuring element: nscale::morphOpen<unsigned char>
 * (src/segment/MorphologicOperations.cpp:2459-2493; GPU twin MorphologicOperationsGPU.cpp:1308).
 * Erosion with the image surrounded by 255, then dilation of the result surrounded by 0, each
 * in OpenCV's convention: at (y, x) the min / max of src(y + i - c, x + j - c) over the
 * element's non-zero (i, j), c = (k - 1) / 2.  `kernel`: HOST array of k x k bytes, row-major,
 * non-zero = in the element; k odd, 3 <= k <= 63, at least one non-zero entry (else
 * NSGB_ERR_BAD_ARG).  The reference applies it with its 19 x 19 disk
 * (HistologicalEntities.cpp:162-185) and a 3 x 3 disk (:481).  out must not overlap in.
 * Workspace: nsgb_workspace_size(NSGB_OP_MORPH_OPEN, NSGB_U8, rows, cols) (the eroded image). */
nsgb_status nsgb_morph_open(const uint8_t* in, uint8_t* out, int64_t rows, int64_t cols, int64_t pitch_in,
                            int64_t pitch_out, const uint8_t* kernel, int k, void* ws, size_t ws_bytes,
                            nsgb_stream_t stream, const nsgb_opts* opts);

/* Euclidean distance transform of a u8 mask: out(y, x) = distance from (y, x) to the nearest
 * zero pixel (0 on zero pixels), as float: the correctly rounded square root of the exact
 * integer squared distance.  This is the map the segmentation takes before its watershed
 * (HistologicalEntities.cpp:341, OpenCV's CV_DIST_L2 with CV_DIST_MASK_PRECISE); the reference's
 * own nscale::distanceTransform (MorphologicOperations.cpp:197-275; GPU
 * nscale::gpu::distanceTransform, MorphologicOperationsGPU.cpp:112) propagates nearest zero
 * pixels between 8-neighbours and can return a larger distance where that propagation misses
 * the nearest one.  basins != 0 writes the watershed basins of HistologicalEntities.cpp:347-356
 * instead: -distance on non-zero pixels, -FLT_MAX on zero pixels.  A mask without any zero
 * pixel gives +inf distances.  out: float, pitch_out in bytes.  rows <= 65535 * 128.
 * Workspace: nsgb_workspace_size(NSGB_OP_DISTANCE, NSGB_U8, rows, cols). */
nsgb_status nsgb_distance_transform(const uint8_t* mask, float* out, int64_t rows, int64_t cols, int64_t pitch_in,
                                    int64_t pitch_out, int basins, void* ws, size_t ws_bytes, nsgb_stream_t stream,
                                    const nsgb_opts* opts);

/* The nucleus-candidate stage after the opening, kept on the device: the tail of
 * HistologicalEntities::plFindNucleusCandidates (src/segment/HistologicalEntities.cpp:195-275;
 * GPU twin HistologicalEntitiesGPU.cpp:307-432):
 *   R    = imreconstruct(rc_open, rc, 8)             in place on `rc_open`
 *   D    = rc - R                                    (u8, saturating)
 *   bw1  = imfillHoles(D > g1, binary, 4)
 *   bw1t = bwareaopen2(bw1, unlabeled, flatten, area_min, area_max, 8)   -> n_kept
 *   seg  = bwselect(D > g2, bw1t, 8) & (rbc == 0)    -> 255 / 0 in `seg_out`
 * The reference uses g1 = 80, g2 = 45 and [11, 1000), and returns NO_CANDIDATES_LEFT when
 * n_kept is 0 without writing its output; here `seg_out` is then all 0 and n_kept tells the
 * caller.  rc_open, rc, rbc and seg_out are u8 device images sharing `pitch` (bytes); seg_out
 * may be rc_open.  n_kept: host (optional; synchronizes) and / or n_kept_dev (device, optional).
 * Workspace: nsgb_workspace_size(NSGB_OP_NUCLEUS_CANDIDATES, NSGB_U8, rows, cols). */
nsgb_status nsgb_nucleus_candidates(uint8_t* rc_open, const uint8_t* rc, const uint8_t* rbc, uint8_t* seg_out,
                                    int64_t rows, int64_t cols, int64_t pitch, double g1, double g2,
                                    int32_t area_min, int32_t area_max, int32_t* n_kept, int32_t* n_kept_dev,
                                    void* ws, size_t ws_bytes, nsgb_stream_t stream, const nsgb_opts* opts);

/* ---- Batches: many images of uneven sizes in one persistent reconstruction launch and one
 * launch per labelling stage (the reference's imreconstructQueueThroughput<T>,
 * MorphologicOperationsGPU.cpp:447-545 -> morphReconVector, cuda/global_queue.cu:903-968,
 * batched up to 70 images with one CTA each; here any number, the work of all images shared
 * by the whole GPU). */
typedef struct {
  void* marker;        /* in: marker; out: reconstruction (in place) */
  const void* mask;
  int64_t rows, cols, pitch; /* pitch in bytes, shared by marker and mask */
  uint8_t* fill_out;   /* chain outputs, dense rows x cols (each optional) */
  int32_t* labels_out;
  uint8_t* area_out;
} nsgb_tile;

/* Host copy of a prepared batch (filled by nsgb_batch_prepare; treat as opaque). */
typedef struct {
  int dtype, n;
  int64_t total_px;
  int recon_tiles, label_tiles, rank_blocks, total_rows, max_cols, max_perimeter;
  void* ws;
  size_t ws_bytes;
  int flood_tiles, bit_words;
  int reserved[6];
} nsgb_batch;

/* Workspace bytes for a batch (total pixels must stay below 2^31). */
size_t nsgb_batch_workspace_size(int dtype, const nsgb_tile* tiles, int n_tiles);
/* Writes the batch's image table into `ws` (synchronous) and fills `batch`.  Afterwards the
 * batch calls below enqueue kernels only, so they can be replayed many times (and recorded
 * once) with the same tiles. */
nsgb_status nsgb_batch_prepare(int dtype, const nsgb_tile* tiles, int n_tiles, void* ws, size_t ws_bytes,
                               nsgb_batch* batch);
/* nsgb_chain on every tile of the batch; n_labels / n_kept: optional host arrays of n_tiles
 * (forcing a synchronization). */
nsgb_status nsgb_chain_batch(const nsgb_batch* batch, int recon_conn, double thr, int fill_conn,
                             int label_conn, int32_t area_min, int32_t area_max, int32_t* n_labels,
                             int32_t* n_kept, nsgb_stream_t stream, const nsgb_opts* opts);
/* Enqueues a copy of the per-tile counts of the last nsgb_chain_batch on this batch into
 * `counts` (device or page-locked host memory, 2 * n_tiles int32: n_labels of tile i at
 * [2i], n_kept at [2i+1]).  No synchronization, so it can be recorded in a CUDA graph after
 * nsgb_chain_batch called with n_labels = n_kept = NULL. */
nsgb_status nsgb_batch_counts_async(const nsgb_batch* batch, int32_t* counts, nsgb_stream_t stream);
/* nsgb_imreconstruct on every tile of the batch, in place on each marker. */
nsgb_status nsgb_imreconstruct_batch(const nsgb_batch* batch, int conn, int erode, nsgb_stream_t stream,
                                     const nsgb_opts* opts);

/* Size of the device scratch built into the library for nsgb_imreconstruct_noalloc: 1 MiB,
 * enough for images of up to 65536 reconstruction tiles -- 134 Mpixel for u8/u16 (tiles of
 * 32 x 64 pixels), 67 Mpixel for i32/f32 (32 x 32), e.g. 8192 x 16384 u8. */
#define NSGB_NOALLOC_SCRATCH_BYTES (1u << 20)

/* No counterpart in the reference: an extra entry point for callers that cannot allocate
 * device memory (a plugin inside a framework that owns the whole GPU pool, a real-time loop
 * that forbids allocation after start-up, a foreign-language host that only receives device
 * buffers).  Same operation and arguments as nsgb_imreconstruct, but without a workspace: the
 * scratch is a fixed NSGB_NOALLOC_SCRATCH_BYTES array in the library's own device memory,
 * held by every GPU that loads the library until the process exits.
 *   - Larger images are refused with NSGB_ERR_WORKSPACE before any GPU work.
 *   - Each call outside stream capture looks up the scratch's device address on the current
 *     device (cudaGetSymbolAddress), so a device reset or a re-created context is followed; a
 *     call made while its stream is capturing uses the address of the last call outside
 *     capture on that device.  Make one call on each device before any stream capture.
 *   - It calls no cudaMalloc / cudaFree and no allocating library routine.
 *   - All calls share the one scratch array and each call re-initialises it; calls whose work
 *     overlaps on the GPU (other streams or host threads) race on it, so serialise them.
 *   - With opts->sync == 0 the call returns once its work is enqueued; its device status
 *     (NOT_CONVERGED, TIMEOUT) is then read with nsgb_noalloc_device_status before the next
 *     call starts, which resets it. */
nsgb_status nsgb_imreconstruct_noalloc(int dtype, void* marker, const void* mask, int64_t rows,
                                       int64_t cols, int64_t pitch, int conn, int erode,
                                       nsgb_stream_t stream, const nsgb_opts* opts);
/* No counterpart in the reference: waits for the work on `stream` and returns the device
 * status of the last nsgb_imreconstruct_noalloc call on the current device (NSGB_OK,
 * NSGB_ERR_NOT_CONVERGED, NSGB_ERR_TIMEOUT), read from the built-in scratch.  Allocates
 * nothing. */
nsgb_status nsgb_noalloc_device_status(nsgb_stream_t stream);

/* ---------------------------------------------------------------------------------------
 * Differentiable float32 reconstruction by dilation.  No counterpart in the reference (its
 * imreconstruct<float>, MorphologicOperations.cpp:665-838 / imreconstructFloatCaller, has no
 * gradient).  Works on `batch` equally sized images stacked `image_stride` bytes apart; all
 * planes (marker, mask, out, prov, gradients) share rows, cols, pitch and image_stride.
 *
 * Forward: out = imreconstruct(marker, mask, conn) (the reference's float semantics,
 * including its zero ring) and prov = the source of each output value:
 *   prov = q       out(p) is marker(q),    q = y * cols + x within the same image
 *   prov = ~q      out(p) is mask(q)
 *   prov = INT32_MIN   out(p) is the constant 0 of the zero ring (border pixels only)
 * Ties (several sources with the value of one connected plateau of equal output) go to a mask
 * source first, then a marker source, then the ring, and the smallest q among those.
 * out must not alias marker.  NaN inputs give NSGB_ERR_BAD_ARG.
 *
 * Backward: grad_marker(q) = sum of grad_out(p) over prov(p) = q, grad_mask(q) = sum over
 * prov(p) = ~q, each the exact sum rounded once to float (nearest, ties to even): the terms
 * are summed as 128-bit fixed-point integers with resolution 2^-96, in which every float from
 * 2^-73 up to 2^31 is exact (smaller magnitudes round to the nearest multiple of 2^-96), so
 * the result does not depend on the order of summation.  |grad_out| < 2^31 and finite, and
 * every sum below 2^31 in magnitude; other gradients, and out-of-range prov entries, are
 * skipped and reported as NSGB_ERR_BAD_ARG. */
size_t nsgb_recon_f32_workspace_size(int64_t batch, int64_t rows, int64_t cols, int backward);
nsgb_status nsgb_recon_f32_fwd(const float* marker, const float* mask, float* out, int32_t* prov, int64_t batch,
                               int64_t rows, int64_t cols, int64_t pitch, int64_t image_stride, int conn, void* ws,
                               size_t ws_bytes, nsgb_stream_t stream, const nsgb_opts* opts);
nsgb_status nsgb_recon_f32_bwd(const float* grad_out, const int32_t* prov, float* grad_marker, float* grad_mask,
                               int64_t batch, int64_t rows, int64_t cols, int64_t pitch, int64_t image_stride,
                               void* ws, size_t ws_bytes, nsgb_stream_t stream, const nsgb_opts* opts);

#ifdef __cplusplus
}
#endif

#endif /* NSGB_H_ */
