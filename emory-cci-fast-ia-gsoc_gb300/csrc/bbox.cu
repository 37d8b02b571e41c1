// Per-label bounding boxes on GB300.
//
// Reference semantics: ConnComponents::boundingBox (src/segment/ConnComponents.cpp:241-284)
// scans the label image in raster order and keeps, per label other than the background, the
// label and its pixels' min x, max x, min y, max y, in the order of the label's first pixel; a
// pixel labelled -1 or 0 that is not the background ends the scan (the reference prints a
// message and stops).  The reference GPU version (cuda/ccl_uf.cu:847-1107, Thrust sort and
// reduce_by_key) orders entries by label value instead; with raster labels (1..n, from the
// relabel) both orders are the same.  This file follows the CPU order.
//
// Schedule: (1) one pass finds where the scan ends (the first -1 / 0 pixel) and the largest
// label, and checks that every label indexes the per-label arrays (which are then initialised
// up to that label only); (2) one pass folds each warp's 32 pixels of a row
// by label (match_any + warp min/max reductions) and updates, per label, its first pixel index
// and the four extremes with one atomic each, skipped when a plain read already shows no
// improvement (the values only move one way, so a stale read can only cost an atomic); (3) the
// first pixel of each present label is marked in a one-bit-per-pixel map, which is counted and
// scanned per 1024-pixel block (the rank machinery of the relabel); (4) each present label
// writes its entry at the rank of its first pixel, i.e. in raster order of first appearance.
#include <climits>

#include "bbox.cuh"
#include "ccl.cuh"
#include "common.cuh"

namespace nsgb {

namespace {

constexpr int kThreads = 256;

size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

struct BWs {
  int* hdr;  // [0] status, [1] stop (first -1 / 0 pixel, or INT_MAX), [2] labels present,
             // [3] largest label seen
  int *first, *mnx, *mxx, *mny, *mxy;
  unsigned* bits;
  size_t bits_bytes;
  int *blk, *wpre;
};

// Per-label planes have px + 1 entries: labels run up to px (an image of isolated pixels).
BWs carve(void* ws, int64_t px) {
  BWs w;
  char* p = (char*)ws;
  const size_t plane = al(sizeof(int) * (size_t)(px + 1));
  const int64_t nblocks = (px + ccl::kBlockPx - 1) / ccl::kBlockPx;
  w.hdr = (int*)p;
  p += 256;
  w.first = (int*)p;
  p += plane;
  w.mnx = (int*)p;
  p += plane;
  w.mxx = (int*)p;
  p += plane;
  w.mny = (int*)p;
  p += plane;
  w.mxy = (int*)p;
  p += plane;
  w.bits = (unsigned*)p;
  w.bits_bytes = sizeof(unsigned) * (size_t)(px / 32 + 2);
  p += al(w.bits_bytes);
  w.blk = (int*)p;
  p += al(sizeof(int) * (size_t)nblocks);
  w.wpre = (int*)p;
  return w;
}

__device__ __forceinline__ int32_t label_at(const Img& m, int y, int x) {
  return *(const int32_t*)((const char*)m.plane + (int64_t)y * m.pitch + (int64_t)x * 4);
}

__global__ void bbox_header(BWs w) {
  w.hdr[0] = 0;
  w.hdr[1] = INT_MAX;
  w.hdr[2] = 0;
  w.hdr[3] = 0;
}

// Label slots in use: 0 .. the largest label seen (raster labels use few of the px + 1 slots).
// A plain load: written by an earlier launch, read by every thread, served from L1 after the
// first warp of each SM.
__device__ __forceinline__ int slots_used(const BWs& w, int n) { return min(n, w.hdr[3] + 1); }

// Per-label arrays to their neutral values, for the slots in use.
__global__ void bbox_init(BWs w, int n_slots) {
  const int n = slots_used(w, n_slots);
  const int stride = gridDim.x * blockDim.x;
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < n; l += stride) {
    w.first[l] = INT_MAX;
    w.mnx[l] = INT_MAX;
    w.mxx[l] = -1;
    w.mny[l] = INT_MAX;
    w.mxy[l] = -1;
  }
}

// Where the scan ends, the largest label, and label range checks.  Every lane of a warp runs the
// loop (lanes past the row end take no part), so the warp reductions see full warps; each block
// folds its rows first and updates the two header words once.
__global__ void __launch_bounds__(kThreads) bbox_scan(Imgs I, int32_t bgval, BWs w) {
  __shared__ int s_stop[kThreads / 32], s_top[kThreads / 32];
  const Img& m = I.one;
  const int n = m.H * m.W;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  int stop = INT_MAX, top = 0;
  for (int y = blockIdx.y; y < m.H; y += gridDim.y) {
    if (x < m.W) {
      const int32_t l = label_at(m, y, x);
      if (l != bgval) {
        if (l == -1 || l == 0) stop = min(stop, y * m.W + x);
        else if (l < 1 || l > n) set_status(w.hdr, NSGB_ERR_BAD_ARG);
        else top = max(top, (int)l);
      }
    }
  }
  stop = __reduce_min_sync(NSGB_FULL, stop);
  top = __reduce_max_sync(NSGB_FULL, top);
  if ((threadIdx.x & 31) == 0) {
    s_stop[threadIdx.x >> 5] = stop;
    s_top[threadIdx.x >> 5] = top;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < kThreads / 32; ++k) {
      stop = min(stop, s_stop[k]);
      top = max(top, s_top[k]);
    }
    if (stop != INT_MAX) atomicMin(w.hdr + 1, stop);
    if (top > 0) atomicMax(w.hdr + 3, top);
  }
}

// Folds each warp's row segment by label, then one update per label and field.  A thread takes
// kAccumRows rows of its column per step and issues all their label loads before using any
// (one load per thread and step left the kernel waiting on load latency).
constexpr int kAccumRows = 8;

__global__ void __launch_bounds__(kThreads) bbox_accum(Imgs I, int32_t bgval, BWs w) {
  const Img& m = I.one;
  const int n = m.H * m.W;
  const int stop = __ldcg(w.hdr + 1);
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  for (int y0 = blockIdx.y * kAccumRows; y0 < m.H; y0 += gridDim.y * kAccumRows) {
    int32_t lab[kAccumRows];
#pragma unroll
    for (int r = 0; r < kAccumRows; ++r) {
      const int y = y0 + r;
      lab[r] = (x < m.W && y < m.H && y * m.W + x < stop) ? label_at(m, y, x) : bgval;
    }
#pragma unroll
    for (int r = 0; r < kAccumRows; ++r) {
      const int y = y0 + r;
      const int32_t l = lab[r];
      const int key = (l != bgval && l >= 1 && l <= n) ? (int)l : -1;
      const unsigned peers = __match_any_sync(NSGB_FULL, key);
      if (key < 0) continue;
      const int xmin = __reduce_min_sync(peers, x);
      const int xmax = __reduce_max_sync(peers, x);
      if (lane != __ffs(peers) - 1) continue;
      const int fi = y * m.W + xmin;
      if (fi < w.first[key]) atomicMin(w.first + key, fi);
      if (xmin < w.mnx[key]) atomicMin(w.mnx + key, xmin);
      if (xmax > w.mxx[key]) atomicMax(w.mxx + key, xmax);
      if (y < w.mny[key]) atomicMin(w.mny + key, y);
      if (y > w.mxy[key]) atomicMax(w.mxy + key, y);
    }
  }
}

// The first pixel of every present label into the bitmap; labels counted.
__global__ void __launch_bounds__(kThreads) bbox_mark(BWs w, int n_slots) {
  const int n = slots_used(w, n_slots);
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const int l = base + threadIdx.x;
    const bool present = l < n && __ldcg(w.mxx + l) >= 0;
    if (present) {
      const int f = __ldcg(w.first + l);
      atomicOr(w.bits + (f >> 5), 1u << (f & 31));
    }
    const unsigned b = __ballot_sync(NSGB_FULL, present);
    if (b && (threadIdx.x & 31) == 0) atomicAdd(w.hdr + 2, __popc(b));
  }
}

// Entry of each present label at the rank of its first pixel.
__global__ void __launch_bounds__(kThreads) bbox_out(BWs w, int n_slots, int32_t* boxes, int64_t cap) {
  const int n = slots_used(w, n_slots);
  const int stride = gridDim.x * blockDim.x;
  for (int l = blockIdx.x * blockDim.x + threadIdx.x; l < n; l += stride) {
    if (__ldcg(w.mxx + l) < 0) continue;
    const int r = ccl::bit_rank(w.bits, w.blk, w.wpre, __ldcg(w.first + l));
    if (r >= cap) continue;
    boxes[r] = l;
    boxes[cap + r] = __ldcg(w.mnx + l);
    boxes[2 * cap + r] = __ldcg(w.mxx + l);
    boxes[3 * cap + r] = __ldcg(w.mny + l);
    boxes[4 * cap + r] = __ldcg(w.mxy + l);
  }
}

}  // namespace

size_t bbox_workspace_bytes(int64_t px) {
  const int64_t nblocks = (px + ccl::kBlockPx - 1) / ccl::kBlockPx;
  return 256 + 5 * al(sizeof(int) * (size_t)(px + 1)) + al(sizeof(unsigned) * (size_t)(px / 32 + 2)) +
         al(sizeof(int) * (size_t)nblocks) + al(sizeof(int) * 32 * (size_t)nblocks);
}

cudaError_t bbox_launch(const Imgs& I, const BatchTotals& t, int32_t bgval, void* ws, int32_t* boxes, int64_t cap,
                        int32_t* count_dev, cudaStream_t s) {
  const int n = (int)t.px + 1;  // label values 0 .. px
  BWs w = carve(ws, t.px);
  cudaError_t e = cudaMemsetAsync(w.bits, 0, w.bits_bytes, s);
  if (e != cudaSuccess) return e;
  const int g = ccl::flat_grid(n);
  const dim3 rows = ccl::rowcol_grid(t.rows, t.max_w);
  bbox_header<<<1, 1, 0, s>>>(w);
  bbox_scan<<<dim3(rows.x, rows.y < 512 ? rows.y : 512), kThreads, 0, s>>>(I, bgval, w);
  bbox_init<<<g, kThreads, 0, s>>>(w, n);
  const int ry = (rows.y + kAccumRows - 1) / kAccumRows;
  bbox_accum<<<dim3(rows.x, ry < 65535 ? ry : 65535), kThreads, 0, s>>>(I, bgval, w);
  bbox_mark<<<g, kThreads, 0, s>>>(w, n);
  e = ccl::rank_bits(I, t, w.bits, w.blk, w.wpre, s);
  if (e != cudaSuccess) return e;
  bbox_out<<<g, kThreads, 0, s>>>(w, n, boxes, cap);
  e = cudaGetLastError();
  if (e == cudaSuccess && count_dev) e = cudaMemcpyAsync(count_dev, w.hdr + 2, sizeof(int32_t), cudaMemcpyDeviceToDevice, s);
  return e;
}

}  // namespace nsgb
