// The operations of the reconstruction / labelling path and their C ABI (include/nsgb.h).
// Each operation is a short sequence of kernels on the caller's stream, using only the
// caller's workspace.  Reference functions are cited at each entry point.
#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>
#include <string.h>

#include <limits>

#include "../../include/nsgb.h"
#include "ccl.cuh"
#include "common.cuh"
#include "recon.cuh"

namespace nsgb {
namespace {

// ------------------------------------------------------------------------------------------
// Pixel access helpers.
template <typename T>
__device__ __forceinline__ T px(const T* base, int64_t pitch, int y, int x) {
  return __ldg((const T*)((const char*)base + (int64_t)y * pitch) + x);
}
template <typename T>
__device__ __forceinline__ T pxcg(const T* base, int64_t pitch, int y, int x) {
  return __ldcg((const T*)((const char*)base + (int64_t)y * pitch) + x);
}
template <typename T>
__device__ __forceinline__ T* pxp(T* base, int64_t pitch, int y, int x) {
  return (T*)((char*)base + (int64_t)y * pitch) + x;
}

// ------------------------------------------------------------------------------------------
// Classifiers (class 0 = background; equal non-zero classes are joined).
struct ClsValueU8 {  // bwlabel: the pixel value
  const uint8_t* img;
  int64_t pitch;
  __device__ uint32_t operator()(int y, int x) const { return px(img, pitch, y, x); }
};
template <typename T>
struct ClsNonZero {  // binary reconstruction, bwselect: mask != 0
  const T* img;
  int64_t pitch;
  __device__ uint32_t operator()(int y, int x) const { return px(img, pitch, y, x) != (T)0 ? 1u : 0u; }
};
template <typename T>
struct ClsNotMax {  // binary hole filling: pixels that are not foreground (max<T>)
  const T* img;
  int64_t pitch;
  __device__ uint32_t operator()(int y, int x) const {
    return px(img, pitch, y, x) != std::numeric_limits<T>::max() ? 1u : 0u;
  }
};
template <typename T>
struct ClsNotAbove {  // hole filling of (R > thr): the complement class !(R > thr)
  const T* img;
  int64_t pitch;
  double thr;
  __device__ uint32_t operator()(int y, int x) const { return !((double)pxcg(img, pitch, y, x) > thr) ? 1u : 0u; }
};

// Seeds (pixels that flag their component's root).
template <class Cls>
struct SeedBorder {
  Cls cls;
  int H, W;
  __device__ bool operator()(int y, int x) const {
    return (y == 0 || y == H - 1 || x == 0 || x == W - 1) && cls(y, x) != 0u;
  }
};
template <typename T>
struct SeedBoth {  // marker != 0 and mask != 0
  const T* a;
  const T* b;
  int64_t pitch;
  __device__ bool operator()(int y, int x) const {
    return pxcg(a, pitch, y, x) != (T)0 && px(b, pitch, y, x) != (T)0;
  }
};

// ------------------------------------------------------------------------------------------
// Output kernels.  Row / column grids (x = column, y strides rows); a pixel's root is
// L[L[i]] after the labelling (ccl::root_of).

// Binary hole filling: 0 where the non-foreground pixel's component touches the border.
template <typename TO>
__global__ void fill_out_kernel(int H, int W, const int* __restrict__ L, const unsigned* __restrict__ bits, TO* out,
                                int64_t pitch_out, TO fg) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= W) return;
  for (int y = blockIdx.y; y < H; y += gridDim.y) {
    const int r = ccl::root_of(L, (int64_t)y * W + x);
    *pxp(out, pitch_out, y, x) = (r >= 0 && ccl::test_bit(bits, r)) ? (TO)0 : fg;
  }
}

// Binary reconstruction output, in place on the marker.
template <typename T>
__global__ void binrecon_out_kernel(T* marker, int64_t pitch, int H, int W, const int* __restrict__ L,
                                    const unsigned* __restrict__ bits) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= W) return;
  for (int y = blockIdx.y; y < H; y += gridDim.y) {
    T* p = pxp(marker, pitch, y, x);
    if (*p != (T)0) continue;
    const int r = ccl::root_of(L, (int64_t)y * W + x);
    if (r >= 0 && ccl::test_bit(bits, r)) *p = std::numeric_limits<T>::max();
  }
}

template <typename T>
__global__ void bwselect_out_kernel(const T* image, T* out, int64_t pitch, int H, int W, const int* __restrict__ L,
                                    const unsigned* __restrict__ bits) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= W) return;
  for (int y = blockIdx.y; y < H; y += gridDim.y) {
    const T v = px(image, pitch, y, x);
    const int r = ccl::root_of(L, (int64_t)y * W + x);
    *pxp(out, pitch, y, x) = (v != (T)0 && r >= 0 && ccl::test_bit(bits, r)) ? v : (T)0;
  }
}

// Labels out: relabel ? (bg 0, root's rank + 1) : root index / -1.  Optional area-filter
// outputs from the same pass.  rank / A are read-only here: L1-cached loads, because a giant
// component's root is read by every one of its pixels.
__global__ void label_out_kernel(int H, int W, const int* __restrict__ L, const int* __restrict__ rank, int relabel,
                                 int32_t* labels, int64_t pitch_labels, const int* __restrict__ A, int lo, int hi,
                                 int32_t* kept_labels, int64_t pitch_kept, uint8_t* flat, int64_t pitch_flat) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= W) return;
  for (int y = blockIdx.y; y < H; y += gridDim.y) {
    const int r = ccl::root_of(L, (int64_t)y * W + x);
    if (labels) *pxp(labels, pitch_labels, y, x) = relabel ? (r < 0 ? 0 : __ldg(&rank[r]) + 1) : r;
    if (A) {
      const int a = r >= 0 ? __ldg(&A[r]) : 0;
      const bool keep = r >= 0 && a >= lo && a < hi;
      if (kept_labels) *pxp(kept_labels, pitch_kept, y, x) = keep ? r : -1;
      if (flat) *pxp(flat, pitch_flat, y, x) = keep ? 255 : 0;
    }
  }
}

// Area of arbitrary int32 labels in [-1, n): dense histogram (background -1 skipped).
__global__ void label_hist_kernel(const int32_t* lab, int64_t pitch, int H, int W, int* __restrict__ A, int* status) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= W) return;
  const int64_t n = (int64_t)H * W;
  for (int y = blockIdx.y; y < H; y += gridDim.y) {
    const int l = px(lab, pitch, y, x);
    if (l == -1) continue;
    if (l < -1 || (int64_t)l >= n) {
      set_status(status, NSGB_ERR_BAD_ARG);
      continue;
    }
    atomicAdd(&A[l], 1);
  }
}

__global__ void labeled_area_out_kernel(const int32_t* lab, int64_t pitch, int H, int W, const int* __restrict__ A,
                                        int lo, int hi, int32_t* kept_labels, int64_t pitch_kept, uint8_t* flat,
                                        int64_t pitch_flat) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= W) return;
  const int64_t n = (int64_t)H * W;
  for (int y = blockIdx.y; y < H; y += gridDim.y) {
    const int l = px(lab, pitch, y, x);
    const int a = (l >= 0 && (int64_t)l < n) ? __ldg(&A[l]) : 0;
    const bool keep = l >= 0 && (int64_t)l < n && a >= lo && a < hi;
    if (kept_labels) *pxp(kept_labels, pitch_kept, y, x) = keep ? l : -1;
    if (flat) *pxp(flat, pitch_flat, y, x) = keep ? 255 : 0;
  }
}

__global__ void count_labels_in_range_kernel(const int* __restrict__ A, int64_t n, int lo, int hi, int* out) {
  int c = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int a = __ldcg(&A[i]);
    if (a > 0 && a >= lo && a < hi) ++c;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(NSGB_FULL, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// ------------------------------------------------------------------------------------------
// Elementwise kernels (row / column grids).
#define NSGB_FOR_PIXELS                                   \
  const int x = blockIdx.x * blockDim.x + threadIdx.x;    \
  if (x >= W) return;                                     \
  for (int y = blockIdx.y; y < H; y += gridDim.y)

template <typename T>
__global__ void threshold_kernel(const T* in, int64_t pitch_in, uint8_t* out, int64_t pitch_out, int H, int W,
                                 double thr) {
  NSGB_FOR_PIXELS { *pxp(out, pitch_out, y, x) = (double)px(in, pitch_in, y, x) > thr ? 255 : 0; }
}

template <typename T>
__device__ __forceinline__ T invert_value(T v) {
  if constexpr (std::numeric_limits<T>::is_integer) {
    if constexpr (std::numeric_limits<T>::is_signed) {
      return v == std::numeric_limits<T>::min() ? std::numeric_limits<T>::max() : (T)(-v);
    } else {
      return (T)(std::numeric_limits<T>::max() - v);
    }
  } else {
    return -v;
  }
}

template <typename T>
__global__ void invert_kernel(const T* in, T* out, int64_t pitch, int H, int W) {
  NSGB_FOR_PIXELS { *pxp(out, pitch, y, x) = invert_value(px(in, pitch, y, x)); }
}

// Hole-filling marker: the image on the border, max<T> inside.
template <typename T>
__global__ void fill_marker_kernel(const T* image, T* out, int64_t pitch, int H, int W) {
  NSGB_FOR_PIXELS {
    const bool border = y == 0 || y == H - 1 || x == 0 || x == W - 1;
    *pxp(out, pitch, y, x) = border ? px(image, pitch, y, x) : std::numeric_limits<T>::max();
  }
}

// h-minima marker: image + h, saturating for integers.
template <typename T>
__global__ void hmin_marker_kernel(const T* image, T* out, int64_t pitch, int H, int W, double h) {
  NSGB_FOR_PIXELS {
    const T v = px(image, pitch, y, x);
    T r;
    if constexpr (std::numeric_limits<T>::is_integer) {
      const int64_t s = (int64_t)v + (int64_t)h;
      r = (T)(s > (int64_t)std::numeric_limits<T>::max() ? (int64_t)std::numeric_limits<T>::max() : s);
    } else {
      r = v + (T)h;
    }
    *pxp(out, pitch, y, x) = r;
  }
}

template <typename T>
__global__ void fill_const_kernel(T* out, int64_t pitch, int H, int W, T v) {
  NSGB_FOR_PIXELS { *pxp(out, pitch, y, x) = v; }
}

// ------------------------------------------------------------------------------------------
// Workspace layout.  [recon region][L: N ints][A: N ints][R: N ints][bits][rank tmp][F: N bytes]
struct Ws {
  int* status;  // == start of the recon region
  void* recon;
  int* L;
  int* A;
  int* R;        // root ranks; before ranking, the list of local roots
  unsigned* bits;
  int* tmp;
  int* counts;   // [2]
  int* nroots;   // [1]
  uint8_t* F;
  ccl::Forest forest(bool areas) const { return ccl::Forest{L, areas ? A : nullptr, R, nroots}; }
};

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

struct WsSizes {
  size_t recon, L, A, R, bits, tmp, F, total;
};

WsSizes ws_sizes(int dtype, int64_t H, int64_t W) {
  WsSizes z;
  const int64_t n = H * W;
  const int rd = dtype >= 0 && dtype <= 3 ? dtype : 0;
  z.recon = align256(recon_workspace_bytes(rd, H, W));
  z.L = align256(sizeof(int) * (size_t)n);
  z.A = z.L;
  z.R = z.L;
  z.bits = align256(sizeof(unsigned) * (size_t)((n + 31) / 32 + 1));
  z.tmp = align256(sizeof(int) * (ccl::rank_tmp_ints(n) + 4));
  z.F = align256((size_t)n);
  z.total = z.recon + z.L + z.A + z.R + z.bits + z.tmp + z.F;
  return z;
}

Ws carve(void* ws, int dtype, int64_t H, int64_t W) {
  const WsSizes z = ws_sizes(dtype, H, W);
  char* p = (char*)ws;
  Ws w;
  w.status = (int*)p;
  w.recon = p;
  p += z.recon;
  w.L = (int*)p;
  p += z.L;
  w.A = (int*)p;
  p += z.A;
  w.R = (int*)p;
  p += z.R;
  w.bits = (unsigned*)p;
  p += z.bits;
  w.tmp = (int*)p;
  w.counts = w.tmp + (ccl::rank_tmp_ints(H * W));
  w.nroots = w.counts + 2;
  p += z.tmp;
  w.F = (uint8_t*)p;
  return w;
}

inline int grid1d(int64_t n) { return ccl::flat_grid(n); }
inline dim3 rc(int64_t rows, int64_t cols) { return ccl::rowcol_grid((int)rows, (int)cols); }

}  // namespace
}  // namespace nsgb

// ============================================================================================
// C ABI
using namespace nsgb;

namespace {

bool valid_dims(int64_t rows, int64_t cols) {
  return rows > 0 && cols > 0 && rows * cols < (int64_t)INT_MAX && rows < INT_MAX && cols < INT_MAX;
}
bool valid_pitch(int64_t pitch, int64_t cols, int esz) { return pitch >= cols * esz && pitch % esz == 0; }
bool valid_conn(int conn) { return conn == 4 || conn == 8; }
bool want_sync(const nsgb_opts* o) { return o == nullptr || o->sync != 0; }

nsgb_status cuda_status(cudaError_t e) { return e == cudaSuccess ? NSGB_OK : NSGB_ERR_CUDA; }

// Records the caller's optional timing event around the reconstruction kernel.
cudaError_t record(const nsgb_opts* o, bool begin, cudaStream_t s) {
  if (!o) return cudaSuccess;
  void* ev = begin ? o->recon_event_begin : o->recon_event_end;
  return ev ? cudaEventRecord((cudaEvent_t)ev, s) : cudaSuccess;
}

// Reconstruction launch bracketed by the optional timing events.
cudaError_t recon_timed(const nsgb_opts* o, int dtype, void* out, const void* marker, const void* mask, int64_t H,
                        int64_t W, int64_t pitch, int conn, bool erode, bool ring, void* ws, cudaStream_t s) {
  cudaError_t e = record(o, true, s);
  if (e != cudaSuccess) return e;
  e = recon_launch(dtype, out, marker, mask, H, W, pitch, conn, erode, ring, ws, s, o ? o->max_visits_per_tile : 0,
                   o ? o->max_visit_iters : 0);
  if (e != cudaSuccess) return e;
  return record(o, false, s);
}

// Finishes a call: reports launch errors; with sync, waits and reports the device status.
nsgb_status finish(cudaError_t e, const void* ws, cudaStream_t s, const nsgb_opts* o) {
  if (e != cudaSuccess) return NSGB_ERR_CUDA;
  e = cudaGetLastError();
  if (e != cudaSuccess) return NSGB_ERR_CUDA;
  if (!want_sync(o)) return NSGB_OK;
  int dev_status = 0;
  e = cudaMemcpyAsync(&dev_status, ws, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return NSGB_ERR_CUDA;
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return NSGB_ERR_CUDA;
  return (nsgb_status)dev_status;
}

nsgb_status check_ws(void* ws, size_t ws_bytes, int op, int dtype, int64_t rows, int64_t cols) {
  if (!ws) return NSGB_ERR_WORKSPACE;
  if (ws_bytes < nsgb_workspace_size(op, dtype, rows, cols)) return NSGB_ERR_WORKSPACE;
  if ((uintptr_t)ws % 256 != 0) return NSGB_ERR_WORKSPACE;
  return NSGB_OK;
}

template <typename F>
cudaError_t dispatch_int(int dtype, F&& f) {
  switch (dtype) {
    case NSGB_U8: return f((uint8_t*)nullptr);
    case NSGB_U16: return f((uint16_t*)nullptr);
    case NSGB_I32: return f((int32_t*)nullptr);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

extern "C" {

size_t nsgb_workspace_size(int op, int dtype, int64_t rows, int64_t cols) {
  if (rows <= 0 || cols <= 0) return 0;
  if (op == NSGB_OP_BWLABEL || op == NSGB_OP_BWAREAOPEN) dtype = NSGB_U8;
  if (op == NSGB_OP_IMRECONSTRUCT || op == NSGB_OP_HMIN) return align256(recon_workspace_bytes(dtype, rows, cols));
  if (op == NSGB_OP_FILL_HOLES) {
    const WsSizes z = ws_sizes(dtype, rows, cols);
    return z.total;
  }
  return ws_sizes(dtype, rows, cols).total;
}

const char* nsgb_status_string(int status) {
  switch (status) {
    case NSGB_OK: return "ok";
    case NSGB_ERR_BAD_ARG: return "bad argument";
    case NSGB_ERR_UNSUPPORTED_DTYPE: return "unsupported dtype for this operation";
    case NSGB_ERR_WORKSPACE: return "workspace missing, misaligned or too small";
    case NSGB_ERR_NOT_CONVERGED: return "iteration budget exhausted before convergence";
    case NSGB_ERR_TIMEOUT: return "a bounded device-side wait timed out";
    case NSGB_ERR_CUDA: return "CUDA runtime error";
    case NSGB_ERR_QUEUE_OVERFLOW: return "device work list overflow";
    default: return "unknown status";
  }
}

nsgb_status nsgb_device_status(const void* ws, nsgb_stream_t stream) {
  if (!ws) return NSGB_ERR_WORKSPACE;
  int v = 0;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaMemcpyAsync(&v, ws, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess) return NSGB_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return NSGB_ERR_CUDA;
  return (nsgb_status)v;
}

nsgb_status nsgb_imreconstruct(int dtype, void* marker, const void* mask, int64_t rows, int64_t cols, int64_t pitch,
                               int conn, int erode, void* ws, size_t ws_bytes, nsgb_stream_t stream,
                               const nsgb_opts* opts) {
  const int esz = elem_size(dtype);
  if (!esz) return NSGB_ERR_UNSUPPORTED_DTYPE;
  if (!marker || !mask || !valid_dims(rows, cols) || !valid_pitch(pitch, cols, esz) || !valid_conn(conn))
    return NSGB_ERR_BAD_ARG;
  nsgb_status st = check_ws(ws, ws_bytes, NSGB_OP_IMRECONSTRUCT, dtype, rows, cols);
  if (st != NSGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const bool ring = !erode && (dtype == NSGB_I32 || dtype == NSGB_F32);
  cudaError_t e = recon_timed(opts, dtype, marker, marker, mask, rows, cols, pitch, conn, erode != 0, ring, ws, s);
  return finish(e, ws, s, opts);
}

nsgb_status nsgb_imreconstruct_binary(int dtype, void* marker, const void* mask, int64_t rows, int64_t cols,
                                      int64_t pitch, int conn, void* ws, size_t ws_bytes, nsgb_stream_t stream,
                                      const nsgb_opts* opts) {
  const int esz = elem_size(dtype);
  if (!esz) return NSGB_ERR_UNSUPPORTED_DTYPE;
  if (dtype == NSGB_F32) return NSGB_ERR_UNSUPPORTED_DTYPE;
  if (!marker || !mask || !valid_dims(rows, cols) || !valid_pitch(pitch, cols, esz) || !valid_conn(conn))
    return NSGB_ERR_BAD_ARG;
  nsgb_status st = check_ws(ws, ws_bytes, NSGB_OP_IMRECONSTRUCT_BINARY, dtype, rows, cols);
  if (st != NSGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int H = (int)rows, W = (int)cols;
  Ws w = carve(ws, dtype, rows, cols);
  cudaError_t e = cudaMemsetAsync(w.status, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.bits, 0, sizeof(unsigned) * (size_t)((rows * cols + 31) / 32 + 1), s);
  if (e == cudaSuccess) {
    e = dispatch_int(dtype, [&](auto* tag) -> cudaError_t {
      using T = std::remove_pointer_t<decltype(tag)>;
      ClsNonZero<T> cls{(const T*)mask, pitch};
      SeedBoth<T> seed{(const T*)marker, (const T*)mask, pitch};
      cudaError_t r = ccl::label(cls, H, W, conn, w.forest(false), s);
      if (r != cudaSuccess) return r;
      ccl::ccl_seed_pixels<SeedBoth<T>><<<rc(rows, cols), 256, 0, s>>>(H, W, w.L, seed, w.bits);
      binrecon_out_kernel<T><<<rc(rows, cols), 256, 0, s>>>((T*)marker, pitch, H, W, w.L, w.bits);
      return cudaGetLastError();
    });
  }
  return finish(e, ws, s, opts);
}

nsgb_status nsgb_imfill_holes(int dtype, const void* image, void* out, int64_t rows, int64_t cols, int64_t pitch,
                              int binary, int conn, void* ws, size_t ws_bytes, nsgb_stream_t stream,
                              const nsgb_opts* opts) {
  const int esz = elem_size(dtype);
  if (!esz) return NSGB_ERR_UNSUPPORTED_DTYPE;
  if (!image || !out || !valid_dims(rows, cols) || !valid_pitch(pitch, cols, esz) || !valid_conn(conn))
    return NSGB_ERR_BAD_ARG;
  if (binary && dtype == NSGB_F32) return NSGB_ERR_UNSUPPORTED_DTYPE;
  nsgb_status st = check_ws(ws, ws_bytes, NSGB_OP_FILL_HOLES, dtype, rows, cols);
  if (st != NSGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int H = (int)rows, W = (int)cols;
  Ws w = carve(ws, dtype, rows, cols);
  cudaError_t e = cudaMemsetAsync(w.status, 0, sizeof(int), s);
  if (e != cudaSuccess) return NSGB_ERR_CUDA;
  if (binary) {
    if (dtype == NSGB_I32) {
      // min<int> is non-zero, so the reference's binary reconstruction has no background to
      // grow into and every pixel comes back as invert(min<int>) = INT_MAX.
      fill_const_kernel<int32_t><<<rc(rows, cols), 256, 0, s>>>((int32_t*)out, pitch, H, W, INT_MAX);
      return finish(cudaGetLastError(), ws, s, opts);
    }
    e = cudaMemsetAsync(w.bits, 0, sizeof(unsigned) * (size_t)((rows * cols + 31) / 32 + 1), s);
    if (e == cudaSuccess) {
      e = dispatch_int(dtype, [&](auto* tag) -> cudaError_t {
        using T = std::remove_pointer_t<decltype(tag)>;
        ClsNotMax<T> cls{(const T*)image, pitch};
        SeedBorder<ClsNotMax<T>> seed{cls, H, W};
        cudaError_t r = ccl::label(cls, H, W, conn, w.forest(false), s);
        if (r != cudaSuccess) return r;
        ccl::ccl_seed_border<SeedBorder<ClsNotMax<T>>><<<grid1d(2 * (rows + cols)), 256, 0, s>>>(H, W, w.L, seed,
                                                                                                w.bits);
        fill_out_kernel<T><<<rc(rows, cols), 256, 0, s>>>(H, W, w.L, w.bits, (T*)out, pitch,
                                                          std::numeric_limits<T>::max());
        return cudaGetLastError();
      });
    }
    return finish(e, ws, s, opts);
  }
  // Grayscale: erosion reconstruction of (image on the border, max inside) above the image.
  if (out == image) return NSGB_ERR_BAD_ARG;
  switch (dtype) {
    case NSGB_U8: fill_marker_kernel<uint8_t><<<rc(rows, cols), 256, 0, s>>>((const uint8_t*)image, (uint8_t*)out, pitch, H, W); break;
    case NSGB_U16: fill_marker_kernel<uint16_t><<<rc(rows, cols), 256, 0, s>>>((const uint16_t*)image, (uint16_t*)out, pitch, H, W); break;
    case NSGB_I32: fill_marker_kernel<int32_t><<<rc(rows, cols), 256, 0, s>>>((const int32_t*)image, (int32_t*)out, pitch, H, W); break;
    case NSGB_F32: fill_marker_kernel<float><<<rc(rows, cols), 256, 0, s>>>((const float*)image, (float*)out, pitch, H, W); break;
  }
  e = recon_launch(dtype, out, out, image, rows, cols, pitch, conn, true, false, ws, s, opts ? opts->max_visits_per_tile : 0,
                   opts ? opts->max_visit_iters : 0);
  return finish(e, ws, s, opts);
}

nsgb_status nsgb_imhmin(int dtype, const void* image, void* out, int64_t rows, int64_t cols, int64_t pitch, double h,
                        int conn, void* ws, size_t ws_bytes, nsgb_stream_t stream, const nsgb_opts* opts) {
  const int esz = elem_size(dtype);
  if (!esz || dtype == NSGB_I32) return NSGB_ERR_UNSUPPORTED_DTYPE;
  if (!image || !out || out == image || !valid_dims(rows, cols) || !valid_pitch(pitch, cols, esz) ||
      !valid_conn(conn))
    return NSGB_ERR_BAD_ARG;
  nsgb_status st = check_ws(ws, ws_bytes, NSGB_OP_HMIN, dtype, rows, cols);
  if (st != NSGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int H = (int)rows, W = (int)cols;
  switch (dtype) {
    case NSGB_U8: hmin_marker_kernel<uint8_t><<<rc(rows, cols), 256, 0, s>>>((const uint8_t*)image, (uint8_t*)out, pitch, H, W, h); break;
    case NSGB_U16: hmin_marker_kernel<uint16_t><<<rc(rows, cols), 256, 0, s>>>((const uint16_t*)image, (uint16_t*)out, pitch, H, W, h); break;
    case NSGB_F32: hmin_marker_kernel<float><<<rc(rows, cols), 256, 0, s>>>((const float*)image, (float*)out, pitch, H, W, h); break;
  }
  // invert(recon(invert(I) - h, invert(I))): the order-reversed reconstruction with the
  // reference's 0-valued padding ring taken in the inverted domain.
  cudaError_t e = recon_launch(dtype, out, out, image, rows, cols, pitch, conn, true, true, ws, s,
                               opts ? opts->max_visits_per_tile : 0, opts ? opts->max_visit_iters : 0);
  return finish(e, ws, s, opts);
}

nsgb_status nsgb_bwselect(int dtype, const void* image, const void* seeds, void* out, int64_t rows, int64_t cols,
                          int64_t pitch, int conn, void* ws, size_t ws_bytes, nsgb_stream_t stream,
                          const nsgb_opts* opts) {
  const int esz = elem_size(dtype);
  if (!esz || dtype == NSGB_F32) return NSGB_ERR_UNSUPPORTED_DTYPE;
  if (!image || !seeds || !out || !valid_dims(rows, cols) || !valid_pitch(pitch, cols, esz) || !valid_conn(conn))
    return NSGB_ERR_BAD_ARG;
  nsgb_status st = check_ws(ws, ws_bytes, NSGB_OP_BWSELECT, dtype, rows, cols);
  if (st != NSGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int H = (int)rows, W = (int)cols;
  Ws w = carve(ws, dtype, rows, cols);
  cudaError_t e = cudaMemsetAsync(w.status, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.bits, 0, sizeof(unsigned) * (size_t)((rows * cols + 31) / 32 + 1), s);
  if (e == cudaSuccess) {
    e = dispatch_int(dtype, [&](auto* tag) -> cudaError_t {
      using T = std::remove_pointer_t<decltype(tag)>;
      ClsNonZero<T> cls{(const T*)image, pitch};
      SeedBoth<T> seed{(const T*)seeds, (const T*)image, pitch};
      cudaError_t r = ccl::label(cls, H, W, conn, w.forest(false), s);
      if (r != cudaSuccess) return r;
      ccl::ccl_seed_pixels<SeedBoth<T>><<<rc(rows, cols), 256, 0, s>>>(H, W, w.L, seed, w.bits);
      bwselect_out_kernel<T><<<rc(rows, cols), 256, 0, s>>>((const T*)image, (T*)out, pitch, H, W, w.L, w.bits);
      return cudaGetLastError();
    });
  }
  return finish(e, ws, s, opts);
}

nsgb_status nsgb_bwlabel(const uint8_t* bin, int32_t* labels, int64_t rows, int64_t cols, int64_t pitch_in,
                         int64_t pitch_labels, int conn, int relabel, int32_t* count, void* ws, size_t ws_bytes,
                         nsgb_stream_t stream, const nsgb_opts* opts) {
  if (!bin || !labels || !valid_dims(rows, cols) || !valid_pitch(pitch_in, cols, 1) ||
      !valid_pitch(pitch_labels, cols, 4) || !valid_conn(conn))
    return NSGB_ERR_BAD_ARG;
  nsgb_status st = check_ws(ws, ws_bytes, NSGB_OP_BWLABEL, NSGB_U8, rows, cols);
  if (st != NSGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int H = (int)rows, W = (int)cols;
  const int64_t n = rows * cols;
  Ws w = carve(ws, NSGB_U8, rows, cols);
  cudaError_t e = cudaMemsetAsync(w.status, 0, sizeof(int), s);
  if (e != cudaSuccess) return NSGB_ERR_CUDA;
  ClsValueU8 cls{bin, pitch_in};
  e = ccl::label(cls, H, W, conn, w.forest(false), s);
  if (e == cudaSuccess) e = ccl::rank_roots(w.L, nullptr, n, 0, 0, w.R, w.tmp, w.counts, s);
  if (e == cudaSuccess) {
    label_out_kernel<<<rc(rows, cols), 256, 0, s>>>(H, W, w.L, w.R, relabel, labels, pitch_labels, nullptr, 0, 0, nullptr,
                                               0, nullptr, 0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && count) {
    e = cudaMemcpyAsync(count, w.counts, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  return finish(e, ws, s, opts);
}

nsgb_status nsgb_bwareaopen(const void* in, int labeled, int32_t* labels_out, uint8_t* flat_out, int64_t rows,
                            int64_t cols, int64_t pitch_in, int64_t pitch_labels, int64_t pitch_flat, int32_t min_size,
                            int32_t max_size, int conn, int32_t* count, void* ws, size_t ws_bytes,
                            nsgb_stream_t stream, const nsgb_opts* opts) {
  if (!in || !valid_dims(rows, cols) || !valid_pitch(pitch_in, cols, labeled ? 4 : 1) || !valid_conn(conn))
    return NSGB_ERR_BAD_ARG;
  if (labels_out && !valid_pitch(pitch_labels, cols, 4)) return NSGB_ERR_BAD_ARG;
  if (flat_out && !valid_pitch(pitch_flat, cols, 1)) return NSGB_ERR_BAD_ARG;
  nsgb_status st = check_ws(ws, ws_bytes, NSGB_OP_BWAREAOPEN, NSGB_U8, rows, cols);
  if (st != NSGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int H = (int)rows, W = (int)cols;
  const int64_t n = rows * cols;
  Ws w = carve(ws, NSGB_U8, rows, cols);
  cudaError_t e = cudaMemsetAsync(w.status, 0, sizeof(int), s);
  if (e != cudaSuccess) return NSGB_ERR_CUDA;
  if (!labeled) {
    ClsValueU8 cls{(const uint8_t*)in, pitch_in};
    e = ccl::label(cls, H, W, conn, w.forest(true), s);
    if (e == cudaSuccess) e = ccl::rank_roots(w.L, w.A, n, min_size, max_size, w.R, w.tmp, w.counts, s);
    if (e == cudaSuccess) {
      label_out_kernel<<<rc(rows, cols), 256, 0, s>>>(H, W, w.L, w.R, 0, nullptr, 0, w.A, min_size, max_size, labels_out,
                                                 pitch_labels, flat_out, pitch_flat);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess && count) {
      e = cudaMemcpyAsync(count, w.counts + 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    }
    return finish(e, ws, s, opts);
  }
  e = cudaMemsetAsync(w.A, 0, sizeof(int) * (size_t)n, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.counts, 0, 2 * sizeof(int), s);
  if (e == cudaSuccess) {
    label_hist_kernel<<<rc(rows, cols), 256, 0, s>>>((const int32_t*)in, pitch_in, H, W, w.A, w.status);
    count_labels_in_range_kernel<<<grid1d(n), 256, 0, s>>>(w.A, n, min_size, max_size, w.counts + 1);
    labeled_area_out_kernel<<<rc(rows, cols), 256, 0, s>>>((const int32_t*)in, pitch_in, H, W, w.A, min_size, max_size,
                                                      labels_out, pitch_labels, flat_out, pitch_flat);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && count) {
    e = cudaMemcpyAsync(count, w.counts + 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  return finish(e, ws, s, opts);
}

nsgb_status nsgb_threshold(int dtype, const void* in, uint8_t* out, int64_t rows, int64_t cols, int64_t pitch_in,
                           int64_t pitch_out, double thr, nsgb_stream_t stream) {
  const int esz = elem_size(dtype);
  if (!esz) return NSGB_ERR_UNSUPPORTED_DTYPE;
  if (!in || !out || !valid_dims(rows, cols) || !valid_pitch(pitch_in, cols, esz) || !valid_pitch(pitch_out, cols, 1))
    return NSGB_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int H = (int)rows, W = (int)cols;
  switch (dtype) {
    case NSGB_U8: threshold_kernel<uint8_t><<<rc(rows, cols), 256, 0, s>>>((const uint8_t*)in, pitch_in, out, pitch_out, H, W, thr); break;
    case NSGB_U16: threshold_kernel<uint16_t><<<rc(rows, cols), 256, 0, s>>>((const uint16_t*)in, pitch_in, out, pitch_out, H, W, thr); break;
    case NSGB_I32: threshold_kernel<int32_t><<<rc(rows, cols), 256, 0, s>>>((const int32_t*)in, pitch_in, out, pitch_out, H, W, thr); break;
    case NSGB_F32: threshold_kernel<float><<<rc(rows, cols), 256, 0, s>>>((const float*)in, pitch_in, out, pitch_out, H, W, thr); break;
  }
  return cuda_status(cudaGetLastError());
}

nsgb_status nsgb_invert(int dtype, const void* in, void* out, int64_t rows, int64_t cols, int64_t pitch,
                        nsgb_stream_t stream) {
  const int esz = elem_size(dtype);
  if (!esz) return NSGB_ERR_UNSUPPORTED_DTYPE;
  if (!in || !out || !valid_dims(rows, cols) || !valid_pitch(pitch, cols, esz)) return NSGB_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int H = (int)rows, W = (int)cols;
  switch (dtype) {
    case NSGB_U8: invert_kernel<uint8_t><<<rc(rows, cols), 256, 0, s>>>((const uint8_t*)in, (uint8_t*)out, pitch, H, W); break;
    case NSGB_U16: invert_kernel<uint16_t><<<rc(rows, cols), 256, 0, s>>>((const uint16_t*)in, (uint16_t*)out, pitch, H, W); break;
    case NSGB_I32: invert_kernel<int32_t><<<rc(rows, cols), 256, 0, s>>>((const int32_t*)in, (int32_t*)out, pitch, H, W); break;
    case NSGB_F32: invert_kernel<float><<<rc(rows, cols), 256, 0, s>>>((const float*)in, (float*)out, pitch, H, W); break;
  }
  return cuda_status(cudaGetLastError());
}

nsgb_status nsgb_chain(int dtype, void* marker, const void* mask, int64_t rows, int64_t cols, int64_t pitch,
                       int recon_conn, double thr, int fill_conn, int label_conn, int32_t area_min, int32_t area_max,
                       uint8_t* fill_out, int32_t* labels_out, uint8_t* area_out, int32_t* n_labels, int32_t* n_kept,
                       void* ws, size_t ws_bytes, nsgb_stream_t stream, const nsgb_opts* opts) {
  const int esz = elem_size(dtype);
  if (!esz || dtype == NSGB_F32) return NSGB_ERR_UNSUPPORTED_DTYPE;
  if (!marker || !mask || !valid_dims(rows, cols) || !valid_pitch(pitch, cols, esz) || !valid_conn(recon_conn) ||
      !valid_conn(fill_conn) || !valid_conn(label_conn))
    return NSGB_ERR_BAD_ARG;
  nsgb_status st = check_ws(ws, ws_bytes, NSGB_OP_CHAIN, dtype, rows, cols);
  if (st != NSGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const int H = (int)rows, W = (int)cols;
  const int64_t n = rows * cols;
  Ws w = carve(ws, dtype, rows, cols);
  uint8_t* F = fill_out ? fill_out : w.F;
  // (a) reconstruction by dilation, in place on the marker.
  cudaError_t e = recon_timed(opts, dtype, marker, marker, mask, rows, cols, pitch, recon_conn, false,
                              dtype == NSGB_I32, ws, s);
  // (b)+(c) threshold fused into the binary hole fill: label the R <= thr class, flag the
  // components that touch the border, F = 0 there and 255 elsewhere.
  if (e == cudaSuccess)
    e = cudaMemsetAsync(w.bits, 0, sizeof(unsigned) * (size_t)((n + 31) / 32 + 1), s);
  if (e == cudaSuccess) {
    e = dispatch_int(dtype, [&](auto* tag) -> cudaError_t {
      using T = std::remove_pointer_t<decltype(tag)>;
      ClsNotAbove<T> cls{(const T*)marker, pitch, thr};
      SeedBorder<ClsNotAbove<T>> seed{cls, H, W};
      cudaError_t r = ccl::label(cls, H, W, fill_conn, w.forest(false), s);
      if (r != cudaSuccess) return r;
      ccl::ccl_seed_border<SeedBorder<ClsNotAbove<T>>><<<grid1d(2 * (rows + cols)), 256, 0, s>>>(H, W, w.L, seed,
                                                                                                  w.bits);
      fill_out_kernel<uint8_t><<<rc(rows, cols), 256, 0, s>>>(H, W, w.L, w.bits, F, (int64_t)W, (uint8_t)255);
      return cudaGetLastError();
    });
  }
  // (d)+(e) one labelling of F serves bwlabel (relabelled) and bwareaopen (areas).
  if (e == cudaSuccess) {
    ClsValueU8 cls{F, (int64_t)W};
    e = ccl::label(cls, H, W, label_conn, w.forest(true), s);
  }
  if (e == cudaSuccess) e = ccl::rank_roots(w.L, w.A, n, area_min, area_max, w.R, w.tmp, w.counts, s);
  if (e == cudaSuccess) {
    label_out_kernel<<<rc(rows, cols), 256, 0, s>>>(H, W, w.L, w.R, 1, labels_out, (int64_t)W * 4, w.A, area_min, area_max,
                                               nullptr, 0, area_out, (int64_t)W);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && (n_labels || n_kept)) {
    int32_t c[2] = {0, 0};
    e = cudaMemcpyAsync(c, w.counts, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (n_labels) *n_labels = c[0];
    if (n_kept) *n_kept = c[1];
  }
  return finish(e, ws, s, opts);
}

}  // extern "C"
