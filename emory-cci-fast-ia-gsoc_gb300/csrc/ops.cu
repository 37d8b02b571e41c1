// The operations of the reconstruction / labelling path and their C ABI (include/nsgb.h).
// Each operation is a short sequence of kernels on the caller's stream, using only the
// caller's workspace.  All kernels take an image table (batch.cuh); a single-image call is a
// batch of one whose image is passed by value.  Reference functions are cited at each entry
// point.
#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>
#include <string.h>

#include <cmath>
#include <limits>
#include <type_traits>
#include <algorithm>
#include <vector>

#include "../../include/nsgb.h"
#include "batch.cuh"
#include "bbox.cuh"
#include "bitfill.cuh"
#include "ccl.cuh"
#include "common.cuh"
#include "edt.cuh"
#include "morph.cuh"
#include "recon.cuh"

namespace nsgb {
namespace {

// ------------------------------------------------------------------------------------------
// Pixel access helpers.
template <typename T>
__device__ __forceinline__ T px(const void* base, int64_t pitch, int y, int x) {
  return __ldg((const T*)((const char*)base + (int64_t)y * pitch) + x);
}
template <typename T>
__device__ __forceinline__ T pxcg(const void* base, int64_t pitch, int y, int x) {
  return __ldcg((const T*)((const char*)base + (int64_t)y * pitch) + x);
}
template <typename T>
__device__ __forceinline__ T* pxp(void* base, int64_t pitch, int y, int x) {
  return (T*)((char*)base + (int64_t)y * pitch) + x;
}

// ------------------------------------------------------------------------------------------
// `x > thr` with thr a double, as OpenCV's `Mat > k` compares (HistologicalEntities.cpp:214),
// without double arithmetic on the device: an integer image compares with floor(thr) (x > thr
// for integer x); a float image with thr converted to float (rounded to nearest), since
// OpenCV's compare converts the scalar to the image's depth.  Both are prepared on the host.
template <typename T>
struct GtThr {
  using K = std::conditional_t<std::is_floating_point<T>::value, float, int64_t>;
  K k;
  static GtThr make(double thr) {
    GtThr g;
    if constexpr (std::is_floating_point<T>::value) {
      g.k = (float)thr;
    } else {
      if (thr != thr) g.k = INT64_MAX;  // NaN: nothing is greater
      else if (thr >= 9.0e18) g.k = INT64_MAX;
      else if (thr <= -9.0e18) g.k = INT64_MIN;
      else g.k = (int64_t)floor(thr);
    }
    return g;
  }
  __device__ __forceinline__ bool operator()(T x) const {
    if constexpr (std::is_floating_point<T>::value) return x > k;
    else return (int64_t)x > k;
  }
};

// ------------------------------------------------------------------------------------------
// Classifiers (class 0 = background; equal non-zero classes are joined).  They read the
// image's plane (Img::plane) or aux plane.
struct ClsValueU8 {  // bwlabel: the pixel value
  __device__ uint32_t operator()(const Img& m, int y, int x) const { return px<uint8_t>(m.plane, m.pitch, y, x); }
};
struct ClsNotFlooded {  // a batch's filled image: the pixels the flood from outside did not reach
  const uint32_t* flooded;  // bit plane, rows of bit_words(W) words from Img::b_base
  __device__ uint32_t operator()(const Img& m, int y, int x) const {
    const uint32_t w = __ldg(flooded + m.b_base + (int64_t)y * ((m.W + 31) / 32) + (x >> 5));
    return ((w >> (x & 31)) & 1u) ^ 1u;
  }
};
struct ClsDenseU8 {  // the chain's filled image F in the workspace (dense, at px_base)
  const uint8_t* F;
  __device__ uint32_t operator()(const Img& m, int y, int x) const {
    return __ldg(F + m.px_base + (int64_t)y * m.W + x);
  }
};
template <typename T>
struct ClsNonZero {  // binary reconstruction (mask = aux), bwselect (image = plane)
  bool use_aux;
  __device__ uint32_t operator()(const Img& m, int y, int x) const {
    return px<T>(use_aux ? m.aux : m.plane, m.pitch, y, x) != (T)0 ? 1u : 0u;
  }
};
template <typename T>
struct ClsNotMax {  // binary hole filling: pixels that are not foreground (max<T>)
  __device__ uint32_t operator()(const Img& m, int y, int x) const {
    return px<T>(m.plane, m.pitch, y, x) != std::numeric_limits<T>::max() ? 1u : 0u;
  }
};
template <typename T>
struct ClsAboveOrNot {  // hole filling and labelling at once: 1 where R > thr, 2 elsewhere
  GtThr<T> gt;
  __device__ uint32_t operator()(const Img& m, int y, int x) const {
    return gt(pxcg<T>(m.plane, m.pitch, y, x)) ? 1u : 2u;
  }
};
template <typename T>
struct ClsNotAbove {  // hole filling of (R > thr): the complement class !(R > thr); R = plane
  GtThr<T> gt;
  __device__ uint32_t operator()(const Img& m, int y, int x) const {
    return gt(pxcg<T>(m.plane, m.pitch, y, x)) ? 0u : 1u;
  }
};

// The red-channel valleys of the nucleus-candidate stage, D = rc - R (OpenCV's saturating u8
// Mat subtraction, HistologicalEntities.cpp:199), from the reconstruction R (plane, written by
// an earlier launch) and the image rc it was taken under (aux).
__device__ __forceinline__ uint8_t valley(const Img& m, int y, int x) {
  const int d = (int)px<uint8_t>(m.aux, m.pitch, y, x) - (int)pxcg<uint8_t>(m.plane, m.pitch, y, x);
  return (uint8_t)(d > 0 ? d : 0);
}
struct ClsValleyAboveOrNot {  // hole filling and labelling of (D > g1) at once: 1 where D > g1, 2 elsewhere
  GtThr<uint8_t> gt;
  __device__ uint32_t operator()(const Img& m, int y, int x) const { return gt(valley(m, y, x)) ? 1u : 2u; }
};
struct ClsValleyAbove {  // bwselect's image D > g2
  GtThr<uint8_t> gt;
  __device__ uint32_t operator()(const Img& m, int y, int x) const { return gt(valley(m, y, x)) ? 1u : 0u; }
};

// Seeds (pixels that flag their component's root).
template <class Cls>
struct SeedBorder {
  Cls cls;
  __device__ bool operator()(const Img& m, int y, int x) const { return cls(m, y, x) != 0u; }
};
template <typename T>
struct SeedBoth {  // a != 0 and b != 0, with a = plane or aux as selected
  bool a_is_plane;
  __device__ bool operator()(const Img& m, int y, int x) const {
    const void* a = a_is_plane ? m.plane : m.aux;
    const void* b = a_is_plane ? m.aux : m.plane;
    return pxcg<T>(a, m.pitch, y, x) != (T)0 && px<T>(b, m.pitch, y, x) != (T)0;
  }
};

// bwselect's seeds in the nucleus-candidate stage: D > g2 on a pixel of a filled component
// (forest LF, areas A) whose area lies in [lo, hi) -- bw2 & bw1_t without writing bw1_t.
struct SeedCandidate {
  GtThr<uint8_t> gt;
  const int* LF;
  const int* A;
  int lo, hi;
  const unsigned* outside;  // roots of LF that are not part of the filled image (optional)
  __device__ bool operator()(const Img& m, int y, int x) const {
    if (!gt(valley(m, y, x))) return false;
    const int r = ccl::root_of_ro(LF, (int64_t)m.px_base + (int64_t)y * m.W + x);
    if (r < 0 || (outside && ccl::test_bit(outside, r))) return false;
    const int a = __ldg(A + r);
    return a >= lo && a < hi;
  }
};

// ------------------------------------------------------------------------------------------
// Output kernels (row grids over all images; a pixel's root is L[L[i]]).

// Binary hole filling: 0 where the non-foreground pixel's component touches the border.
// Writes the workspace plane F (dense, if given) and the caller's output (single image:
// `out` / `pitch_out`; batch: Img::fill, dense).
// Stores of four consecutive outputs (one vector store when aligned).
__device__ __forceinline__ void store4_u8(uint8_t* p, int n, const uint8_t (&v)[4]) {
  if (n == 4 && (((uintptr_t)p & 3) == 0)) {
    *(uchar4*)p = make_uchar4(v[0], v[1], v[2], v[3]);
  } else {
    for (int k = 0; k < n; ++k) p[k] = v[k];
  }
}
__device__ __forceinline__ void store4_i32(int32_t* p, int n, const int (&v)[4]) {
  if (n == 4 && (((uintptr_t)p & 15) == 0)) {
    *(int4*)p = make_int4(v[0], v[1], v[2], v[3]);
  } else {
    for (int k = 0; k < n; ++k) p[k] = v[k];
  }
}

template <typename TO>
__global__ void fill_out_kernel(Imgs I, int total_rows, const int* __restrict__ L, const unsigned* __restrict__ bits,
                                uint8_t* F, TO* out, int64_t pitch_out, TO fg) {
  ccl::for_batch_quads(I, total_rows, [&](const Img& m, int y, int x, int n) {
    const int64_t gi = (int64_t)m.px_base + (int64_t)y * m.W + x;
    int r[4];
    ccl::roots4_ro(L, gi, n, r);
    uint8_t f[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
      f[k] = (k > 0 && r[k] == r[k - 1]) ? f[k - 1] : ((r[k] >= 0 && ccl::test_bit(bits, r[k])) ? 0 : (uint8_t)fg);
    if (F) store4_u8(F + gi, n, f);
    TO* o = nullptr;
    if (!I.d) o = out ? pxp<TO>(out, pitch_out, y, x) : nullptr;
    else if (m.fill) o = (TO*)m.fill + (int64_t)y * m.W + x;
    if (!o) return;
    if constexpr (sizeof(TO) == 1) {
      store4_u8((uint8_t*)o, n, f);
    } else {
      for (int k = 0; k < n; ++k) o[k] = f[k] ? fg : (TO)0;
    }
  });
}

// Bit planes for the chain's hole fill (bitfill.cu): open = 1 where the reconstruction is not
// above the threshold (the class the fill works on), flooded = 0.  One lane per 32-pixel word of
// the planes of all images (a flat walk, so narrow images leave no lane idle).  Where every
// lane's word starts on a 16-byte boundary the lanes load their own words with vector loads;
// otherwise (rows of an odd width start anywhere) the warp loads each lane's word in turn, one
// pixel per lane, and forms it with a ballot: every load then reads consecutive bytes, where
// per-lane scalar loads would touch 32 sectors per instruction.
struct BBase { __device__ int operator()(const Img& m) const { return m.b_base; } };

template <typename T>
__global__ void pack_open_kernel(Imgs I, int total_words, GtThr<T> gt, uint32_t* __restrict__ open,
                                 uint32_t* __restrict__ flooded) {
  const int lane = threadIdx.x & 31;
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x + threadIdx.x - lane; base < total_words; base += stride) {
    const int wi = base + lane;
    const T* row = nullptr;
    int n = 0;
    if (wi < total_words) {
      const Img& m = I.d ? I.d[img_of(I, wi, BBase())] : I.one;
      const int nw = bit_words(m.W);
      const int rel = wi - m.b_base;
      const int y = rel / nw, k = rel - y * nw;
      row = (const T*)((const char*)m.plane + (int64_t)y * m.pitch) + 32 * k;
      n = min(32, m.W - 32 * k);
    }
    uint32_t bits = 0;
    if (__all_sync(NSGB_FULL, n == 0 || (n == 32 && ((uintptr_t)row & 15) == 0))) {
      if (n == 32) {
        constexpr int V = 16 / sizeof(T);
#pragma unroll
        for (int q = 0; q < 32 / V; ++q) {
          const uint4 v = __ldg((const uint4*)row + q);
          T e[V];
          memcpy(e, &v, 16);
#pragma unroll
          for (int j = 0; j < V; ++j) bits |= (gt(e[j]) ? 0u : 1u) << (q * V + j);
        }
      }
    } else {
#pragma unroll 4
      for (int src = 0; src < 32; ++src) {
        const T* r = (const T*)__shfl_sync(NSGB_FULL, (unsigned long long)row, src);
        const int ns = __shfl_sync(NSGB_FULL, n, src);
        const uint32_t b = __ballot_sync(NSGB_FULL, lane < ns && !gt(__ldg(r + lane)));
        if (lane == src) bits = b;
      }
    }
    if (wi < total_words) {
      open[wi] = bits;
      flooded[wi] = 0u;
    }
  }
}

// Binary reconstruction output, in place on the marker (= plane).
template <typename T>
__global__ void binrecon_out_kernel(Imgs I, int total_rows, const int* __restrict__ L,
                                    const unsigned* __restrict__ bits) {
  ccl::for_batch_pixels(I, total_rows, [&](const Img& m, int y, int x) {
    T* p = pxp<T>(m.plane, m.pitch, y, x);
    if (*p != (T)0) return;
    const int r = ccl::root_of_ro(L, (int64_t)m.px_base + (int64_t)y * m.W + x);
    if (r >= 0 && ccl::test_bit(bits, r)) *p = std::numeric_limits<T>::max();
  });
}

template <typename T>
__global__ void bwselect_out_kernel(Imgs I, int total_rows, void* out, const int* __restrict__ L,
                                    const unsigned* __restrict__ bits) {
  ccl::for_batch_pixels(I, total_rows, [&](const Img& m, int y, int x) {
    const T v = px<T>(m.plane, m.pitch, y, x);
    const int r = ccl::root_of_ro(L, (int64_t)m.px_base + (int64_t)y * m.W + x);
    *pxp<T>(out, m.pitch, y, x) = (v != (T)0 && r >= 0 && ccl::test_bit(bits, r)) ? v : (T)0;
  });
}

// Nucleus candidates: 255 on a component of (D > g2) that holds a seed, where rbc is 0
// (bwselect(bw2, bw1_t, 8) & (rbc == 0), HistologicalEntities.cpp:268-271).  L2 is the forest
// of D > g2 (root -1 off it), `bits` its seeded roots.
__global__ void candidates_out_kernel(Imgs I, int total_rows, const int* __restrict__ L2,
                                      const unsigned* __restrict__ bits, const uint8_t* __restrict__ rbc,
                                      uint8_t* out) {
  ccl::for_batch_quads(I, total_rows, [&](const Img& m, int y, int x, int n) {
    int r[4];
    ccl::roots4_ro(L2, (int64_t)m.px_base + (int64_t)y * m.W + x, n, r);
    const uint8_t* q = rbc + (int64_t)y * m.pitch + x;
    bool sel[4];
    uint8_t o[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      sel[k] = (k > 0 && r[k] == r[k - 1]) ? sel[k - 1] : (r[k] >= 0 && ccl::test_bit(bits, r[k]));
      o[k] = (k < n && sel[k] && __ldg(q + k) == 0) ? 255 : 0;
    }
    store4_u8(pxp<uint8_t>(out, m.pitch, y, x), n, o);
  });
}

// Labels out: relabel ? (bg 0, root's rank + 1) : the root's raster index in its image / -1.
// Optional area-filter outputs from the same pass.  rank / A are read-only here: L1-cached
// loads, because a giant component's root is read by every one of its pixels.  Single image:
// explicit output pointers / pitches; batch: Img::labels / Img::area (dense).
// RELABEL: raster rank labels (else root indices); AREA: area-filter outputs (A non-null).
// FILLED: the labelled pixels are the filled image, written as 255 (0 elsewhere) to `filled`
// (single image, optional) or Img::fill (batch); with `outside` (the forest of
// ccl::label_filled) the roots it marks are background too.
template <bool RELABEL, bool AREA, bool FILLED = false>
__global__ void label_out_kernel(Imgs I, int total_rows, const int* __restrict__ L, const int* __restrict__ rank,
                                 int32_t* labels, int64_t pitch_labels, const int* __restrict__ A, int lo,
                                 int hi, int32_t* kept_labels, int64_t pitch_kept, uint8_t* flat, int64_t pitch_flat,
                                 const unsigned* __restrict__ outside = nullptr, uint8_t* filled = nullptr,
                                 int64_t pitch_filled = 0) {
  pdl_wait();
  pdl_release();
  ccl::for_batch_quads(I, total_rows, [&](const Img& m, int y, int x, int n) {
    int r[4], lab[4], kl[4];
    uint8_t fl[4];
    ccl::roots4_ro(L, (int64_t)m.px_base + (int64_t)y * m.W + x, n, r);
    if (FILLED) {
      bool out[4];
      uint8_t fi[4];
#pragma unroll
      for (int k = 0; k < 4; ++k)
        out[k] = (k > 0 && r[k] == r[k - 1]) ? out[k - 1] : (r[k] >= 0 && outside && ccl::test_bit(outside, r[k]));
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        if (out[k]) r[k] = -1;
        fi[k] = r[k] >= 0 ? 255 : 0;
      }
      if (!I.d) {
        if (filled) store4_u8(pxp<uint8_t>(filled, pitch_filled, y, x), n, fi);
      } else if (m.fill) {
        store4_u8(m.fill + (int64_t)y * m.W + x, n, fi);
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const bool same = k > 0 && r[k] == r[k - 1];
      lab[k] = same ? lab[k - 1]
                    : (RELABEL ? (r[k] < 0 ? 0 : __ldg(&rank[r[k]]) + 1) : (r[k] < 0 ? -1 : r[k] - m.px_base));
      bool keep = false;
      if (AREA) {
        if (same) {
          keep = fl[k - 1] != 0;
        } else {
          const int a = r[k] >= 0 ? __ldg(&A[r[k]]) : 0;
          keep = r[k] >= 0 && a >= lo && a < hi;
        }
      }
      fl[k] = keep ? 255 : 0;
      kl[k] = keep ? r[k] - m.px_base : -1;
    }
    if (!I.d) {
      if (labels) store4_i32(pxp<int32_t>(labels, pitch_labels, y, x), n, lab);
      if (AREA && kept_labels) store4_i32(pxp<int32_t>(kept_labels, pitch_kept, y, x), n, kl);
      if (AREA && flat) store4_u8(pxp<uint8_t>(flat, pitch_flat, y, x), n, fl);
    } else {
      const int64_t li = (int64_t)y * m.W + x;
      if (m.labels) store4_i32(m.labels + li, n, lab);
      if (AREA && m.area) store4_u8(m.area + li, n, fl);
    }
  });
}

// Area of arbitrary int32 labels in [-1, n): dense histogram (background -1 skipped).
__global__ void label_hist_kernel(Imgs I, int total_rows, int* __restrict__ A, int* status) {
  ccl::for_batch_pixels(I, total_rows, [&](const Img& m, int y, int x) {
    const int64_t n = (int64_t)m.H * m.W;
    const int l = px<int32_t>(m.plane, m.pitch, y, x);
    if (l == -1) return;
    if (l < -1 || (int64_t)l >= n) {
      set_status(status, NSGB_ERR_BAD_ARG);
      return;
    }
    atomicAdd(&A[l], 1);
  });
}

__global__ void labeled_area_out_kernel(Imgs I, int total_rows, const int* __restrict__ A, int lo, int hi,
                                        int32_t* kept_labels, int64_t pitch_kept, uint8_t* flat, int64_t pitch_flat) {
  ccl::for_batch_pixels(I, total_rows, [&](const Img& m, int y, int x) {
    const int64_t n = (int64_t)m.H * m.W;
    const int l = px<int32_t>(m.plane, m.pitch, y, x);
    const int a = (l >= 0 && (int64_t)l < n) ? __ldg(&A[l]) : 0;
    const bool keep = l >= 0 && (int64_t)l < n && a >= lo && a < hi;
    if (kept_labels) *pxp<int32_t>(kept_labels, pitch_kept, y, x) = keep ? l : -1;
    if (flat) *pxp<uint8_t>(flat, pitch_flat, y, x) = keep ? 255 : 0;
  });
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
// Elementwise kernels on one image (row / column grids).
#define NSGB_FOR_PIXELS                                   \
  const int x = blockIdx.x * blockDim.x + threadIdx.x;    \
  if (x >= W) return;                                     \
  for (int y = blockIdx.y; y < H; y += gridDim.y)

template <typename T>
struct alignas(4 * sizeof(T)) Vec4 {
  T v[4];
};

// Four pixels per thread (x grid over W / 4); VEC: rows and bases allow one vector load and
// one 32-bit store per thread.
#define NSGB_FOR_QUADS                                        \
  const int x = 4 * (blockIdx.x * blockDim.x + threadIdx.x);  \
  if (x >= W) return;                                         \
  for (int y = blockIdx.y; y < H; y += gridDim.y)

template <typename T, bool VEC>
__global__ void threshold_kernel(const T* in, int64_t pitch_in, uint8_t* out, int64_t pitch_out, int H, int W,
                                 GtThr<T> gt) {
  NSGB_FOR_QUADS {
    const T* r = (const T*)((const char*)in + (int64_t)y * pitch_in) + x;
    uint8_t* o = out + (int64_t)y * pitch_out + x;
    if (VEC && x + 4 <= W) {
      const Vec4<T> v = *(const Vec4<T>*)r;
      uchar4 q;
      q.x = gt(v.v[0]) ? 255 : 0;
      q.y = gt(v.v[1]) ? 255 : 0;
      q.z = gt(v.v[2]) ? 255 : 0;
      q.w = gt(v.v[3]) ? 255 : 0;
      *(uchar4*)o = q;
    } else {
      for (int k = 0; k < 4 && x + k < W; ++k) o[k] = gt(r[k]) ? 255 : 0;
    }
  }
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
    return (T)0 - v;  // OpenCV's `-img` is `0 - img`: +0.0 for both zeros
  }
}

// -0.0 -> +0.0 over a float plane.  The reference's float imhmin and imfillHoles end with
// PixelOperations::invert (`0 - x`, never -0.0); the order-reversed reconstruction here flips
// the sign bit instead, so their outputs pass through this once.
__global__ void canon_zero_f32_kernel(float* out, int64_t pitch, int H, int W) {
  NSGB_FOR_QUADS {
    unsigned* o = (unsigned*)((char*)out + (int64_t)y * pitch) + x;
    for (int k = 0; k < 4 && x + k < W; ++k)
      if (o[k] == 0x80000000u) o[k] = 0u;
  }
}

template <typename T, bool VEC>
__global__ void invert_kernel(const T* in, T* out, int64_t pitch, int H, int W) {
  NSGB_FOR_QUADS {
    const T* r = (const T*)((const char*)in + (int64_t)y * pitch) + x;
    T* o = (T*)((char*)out + (int64_t)y * pitch) + x;
    if (VEC && x + 4 <= W) {
      Vec4<T> v = *(const Vec4<T>*)r;
#pragma unroll
      for (int k = 0; k < 4; ++k) v.v[k] = invert_value(v.v[k]);
      *(Vec4<T>*)o = v;
    } else {
      for (int k = 0; k < 4 && x + k < W; ++k) o[k] = invert_value(r[k]);
    }
  }
}

inline dim3 quad_grid(int64_t rows, int64_t cols) { return ccl::quadrow_grid((int)rows, (int)cols); }

// Hole-filling marker: the image on the border, max<T> inside.
template <typename T>
__global__ void fill_marker_kernel(const T* image, T* out, int64_t pitch, int H, int W) {
  NSGB_FOR_PIXELS {
    const bool border = y == 0 || y == H - 1 || x == 0 || x == W - 1;
    *pxp<T>(out, pitch, y, x) = border ? px<T>(image, pitch, y, x) : std::numeric_limits<T>::max();
  }
}

// h-minima marker: image + h, saturating for integers.
template <typename T>
__global__ void hmin_marker_kernel(const T* image, T* out, int64_t pitch, int H, int W, double h) {
  NSGB_FOR_PIXELS {
    const T v = px<T>(image, pitch, y, x);
    T r;
    if constexpr (std::numeric_limits<T>::is_integer) {
      const int64_t s = (int64_t)v + (int64_t)h;
      r = (T)(s > (int64_t)std::numeric_limits<T>::max() ? (int64_t)std::numeric_limits<T>::max() : s);
    } else {
      r = v + (T)h;
    }
    *pxp<T>(out, pitch, y, x) = r;
  }
}

template <typename T>
__global__ void fill_const_kernel(T* out, int64_t pitch, int H, int W, T v) {
  NSGB_FOR_PIXELS { *pxp<T>(out, pitch, y, x) = v; }
}

// ------------------------------------------------------------------------------------------
// Plans and workspace.

struct Plan {
  Imgs I;
  BatchTotals t;
};

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Fills the labelling / rank / row fields of `m` and advances the running totals.
void add_image(Img& m, BatchTotals& t) {
  m.c_tiles_x = (m.W + ccl::kTile - 1) / ccl::kTile;
  const int c_tiles_y = (m.H + ccl::kTile - 1) / ccl::kTile;
  m.r_tile_base = t.r_tiles;
  m.r_stile_base = t.r_stiles;
  m.r_even_base = t.r_even;
  for (int c = 0; c < 3; ++c) m.r_col_base[c] = t.r_col[c];
  m.c_tile_base = t.c_tiles;
  m.px_base = (int)t.px;
  m.blk_base = t.blocks;
  m.row_base = t.rows;
  m.b_base = (int)t.b_words;
  m.f_tile_base = t.f_tiles;
  const int64_t npx = (int64_t)m.H * m.W;
  t.b_words += (int64_t)m.H * bit_words(m.W);
  t.f_tiles += flood_tiles_x(m.W) * flood_tiles_y(m.H);
  t.r_tiles += m.r_tiles_x * m.r_tiles_y;
  if (m.r_tw > 0) t.r_stiles += ((m.H + 47) / 32) * ((m.W + m.r_tw / 2 + m.r_tw - 1) / m.r_tw);
  t.r_even += even_tiles(m.r_tiles_x, m.r_tiles_y);
  for (int c = 0; c < 3; ++c) t.r_col[c] += colour_tiles(m.r_tiles_x, m.r_tiles_y, c);
  t.c_tiles += m.c_tiles_x * c_tiles_y;
  t.px += npx;
  t.blocks += (int)((npx + ccl::kBlockPx - 1) / ccl::kBlockPx);
  t.rows += m.H;
  if (m.W > t.max_w) t.max_w = m.W;
  if (2 * (m.H + m.W) > t.perimeter_max) t.perimeter_max = 2 * (m.H + m.W);
  t.n += 1;
}

Plan single_plan(int dtype, void* plane, const void* aux, int64_t H, int64_t W, int64_t pitch) {
  Plan P = {};
  P.I.n = 1;
  P.I.d = nullptr;
  P.I.one = recon_image(dtype, plane, aux, H, W, pitch);
  add_image(P.I.one, P.t);
  return P;
}

struct WsSizes {
  size_t recon, L, A, R, roots, bits, tmp, wpre, F, table, maps, total;
};

WsSizes ws_sizes(const BatchTotals& t) {
  WsSizes z;
  z.recon = align256(recon_workspace_bytes_tiles(t.r_tiles > 0 ? t.r_tiles : 1));
  z.L = align256(sizeof(int) * (size_t)t.px);
  z.A = z.L;
  z.R = z.L;
  z.roots = z.L;
  z.bits = align256(sizeof(unsigned) * (size_t)(t.px / 32 + 2));
  z.tmp = align256(sizeof(int) * (size_t)(2 * (int64_t)t.blocks + 2 * (int64_t)t.n + 8));
  z.wpre = align256(sizeof(int) * 32 * (size_t)t.blocks);
  z.F = align256((size_t)t.px);
  z.table = t.n > 1 ? align256(sizeof(Img) * (size_t)t.n) : 0;
  z.maps = t.n > 1 ? align256(sizeof(int) * ((size_t)t.r_tiles + (size_t)t.c_tiles)) : 0;
  z.total = z.recon + z.L + z.A + z.R + z.roots + z.bits + z.tmp + z.wpre + z.F + z.table + z.maps;
  return z;
}

struct Ws {
  int* status;  // == start of the recon region
  void* recon;
  int* L;
  int* A;
  int* R;        // root ranks (at roots)
  int* roots;    // list of local roots
  unsigned* bits;
  int* tmp;      // 2 ints per rank block
  int* counts;   // 2 per image
  int* nroots;   // [1]
  int* wpre;     // 32 per rank block
  uint8_t* F;
  Img* table;
  int* r_img;  // batches: image of every reconstruction tile
  int* c_img;  // batches: image of every labelling tile
  size_t bits_bytes;
  ccl::Forest forest(bool areas) const { return ccl::Forest{L, areas ? A : nullptr, roots, nroots}; }
};

Ws carve(void* ws, const BatchTotals& t) {
  const WsSizes z = ws_sizes(t);
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
  w.roots = (int*)p;
  p += z.roots;
  w.bits = (unsigned*)p;
  w.bits_bytes = sizeof(unsigned) * (size_t)(t.px / 32 + 2);
  p += z.bits;
  w.tmp = (int*)p;
  w.counts = w.tmp + 2 * (int64_t)t.blocks;
  w.nroots = w.counts + 2 * (int64_t)t.n;
  p += z.tmp;
  w.wpre = (int*)p;
  p += z.wpre;
  w.F = (uint8_t*)p;
  p += z.F;
  w.table = t.n > 1 ? (Img*)p : nullptr;
  p += z.table;
  w.r_img = t.n > 1 ? (int*)p : nullptr;
  w.c_img = t.n > 1 ? w.r_img + t.r_tiles : nullptr;
  return w;
}

inline int grid1d(int64_t n) { return ccl::flat_grid(n); }
inline dim3 rc(int64_t rows, int64_t cols) { return ccl::rowcol_grid((int)rows, (int)cols); }
inline dim3 rcb(const BatchTotals& t) { return ccl::rowcol_grid(t.rows, t.max_w); }
inline dim3 qr(int64_t rows, int64_t cols) { return ccl::quadrow_grid((int)rows, (int)cols); }
inline dim3 qrb(const BatchTotals& t) { return ccl::quadrow_grid(t.rows, t.max_w); }

// Records the caller's optional timing event around the reconstruction kernel.  While the
// stream is being captured into a CUDA graph the record becomes an external event-record node,
// so the event is recorded at every replay (a plain record in a capture only orders streams).
cudaError_t record(const nsgb_opts* o, bool begin, cudaStream_t s) {
  if (!o) return cudaSuccess;
  void* ev = begin ? o->recon_event_begin : o->recon_event_end;
  if (!ev) return cudaSuccess;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &cap);
  if (e != cudaSuccess) return e;
  return cap == cudaStreamCaptureStatusActive ? cudaEventRecordWithFlags((cudaEvent_t)ev, s, cudaEventRecordExternal)
                                              : cudaEventRecord((cudaEvent_t)ev, s);
}

// Reconstruction of the whole plan bracketed by the optional timing events.
cudaError_t recon_timed(const nsgb_opts* o, int dtype, const Plan& P, int conn, bool erode, bool ring, void* ws,
                        cudaStream_t s, int resweeps = 0) {
  cudaError_t e = record(o, true, s);
  if (e != cudaSuccess) return e;
  e = recon_launch_batch(dtype, P.I, P.t.r_tiles, conn, erode, ring, ws, s, o ? o->max_visits_per_tile : 0,
                         o ? o->max_visit_iters : 0, resweeps, o ? o->queue_poll_limit : 0, o ? o->recon_passes : 0,
                         P.t.r_stiles, o ? o->recon_order : 0, (long long)P.t.px, o ? o->recon_ctas_per_sm : 0);
  if (e != cudaSuccess) return e;
  return record(o, false, s);
}

template <typename F>
void dispatch_all(int dtype, F&& f) {
  switch (dtype) {
    case NSGB_U8: f((uint8_t*)nullptr); break;
    case NSGB_U16: f((uint16_t*)nullptr); break;
    case NSGB_I32: f((int32_t*)nullptr); break;
    case NSGB_F32: f((float*)nullptr); break;
    default: break;
  }
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

// The single-tile / batched chain on a prepared plan: (a) reconstruction in place,
// (b)+(c) threshold fused into the binary hole fill, (d)+(e) one labelling of the filled image
// for both the raster relabel and the areas.  Counts land in w.counts (2 per image).
cudaError_t chain_impl(int dtype, const Plan& P, const Ws& w, int recon_conn, double thr, int fill_conn,
                       int label_conn, int area_min, int area_max, uint8_t* fill_out, int32_t* labels_out,
                       uint8_t* area_out, const nsgb_opts* opts, cudaStream_t s) {
  const BatchTotals& t = P.t;
  cudaError_t e = recon_timed(opts, dtype, P, recon_conn, false, dtype == NSGB_I32, w.recon, s);
  const bool dual = (fill_conn == 4 && label_conn == 8) || (fill_conn == 8 && label_conn == 4);
  if (e == cudaSuccess && dual && !(P.I.d && t.n > 1)) {
    // (b)-(e) on one image with one labelling.  With dual connectivities (the not-above class
    // flooded 4-connected, the filled image labelled 8-connected, or the other way round) the
    // components of R > thr and of its complement form a tree by enclosure, and a component of
    // the filled image is a top-level component of R > thr with everything it encloses: both
    // classes are labelled in one forest, each component joined to its parent (the component
    // above its first pixel) unless that is a complement component touching the border.  The
    // bitmap of those outside components lives in F, which this path does not otherwise use.
    unsigned* outside = (unsigned*)w.F;
    const int code = label_conn == 8 ? ccl::kConnFg8Bg4 : ccl::kConnFg4Bg8;
    e = dispatch_int(dtype, [&](auto* tag) -> cudaError_t {
      using T = std::remove_pointer_t<decltype(tag)>;
      // the ranking's bitmap and counts are cleared by the labelling's first launch
      const ccl::ZeroSpans rank_zero{{nullptr, nullptr, w.bits, (unsigned*)w.counts},
                                     {0, 0, (int)(w.bits_bytes / sizeof(unsigned)), 2 * t.n}};
      return ccl::label_filled(ClsAboveOrNot<T>{GtThr<T>::make(thr)}, P.I, t, code, w.forest(true), outside,
                               w.bits_bytes, s, true, rank_zero);
    });
    // From the labelling on, every launch is a programmatic dependent of the one before it.
    if (e == cudaSuccess)
      e = ccl::rank_roots(P.I, t, w.forest(true), area_min, area_max, w.R, w.bits, w.bits_bytes, w.tmp, w.wpre,
                          w.counts, s, outside, true, true);
    if (e == cudaSuccess) {
      const int64_t W1 = P.I.d ? 0 : P.I.one.W;
      e = launch_dependent(label_out_kernel<true, true, true>, qrb(t), dim3(256), s, P.I, t.rows, (const int*)w.L,
                           (const int*)w.R, labels_out, W1 * 4, (const int*)w.A, area_min, area_max,
                           (int32_t*)nullptr, (int64_t)0, area_out, W1, (const unsigned*)outside, fill_out, W1);
    }
    return e;
  }
  if (e == cudaSuccess && P.I.d && t.n > 1) {
    // (b)-(e) on a batch: the pixels not above the threshold as a bit plane, flooded from
    // outside each image (bitfill.cu); the filled image is what the flood does not reach, and
    // it is labelled straight from the flooded plane, the label output writing it out.  The
    // planes L and R hold the open and flooded bit planes until the labelling (L) and the rank
    // (R) overwrite them.  A flood is a chain of dependent tile visits from the border inwards;
    // many images flood at once, so the batch hides that latency, and it then costs a fraction
    // of the labelling (pack and flood touch 1 bit per pixel where a labelling writes an int).
    uint32_t* open = (uint32_t*)w.L;
    uint32_t* flooded = (uint32_t*)w.R;
    e = dispatch_int(dtype, [&](auto* tag) -> cudaError_t {
      using T = std::remove_pointer_t<decltype(tag)>;
      pack_open_kernel<T><<<ccl::flat_grid(t.b_words), 256, 0, s>>>(P.I, (int)t.b_words, GtThr<T>::make(thr), open,
                                                                   flooded);
      return cudaGetLastError();
    });
    if (e == cudaSuccess)
      e = flood_launch(P.I, t.f_tiles, open, flooded, fill_conn, w.recon, s, opts ? opts->queue_poll_limit : 0);
    if (e == cudaSuccess) e = ccl::label(ClsNotFlooded{flooded}, P.I, t, label_conn, w.forest(true), s);
    if (e == cudaSuccess)
      e = ccl::rank_roots(P.I, t, w.forest(true), area_min, area_max, w.R, w.bits, w.bits_bytes, w.tmp, w.wpre,
                          w.counts, s);
    if (e == cudaSuccess) {
      label_out_kernel<true, true, true><<<qrb(t), 256, 0, s>>>(P.I, t.rows, w.L, w.R, labels_out, 0, w.A, area_min,
                                                                area_max, nullptr, 0, area_out, 0, nullptr, fill_out,
                                                                0);
      e = cudaGetLastError();
    }
    return e;
  }
  if (e == cudaSuccess) {
    // (b)+(c) on one image: the threshold fused into the labelling's classifier, components
    // touching the border seeded.  (One image's flood is a chain of dependent tile visits that
    // the labelling does not have: 0.58 against 0.49 ms for the 4096^2 chain.)
    e = cudaMemsetAsync(w.bits, 0, w.bits_bytes, s);
    if (e == cudaSuccess) {
      e = dispatch_int(dtype, [&](auto* tag) -> cudaError_t {
        using T = std::remove_pointer_t<decltype(tag)>;
        ClsNotAbove<T> cls{GtThr<T>::make(thr)};
        cudaError_t r = ccl::label(cls, P.I, t, fill_conn, w.forest(false), s);
        if (r != cudaSuccess) return r;
        const int gx = grid1d(t.perimeter_max) > 64 ? 64 : grid1d(t.perimeter_max);
        ccl::ccl_seed_border<SeedBorder<ClsNotAbove<T>>><<<dim3(gx, t.n), 256, 0, s>>>(
            P.I, w.L, SeedBorder<ClsNotAbove<T>>{cls}, w.bits);
        fill_out_kernel<uint8_t><<<qrb(t), 256, 0, s>>>(P.I, t.rows, w.L, w.bits, w.F, fill_out,
                                                        P.I.d ? 0 : (int64_t)P.I.one.W, (uint8_t)255);
        return cudaGetLastError();
      });
    }
  }
  if (e == cudaSuccess) e = ccl::label(ClsDenseU8{w.F}, P.I, t, label_conn, w.forest(true), s);
  if (e == cudaSuccess) e = ccl::rank_roots(P.I, t, w.forest(true), area_min, area_max, w.R, w.bits, w.bits_bytes, w.tmp, w.wpre, w.counts, s);
  if (e == cudaSuccess) {
    const int64_t W1 = P.I.d ? 0 : P.I.one.W;
    label_out_kernel<true, true><<<qrb(t), 256, 0, s>>>(P.I, t.rows, w.L, w.R, labels_out, W1 * 4, w.A, area_min,
                                                        area_max, nullptr, 0, area_out, W1);
    e = cudaGetLastError();
  }
  return e;
}

// The nucleus-candidate stage on one image (plane = rc_open, reconstructed in place; aux = rc):
// (a) R = recon(rc_open, rc, 8); (b) bw1 = imfillHoles(D > g1, 4) and (c) bw1's 8-connected
// components with their areas, from one labelling of D > g1 and its complement (the threshold
// in the classifier), the kept ones counted (w.counts[1]); (d) bwselect(D > g2, bw1_t, 8): D > g2 labelled into a second
// forest (the rank array R, unused here), its roots seeded straight from bw1's forest and
// areas, so bw1_t is never written; (e) the output with rbc == 0 folded in.
cudaError_t candidates_impl(const Plan& P, const Ws& w, double g1, double g2, int lo, int hi, const uint8_t* rbc,
                            uint8_t* out, const nsgb_opts* opts, cudaStream_t s) {
  const BatchTotals& t = P.t;
  const GtThr<uint8_t> gt1 = GtThr<uint8_t>::make(g1);
  const GtThr<uint8_t> gt2 = GtThr<uint8_t>::make(g2);
  cudaError_t e = recon_timed(opts, NSGB_U8, P, 8, false, false, w.recon, s);
  // (b)+(c) as one labelling of D > g1 (8-connected) and its complement (4-connected), each
  // component joined to the one enclosing it (ccl::label_filled); the complement components
  // that touch the border are marked in F (used as a bitmap here) and are not part of bw1.
  unsigned* outside = (unsigned*)w.F;
  if (e == cudaSuccess)
    e = ccl::label_filled(ClsValleyAboveOrNot{gt1}, P.I, t, ccl::kConnFg8Bg4, w.forest(true), outside,
                          w.bits_bytes, s, true);
  if (e == cudaSuccess) e = ccl::count_roots(P.I, t, w.forest(true), lo, hi, w.bits, w.counts, s, outside);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.bits, 0, w.bits_bytes, s);
  const ccl::Forest sel{w.R, nullptr, w.roots, w.nroots};
  if (e == cudaSuccess) e = ccl::label(ClsValleyAbove{gt2}, P.I, t, 8, sel, s);
  if (e == cudaSuccess) {
    ccl::ccl_seed_quads<SeedCandidate><<<qrb(t), 256, 0, s>>>(P.I, t.rows, w.R, SeedCandidate{gt2, w.L, w.A, lo, hi, outside},
                                                               w.bits);
    candidates_out_kernel<<<qrb(t), 256, 0, s>>>(P.I, t.rows, w.R, w.bits, rbc, out);
    e = cudaGetLastError();
  }
  return e;
}

}  // namespace
}  // namespace nsgb

// ============================================================================================
// C ABI
using namespace nsgb;

namespace {

bool want_sync(const nsgb_opts* o) { return o == nullptr || o->sync != 0; }

nsgb_status cuda_status(cudaError_t e) { return e == cudaSuccess ? NSGB_OK : NSGB_ERR_CUDA; }

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

nsgb_status check_ws_bytes(void* ws, size_t ws_bytes, size_t need) {
  if (!ws) return NSGB_ERR_WORKSPACE;
  if (ws_bytes < need) return NSGB_ERR_WORKSPACE;
  if ((uintptr_t)ws % 256 != 0) return NSGB_ERR_WORKSPACE;
  return NSGB_OK;
}

nsgb_status check_ws(void* ws, size_t ws_bytes, int op, int dtype, int64_t rows, int64_t cols) {
  return check_ws_bytes(ws, ws_bytes, nsgb_workspace_size(op, dtype, rows, cols));
}

}  // namespace

extern "C" {

size_t nsgb_workspace_size(int op, int dtype, int64_t rows, int64_t cols) {
  if (rows <= 0 || cols <= 0 || op < 0 || op > NSGB_OP_DISTANCE) return 0;
  if (op == NSGB_OP_BWLABEL || op == NSGB_OP_BWAREAOPEN || op == NSGB_OP_NUCLEUS_CANDIDATES ||
      op == NSGB_OP_MORPH_OPEN || op == NSGB_OP_DISTANCE)
    dtype = NSGB_U8;
  if (dtype < 0 || dtype > 3) return 0;
  if (op == NSGB_OP_IMRECONSTRUCT || op == NSGB_OP_HMIN) return align256(recon_workspace_bytes(dtype, rows, cols));
  if (op == NSGB_OP_BOUNDING_BOX) return align256(bbox_workspace_bytes(rows * cols));
  if (op == NSGB_OP_MORPH_OPEN) return align256(morph_open_workspace_bytes(rows, cols));
  if (op == NSGB_OP_DISTANCE) return align256(edt_workspace_bytes(rows, cols));
  const Plan P = single_plan(dtype, nullptr, nullptr, rows, cols, cols * elem_size(dtype));
  return ws_sizes(P.t).total;
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
  const Plan P = single_plan(dtype, marker, mask, rows, cols, pitch);
  cudaError_t e = recon_timed(opts, dtype, P, conn, erode != 0, ring, ws, s);
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
  const Plan P = single_plan(dtype, marker, mask, rows, cols, pitch);
  Ws w = carve(ws, P.t);
  cudaError_t e = cudaMemsetAsync(w.status, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.bits, 0, w.bits_bytes, s);
  if (e == cudaSuccess) {
    e = dispatch_int(dtype, [&](auto* tag) -> cudaError_t {
      using T = std::remove_pointer_t<decltype(tag)>;
      ClsNonZero<T> cls{true};
      cudaError_t r = ccl::label(cls, P.I, P.t, conn, w.forest(false), s);
      if (r != cudaSuccess) return r;
      ccl::ccl_seed_pixels<SeedBoth<T>><<<rc(rows, cols), 256, 0, s>>>(P.I, P.t.rows, w.L, SeedBoth<T>{true}, w.bits);
      binrecon_out_kernel<T><<<rc(rows, cols), 256, 0, s>>>(P.I, P.t.rows, w.L, w.bits);
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
  const Plan P = single_plan(dtype, (void*)image, nullptr, rows, cols, pitch);
  Ws w = carve(ws, P.t);
  cudaError_t e = cudaMemsetAsync(w.status, 0, sizeof(int), s);
  if (e != cudaSuccess) return NSGB_ERR_CUDA;
  if (binary) {
    if (dtype == NSGB_I32) {
      // min<int> is non-zero, so the reference's binary reconstruction has no background to
      // grow into and every pixel comes back as invert(min<int>) = INT_MAX.
      fill_const_kernel<int32_t><<<rc(rows, cols), 256, 0, s>>>((int32_t*)out, pitch, H, W, INT_MAX);
      return finish(cudaGetLastError(), ws, s, opts);
    }
    e = cudaMemsetAsync(w.bits, 0, w.bits_bytes, s);
    if (e == cudaSuccess) {
      e = dispatch_int(dtype, [&](auto* tag) -> cudaError_t {
        using T = std::remove_pointer_t<decltype(tag)>;
        ClsNotMax<T> cls;
        cudaError_t r = ccl::label(cls, P.I, P.t, conn, w.forest(false), s);
        if (r != cudaSuccess) return r;
        ccl::ccl_seed_border<SeedBorder<ClsNotMax<T>>><<<dim3(grid1d(2 * (rows + cols)), 1), 256, 0, s>>>(
            P.I, w.L, SeedBorder<ClsNotMax<T>>{cls}, w.bits);
        fill_out_kernel<T><<<qr(rows, cols), 256, 0, s>>>(P.I, P.t.rows, w.L, w.bits, nullptr, (T*)out, pitch,
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
  const Plan R = single_plan(dtype, out, image, rows, cols, pitch);
  // front from the border: re-sweep a tile up to four times when a neighbour changed while it
  // ran (16384^2 fills, 8-connected: 11.76 -> 11.53 ms u8, 18.48 -> 17.93 ms i32 against two)
  e = recon_timed(opts, dtype, R, conn, true, false, ws, s, 4);
  if (e == cudaSuccess && dtype == NSGB_F32) {
    canon_zero_f32_kernel<<<quad_grid(rows, cols), 256, 0, s>>>((float*)out, pitch, H, W);
    e = cudaGetLastError();
  }
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
  const Plan P = single_plan(dtype, out, image, rows, cols, pitch);
  cudaError_t e = recon_timed(opts, dtype, P, conn, true, true, ws, s);
  if (e == cudaSuccess && dtype == NSGB_F32) {
    canon_zero_f32_kernel<<<quad_grid(rows, cols), 256, 0, s>>>((float*)out, pitch, H, W);
    e = cudaGetLastError();
  }
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
  const Plan P = single_plan(dtype, (void*)image, seeds, rows, cols, pitch);
  Ws w = carve(ws, P.t);
  cudaError_t e = cudaMemsetAsync(w.status, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.bits, 0, w.bits_bytes, s);
  if (e == cudaSuccess) {
    e = dispatch_int(dtype, [&](auto* tag) -> cudaError_t {
      using T = std::remove_pointer_t<decltype(tag)>;
      ClsNonZero<T> cls{false};
      cudaError_t r = ccl::label(cls, P.I, P.t, conn, w.forest(false), s);
      if (r != cudaSuccess) return r;
      // seeds (aux) != 0 and image (plane) != 0
      ccl::ccl_seed_pixels<SeedBoth<T>><<<rc(rows, cols), 256, 0, s>>>(P.I, P.t.rows, w.L, SeedBoth<T>{false},
                                                                        w.bits);
      bwselect_out_kernel<T><<<rc(rows, cols), 256, 0, s>>>(P.I, P.t.rows, out, w.L, w.bits);
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
  const Plan P = single_plan(NSGB_U8, (void*)bin, nullptr, rows, cols, pitch_in);
  Ws w = carve(ws, P.t);
  cudaError_t e = cudaMemsetAsync(w.status, 0, sizeof(int), s);
  if (e != cudaSuccess) return NSGB_ERR_CUDA;
  e = ccl::label(ClsValueU8{}, P.I, P.t, conn, w.forest(false), s);
  if (e == cudaSuccess) e = ccl::rank_roots(P.I, P.t, w.forest(false), 0, 0, w.R, w.bits, w.bits_bytes, w.tmp, w.wpre, w.counts, s);
  if (e == cudaSuccess) {
    if (relabel)
      label_out_kernel<true, false><<<qr(rows, cols), 256, 0, s>>>(P.I, P.t.rows, w.L, w.R, labels, pitch_labels,
                                                                   nullptr, 0, 0, nullptr, 0, nullptr, 0);
    else
      label_out_kernel<false, false><<<qr(rows, cols), 256, 0, s>>>(P.I, P.t.rows, w.L, w.R, labels, pitch_labels,
                                                                    nullptr, 0, 0, nullptr, 0, nullptr, 0);
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
  const int64_t n = rows * cols;
  const Plan P = single_plan(NSGB_U8, (void*)in, nullptr, rows, cols, pitch_in);
  Ws w = carve(ws, P.t);
  cudaError_t e = cudaMemsetAsync(w.status, 0, sizeof(int), s);
  if (e != cudaSuccess) return NSGB_ERR_CUDA;
  if (!labeled) {
    e = ccl::label(ClsValueU8{}, P.I, P.t, conn, w.forest(true), s);
    if (e == cudaSuccess) e = ccl::rank_roots(P.I, P.t, w.forest(true), min_size, max_size, w.R, w.bits, w.bits_bytes, w.tmp, w.wpre, w.counts, s);
    if (e == cudaSuccess) {
      label_out_kernel<false, true><<<qr(rows, cols), 256, 0, s>>>(P.I, P.t.rows, w.L, w.R, nullptr, 0, w.A, min_size,
                                                                   max_size, labels_out, pitch_labels, flat_out,
                                                                   pitch_flat);
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
    label_hist_kernel<<<rc(rows, cols), 256, 0, s>>>(P.I, P.t.rows, w.A, w.status);
    count_labels_in_range_kernel<<<grid1d(n), 256, 0, s>>>(w.A, n, min_size, max_size, w.counts + 1);
    labeled_area_out_kernel<<<rc(rows, cols), 256, 0, s>>>(P.I, P.t.rows, w.A, min_size, max_size, labels_out,
                                                            pitch_labels, flat_out, pitch_flat);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && count) {
    e = cudaMemcpyAsync(count, w.counts + 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  return finish(e, ws, s, opts);
}

nsgb_status nsgb_bounding_boxes(const int32_t* labels, int64_t rows, int64_t cols, int64_t pitch, int32_t bgval,
                                int32_t* boxes, int64_t capacity, int32_t* count, int32_t* count_dev, void* ws,
                                size_t ws_bytes, nsgb_stream_t stream, const nsgb_opts* opts) {
  if (!labels || !valid_dims(rows, cols) || !valid_pitch(pitch, cols, 4) || capacity < 0 || (capacity > 0 && !boxes))
    return NSGB_ERR_BAD_ARG;
  nsgb_status st = check_ws(ws, ws_bytes, NSGB_OP_BOUNDING_BOX, NSGB_I32, rows, cols);
  if (st != NSGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const Plan P = single_plan(NSGB_I32, (void*)labels, nullptr, rows, cols, pitch);
  cudaError_t e = bbox_launch(P.I, P.t, bgval, ws, boxes, capacity, count_dev, s);
  if (e == cudaSuccess && count) {
    e = cudaMemcpyAsync(count, (const int*)ws + 2, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  return finish(e, ws, s, opts);
}

nsgb_status nsgb_morph_open(const uint8_t* in, uint8_t* out, int64_t rows, int64_t cols, int64_t pitch_in,
                            int64_t pitch_out, const uint8_t* kernel, int k, void* ws, size_t ws_bytes,
                            nsgb_stream_t stream, const nsgb_opts* opts) {
  if (!in || !out || !valid_dims(rows, cols) || !valid_pitch(pitch_in, cols, 1) || !valid_pitch(pitch_out, cols, 1))
    return NSGB_ERR_BAD_ARG;
  MorphElement e;
  if (!morph_element(kernel, k, &e)) return NSGB_ERR_BAD_ARG;
  const char *a0 = (const char*)in, *a1 = a0 + (rows - 1) * pitch_in + cols;
  const char *b0 = (const char*)out, *b1 = b0 + (rows - 1) * pitch_out + cols;
  if (a0 < b1 && b0 < a1) return NSGB_ERR_BAD_ARG;  // out overlaps in
  nsgb_status st = check_ws(ws, ws_bytes, NSGB_OP_MORPH_OPEN, NSGB_U8, rows, cols);
  if (st != NSGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e2 = cudaMemsetAsync(ws, 0, sizeof(int), s);
  if (e2 == cudaSuccess)
    e2 = morph_open_launch(in, pitch_in, out, pitch_out, (int)rows, (int)cols, e, (uint8_t*)ws + 256, s);
  return finish(e2, ws, s, opts);
}

nsgb_status nsgb_distance_transform(const uint8_t* mask, float* out, int64_t rows, int64_t cols, int64_t pitch_in,
                                    int64_t pitch_out, int basins, void* ws, size_t ws_bytes, nsgb_stream_t stream,
                                    const nsgb_opts* opts) {
  if (!mask || !out || !valid_dims(rows, cols) || !valid_pitch(pitch_in, cols, 1) || !valid_pitch(pitch_out, cols, 4) ||
      rows > 65535LL * 128)
    return NSGB_ERR_BAD_ARG;
  nsgb_status st = check_ws(ws, ws_bytes, NSGB_OP_DISTANCE, NSGB_U8, rows, cols);
  if (st != NSGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(ws, 0, sizeof(int), s);
  if (e == cudaSuccess) e = edt_launch(mask, pitch_in, out, pitch_out, (int)rows, (int)cols, basins != 0, ws, s);
  return finish(e, ws, s, opts);
}

nsgb_status nsgb_nucleus_candidates(uint8_t* rc_open, const uint8_t* rc, const uint8_t* rbc, uint8_t* seg_out,
                                    int64_t rows, int64_t cols, int64_t pitch, double g1, double g2,
                                    int32_t area_min, int32_t area_max, int32_t* n_kept, int32_t* n_kept_dev,
                                    void* ws, size_t ws_bytes, nsgb_stream_t stream, const nsgb_opts* opts) {
  if (!rc_open || !rc || !rbc || !seg_out || !valid_dims(rows, cols) || !valid_pitch(pitch, cols, 1))
    return NSGB_ERR_BAD_ARG;
  nsgb_status st = check_ws(ws, ws_bytes, NSGB_OP_NUCLEUS_CANDIDATES, NSGB_U8, rows, cols);
  if (st != NSGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const Plan P = single_plan(NSGB_U8, rc_open, rc, rows, cols, pitch);
  Ws w = carve(ws, P.t);
  cudaError_t e = candidates_impl(P, w, g1, g2, area_min, area_max, rbc, seg_out, opts, s);
  if (e == cudaSuccess && n_kept_dev)
    e = cudaMemcpyAsync(n_kept_dev, w.counts + 1, sizeof(int32_t), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && n_kept) {
    e = cudaMemcpyAsync(n_kept, w.counts + 1, sizeof(int32_t), cudaMemcpyDeviceToHost, s);
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
  const bool vec = ((uintptr_t)in % (4 * esz)) == 0 && pitch_in % (4 * esz) == 0 && ((uintptr_t)out % 4) == 0 &&
                   pitch_out % 4 == 0;
  dispatch_all(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    const GtThr<T> gt = GtThr<T>::make(thr);
    if (vec) threshold_kernel<T, true><<<quad_grid(rows, cols), 256, 0, s>>>((const T*)in, pitch_in, out, pitch_out, H, W, gt);
    else threshold_kernel<T, false><<<quad_grid(rows, cols), 256, 0, s>>>((const T*)in, pitch_in, out, pitch_out, H, W, gt);
  });
  return cuda_status(cudaGetLastError());
}

nsgb_status nsgb_invert(int dtype, const void* in, void* out, int64_t rows, int64_t cols, int64_t pitch,
                        nsgb_stream_t stream) {
  const int esz = elem_size(dtype);
  if (!esz) return NSGB_ERR_UNSUPPORTED_DTYPE;
  if (!in || !out || !valid_dims(rows, cols) || !valid_pitch(pitch, cols, esz)) return NSGB_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const int H = (int)rows, W = (int)cols;
  const bool vec = ((uintptr_t)in % (4 * esz)) == 0 && ((uintptr_t)out % (4 * esz)) == 0 && pitch % (4 * esz) == 0;
  dispatch_all(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    if (vec) invert_kernel<T, true><<<quad_grid(rows, cols), 256, 0, s>>>((const T*)in, (T*)out, pitch, H, W);
    else invert_kernel<T, false><<<quad_grid(rows, cols), 256, 0, s>>>((const T*)in, (T*)out, pitch, H, W);
  });
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
  const Plan P = single_plan(dtype, marker, mask, rows, cols, pitch);
  Ws w = carve(ws, P.t);
  cudaError_t e = chain_impl(dtype, P, w, recon_conn, thr, fill_conn, label_conn, area_min, area_max, fill_out,
                             labels_out, area_out, opts, s);
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

// ---------------------------------------------------------------------------------------------
// Batches.  nsgb_batch_prepare writes the image table into the workspace once and fills the
// caller's nsgb_batch (host copy of the totals); nsgb_chain_batch / nsgb_imreconstruct_batch
// then only enqueue kernels and memsets (plus small count reads when asked for).

namespace {

bool batch_totals(int dtype, const nsgb_tile* tiles, int n, std::vector<Img>* imgs, BatchTotals* t) {
  *t = BatchTotals{};
  if (imgs) imgs->clear();
  const int esz = elem_size(dtype);
  if (!esz || !tiles || n <= 0) return false;
  for (int i = 0; i < n; ++i) {
    const nsgb_tile& tl = tiles[i];
    if (!tl.marker || !tl.mask || !valid_dims(tl.rows, tl.cols) || !valid_pitch(tl.pitch, tl.cols, esz))
      return false;
    Img m = recon_image(dtype, tl.marker, tl.mask, tl.rows, tl.cols, tl.pitch);
    add_image(m, *t);
    m.fill = tl.fill_out;
    m.labels = tl.labels_out;
    m.area = tl.area_out;
    if (t->px >= (int64_t)INT_MAX) return false;
    if (imgs) imgs->push_back(m);
  }
  return true;
}

// Batch workspaces always carry the device table, even for one image.
BatchTotals table_totals(BatchTotals t) {
  if (t.n == 1) t.n = 2;
  return t;
}

nsgb_status batch_plan(const nsgb_batch* b, Plan* P, Ws* w) {
  if (!b || !b->ws) return NSGB_ERR_BAD_ARG;
  BatchTotals t{};
  t.n = b->n;
  t.px = b->total_px;
  t.r_tiles = b->recon_tiles;
  t.c_tiles = b->label_tiles;
  t.blocks = b->rank_blocks;
  t.rows = b->total_rows;
  t.max_w = b->max_cols;
  t.perimeter_max = b->max_perimeter;
  t.f_tiles = b->flood_tiles;
  t.b_words = b->bit_words;
  if (t.n <= 0) return NSGB_ERR_BAD_ARG;
  if (b->ws_bytes < ws_sizes(table_totals(t)).total) return NSGB_ERR_WORKSPACE;
  *w = carve(b->ws, table_totals(t));
  P->t = t;
  P->I = Imgs{};
  P->I.n = t.n;
  P->I.d = w->table;
  P->I.r_img = w->r_img;
  P->I.c_img = w->c_img;
  return NSGB_OK;
}

}  // namespace

extern "C" {

size_t nsgb_batch_workspace_size(int dtype, const nsgb_tile* tiles, int n_tiles) {
  BatchTotals t{};
  if (!batch_totals(dtype, tiles, n_tiles, nullptr, &t)) return 0;
  return ws_sizes(table_totals(t)).total;
}

nsgb_status nsgb_batch_prepare(int dtype, const nsgb_tile* tiles, int n_tiles, void* ws, size_t ws_bytes,
                               nsgb_batch* batch) {
  if (!batch) return NSGB_ERR_BAD_ARG;
  std::vector<Img> imgs;
  BatchTotals t{};
  if (!batch_totals(dtype, tiles, n_tiles, &imgs, &t)) return NSGB_ERR_BAD_ARG;
  nsgb_status st = check_ws_bytes(ws, ws_bytes, nsgb_batch_workspace_size(dtype, tiles, n_tiles));
  if (st != NSGB_OK) return st;
  Ws w = carve(ws, table_totals(t));
  // The tile maps: image of every reconstruction tile, then of every labelling tile.
  std::vector<int> maps((size_t)t.r_tiles + (size_t)t.c_tiles);
  for (int i = 0; i < (int)imgs.size(); ++i) {
    const Img& m = imgs[i];
    const int nr = m.r_tiles_x * m.r_tiles_y;
    const int nc = m.c_tiles_x * ((m.H + ccl::kTile - 1) / ccl::kTile);
    std::fill(maps.begin() + m.r_tile_base, maps.begin() + m.r_tile_base + nr, i);
    std::fill(maps.begin() + t.r_tiles + m.c_tile_base, maps.begin() + t.r_tiles + m.c_tile_base + nc, i);
  }
  // Synchronous copies: the host arrays go away when this returns.
  if (cudaMemcpy(w.table, imgs.data(), sizeof(Img) * imgs.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return NSGB_ERR_CUDA;
  if (cudaMemcpy(w.r_img, maps.data(), sizeof(int) * maps.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return NSGB_ERR_CUDA;
  memset(batch, 0, sizeof(*batch));
  batch->dtype = dtype;
  batch->n = t.n;
  batch->total_px = t.px;
  batch->recon_tiles = t.r_tiles;
  batch->label_tiles = t.c_tiles;
  batch->rank_blocks = t.blocks;
  batch->total_rows = t.rows;
  batch->max_cols = t.max_w;
  batch->max_perimeter = t.perimeter_max;
  batch->flood_tiles = t.f_tiles;
  batch->bit_words = (int)t.b_words;
  batch->ws = ws;
  batch->ws_bytes = ws_bytes;
  return NSGB_OK;
}

nsgb_status nsgb_chain_batch(const nsgb_batch* batch, int recon_conn, double thr, int fill_conn, int label_conn,
                             int32_t area_min, int32_t area_max, int32_t* n_labels, int32_t* n_kept,
                             nsgb_stream_t stream, const nsgb_opts* opts) {
  if (!valid_conn(recon_conn) || !valid_conn(fill_conn) || !valid_conn(label_conn)) return NSGB_ERR_BAD_ARG;
  Plan P;
  Ws w;
  nsgb_status st = batch_plan(batch, &P, &w);
  if (st != NSGB_OK) return st;
  if (batch->dtype == NSGB_F32 || !elem_size(batch->dtype)) return NSGB_ERR_UNSUPPORTED_DTYPE;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = chain_impl(batch->dtype, P, w, recon_conn, thr, fill_conn, label_conn, area_min, area_max,
                             nullptr, nullptr, nullptr, opts, s);
  if (e == cudaSuccess && (n_labels || n_kept)) {
    std::vector<int32_t> c(2 * (size_t)P.t.n);
    e = cudaMemcpyAsync(c.data(), w.counts, c.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    for (int i = 0; i < P.t.n && e == cudaSuccess; ++i) {
      if (n_labels) n_labels[i] = c[2 * i];
      if (n_kept) n_kept[i] = c[2 * i + 1];
    }
  }
  return finish(e, w.status, s, opts);
}

nsgb_status nsgb_batch_counts_async(const nsgb_batch* batch, int32_t* counts, nsgb_stream_t stream) {
  Plan P;
  Ws w;
  if (!counts) return NSGB_ERR_BAD_ARG;
  nsgb_status st = batch_plan(batch, &P, &w);
  if (st != NSGB_OK) return st;
  return cuda_status(cudaMemcpyAsync(counts, w.counts, 2 * sizeof(int32_t) * (size_t)P.t.n, cudaMemcpyDefault,
                                     (cudaStream_t)stream));
}

nsgb_status nsgb_imreconstruct_batch(const nsgb_batch* batch, int conn, int erode, nsgb_stream_t stream,
                                     const nsgb_opts* opts) {
  if (!valid_conn(conn)) return NSGB_ERR_BAD_ARG;
  Plan P;
  Ws w;
  nsgb_status st = batch_plan(batch, &P, &w);
  if (st != NSGB_OK) return st;
  if (!elem_size(batch->dtype)) return NSGB_ERR_UNSUPPORTED_DTYPE;
  cudaStream_t s = (cudaStream_t)stream;
  const bool ring = !erode && (batch->dtype == NSGB_I32 || batch->dtype == NSGB_F32);
  cudaError_t e = recon_timed(opts, batch->dtype, P, conn, erode != 0, ring, w.recon, s);
  return finish(e, w.status, s, opts);
}

}  // extern "C"

// ============================================================================================
// Differentiable float32 reconstruction by dilation (an extension: the reference has no
// gradient).  The result only ever copies input values, so each R(p) has one source pixel:
// mask(q) (clamped at q), marker(q), or the zero ring the reference pads around the image
// (MorphologicOperations.cpp:671-674, which can only win on a border pixel, as 0).  A source
// and the pixels that took its value form a plateau (connected, equal R), so the forward
// labels the plateaus of R with the union-find labeller and gives each the best source it
// contains (mask before marker before ring, then the smallest raster index):
//   prov = ~q (mask q), q (marker q), INT32_MIN (ring); q = y * cols + x within the image.
// The adjoint scatters the upstream gradient along prov with exact 128-bit fixed-point sums
// (resolution 2^-96) and rounds each sum to float once.
namespace nsgb {
namespace {

constexpr int kKeyNone = 0x7F7F7F7F;  // memset byte 0x7F: no source seen yet

// Plateau class: all 32 bits of R (+0 and -0 merged), plus one so that no value is background.
struct ClsPlateau {
  using class_t = uint32_t;
  __device__ uint32_t operator()(const Img& m, int y, int x) const {
    uint32_t v = __float_as_uint(pxcg<float>(m.plane, m.pitch, y, x));
    if ((v << 1) == 0u) v = 0u;
    return v + 1u;
  }
};

__device__ __forceinline__ const void* shifted(const void* p, int64_t off) {
  return (const void*)((uintptr_t)p + (uintptr_t)off);
}

// Source key of pixel (y, x): mask q < marker n + q < ring 2n; kKeyNone if p is no source.
// plane = R, aux = mask, the marker sits `marker_off` bytes from R in every image.
__device__ __forceinline__ int source_key(const Img& m, int64_t marker_off, int y, int x) {
  const float r = pxcg<float>(m.plane, m.pitch, y, x);
  const int n = m.H * m.W, q = y * m.W + x;
  if (r == px<float>(m.aux, m.pitch, y, x)) return q;
  if (r == px<float>(shifted(m.plane, marker_off), m.pitch, y, x)) return n + q;
  if (r == 0.0f && (y == 0 || y == m.H - 1 || x == 0 || x == m.W - 1)) return 2 * n;
  return kKeyNone;
}

// Four pixels per thread; equal roots among them (one plateau) are merged before the atomic.
__global__ void source_best_kernel(Imgs I, int total_rows, int64_t marker_off, const int* __restrict__ L,
                                   int* __restrict__ best) {
  ccl::for_batch_quads(I, total_rows, [&](const Img& m, int y, int x, int n) {
    int key[4], r[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) key[k] = k < n ? source_key(m, marker_off, y, x + k) : kKeyNone;
    if (key[0] == kKeyNone && key[1] == kKeyNone && key[2] == kKeyNone && key[3] == kKeyNone) return;
    ccl::roots4_ro(L, (int64_t)m.px_base + (int64_t)y * m.W + x, n, r);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (key[k] == kKeyNone) continue;
      if (k < 3 && r[k + 1] == r[k]) {  // pass the smaller key on to the next pixel of the plateau
        key[k + 1] = min(key[k + 1], key[k]);
        continue;
      }
      if (key[k] < __ldcg(&best[r[k]])) atomicMin(&best[r[k]], key[k]);
    }
  });
}

__global__ void prov_out_kernel(Imgs I, int total_rows, const int* __restrict__ L, const int* __restrict__ best,
                                int64_t prov_off, int* status) {
  ccl::for_batch_quads(I, total_rows, [&](const Img& m, int y, int x, int n) {
    int r[4], p[4];
    ccl::roots4_ro(L, (int64_t)m.px_base + (int64_t)y * m.W + x, n, r);
    const int np = m.H * m.W;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (k >= n) {
        p[k] = INT_MIN;
        continue;
      }
      const int key = (k > 0 && r[k] == r[k - 1]) ? -1 : __ldg(&best[r[k]]);
      if (key < 0) {
        p[k] = p[k - 1];
      } else if (key < np) {
        p[k] = ~key;
      } else if (key < 2 * np) {
        p[k] = key - np;
      } else {
        p[k] = INT_MIN;
        if (key != 2 * np) set_status(status, NSGB_ERR_BAD_ARG);  // a plateau without a source: NaN input
      }
    }
    store4_i32(pxp<int32_t>((void*)shifted(m.plane, prov_off), m.pitch, y, x), n, p);
  });
}

// Exact fixed point for the adjoint: a value is held as a 128-bit two's-complement integer S
// (lo, hi words) standing for S * 2^-96.  Every float32 g with 2^-73 <= |g| < 2^31 converts
// exactly (its last mantissa bit is worth at least 2^-96); smaller magnitudes round to the
// nearest multiple of 2^-96 (ties to even).  Sums of such values are exact as long as they
// stay below 2^31 in magnitude, and the order in which atomics land does not matter.
struct Fix128 {
  unsigned long long lo;
  long long hi;
};

// Returns false for |g| >= 2^31, inf and NaN.
__device__ __forceinline__ bool fix_from_float(float g, Fix128& out) {
  const uint32_t b = __float_as_uint(g);
  const uint32_t ex = (b >> 23) & 0xFFu;
  uint32_t man = b & 0x7FFFFFu;
  if (ex >= 127u + 31u) return false;
  int sh;  // value = man * 2^sh
  if (ex == 0) {
    sh = -149;
  } else {
    man |= 0x800000u;
    sh = (int)ex - 150;
  }
  // fixed = man * 2^(sh + 96)
  unsigned long long lo = 0, hi = 0;
  const int s = sh + 96;
  if (s >= 0) {  // s <= 157 - 150 + 96 - 1 = 102, man < 2^24: fits in 126 bits
    if (s < 64) {
      lo = (unsigned long long)man << s;
      hi = s == 0 ? 0ull : (unsigned long long)man >> (64 - s);
    } else {
      hi = (unsigned long long)man << (s - 64);
    }
  } else if (-s < 32) {  // round man * 2^s (ties to even)
    const int r = -s;
    const uint32_t q = man >> r, rem = man & ((1u << r) - 1u), half = 1u << (r - 1);
    lo = q + ((rem > half || (rem == half && (q & 1u))) ? 1u : 0u);
  }
  if (b >> 31) {  // negate: two's complement over 128 bits
    lo = ~lo + 1ull;
    hi = ~hi + (lo == 0ull ? 1ull : 0ull);
  }
  out.lo = lo;
  out.hi = (long long)hi;
  return true;
}

__device__ __forceinline__ Fix128 fix_add(const Fix128& a, const Fix128& b) {
  Fix128 r;
  r.lo = a.lo + b.lo;
  r.hi = a.hi + b.hi + (r.lo < a.lo ? 1ll : 0ll);
  return r;
}

// S * 2^-96 rounded to the nearest float (ties to even).  |S| < 2^127, so the result is a
// normal float or zero (the smallest non-zero magnitude, 2^-96, is far above 2^-126).
__device__ __forceinline__ float fix_to_float(unsigned long long lo, long long hi) {
  const bool neg = hi < 0;
  unsigned long long ml = lo, mh = (unsigned long long)hi;
  if (neg) {
    ml = ~ml + 1ull;
    mh = ~mh + (ml == 0ull ? 1ull : 0ull);
  }
  if ((ml | mh) == 0ull) return 0.0f;
  const int lead = mh ? 127 - __clzll((long long)mh) : 63 - __clzll((long long)ml);  // top set bit
  // 24 significant bits: m = floor(M / 2^(lead - 23)), remainder decides the rounding
  uint32_t m;
  bool above_half = false, exactly_half = false;
  if (lead <= 23) {
    m = (uint32_t)(ml << (23 - lead));
  } else {
    const int r = lead - 23;  // bits dropped, 1..104
    // m = bits [r, r + 24) of (mh:ml)
    unsigned long long q;
    if (r >= 64) q = mh >> (r - 64);
    else q = (ml >> r) | (r == 0 ? 0ull : (mh << (64 - r)));
    m = (uint32_t)q;
    // the dropped bits: half = bit r - 1, sticky = bits below it
    const int hb = r - 1;
    const bool hbit = hb >= 64 ? ((mh >> (hb - 64)) & 1ull) : ((ml >> hb) & 1ull);
    bool sticky;
    if (hb >= 64) sticky = ml != 0ull || (hb > 64 && (mh & ((1ull << (hb - 64)) - 1ull)) != 0ull);
    else sticky = hb > 0 && (ml & ((1ull << hb) - 1ull)) != 0ull;
    above_half = hbit && sticky;
    exactly_half = hbit && !sticky;
  }
  int e = lead - 96;  // value = m * 2^(e - 23)
  if (above_half || (exactly_half && (m & 1u))) {
    ++m;
    if (m == (1u << 24)) {
      m >>= 1;
      ++e;
    }
  }
  const uint32_t bits = ((uint32_t)(e + 127) << 23) | (m & 0x7FFFFFu) | (neg ? 0x80000000u : 0u);
  return __uint_as_float(bits);
}

// Adjoint, pass 1: every pixel adds its gradient, as an exact 128-bit fixed-point value, to the
// accumulator of its source.  Lanes of a warp hold consecutive pixels of one row, which mostly
// share a source: a segmented warp scan sums runs of equal targets first, so only the last lane
// of each run issues the atomics (low word, then the high word with the low word's carry).
// plane = g, aux = prov.  acc: two words per source, marker sources then mask sources.
__global__ void grad_scatter_kernel(Imgs I, int total_rows, unsigned long long* __restrict__ acc_marker,
                                    unsigned long long* __restrict__ acc_mask, int* status) {
  const int lane = threadIdx.x & 31;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  for (int gr = blockIdx.y; gr < total_rows; gr += gridDim.y) {  // uniform per block
    const Img m = img_at(I, img_of(I, gr, RowBase()));
    const int y = gr - m.row_base;
    long long key = -1;
    Fix128 v = {0ull, 0ll};
    if (x < m.W) {
      const int32_t p = px<int32_t>(m.aux, m.pitch, y, x);
      if (p != INT_MIN) {
        const int64_t q = p >= 0 ? (int64_t)p : ~(int64_t)p;
        if (q < (int64_t)m.H * m.W && fix_from_float(px<float>(m.plane, m.pitch, y, x), v)) {
          key = ((int64_t)m.px_base + q) | (p < 0 ? (1ll << 40) : 0ll);
        } else {
          set_status(status, NSGB_ERR_BAD_ARG);
          v = Fix128{0ull, 0ll};
        }
      }
    }
    const long long kprev = __shfl_up_sync(NSGB_FULL, key, 1);
    const long long knext = __shfl_down_sync(NSGB_FULL, key, 1);
    bool head = lane == 0 || kprev != key;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      Fix128 v2;
      v2.lo = __shfl_up_sync(NSGB_FULL, v.lo, o);
      v2.hi = __shfl_up_sync(NSGB_FULL, v.hi, o);
      const bool h2 = __shfl_up_sync(NSGB_FULL, head, o);
      if (lane >= o && !head) {
        v = fix_add(v, v2);
        head = h2;
      }
    }
    const bool tail = lane == 31 || knext != key;
    if (tail && key >= 0) {
      unsigned long long* a = ((key >> 40) ? acc_mask : acc_marker) + 2 * (key & ((1ll << 40) - 1));
      const unsigned long long old = atomicAdd(a, v.lo);
      const unsigned long long carry = old + v.lo < old ? 1ull : 0ull;
      atomicAdd(a + 1, (unsigned long long)v.hi + carry);
    }
  }
}

// Adjoint, pass 2: accumulators to float, one rounding each.  plane = g; dmarker / dmask at
// byte offsets.
__global__ void grad_out_kernel(Imgs I, int total_rows, const unsigned long long* __restrict__ acc_marker,
                                const unsigned long long* __restrict__ acc_mask, int64_t dmarker_off,
                                int64_t dmask_off) {
  ccl::for_batch_quads(I, total_rows, [&](const Img& m, int y, int x, int n) {
    const int64_t gi = (int64_t)m.px_base + (int64_t)y * m.W + x;
    float* dm = pxp<float>((void*)shifted(m.plane, dmarker_off), m.pitch, y, x);
    float* dk = pxp<float>((void*)shifted(m.plane, dmask_off), m.pitch, y, x);
    float a[4], b[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (k < n) {
        const ulonglong2 am = __ldcs((const ulonglong2*)(acc_marker + 2 * (gi + k)));
        const ulonglong2 ak = __ldcs((const ulonglong2*)(acc_mask + 2 * (gi + k)));
        a[k] = fix_to_float(am.x, (long long)am.y);
        b[k] = fix_to_float(ak.x, (long long)ak.y);
      } else {
        a[k] = b[k] = 0.f;
      }
    }
    if (n == 4 && (((uintptr_t)dm | (uintptr_t)dk) & 15) == 0) {
      *(float4*)dm = make_float4(a[0], a[1], a[2], a[3]);
      *(float4*)dk = make_float4(b[0], b[1], b[2], b[3]);
    } else {
      for (int k = 0; k < n; ++k) {
        dm[k] = a[k];
        dk[k] = b[k];
      }
    }
  });
}

// Image table of `n` equally sized images `stride` bytes apart (image 0 = proto).
__global__ void stack_table_kernel(Img proto, int n, int64_t stride, BatchTotals one, Img* table) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  Img m = proto;
  m.plane = (void*)((uintptr_t)proto.plane + (uintptr_t)(i * stride));
  m.aux = (const void*)((uintptr_t)proto.aux + (uintptr_t)(i * stride));
  m.r_tile_base = i * one.r_tiles;
  m.r_stile_base = i * one.r_stiles;
  m.r_even_base = i * even_tiles(proto.r_tiles_x, proto.r_tiles_y);
  for (int c = 0; c < 3; ++c) m.r_col_base[c] = i * colour_tiles(proto.r_tiles_x, proto.r_tiles_y, c);
  m.c_tile_base = i * one.c_tiles;
  m.px_base = (int)(i * one.px);
  m.blk_base = i * one.blocks;
  m.row_base = i * one.rows;
  m.b_base = (int)(i * one.b_words);
  m.f_tile_base = i * one.f_tiles;
  table[i] = m;
}

// Totals of `n` stacked copies of one image's plan.
BatchTotals stacked_totals(const BatchTotals& one, int64_t n) {
  BatchTotals t = one;
  t.n = (int)n;
  t.px = one.px * n;
  t.r_tiles = (int)(one.r_tiles * n);
  t.r_stiles = (int)(one.r_stiles * n);
  t.r_even = (int)(one.r_even * n);
  for (int c = 0; c < 3; ++c) t.r_col[c] = (int)(one.r_col[c] * n);
  t.c_tiles = (int)(one.c_tiles * n);
  t.blocks = (int)(one.blocks * n);
  t.rows = (int)(one.rows * n);
  t.b_words = one.b_words * n;
  t.f_tiles = (int)(one.f_tiles * n);
  return t;
}

bool f32_dims_ok(int64_t batch, int64_t rows, int64_t cols, int64_t pitch, int64_t stride) {
  if (batch <= 0 || rows <= 0 || cols <= 0 || rows >= INT_MAX || cols >= INT_MAX) return false;
  if (pitch < cols * 4 || pitch % 4) return false;
  const int64_t n = rows * cols;
  if (2 * n >= kKeyNone || n * batch >= (int64_t)INT_MAX || rows * batch >= (int64_t)INT_MAX) return false;
  if (batch > 1 && (stride < rows * pitch || stride % 4)) return false;
  return true;
}

size_t f32_fwd_bytes(int64_t batch, int64_t rows, int64_t cols) {
  const Plan P1 = single_plan(NSGB_F32, nullptr, nullptr, rows, cols, cols * 4);
  return ws_sizes(stacked_totals(P1.t, batch)).total;
}

size_t f32_bwd_bytes(int64_t batch, int64_t rows, int64_t cols) {
  const size_t px = (size_t)(batch * rows * cols);
  return 256 + 2 * align256(16 * px) + (batch > 1 ? align256(sizeof(Img) * (size_t)batch) : 0);
}

// Plan over the stacked images; with more than one image the table is built on the device.
cudaError_t stacked_plan(void* plane, const void* aux, int64_t batch, int64_t rows, int64_t cols, int64_t pitch,
                         int64_t stride, Img* table, Plan* P, cudaStream_t s) {
  const Plan P1 = single_plan(NSGB_F32, plane, aux, rows, cols, pitch);
  P->t = stacked_totals(P1.t, batch);
  P->I = P1.I;
  P->I.n = (int)batch;
  if (batch == 1) return cudaSuccess;
  Img proto = P1.I.one;
  proto.aligned = proto.aligned && (stride % 4 == 0);
  P->I.one = proto;
  P->I.d = table;
  P->I.r_per = P1.t.r_tiles;
  P->I.c_per = P1.t.c_tiles;
  stack_table_kernel<<<(unsigned)((batch + 127) / 128), 128, 0, s>>>(proto, (int)batch, stride, P1.t, table);
  return cudaGetLastError();
}

}  // namespace
}  // namespace nsgb

extern "C" {

size_t nsgb_recon_f32_workspace_size(int64_t batch, int64_t rows, int64_t cols, int backward) {
  if (!f32_dims_ok(batch, rows, cols, cols * 4, rows * cols * 4)) return 0;
  return backward ? f32_bwd_bytes(batch, rows, cols) : f32_fwd_bytes(batch, rows, cols);
}

nsgb_status nsgb_recon_f32_fwd(const float* marker, const float* mask, float* out, int32_t* prov, int64_t batch,
                               int64_t rows, int64_t cols, int64_t pitch, int64_t image_stride, int conn, void* ws,
                               size_t ws_bytes, nsgb_stream_t stream, const nsgb_opts* opts) {
  if (!marker || !mask || !out || !prov || (const void*)out == (const void*)marker || !valid_conn(conn) ||
      !f32_dims_ok(batch, rows, cols, pitch, image_stride))
    return NSGB_ERR_BAD_ARG;
  nsgb_status st = check_ws_bytes(ws, ws_bytes, f32_fwd_bytes(batch, rows, cols));
  if (st != NSGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const Plan P1 = single_plan(NSGB_F32, out, mask, rows, cols, pitch);
  const Ws w = carve(ws, stacked_totals(P1.t, batch));
  Plan P;
  cudaError_t e = stacked_plan(out, mask, batch, rows, cols, pitch, image_stride, w.table, &P, s);
  // out = marker, image by image (one 2-D copy when the stack is contiguous)
  const bool dense = batch == 1 || image_stride == rows * pitch;
  for (int64_t b = 0; e == cudaSuccess && b < (dense ? 1 : batch); ++b)
    e = cudaMemcpy2DAsync((char*)out + b * image_stride, pitch, (const char*)marker + b * image_stride, pitch,
                          (size_t)cols * 4, (size_t)(dense ? rows * batch : rows), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = recon_timed(opts, NSGB_F32, P, conn, false, true, w.recon, s);
  if (e == cudaSuccess) e = ccl::label(ClsPlateau{}, P.I, P.t, conn, w.forest(false), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w.A, 0x7F, sizeof(int) * (size_t)P.t.px, s);
  if (e == cudaSuccess) {
    const int64_t moff = (int64_t)((uintptr_t)marker - (uintptr_t)out);
    const int64_t poff = (int64_t)((uintptr_t)prov - (uintptr_t)out);
    source_best_kernel<<<qrb(P.t), 256, 0, s>>>(P.I, P.t.rows, moff, w.L, w.A);
    prov_out_kernel<<<qrb(P.t), 256, 0, s>>>(P.I, P.t.rows, w.L, w.A, poff, w.status);
    e = cudaGetLastError();
  }
  return finish(e, ws, s, opts);
}

nsgb_status nsgb_recon_f32_bwd(const float* grad_out, const int32_t* prov, float* grad_marker, float* grad_mask,
                               int64_t batch, int64_t rows, int64_t cols, int64_t pitch, int64_t image_stride,
                               void* ws, size_t ws_bytes, nsgb_stream_t stream, const nsgb_opts* opts) {
  if (!grad_out || !prov || !grad_marker || !grad_mask || !f32_dims_ok(batch, rows, cols, pitch, image_stride))
    return NSGB_ERR_BAD_ARG;
  nsgb_status st = check_ws_bytes(ws, ws_bytes, f32_bwd_bytes(batch, rows, cols));
  if (st != NSGB_OK) return st;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t px = (size_t)(batch * rows * cols);
  char* p = (char*)ws;
  int* status = (int*)p;
  auto* am = (unsigned long long*)(p + 256);
  auto* ak = (unsigned long long*)(p + 256 + align256(16 * px));
  Img* table = batch > 1 ? (Img*)(p + 256 + 2 * align256(16 * px)) : nullptr;
  Plan P;
  cudaError_t e = cudaMemsetAsync(status, 0, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(am, 0, 2 * align256(16 * px), s);
  if (e == cudaSuccess) e = stacked_plan((void*)grad_out, prov, batch, rows, cols, pitch, image_stride, table, &P, s);
  if (e == cudaSuccess) {
    grad_scatter_kernel<<<rcb(P.t), 256, 0, s>>>(P.I, P.t.rows, am, ak, status);
    const int64_t dmo = (int64_t)((uintptr_t)grad_marker - (uintptr_t)grad_out);
    const int64_t dko = (int64_t)((uintptr_t)grad_mask - (uintptr_t)grad_out);
    grad_out_kernel<<<qrb(P.t), 256, 0, s>>>(P.I, P.t.rows, am, ak, dmo, dko);
    e = cudaGetLastError();
  }
  return finish(e, ws, s, opts);
}

}  // extern "C"
