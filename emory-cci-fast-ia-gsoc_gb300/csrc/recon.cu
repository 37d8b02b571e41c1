// Grayscale morphological reconstruction (dilation; erosion through the order-reversing
// dual) on GB300.
//
// Reference semantics: nscale::imreconstruct<T> (MorphologicOperations.cpp:665-838) computes
// the reconstruction of min(marker, mask) under mask with Vincent's hybrid algorithm over a
// 0-padded image.  Its result is the unique fixed point of
//     R(p) = min(mask(p), max(R(p), R(q) for q in N(p)))   starting from min(marker, mask),
// with the padding ring acting as fixed 0-valued neighbours.  Any algorithm that reaches that
// fixed point is bit-identical to it, so this file uses a schedule designed for the GPU
// instead of the serial FIFO:
//
//   * The image is cut into 32-row tiles, one warp per tile visit.  A visit keeps the tile in
//     registers as packed 32-bit words (two 16-bit lanes for u8/u16, one lane for i32/f32),
//     loads a one-pixel halo, and sweeps to the tile's local fixed point: a row pass (left to
//     right and back, a clamp-composition scan) on a transposed copy, then a column pass (down
//     and up, with the diagonals for 8-connectivity), repeated until a column pass changes
//     nothing.  min/max run as max.u16x2 / min.u16x2 on pairs of pixels.
//   * One persistent cooperative kernel runs all visits from a device work queue (a bounded
//     multi-producer / multi-consumer ring with per-slot sequence numbers).  Every tile starts
//     queued in raster order.  Each tile has a state IDLE / QUEUED / RUNNING / RUNNING_DIRTY:
//     a visit that could raise a pixel of a neighbouring tile queues it if it is idle, marks
//     it dirty if it is running (its owner re-runs it before releasing it), and leaves it
//     alone if it is already queued (it has not loaded its halo yet and will read the new
//     values).  A tile is therefore processed by one warp at a time and as soon as it can
//     change; `pending` counts queued and running tiles and the kernel ends when it reaches 0.
//     Stores and state reads / writes are separated by SC fences on both sides, so a neighbour
//     either sees the new values or is re-run.
//
// Every wait is bounded (status NSGB_ERR_TIMEOUT), and the per-visit sweep count and the
// total number of visits are capped (status NSGB_ERR_NOT_CONVERGED).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

#include <atomic>

#include "batch.cuh"
#include "common.cuh"
#include "recon.cuh"
#include "tilequeue.cuh"

namespace nsgb {

namespace {

using namespace tq;

constexpr int kWarps = 4;   // warps (independent tile workers) per CTA
constexpr int kRows = 32;   // rows per tile

// Shared-memory rows are kS = 34 words apart: pairs of words (even index) are 8-byte aligned
// and move as one 64-bit access, and the 16 lanes of each half-warp phase of such an access
// hit 32 distinct banks.
constexpr int kS = 34;

struct alignas(16) WarpBuf {
  uint32_t xp[32 * kS];  // transpose scratch
  uint32_t mh[32 * kS];  // mask, row-pass layout  [lane*kS + j]
  uint32_t mv[32 * kS];  // mask, column-pass layout [lane*kS + i]
  uint32_t lv[36], rv[36];  // halo columns (values), index r + 1 for rows r = -1 .. 32
  uint32_t lm[36], rm[36];  // halo columns (masks)
  uint32_t c0[32], c1[32];  // final first / last tile column, for the neighbour test
  uint32_t hl[32], hr[32];  // per row: what the halo columns give the first / last column
};

// Optional phase timers (compile with -DNSGB_RECON_PROFILE): lane 0 of every warp adds the
// clock cycles spent per phase into 64-bit counters in the workspace header.
#ifdef NSGB_RECON_PROFILE
#define PROF_T0() const long long _pt0 = clock64(); long long _pt = _pt0
#define PROF_MARK(slot)                                                        \
  do {                                                                         \
    const long long _now = clock64();                                          \
    if (lane == 0) atomicAdd(a.c.prof + (slot), (unsigned long long)(_now - _pt)); \
    _pt = _now;                                                                \
  } while (0)
__device__ unsigned long long g_prof_times[1 << 20];  // per-visit start times (ns)
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
#else
#define PROF_T0() \
  do {            \
  } while (0)
#define PROF_MARK(slot) \
  do {                  \
  } while (0)
#endif

// Images of the batch: Img::plane is reconstructed in place (it holds the marker on entry),
// Img::aux is the mask.  Tiles of all images are numbered consecutively.
struct Args {
  Imgs I;
  int ntiles;
  int flip, ring;
  int max_iters;
  int resweeps;  // in-register re-sweeps of a tile marked dirty while it ran
  Ctl c;
};

template <typename T>
__device__ __forceinline__ const T* row_ptr(const T* base, int64_t pitch, int y) {
  return (const T*)((const char*)base + (int64_t)y * pitch);
}
template <typename T>
__device__ __forceinline__ T* row_ptr(T* base, int64_t pitch, int y) {
  return (T*)((char*)base + (int64_t)y * pitch);
}

// Loads the word holding elements (y, x .. x+E-1), flipped into the working order; elements
// outside the image read as LOW.  `coherent` selects L2-coherent loads for planes that other
// warps write during the kernel.
template <typename T>
__device__ __forceinline__ uint32_t load_word(const T* base, int64_t pitch, int y, int x, int H, int W,
                                              bool fast, bool coherent, bool flip) {
  using P = Px<T>;
  const uint32_t ef = flip ? P::ELEM_FLIP : 0u;
  if (y < 0 || y >= H) return P::LOW;
  const T* r = row_ptr(base, pitch, y) + x;
  if constexpr (P::E == 2) {
    if (fast) {
      uint32_t w;
      if constexpr (sizeof(T) == 1) {
        unsigned short v = coherent ? __ldcg((const unsigned short*)r) : __ldg((const unsigned short*)r);
        w = __byte_perm((uint32_t)v, 0u, 0x7170);  // bytes b0,b1 -> 16-bit lanes
      } else {
        w = coherent ? __ldcg((const unsigned int*)r) : __ldg((const unsigned int*)r);
      }
      return w ^ (flip ? P::FLIP : 0u);
    }
    uint32_t e0 = P::LOW, e1 = P::LOW;
    if (x >= 0 && x < W) e0 = (coherent ? P::load_elem(r) : P::load_elem_ro(r)) ^ ef;
    if (x + 1 >= 0 && x + 1 < W) e1 = (coherent ? P::load_elem(r + 1) : P::load_elem_ro(r + 1)) ^ ef;
    return P::pack(e0, e1);
  } else {
    if (x < 0 || x >= W) return P::LOW;
    return (coherent ? P::load_elem(r) : P::load_elem_ro(r)) ^ ef;
  }
}

template <typename T>
__device__ __forceinline__ void store_word(T* base, int64_t pitch, int y, int x, int H, int W, uint32_t w,
                                           bool fast, bool flip) {
  using P = Px<T>;
  if (y < 0 || y >= H) return;
  T* r = row_ptr(base, pitch, y) + x;
  if constexpr (P::E == 2) {
    w ^= flip ? P::FLIP : 0u;
    if (fast) {
      if constexpr (sizeof(T) == 1) {
        __stcg((unsigned short*)r, (unsigned short)__byte_perm(w, 0u, 0x0020));
      } else {
        __stcg((unsigned int*)r, w);
      }
      return;
    }
    if (x >= 0 && x < W) P::store_elem(r, P::elem(w, 0));
    if (x + 1 >= 0 && x + 1 < W) P::store_elem(r + 1, P::elem(w, 1));
  } else {
    if (x < 0 || x >= W) return;
    P::store_elem(r, w ^ (flip ? P::ELEM_FLIP : 0u));
  }
}

// Interior-tile word access at a precomputed address (flip = xor with fx).
// `pairs`: the two elements of a 16-bit-lane word are loaded (stored) separately, for images
// whose rows are not word aligned (an odd u8 width, say); the choice is the same for the whole
// image, so it never diverges.
template <typename T>
__device__ __forceinline__ uint32_t fast_word(const char* p, bool coherent, uint32_t fx, bool pairs) {
  if constexpr (sizeof(T) == 1) {
    if (pairs) {
      const uint32_t b0 = coherent ? __ldcg((const unsigned char*)p) : __ldg((const unsigned char*)p);
      const uint32_t b1 = coherent ? __ldcg((const unsigned char*)p + 1) : __ldg((const unsigned char*)p + 1);
      return (b0 | (b1 << 16)) ^ fx;
    }
    const unsigned short v = coherent ? __ldcg((const unsigned short*)p) : __ldg((const unsigned short*)p);
    return __byte_perm((uint32_t)v, 0u, 0x7170) ^ fx;  // bytes b0,b1 -> 16-bit lanes
  } else if constexpr (sizeof(T) == 2) {
    if (pairs) {
      const uint32_t h0 = coherent ? __ldcg((const unsigned short*)p) : __ldg((const unsigned short*)p);
      const uint32_t h1 = coherent ? __ldcg((const unsigned short*)p + 1) : __ldg((const unsigned short*)p + 1);
      return (h0 | (h1 << 16)) ^ fx;
    }
    return (coherent ? __ldcg((const unsigned int*)p) : __ldg((const unsigned int*)p)) ^ fx;
  } else {
    return (coherent ? __ldcg((const unsigned int*)p) : __ldg((const unsigned int*)p)) ^ fx;
  }
}

template <typename T>
__device__ __forceinline__ void fast_store(char* p, uint32_t w, uint32_t fx, bool pairs) {
  w ^= fx;
  if constexpr (sizeof(T) == 1) {
    if (pairs) {
      __stcg((unsigned char*)p, (unsigned char)(w & 0xFFu));
      __stcg((unsigned char*)p + 1, (unsigned char)((w >> 16) & 0xFFu));
      return;
    }
    __stcg((unsigned short*)p, (unsigned short)__byte_perm(w, 0u, 0x0020));
  } else if constexpr (sizeof(T) == 2) {
    if (pairs) {
      __stcg((unsigned short*)p, (unsigned short)(w & 0xFFFFu));
      __stcg((unsigned short*)p + 1, (unsigned short)(w >> 16));
      return;
    }
    __stcg((unsigned int*)p, w);
  } else {
    __stcg((unsigned int*)p, w);
  }
}

// Initial value rule applied to every loaded value: min(v, mask), and on the image border
// (signed / float dilation only) max with min(0, mask) -- the reference's 0-valued padding.
template <typename T>
__device__ __forceinline__ uint32_t init_word(uint32_t v, uint32_t m, int y, int x, int H, int W, bool ring) {
  using P = Px<T>;
  v = P::vmin(v, m);
  if constexpr (P::E == 1) {
    if (ring && (y == 0 || y == H - 1 || x == 0 || x == W - 1) && y >= 0 && y < H && x >= 0 && x < W)
      v = P::vmax(v, P::vmin(P::ZERO, m));
  }
  return v;
}

template <typename T>
__device__ __forceinline__ uint32_t init_elem(uint32_t v, uint32_t m, int y, int x, int H, int W, bool ring) {
  return init_word<T>(v, m, y, x, H, W, ring);
}

template <typename T>
__device__ __forceinline__ uint32_t load_elem_at(const T* base, int64_t pitch, int y, int x, int H, int W,
                                                 bool coherent, bool flip) {
  using P = Px<T>;
  if (y < 0 || y >= H || x < 0 || x >= W) return P::LOW;
  const T* r = row_ptr(base, pitch, y) + x;
  return (coherent ? P::load_elem(r) : P::load_elem_ro(r)) ^ (flip ? P::ELEM_FLIP : 0u);
}

__device__ __forceinline__ void sts2(uint32_t* p, uint32_t a, uint32_t b) {
  *reinterpret_cast<uint2*>(p) = make_uint2(a, b);
}
__device__ __forceinline__ uint2 lds2(const uint32_t* p) { return *reinterpret_cast<const uint2*>(p); }

// ------------------------------------------------------------------------------------------
// Layout changes.  Column layout: lane l holds words O[i] = (row i, cols E*l .. E*l+E-1).
// Row layout (E = 2): lane h = q + 16*half holds words OH[j] = (rows 2q, 2q+1; col 32*half+j).
// Row layout (E = 1): lane h = row h holds OH[j] = (row h, col j).

template <int E>
__device__ __forceinline__ void col_to_row(uint32_t (&O)[32], uint32_t* xp, int lane) {
#pragma unroll
  for (int i = 0; i < 32; i += 2) sts2(xp + lane * kS + i, O[i], O[i + 1]);
  __syncwarp();
  if constexpr (E == 2) {
    const int q = lane & 15, half = lane >> 4;
#pragma unroll
    for (int j = 0; j < 32; j += 2) {
      const uint2 ab = lds2(xp + (16 * half + (j >> 1)) * kS + 2 * q);
      O[j] = __byte_perm(ab.x, ab.y, 0x5410);
      O[j + 1] = __byte_perm(ab.x, ab.y, 0x7632);
    }
  } else {
#pragma unroll
    for (int j = 0; j < 32; ++j) O[j] = xp[j * kS + lane];
  }
  __syncwarp();
}

template <int E>
__device__ __forceinline__ void row_to_col(uint32_t (&O)[32], uint32_t* xp, int lane) {
#pragma unroll
  for (int j = 0; j < 32; j += 2) sts2(xp + lane * kS + j, O[j], O[j + 1]);
  __syncwarp();
  if constexpr (E == 2) {
    const int h0 = 16 * (lane >> 4);
    const int j0 = (2 * lane) & 31;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const uint2 w = lds2(xp + (h0 + q) * kS + j0);
      O[2 * q] = __byte_perm(w.x, w.y, 0x5410);
      O[2 * q + 1] = __byte_perm(w.x, w.y, 0x7632);
    }
  } else {
#pragma unroll
    for (int i = 0; i < 32; ++i) O[i] = xp[i * kS + lane];
  }
  __syncwarp();
}

// Change tracking.  Values only ever rise during the sweeps, so for u8 (two 16-bit lanes per
// word, each at most 255) the warp-wide sum of all pixels changes if and only if some pixel
// changed: 32 words per lane sum to at most 32 * 255 per 16-bit lane, so nothing carries from
// the low lane of the sum into the high one, and the total does not depend on the layout.  The
// other types compare every word (xor / or), which costs about four times the instructions.
template <typename T>
struct SumTrack { static constexpr bool value = false; };
template <>
struct SumTrack<uint8_t> { static constexpr bool value = true; };

template <typename T>
__device__ __forceinline__ uint32_t tile_sum(const uint32_t (&O)[32]) {
  uint32_t s = 0;
#pragma unroll
  for (int i = 0; i < 32; i += 2) s += O[i] + O[i + 1];
  s = (s & 0xFFFFu) + (s >> 16);
  return __reduce_add_sync(NSGB_FULL, s);
}

// Row pass on the row layout: left-to-right then right-to-left clamp propagation,
// f_j(v) = min(max(v, o_j), m_j).  For E = 2 each row is split over two lanes (columns 0..31 in
// lane q, 32..63 in lane q + 16).  The value entering a half across that seam is the other
// half's current boundary word (before the pass for the left-to-right scan, after it for the
// right-to-left one), so both halves scan at once.  That is a valid update (it only uses actual
// values), but not necessarily a complete one: `exact` reports whether the seam is stable after
// the pass, i.e. whether neither boundary pixel can raise the other.  Only then is the state
// after the pass stable along every row (each half's two scans leave it stable inside the half
// and against the constant halo carries).  If the pass changes nothing, its seam inputs were the
// final values, so it is exact as well.  TRACK: return the xor / or change word.
template <typename T, bool TRACK>
__device__ __forceinline__ uint32_t row_pass(uint32_t (&O)[32], const uint32_t* mh, const WarpBuf& B, int lane,
                                             bool& exact) {
  using P = Px<T>;
  uint32_t acc = 0;
  if constexpr (P::E == 2) {
    const int q = lane & 15, half = lane >> 4;
    const uint32_t carry_l = P::pack(B.hl[2 * q], B.hl[2 * q + 1]);
    const uint32_t carry_r = P::pack(B.hr[2 * q], B.hr[2 * q + 1]);
    const uint32_t seam_l = __shfl_sync(NSGB_FULL, O[31], q);  // left half's last word, before the pass
    uint32_t v = half ? seam_l : carry_l;
#pragma unroll
    for (int j = 0; j < 32; j += 2) {
      const uint2 m = lds2(mh + lane * kS + j);
      const uint32_t n0 = P::vmin(P::vmax(O[j], v), m.x);
      const uint32_t n1 = P::vmin(P::vmax(O[j + 1], n0), m.y);
      if constexpr (TRACK) acc |= (n0 ^ O[j]) | (n1 ^ O[j + 1]);
      O[j] = n0;
      O[j + 1] = n1;
      v = n1;
    }
    const uint32_t seam_r = __shfl_sync(NSGB_FULL, O[0], q + 16);  // right half's first word, after it
    v = half ? carry_r : seam_r;
#pragma unroll
    for (int j = 30; j >= 0; j -= 2) {
      const uint2 m = lds2(mh + lane * kS + j);
      const uint32_t n1 = P::vmin(P::vmax(O[j + 1], v), m.y);
      const uint32_t n0 = P::vmin(P::vmax(O[j], n1), m.x);
      if constexpr (TRACK) acc |= (n0 ^ O[j]) | (n1 ^ O[j + 1]);
      O[j] = n0;
      O[j + 1] = n1;
      v = n0;
    }
    // seam test: can the word across the seam raise this lane's boundary word?
    const uint32_t own = half ? O[0] : O[31];
    const uint32_t other = __shfl_xor_sync(NSGB_FULL, own, 16);
    const uint32_t own_m = mh[lane * kS + (half ? 0 : 31)];
    exact = !__any_sync(NSGB_FULL, P::vmax(own, P::vmin(other, own_m)) != own);
  } else {
    uint32_t v = B.hl[lane];
#pragma unroll
    for (int j = 0; j < 32; j += 2) {
      const uint2 m = lds2(mh + lane * kS + j);
      const uint32_t n0 = P::vmin(P::vmax(O[j], v), m.x);
      const uint32_t n1 = P::vmin(P::vmax(O[j + 1], n0), m.y);
      if constexpr (TRACK) acc |= (n0 ^ O[j]) | (n1 ^ O[j + 1]);
      O[j] = n0;
      O[j + 1] = n1;
      v = n1;
    }
    v = B.hr[lane];
#pragma unroll
    for (int j = 30; j >= 0; j -= 2) {
      const uint2 m = lds2(mh + lane * kS + j);
      const uint32_t n1 = P::vmin(P::vmax(O[j + 1], v), m.y);
      const uint32_t n0 = P::vmin(P::vmax(O[j], n1), m.x);
      if constexpr (TRACK) acc |= (n0 ^ O[j]) | (n1 ^ O[j + 1]);
      O[j] = n0;
      O[j + 1] = n1;
      v = n0;
    }
    exact = true;
  }
  return acc;
}

// One step of a column pass: pixel word o (row i) against the new word of the row before it,
// min(mask, max(o, prev and, for 8-connectivity, prev's left and right neighbours)).  max(o, prev)
// is taken while the shuffles are in flight, so the chain from one row to the next is shuffle,
// funnel shift, two max and one min.  The shuffles return the lane's own word at lanes 0 and 31;
// the neighbour read there instead of one beyond the tile edge is another 8-neighbour of the
// target pixel (the pixel two columns over in the row of the source word, or the pixel above
// it), so it adds nothing beyond the tile.
template <typename T, int CONN>
__device__ __forceinline__ uint32_t col_step(uint32_t o, uint32_t prev, uint32_t m) {
  using P = Px<T>;
  const uint32_t t = P::vmax(o, prev);
  if constexpr (CONN == 8) {
    const uint32_t l = __shfl_up_sync(NSGB_FULL, prev, 1);
    const uint32_t r = __shfl_down_sync(NSGB_FULL, prev, 1);
    return P::vmin(P::vmax(t, P::vmax(P::from_left(l, prev), P::from_right(prev, r))), m);
  } else {
    return P::vmin(t, m);
  }
}

// Column pass on the column layout: top-to-bottom then bottom-to-top, each step taking the
// previous row's new values (and their left/right neighbours for 8-connectivity).  The halo
// columns' contributions (diagonals and corners included) enter through the row pass's
// carries, so the first and last lanes see nothing beyond the tile here.
//
// The rows are scanned as col_chains<T>() interleaved chains of 32 / col_chains<T>() rows each, so that
// the dependent steps of one chain (shuffle, funnel shift, max, min) overlap those of the others.
// A chain that starts inside the tile takes the value of the row before it as it was before the
// pass (top-down) or after the top-down scan (bottom-up).  That is a valid update but may leave a
// seam between chains unstable; a pass that changes nothing has used the final values
// throughout, and the sweep loop only ends on such a pass.
// Two chains for the 16-bit pairs (u8 / u16), four for one element per word (i32 / f32):
// measured 2.5% faster for i32, while u8 took more sweeps per visit with four for no gain.
template <typename T>
constexpr int col_chains() { return Px<T>::E == 1 ? 4 : 2; }

// 4-connectivity only: are the seams between the chains stable after a column pass, i.e. can
// no row at a seam raise the row across it?  (The 4-connected sweep loop may end on an unchanged
// row pass, which needs the column pass before it to have left every column stable.)
template <typename T>
__device__ __forceinline__ bool col_seams_stable(const uint32_t (&O)[32], const WarpBuf& B, int lane) {
  using P = Px<T>;
  constexpr int L = 32 / col_chains<T>();
  bool ok = true;
#pragma unroll
  for (int k = 1; k < col_chains<T>(); ++k) {
    const int i = k * L;  // the seam between rows i - 1 and i (i is even)
    const uint32_t m_above = lds2(B.mv + lane * kS + i - 2).y;  // mask of row i - 1
    const uint32_t m_below = lds2(B.mv + lane * kS + i).x;      // mask of row i
    ok &= P::vmax(O[i], P::vmin(O[i - 1], m_below)) == O[i];
    ok &= P::vmax(O[i - 1], P::vmin(O[i], m_above)) == O[i - 1];
  }
  return __all_sync(NSGB_FULL, ok);
}

template <typename T, int CONN, bool TRACK>
__device__ __forceinline__ uint32_t col_pass(uint32_t (&O)[32], const WarpBuf& B, uint32_t top, uint32_t bot,
                                             int lane) {
  constexpr int NC = col_chains<T>(), L = 32 / NC;
  uint32_t acc = 0;
  uint32_t up[NC];
  up[0] = top;
#pragma unroll
  for (int k = 1; k < NC; ++k) up[k] = O[k * L - 1];
#pragma unroll
  for (int s = 0; s < L; ++s) {
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      const int i = k * L + s;
      const uint32_t m = (i & 1) ? lds2(B.mv + lane * kS + i - 1).y : lds2(B.mv + lane * kS + i).x;
      const uint32_t n = col_step<T, CONN>(O[i], up[k], m);
      if constexpr (TRACK) acc |= n ^ O[i];
      O[i] = n;
      up[k] = n;
    }
  }
  uint32_t dn[NC];
  dn[NC - 1] = bot;
#pragma unroll
  for (int k = 0; k < NC - 1; ++k) dn[k] = O[(k + 1) * L];
#pragma unroll
  for (int s = 0; s < L; ++s) {
#pragma unroll
    for (int k = 0; k < NC; ++k) {
      const int i = (k + 1) * L - 1 - s;
      const uint32_t m = (i & 1) ? lds2(B.mv + lane * kS + i - 1).y : lds2(B.mv + lane * kS + i).x;
      const uint32_t n = col_step<T, CONN>(O[i], dn[k], m);
      if constexpr (TRACK) acc |= n ^ O[i];
      O[i] = n;
      dn[k] = n;
    }
  }
  return acc;
}

template <typename T, int CONN>
__device__ __forceinline__ void halo_carries(WarpBuf& B, int lane) {
  using P = Px<T>;
  uint32_t hl = B.lv[lane + 1], hr = B.rv[lane + 1];
  if constexpr (CONN == 8) {
    hl = P::emax(hl, P::emax(B.lv[lane], B.lv[lane + 2]));
    hr = P::emax(hr, P::emax(B.rv[lane], B.rv[lane + 2]));
  }
  B.hl[lane] = hl;
  B.hr[lane] = hr;
  __syncwarp();
}

// Sweeps a tile in registers (column layout) to its local fixed point: a row pass, then a
// column pass, until a column pass changes nothing after an exact row pass (the state is then
// stable along rows and along columns, diagonals included).  With 4-connectivity both passes
// are idempotent, so a row pass that changes nothing after a column pass ends it too.  Returns
// the number of column passes; a change of any value sets a bit of `any_change` in some lane.
// After `max_iters` column passes the status word gets kDevNotConverged.
template <typename T, int CONN>
__device__ __forceinline__ int sweep_tile(uint32_t (&O)[32], WarpBuf& B, uint32_t topv, uint32_t botv, int lane,
                                          int max_iters, int* status, uint32_t& any_change) {
  constexpr int E = Px<T>::E;
  constexpr bool SUM = SumTrack<T>::value;
  uint32_t total = 0, total0 = 0;
  if constexpr (SUM) total0 = total = tile_sum<T>(O);
  int it = 0;
  bool col_exact = true;  // the last column pass left every column stable (4-connectivity)
  for (;;) {
    col_to_row<E>(O, B.xp, lane);
    bool exact;
    const uint32_t racc = row_pass<T, !SUM>(O, B.mh, B, lane, exact);
    bool rch = true;
    if constexpr (SUM) {
      const uint32_t s = tile_sum<T>(O);
      rch = s != total;
      total = s;
    } else {
      any_change |= racc;
      if constexpr (CONN == 4) rch = __any_sync(NSGB_FULL, racc != 0);
    }
    row_to_col<E>(O, B.xp, lane);
    if (CONN == 4 && it > 0 && !rch && col_exact) break;
    const uint32_t acc = col_pass<T, CONN, !SUM>(O, B, topv, botv, lane);
    if constexpr (CONN == 4 && col_chains<T>() > 1) col_exact = col_seams_stable<T>(O, B, lane);
    bool cch;
    if constexpr (SUM) {
      const uint32_t s = tile_sum<T>(O);
      cch = s != total;
      total = s;
    } else {
      any_change |= acc;
      cch = __any_sync(NSGB_FULL, acc != 0);
    }
    ++it;
    if (!cch && exact) break;
    if (it >= max_iters) {
      if (lane == 0) set_status(status, kDevNotConverged);
      break;
    }
  }
  if constexpr (SUM) any_change |= total != total0 ? 1u : 0u;
  return it;
}

// Image fields: from the kernel parameters for a single image (constant bank, nothing pinned
// in registers), from the device table for a batch.
#define IMF(field) (BATCH ? a.I.d[ii].field : a.I.one.field)

template <typename T, int CONN, bool BATCH, bool RS>
__device__ __forceinline__ void visit(const Args& a, WarpBuf& B, int t, int lane) {
  using P = Px<T>;
  constexpr int E = P::E;
  constexpr int TW = 32 * E;
  const int ii = BATCH ? img_of_tile(a.I, t, a.I.r_img, a.I.r_per, RTileBase()) : 0;
  const int lt = t - IMF(r_tile_base);
  const int ty = lt / IMF(r_tiles_x), tx = lt - ty * IMF(r_tiles_x);
  const int y0 = ty * kRows, x0 = tx * TW;
  const int H = IMF(H), W = IMF(W);
  const bool flip = a.flip != 0, ring = a.ring != 0;
  T* const out = (T*)IMF(plane);
  const T* const mask = (const T*)IMF(aux);
  const int64_t pitch = IMF(pitch);

  PROF_T0();
  const T* src = out;
  const bool coh = true;
  const bool interior = (y0 + kRows <= H) && (x0 + TW <= W);
  // Batches mix odd and even widths (rows of an odd-width u8 image are not word aligned): there
  // every interior tile takes the straight-line path with element loads and stores, which
  // measured 7% faster on the uneven-tile workload than sending unaligned images to the edge
  // path.  A single image takes word loads when its rows are aligned.
  const bool fast = BATCH ? interior : interior && IMF(aligned);
  const bool pairs = BATCH;
  const int xl = x0 + E * lane;
  const uint32_t fx = flip ? P::FLIP : 0u;

  // The caller has taken the tile with an acquire exchange (lane 0); the warp barrier orders
  // every lane's loads after it.
  uint32_t O[32], M[32];
  __syncwarp();
  PROF_MARK(1);

  // All loads of the tile and its halo are issued before any is used, so the visit waits for
  // about one L2 round trip instead of a chain of them.
  if (fast) {
    const char* mp = (const char*)mask + (int64_t)y0 * pitch + (int64_t)xl * sizeof(T);
#pragma unroll
    for (int i = 0; i < 32; ++i) M[i] = fast_word<T>(mp + i * pitch, false, fx, pairs);
  }
  if (fast) {  // interior tile: straight-line loads through running row pointers, no checks
    const char* op = (const char*)src + (int64_t)y0 * pitch + (int64_t)xl * sizeof(T);
#pragma unroll
    for (int i = 0; i < 32; ++i) O[i] = fast_word<T>(op + i * pitch, true, fx, pairs);
  } else {
    // Edge tile: bounds-checked loads in a rolled loop through shared memory
    // (keeps this rarely used path out of the instruction cache's way).
#pragma unroll 1
    for (int i = 0; i < 32; ++i) {
      B.xp[lane * kS + i] = load_word<T>(mask, pitch, y0 + i, xl, H, W, false, false, flip);
      B.mh[lane * kS + i] = load_word<T>(src, pitch, y0 + i, xl, H, W, false, true, flip);
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      M[i] = B.xp[lane * kS + i];
      O[i] = B.mh[lane * kS + i];
    }
    __syncwarp();
  }
  // Halo rows (column layout words) and halo columns (single elements).
  const bool fast_top = fast && !pairs && y0 > 0;
  const bool fast_bot = fast && !pairs && y0 + kRows < H;
  const uint32_t topm = load_word<T>(mask, pitch, y0 - 1, xl, H, W, fast_top, false, flip);
  const uint32_t topv_raw = load_word<T>(src, pitch, y0 - 1, xl, H, W, fast_top, coh, flip);
  const uint32_t botm = load_word<T>(mask, pitch, y0 + kRows, xl, H, W, fast_bot, false, flip);
  const uint32_t botv_raw = load_word<T>(src, pitch, y0 + kRows, xl, H, W, fast_bot, coh, flip);
  uint32_t hm[4], hv[4];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int k = lane + 32 * j;
    const int y = y0 - 1 + k;
    const bool ok = k < 34;
    hm[2 * j] = ok ? load_elem_at<T>(mask, pitch, y, x0 - 1, H, W, false, flip) : P::LOW;
    hm[2 * j + 1] = ok ? load_elem_at<T>(mask, pitch, y, x0 + TW, H, W, false, flip) : P::LOW;
    hv[2 * j] = ok ? load_elem_at<T>(src, pitch, y, x0 - 1, H, W, coh, flip) : P::LOW;
    hv[2 * j + 1] = ok ? load_elem_at<T>(src, pitch, y, x0 + TW, H, W, coh, flip) : P::LOW;
  }
  // any_change: did this visit change a stored value (the clamp to the mask on load counts).
  uint32_t any_change = 0;
#pragma unroll
  for (int i = 0; i < 32; i += 2) sts2(B.mv + lane * kS + i, M[i], M[i + 1]);
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    const uint32_t v = init_word<T>(O[i], M[i], y0 + i, xl, H, W, ring);
    any_change |= v ^ O[i];
    O[i] = v;
  }
  uint32_t topv = init_word<T>(topv_raw, topm, y0 - 1, xl, H, W, ring);
  uint32_t botv = init_word<T>(botv_raw, botm, y0 + kRows, xl, H, W, ring);
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int k = lane + 32 * j;
    if (k < 34) {
      const int y = y0 - 1 + k;
      B.lm[k] = hm[2 * j];
      B.rm[k] = hm[2 * j + 1];
      B.lv[k] = init_elem<T>(hv[2 * j], hm[2 * j], y, x0 - 1, H, W, ring);
      B.rv[k] = init_elem<T>(hv[2 * j + 1], hm[2 * j + 1], y, x0 + TW, H, W, ring);
    }
  }
  __syncwarp();
  // What the (constant) halo columns give each row's first / last pixel: the same-row halo
  // pixel, and for 8-connectivity also the ones above and below (corners included).
  halo_carries<T, CONN>(B, lane);
  // Mask in the row layout.
  if constexpr (E == 2) {
    const int q = lane & 15, half = lane >> 4;
#pragma unroll
    for (int j = 0; j < 32; j += 2) {
      const uint2 m = lds2(B.mv + (16 * half + (j >> 1)) * kS + 2 * q);
      sts2(B.mh + lane * kS + j, __byte_perm(m.x, m.y, 0x5410), __byte_perm(m.x, m.y, 0x7632));
    }
  } else {
#pragma unroll
    for (int j = 0; j < 32; ++j) B.mh[lane * kS + j] = B.mv[j * kS + lane];
  }
  __syncwarp();

  PROF_MARK(2);
#pragma unroll 1
  for (int round = 0;; ++round) {
  const int it = sweep_tile<T, CONN>(O, B, topv, botv, lane, a.max_iters, a.c.status, any_change);
  if (lane == 0) {
    atomicAdd(&a.c.stats[0], 1);
    atomicAdd(&a.c.stats[1], it);
  }

  PROF_MARK(3);
  // Write the tile back, unless the visit changed nothing.
  if (__any_sync(NSGB_FULL, any_change != 0)) {
    if (fast) {
      char* sp = (char*)out + (int64_t)y0 * pitch + (int64_t)xl * sizeof(T);
#pragma unroll
      for (int i = 0; i < 32; ++i) fast_store<T>(sp + i * pitch, O[i], fx, pairs);
    } else {
#pragma unroll
      for (int i = 0; i < 32; ++i) B.xp[lane * kS + i] = O[i];
      __syncwarp();
#pragma unroll 1
      for (int i = 0; i < 32; ++i) store_word<T>(out, pitch, y0 + i, xl, H, W, B.xp[lane * kS + i], false, flip);
      __syncwarp();
    }
  }

  PROF_MARK(4);
  // Which neighbouring tiles could be raised by the new border values?
  unsigned dirs = 0;  // bit (dy+1)*3 + (dx+1)
  {
    // top / bottom rows against the halo rows
    uint32_t c_top = O[0], c_bot = O[31];
    if constexpr (CONN == 8) {
      uint32_t l = __shfl_up_sync(NSGB_FULL, O[0], 1), r = __shfl_down_sync(NSGB_FULL, O[0], 1);
      if (lane == 0) l = P::LOW;
      if (lane == 31) r = P::LOW;
      c_top = P::vmax(c_top, P::vmax(P::from_left(l, O[0]), P::from_right(O[0], r)));
      l = __shfl_up_sync(NSGB_FULL, O[31], 1);
      r = __shfl_down_sync(NSGB_FULL, O[31], 1);
      if (lane == 0) l = P::LOW;
      if (lane == 31) r = P::LOW;
      c_bot = P::vmax(c_bot, P::vmax(P::from_left(l, O[31]), P::from_right(O[31], r)));
    }
    c_top = P::vmin(c_top, topm);
    c_bot = P::vmin(c_bot, botm);
    if (__any_sync(NSGB_FULL, P::vmax(topv, c_top) != topv)) dirs |= 1u << 1;
    if (__any_sync(NSGB_FULL, P::vmax(botv, c_bot) != botv)) dirs |= 1u << 7;
  }
  {
    // first / last columns against the halo columns
    if (lane == 0) {
#pragma unroll
      for (int i = 0; i < 32; ++i) B.c0[i] = P::elem(O[i], 0);
    }
    if (lane == 31) {
#pragma unroll
      for (int i = 0; i < 32; ++i) B.c1[i] = P::elem(O[i], E - 1);
    }
    __syncwarp();
    const int r = lane;
    uint32_t cl = B.c0[r], cr = B.c1[r];
    if constexpr (CONN == 8) {
      if (r > 0) {
        cl = P::emax(cl, B.c0[r - 1]);
        cr = P::emax(cr, B.c1[r - 1]);
      }
      if (r < 31) {
        cl = P::emax(cl, B.c0[r + 1]);
        cr = P::emax(cr, B.c1[r + 1]);
      }
    }
    const bool rl = P::lt(B.lv[r + 1], P::emin(cl, B.lm[r + 1]));
    const bool rr = P::lt(B.rv[r + 1], P::emin(cr, B.rm[r + 1]));
    if (__any_sync(NSGB_FULL, rl)) dirs |= 1u << 3;
    if (__any_sync(NSGB_FULL, rr)) dirs |= 1u << 5;
    if constexpr (CONN == 8) {
      if (P::lt(B.lv[0], P::emin(B.c0[0], B.lm[0]))) dirs |= 1u << 0;
      if (P::lt(B.rv[0], P::emin(B.c1[0], B.rm[0]))) dirs |= 1u << 2;
      if (P::lt(B.lv[33], P::emin(B.c0[31], B.lm[33]))) dirs |= 1u << 6;
      if (P::lt(B.rv[33], P::emin(B.c1[31], B.rm[33]))) dirs |= 1u << 8;
    }
  }
  // The warp barrier orders every lane's stores before the release atomics below.
  __syncwarp();
  PROF_MARK(5);
  // Lane d marks the neighbour in direction d (one copy of the marking code, up to eight
  // neighbours marked in parallel).
  if (lane < 9 && ((dirs >> lane) & 1u)) {
    const int ny = ty + lane / 3 - 1, nx = tx + lane % 3 - 1;
    if (ny >= 0 && ny < IMF(r_tiles_y) && nx >= 0 && nx < IMF(r_tiles_x))
      mark_tile(a.c, IMF(r_tile_base) + ny * IMF(r_tiles_x) + nx);
  }
  __syncwarp();
  PROF_MARK(6);

  // Release the tile.  If a neighbour changed while it ran, only its halo can be stale (no
  // other warp writes its pixels).  Up to `resweeps` times the warp then takes the tile back,
  // reloads just the halo and sweeps again from the values in its registers; otherwise the
  // tile goes to the back of the queue, so that the neighbours still running finish first.
  // Re-sweeping pays off where a front crosses the image (hole filling from the border: about
  // a third less time at 16384^2) and costs time where many neighbours run at once (the
  // h-maxima style marker of the chain: about 8% more), so the caller chooses.
  if constexpr (!RS) {
    // (without re-sweeps the loop body runs once: kept separate so that the compiler emits
    // one copy of the sweep code)
    if (lane == 0) {
      if (atom_cas_acq_rel(&a.c.state[t], kRunning, kIdle) == kRunning) {
        pending_release(a.c);
      } else {
        atom_exch_acq_rel(&a.c.state[t], kQueued);
        atomicAdd(&a.c.stats[2], 1);
        queue_push(a.c, t);
      }
    }
    __syncwarp();
    return;
  }
  int st = 0;
  if (lane == 0) {
    if (atom_cas_acq_rel(&a.c.state[t], kRunning, kIdle) == kRunning) {
      pending_release(a.c);
      st = 0;
    } else if (round < a.resweeps) {
      atom_exch_acq_rel(&a.c.state[t], kRunning);
      atomicAdd(&a.c.stats[3], 1);
      st = 1;
    } else {
      atom_exch_acq_rel(&a.c.state[t], kQueued);
      atomicAdd(&a.c.stats[2], 1);
      queue_push(a.c, t);
      st = 0;
    }
  }
  if (__shfl_sync(NSGB_FULL, st, 0) == 0) return;
  // the acquire exchange above orders reading the halo again after the markers' stores
  __syncwarp();
  {
    const uint32_t tv = load_word<T>(src, pitch, y0 - 1, xl, H, W, fast_top, coh, flip);
    const uint32_t bv = load_word<T>(src, pitch, y0 + kRows, xl, H, W, fast_bot, coh, flip);
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int k = lane + 32 * j;
      const int y = y0 - 1 + k;
      const bool ok = k < 34;
      hv[2 * j] = ok ? load_elem_at<T>(src, pitch, y, x0 - 1, H, W, coh, flip) : P::LOW;
      hv[2 * j + 1] = ok ? load_elem_at<T>(src, pitch, y, x0 + TW, H, W, coh, flip) : P::LOW;
    }
    topv = init_word<T>(tv, topm, y0 - 1, xl, H, W, ring);
    botv = init_word<T>(bv, botm, y0 + kRows, xl, H, W, ring);
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int k = lane + 32 * j;
      if (k < 34) {
        const int y = y0 - 1 + k;
        B.lv[k] = init_elem<T>(hv[2 * j], B.lm[k], y, x0 - 1, H, W, ring);
        B.rv[k] = init_elem<T>(hv[2 * j + 1], B.rm[k], y, x0 + TW, H, W, ring);
      }
    }
    __syncwarp();
    halo_carries<T, CONN>(B, lane);
  }
  any_change = 0;
  }
}

// ------------------------------------------------------------------------------------------
// Streaming passes (before the work queue).  A pass sweeps every tile of a grid to its local
// fixed point once, with the halo read from the current state, in parallel and without queue,
// tile states or fences (the passes are separate launches, so each sees the previous one's
// stores).  The grid alternates between the tile grid and the grid shifted by half a tile in
// each direction: the boundaries of one pass lie inside the tiles of the next, so what a pass
// could not carry across its tile boundaries the next one carries inside its tiles.  All
// updates only ever raise values towards the fixed point, so the passes give a valid starting
// state for the queue whatever they achieve.  The last pass is on the tile grid and runs the
// queue visit's neighbour test: every tile whose halo it could still raise is flagged in the
// state array, and the queue starts from exactly the flagged tiles.  Every other tile was
// swept to its local fixed point and no neighbour could raise its halo since, so the queue's
// invariant (a tile that is not queued or running is stable) holds from the start.
struct PassArgs {
  Imgs I;
  int ntiles;      // tiles of this pass's grid (all images)
  int oy, ox;      // grid offset in pixels (0, or half a tile)
  int flip, ring;
  int max_iters;
  int* status;
  int* flags;      // last pass: the queue's tile state array (flagged neighbours set to kQueued)
};

struct RSTileBase { __device__ int operator()(const Img& m) const { return m.r_stile_base; } };

template <typename T, int CONN, bool BATCH, bool FLAGS>
__device__ __forceinline__ void pass_tile(const PassArgs& a, WarpBuf& B, int t, int lane) {
  using P = Px<T>;
  constexpr int E = P::E;
  constexpr int TW = 32 * E;
  const bool shifted = a.oy != 0;
  const int ii = BATCH ? (shifted ? img_of(a.I, t, RSTileBase()) : img_of_tile(a.I, t, a.I.r_img, a.I.r_per, RTileBase()))
                       : 0;
  const Img& m = BATCH ? a.I.d[ii] : a.I.one;
  const int H = m.H, W = m.W;
  const int ntx = shifted ? (W + a.ox + TW - 1) / TW : m.r_tiles_x;
  const int lt = t - (BATCH ? (shifted ? m.r_stile_base : m.r_tile_base) : 0);
  const int ty = lt / ntx, tx = lt - ty * ntx;
  const int y0 = ty * kRows - a.oy, x0 = tx * TW - a.ox;
  const bool flip = a.flip != 0, ring = a.ring != 0;
  T* const out = (T*)m.plane;
  const T* const mask = (const T*)m.aux;
  const int64_t pitch = m.pitch;
  const bool interior = y0 >= 0 && x0 >= 0 && (y0 + kRows <= H) && (x0 + TW <= W);
  const bool fast = BATCH ? interior : interior && m.aligned;
  const bool pairs = BATCH;
  const int xl = x0 + E * lane;
  const uint32_t fx = flip ? P::FLIP : 0u;

  uint32_t O[32], M[32];
  if (fast) {
    const char* mp = (const char*)mask + (int64_t)y0 * pitch + (int64_t)xl * sizeof(T);
    const char* op = (const char*)out + (int64_t)y0 * pitch + (int64_t)xl * sizeof(T);
#pragma unroll
    for (int i = 0; i < 32; ++i) M[i] = fast_word<T>(mp + i * pitch, false, fx, pairs);
#pragma unroll
    for (int i = 0; i < 32; ++i) O[i] = fast_word<T>(op + i * pitch, true, fx, pairs);
  } else {
#pragma unroll 1
    for (int i = 0; i < 32; ++i) {
      B.xp[lane * kS + i] = load_word<T>(mask, pitch, y0 + i, xl, H, W, false, false, flip);
      B.mh[lane * kS + i] = load_word<T>(out, pitch, y0 + i, xl, H, W, false, true, flip);
    }
    __syncwarp();
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      M[i] = B.xp[lane * kS + i];
      O[i] = B.mh[lane * kS + i];
    }
    __syncwarp();
  }
  const bool fast_top = fast && !pairs && y0 > 0;
  const bool fast_bot = fast && !pairs && y0 + kRows < H;
  const uint32_t topm = load_word<T>(mask, pitch, y0 - 1, xl, H, W, fast_top, false, flip);
  const uint32_t topv_raw = load_word<T>(out, pitch, y0 - 1, xl, H, W, fast_top, true, flip);
  const uint32_t botm = load_word<T>(mask, pitch, y0 + kRows, xl, H, W, fast_bot, false, flip);
  const uint32_t botv_raw = load_word<T>(out, pitch, y0 + kRows, xl, H, W, fast_bot, true, flip);
  uint32_t hm[4], hv[4];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int k = lane + 32 * j;
    const int y = y0 - 1 + k;
    const bool ok = k < 34;
    hm[2 * j] = ok ? load_elem_at<T>(mask, pitch, y, x0 - 1, H, W, false, flip) : P::LOW;
    hm[2 * j + 1] = ok ? load_elem_at<T>(mask, pitch, y, x0 + TW, H, W, false, flip) : P::LOW;
    hv[2 * j] = ok ? load_elem_at<T>(out, pitch, y, x0 - 1, H, W, true, flip) : P::LOW;
    hv[2 * j + 1] = ok ? load_elem_at<T>(out, pitch, y, x0 + TW, H, W, true, flip) : P::LOW;
  }
  uint32_t any_change = 0;
#pragma unroll
  for (int i = 0; i < 32; i += 2) sts2(B.mv + lane * kS + i, M[i], M[i + 1]);
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    const uint32_t v = init_word<T>(O[i], M[i], y0 + i, xl, H, W, ring);
    any_change |= v ^ O[i];
    O[i] = v;
  }
  const uint32_t topv = init_word<T>(topv_raw, topm, y0 - 1, xl, H, W, ring);
  const uint32_t botv = init_word<T>(botv_raw, botm, y0 + kRows, xl, H, W, ring);
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int k = lane + 32 * j;
    if (k < 34) {
      const int y = y0 - 1 + k;
      B.lm[k] = hm[2 * j];
      B.rm[k] = hm[2 * j + 1];
      B.lv[k] = init_elem<T>(hv[2 * j], hm[2 * j], y, x0 - 1, H, W, ring);
      B.rv[k] = init_elem<T>(hv[2 * j + 1], hm[2 * j + 1], y, x0 + TW, H, W, ring);
    }
  }
  __syncwarp();
  halo_carries<T, CONN>(B, lane);
  if constexpr (E == 2) {
    const int q = lane & 15, half = lane >> 4;
#pragma unroll
    for (int j = 0; j < 32; j += 2) {
      const uint2 mm = lds2(B.mv + (16 * half + (j >> 1)) * kS + 2 * q);
      sts2(B.mh + lane * kS + j, __byte_perm(mm.x, mm.y, 0x5410), __byte_perm(mm.x, mm.y, 0x7632));
    }
  } else {
#pragma unroll
    for (int j = 0; j < 32; ++j) B.mh[lane * kS + j] = B.mv[j * kS + lane];
  }
  __syncwarp();

  sweep_tile<T, CONN>(O, B, topv, botv, lane, a.max_iters, a.status, any_change);

  if (__any_sync(NSGB_FULL, any_change != 0)) {
    if (fast) {
      char* sp = (char*)out + (int64_t)y0 * pitch + (int64_t)xl * sizeof(T);
#pragma unroll
      for (int i = 0; i < 32; ++i) fast_store<T>(sp + i * pitch, O[i], fx, pairs);
    } else {
#pragma unroll
      for (int i = 0; i < 32; ++i) B.xp[lane * kS + i] = O[i];
      __syncwarp();
#pragma unroll 1
      for (int i = 0; i < 32; ++i) store_word<T>(out, pitch, y0 + i, xl, H, W, B.xp[lane * kS + i], false, flip);
      __syncwarp();
    }
  }
  if constexpr (FLAGS) {
    // the queue visit's neighbour test: which neighbouring tiles could the border raise?
    unsigned dirs = 0;
    {
      uint32_t c_top = O[0], c_bot = O[31];
      if constexpr (CONN == 8) {
        uint32_t l = __shfl_up_sync(NSGB_FULL, O[0], 1), r = __shfl_down_sync(NSGB_FULL, O[0], 1);
        if (lane == 0) l = P::LOW;
        if (lane == 31) r = P::LOW;
        c_top = P::vmax(c_top, P::vmax(P::from_left(l, O[0]), P::from_right(O[0], r)));
        l = __shfl_up_sync(NSGB_FULL, O[31], 1);
        r = __shfl_down_sync(NSGB_FULL, O[31], 1);
        if (lane == 0) l = P::LOW;
        if (lane == 31) r = P::LOW;
        c_bot = P::vmax(c_bot, P::vmax(P::from_left(l, O[31]), P::from_right(O[31], r)));
      }
      c_top = P::vmin(c_top, topm);
      c_bot = P::vmin(c_bot, botm);
      if (__any_sync(NSGB_FULL, P::vmax(topv, c_top) != topv)) dirs |= 1u << 1;
      if (__any_sync(NSGB_FULL, P::vmax(botv, c_bot) != botv)) dirs |= 1u << 7;
    }
    {
      if (lane == 0) {
#pragma unroll
        for (int i = 0; i < 32; ++i) B.c0[i] = P::elem(O[i], 0);
      }
      if (lane == 31) {
#pragma unroll
        for (int i = 0; i < 32; ++i) B.c1[i] = P::elem(O[i], E - 1);
      }
      __syncwarp();
      const int r = lane;
      uint32_t cl = B.c0[r], cr = B.c1[r];
      if constexpr (CONN == 8) {
        if (r > 0) {
          cl = P::emax(cl, B.c0[r - 1]);
          cr = P::emax(cr, B.c1[r - 1]);
        }
        if (r < 31) {
          cl = P::emax(cl, B.c0[r + 1]);
          cr = P::emax(cr, B.c1[r + 1]);
        }
      }
      const bool rl = P::lt(B.lv[r + 1], P::emin(cl, B.lm[r + 1]));
      const bool rr = P::lt(B.rv[r + 1], P::emin(cr, B.rm[r + 1]));
      if (__any_sync(NSGB_FULL, rl)) dirs |= 1u << 3;
      if (__any_sync(NSGB_FULL, rr)) dirs |= 1u << 5;
      if constexpr (CONN == 8) {
        if (P::lt(B.lv[0], P::emin(B.c0[0], B.lm[0]))) dirs |= 1u << 0;
        if (P::lt(B.rv[0], P::emin(B.c1[0], B.rm[0]))) dirs |= 1u << 2;
        if (P::lt(B.lv[33], P::emin(B.c0[31], B.lm[33]))) dirs |= 1u << 6;
        if (P::lt(B.rv[33], P::emin(B.c1[31], B.rm[33]))) dirs |= 1u << 8;
      }
      __syncwarp();
    }
    if (lane < 9 && ((dirs >> lane) & 1u)) {
      const int ny = ty + lane / 3 - 1, nx = tx + lane % 3 - 1;
      if (ny >= 0 && ny < m.r_tiles_y && nx >= 0 && nx < m.r_tiles_x)
        a.flags[(BATCH ? m.r_tile_base : 0) + ny * m.r_tiles_x + nx] = kQueued;
    }
    __syncwarp();
  }
}

// One warp per tile of the pass's grid.
template <typename T, int CONN, bool BATCH, bool FLAGS>
__global__ void __launch_bounds__(kWarps * 32, 4) recon_pass_kernel(PassArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpBuf& B = reinterpret_cast<WarpBuf*>(smem_raw)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const int t = blockIdx.x * kWarps + (threadIdx.x >> 5);
  if (t >= a.ntiles) return;
  pass_tile<T, CONN, BATCH, FLAGS>(a, B, t, lane);
}

// The queue's starting state after the passes: the tiles the last pass flagged (state
// kQueued) go into the ring, every other tile is idle.  If none was flagged the done flag is
// raised at once, so the queue kernel ends without work.
__global__ void recon_seed_kernel(Ctl c, int ntiles, unsigned* counter) {
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < c.cap; i += gridDim.x * blockDim.x) {
    if ((int)i < ntiles && c.state[i] == kQueued) {
      const unsigned k = atomicAdd(counter, 1u);
      c.slots[k].val = (int)i;
      c.slots[k].seq = k + 1u;
    }
  }
}
// The passes' tile visits count towards the visit budget: the queue's counter starts there.
__global__ void recon_seed_finish_kernel(Ctl c, const unsigned* counter, unsigned long long pass_visits) {
  // slots k >= count: empty for this lap
  const unsigned n = *counter;
  for (unsigned i = n + blockIdx.x * blockDim.x + threadIdx.x; i < c.cap; i += gridDim.x * blockDim.x) {
    c.slots[i].val = -1;
    c.slots[i].seq = i;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *c.head = 0u;
    *c.tail = n;
    *c.pending = (int)n;
    *c.visit_count = pass_visits;
    if (pass_visits > (unsigned long long)c.max_visits) set_status(c.status, kDevNotConverged);
    if (n == 0) *c.done = 1;
  }
}

template <typename T, int CONN, bool BATCH, bool RS>
__global__ void __launch_bounds__(kWarps * 32, 4) recon_kernel(Args a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpBuf& B = reinterpret_cast<WarpBuf*>(smem_raw)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  int visits_here = 0;
  for (;;) {
    int t = 0;
#ifdef NSGB_RECON_PROFILE
    const long long _pp = clock64();
#endif
    if (lane == 0) t = queue_pop(a.c);
    t = __shfl_sync(NSGB_FULL, t, 0);
#ifdef NSGB_RECON_PROFILE
    if (lane == 0) atomicAdd(a.c.prof + 0, (unsigned long long)(clock64() - _pp));
#endif
    if (t < 0) break;
#ifdef NSGB_RECON_PROFILE
    if (lane == 0) {
      const unsigned k = atomicAdd((unsigned*)&a.c.stats[4], 1u);
      if (k < (1u << 20)) g_prof_times[k] = global_ns();
    }
#endif
    if (lane == 0) atom_exch_acquire(&a.c.state[t], kRunning);
    visit<T, CONN, BATCH, RS>(a, B, t, lane);
#ifdef NSGB_RECON_PROFILE
    const long long _pe = clock64();
#endif
    if (lane == 0) {
      // the visit budget is checked every `budget_step` visits of this warp (every visit
      // when the caller set a budget, every 16 against the default one)
      if (++visits_here == a.c.budget_step) {
        if (atomicAdd(a.c.visit_count, (unsigned long long)visits_here) + (unsigned long long)visits_here >
            (unsigned long long)a.c.max_visits)
          set_status(a.c.status, kDevNotConverged);
        visits_here = 0;
      }
    }
    __syncwarp();
#ifdef NSGB_RECON_PROFILE
    if (lane == 0) atomicAdd(a.c.prof + 7, (unsigned long long)(clock64() - _pe));
#endif
    if (ld_relaxed(a.c.status) != 0) break;
  }
}

// Initial ring contents: every tile queued once.  A batch queues the tiles of each colour of
// the image's order (checkerboard: 2 colours, four-colour order: 4) for all images before any
// tile of the next colour, so tiles taken at the same time are not neighbours across the whole
// batch (per image, the first colour of a small image would otherwise run next to the second
// one).
__global__ void recon_init_kernel(Ctl c, Imgs I, int ntiles, int order) {
  int even_total = 0;
  int col_end[4] = {0, 0, 0, 0};  // four-colour order: end of each colour's range in the ring
  if (I.d && order == 1) {
    const Img& last = I.d[I.n - 1];
    even_total = last.r_even_base + even_tiles(last.r_tiles_x, last.r_tiles_y);
  }
  if (I.d && order == 2) {
    const Img& last = I.d[I.n - 1];
    int acc = 0;
    for (int k = 0; k < 4; ++k) {
      acc += RColBase{k}(last) + colour_tiles(last.r_tiles_x, last.r_tiles_y, k);
      col_end[k] = acc;
    }
  }
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < c.cap; i += gridDim.x * blockDim.x) {
    if ((int)i < ntiles) {
      Img im;
      int local;
      if (I.d && order == 2) {
        int k = 0;
        while (k < 3 && (int)i >= col_end[k]) ++k;
        const int j = (int)i - (k ? col_end[k - 1] : 0);
        im = I.d[img_of(I, j, RColBase{k})];
        local = j - RColBase{k}(im);
        for (int q = 0; q < k; ++q) local += colour_tiles(im.r_tiles_x, im.r_tiles_y, q);
      } else if (I.d && order == 1) {
        if ((int)i < even_total) {
          im = I.d[img_of(I, (int)i, REvenBase())];
          local = (int)i - im.r_even_base;
        } else {
          const int j = (int)i - even_total;
          im = I.d[img_of(I, j, ROddBase())];
          local = even_tiles(im.r_tiles_x, im.r_tiles_y) + j - (im.r_tile_base - im.r_even_base);
        }
      } else {
        im = img_at(I, img_of(I, (int)i, RTileBase()));
        local = (int)i - im.r_tile_base;
      }
      c.slots[i].val = im.r_tile_base + initial_tile(local, im.r_tiles_x * im.r_tiles_y, im.r_tiles_x, order);
      c.slots[i].seq = i + 1u;
      c.state[i] = kQueued;
    } else {
      c.slots[i].val = -1;
      c.slots[i].seq = i;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *c.head = 0u;
    *c.tail = (unsigned)ntiles;
    *c.pending = ntiles;
  }
}

// Workspace layout (ints): [0] status, [1..4] stats (visits, sweeps, re-runs, re-sweeps),
// [5] profiler visit index, [6..7] visit counter (64-bit), [8] tiles seeded by the streaming
// passes, [32] head, [64] tail, [96] pending,
// [128] done flag, [160..175] phase timers (8 x 64-bit); from int kHdrInts: state[ntiles],
// then the ring (2 ints per slot, cap slots).  Head, tail, pending and the done flag sit on
// separate 128-byte lines: the atomics of the working warps and the polls of the waiting
// ones then do not queue behind one another.
constexpr int kHdrInts = 192;
constexpr int kSeedCounter = 8;  // header int: tiles flagged by the last streaming pass

template <typename T>
int tiles_x_for(int64_t W) { return (int)((W + 32 * Px<T>::E - 1) / (32 * Px<T>::E)); }

// The schedule's tuned defaults: the autotuner (tune.py) writes tuning.json, and the build
// compiles it into kTuning (tuning.inc, generated): per dtype, connectivity, direction, single
// image or batch and image size, the number of streaming passes and the initial ring order.
// Without an entry: no passes, and the ring order measured best on the synthetic tiles (single
// images: checkerboard for 32 x 64 tiles, four colours for 32 x 32; batches: four colours).  NSGB_RECON_PASSES / NSGB_RECON_ORDER override the defaults for experiments.
struct TuneEntry {
  int dtype, conn, erode, batch;
  long long max_px;
  int passes, order, ctas;
};
#include "tuning.inc"

struct Schedule {
  int passes, order, ctas;  // ctas: queue CTAs per SM, 0 = as many as fit
};

int env_int(const char* name, std::atomic<int>& cache) {
  int v = cache.load(std::memory_order_relaxed);
  if (v == -2) {
    const char* e = getenv(name);
    v = (e && *e) ? atoi(e) : -1;
    cache.store(v, std::memory_order_relaxed);
  }
  return v;
}

Schedule tuned_schedule(int dtype, int conn, bool erode, bool batch, long long px) {
  Schedule sc;
  sc.passes = 0;
  sc.ctas = 0;
  sc.order = batch ? 2 : ((dtype == NSGB_U8 || dtype == NSGB_U16) ? 1 : 2);
  for (const TuneEntry& t : kTuning) {
    if (t.max_px > 0 && t.dtype == dtype && t.conn == conn && t.erode == (erode ? 1 : 0) &&
        t.batch == (batch ? 1 : 0) && px <= t.max_px) {
      sc.passes = t.passes;
      sc.order = t.order;
      sc.ctas = t.ctas;
      break;
    }
  }
  static std::atomic<int> env_passes{-2}, env_order{-2}, env_ctas{-2};
  const int ep = env_int("NSGB_RECON_PASSES", env_passes), eo = env_int("NSGB_RECON_ORDER", env_order);
  const int ec = env_int("NSGB_RECON_CTAS", env_ctas);
  if (ep >= 0) sc.passes = ep;
  if (eo >= 0) sc.order = eo;
  if (ec >= 0) sc.ctas = ec;
  return sc;
}

// Streaming passes before the queue (see recon_pass_kernel): `passes` launches alternating
// between the shifted and the tile grid, the last on the tile grid with neighbour flags, then
// the ring is seeded with the flagged tiles.  Returns false if the passes do not apply (a
// batch without shifted-grid bases).
template <typename T, int CONN, bool BATCH>
cudaError_t run_passes(const Imgs& I, int ntiles, int nstiles, const Ctl& c, int* wi, bool erode, bool ring,
                       int max_iters, int passes, cudaStream_t s) {
  constexpr int TW = 32 * Px<T>::E;
  const size_t smem = sizeof(WarpBuf) * kWarps;
  cudaError_t e = cudaMemsetAsync(c.state, 0, sizeof(int) * (size_t)ntiles, s);
  if (e != cudaSuccess) return e;
  PassArgs p;
  p.I = I;
  p.flip = erode ? 1 : 0;
  p.ring = ring ? 1 : 0;
  p.max_iters = max_iters;
  p.status = c.status;
  p.flags = c.state;
  for (int k = 0; k < passes; ++k) {
    const bool shifted = ((passes - 1 - k) & 1) != 0;
    const bool last = k == passes - 1;
    p.oy = shifted ? kRows / 2 : 0;
    p.ox = shifted ? TW / 2 : 0;
    p.ntiles = shifted ? nstiles : ntiles;
    const dim3 grid((p.ntiles + kWarps - 1) / kWarps);
    if (last) {
      e = cudaFuncSetAttribute(recon_pass_kernel<T, CONN, BATCH, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
      if (e != cudaSuccess) return e;
      recon_pass_kernel<T, CONN, BATCH, true><<<grid, kWarps * 32, smem, s>>>(p);
    } else {
      e = cudaFuncSetAttribute(recon_pass_kernel<T, CONN, BATCH, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
      if (e != cudaSuccess) return e;
      recon_pass_kernel<T, CONN, BATCH, false><<<grid, kWarps * 32, smem, s>>>(p);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  unsigned* counter = (unsigned*)(wi + kSeedCounter);
  const int sgrid = (int)((c.cap + 255) / 256);
  unsigned long long visits = 0;
  for (int k = 0; k < passes; ++k) visits += (((passes - 1 - k) & 1) != 0) ? (unsigned)nstiles : (unsigned)ntiles;
  recon_seed_kernel<<<sgrid, 256, 0, s>>>(c, ntiles, counter);
  recon_seed_finish_kernel<<<sgrid, 256, 0, s>>>(c, counter, visits);
  return cudaGetLastError();
}

template <typename T, int CONN, bool BATCH, bool RS>
cudaError_t launch_typed(const Imgs& I, int ntiles, bool erode, bool ring, void* ws, cudaStream_t s,
                         int max_visits_per_tile, int max_iters, int resweeps, long long poll_limit, int passes,
                         int nstiles, int order, int ctas) {
  Args a;
  a.I = I;
  a.ntiles = ntiles;
  a.flip = erode ? 1 : 0;
  a.ring = ring ? 1 : 0;
  a.max_iters = max_iters > 0 ? max_iters : 4096;
  a.resweeps = resweeps;
  int* wi = (int*)ws;
  a.c.status = wi + 0;
  a.c.stats = wi + 1;
  a.c.visit_count = (unsigned long long*)(wi + 6);
  a.c.prof = (unsigned long long*)(wi + 160);
  a.c.head = (unsigned*)(wi + 32);
  a.c.tail = (unsigned*)(wi + 64);
  a.c.pending = wi + 96;
  a.c.done = wi + 128;
  a.c.state = wi + kHdrInts;
  a.c.cap = ring_cap(ntiles);
  a.c.slots = (Slot*)(a.c.state + ((ntiles + 1) & ~1));
  a.c.max_visits = (long long)(max_visits_per_tile > 0 ? max_visits_per_tile : 1 << 20) * ntiles;
  a.c.budget_step = max_visits_per_tile > 0 ? 1 : 16;
  a.c.spin_limit = poll_limit > 0 ? poll_limit : kSpinLimit;

  cudaError_t e = cudaMemsetAsync(wi, 0, sizeof(int) * kHdrInts, s);
  if (e != cudaSuccess) return e;
  if (passes > 0 && (!BATCH || nstiles > 0)) {
    e = run_passes<T, CONN, BATCH>(I, ntiles, nstiles, a.c, wi, erode, ring, a.max_iters, passes, s);
  } else {
    recon_init_kernel<<<(a.c.cap + 255) / 256, 256, 0, s>>>(a.c, I, ntiles, order);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return e;

  const size_t smem = sizeof(WarpBuf) * kWarps;
  // The shared-memory opt-in is set on every launch (it belongs to the context, which a device
  // reset replaces); the co-resident grid size is computed once per device and instantiation.
  // Two host threads' first calls may both compute it: they store the same value.
  e = cudaFuncSetAttribute(recon_kernel<T, CONN, BATCH, RS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  constexpr int kOccDevices = 64;
  static std::atomic<int> occ_cache[kOccDevices];
  int dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const bool cached = dev >= 0 && dev < kOccDevices;
  int occ = cached ? occ_cache[dev].load(std::memory_order_relaxed) : 0;
  if (occ == 0) {
    int bps = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, recon_kernel<T, CONN, BATCH, RS>, kWarps * 32, smem);
    if (e != cudaSuccess) return e;
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    occ = bps * sms;
    if (occ <= 0) return cudaErrorLaunchOutOfResources;
    if (cached) occ_cache[dev].store(occ, std::memory_order_relaxed);
  }
  if (ctas > 0) {
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    if ((long long)ctas * sms < occ) occ = ctas * sms;
  }
  int grid = (ntiles + kWarps - 1) / kWarps;
  if (grid > occ) grid = occ;
  if (grid < 1) grid = 1;
  void* args[] = {&a};
  // Cooperative launch: all CTAs are co-resident, so warps waiting on the queue never block
  // warps that still have to be scheduled.
  return cudaLaunchCooperativeKernel((const void*)recon_kernel<T, CONN, BATCH, RS>, dim3(grid), dim3(kWarps * 32), args, smem,
                                     s);
}

}  // namespace

int recon_tiles_x(int dtype, int64_t W) {
  switch (dtype) {
    case NSGB_U8: return tiles_x_for<uint8_t>(W);
    case NSGB_U16: return tiles_x_for<uint16_t>(W);
    case NSGB_I32: return tiles_x_for<int32_t>(W);
    case NSGB_F32: return tiles_x_for<float>(W);
    default: return 0;
  }
}

int recon_tiles_y(int64_t H) { return (int)((H + kRows - 1) / kRows); }

// Tiles of the grid shifted by half a tile (rows -16 .., columns -TW/2 ..) covering the image.
int recon_stiles(int dtype, int64_t H, int64_t W) {
  const int E = (dtype == NSGB_U8 || dtype == NSGB_U16) ? 2 : 1;
  const int64_t TW = 32 * E;
  const int64_t ny = (H + kRows / 2 + kRows - 1) / kRows, nx = (W + TW / 2 + TW - 1) / TW;
  return (int)(ny * nx);
}

size_t recon_workspace_bytes_tiles(int64_t nt) {
  return sizeof(int) * (size_t)(kHdrInts + ((nt + 1) & ~1) + 2 * (int64_t)ring_cap(nt));
}

size_t recon_workspace_bytes(int dtype, int64_t H, int64_t W) {
  const int tx = recon_tiles_x(dtype, W);
  if (tx <= 0) return 0;
  return recon_workspace_bytes_tiles((int64_t)tx * recon_tiles_y(H));
}

namespace {
// Kernel instantiation for a call: image table or single image, connectivity, and re-sweeps
// (their loop is a separate kernel, so that the common path keeps one copy of the sweep code;
// re-sweeps are offered for single images, where hole filling uses them).
template <typename T, bool RS>
cudaError_t dispatch_conn(const Imgs& I, int ntiles, int conn, bool erode, bool ring, void* ws, cudaStream_t s,
                          int max_visits, int max_iters, int resweeps, long long poll, int passes, int nstiles,
                          int order, int ctas) {
  if (I.d)
    return conn == 8 ? launch_typed<T, 8, true, false>(I, ntiles, erode, ring, ws, s, max_visits, max_iters, 0, poll,
                                                       passes, nstiles, order, ctas)
                     : launch_typed<T, 4, true, false>(I, ntiles, erode, ring, ws, s, max_visits, max_iters, 0, poll,
                                                       passes, nstiles, order, ctas);
  return conn == 8 ? launch_typed<T, 8, false, RS>(I, ntiles, erode, ring, ws, s, max_visits, max_iters, resweeps, poll,
                                                   passes, nstiles, order, ctas)
                   : launch_typed<T, 4, false, RS>(I, ntiles, erode, ring, ws, s, max_visits, max_iters, resweeps, poll,
                                                   passes, nstiles, order, ctas);
}

}  // namespace

cudaError_t recon_launch_batch(int dtype, const Imgs& I, int ntiles, int conn, bool erode, bool ring, void* ws,
                               cudaStream_t s, int max_visits, int max_iters, int resweeps, long long poll_limit,
                               int passes, int nstiles, int order, long long total_px, int ctas) {
  if (!I.d) {
    nstiles = recon_stiles(dtype, I.one.H, I.one.W);
    total_px = (long long)I.one.H * I.one.W;
  }
  const Schedule sc = tuned_schedule(dtype, conn, erode, I.d != nullptr, I.d ? total_px / (I.n > 0 ? I.n : 1) : total_px);
  passes = passes > 0 ? passes : passes < 0 ? 0 : sc.passes;
  order = order > 0 ? order - 1 : sc.order;
  ctas = ctas > 0 ? ctas : sc.ctas;
  switch (dtype) {
#define NSGB_RECON_CASE(CODE, TYPE)                                                                           \
  case CODE:                                                                                                   \
    return resweeps > 0 ? dispatch_conn<TYPE, true>(I, ntiles, conn, erode, ring, ws, s, max_visits, max_iters,  \
                                                    resweeps, poll_limit, passes, nstiles, order, ctas)         \
                        : dispatch_conn<TYPE, false>(I, ntiles, conn, erode, ring, ws, s, max_visits, max_iters, \
                                                     resweeps, poll_limit, passes, nstiles, order, ctas);
    NSGB_RECON_CASE(NSGB_U8, uint8_t)
    NSGB_RECON_CASE(NSGB_U16, uint16_t)
    NSGB_RECON_CASE(NSGB_I32, int32_t)
    NSGB_RECON_CASE(NSGB_F32, float)
#undef NSGB_RECON_CASE
    default: return cudaErrorInvalidValue;
  }
}

Img recon_image(int dtype, void* plane, const void* mask, int64_t H, int64_t W, int64_t pitch) {
  Img m = {};
  m.plane = plane;
  m.aux = mask;
  m.pitch = pitch;
  m.H = (int)H;
  m.W = (int)W;
  const int esz = elem_size(dtype);
  const int vec = (dtype == NSGB_U8 || dtype == NSGB_U16) ? 2 * esz : esz;
  m.aligned = (((uintptr_t)plane % vec) == 0 && ((uintptr_t)mask % vec) == 0 && (pitch % vec) == 0) ? 1 : 0;
  m.r_tiles_x = recon_tiles_x(dtype, W);
  m.r_tiles_y = recon_tiles_y(H);
  m.r_tile_base = 0;
  m.r_tw = (dtype == NSGB_U8 || dtype == NSGB_U16) ? 64 : 32;
  m.r_stile_base = 0;
  return m;
}

cudaError_t recon_launch(int dtype, void* out, const void* marker, const void* mask, int64_t H, int64_t W,
                         int64_t pitch, int conn, bool erode, bool ring, void* ws, cudaStream_t s, int max_visits,
                         int max_iters, long long poll_limit, int passes, int order, int ctas) {
  if (marker != out) {
    // The kernel works in place; start from a copy of the marker.
    const int esz = elem_size(dtype);
    cudaError_t e = cudaMemcpy2DAsync(out, pitch, marker, pitch, (size_t)W * esz, (size_t)H, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  Imgs I = {};
  I.n = 1;
  I.one = recon_image(dtype, out, mask, H, W, pitch);
  return recon_launch_batch(dtype, I, I.one.r_tiles_x * I.one.r_tiles_y, conn, erode, ring, ws, s, max_visits,
                            max_iters, 0, poll_limit, passes, 0, order, 0, ctas);
}

}  // namespace nsgb

#ifdef NSGB_RECON_PROFILE
extern "C" int nsgb_prof_times(void* dst, int n) {
  return (int)cudaMemcpyFromSymbol(dst, nsgb::g_prof_times, sizeof(unsigned long long) * (size_t)n);
}
#endif
