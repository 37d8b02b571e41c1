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
//   * One persistent cooperative kernel runs all visits.  Round 0 visits every tile; a visit
//     that could raise a pixel of a neighbouring tile puts that tile on the next round's work
//     list (deduplicated with round stamps); a neighbour already queued for the current round
//     and not yet started is skipped because it will read the new values.  Rounds are
//     separated by a bounded grid barrier; the kernel ends when a round queues nothing.
//
// Every wait is bounded (status NSGB_ERR_TIMEOUT), and the per-visit sweep count and the
// number of rounds are capped (status NSGB_ERR_NOT_CONVERGED).
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "recon.cuh"

namespace nsgb {

namespace {

constexpr int kWarps = 4;   // warps (independent tile workers) per CTA
constexpr int kRows = 32;   // rows per tile

struct alignas(16) WarpBuf {
  uint32_t xp[32 * 33];  // transpose scratch
  uint32_t mh[32 * 33];  // mask, row-pass layout  [lane*33 + j]
  uint32_t mv[32 * 33];  // mask, column-pass layout [lane*33 + i]
  uint32_t lv[36], rv[36];  // halo columns (values), index r + 1 for rows r = -1 .. 32
  uint32_t lm[36], rm[36];  // halo columns (masks)
  uint32_t c0[32], c1[32];  // final first / last tile column, for the neighbour test
};

struct Ctl {
  int* enq;     // [ntiles] round in which the tile is next scheduled
  int* start;   // [ntiles] last round in which the tile was started
  int* list0;   // [ntiles]
  int* list1;   // [ntiles]
  int* claim;   // [3] per-round claim counters (slot = round % 3)
  int* count;   // [3] per-round list lengths
  unsigned* bar;  // [2] grid barrier
  int* status;
  int* stats;   // [0] rounds, [1] visits, [2] sweeps
};

template <typename T>
struct Args {
  T* out;
  const T* marker;
  const T* mask;
  int64_t pitch;  // bytes, shared by the three planes
  int H, W;
  int tiles_x, tiles_y, ntiles;
  int flip, ring, aligned;
  int max_rounds, max_iters;
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

// ------------------------------------------------------------------------------------------
// Layout changes.  Column layout: lane l holds words O[i] = (row i, cols E*l .. E*l+E-1).
// Row layout (E = 2): lane h = q + 16*half holds words OH[j] = (rows 2q, 2q+1; col 32*half+j).
// Row layout (E = 1): lane h = row h holds OH[j] = (row h, col j).

template <int E>
__device__ __forceinline__ void col_to_row(uint32_t (&O)[32], uint32_t* xp, int lane) {
#pragma unroll
  for (int i = 0; i < 32; ++i) xp[lane * 33 + i] = O[i];
  __syncwarp();
  if constexpr (E == 2) {
    const int q = lane & 15, half = lane >> 4;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int l = 16 * half + (j >> 1);
      uint32_t a = xp[l * 33 + 2 * q], b = xp[l * 33 + 2 * q + 1];
      O[j] = (j & 1) ? __byte_perm(a, b, 0x7632) : __byte_perm(a, b, 0x5410);
    }
  } else {
#pragma unroll
    for (int j = 0; j < 32; ++j) O[j] = xp[j * 33 + lane];
  }
  __syncwarp();
}

template <int E>
__device__ __forceinline__ void row_to_col(uint32_t (&O)[32], uint32_t* xp, int lane) {
#pragma unroll
  for (int j = 0; j < 32; ++j) xp[lane * 33 + j] = O[j];
  __syncwarp();
  if constexpr (E == 2) {
    const int h0 = 16 * (lane >> 4);
    const int j0 = (2 * lane) & 31;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      uint32_t w0 = xp[(h0 + q) * 33 + j0], w1 = xp[(h0 + q) * 33 + j0 + 1];
      O[2 * q] = __byte_perm(w0, w1, 0x5410);
      O[2 * q + 1] = __byte_perm(w0, w1, 0x7632);
    }
  } else {
#pragma unroll
    for (int i = 0; i < 32; ++i) O[i] = xp[i * 33 + lane];
  }
  __syncwarp();
}

// Row pass on the row layout: left-to-right then right-to-left clamp propagation.
// f_j(v) = min(max(v, o_j), m_j); for E = 2 each row is split over two lanes, whose
// composed clamps (lo, hi) carry the left half's exit value into the right half.
template <typename T>
__device__ __forceinline__ uint32_t row_pass(uint32_t (&O)[32], const uint32_t* mh, const WarpBuf& B, int lane) {
  using P = Px<T>;
  uint32_t acc = 0;
  if constexpr (P::E == 2) {
    const int q = lane & 15, half = lane >> 4;
    // ---- left to right
    {
      uint32_t lo = P::LOW, hi = P::HIGH;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const uint32_t m = mh[lane * 33 + j];
        lo = P::vmin(P::vmax(lo, O[j]), m);
        hi = P::vmin(P::vmax(hi, O[j]), m);
      }
      const uint32_t carry = P::pack(B.lv[2 * q + 1], B.lv[2 * q + 2]);
      const uint32_t ex = P::vmin(P::vmax(carry, lo), hi);
      const uint32_t from0 = __shfl_up_sync(NSGB_FULL, ex, 16);
      uint32_t v = half ? from0 : carry;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const uint32_t m = mh[lane * 33 + j];
        const uint32_t n = P::vmin(P::vmax(O[j], v), m);
        acc |= n ^ O[j];
        O[j] = n;
        v = n;
      }
    }
    // ---- right to left
    {
      uint32_t lo = P::LOW, hi = P::HIGH;
#pragma unroll
      for (int j = 31; j >= 0; --j) {
        const uint32_t m = mh[lane * 33 + j];
        lo = P::vmin(P::vmax(lo, O[j]), m);
        hi = P::vmin(P::vmax(hi, O[j]), m);
      }
      const uint32_t carry = P::pack(B.rv[2 * q + 1], B.rv[2 * q + 2]);
      const uint32_t ex = P::vmin(P::vmax(carry, lo), hi);
      const uint32_t from1 = __shfl_down_sync(NSGB_FULL, ex, 16);
      uint32_t v = half ? carry : from1;
#pragma unroll
      for (int j = 31; j >= 0; --j) {
        const uint32_t m = mh[lane * 33 + j];
        const uint32_t n = P::vmin(P::vmax(O[j], v), m);
        acc |= n ^ O[j];
        O[j] = n;
        v = n;
      }
    }
  } else {
    uint32_t v = B.lv[lane + 1];
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const uint32_t m = mh[lane * 33 + j];
      const uint32_t n = P::vmin(P::vmax(O[j], v), m);
      acc |= n ^ O[j];
      O[j] = n;
      v = n;
    }
    v = B.rv[lane + 1];
#pragma unroll
    for (int j = 31; j >= 0; --j) {
      const uint32_t m = mh[lane * 33 + j];
      const uint32_t n = P::vmin(P::vmax(O[j], v), m);
      acc |= n ^ O[j];
      O[j] = n;
      v = n;
    }
  }
  return acc;
}

// Column pass on the column layout: top-to-bottom then bottom-to-top, each step taking the
// previous row's new values (and their left/right neighbours for 8-connectivity).
template <typename T, int CONN>
__device__ __forceinline__ uint32_t col_pass(uint32_t (&O)[32], const WarpBuf& B, uint32_t top, uint32_t bot,
                                             int lane) {
  using P = Px<T>;
  uint32_t acc = 0;
  uint32_t up = top;
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    uint32_t a = up;
    if constexpr (CONN == 8) {
      uint32_t l = __shfl_up_sync(NSGB_FULL, up, 1);
      uint32_t r = __shfl_down_sync(NSGB_FULL, up, 1);
      if (lane == 0) l = P::as_last(B.lv[i]);
      if (lane == 31) r = P::as_first(B.rv[i]);
      a = P::vmax(a, P::vmax(P::from_left(l, up), P::from_right(up, r)));
    }
    const uint32_t m = B.mv[lane * 33 + i];
    const uint32_t n = P::vmin(P::vmax(O[i], a), m);
    acc |= n ^ O[i];
    O[i] = n;
    up = n;
  }
  uint32_t dn = bot;
#pragma unroll
  for (int i = 31; i >= 0; --i) {
    uint32_t a = dn;
    if constexpr (CONN == 8) {
      uint32_t l = __shfl_up_sync(NSGB_FULL, dn, 1);
      uint32_t r = __shfl_down_sync(NSGB_FULL, dn, 1);
      if (lane == 0) l = P::as_last(B.lv[i + 2]);
      if (lane == 31) r = P::as_first(B.rv[i + 2]);
      a = P::vmax(a, P::vmax(P::from_left(l, dn), P::from_right(dn, r)));
    }
    const uint32_t m = B.mv[lane * 33 + i];
    const uint32_t n = P::vmin(P::vmax(O[i], a), m);
    acc |= n ^ O[i];
    O[i] = n;
    dn = n;
  }
  return acc;
}

__device__ __forceinline__ void mark_tile(const Ctl& c, int nt, int round) {
  if (round > 0) {
    // Queued for this round and not started: it will read the values just written.
    if (ld_relaxed(&c.enq[nt]) == round && ld_relaxed(&c.start[nt]) < round) return;
  }
  if (atomicMax(&c.enq[nt], round + 1) < round + 1) {
    int* next = ((round + 1) & 1) ? c.list1 : c.list0;
    const int idx = atomicAdd(&c.count[(round + 1) % 3], 1);
    next[idx] = nt;
  }
}

template <typename T, int CONN>
__device__ __forceinline__ void visit(const Args<T>& a, WarpBuf& B, int t, int round, int lane) {
  using P = Px<T>;
  constexpr int E = P::E;
  constexpr int TW = 32 * E;
  const int ty = t / a.tiles_x, tx = t - ty * a.tiles_x;
  const int y0 = ty * kRows, x0 = tx * TW;
  const int H = a.H, W = a.W;
  const bool flip = a.flip != 0, ring = a.ring != 0;

  if (lane == 0) atomicExch(&a.c.start[t], round);
  __syncwarp();
  __threadfence();

  const bool first = (round == 0);
  const T* src = first ? a.marker : a.out;
  const bool coh = !first || (a.marker == a.out);
  const bool interior = (y0 + kRows <= H) && (x0 + TW <= W);
  const bool fast = interior && a.aligned;
  const int xl = x0 + E * lane;

  uint32_t O[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    const int y = y0 + i;
    const uint32_t m = load_word<T>(a.mask, a.pitch, y, xl, H, W, fast, false, flip);
    const uint32_t v = load_word<T>(src, a.pitch, y, xl, H, W, fast, coh, flip);
    B.mv[lane * 33 + i] = m;
    O[i] = init_word<T>(v, m, y, xl, H, W, ring);
  }
  // Halo rows (column layout words) and halo columns (single elements).
  const bool fast_top = fast && y0 > 0;
  const bool fast_bot = fast && y0 + kRows < H;
  const uint32_t topm = load_word<T>(a.mask, a.pitch, y0 - 1, xl, H, W, fast_top, false, flip);
  const uint32_t topv = init_word<T>(load_word<T>(src, a.pitch, y0 - 1, xl, H, W, fast_top, coh, flip), topm,
                                     y0 - 1, xl, H, W, ring);
  const uint32_t botm = load_word<T>(a.mask, a.pitch, y0 + kRows, xl, H, W, fast_bot, false, flip);
  const uint32_t botv = init_word<T>(load_word<T>(src, a.pitch, y0 + kRows, xl, H, W, fast_bot, coh, flip), botm,
                                     y0 + kRows, xl, H, W, ring);
  for (int k = lane; k < 34; k += 32) {
    const int y = y0 - 1 + k;
    const uint32_t lm = load_elem_at<T>(a.mask, a.pitch, y, x0 - 1, H, W, false, flip);
    const uint32_t rm = load_elem_at<T>(a.mask, a.pitch, y, x0 + TW, H, W, false, flip);
    B.lm[k] = lm;
    B.rm[k] = rm;
    B.lv[k] = init_elem<T>(load_elem_at<T>(src, a.pitch, y, x0 - 1, H, W, coh, flip), lm, y, x0 - 1, H, W, ring);
    B.rv[k] = init_elem<T>(load_elem_at<T>(src, a.pitch, y, x0 + TW, H, W, coh, flip), rm, y, x0 + TW, H, W, ring);
  }
  __syncwarp();
  // Mask in the row layout.
  if constexpr (E == 2) {
    const int q = lane & 15, half = lane >> 4;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int l = 16 * half + (j >> 1);
      const uint32_t m0 = B.mv[l * 33 + 2 * q], m1 = B.mv[l * 33 + 2 * q + 1];
      B.mh[lane * 33 + j] = (j & 1) ? __byte_perm(m0, m1, 0x7632) : __byte_perm(m0, m1, 0x5410);
    }
  } else {
#pragma unroll
    for (int j = 0; j < 32; ++j) B.mh[lane * 33 + j] = B.mv[j * 33 + lane];
  }
  __syncwarp();

  // Sweep to the local fixed point.
  int it = 0;
  for (;;) {
    col_to_row<E>(O, B.xp, lane);
    row_pass<T>(O, B.mh, B, lane);
    row_to_col<E>(O, B.xp, lane);
    const uint32_t acc = col_pass<T, CONN>(O, B, topv, botv, lane);
    ++it;
    if (!__any_sync(NSGB_FULL, acc != 0)) break;
    if (it >= a.max_iters) {
      if (lane == 0) set_status(a.c.status, kDevNotConverged);
      break;
    }
  }
  if (lane == 0) {
    atomicAdd(&a.c.stats[1], 1);
    atomicAdd(&a.c.stats[2], it);
  }

  // Write the tile back.
#pragma unroll
  for (int i = 0; i < 32; ++i) store_word<T>(a.out, a.pitch, y0 + i, xl, H, W, O[i], fast, flip);

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
  __threadfence();
  __syncwarp();
  if (lane == 0 && dirs) {
#pragma unroll
    for (int d = 0; d < 9; ++d) {
      if (!((dirs >> d) & 1u)) continue;
      const int ny = ty + d / 3 - 1, nx = tx + d % 3 - 1;
      if (ny < 0 || ny >= a.tiles_y || nx < 0 || nx >= a.tiles_x) continue;
      mark_tile(a.c, ny * a.tiles_x + nx, round);
    }
  }
  __syncwarp();
}

template <typename T, int CONN>
__global__ void __launch_bounds__(kWarps * 32, 4) recon_kernel(Args<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  WarpBuf& B = reinterpret_cast<WarpBuf*>(smem_raw)[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  int round = 0;
  for (;;) {
    const int n_cur = (round == 0) ? a.ntiles : ld_acquire(&a.c.count[round % 3]);
    const int* list = (round & 1) ? a.c.list1 : a.c.list0;
    for (;;) {
      int idx = 0;
      if (lane == 0) idx = atomicAdd(&a.c.claim[round % 3], 1);
      idx = __shfl_sync(NSGB_FULL, idx, 0);
      if (idx >= n_cur) break;
      const int t = (round == 0) ? idx : __ldcg(&list[idx]);
      visit<T, CONN>(a, B, t, round, lane);
      if (ld_relaxed(a.c.status) != 0) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.c.claim[(round + 2) % 3] = 0;
      a.c.count[(round + 2) % 3] = 0;
    }
    if (!grid_barrier(a.c.bar, gridDim.x, a.c.status)) break;
    const int nn = ld_acquire(&a.c.count[(round + 1) % 3]);
    if (nn == 0 || ld_relaxed(a.c.status) != 0) break;
    if (++round >= a.max_rounds) {
      if (blockIdx.x == 0 && threadIdx.x == 0) set_status(a.c.status, kDevNotConverged);
      break;
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) a.c.stats[0] = round + 1;
}

// Workspace layout (ints): status, stats[3], claim[3], count[3], bar[2] (unsigned), pad to 32;
// then enq, start, list0, list1 (ntiles each).
constexpr int kHdrInts = 32;

template <typename T>
int tiles_x_for(int64_t W) { return (int)((W + 32 * Px<T>::E - 1) / (32 * Px<T>::E)); }

template <typename T, int CONN>
cudaError_t launch_typed(void* out, const void* marker, const void* mask, int64_t H, int64_t W, int64_t pitch,
                         bool erode, bool ring, void* ws, cudaStream_t s, int max_rounds, int max_iters) {
  Args<T> a;
  a.out = (T*)out;
  a.marker = (const T*)marker;
  a.mask = (const T*)mask;
  a.pitch = pitch;
  a.H = (int)H;
  a.W = (int)W;
  a.tiles_x = tiles_x_for<T>(W);
  a.tiles_y = (int)((H + kRows - 1) / kRows);
  a.ntiles = a.tiles_x * a.tiles_y;
  a.flip = erode ? 1 : 0;
  a.ring = ring ? 1 : 0;
  const int vec = Px<T>::E == 2 ? 2 * (int)sizeof(T) : (int)sizeof(T);
  a.aligned = (((uintptr_t)out % vec) == 0 && ((uintptr_t)marker % vec) == 0 && ((uintptr_t)mask % vec) == 0 &&
               (pitch % vec) == 0)
                  ? 1
                  : 0;
  a.max_rounds = max_rounds > 0 ? max_rounds : (1 << 24);
  a.max_iters = max_iters > 0 ? max_iters : 4096;
  int* wi = (int*)ws;
  a.c.status = wi + 0;
  a.c.stats = wi + 1;
  a.c.claim = wi + 4;
  a.c.count = wi + 7;
  a.c.bar = (unsigned*)(wi + 10);
  a.c.enq = wi + kHdrInts;
  a.c.start = a.c.enq + a.ntiles;
  a.c.list0 = a.c.start + a.ntiles;
  a.c.list1 = a.c.list0 + a.ntiles;

  cudaError_t e;
  // Header and enq = 0; start = -1.
  e = cudaMemsetAsync(wi, 0, sizeof(int) * (kHdrInts + (size_t)a.ntiles), s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(a.c.start, 0xFF, sizeof(int) * (size_t)a.ntiles, s);
  if (e != cudaSuccess) return e;

  const size_t smem = sizeof(WarpBuf) * kWarps;
  static int occ_cache[8][2] = {{0}};  // per device, per instantiation set below
  int dev = 0;
  cudaGetDevice(&dev);
  int& occ = occ_cache[dev & 7][0];
  if (occ == 0) {
    e = cudaFuncSetAttribute(recon_kernel<T, CONN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int bps = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, recon_kernel<T, CONN>, kWarps * 32, smem);
    if (e != cudaSuccess) return e;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    occ = bps * sms;
    if (occ <= 0) return cudaErrorLaunchOutOfResources;
  }
  int grid = (a.ntiles + kWarps - 1) / kWarps;
  if (grid > occ) grid = occ;
  if (grid < 1) grid = 1;
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel((const void*)recon_kernel<T, CONN>, dim3(grid), dim3(kWarps * 32), args, smem,
                                     s);
}

}  // namespace

size_t recon_workspace_bytes(int dtype, int64_t H, int64_t W) {
  int64_t tx = 0;
  switch (dtype) {
    case NSGB_U8: tx = tiles_x_for<uint8_t>(W); break;
    case NSGB_U16: tx = tiles_x_for<uint16_t>(W); break;
    case NSGB_I32: tx = tiles_x_for<int32_t>(W); break;
    case NSGB_F32: tx = tiles_x_for<float>(W); break;
    default: return 0;
  }
  const int64_t ty = (H + kRows - 1) / kRows;
  return sizeof(int) * (size_t)(kHdrInts + 4 * tx * ty);
}

cudaError_t recon_launch(int dtype, void* out, const void* marker, const void* mask, int64_t H, int64_t W,
                         int64_t pitch, int conn, bool erode, bool ring, void* ws, cudaStream_t s, int max_rounds,
                         int max_iters) {
  switch (dtype) {
#define NSGB_RECON_CASE(CODE, TYPE)                                                                         \
  case CODE:                                                                                                 \
    return conn == 8 ? launch_typed<TYPE, 8>(out, marker, mask, H, W, pitch, erode, ring, ws, s, max_rounds, \
                                             max_iters)                                                      \
                     : launch_typed<TYPE, 4>(out, marker, mask, H, W, pitch, erode, ring, ws, s, max_rounds, \
                                             max_iters);
    NSGB_RECON_CASE(NSGB_U8, uint8_t)
    NSGB_RECON_CASE(NSGB_U16, uint16_t)
    NSGB_RECON_CASE(NSGB_I32, int32_t)
    NSGB_RECON_CASE(NSGB_F32, float)
#undef NSGB_RECON_CASE
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace nsgb
