// Flat grayscale erosion and dilation of u8 images by a k x k structuring element, and the
// opening nscale::morphOpen<unsigned char> builds from them (src/segment/MorphologicOperations.cpp:
// 2459-2493: copyMakeBorder by (k-1)/2 with 255, cv::erode, crop; copyMakeBorder with 0,
// cv::dilate, crop).  OpenCV's erode / dilate take, at (y, x), the min / max of
// src(y + i - bw, x + j - bw) over the element's non-zero (i, j), bw = (k-1)/2 (the element is
// not reflected for the dilation); pixels outside the image read the padding value.
//
// One CTA computes a 64-row x 128-column output tile.  Pixels are handled four to a 32-bit word
// (byte-wise __vminu4 / __vmaxu4), one word column per lane, eight rows per warp.  The input rows
// the tile needs (64 + 2 bw, with 32 columns of halo on each side) are staged in shared memory
// once, padding values filled in; the word starting at any column offset is one funnel shift of
// two staged words.
//
// Fast path (every element row is one run of columns centred on the middle column: disks,
// rectangles, diamonds): for r = 0, 1, .., the largest run radius, a shared plane holds the
// min (max) over columns x - r .. x + r of every staged row, grown in place from r - 1 by the two
// new columns; after each step, the element rows of radius r fold that plane's rows into the
// per-row accumulators.  Work per output word: about (64 + 2 bw) / 64 x 2 r_max shifts and
// folds for the runs plus one fold per element row, against one per element pixel directly
// (about 23 + 19 against 321 for the 19 x 19 disk).  Other elements take the direct path: one
// fold per element pixel.
#include <string.h>

#include "morph.cuh"

namespace nsgb {

namespace {

constexpr int kTileRows = 64;
constexpr int kTileWords = 32;   // 128 columns
constexpr int kHaloWords = 8;    // 32 columns each side: covers offsets up to 31
constexpr int kRowWords = kTileWords + 2 * kHaloWords;
constexpr int kStageRows = kTileRows + 2 * (kMorphMaxK / 2);
constexpr int kThreads = 256;
constexpr int kRowsPerWarp = kTileRows / (kThreads / 32);

template <bool MAX>
__device__ __forceinline__ uint32_t fold(uint32_t a, uint32_t b) {
  return MAX ? __vmaxu4(a, b) : __vminu4(a, b);
}

// The four pixels starting `s` columns right of word column `cw` of a staged row.
__device__ __forceinline__ uint32_t word_at(const uint32_t* row, int cw, int s) {
  const int pos = 4 * (kHaloWords + cw) + s;
  return __funnelshift_r(row[pos >> 2], row[(pos >> 2) + 1], 8 * (pos & 3));
}

// MAX = false: erosion, padding 255; MAX = true: dilation, padding 0.
template <bool MAX>
__global__ void __launch_bounds__(kThreads) morph_kernel(const uint8_t* __restrict__ in, int64_t pitch_in,
                                                         bool in_words, uint8_t* __restrict__ out,
                                                         int64_t pitch_out, bool out_words, int H, int W,
                                                         const __grid_constant__ MorphElement e) {
  __shared__ uint32_t S[kStageRows][kRowWords];
  __shared__ uint32_t R[kStageRows][kTileWords];
  const uint32_t pad_byte = MAX ? 0u : 255u;
  const uint32_t pad = MAX ? 0u : 0xFFFFFFFFu;
  const int bw = e.bw;
  const int x0 = blockIdx.x * 4 * kTileWords;
  const int rows_in = kTileRows + 2 * bw;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // tile rows stride by the grid's y extent (65535 at most)
  for (int64_t ty = blockIdx.y; ty * kTileRows < H; ty += gridDim.y) {
    const int y0 = (int)(ty * kTileRows);
    for (int idx = threadIdx.x; idx < rows_in * kRowWords; idx += kThreads) {
      const int i = idx / kRowWords, wd = idx - i * kRowWords;
      const int y = y0 - bw + i;
      const int xb = x0 + 4 * (wd - kHaloWords);
      uint32_t v = pad;
      if (y >= 0 && y < H) {
        const uint8_t* row = in + (int64_t)y * pitch_in;
        if (in_words && xb >= 0 && xb + 4 <= W) {
          v = __ldg((const uint32_t*)(row + xb));
        } else if (xb + 4 > 0 && xb < W) {
          v = 0;
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int x = xb + b;
            v |= (x >= 0 && x < W ? (uint32_t)__ldg(row + x) : pad_byte) << (8 * b);
          }
        }
      }
      S[i][wd] = v;
    }
    __syncthreads();

    uint32_t acc[kRowsPerWarp];
#pragma unroll
    for (int j = 0; j < kRowsPerWarp; ++j) acc[j] = pad;
    const int j0 = warp * kRowsPerWarp;  // this warp's first output row in the tile

    if (e.centred) {
      for (int i = warp; i < rows_in; i += kThreads / 32) R[i][lane] = S[i][kHaloWords + lane];
      __syncthreads();
      for (int r = 0; r <= e.max_radius; ++r) {
        if (r > 0) {
          for (int i = warp; i < rows_in; i += kThreads / 32)
            R[i][lane] = fold<MAX>(R[i][lane], fold<MAX>(word_at(S[i], lane, -r), word_at(S[i], lane, r)));
          __syncthreads();
        }
        for (uint64_t m = e.dy_of_radius[r]; m; m &= m - 1) {
          const int kr = __ffsll((long long)m) - 1;  // element row: tile row j reads staged row j + kr
#pragma unroll
          for (int j = 0; j < kRowsPerWarp; ++j) acc[j] = fold<MAX>(acc[j], R[j0 + j + kr][lane]);
        }
        __syncthreads();
      }
    } else {
      for (int kr = 0; kr < e.k; ++kr) {
        const uint64_t bits = e.row_bits[kr];
        if (!bits) continue;
#pragma unroll
        for (int j = 0; j < kRowsPerWarp; ++j) {
          const uint32_t* row = S[j0 + j + kr];
          for (uint64_t m = bits; m; m &= m - 1)
            acc[j] = fold<MAX>(acc[j], word_at(row, lane, __ffsll((long long)m) - 1 - bw));
        }
      }
    }

    const int xb = x0 + 4 * lane;
#pragma unroll
    for (int j = 0; j < kRowsPerWarp; ++j) {
      const int y = y0 + j0 + j;
      if (y >= H || xb >= W) break;
      uint8_t* o = out + (int64_t)y * pitch_out + xb;
      if (out_words && xb + 4 <= W) {
        *(uint32_t*)o = acc[j];
      } else {
        for (int b = 0; b < 4 && xb + b < W; ++b) o[b] = (uint8_t)(acc[j] >> (8 * b));
      }
    }
    __syncthreads();  // the next tile restages S
  }
}

bool words_ok(const void* p, int64_t pitch) { return ((uintptr_t)p % 4) == 0 && pitch % 4 == 0; }

}  // namespace

bool morph_element(const uint8_t* kernel, int k, MorphElement* e) {
  if (!kernel || !e || k < 3 || k > kMorphMaxK || k % 2 == 0) return false;
  memset(e, 0, sizeof(*e));
  e->k = k;
  e->bw = (k - 1) / 2;
  e->centred = 1;
  e->max_radius = 0;
  bool any = false;
  for (int i = 0; i < k; ++i) {
    uint64_t bits = 0;
    for (int j = 0; j < k; ++j)
      if (kernel[i * k + j]) bits |= 1ull << j;
    e->row_bits[i] = bits;
    e->radius[i] = -1;
    if (!bits) continue;
    any = true;
    const int lo = __builtin_ctzll(bits), hi = 63 - __builtin_clzll(bits);
    const bool run = __builtin_popcountll(bits) == hi - lo + 1;
    if (run && lo + hi == 2 * e->bw) {
      const int r = e->bw - lo;
      e->radius[i] = (int8_t)r;
      e->dy_of_radius[r] |= 1ull << i;
      if (r > e->max_radius) e->max_radius = r;
    } else {
      e->centred = 0;
    }
  }
  return any;
}

cudaError_t morph_open_launch(const uint8_t* in, int64_t pitch_in, uint8_t* out, int64_t pitch_out, int rows,
                              int cols, const MorphElement& e, uint8_t* tmp, cudaStream_t s) {
  const int64_t pitch_tmp = ((int64_t)cols + 127) & ~(int64_t)127;
  const int tiles_y = (rows + kTileRows - 1) / kTileRows;
  const dim3 grid((cols + 4 * kTileWords - 1) / (4 * kTileWords), tiles_y < 65535 ? tiles_y : 65535);
  morph_kernel<false><<<grid, kThreads, 0, s>>>(in, pitch_in, words_ok(in, pitch_in), tmp, pitch_tmp, true, rows,
                                                cols, e);
  morph_kernel<true><<<grid, kThreads, 0, s>>>(tmp, pitch_tmp, true, out, pitch_out, words_ok(out, pitch_out), rows,
                                               cols, e);
  return cudaGetLastError();
}

size_t morph_open_workspace_bytes(int64_t rows, int64_t cols) {
  return 256 + (size_t)rows * (size_t)(((cols + 127) / 128) * 128);
}

}  // namespace nsgb
