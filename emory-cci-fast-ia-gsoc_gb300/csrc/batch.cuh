// Image tables: every kernel works on a batch of images (a single-image call is a batch of
// one).  Work items of all images (reconstruction tiles, labelling tiles, rank blocks, rows)
// are numbered consecutively; each image records where its range starts.  Tiles find their
// image through a per-tile map; other work items with a binary search over the range starts
// (row kernels look it up once per range of rows).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace nsgb {

struct Img {
  void* plane;        // reconstruction: marker in / result out; labelling: the classified image
  const void* aux;    // reconstruction: mask; bwselect: seeds
  int64_t pitch;      // bytes, for plane and aux
  int H, W;
  int aligned;        // plane / aux aligned for vector tile loads
  int r_tiles_x, r_tiles_y, r_tile_base;  // reconstruction tiles
  int r_stile_base;   // first of its tiles on the half-tile-shifted grid (streaming passes)
  int r_tw;           // reconstruction tile width in pixels (64 for u8/u16, 32 for i32/f32)
  int r_even_base;    // first of its checkerboard colour-0 tiles among all images' colour-0 tiles
  int r_col_base[3];  // the same for the first three colours of the four-colour order
  int c_tiles_x, c_tile_base;             // 32x32 labelling tiles
  int px_base;        // first pixel in the concatenated label planes
  int blk_base;       // first 1024-pixel rank block
  int row_base;       // first row in the concatenated row space
  int b_base;         // first word of its bit planes (hole filling on bits)
  int f_tile_base;    // first of its flood tiles (32 rows x 1024 pixels)
  // outputs of the chain (dense rows, may be null)
  uint8_t* fill;
  int32_t* labels;
  uint8_t* area;
};

struct Imgs {
  const Img* d;  // device table (batches), or null: a single image passed in `one`
  int n;
  Img one;       // the image itself when d == null (kernel parameter, no table needed)
  // Batches: the image of every reconstruction tile and of every labelling tile (written by
  // nsgb_batch_prepare), so that a work item finds its image with one load.  A stack of equal
  // images has no maps; its tiles per image divide the tile index instead.
  const int* r_img;
  const int* c_img;
  int r_per, c_per;  // stack: reconstruction / labelling tiles per image (0: not a stack)
};

__device__ __forceinline__ Img img_at(const Imgs& I, int i) { return I.d ? I.d[i] : I.one; }

// Largest image index whose range start (selected by `field`) is <= key.
template <typename F>
__device__ __forceinline__ int img_of(const Imgs& I, int key, F field) {
  if (!I.d) return 0;
  int lo = 0, hi = I.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (field(I.d[mid]) <= key) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Image of reconstruction tile / labelling tile `t` (tile map, stack division, or the search).
template <typename F>
__device__ __forceinline__ int img_of_tile(const Imgs& I, int t, const int* map, int per, F field) {
  if (!I.d) return 0;
  if (map) return __ldg(map + t);
  if (per > 0) return t / per;
  return img_of(I, t, field);
}

struct RTileBase { __device__ int operator()(const Img& m) const { return m.r_tile_base; } };
struct CTileBase { __device__ int operator()(const Img& m) const { return m.c_tile_base; } };
struct BlkBase { __device__ int operator()(const Img& m) const { return m.blk_base; } };
struct RowBase { __device__ int operator()(const Img& m) const { return m.row_base; } };
struct PxBase { __device__ int operator()(const Img& m) const { return m.px_base; } };
struct FTileBase { __device__ int operator()(const Img& m) const { return m.f_tile_base; } };
struct REvenBase { __device__ int operator()(const Img& m) const { return m.r_even_base; } };
struct ROddBase { __device__ int operator()(const Img& m) const { return m.r_tile_base - m.r_even_base; } };

// Reconstruction tiles of checkerboard colour 0 ((tile row + tile column) even) in an image.
__host__ __device__ inline int even_tiles(int tiles_x, int tiles_y) {
  return ((tiles_y + 1) / 2) * ((tiles_x + 1) / 2) + (tiles_y / 2) * (tiles_x / 2);
}

// Four-colour order: colour c = 0..3 is (tile row parity, tile column parity) = (0,0), (1,1),
// (0,1), (1,0); tiles of colour c in an image.
__host__ __device__ inline int colour_tiles(int tiles_x, int tiles_y, int c) {
  const int py = (c == 1 || c == 3) ? 1 : 0, px = (c == 1 || c == 2) ? 1 : 0;
  return ((tiles_y - py + 1) / 2) * ((tiles_x - px + 1) / 2);
}

// Start of an image's colour-c tiles among all images' colour-c tiles (four-colour order).
struct RColBase {
  int c;
  __device__ int operator()(const Img& m) const {
    return c < 3 ? m.r_col_base[c] : m.r_tile_base - m.r_col_base[0] - m.r_col_base[1] - m.r_col_base[2];
  }
};

// Totals of a batch, known on the host (grid sizes).
struct BatchTotals {
  int n;
  int64_t px;      // total pixels (< 2^31)
  int64_t b_words; // words of one bit plane over all images (rows x ceil(cols / 32))
  int f_tiles;     // flood tiles
  int r_tiles;     // reconstruction tiles
  int r_stiles;    // reconstruction tiles of the half-tile-shifted grid
  int r_even;      // reconstruction tiles of checkerboard colour 0
  int r_col[3];    // reconstruction tiles of the first three colours of the four-colour order
  int c_tiles;     // labelling tiles
  int blocks;      // rank blocks
  int rows;        // total rows
  int max_w;       // widest image
  int perimeter_max;  // largest 2*(H+W)
};

}  // namespace nsgb
