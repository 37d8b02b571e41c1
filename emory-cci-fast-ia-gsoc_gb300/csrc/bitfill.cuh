// Binary hole filling on bit planes (one bit per pixel): the border-connected part of the
// "open" pixels, found by a flood from outside the image.  Used by the chain's step (c),
// imfillHoles(binary) of the thresholded reconstruction: the open pixels are the ones that are
// not foreground (R <= thr), the flood marks those connected to the image border, and the
// filled image is 255 wherever the flood did not reach.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "batch.cuh"

namespace nsgb {

// Bit-plane layout of image m: row y, word k (pixels 32k .. 32k+31, bit b = pixel 32k + b) at
// word m.b_base + y * bit_words(m.W) + k, in the open plane and in the flooded plane alike.
__host__ __device__ inline int bit_words(int W) { return (W + 31) / 32; }

// Flood tiles: 32 rows x 32 words (1024 pixels) per warp.
__host__ __device__ inline int flood_tiles_x(int W) { return (bit_words(W) + 31) / 32; }
__host__ __device__ inline int flood_tiles_y(int H) { return (H + 31) / 32; }

// Floods the open plane `open` of every image from outside the image (conn 4 or 8) into
// `flooded` (which must hold zeros on entry).  `ntiles` = total flood tiles; `ws` is a
// reconstruction workspace of at least recon_workspace_bytes_tiles(ntiles) bytes (status word,
// tile states, work ring), shared with the caller's status word.
cudaError_t flood_launch(const Imgs& I, int ntiles, const uint32_t* open, uint32_t* flooded, int conn, void* ws,
                         cudaStream_t s, long long poll_limit);

}  // namespace nsgb
