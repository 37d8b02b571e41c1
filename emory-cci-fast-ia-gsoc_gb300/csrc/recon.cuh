// Internal interface of the reconstruction kernels (recon.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "batch.cuh"

namespace nsgb {

// Reconstruction tile grid of an image (tiles are 32 rows x 32 packed words).
int recon_tiles_x(int dtype, int64_t W);
int recon_tiles_y(int64_t H);
// Tiles of the half-tile-shifted grid that the streaming passes alternate with.
int recon_stiles(int dtype, int64_t H, int64_t W);
size_t recon_workspace_bytes_tiles(int64_t ntiles);
// An image descriptor for reconstruction (tile bases left at 0).
Img recon_image(int dtype, void* plane, const void* mask, int64_t H, int64_t W, int64_t pitch);
// Reconstructs every image of the batch in place (Img::plane holds the marker, Img::aux the
// mask) in one persistent launch over all their tiles.  resweeps: how often a tile marked
// dirty while it ran is swept again at once from its registers (after a halo reload) instead
// of being queued again -- worth it for front-like propagation such as hole filling.
// poll_limit: polls of a queue wait before it reports NSGB_ERR_TIMEOUT (0 = kSpinLimit).
// passes: streaming passes before the queue (> 0 that many, < 0 none, 0 the tuned default);
// nstiles / total_px: shifted-grid tiles and pixels of all images (batches; computed for a
// single image); order: initial ring order + 1 (0 the tuned default).
cudaError_t recon_launch_batch(int dtype, const Imgs& I, int ntiles, int conn, bool erode, bool ring, void* ws,
                               cudaStream_t s, int max_visits, int max_iters, int resweeps = 0,
                               long long poll_limit = 0, int passes = 0, int nstiles = 0, int order = 0,
                               long long total_px = 0, int ctas = 0);

// Workspace bytes for a reconstruction of an H x W image of `dtype`.
size_t recon_workspace_bytes(int dtype, int64_t H, int64_t W);

// Enqueues the reconstruction of `marker` under `mask` into `out` (out may equal marker;
// otherwise the marker is first copied into out).  max_visits caps tile visits in units of the
// tile count.
// erode: order-reversed (dual) operator.  ring: apply the reference's 0-valued padding ring
// (only meaningful for signed / float dilation).  Status words live at the start of `ws`.
cudaError_t recon_launch(int dtype, void* out, const void* marker, const void* mask, int64_t H, int64_t W,
                         int64_t pitch, int conn, bool erode, bool ring, void* ws, cudaStream_t s, int max_visits,
                         int max_iters, long long poll_limit = 0, int passes = 0, int order = 0, int ctas = 0);

}  // namespace nsgb
