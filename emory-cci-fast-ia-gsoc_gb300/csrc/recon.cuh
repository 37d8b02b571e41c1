// Internal interface of the reconstruction kernels (recon.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace nsgb {

// Workspace bytes for a reconstruction of an H x W image of `dtype`.
size_t recon_workspace_bytes(int dtype, int64_t H, int64_t W);

// Enqueues the reconstruction of `marker` under `mask` into `out` (out may equal marker;
// otherwise the marker is first copied into out).  max_visits caps tile visits in units of the
// tile count.
// erode: order-reversed (dual) operator.  ring: apply the reference's 0-valued padding ring
// (only meaningful for signed / float dilation).  Status words live at the start of `ws`.
cudaError_t recon_launch(int dtype, void* out, const void* marker, const void* mask, int64_t H, int64_t W,
                         int64_t pitch, int conn, bool erode, bool ring, void* ws, cudaStream_t s, int max_visits,
                         int max_iters);

}  // namespace nsgb
