// Per-label bounding boxes of an int32 label image (internal interface of csrc/bbox.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include "batch.cuh"

namespace nsgb {

// Workspace bytes for an image of `px` pixels (status word first, as in every workspace).
size_t bbox_workspace_bytes(int64_t px);

// Boxes of a single image I (Img::plane = int32 labels, Img::pitch) into `boxes` (five arrays of
// stride `cap`); `count_dev` (device, optional) receives the number of labels present.
cudaError_t bbox_launch(const Imgs& I, const BatchTotals& t, int32_t bgval, void* ws, int32_t* boxes, int64_t cap,
                        int32_t* count_dev, cudaStream_t s);

}  // namespace nsgb
