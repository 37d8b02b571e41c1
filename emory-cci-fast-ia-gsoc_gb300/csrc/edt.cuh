// Euclidean distance transform of a u8 mask (internal interface of csrc/edt.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace nsgb {

// Workspace bytes: the status word, the column distances, the row pass's two stacks and the
// per-chunk zero rows.
size_t edt_workspace_bytes(int64_t rows, int64_t cols);

// out(y, x) = distance from (y, x) to the nearest zero pixel of `mask` (+inf when there is
// none); basins: -distance on non-zero pixels and -FLT_MAX on zero pixels instead.
cudaError_t edt_launch(const uint8_t* mask, int64_t pitch_in, float* out, int64_t pitch_out, int rows, int cols,
                       bool basins, void* ws, cudaStream_t s);

}  // namespace nsgb
