// Flat grayscale erosion / dilation and the opening built from them (internal interface of
// csrc/morph.cu).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace nsgb {

constexpr int kMorphMaxK = 63;  // largest structuring element side (half-width 31)

// A k x k structuring element (k odd), as the kernels read it.  Row `i` of the element is the
// image row offset i - bw; `row_bits[i]` bit j = element (i, j) non-zero, column offset j - bw.
// `radius[i]` >= 0 when row i is one run of columns centred on the middle column (bw - r ..
// bw + r), -1 when it is empty; `dy_of_radius[r]` = the rows whose run has radius r.  `centred`:
// every non-empty row is such a run (disks, rectangles, diamonds), which takes the fast path.
struct MorphElement {
  int k, bw, centred, max_radius;
  uint64_t row_bits[kMorphMaxK];
  int8_t radius[kMorphMaxK + 1];
  uint64_t dy_of_radius[kMorphMaxK / 2 + 1];
};

// Builds the element from a host k x k array (non-zero = in the element).  Returns false for an
// even or out-of-range k or an element without a non-zero entry.
bool morph_element(const uint8_t* kernel, int k, MorphElement* e);

// Workspace bytes of the opening: the status word, then the eroded image (rows padded to 128).
size_t morph_open_workspace_bytes(int64_t rows, int64_t cols);

// Opening of a u8 image as nscale::morphOpen<unsigned char> computes it: erosion with the image
// surrounded by 255, then dilation of the eroded image surrounded by 0.  `tmp` holds the eroded
// image (rows x cols, dense).
cudaError_t morph_open_launch(const uint8_t* in, int64_t pitch_in, uint8_t* out, int64_t pitch_out, int rows,
                              int cols, const MorphElement& e, uint8_t* tmp, cudaStream_t s);

}  // namespace nsgb
