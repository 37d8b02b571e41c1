// C++ host interface mirroring the reference's nscale:: / nscale::gpu:: morphology API
// (fastIA-master/src/segment/MorphologicOperations.h:21-190) on top of the C ABI (nsgb.h).
//
// OpenCV is not required: a minimal header-only stand-in provides the members of cv::Mat,
// cv::gpu::GpuMat and cv::gpu::Stream that the reference's call sites use (rows, cols,
// step, type(), data, ptr<T>(), create, upload / download, empty).  Where real OpenCV 2.x
// is available, define NSGB_USE_OPENCV before including this header and the functions bind
// to cv::Mat / cv::gpu::GpuMat directly (same member names).
//
// Behaviour mirrors the reference:
//   * results are new images (the inputs are not modified);
//   * bad channel counts / types raise cv::Exception (the reference's CV_Assert);
//   * calls block until the GPU work is done (the reference synchronises its streams);
//   * the nscale:: (CPU-signature) functions take host cv::Mat and run on the GPU -- there is
//     no CPU code path in this library.
// Unlike the C ABI, this layer allocates device memory (results and a cached workspace per
// device), as cv::gpu::GpuMat does.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "nsgb.h"

#ifndef NSGB_USE_OPENCV
// OpenCV's depth / type constants (macros at global scope, as OpenCV defines them; single
// channel types equal their depth).
#ifndef CV_8U
#define CV_8U 0
#define CV_8S 1
#define CV_16U 2
#define CV_16S 3
#define CV_32S 4
#define CV_32F 5
#define CV_64F 6
#define CV_8UC1 CV_8U
#define CV_16UC1 CV_16U
#define CV_32SC1 CV_32S
#define CV_32FC1 CV_32F
#endif

namespace cv {

struct Exception : public std::runtime_error {
  int code;
  Exception(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

#define NSGB_CV_ASSERT(expr)                                                     \
  do {                                                                           \
    if (!(expr)) throw ::cv::Exception(-215, std::string("Assertion failed: ") + #expr); \
  } while (0)

inline size_t elem_size_of(int type) {
  switch (type) {
    case CV_8U: case CV_8S: return 1;
    case CV_16U: case CV_16S: return 2;
    case CV_32S: case CV_32F: return 4;
    case CV_64F: return 8;
    default: return 0;
  }
}

// Host image (single channel, row-major, owning or borrowed storage).
class Mat {
 public:
  int rows = 0, cols = 0;
  size_t step = 0;  // bytes per row
  unsigned char* data = nullptr;

  Mat() = default;
  Mat(int r, int c, int t) { create(r, c, t); }
  Mat(int r, int c, int t, void* ext, size_t st = 0) : rows(r), cols(c), step(st ? st : c * elem_size_of(t)),
                                                      data((unsigned char*)ext), type_(t) {}
  void create(int r, int c, int t) {
    rows = r;
    cols = c;
    type_ = t;
    step = (size_t)c * elem_size_of(t);
    store_ = std::make_shared<std::vector<unsigned char>>(step * (size_t)r);
    data = store_->data();
  }
  int type() const { return type_; }
  int depth() const { return type_; }
  int channels() const { return 1; }
  bool empty() const { return data == nullptr || rows == 0 || cols == 0; }
  size_t elemSize() const { return elem_size_of(type_); }
  template <typename T>
  T* ptr(int y = 0) { return (T*)(data + (size_t)y * step); }
  template <typename T>
  const T* ptr(int y = 0) const { return (const T*)(data + (size_t)y * step); }

 private:
  int type_ = CV_8U;
  std::shared_ptr<std::vector<unsigned char>> store_;
};

namespace gpu {

class Stream {
 public:
  Stream() = default;
  explicit Stream(cudaStream_t s) : s_(s) {}
  static Stream& Null() {
    static Stream z;
    return z;
  }
  cudaStream_t raw() const { return s_; }
  void waitForCompletion() const { cudaStreamSynchronize(s_); }

 private:
  cudaStream_t s_ = nullptr;
};

// Device image; storage is continuous (step == cols * elemSize), as createContinuous gives.
class GpuMat {
 public:
  int rows = 0, cols = 0;
  size_t step = 0;
  unsigned char* data = nullptr;

  GpuMat() = default;
  GpuMat(int r, int c, int t) { create(r, c, t); }
  explicit GpuMat(const Mat& m) { upload(m); }
  void create(int r, int c, int t) {
    if (r == rows && c == cols && t == type_ && data) return;
    rows = r;
    cols = c;
    type_ = t;
    step = (size_t)c * elem_size_of(t);
    void* p = nullptr;
    if (cudaMalloc(&p, step * (size_t)r) != cudaSuccess) throw Exception(-217, "cudaMalloc failed");
    store_ = std::shared_ptr<unsigned char>((unsigned char*)p, [](unsigned char* q) { cudaFree(q); });
    data = store_.get();
  }
  void release() {
    store_.reset();
    data = nullptr;
    rows = cols = 0;
  }
  void upload(const Mat& m) {
    create(m.rows, m.cols, m.type());
    if (cudaMemcpy2D(data, step, m.data, m.step, step, rows, cudaMemcpyHostToDevice) != cudaSuccess)
      throw Exception(-217, "upload failed");
  }
  void download(Mat& m) const {
    m.create(rows, cols, type_);
    if (cudaMemcpy2D(m.data, m.step, data, step, step, rows, cudaMemcpyDeviceToHost) != cudaSuccess)
      throw Exception(-217, "download failed");
  }
  int type() const { return type_; }
  int depth() const { return type_; }
  int channels() const { return 1; }
  bool empty() const { return data == nullptr; }
  bool isContinuous() const { return true; }
  size_t elemSize() const { return elem_size_of(type_); }
  GpuMat clone() const {
    GpuMat g(rows, cols, type_);
    cudaMemcpy(g.data, data, step * (size_t)rows, cudaMemcpyDeviceToDevice);
    return g;
  }
  template <typename T>
  T* ptr(int y = 0) { return (T*)(data + (size_t)y * step); }

 private:
  int type_ = CV_8U;
  std::shared_ptr<unsigned char> store_;
};

}  // namespace gpu
}  // namespace cv
#else
#define NSGB_CV_ASSERT(expr) CV_Assert(expr)
#endif

namespace nscale {

namespace detail {

template <typename T>
struct DType;
template <> struct DType<unsigned char> { static constexpr int code = NSGB_U8; static constexpr int cv = CV_8U; };
template <> struct DType<unsigned short> { static constexpr int code = NSGB_U16; static constexpr int cv = CV_16U; };
template <> struct DType<int> { static constexpr int code = NSGB_I32; static constexpr int cv = CV_32S; };
template <> struct DType<float> { static constexpr int code = NSGB_F32; static constexpr int cv = CV_32F; };

inline void check(nsgb_status st, const char* where) {
  if (st != NSGB_OK) throw cv::Exception(-(int)st, std::string(where) + ": " + nsgb_status_string(st));
}

// Device workspace cached per (device, stream) and grown on demand, so calls on different
// streams never share one.  A buffer is replaced only after the device has finished all work
// queued so far (cudaDeviceSynchronize), since a kernel of an earlier call may still use it.
inline void* workspace(size_t bytes, cudaStream_t stream) {
  static std::mutex mu;
  static std::map<std::pair<int, cudaStream_t>, std::pair<void*, size_t>> cache;
  std::lock_guard<std::mutex> lock(mu);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) throw cv::Exception(-217, "cudaGetDevice failed");
  auto& e = cache[{dev, stream}];
  if (e.second < bytes) {
    if (e.first) {
      if (cudaDeviceSynchronize() != cudaSuccess) throw cv::Exception(-217, "cudaDeviceSynchronize failed");
      cudaFree(e.first);
      e = {nullptr, 0};
    }
    void* p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) throw cv::Exception(-217, "workspace cudaMalloc failed");
    e = {p, bytes};
  }
  return e.first;
}

inline nsgb_stream_t raw(cv::gpu::Stream& s) { return (nsgb_stream_t)s.raw(); }
inline void* workspace(size_t bytes, cv::gpu::Stream& s) { return workspace(bytes, (cudaStream_t)s.raw()); }

}  // namespace detail

namespace gpu {
using cv::gpu::GpuMat;
using cv::gpu::Stream;

// nscale::gpu::imreconstruct<T> (MorphologicOperations.h:102-119).  `iter` receives the
// number of tile visits the reconstruction used (the reference reported scan iterations).
template <typename T>
GpuMat imreconstruct(const GpuMat& seeds, const GpuMat& image, int connectivity, Stream& stream, unsigned int& iter) {
  NSGB_CV_ASSERT(image.channels() == 1 && seeds.channels() == 1);
  NSGB_CV_ASSERT(image.type() == detail::DType<T>::cv && seeds.type() == image.type());
  NSGB_CV_ASSERT(image.rows == seeds.rows && image.cols == seeds.cols);
  GpuMat out = seeds.clone();
  const size_t nb = nsgb_workspace_size(NSGB_OP_IMRECONSTRUCT, detail::DType<T>::code, image.rows, image.cols);
  void* ws = detail::workspace(nb, stream);
  detail::check(nsgb_imreconstruct(detail::DType<T>::code, out.data, image.data, image.rows, image.cols,
                                   (int64_t)image.step, connectivity, 0, ws, nb, detail::raw(stream), nullptr),
                "imreconstruct");
  // the workspace header holds {status, visits}: read it on the call's stream
  int hdr[2] = {0, 0};
  if (cudaMemcpyAsync(hdr, ws, sizeof(hdr), cudaMemcpyDeviceToHost, (cudaStream_t)stream.raw()) != cudaSuccess ||
      cudaStreamSynchronize((cudaStream_t)stream.raw()) != cudaSuccess)
    throw cv::Exception(-217, "imreconstruct: reading the visit count failed");
  iter = (unsigned)hdr[1];
  return out;
}

template <typename T>
GpuMat imreconstruct(const GpuMat& seeds, const GpuMat& image, int connectivity, Stream& stream) {
  unsigned int iter;
  return imreconstruct<T>(seeds, image, connectivity, stream, iter);
}

// The reference's queue variants (MorphologicOperations.h:105-116) compute the same
// reconstruction; their tuning arguments (first-pass count, block count, queue factor)
// have no meaning for this implementation and are accepted for source compatibility.
template <typename T>
GpuMat imreconstructQueue(const GpuMat& seeds, const GpuMat& image, int connectivity, Stream& stream) {
  return imreconstruct<T>(seeds, image, connectivity, stream);
}
template <typename T>
GpuMat imreconstructBinary(const GpuMat& seeds, const GpuMat& binaryImage, int connectivity, Stream& stream);
// binary = true is the reference's binary first pass (imreconstructBinaryCallerBuildQueue,
// MorphologicOperationsGPU.cpp:319-323), which keeps the marker where the mask is 0 as
// imreconstructBinary does: it maps to the binary reconstruction.
template <typename T>
GpuMat imreconstructQueueSpeedup(GpuMat& seeds, GpuMat& image, int connectivity, int /*nItFirstPass*/,
                                 Stream& stream, int /*nBlocks*/ = 14, bool binary = false) {
  if (binary) return imreconstructBinary<T>(seeds, image, connectivity, stream);
  return imreconstruct<T>(seeds, image, connectivity, stream);
}
inline GpuMat imreconstructQueueSpeedupFloat(GpuMat& seeds, GpuMat& image, int connectivity, int /*nItFirstPass*/,
                                             Stream& stream, int /*nBlocks*/ = 14) {
  return imreconstruct<float>(seeds, image, connectivity, stream);
}
template <typename T>
GpuMat imreconstructQ(const GpuMat& seeds, const GpuMat& image, int connectivity, Stream& stream) {
  return imreconstruct<T>(seeds, image, connectivity, stream);
}
// nscale::gpu::imreconstructQueueThroughput<T> (MorphologicOperationsGPU.cpp:447-545): all
// images in one batched launch (nsgb_batch_prepare + nsgb_imreconstruct_batch).
template <typename T>
std::vector<GpuMat> imreconstructQueueThroughput(std::vector<GpuMat>& seeds, std::vector<GpuMat>& image,
                                                 int connectivity, int /*nItFirstPass*/, Stream& stream) {
  NSGB_CV_ASSERT(seeds.size() == image.size());
  std::vector<GpuMat> out;
  if (seeds.empty()) return out;
  std::vector<nsgb_tile> tiles(seeds.size());
  out.reserve(seeds.size());
  for (size_t i = 0; i < seeds.size(); ++i) {
    NSGB_CV_ASSERT(image[i].type() == detail::DType<T>::cv && seeds[i].type() == image[i].type());
    NSGB_CV_ASSERT(image[i].rows == seeds[i].rows && image[i].cols == seeds[i].cols && image[i].step == seeds[i].step);
    out.push_back(seeds[i].clone());
    tiles[i] = nsgb_tile{out[i].data, image[i].data, image[i].rows, image[i].cols, (int64_t)image[i].step,
                         nullptr, nullptr, nullptr};
  }
  const size_t nb = nsgb_batch_workspace_size(detail::DType<T>::code, tiles.data(), (int)tiles.size());
  NSGB_CV_ASSERT(nb > 0);
  nsgb_batch batch;
  detail::check(nsgb_batch_prepare(detail::DType<T>::code, tiles.data(), (int)tiles.size(), detail::workspace(nb, stream), nb,
                                   &batch),
                "imreconstructQueueThroughput");
  detail::check(nsgb_imreconstruct_batch(&batch, connectivity, 0, detail::raw(stream), nullptr),
                "imreconstructQueueThroughput");
  return out;
}

// nscale::gpu::imreconstructBinary<T> (MorphologicOperations.h:121-129).
template <typename T>
GpuMat imreconstructBinary(const GpuMat& seeds, const GpuMat& binaryImage, int connectivity, Stream& stream) {
  NSGB_CV_ASSERT(binaryImage.channels() == 1 && seeds.channels() == 1);
  NSGB_CV_ASSERT(binaryImage.type() == detail::DType<T>::cv && seeds.type() == binaryImage.type());
  GpuMat out = seeds.clone();
  const size_t nb =
      nsgb_workspace_size(NSGB_OP_IMRECONSTRUCT_BINARY, detail::DType<T>::code, binaryImage.rows, binaryImage.cols);
  detail::check(nsgb_imreconstruct_binary(detail::DType<T>::code, out.data, binaryImage.data, binaryImage.rows,
                                          binaryImage.cols, (int64_t)binaryImage.step, connectivity,
                                          detail::workspace(nb, stream), nb, detail::raw(stream), nullptr),
                "imreconstructBinary");
  return out;
}
template <typename T>
GpuMat imreconstructBinary(const GpuMat& seeds, const GpuMat& binaryImage, int connectivity, Stream& stream,
                           unsigned int& iter) {
  iter = 1;
  return imreconstructBinary<T>(seeds, binaryImage, connectivity, stream);
}

// nscale::gpu::imfillHoles<T> (MorphologicOperations.h:147).
template <typename T>
GpuMat imfillHoles(const GpuMat& image, bool binary, int connectivity, Stream& stream) {
  NSGB_CV_ASSERT(image.channels() == 1 && image.type() == detail::DType<T>::cv);
  GpuMat out(image.rows, image.cols, image.type());
  const size_t nb = nsgb_workspace_size(NSGB_OP_FILL_HOLES, detail::DType<T>::code, image.rows, image.cols);
  detail::check(nsgb_imfill_holes(detail::DType<T>::code, image.data, out.data, image.rows, image.cols,
                                  (int64_t)image.step, binary ? 1 : 0, connectivity, detail::workspace(nb, stream), nb,
                                  detail::raw(stream), nullptr),
                "imfillHoles");
  return out;
}

// nscale::gpu::bwselect<T> (MorphologicOperations.h:152).
template <typename T>
GpuMat bwselect(const GpuMat& binaryImage, const GpuMat& seeds, int connectivity, Stream& stream) {
  NSGB_CV_ASSERT(binaryImage.channels() == 1 && seeds.channels() == 1);
  NSGB_CV_ASSERT(binaryImage.type() == detail::DType<T>::cv && seeds.type() == binaryImage.type());
  GpuMat out(binaryImage.rows, binaryImage.cols, binaryImage.type());
  const size_t nb = nsgb_workspace_size(NSGB_OP_BWSELECT, detail::DType<T>::code, binaryImage.rows, binaryImage.cols);
  detail::check(nsgb_bwselect(detail::DType<T>::code, binaryImage.data, seeds.data, out.data, binaryImage.rows,
                              binaryImage.cols, (int64_t)binaryImage.step, connectivity, detail::workspace(nb, stream), nb,
                              detail::raw(stream), nullptr),
                "bwselect");
  return out;
}

// nscale::gpu::bwlabel (MorphologicOperations.h:154).  int32 labels.
inline GpuMat bwlabel(const GpuMat& binaryImage, int connectivity, bool relab, Stream& stream) {
  NSGB_CV_ASSERT(binaryImage.channels() == 1 && binaryImage.type() == CV_8U);
  GpuMat out(binaryImage.rows, binaryImage.cols, CV_32S);
  const size_t nb = nsgb_workspace_size(NSGB_OP_BWLABEL, NSGB_U8, binaryImage.rows, binaryImage.cols);
  detail::check(nsgb_bwlabel(binaryImage.data, (int32_t*)out.data, binaryImage.rows, binaryImage.cols,
                             (int64_t)binaryImage.step, (int64_t)out.step, connectivity, relab ? 1 : 0, nullptr,
                             detail::workspace(nb, stream), nb, detail::raw(stream), nullptr),
                "bwlabel");
  return out;
}

// nscale::gpu::bwareaopen2 / bwareaopen (MorphologicOperations.h:168-169): [minSize, maxSize).
inline GpuMat bwareaopen2(const GpuMat& binaryImage, bool labeled, bool flatten, int minSize, int maxSize,
                          int connectivity, int& count, Stream& stream) {
  NSGB_CV_ASSERT(binaryImage.channels() == 1);
  NSGB_CV_ASSERT(binaryImage.type() == (labeled ? CV_32S : CV_8U));
  GpuMat out(binaryImage.rows, binaryImage.cols, flatten ? CV_8U : CV_32S);
  const size_t nb = nsgb_workspace_size(NSGB_OP_BWAREAOPEN, NSGB_U8, binaryImage.rows, binaryImage.cols);
  int32_t c = 0;
  detail::check(nsgb_bwareaopen(binaryImage.data, labeled ? 1 : 0, flatten ? nullptr : (int32_t*)out.data,
                                flatten ? out.data : nullptr, binaryImage.rows, binaryImage.cols,
                                (int64_t)binaryImage.step, (int64_t)out.step, (int64_t)out.step, minSize, maxSize,
                                connectivity, &c, detail::workspace(nb, stream), nb, detail::raw(stream), nullptr),
                "bwareaopen2");
  count = c;
  return out;
}
inline GpuMat bwareaopen(const GpuMat& binaryImage, bool labeled, bool flatten, int minSize, int maxSize,
                         int connectivity, int& count, Stream& stream) {
  return bwareaopen2(binaryImage, labeled, flatten, minSize, maxSize, connectivity, count, stream);
}

// nscale::gpu::boundingBox2 (cuda/ccl_uf.cuh:16, used at HistologicalEntitiesGPU.cpp:825):
// per-label boxes of a device int32 label image (w x h, dense rows), returned as a device array
// of 5 * compcount ints (labels, then min x, max x, min y, max y, each compcount long) that the
// caller frees with cudaFree, as with the reference.  Entries follow the raster order of each
// label's first pixel (ConnComponents::boundingBox, ConnComponents.cpp:241-284).
inline int* boundingBox2(const int w, const int h, int* d_label, int bgval, int& compcount, cudaStream_t stream) {
  const size_t nb = nsgb_workspace_size(NSGB_OP_BOUNDING_BOX, NSGB_I32, h, w);
  const int64_t cap = (int64_t)w * h;
  int32_t* tmp = nullptr;
  if (cudaMalloc(&tmp, sizeof(int32_t) * 5 * (size_t)(cap > 0 ? cap : 1)) != cudaSuccess)
    throw cv::Exception(-217, "boundingBox2: cudaMalloc failed");
  int32_t c = 0;
  const nsgb_status st = nsgb_bounding_boxes(d_label, h, w, (int64_t)w * 4, bgval, tmp, cap, &c, nullptr,
                                             detail::workspace(nb, stream), nb, (nsgb_stream_t)stream, nullptr);
  if (st != NSGB_OK) {
    cudaFree(tmp);
    detail::check(st, "boundingBox2");
  }
  int* out = nullptr;
  if (cudaMalloc(&out, sizeof(int) * 5 * (size_t)(c > 0 ? c : 1)) != cudaSuccess) {
    cudaFree(tmp);
    throw cv::Exception(-217, "boundingBox2: cudaMalloc failed");
  }
  if (c > 0 && (cudaMemcpy2DAsync(out, sizeof(int) * (size_t)c, tmp, sizeof(int) * (size_t)cap,
                                  sizeof(int) * (size_t)c, 5, cudaMemcpyDeviceToDevice, stream) != cudaSuccess ||
                cudaStreamSynchronize(stream) != cudaSuccess)) {
    cudaFree(tmp);
    cudaFree(out);
    throw cv::Exception(-217, "boundingBox2: copy failed");
  }
  cudaFree(tmp);
  compcount = c;
  return out;
}

// nscale::gpu::imhmin<T> (MorphologicOperations.h:172).
template <typename T>
GpuMat imhmin(const GpuMat& image, T h, int connectivity, Stream& stream) {
  NSGB_CV_ASSERT(image.channels() == 1 && image.type() == detail::DType<T>::cv);
  GpuMat out(image.rows, image.cols, image.type());
  const size_t nb = nsgb_workspace_size(NSGB_OP_HMIN, detail::DType<T>::code, image.rows, image.cols);
  detail::check(nsgb_imhmin(detail::DType<T>::code, image.data, out.data, image.rows, image.cols, (int64_t)image.step,
                            (double)h, connectivity, detail::workspace(nb, stream), nb, detail::raw(stream), nullptr),
                "imhmin");
  return out;
}

// nscale::gpu::morphOpen<T> (MorphologicOperations.h:182, MorphologicOperationsGPU.cpp:1308),
// with the CPU version's borders (255 around the erosion, 0 around the dilation).  `kernel`: a
// host CV_8UC1 k x k element, k odd; the reference instantiates unsigned char only.
template <typename T>
GpuMat morphOpen(const GpuMat& image, const cv::Mat& kernel, Stream& stream) {
  static_assert(sizeof(T) == 1, "morphOpen: the reference instantiates unsigned char only");
  NSGB_CV_ASSERT(image.channels() == 1 && image.type() == CV_8UC1);
  NSGB_CV_ASSERT(kernel.rows == kernel.cols && kernel.rows > 1 && kernel.rows % 2 == 1 && kernel.type() == CV_8UC1);
  std::vector<unsigned char> k((size_t)kernel.rows * kernel.cols);
  for (int i = 0; i < kernel.rows; ++i)
    std::memcpy(&k[(size_t)i * kernel.cols], kernel.ptr<unsigned char>(i), (size_t)kernel.cols);
  GpuMat out(image.rows, image.cols, image.type());
  const size_t nb = nsgb_workspace_size(NSGB_OP_MORPH_OPEN, NSGB_U8, image.rows, image.cols);
  detail::check(nsgb_morph_open(image.data, out.data, image.rows, image.cols, (int64_t)image.step,
                                (int64_t)out.step, k.data(), kernel.rows, detail::workspace(nb, stream), nb,
                                detail::raw(stream), nullptr),
                "morphOpen");
  return out;
}

// nscale::gpu::distanceTransform (MorphologicOperations.h:188): CV_32FC1 distance to the nearest
// zero pixel of a CV_8UC1 mask, exact (the reference's queue propagation can overshoot; see
// nsgb.h).  Only the distance map (calcDist = true) is provided; the tiling arguments are
// accepted and ignored.
inline GpuMat distanceTransform(const GpuMat& mask, Stream& stream, bool calcDist = true, int /*tIdX*/ = 0,
                                int /*tIdY*/ = 0, int /*tileSize*/ = 0, int /*imgCols*/ = 0) {
  NSGB_CV_ASSERT(mask.channels() == 1 && mask.type() == CV_8UC1);
  NSGB_CV_ASSERT(calcDist);
  GpuMat out(mask.rows, mask.cols, CV_32FC1);
  const size_t nb = nsgb_workspace_size(NSGB_OP_DISTANCE, NSGB_U8, mask.rows, mask.cols);
  detail::check(nsgb_distance_transform(mask.data, (float*)out.data, mask.rows, mask.cols, (int64_t)mask.step,
                                        (int64_t)out.step, 0, detail::workspace(nb, stream), nb, detail::raw(stream), nullptr),
                "distanceTransform");
  return out;
}

}  // namespace gpu

// ---- nscale:: (host cv::Mat signatures, MorphologicOperations.h:21-94), run on the GPU ----
namespace detail {
template <typename F>
cv::Mat via_gpu(const cv::Mat& a, F&& f) {
  cv::gpu::GpuMat g(a);
  cv::gpu::GpuMat r = f(g);
  cv::Mat out;
  r.download(out);
  return out;
}
}  // namespace detail

template <typename T>
cv::Mat imreconstruct(const cv::Mat& seeds, const cv::Mat& image, int connectivity) {
  cv::gpu::GpuMat s(seeds), m(image);
  cv::Mat out;
  gpu::imreconstruct<T>(s, m, connectivity, cv::gpu::Stream::Null()).download(out);
  return out;
}
template <typename T>
cv::Mat imreconstructBinary(const cv::Mat& seeds, const cv::Mat& binaryImage, int connectivity) {
  cv::gpu::GpuMat s(seeds), m(binaryImage);
  cv::Mat out;
  gpu::imreconstructBinary<T>(s, m, connectivity, cv::gpu::Stream::Null()).download(out);
  return out;
}
template <typename T>
cv::Mat imfillHoles(const cv::Mat& image, bool binary, int connectivity) {
  return detail::via_gpu(image, [&](cv::gpu::GpuMat& g) {
    return gpu::imfillHoles<T>(g, binary, connectivity, cv::gpu::Stream::Null());
  });
}
template <typename T>
cv::Mat bwselect(const cv::Mat& binaryImage, const cv::Mat& seeds, int connectivity) {
  cv::gpu::GpuMat b(binaryImage), s(seeds);
  cv::Mat out;
  gpu::bwselect<T>(b, s, connectivity, cv::gpu::Stream::Null()).download(out);
  return out;
}
inline cv::Mat bwlabel2(const cv::Mat& binaryImage, int connectivity, bool relab) {
  return detail::via_gpu(binaryImage, [&](cv::gpu::GpuMat& g) {
    return gpu::bwlabel(g, connectivity, relab, cv::gpu::Stream::Null());
  });
}
inline cv::Mat bwareaopen2(const cv::Mat& image, bool labeled, bool flatten, int minSize, int maxSize,
                           int connectivity, int& count) {
  return detail::via_gpu(image, [&](cv::gpu::GpuMat& g) {
    return gpu::bwareaopen2(g, labeled, flatten, minSize, maxSize, connectivity, count, cv::gpu::Stream::Null());
  });
}
template <typename T>
cv::Mat imhmin(const cv::Mat& image, T h, int connectivity) {
  return detail::via_gpu(image, [&](cv::gpu::GpuMat& g) {
    return gpu::imhmin<T>(g, h, connectivity, cv::gpu::Stream::Null());
  });
}

// nscale::distanceTransform (MorphologicOperations.h:92), distance map only.
inline cv::Mat distanceTransform(const cv::Mat& mask, bool calcDist = true) {
  return detail::via_gpu(mask, [&](cv::gpu::GpuMat& g) {
    return gpu::distanceTransform(g, cv::gpu::Stream::Null(), calcDist);
  });
}

// nscale::morphOpen<T> (MorphologicOperations.h:89).
template <typename T>
cv::Mat morphOpen(const cv::Mat& image, const cv::Mat& kernel) {
  return detail::via_gpu(image, [&](cv::gpu::GpuMat& g) {
    return gpu::morphOpen<T>(g, kernel, cv::gpu::Stream::Null());
  });
}

}  // namespace nscale
