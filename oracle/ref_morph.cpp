// C entry points over the reference's own serial reconstruction code, compiled unmodified:
// oracle/build_ref.sh copies these line ranges of the reference, as text, into
// oracle/_ref/src/ and this file includes them inside namespace nscale:
//   src/segment/PixelOperations.cpp        17-39     PixelOperations::invert<T>
//   src/segment/MorphologicOperations.cpp  428-439   propagate<T>
//                                          665-838   imreconstruct<T>
//                                          1665-1673 propagateBinary<T>
//                                          1688-1829 imreconstructBinary<T>
//                                          1859-1926 imfillHoles<T>
//                                          1929-1951 bwselect<T>
//                                          2012-2035 bwlabel2
//                                          2199-2232 bwareaopen2
//                                          2260-2282 imhmin<T>
// with src/common/TypeUtils.h and src/segment/ConnComponents.h from the reference tree and
// ConnComponents.cpp compiled beside it.  OpenCV is replaced by oracle/cv_shim.hpp.
// TEST INFRASTRUCTURE ONLY: it pins the oracle's restatement (recon_oracle.hpp) and times the
// reference's CPU path in bench.py's reference arm.  Nothing in the product links it.
//
// dtype codes: 0 = u8, 1 = u16 (the templates instantiated at uint16_t: the reference has no
// u16 instantiation), 2 = i32, 3 = f32.  Images are dense row-major.  Every function returns
// 0, or -1 for an unsupported dtype / -2 when the reference code threw (a CV_Assert).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <limits>
#include <queue>
#include <thread>
#include <vector>

#include "cv_shim.hpp"

#include "ConnComponents.h"
#include "TypeUtils.h"

namespace nscale {
using namespace cv;
using namespace std;

class PixelOperations {
 public:
  template <typename T>
  static ::cv::Mat invert(const ::cv::Mat& img);
};

#include "pixel_invert.inc"
#include "morph_ref.inc"

}  // namespace nscale

namespace {

template <typename F>
int dispatch(int dtype, F&& f) {
  try {
    switch (dtype) {
      case 0: f((unsigned char*)nullptr); return 0;
      case 1: f((unsigned short*)nullptr); return 0;
      case 2: f((int*)nullptr); return 0;
      case 3: f((float*)nullptr); return 0;
      default: return -1;
    }
  } catch (const std::exception& e) {
    std::cerr << "reference code: " << e.what() << std::endl;
    return -2;
  }
}

template <typename T>
cv::Mat wrap(const void* p, int64_t H, int64_t W) {
  return cv::Mat((int)H, (int)W, cv::DepthOf<T>::value, const_cast<void*>(p));
}

// Copies a (possibly non-continuous ROI) result into dense memory.
void store(const cv::Mat& m, void* out) {
  const size_t rb = (size_t)m.cols * m.elemSize();
  for (int y = 0; y < m.rows; ++y) std::memcpy((char*)out + y * rb, m.ptr(y), rb);
}

}  // namespace

extern "C" {

int ref_imreconstruct(int dtype, const void* marker, const void* mask, int64_t H, int64_t W, int conn, void* out) {
  return dispatch(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    store(nscale::imreconstruct<T>(wrap<T>(marker, H, W), wrap<T>(mask, H, W), conn), out);
  });
}

int ref_imreconstruct_binary(int dtype, const void* marker, const void* mask, int64_t H, int64_t W, int conn,
                             void* out) {
  return dispatch(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    store(nscale::imreconstructBinary<T>(wrap<T>(marker, H, W), wrap<T>(mask, H, W), conn), out);
  });
}

int ref_imfill_holes(int dtype, const void* image, int64_t H, int64_t W, int binary, int conn, void* out) {
  return dispatch(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    store(nscale::imfillHoles<T>(wrap<T>(image, H, W), binary != 0, conn), out);
  });
}

int ref_imhmin(int dtype, const void* image, int64_t H, int64_t W, double h, int conn, void* out) {
  return dispatch(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    store(nscale::imhmin<T>(wrap<T>(image, H, W), (T)h, conn), out);
  });
}

int ref_bwselect(int dtype, const void* image, const void* seeds, int64_t H, int64_t W, int conn, void* out) {
  return dispatch(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    store(nscale::bwselect<T>(wrap<T>(image, H, W), wrap<T>(seeds, H, W), conn), out);
  });
}

// `image > thr` (the reference's threshold, e.g. HistologicalEntities.cpp:214), 255 / 0.
int ref_threshold_gt(int dtype, const void* image, int64_t H, int64_t W, double thr, uint8_t* out) {
  return dispatch(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    store(wrap<T>(image, H, W) > thr, out);
  });
}

// bwlabel2; returns the largest label (the component count after a raster relabel).
int ref_bwlabel2(const uint8_t* bin, int64_t H, int64_t W, int conn, int relab, int32_t* out) {
  int r = dispatch(0, [&](auto*) {
    cv::Mat_<int> lab = nscale::bwlabel2(wrap<unsigned char>(bin, H, W), conn, relab != 0);
    store(lab, out);
  });
  if (r != 0) return -1;
  int32_t mx = 0;
  for (int64_t i = 0; i < H * W; ++i) mx = std::max(mx, out[i]);
  return mx;
}

// bwareaopen2 on a u8 image (labeled = 0) or int32 labels (labeled = 1); out is u8 when
// flatten, int32 otherwise.  Returns the reference's count, or -1.
int ref_bwareaopen2(const void* image, int labeled, int flatten, int32_t lo, int32_t hi, int conn, int64_t H,
                    int64_t W, void* out) {
  int count = -1;
  int r = dispatch(0, [&](auto*) {
    cv::Mat in = labeled ? wrap<int>(image, H, W) : wrap<unsigned char>(image, H, W);
    store(nscale::bwareaopen2(in, labeled != 0, flatten != 0, lo, hi, conn, count), out);
  });
  return r == 0 ? count : -1;
}

// The single-tile chain as the reference's own functions compose it: (a) imreconstruct,
// (b) `> thr`, (c) imfillHoles<uchar>(binary), (d) bwlabel2(relabel), (e) bwareaopen2 on the
// filled image, flattened.  Null outputs are skipped.  Returns the count of (e), or -1.
int32_t ref_chain(int dtype, const void* marker, const void* mask, int64_t H, int64_t W, int recon_conn, double thr,
                  int fill_conn, int label_conn, int32_t lo, int32_t hi, void* recon_out, uint8_t* thr_out,
                  uint8_t* fill_out, int32_t* label_out, int32_t* n_labels, uint8_t* area_out) {
  int count = -1;
  int r = dispatch(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    cv::Mat rec = nscale::imreconstruct<T>(wrap<T>(marker, H, W), wrap<T>(mask, H, W), recon_conn);
    cv::Mat bin = rec > thr;
    cv::Mat fill = nscale::imfillHoles<unsigned char>(bin, true, fill_conn);
    cv::Mat_<int> lab = nscale::bwlabel2(fill, label_conn, true);
    cv::Mat area = nscale::bwareaopen2(fill, false, true, lo, hi, label_conn, count);
    if (recon_out) store(rec, recon_out);
    if (thr_out) store(bin, thr_out);
    if (fill_out) store(fill, fill_out);
    if (label_out) store(lab, label_out);
    if (n_labels) {
      int32_t mx = 0;
      for (int y = 0; y < lab.rows; ++y)
        for (int x = 0; x < lab.cols; ++x) mx = std::max(mx, lab.ptr<int>(y)[x]);
      *n_labels = mx;
    }
    if (area_out) store(area, area_out);
  });
  return r == 0 ? count : -1;
}

// Runs the u8 chain (8-conn reconstruction, > 128, 4-conn binary fill, 8-conn bwlabel2 and
// bwareaopen2 [11, 1000)) `reps` times on each of `threads` host threads, each thread on its
// own copy of the tile, and returns the wall time in seconds.  Used to time the reference's
// CPU path.
double ref_chain_replicas_seconds(const uint8_t* marker, const uint8_t* mask, int64_t H, int64_t W, int threads,
                                  int reps) {
  if (threads < 1) threads = 1;
  const int64_t n = H * W;
  std::vector<std::vector<uint8_t>> mk(threads), ms(threads);
  for (int t = 0; t < threads; ++t) {
    mk[t].assign(marker, marker + n);
    ms[t].assign(mask, mask + n);
  }
  std::atomic<int> failed{0};
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) {
    pool.emplace_back([&, t] {
      for (int r = 0; r < reps; ++r)
        if (ref_chain(0, mk[t].data(), ms[t].data(), H, W, 8, 128.0, 4, 8, 11, 1000, nullptr, nullptr, nullptr,
                      nullptr, nullptr, nullptr) < 0)
          failed = 1;
    });
  }
  for (auto& th : pool) th.join();
  auto t1 = std::chrono::steady_clock::now();
  return failed ? -1.0 : std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
