// A minimal stand-in for the part of OpenCV 2.4's core that the reference's serial
// reconstruction code uses (containers, constant padding, ROIs and the few per-element
// operators).  TEST INFRASTRUCTURE ONLY: it lets oracle/build_ref.sh compile the reference's
// own nscale::imreconstruct / imreconstructBinary / imfillHoles / bwselect / imhmin /
// bwlabel2 / bwareaopen2 and PixelOperations::invert, unmodified, without OpenCV (which is
// not installed).  Nothing in the product includes it.
//
// OpenCV (2.4.x, the version the reference names in README_QTCREATOR.txt) is not vendored by
// the reference, so its arithmetic is restated here from its documented behaviour:
//   * every result is converted to the destination depth with saturate_cast: clamped to the
//     range of 8U / 8S / 16U / 16S, rounded for integer results of float arithmetic;
//   * CV_32S results are NOT saturated ("Saturation is not applied when the output array has
//     the depth CV_32S. You may even get result of an incorrect sign in the case of
//     overflow", the note on cv::add / cv::subtract): they wrap in two's complement.  Built
//     with -DNSGB_SHIM_SATURATE_32S the shim saturates them instead, the other reading;
//   * arithmetic with a scalar on an integer matrix runs in int on the scalar rounded to int;
//     on a CV_32F matrix it runs in float on the scalar converted to float;
//   * `-m` is `0 - m` (MatExpr with alpha -1 assigned through cv::subtract), so a float
//     -0.0 becomes +0.0;
//   * `m > s` gives 255 / 0 in CV_8U; an integer matrix compares with floor(s) (x > s for
//     integer x), a float matrix with s converted to float.
// Matrices are single-channel, row-major, with a byte step; ROIs share the parent's buffer,
// and assignment shares the buffer (reference counting), as in OpenCV.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>

#define CV_8U 0
#define CV_8S 1
#define CV_16U 2
#define CV_16S 3
#define CV_32S 4
#define CV_32F 5
#define CV_64F 6
#define CV_Assert(expr)                                                             \
  do {                                                                              \
    if (!(expr)) throw std::runtime_error(std::string("CV_Assert failed: ") + #expr); \
  } while (0)

namespace cv {

enum { BORDER_CONSTANT = 0 };

struct Size {
  int width = 0, height = 0;
  Size() = default;
  Size(int w, int h) : width(w), height(h) {}
  Size operator+(const Size& o) const { return Size(width + o.width, height + o.height); }
};

struct Range {
  int start = 0, end = 0;
  Range(int s, int e) : start(s), end(e) {}
};

struct Rect {
  int x = 0, y = 0, width = 0, height = 0;
  Rect(int x_, int y_, int w, int h) : x(x_), y(y_), width(w), height(h) {}
};

struct Scalar {
  double val[4] = {0, 0, 0, 0};
  Scalar(double v = 0.0) { val[0] = v; }
  double operator[](int i) const { return val[i]; }
};

inline size_t depth_size(int depth) {
  switch (depth) {
    case CV_8U: case CV_8S: return 1;
    case CV_16U: case CV_16S: return 2;
    case CV_32S: case CV_32F: return 4;
    case CV_64F: return 8;
  }
  throw std::runtime_error("unsupported depth");
}

class Mat {
 public:
  int rows = 0, cols = 0;
  size_t step = 0;
  unsigned char* data = nullptr;

  Mat() = default;
  Mat(int r, int c, int type) { create(r, c, type); }
  Mat(Size sz, int type) { create(sz.height, sz.width, type); }
  Mat(Size sz, int type, const Scalar& s) {
    create(sz.height, sz.width, type);
    setTo(s);
  }
  // Header over caller memory (not owned), as cv::Mat(rows, cols, type, data, step).
  Mat(int r, int c, int type, void* p, size_t st = 0)
      : rows(r), cols(c), data((unsigned char*)p), type_(type) {
    step = st ? st : (size_t)c * depth_size(type);
  }

  static Mat zeros(Size sz, int type) { return Mat(sz, type, Scalar(0)); }
  static Mat zeros(int r, int c, int type) { return Mat(Size(c, r), type, Scalar(0)); }

  int type() const { return type_; }
  int depth() const { return type_; }
  int channels() const { return 1; }
  size_t elemSize() const { return depth_size(type_); }
  Size size() const { return Size(cols, rows); }
  bool empty() const { return data == nullptr || rows == 0 || cols == 0; }
  bool isContinuous() const { return step == (size_t)cols * elemSize(); }

  void create(int r, int c, int type) {
    if (data && buf_ && r == rows && c == cols && type == type_ && isContinuous()) return;
    rows = r;
    cols = c;
    type_ = type;
    step = (size_t)c * depth_size(type);
    const size_t n = step * (size_t)r;
    buf_ = std::shared_ptr<unsigned char>(new unsigned char[n ? n : 1], std::default_delete<unsigned char[]>());
    data = buf_.get();
  }
  void release() {
    buf_.reset();
    data = nullptr;
    rows = cols = 0;
    step = 0;
  }

  unsigned char* ptr(int y) { return data + (size_t)y * step; }
  const unsigned char* ptr(int y) const { return data + (size_t)y * step; }
  template <typename T>
  T* ptr(int y) { return reinterpret_cast<T*>(data + (size_t)y * step); }
  template <typename T>
  const T* ptr(int y) const { return reinterpret_cast<const T*>(data + (size_t)y * step); }

  Mat operator()(const Range& ry, const Range& rx) const {
    Mat m = *this;
    m.data = data + (size_t)ry.start * step + (size_t)rx.start * elemSize();
    m.rows = ry.end - ry.start;
    m.cols = rx.end - rx.start;
    return m;
  }
  Mat operator()(const Rect& r) const { return (*this)(Range(r.y, r.y + r.height), Range(r.x, r.x + r.width)); }

  void setTo(const Scalar& s);
  void copyTo(Mat& dst) const {
    if (dst.data == data && dst.rows == rows && dst.cols == cols && dst.type_ == type_) return;
    dst.create(rows, cols, type_);
    for (int y = 0; y < rows; ++y) std::memcpy(dst.ptr(y), ptr(y), (size_t)cols * elemSize());
  }
  // Copies the elements where mask != 0; dst keeps its other elements when it already has
  // this size and type (cv::Mat::copyTo(dst, mask)).
  void copyTo(Mat& dst, const Mat& mask) const;
  Mat clone() const {
    Mat m;
    copyTo(m);
    return m;
  }

 protected:
  int type_ = CV_8U;
  std::shared_ptr<unsigned char> buf_;
};

template <typename T>
struct DepthOf;
template <> struct DepthOf<unsigned char> { static constexpr int value = CV_8U; };
template <> struct DepthOf<signed char> { static constexpr int value = CV_8S; };
template <> struct DepthOf<unsigned short> { static constexpr int value = CV_16U; };
template <> struct DepthOf<short> { static constexpr int value = CV_16S; };
template <> struct DepthOf<int> { static constexpr int value = CV_32S; };
template <> struct DepthOf<float> { static constexpr int value = CV_32F; };
template <> struct DepthOf<double> { static constexpr int value = CV_64F; };

template <typename T>
class Mat_ : public Mat {
 public:
  Mat_() : Mat() { type_ = DepthOf<T>::value; }
  explicit Mat_(Size sz) : Mat(sz, DepthOf<T>::value) {}
  Mat_(const Mat& m) : Mat(m) { CV_Assert(m.empty() || m.type() == DepthOf<T>::value); }
  Mat_& operator=(const Mat& m) {
    CV_Assert(m.empty() || m.type() == DepthOf<T>::value);
    Mat::operator=(m);
    return *this;
  }
  static Mat_ zeros(Size sz) { return Mat_(Mat::zeros(sz, DepthOf<T>::value)); }
};

// ---- per-element conversion and arithmetic ----------------------------------------------

namespace shim {

// The destination conversion of an integer result (computed in 64 bits).
template <typename T>
inline T from_int(int64_t v) {
  if constexpr (std::is_same_v<T, int>) {
#ifdef NSGB_SHIM_SATURATE_32S
    if (v > std::numeric_limits<int>::max()) return std::numeric_limits<int>::max();
    if (v < std::numeric_limits<int>::min()) return std::numeric_limits<int>::min();
    return (int)v;
#else
    return (int)(uint32_t)(uint64_t)v;  // two's-complement wrap
#endif
  } else {
    if (v > (int64_t)std::numeric_limits<T>::max()) return std::numeric_limits<T>::max();
    if (v < (int64_t)std::numeric_limits<T>::min()) return std::numeric_limits<T>::min();
    return (T)v;
  }
}

inline int64_t scalar_to_int(double s) { return (int64_t)std::nearbyint(s); }

// Calls f(T*) for the element type of `depth`.
template <typename F>
void by_depth(int depth, F&& f) {
  switch (depth) {
    case CV_8U: f((unsigned char*)nullptr); return;
    case CV_8S: f((signed char*)nullptr); return;
    case CV_16U: f((unsigned short*)nullptr); return;
    case CV_16S: f((short*)nullptr); return;
    case CV_32S: f((int*)nullptr); return;
    case CV_32F: f((float*)nullptr); return;
    case CV_64F: f((double*)nullptr); return;
  }
  throw std::runtime_error("unsupported depth");
}

// dst = op(src) elementwise, dst a new matrix of depth `dst_depth`.
template <typename Op>
Mat unary(const Mat& a, int dst_depth, Op op) {
  Mat d(a.rows, a.cols, dst_depth);
  by_depth(a.depth(), [&](auto* ts) {
    using S = std::remove_pointer_t<decltype(ts)>;
    by_depth(dst_depth, [&](auto* td) {
      using D = std::remove_pointer_t<decltype(td)>;
      for (int y = 0; y < a.rows; ++y) {
        const S* s = a.ptr<S>(y);
        D* o = d.ptr<D>(y);
        for (int x = 0; x < a.cols; ++x) o[x] = op(s[x], (D*)nullptr);
      }
    });
  });
  return d;
}

// a + s (s_sign = +1) or s - a (s_sign = -1), OpenCV's add / subtract with a scalar.
inline Mat add_scalar(const Mat& a, double s, int a_sign) {
  return unary(a, a.depth(), [&](auto x, auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    if constexpr (std::is_floating_point_v<T>) {
      const T sc = (T)s;
      return a_sign > 0 ? (T)(x + sc) : (T)(sc - x);
    } else {
      const int64_t si = scalar_to_int(s);
      return from_int<T>(a_sign > 0 ? (int64_t)x + si : si - (int64_t)x);
    }
  });
}

}  // namespace shim

inline void Mat::setTo(const Scalar& s) {
  shim::by_depth(depth(), [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    T v;
    if constexpr (std::is_floating_point_v<T>) {
      v = (T)s[0];
    } else {
      const int64_t si = shim::scalar_to_int(s[0]);
      v = si > (int64_t)std::numeric_limits<T>::max()   ? std::numeric_limits<T>::max()
          : si < (int64_t)std::numeric_limits<T>::min() ? std::numeric_limits<T>::min()
                                                        : (T)si;
    }
    for (int y = 0; y < rows; ++y) {
      T* p = ptr<T>(y);
      for (int x = 0; x < cols; ++x) p[x] = v;
    }
  });
}

inline void Mat::copyTo(Mat& dst, const Mat& mask) const {
  CV_Assert(mask.rows == rows && mask.cols == cols);
  if (!(dst.data && dst.rows == rows && dst.cols == cols && dst.type() == type_)) dst.create(rows, cols, type_);
  const size_t es = elemSize(), ms = mask.elemSize();
  for (int y = 0; y < rows; ++y) {
    const unsigned char* s = ptr(y);
    const unsigned char* m = mask.ptr(y);
    unsigned char* d = dst.ptr(y);
    for (int x = 0; x < cols; ++x) {
      bool nz = false;
      for (size_t b = 0; b < ms; ++b) nz |= m[x * ms + b] != 0;
      if (nz) std::memcpy(d + x * es, s + x * es, es);
    }
  }
}

// copyMakeBorder(src, dst, top, bottom, left, right, BORDER_CONSTANT, value).
inline void copyMakeBorder(const Mat& src, Mat& dst, int top, int bottom, int left, int right, int border,
                           const Scalar& value) {
  CV_Assert(border == BORDER_CONSTANT);
  Mat out(Size(src.cols + left + right, src.rows + top + bottom), src.type(), value);
  const size_t es = src.elemSize();
  for (int y = 0; y < src.rows; ++y) std::memcpy(out.ptr(y + top) + (size_t)left * es, src.ptr(y), (size_t)src.cols * es);
  dst = out;
}

inline void bitwise_not(const Mat& a, Mat& out) {
  Mat d(a.rows, a.cols, a.type());
  const size_t n = (size_t)a.cols * a.elemSize();
  for (int y = 0; y < a.rows; ++y)
    for (size_t i = 0; i < n; ++i) d.ptr(y)[i] = (unsigned char)~a.ptr(y)[i];
  out = d;
}

inline Mat bitwise_binary(const Mat& a, const Mat& b, bool is_or) {
  CV_Assert(a.rows == b.rows && a.cols == b.cols && a.type() == b.type());
  Mat d(a.rows, a.cols, a.type());
  const size_t n = (size_t)a.cols * a.elemSize();
  for (int y = 0; y < a.rows; ++y)
    for (size_t i = 0; i < n; ++i)
      d.ptr(y)[i] = is_or ? (unsigned char)(a.ptr(y)[i] | b.ptr(y)[i]) : (unsigned char)(a.ptr(y)[i] & b.ptr(y)[i]);
  return d;
}

inline Mat operator|(const Mat& a, const Mat& b) { return bitwise_binary(a, b, true); }
inline Mat operator&(const Mat& a, const Mat& b) { return bitwise_binary(a, b, false); }
inline Mat operator+(const Mat& a, double s) { return shim::add_scalar(a, s, +1); }
inline Mat operator-(const Mat& a, double s) { return shim::add_scalar(a, -s, +1); }
inline Mat operator-(double s, const Mat& a) { return shim::add_scalar(a, s, -1); }
inline Mat operator-(const Mat& a) { return shim::add_scalar(a, 0.0, -1); }

inline Mat operator>(const Mat& a, double s) {
  return shim::unary(a, CV_8U, [&](auto x, auto*) -> unsigned char {
    using T = decltype(x);
    bool gt;
    if constexpr (std::is_same_v<T, float>) gt = x > (float)s;
    else gt = (double)x > s;
    return gt ? 255 : 0;
  });
}

}  // namespace cv
