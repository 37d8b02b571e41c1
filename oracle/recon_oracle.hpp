// CPU oracle for the reconstruction / labelling path.  TEST INFRASTRUCTURE ONLY.
//
// This file restates, on plain arrays, the reference's serial CPU algorithms.  It is the
// checker that the CUDA path is compared against; the product never links or calls it.
// Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use it.
//
// Every function cites the reference function it follows (paths relative to the
// reference project root, fastIA-master/).  The restatement keeps the reference's
// semantics: 0-padding of marker and mask, the raster / anti-raster / FIFO order of
// Vincent's hybrid algorithm, numeric_limits-based padding values, and the union-find
// root = smallest raster index rule.  It is written from the algorithm, not copied.
//
// Parity pins: everything restated from the reference is checked against the reference's
// own code compiled from its sources (oracle/build_ref.sh): ConnComponents.cpp for the
// union-find part, and MorphologicOperations.cpp's imreconstruct / imreconstructBinary /
// imfillHoles / bwselect / imhmin / bwlabel2 / bwareaopen2 (over a small OpenCV stand-in) for
// the reconstruction part, through committed fixtures and, where the reference builds, live
// (tests/test_oracle_ref_recon_cpu.py).  The float provenance and adjoint have no reference
// counterpart.
#pragma once

#include <algorithm>
#include <cmath>
#include <climits>
#include <cstdint>
#include <cstring>
#include <deque>
#include <limits>
#include <type_traits>
#include <unordered_map>
#include <vector>

namespace orc {

// src/common/TypeUtils.h:34-41: lowest value used for padding ("-inf").
template <typename T>
inline T type_min() {
  if constexpr (std::numeric_limits<T>::is_integer) return std::numeric_limits<T>::min();
  else return -std::numeric_limits<T>::max();
}

// src/segment/PixelOperations.cpp:18-39.  Unsigned: max - x.  Signed: bitwise_not(x) + 1
// through OpenCV arithmetic; the one value where that overflows (INT_MIN) is taken with
// saturating arithmetic, i.e. invert(INT_MIN) = INT_MAX.  OpenCV itself does not saturate
// CV_32S (it wraps, and the reference's imfillHoles<int> then returns INT_MIN everywhere;
// tests/test_oracle_ref_recon_cpu.py pins both readings against the reference's code).
// Float: OpenCV evaluates `-img` as `0 - img`, so the result is never -0.0.
template <typename T>
inline T invert_px(T x) {
  if constexpr (std::numeric_limits<T>::is_integer) {
    if constexpr (std::numeric_limits<T>::is_signed) {
      if (x == std::numeric_limits<T>::min()) return std::numeric_limits<T>::max();
      return (T)(-x);
    } else {
      return (T)(std::numeric_limits<T>::max() - x);
    }
  } else {
    return (T)0 - x;
  }
}

// std::min / std::max as the reference uses them (ties keep the first argument for max
// when !(a < b), and the first argument for min when !(b < a)).
template <typename T>
inline T vmax(T a, T b) { return (a < b) ? b : a; }
template <typename T>
inline T vmin(T a, T b) { return (b < a) ? b : a; }

// A (rows x cols) row-major plane.
template <typename T>
struct Plane {
  int64_t rows = 0, cols = 0;
  std::vector<T> d;
  Plane() = default;
  Plane(int64_t r, int64_t c, T v) : rows(r), cols(c), d((size_t)(r * c), v) {}
  T* row(int64_t y) { return d.data() + y * cols; }
  const T* row(int64_t y) const { return d.data() + y * cols; }
};

// copyMakeBorder(src, dst, 1, 1, 1, 1, BORDER_CONSTANT, v)
template <typename T>
Plane<T> pad1(const T* src, int64_t H, int64_t W, T v) {
  Plane<T> p(H + 2, W + 2, v);
  for (int64_t y = 0; y < H; ++y) std::memcpy(p.row(y + 1) + 1, src + y * W, (size_t)W * sizeof(T));
  return p;
}

template <typename T>
void crop1(const Plane<T>& p, T* dst) {
  const int64_t H = p.rows - 2, W = p.cols - 2;
  for (int64_t y = 0; y < H; ++y) std::memcpy(dst + y * W, p.row(y + 1) + 1, (size_t)W * sizeof(T));
}

// Grayscale reconstruction by dilation of `seeds` under `image`.
// src/segment/MorphologicOperations.cpp:665-838 (imreconstruct<T>) with the propagation
// step of MorphologicOperations.cpp:428-439 (propagate<T>).
template <typename T>
void imreconstruct(const T* seeds, const T* image, int64_t H, int64_t W, int conn, T* out) {
  Plane<T> o = pad1<T>(seeds, H, W, (T)0);
  Plane<T> in = pad1<T>(image, H, W, (T)0);
  const int64_t C = o.cols;
  const int64_t maxx = o.cols - 1, maxy = o.rows - 1;
  T* O = o.d.data();
  const T* I = in.d.data();
  std::deque<int64_t> fifo;

  // Raster scan: N+(p) = left, up (and up-left, up-right for 8-connectivity).
  for (int64_t y = 1; y < maxy; ++y) {
    T* r = O + y * C;
    const T* ru = r - C;
    const T* ir = I + y * C;
    T left = r[0];
    for (int64_t x = 1; x < maxx; ++x) {
      T v = vmax(r[x], vmax(left, ru[x]));
      if (conn == 8) v = vmax(v, vmax(ru[x + 1], ru[x - 1]));
      left = vmin(v, ir[x]);
      r[x] = left;
    }
  }
  // Anti-raster scan: N-(p) = right, down (and down-right, down-left), then seed the FIFO
  // with every p that could still raise one of its N-(p) neighbours.
  for (int64_t y = maxy - 1; y > 0; --y) {
    T* r = O + y * C;
    T* rd = r + C;
    const T* ir = I + y * C;
    const T* ird = ir + C;
    T right = r[maxx];
    for (int64_t x = maxx - 1; x > 0; --x) {
      T v = vmax(r[x], vmax(right, rd[x]));
      if (conn == 8) v = vmax(v, vmax(rd[x + 1], rd[x - 1]));
      right = vmin(v, ir[x]);
      r[x] = right;
      const T p = r[x];
      if (r[x + 1] < vmin(p, ir[x + 1]) || rd[x] < vmin(p, ird[x])) {
        fifo.push_back(y * C + x);
        continue;
      }
      if (conn == 8 && (rd[x + 1] < vmin(p, ird[x + 1]) || rd[x - 1] < vmin(p, ird[x - 1]))) {
        fifo.push_back(y * C + x);
      }
    }
  }
  // FIFO propagation.
  auto propagate = [&](int64_t q, T p) {
    const T qv = O[q], iv = I[q];
    if (qv < p && iv != qv) {
      O[q] = vmin(p, iv);
      fifo.push_back(q);
    }
  };
  while (!fifo.empty()) {
    const int64_t i = fifo.front();
    fifo.pop_front();
    const int64_t y = i / C, x = i % C;
    const T p = O[i];
    if (y > 0) propagate(i - C, p);
    if (y < maxy) propagate(i + C, p);
    if (x > 0) propagate(i - 1, p);
    if (x < maxx) propagate(i + 1, p);
    if (conn == 8) {
      if (y > 0) {
        if (x > 0) propagate(i - C - 1, p);
        if (x < maxx) propagate(i - C + 1, p);
      }
      if (y < maxy) {
        if (x > 0) propagate(i + C - 1, p);
        if (x < maxx) propagate(i + C + 1, p);
      }
    }
  }
  crop1(o, out);
}

// Binary reconstruction (background 0, foreground != 0; filled pixels get max<T>).
// src/segment/MorphologicOperations.cpp:1688-1829 (imreconstructBinary<T>) with
// propagateBinary<T> at 1665-1673.  The marker is not clamped by the mask.
template <typename T>
void imreconstruct_binary(const T* seeds, const T* image, int64_t H, int64_t W, int conn, T* out) {
  Plane<T> o = pad1<T>(seeds, H, W, (T)0);
  Plane<T> in = pad1<T>(image, H, W, (T)0);
  const int64_t C = o.cols;
  const int64_t maxx = o.cols - 1, maxy = o.rows - 1;
  T* O = o.d.data();
  const T* I = in.d.data();
  std::deque<int64_t> fifo;
  // Contour pixels: marker and mask both non-zero with a zero neighbour in the marker.
  for (int64_t y = 1; y < maxy; ++y) {
    for (int64_t x = 1; x < maxx; ++x) {
      const int64_t i = y * C + x;
      if (O[i] != 0 && I[i] != 0) {
        if (O[i - C] == 0 || O[i + C] == 0 || O[i + 1] == 0 || O[i - 1] == 0) {
          fifo.push_back(i);
          continue;
        }
        if (conn == 8 && (O[i - C - 1] == 0 || O[i - C + 1] == 0 || O[i + C - 1] == 0 || O[i + C + 1] == 0)) {
          fifo.push_back(i);
        }
      }
    }
  }
  const T fg = std::numeric_limits<T>::max();
  auto propagate = [&](int64_t q) {
    if (O[q] == 0 && I[q] != 0) {
      O[q] = fg;
      fifo.push_back(q);
    }
  };
  while (!fifo.empty()) {
    const int64_t i = fifo.front();
    fifo.pop_front();
    const int64_t y = i / C, x = i % C;
    if (y > 0) propagate(i - C);
    if (y < maxy) propagate(i + C);
    if (x > 0) propagate(i - 1);
    if (x < maxx) propagate(i + 1);
    if (conn == 8) {
      if (y > 0) {
        if (x > 0) propagate(i - C - 1);
        if (x < maxx) propagate(i - C + 1);
      }
      if (y < maxy) {
        if (x > 0) propagate(i + C - 1);
        if (x < maxx) propagate(i + C + 1);
      }
    }
  }
  crop1(o, out);
}

// Hole filling.  src/segment/MorphologicOperations.cpp:1859-1926 (imfillHoles<T>): the
// image is padded with min<T>, the marker is min<T> inside and max<T> on the padding ring,
// the mask is inverted, reconstructed (binary or grayscale), inverted back and cropped.
template <typename T>
void imfill_holes(const T* image, int64_t H, int64_t W, bool binary, int conn, T* out) {
  const T mn = type_min<T>();
  const T mx = std::numeric_limits<T>::max();
  Plane<T> mask = pad1<T>(image, H, W, mn);
  Plane<T> marker(H + 2, W + 2, mx);
  for (int64_t y = 1; y <= H; ++y)
    for (int64_t x = 1; x <= W; ++x) marker.row(y)[x] = mn;
  for (auto& v : mask.d) v = invert_px(v);
  Plane<T> rec(H + 2, W + 2, (T)0);
  if (binary)
    imreconstruct_binary<T>(marker.d.data(), mask.d.data(), H + 2, W + 2, conn, rec.d.data());
  else
    imreconstruct<T>(marker.d.data(), mask.d.data(), H + 2, W + 2, conn, rec.d.data());
  for (auto& v : rec.d) v = invert_px(v);
  crop1(rec, out);
}

// Saturating subtraction as OpenCV's `Mat - scalar` does for 8/16-bit types; for 32-bit
// integers the result is clamped as well; float is plain subtraction.
template <typename T>
inline T sub_sat(T a, T h) {
  if constexpr (std::numeric_limits<T>::is_integer) {
    const int64_t r = (int64_t)a - (int64_t)h;
    if (r < (int64_t)std::numeric_limits<T>::min()) return std::numeric_limits<T>::min();
    if (r > (int64_t)std::numeric_limits<T>::max()) return std::numeric_limits<T>::max();
    return (T)r;
  } else {
    return a - h;
  }
}

// h-minima transform.  src/segment/MorphologicOperations.cpp:2260-2282 (imhmin<T>):
// invert(imreconstruct(invert(I) - h, invert(I))).
template <typename T>
void imhmin(const T* image, int64_t H, int64_t W, T h, int conn, T* out) {
  const int64_t n = H * W;
  std::vector<T> mask((size_t)n), marker((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    mask[i] = invert_px(image[i]);
    marker[i] = sub_sat(mask[i], h);
  }
  imreconstruct<T>(marker.data(), mask.data(), H, W, conn, out);
  for (int64_t i = 0; i < n; ++i) out[i] = invert_px(out[i]);
}

// src/segment/MorphologicOperations.cpp:1929-1951 (bwselect<T>): binary reconstruction
// of the image restricted to the seed pixels, ANDed with the image.
template <typename T>
void bwselect(const T* image, const T* seeds, int64_t H, int64_t W, int conn, T* out) {
  const int64_t n = H * W;
  std::vector<T> marker((size_t)n);
  for (int64_t i = 0; i < n; ++i) marker[i] = seeds[i] != 0 ? image[i] : (T)0;
  imreconstruct_binary<T>(marker.data(), image, H, W, conn, out);
  for (int64_t i = 0; i < n; ++i) out[i] = (T)(out[i] & image[i]);
}

// ---------------------------------------------------------------------------------------
// Union-find labelling.  src/segment/ConnComponents.cpp.

// ConnComponents::find (24-32) with path compression, written iteratively.
inline int32_t uf_find(int32_t* L, int32_t x) {
  int32_t r = x;
  while (L[r] != r) r = L[r];
  while (L[x] != r) {
    int32_t n = L[x];
    L[x] = r;
    x = n;
  }
  return r;
}

// ConnComponents::merge (34-43): the root with the smaller index wins.
inline void uf_merge(int32_t* L, int32_t a, int32_t b) {
  a = uf_find(L, a);
  b = uf_find(L, b);
  if (a < b) L[b] = a;
  else if (a > b) L[a] = b;
}

// ConnComponents::label (52-86): equal-valued non-zero neighbours are joined; background
// gets bgval; every foreground pixel ends with the smallest raster index of its component
// (ConnComponents::flatten, 137-148).
inline void cc_label(const uint8_t* img, int64_t W, int64_t H, int32_t* L, int32_t bgval, int conn) {
  const int64_t n = W * H;
  for (int64_t i = 0; i < n; ++i) L[i] = (int32_t)i;
  for (int64_t y = 0; y < H; ++y) {
    for (int64_t x = 0; x < W; ++x) {
      const int64_t i = y * W + x;
      const uint8_t p = img[i];
      if (p == 0) {
        L[i] = bgval;
        continue;
      }
      if (x > 0 && p == img[i - 1]) uf_merge(L, (int32_t)i, (int32_t)(i - 1));
      if (y > 0 && p == img[i - W]) uf_merge(L, (int32_t)i, (int32_t)(i - W));
      if (conn == 8) {
        if (y > 0 && x > 0 && p == img[i - W - 1]) uf_merge(L, (int32_t)i, (int32_t)(i - W - 1));
        if (y > 0 && x < W - 1 && p == img[i - W + 1]) uf_merge(L, (int32_t)i, (int32_t)(i - W + 1));
      }
    }
  }
  for (int64_t i = 0; i < n; ++i) {
    if (L[i] == bgval) continue;
    int32_t r = (int32_t)i;
    while (L[r] != r) r = L[r];
    L[i] = r;
  }
}

// ConnComponents::relabel (89-118): roots numbered 1..n in raster order, bgval -> 0.
inline int32_t cc_relabel(int64_t W, int64_t H, int32_t* L, int32_t bgval) {
  const int64_t n = W * H;
  std::vector<int32_t> id((size_t)n, 0);
  int32_t j = 1;
  for (int64_t i = 0; i < n; ++i)
    if (L[i] == (int32_t)i) id[i] = j++;
  for (int64_t i = 0; i < n; ++i) L[i] = (L[i] == bgval) ? 0 : id[L[i]];
  return j - 1;
}

// ConnComponents::areaThresholdLabeled (205-239): keep labels whose pixel count is in
// [lower, upper); the rest become bgval.  Returns the number kept.
inline int32_t cc_area_threshold_labeled(const int32_t* L, int64_t W, int64_t H, int32_t* out,
                                         int32_t bgval, int32_t lower, int32_t upper) {
  const int64_t n = W * H;
  // Labels are raster indices here (or any value < n); count with a dense array where
  // possible, otherwise sort.
  std::vector<int64_t> keys;
  keys.reserve(1024);
  std::vector<int32_t> area;
  bool dense = true;
  for (int64_t i = 0; i < n; ++i)
    if (L[i] != bgval && (L[i] < 0 || L[i] >= n)) dense = false;
  int32_t kept = 0;
  if (dense) {
    area.assign((size_t)n, 0);
    for (int64_t i = 0; i < n; ++i)
      if (L[i] != bgval) ++area[L[i]];
    for (int64_t i = 0; i < n; ++i)
      if (area[i] > 0 && area[i] >= lower && area[i] < upper) ++kept;
    for (int64_t i = 0; i < n; ++i) {
      const int32_t l = L[i];
      out[i] = (l != bgval && area[l] >= lower && area[l] < upper) ? l : bgval;
    }
    return kept;
  }
  std::vector<int32_t> s;
  for (int64_t i = 0; i < n; ++i)
    if (L[i] != bgval) s.push_back(L[i]);
  std::sort(s.begin(), s.end());
  std::vector<std::pair<int32_t, int32_t>> runs;
  for (size_t a = 0; a < s.size();) {
    size_t b = a;
    while (b < s.size() && s[b] == s[a]) ++b;
    runs.push_back({s[a], (int32_t)(b - a)});
    if ((int32_t)(b - a) >= lower && (int32_t)(b - a) < upper) ++kept;
    a = b;
  }
  for (int64_t i = 0; i < n; ++i) {
    out[i] = bgval;
    if (L[i] == bgval) continue;
    auto it = std::lower_bound(runs.begin(), runs.end(), std::make_pair(L[i], (int32_t)-1));
    if (it->second >= lower && it->second < upper) out[i] = L[i];
  }
  return kept;
}

// ConnComponents::boundingBox (ConnComponents.cpp:241-284): one entry per label other than
// bgval, in the order of the label's first pixel in raster order, holding the label and its
// pixels' min x, max x, min y, max y.  A pixel labelled -1 or 0 that is not bgval ends the scan
// there (the reference prints a message and stops).  Writes min(count, cap) entries as five
// arrays of stride `cap` (label, minx, maxx, miny, maxy) and returns the count.
inline int32_t cc_bounding_box(const int32_t* L, int64_t W, int64_t H, int32_t bgval, int32_t* out,
                               int64_t cap) {
  std::unordered_map<int32_t, size_t> at;
  std::vector<int32_t> lab, mnx, mxx, mny, mxy;
  const int64_t n = W * H;
  for (int64_t i = 0; i < n; ++i) {
    const int32_t l = L[i];
    if (l == bgval) continue;
    if (l == -1 || l == 0) break;
    const int32_t x = (int32_t)(i % W), y = (int32_t)(i / W);
    auto it = at.find(l);
    if (it == at.end()) {
      at.emplace(l, lab.size());
      lab.push_back(l);
      mnx.push_back(x);
      mxx.push_back(x);
      mny.push_back(y);
      mxy.push_back(y);
    } else {
      const size_t k = it->second;
      mnx[k] = std::min(mnx[k], x);
      mxx[k] = std::max(mxx[k], x);
      mny[k] = std::min(mny[k], y);
      mxy[k] = std::max(mxy[k], y);
    }
  }
  const int64_t m = std::min<int64_t>((int64_t)lab.size(), cap);
  for (int64_t k = 0; k < m; ++k) {
    out[k] = lab[k];
    out[cap + k] = mnx[k];
    out[2 * cap + k] = mxx[k];
    out[3 * cap + k] = mny[k];
    out[4 * cap + k] = mxy[k];
  }
  return (int32_t)lab.size();
}

// src/segment/MorphologicOperations.cpp:2012-2035 (bwlabel2).
inline int32_t bwlabel2(const uint8_t* bin, int64_t H, int64_t W, int conn, bool relab, int32_t* out) {
  cc_label(bin, W, H, out, -1, conn);
  if (relab) return cc_relabel(W, H, out, -1);
  return 0;
}

// src/segment/MorphologicOperations.cpp:2199-2232 (bwareaopen2): label (unless already
// labelled), keep areas in [minSize, maxSize), optionally flatten to 255 / 0 (`> -1`).
inline int32_t bwareaopen2(const void* image, bool labeled, bool flatten, int32_t minSize,
                           int32_t maxSize, int conn, int64_t H, int64_t W, int32_t* labels_out,
                           uint8_t* flat_out) {
  const int64_t n = H * W;
  std::vector<int32_t> lab((size_t)n);
  if (!labeled) cc_label((const uint8_t*)image, W, H, lab.data(), -1, conn);
  else std::memcpy(lab.data(), image, (size_t)n * sizeof(int32_t));
  std::vector<int32_t> kept((size_t)n);
  int32_t count = cc_area_threshold_labeled(lab.data(), W, H, kept.data(), -1, minSize, maxSize);
  if (labels_out) std::memcpy(labels_out, kept.data(), (size_t)n * sizeof(int32_t));
  if (flatten && flat_out)
    for (int64_t i = 0; i < n; ++i) flat_out[i] = kept[i] > -1 ? 255 : 0;
  return count;
}

// `Mat > k` (HistologicalEntities.cpp:214): 255 where strictly greater, else 0.  OpenCV's
// compare converts the scalar to the image's depth: an integer image compares with floor(k)
// (the same as x > k for integer x; u8 `> -1` is true everywhere), a float image with k
// rounded to float.
template <typename T>
inline void threshold_gt(const T* in, int64_t n, double k, uint8_t* out) {
  if constexpr (std::is_floating_point_v<T>) {
    const T kk = (T)k;
    for (int64_t i = 0; i < n; ++i) out[i] = in[i] > kk ? 255 : 0;
  } else {
    for (int64_t i = 0; i < n; ++i) out[i] = (double)in[i] > k ? 255 : 0;
  }
}

// ---------------------------------------------------------------------------------------
// Differentiable float reconstruction (an extension: the reference has no gradient).
//
// The reconstruction R only ever copies input values, so every R(p) is the value of one
// source: mask(q) (the mask clamped at q), marker(q) (q's marker survived), or the constant 0
// of the zero ring that the reference pads around the image (MorphologicOperations.cpp:
// 671-674; it can only win on a border pixel, as 0).  A source and every pixel that took its
// value form one plateau: a connected set (same connectivity) of equal R.  The provenance of
// p names the source of p's plateau, preferring a mask source, then a marker source, then the
// ring, and the smallest raster index among equals:
//   prov = ~q (mask source q), q (marker source q), INT32_MIN (ring).
// Found here by a breadth-first flood of each plateau (the GPU uses union-find).  Returns
// false if some plateau has no source (only possible with NaN inputs).
template <typename T>
bool recon_provenance(const T* marker, const T* mask, const T* R, int64_t H, int64_t W, int conn,
                      int32_t* prov) {
  const int64_t n = H * W;
  std::vector<uint8_t> seen((size_t)n, 0);
  std::vector<int64_t> comp;
  std::vector<int64_t> stack;
  for (int64_t s = 0; s < n; ++s) {
    if (seen[s]) continue;
    comp.clear();
    stack.assign(1, s);
    seen[s] = 1;
    const T v = R[s];
    int64_t best = INT64_MAX;
    while (!stack.empty()) {
      const int64_t i = stack.back();
      stack.pop_back();
      comp.push_back(i);
      const int64_t y = i / W, x = i % W;
      int64_t key = INT64_MAX;
      if (R[i] == mask[i]) key = i;
      else if (R[i] == marker[i]) key = n + i;
      else if (R[i] == (T)0 && (y == 0 || y == H - 1 || x == 0 || x == W - 1)) key = 2 * n;
      best = std::min(best, key);
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          if (!dy && !dx) continue;
          if (conn == 4 && dy && dx) continue;
          const int64_t yy = y + dy, xx = x + dx;
          if (yy < 0 || yy >= H || xx < 0 || xx >= W) continue;
          const int64_t j = yy * W + xx;
          if (!seen[j] && R[j] == v) {
            seen[j] = 1;
            stack.push_back(j);
          }
        }
    }
    int32_t pv;
    if (best < n) pv = (int32_t)~best;
    else if (best < 2 * n) pv = (int32_t)(best - n);
    else if (best == 2 * n) pv = INT32_MIN;
    else return false;
    for (int64_t i : comp) prov[i] = pv;
  }
  return true;
}

// Adjoint of R with respect to marker and mask for an upstream gradient g:
//   dmarker(q) = sum of g(p) over p with prov(p) = q,  dmask(q) = sum over prov(p) = ~q.
// The CPU reference gradient: for every source q, the exact sum of g(p) over the pixels whose
// provenance is q, rounded once to float (nearest, ties to even).  Each g is taken as an exact
// multiple of 2^-96 (every float32 from 2^-73 up is one; smaller magnitudes are rounded to the
// nearest multiple, ties to even), summed in 128-bit integers, and the sum * 2^-96 is rounded
// to float by explicit integer rounding.  |g| >= 2^31 (or not finite) returns false.
inline bool fix96_of(float g, __int128& out) {
  if (!std::isfinite(g) || std::fabs(g) >= 2147483648.0f) return false;
  int e = 0;
  const float fr = std::frexp(std::fabs(g), &e);  // |g| = fr * 2^e, fr in [0.5, 1)
  if (fr == 0.0f) {
    out = 0;
    return true;
  }
  const int64_t m = (int64_t)std::ldexp(fr, 24);  // |g| = m * 2^(e - 24), m < 2^24 exact
  const int s = e - 24 + 96;
  __int128 v;
  if (s >= 0) {
    v = (__int128)m << s;
  } else if (-s >= 40) {
    v = 0;
  } else {
    const int r = -s;
    const int64_t q = m >> r, rem = m & ((int64_t(1) << r) - 1), half = int64_t(1) << (r - 1);
    v = q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
  }
  out = g < 0 ? -v : v;
  return true;
}

inline float fix96_to_float(__int128 S) {
  if (S == 0) return 0.0f;
  const bool neg = S < 0;
  unsigned __int128 M = neg ? (unsigned __int128)(-S) : (unsigned __int128)S;
  int lead = 127;
  while (!((M >> lead) & 1)) --lead;
  int e = lead - 96;
  uint32_t m;
  if (lead <= 23) {
    m = (uint32_t)(M << (23 - lead));
  } else {
    const int r = lead - 23;
    m = (uint32_t)(M >> r);
    const unsigned __int128 rem = M & (((unsigned __int128)1 << r) - 1), half = (unsigned __int128)1 << (r - 1);
    if (rem > half || (rem == half && (m & 1u))) ++m;
    if (m == (1u << 24)) {
      m >>= 1;
      ++e;
    }
  }
  const float f = std::ldexp((float)m, e - 23);  // m < 2^24 and the exponent in range: exact
  return neg ? -f : f;
}

inline bool recon_grad_fixed(const float* g, const int32_t* prov, int64_t n, float* dmarker, float* dmask) {
  std::vector<__int128> am((size_t)n, 0), ak((size_t)n, 0);
  bool ok = true;
  for (int64_t p = 0; p < n; ++p) {
    const int32_t v = prov[p];
    if (v == INT32_MIN) continue;
    const int64_t q = v >= 0 ? v : ~(int64_t)v;
    if (q >= n) continue;
    __int128 f;
    if (!fix96_of(g[p], f)) {
      ok = false;
      continue;
    }
    if (v >= 0) am[q] += f;
    else ak[q] += f;
  }
  for (int64_t q = 0; q < n; ++q) {
    dmarker[q] = fix96_to_float(am[q]);
    dmask[q] = fix96_to_float(ak[q]);
  }
  return ok;
}

// Flat erosion (MAX = false) / dilation (MAX = true) of a u8 image by a k x k element, as
// cv::erode / cv::dilate compute them on the bordered image that morphOpen builds: at (y, x)
// the min / max over the element's non-zero (i, j) of src(y + i - c, x + j - c), c = (k-1)/2,
// pixels outside the image reading `pad`.
inline void morph_u8(const uint8_t* src, int64_t H, int64_t W, const uint8_t* kern, int k, bool max_op,
                     uint8_t pad, uint8_t* dst) {
  const int c = (k - 1) / 2;
  for (int64_t y = 0; y < H; ++y)
    for (int64_t x = 0; x < W; ++x) {
      int v = max_op ? 0 : 255;
      for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) {
          if (!kern[i * k + j]) continue;
          const int64_t yy = y + i - c, xx = x + j - c;
          const int p = (yy < 0 || yy >= H || xx < 0 || xx >= W) ? pad : src[yy * W + xx];
          v = max_op ? (p > v ? p : v) : (p < v ? p : v);
        }
      dst[y * W + x] = (uint8_t)v;
    }
}

// src/segment/MorphologicOperations.cpp:2459-2493 (morphOpen<unsigned char>): copyMakeBorder by
// c with 255, erode, crop; copyMakeBorder by c with 0, dilate, crop.  The crops keep only pixels
// whose element reach stays inside the bordered image, so OpenCV's own border mode never
// enters.
inline void morph_open_u8(const uint8_t* src, int64_t H, int64_t W, const uint8_t* kern, int k, uint8_t* dst) {
  std::vector<uint8_t> eroded((size_t)(H * W));
  morph_u8(src, H, W, kern, k, false, 255, eroded.data());
  morph_u8(eroded.data(), H, W, kern, k, true, 0, dst);
}

// Exact Euclidean distance to the nearest zero pixel of a u8 mask: the definition behind
// OpenCV's distanceTransform(CV_DIST_L2, CV_DIST_MASK_PRECISE) at HistologicalEntities.cpp:341,
// as float = the correctly rounded square root of the integer squared distance.  Column
// distances first, then per pixel an outward search along the row that stops once the column
// offset alone exceeds the best distance found.  No zero pixel: +inf.  basins: -distance on
// non-zero pixels, -FLT_MAX on zero ones (HistologicalEntities.cpp:347-356).
inline void edt_exact_u8(const uint8_t* m, int64_t H, int64_t W, bool basins, float* out) {
  const int64_t inf = H + W;
  std::vector<int64_t> g((size_t)(H * W));
  for (int64_t x = 0; x < W; ++x) {
    int64_t d = inf;
    for (int64_t y = 0; y < H; ++y) {
      d = m[y * W + x] == 0 ? 0 : std::min(d + 1, inf);
      g[y * W + x] = d;
    }
    d = inf;
    for (int64_t y = H - 1; y >= 0; --y) {
      d = m[y * W + x] == 0 ? 0 : std::min(d + 1, inf);
      g[y * W + x] = std::min(g[y * W + x], d);
    }
  }
  for (int64_t y = 0; y < H; ++y)
    for (int64_t x = 0; x < W; ++x) {
      const int64_t* gr = &g[y * W];
      int64_t best = gr[x] * gr[x];
      for (int64_t k = 1; k < W && k * k < best; ++k) {
        if (x - k >= 0) best = std::min(best, k * k + gr[x - k] * gr[x - k]);
        if (x + k < W) best = std::min(best, k * k + gr[x + k] * gr[x + k]);
      }
      const float d = best >= inf * inf ? std::numeric_limits<float>::infinity() : (float)std::sqrt((double)best);
      out[y * W + x] = basins ? (m[y * W + x] != 0 ? -d : -std::numeric_limits<float>::max()) : d;
    }
}

// The reference's own queue-based transform: src/segment/MorphologicOperations.cpp:197-275
// (nscale::distanceTransform) with checkDistNeighbors8 (31-89), propagateDist (91-121) and
// propagateDist8 (123-195).  Zero pixels with a non-zero 8-neighbour seed a FIFO queue in raster
// order; a popped pixel offers its nearest zero pixel to its neighbours (upper left, upper
// right, upper, lower left, lower right, lower, left, right), which take it when it is strictly
// closer (float distances) and are queued again.  Non-zero pixels start at the index
// rows*cols*3.  The result is the distance to the nearest zero pixel found.
inline void dist_queue_u8(const uint8_t* m, int64_t H, int64_t W, float* out) {
  std::vector<int> nn((size_t)(H * W));
  std::deque<std::pair<int, int>> q;
  const int far = (int)(H * W * 3);
  auto fdist = [&](int64_t px, int64_t py, int idx) {
    const double dx = (double)(px - idx % W), dy = (double)(py - idx / W);
    return (float)std::sqrt(dx * dx + dy * dy);
  };
  for (int64_t y = 0; y < H; ++y)
    for (int64_t x = 0; x < W; ++x) {
      nn[y * W + x] = far;
      if (m[y * W + x] != 0) continue;
      nn[y * W + x] = (int)(y * W + x);
      bool edge = false;
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const int64_t yy = y + dy, xx = x + dx;
          if ((dx || dy) && yy >= 0 && yy < H && xx >= 0 && xx < W && m[yy * W + xx] != 0) edge = true;
        }
      if (edge) q.emplace_back((int)x, (int)y);
    }
  const int order[8][2] = {{-1, -1}, {1, -1}, {0, -1}, {-1, 1}, {1, 1}, {0, 1}, {-1, 0}, {1, 0}};
  while (!q.empty()) {
    const int x = q.front().first, y = q.front().second;
    q.pop_front();
    for (const auto& o : order) {
      const int64_t tx = x + o[0], ty = y + o[1];
      if (tx < 0 || tx >= W || ty < 0 || ty >= H) continue;
      const int cur = nn[y * W + x];
      if (fdist(tx, ty, cur) < fdist(tx, ty, nn[ty * W + tx])) {
        nn[ty * W + tx] = cur;
        q.emplace_back((int)tx, (int)ty);
      }
    }
  }
  for (int64_t y = 0; y < H; ++y)
    for (int64_t x = 0; x < W; ++x) {
      const int64_t c = nn[y * W + x], dx = x - c % W, dy = y - c / W;
      out[y * W + x] = (float)std::sqrt((double)(dx * dx + dy * dy));
    }
}

}  // namespace orc
