// C entry points over the CPU oracle (recon_oracle.hpp), for the Python tests and the
// CPU-baseline leg of bench.py.  TEST INFRASTRUCTURE ONLY: the product never calls these.
//
// All images are dense row-major (pitch == width).  dtype codes: 0 = u8, 1 = u16,
// 2 = i32, 3 = f32 (the same codes as the product's C ABI).
#include <atomic>
#include <chrono>
#include <cstdint>
#include <thread>
#include <vector>

#include "recon_oracle.hpp"

namespace {

template <typename F>
int dispatch(int dtype, F&& f) {
  switch (dtype) {
    case 0: f((uint8_t*)nullptr); return 0;
    case 1: f((uint16_t*)nullptr); return 0;
    case 2: f((int32_t*)nullptr); return 0;
    case 3: f((float*)nullptr); return 0;
    default: return -1;
  }
}

// Runs f(0..n-1) on up to `threads` host threads.
template <typename F>
void parallel_for(int64_t n, int threads, F&& f) {
  if (threads < 1) threads = 1;
  std::atomic<int64_t> next{0};
  std::vector<std::thread> pool;
  for (int t = 0; t < threads && t < n; ++t)
    pool.emplace_back([&] {
      for (int64_t i = next++; i < n; i = next++) f(i);
    });
  for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

int orc_imreconstruct(int dtype, const void* marker, const void* mask, int64_t H, int64_t W,
                      int conn, void* out) {
  return dispatch(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    orc::imreconstruct<T>((const T*)marker, (const T*)mask, H, W, conn, (T*)out);
  });
}

int orc_imreconstruct_binary(int dtype, const void* marker, const void* mask, int64_t H,
                             int64_t W, int conn, void* out) {
  return dispatch(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    if constexpr (std::is_integral_v<T>)
      orc::imreconstruct_binary<T>((const T*)marker, (const T*)mask, H, W, conn, (T*)out);
  });
}

int orc_imfill_holes(int dtype, const void* image, int64_t H, int64_t W, int binary, int conn,
                     void* out) {
  return dispatch(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    if constexpr (std::is_integral_v<T>) {
      orc::imfill_holes<T>((const T*)image, H, W, binary != 0, conn, (T*)out);
    } else {
      if (!binary) orc::imfill_holes<T>((const T*)image, H, W, false, conn, (T*)out);
    }
  });
}

int orc_imhmin(int dtype, const void* image, int64_t H, int64_t W, double h, int conn, void* out) {
  return dispatch(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    orc::imhmin<T>((const T*)image, H, W, (T)h, conn, (T*)out);
  });
}

int orc_bwselect(int dtype, const void* image, const void* seeds, int64_t H, int64_t W, int conn,
                 void* out) {
  return dispatch(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    if constexpr (std::is_integral_v<T>)
      orc::bwselect<T>((const T*)image, (const T*)seeds, H, W, conn, (T*)out);
  });
}

int orc_threshold_gt(int dtype, const void* in, int64_t n, double k, uint8_t* out) {
  return dispatch(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    orc::threshold_gt<T>((const T*)in, n, k, out);
  });
}

int orc_morph_open_u8(const uint8_t* in, int64_t H, int64_t W, const uint8_t* kern, int k, uint8_t* out) {
  if (k < 1 || k % 2 == 0) return -1;
  orc::morph_open_u8(in, H, W, kern, k, out);
  return 0;
}

int orc_edt_exact_u8(const uint8_t* m, int64_t H, int64_t W, int basins, float* out) {
  orc::edt_exact_u8(m, H, W, basins != 0, out);
  return 0;
}

int orc_dist_queue_u8(const uint8_t* m, int64_t H, int64_t W, float* out) {
  orc::dist_queue_u8(m, H, W, out);
  return 0;
}

int32_t orc_bwlabel2(const uint8_t* bin, int64_t H, int64_t W, int conn, int relab, int32_t* out) {
  return orc::bwlabel2(bin, H, W, conn, relab != 0, out);
}

int32_t orc_bounding_box(const int32_t* labels, int64_t H, int64_t W, int32_t bgval, int32_t* out, int64_t cap) {
  return orc::cc_bounding_box(labels, W, H, bgval, out, cap);
}

int32_t orc_bwareaopen2(const void* image, int labeled, int flatten, int32_t minSize, int32_t maxSize,
                        int conn, int64_t H, int64_t W, int32_t* labels_out, uint8_t* flat_out) {
  return orc::bwareaopen2(image, labeled != 0, flatten != 0, minSize, maxSize, conn, H, W,
                          labels_out, flat_out);
}

// The single-tile chain: (a) reconstruction by dilation, (b) `> thr`, (c) binary hole fill,
// (d) bwlabel2 with raster relabel, (e) bwareaopen2 on the filled image.  Any output pointer
// may be null.  Returns the number of components kept by (e), or -1 on a bad dtype.
int32_t orc_chain(int dtype, const void* marker, const void* mask, int64_t H, int64_t W,
                  int recon_conn, double thr, int fill_conn, int label_conn, int32_t area_min,
                  int32_t area_max, void* recon_out, uint8_t* thr_out, uint8_t* fill_out,
                  int32_t* label_out, int32_t* n_labels, uint8_t* area_out) {
  const int64_t n = H * W;
  int32_t kept = -1;
  dispatch(dtype, [&](auto* tag) {
    using T = std::remove_pointer_t<decltype(tag)>;
    std::vector<T> rec((size_t)n);
    orc::imreconstruct<T>((const T*)marker, (const T*)mask, H, W, recon_conn, rec.data());
    std::vector<uint8_t> b((size_t)n), f((size_t)n), a((size_t)n);
    orc::threshold_gt<T>(rec.data(), n, thr, b.data());
    orc::imfill_holes<uint8_t>(b.data(), H, W, true, fill_conn, f.data());
    std::vector<int32_t> lab((size_t)n);
    int32_t nl = orc::bwlabel2(f.data(), H, W, label_conn, true, lab.data());
    kept = orc::bwareaopen2(f.data(), false, true, area_min, area_max, label_conn, H, W, nullptr, a.data());
    if (recon_out) std::memcpy(recon_out, rec.data(), (size_t)n * sizeof(T));
    if (thr_out) std::memcpy(thr_out, b.data(), (size_t)n);
    if (fill_out) std::memcpy(fill_out, f.data(), (size_t)n);
    if (label_out) std::memcpy(label_out, lab.data(), (size_t)n * sizeof(int32_t));
    if (n_labels) *n_labels = nl;
    if (area_out) std::memcpy(area_out, a.data(), (size_t)n);
  });
  return kept;
}

// Runs the u8 chain `reps` times on each of `threads` host threads (each thread on its own
// copy of the inputs, as independent tiles) and returns the wall time in seconds.  Used
// only to time the CPU baseline.
double orc_chain_replicas_seconds(const uint8_t* marker, const uint8_t* mask, int64_t H, int64_t W,
                                  int threads, int reps) {
  if (threads < 1) threads = 1;
  const int64_t n = H * W;
  std::vector<std::vector<uint8_t>> mk(threads), ms(threads);
  for (int t = 0; t < threads; ++t) {
    mk[t].assign(marker, marker + n);
    ms[t].assign(mask, mask + n);
  }
  auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> pool;
  for (int t = 0; t < threads; ++t) {
    pool.emplace_back([&, t] {
      for (int r = 0; r < reps; ++r)
        orc_chain(0, mk[t].data(), ms[t].data(), H, W, 8, 128.0, 4, 8, 11, 1000, nullptr,
                  nullptr, nullptr, nullptr, nullptr, nullptr);
    });
  }
  for (auto& th : pool) th.join();
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

// Float32 reconstruction by dilation with provenance over a stack of `B` dense H x W images,
// one host thread per image.  Returns 0, or -1 if a plateau had no source.
int orc_recon_f32_prov(const float* marker, const float* mask, int64_t B, int64_t H, int64_t W, int conn,
                       float* R, int32_t* prov, int threads) {
  const int64_t n = H * W;
  std::vector<int> bad((size_t)B, 0);
  parallel_for(B, threads, [&](int64_t b) {
    orc::imreconstruct<float>(marker + b * n, mask + b * n, H, W, conn, R + b * n);
    bad[b] = !orc::recon_provenance<float>(marker + b * n, mask + b * n, R + b * n, H, W, conn, prov + b * n);
  });
  for (int v : bad)
    if (v) return -1;
  return 0;
}

// The CPU reference gradient (exact sums rounded once, see recon_grad_fixed) over B stacked
// images.  Returns 0, or -1 if some |g| >= 2^31 or is not finite.
int orc_recon_f32_grad(const float* g, const int32_t* prov, int64_t B, int64_t H, int64_t W, float* dmarker,
                       float* dmask, int threads) {
  const int64_t n = H * W;
  std::vector<int> bad((size_t)B, 0);
  parallel_for(B, threads, [&](int64_t b) {
    bad[b] = !orc::recon_grad_fixed(g + b * n, prov + b * n, n, dmarker + b * n, dmask + b * n);
  });
  for (int v : bad)
    if (v) return -1;
  return 0;
}

// Central finite differences of L = sum_p g(p) R(p) for one H x W float image, evaluated in
// float64: for each listed pixel, marker (kind 0) and mask (kind 1) are moved by +-h and the
// reconstruction recomputed in double.  fd = sum_p g(p) (R+(p) - R-(p)) / 2h.  valid = the
// provenance map at x+h and at x-h equals the one at x (otherwise the function is not
// locally linear there and the pixel is rejected).
void orc_recon_fd(const float* marker, const float* mask, const float* g, int64_t H, int64_t W, int conn,
                  const int64_t* idx, int64_t n_idx, double h, double* fd, int32_t* valid, int threads) {
  const int64_t n = H * W;
  std::vector<double> mk(marker, marker + n), ms(mask, mask + n), R0((size_t)n);
  std::vector<int32_t> p0((size_t)n);
  orc::imreconstruct<double>(mk.data(), ms.data(), H, W, conn, R0.data());
  orc::recon_provenance<double>(mk.data(), ms.data(), R0.data(), H, W, conn, p0.data());
  parallel_for(2 * n_idx, threads, [&](int64_t t) {
    const int64_t i = idx[t / 2];
    const int kind = (int)(t % 2);
    std::vector<double> a = kind == 0 ? mk : ms;
    const std::vector<double>& other = kind == 0 ? ms : mk;
    std::vector<double> Rp((size_t)n), Rm((size_t)n);
    std::vector<int32_t> pp((size_t)n), pm((size_t)n);
    const double x0 = a[i];
    a[i] = x0 + h;
    const double* mkp = kind == 0 ? a.data() : other.data();
    const double* msp = kind == 0 ? other.data() : a.data();
    orc::imreconstruct<double>(mkp, msp, H, W, conn, Rp.data());
    bool ok = orc::recon_provenance<double>(mkp, msp, Rp.data(), H, W, conn, pp.data());
    a[i] = x0 - h;
    orc::imreconstruct<double>(mkp, msp, H, W, conn, Rm.data());
    ok = ok && orc::recon_provenance<double>(mkp, msp, Rm.data(), H, W, conn, pm.data());
    double s = 0.0;
    for (int64_t p = 0; p < n; ++p)
      if (Rp[p] != Rm[p]) s += (double)g[p] * (Rp[p] - Rm[p]);
    fd[t] = s / (2.0 * h);
    valid[t] = ok && pp == p0 && pm == p0;
  });
}

}  // extern "C"
