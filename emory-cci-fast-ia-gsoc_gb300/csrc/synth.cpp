// Deterministic synthetic pathology-tile generator (host code).
//
// The reference's tests read 4096x4096 pathology tiles from a data directory that is not
// distributed with it (test/TestUtils.h:9-17, CMakeLists.txt:171).  This generator stands
// in for those tiles with the same shapes and value ranges: a bright, noisy background
// with dark elliptical "nuclei", the input that HistologicalEntities.cpp:155-214 feeds to
// imreconstruct.
//
// Definition (every step is integer arithmetic or a single IEEE-754 double operation, and
// the file is compiled with -ffp-contract=off, so x86-64 and aarch64 produce the same
// bytes):
//   h(seed, stream, i) = splitmix64(splitmix64(seed ^ (stream << 56)) + i)
//   u01(h)            = (h >> 11) * 2^-53                        (double in [0, 1))
//   below(h, n)       = ((h >> 32) * n) >> 32                    (integer in [0, n))
//   background        = 200 + below(h(seed, 0, y*W + x), 31) - 15     (185..215)
//   ellipse k         : cx = u01(h(seed,1,8k))*W, cy = u01(h(seed,1,8k+1))*H,
//                       a = 4 + 16*u01(h(seed,1,8k+2)), b = 4 + 16*u01(h(seed,1,8k+3)),
//                       v = 40 + below(h(seed,1,8k+4), 51)
//                       orientation: first (u, w) = (2*u01 - 1, u01) from stream 2 with
//                       1e-4 < u^2 + w^2 <= 1 (rejection sampling, angle uniform in [0, pi)),
//                       c = u / sqrt(r2), s = w / sqrt(r2)
//   pixel (x, y) is inside ellipse k iff (dx*c + dy*s)^2 * b^2 + (dy*c - dx*s)^2 * a^2
//                       <= a^2 * b^2 with dx = x - cx, dy = y - cy.
//   Ellipses are painted in order k = 0, 1, ...; a later ellipse overwrites an earlier one
//   (no blending).
//   marker = max(mask - 10, 0).
#include <cmath>
#include <cstdint>
#include <cstring>

#include "../../include/nsgb_synth.h"

namespace {

inline uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Stream {
  uint64_t key;
  Stream(uint64_t seed, uint64_t stream) : key(splitmix64(seed ^ (stream << 56))) {}
  uint64_t at(uint64_t i) const { return splitmix64(key + i); }
};

inline double u01(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }
inline uint32_t below(uint64_t h, uint32_t n) { return (uint32_t)(((h >> 32) * (uint64_t)n) >> 32); }

struct Ellipse {
  double cx, cy, a, b, c, s;
  int v;
};

Ellipse draw_ellipse(const Stream& geo, const Stream& dir, int64_t k, int64_t H, int64_t W) {
  Ellipse e;
  e.cx = u01(geo.at(8 * k + 0)) * (double)W;
  e.cy = u01(geo.at(8 * k + 1)) * (double)H;
  e.a = 4.0 + 16.0 * u01(geo.at(8 * k + 2));
  e.b = 4.0 + 16.0 * u01(geo.at(8 * k + 3));
  e.v = 40 + (int)below(geo.at(8 * k + 4), 51);
  e.c = 1.0;
  e.s = 0.0;
  for (int t = 0; t < 32; ++t) {
    double u = 2.0 * u01(dir.at(64 * k + 2 * t)) - 1.0;
    double w = u01(dir.at(64 * k + 2 * t + 1));
    double r2 = u * u + w * w;
    if (r2 > 1e-4 && r2 <= 1.0) {
      double r = std::sqrt(r2);
      e.c = u / r;
      e.s = w / r;
      break;
    }
  }
  return e;
}

}  // namespace

extern "C" {

int nsgb_synth_tile_u8(uint8_t* mask, uint8_t* marker, int64_t H, int64_t W, int64_t pitch,
                       int64_t n_ellipses, uint64_t seed) {
  if (!mask || H <= 0 || W <= 0 || pitch < W || n_ellipses < 0) return -1;
  Stream noise(seed, 0), geo(seed, 1), dir(seed, 2);
  for (int64_t y = 0; y < H; ++y) {
    uint8_t* row = mask + y * pitch;
    for (int64_t x = 0; x < W; ++x) row[x] = (uint8_t)(185 + below(noise.at((uint64_t)(y * W + x)), 31));
  }
  for (int64_t k = 0; k < n_ellipses; ++k) {
    Ellipse e = draw_ellipse(geo, dir, k, H, W);
    double R = e.a > e.b ? e.a : e.b;
    int64_t x0 = (int64_t)std::ceil(e.cx - R), x1 = (int64_t)std::floor(e.cx + R);
    int64_t y0 = (int64_t)std::ceil(e.cy - R), y1 = (int64_t)std::floor(e.cy + R);
    if (x0 < 0) x0 = 0;
    if (y0 < 0) y0 = 0;
    if (x1 > W - 1) x1 = W - 1;
    if (y1 > H - 1) y1 = H - 1;
    double a2 = e.a * e.a, b2 = e.b * e.b, ab2 = a2 * b2;
    for (int64_t y = y0; y <= y1; ++y) {
      double dy = (double)y - e.cy;
      uint8_t* row = mask + y * pitch;
      for (int64_t x = x0; x <= x1; ++x) {
        double dx = (double)x - e.cx;
        double p = dx * e.c + dy * e.s;
        double q = dy * e.c - dx * e.s;
        double lhs = p * p * b2 + q * q * a2;
        if (lhs <= ab2) row[x] = (uint8_t)e.v;
      }
    }
  }
  if (marker) {
    for (int64_t y = 0; y < H; ++y) {
      const uint8_t* m = mask + y * pitch;
      uint8_t* o = marker + y * pitch;
      for (int64_t x = 0; x < W; ++x) o[x] = m[x] > 10 ? (uint8_t)(m[x] - 10) : (uint8_t)0;
    }
  }
  return 0;
}

int nsgb_synth_scale_u16(const uint8_t* src, uint16_t* mask, uint16_t* marker, int64_t n) {
  if (!src || !mask || n < 0) return -1;
  for (int64_t i = 0; i < n; ++i) {
    uint32_t v = (uint32_t)src[i] * 257u;
    mask[i] = (uint16_t)v;
    if (marker) marker[i] = (uint16_t)(v > 2570u ? v - 2570u : 0u);
  }
  return 0;
}

int nsgb_synth_scale_i32(const uint8_t* src, int32_t* mask, int32_t* marker, int64_t n) {
  if (!src || !mask || n < 0) return -1;
  for (int64_t i = 0; i < n; ++i) {
    int32_t v = (int32_t)src[i] * 1000;
    mask[i] = v;
    if (marker) marker[i] = v > 10000 ? v - 10000 : 0;
  }
  return 0;
}

int nsgb_synth_float(float* mask, float* marker, int64_t n, uint64_t seed) {
  if (!mask || n < 0) return -1;
  Stream sm(seed, 4), su(seed, 5);
  for (int64_t i = 0; i < n; ++i) {
    float mv = (float)(sm.at((uint64_t)i) >> 40) * (1.0f / 16777216.0f);
    mask[i] = mv;
    if (marker) {
      float u = 0.5f + (float)(su.at((uint64_t)i) >> 41) * (1.0f / 16777216.0f);
      marker[i] = mv * u;
    }
  }
  return 0;
}

int nsgb_synth_tile_sizes(int32_t* heights, int32_t* widths, int64_t n_tiles, int32_t lo,
                          int32_t hi, uint64_t seed) {
  if (!heights || !widths || n_tiles < 0 || lo <= 0 || hi < lo) return -1;
  Stream st(seed, 3);
  uint32_t span = (uint32_t)(hi - lo + 1);
  for (int64_t t = 0; t < n_tiles; ++t) {
    heights[t] = lo + (int32_t)below(st.at((uint64_t)(2 * t)), span);
    widths[t] = lo + (int32_t)below(st.at((uint64_t)(2 * t + 1)), span);
  }
  return 0;
}

}  // extern "C"
