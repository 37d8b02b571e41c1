// Shared device helpers: element traits for the packed compute words, bounded waits,
// device status words, and the grid barrier used by the persistent kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/nsgb.h"

#define NSGB_FULL 0xFFFFFFFFu

namespace nsgb {

// Device status words (one int in every workspace).  Values map to nsgb_status.
enum DevStatus : int {
  kDevOk = 0,
  kDevNotConverged = NSGB_ERR_NOT_CONVERGED,
  kDevTimeout = NSGB_ERR_TIMEOUT,
  kDevOverflow = NSGB_ERR_QUEUE_OVERFLOW,
};

// Every device-side spin gives up after this many polls (each poll sleeps ~256 ns, so the
// limit is roughly 2 s) and records kDevTimeout instead of waiting forever.
constexpr long long kSpinLimit = 1ll << 23;

__device__ __forceinline__ void set_status(int* status, int code) {
  atomicCAS(status, 0, code);
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_acquire_u(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Sense-free generation barrier over all CTAs of a cooperative launch.  `bar[0]` counts
// arrivals, `bar[1]` is the generation.  Returns false (and sets the status) if a wait timed
// out; the caller then leaves its loop.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned nblocks, int* status) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    s_ok = 1;
    unsigned gen = ld_acquire_u(bar + 1);
    __threadfence();
    unsigned arrived = atomicAdd(bar, 1u) + 1u;
    if (arrived == nblocks) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long spins = 0;
      while (ld_acquire_u(bar + 1) == gen) {
        if (++spins > kSpinLimit) {
          set_status(status, kDevTimeout);
          s_ok = 0;
          break;
        }
        __nanosleep(256);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return s_ok != 0;
}

// ---------------------------------------------------------------------------------------
// Packed compute words.  A 32-bit word carries E elements of the working type:
//   u8 and u16 pixels -> two 16-bit lanes (native max.u16x2 / min.u16x2),
//   i32 -> one signed 32-bit lane, f32 -> one float lane.
// LOW is the inert value used outside the image (below every pixel), HIGH the identity
// upper bound of a clamp, FLIP the xor that reverses the order (dual operator).

__device__ __forceinline__ uint32_t vmax_u16x2(uint32_t a, uint32_t b) {
  uint32_t r;
  asm("max.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint32_t vmin_u16x2(uint32_t a, uint32_t b) {
  uint32_t r;
  asm("min.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
  return r;
}

template <typename T>
struct Px;

template <>
struct Px<uint8_t> {
  static constexpr int E = 2;
  static constexpr uint32_t LOW = 0u, HIGH = 0xFFFFFFFFu, FLIP = 0x00FF00FFu, ZERO = 0u;
  static constexpr uint32_t ELEM_FLIP = 0xFFu;
  __device__ static __forceinline__ uint32_t vmax(uint32_t a, uint32_t b) { return vmax_u16x2(a, b); }
  __device__ static __forceinline__ uint32_t vmin(uint32_t a, uint32_t b) { return vmin_u16x2(a, b); }
  // element k <- element k-1, element 0 <- last element of prev
  __device__ static __forceinline__ uint32_t from_left(uint32_t prev, uint32_t cur) { return __funnelshift_l(prev, cur, 16); }
  // element k <- element k+1, last element <- element 0 of next
  __device__ static __forceinline__ uint32_t from_right(uint32_t cur, uint32_t next) { return __funnelshift_r(cur, next, 16); }
  __device__ static __forceinline__ uint32_t elem(uint32_t w, int k) { return (w >> (16 * k)) & 0xFFFFu; }
  __device__ static __forceinline__ uint32_t pack(uint32_t e0, uint32_t e1) { return e0 | (e1 << 16); }
  __device__ static __forceinline__ uint32_t as_last(uint32_t e) { return e << 16; }
  __device__ static __forceinline__ uint32_t as_first(uint32_t e) { return e; }
  __device__ static __forceinline__ uint32_t load_elem(const uint8_t* p) { return (uint32_t)__ldcg(p); }
  __device__ static __forceinline__ uint32_t load_elem_ro(const uint8_t* p) { return (uint32_t)__ldg(p); }
  __device__ static __forceinline__ void store_elem(uint8_t* p, uint32_t v) { __stcg(p, (uint8_t)v); }
  // Ordered comparison of single elements (already extracted).
  __device__ static __forceinline__ bool lt(uint32_t a, uint32_t b) { return a < b; }
  __device__ static __forceinline__ uint32_t emax(uint32_t a, uint32_t b) { return a > b ? a : b; }
  __device__ static __forceinline__ uint32_t emin(uint32_t a, uint32_t b) { return a < b ? a : b; }
};

template <>
struct Px<uint16_t> {
  static constexpr int E = 2;
  static constexpr uint32_t LOW = 0u, HIGH = 0xFFFFFFFFu, FLIP = 0xFFFFFFFFu, ZERO = 0u;
  static constexpr uint32_t ELEM_FLIP = 0xFFFFu;
  __device__ static __forceinline__ uint32_t vmax(uint32_t a, uint32_t b) { return vmax_u16x2(a, b); }
  __device__ static __forceinline__ uint32_t vmin(uint32_t a, uint32_t b) { return vmin_u16x2(a, b); }
  __device__ static __forceinline__ uint32_t from_left(uint32_t prev, uint32_t cur) { return __funnelshift_l(prev, cur, 16); }
  __device__ static __forceinline__ uint32_t from_right(uint32_t cur, uint32_t next) { return __funnelshift_r(cur, next, 16); }
  __device__ static __forceinline__ uint32_t elem(uint32_t w, int k) { return (w >> (16 * k)) & 0xFFFFu; }
  __device__ static __forceinline__ uint32_t pack(uint32_t e0, uint32_t e1) { return e0 | (e1 << 16); }
  __device__ static __forceinline__ uint32_t as_last(uint32_t e) { return e << 16; }
  __device__ static __forceinline__ uint32_t as_first(uint32_t e) { return e; }
  __device__ static __forceinline__ uint32_t load_elem(const uint16_t* p) { return (uint32_t)__ldcg(p); }
  __device__ static __forceinline__ uint32_t load_elem_ro(const uint16_t* p) { return (uint32_t)__ldg(p); }
  __device__ static __forceinline__ void store_elem(uint16_t* p, uint32_t v) { __stcg(p, (uint16_t)v); }
  __device__ static __forceinline__ bool lt(uint32_t a, uint32_t b) { return a < b; }
  __device__ static __forceinline__ uint32_t emax(uint32_t a, uint32_t b) { return a > b ? a : b; }
  __device__ static __forceinline__ uint32_t emin(uint32_t a, uint32_t b) { return a < b ? a : b; }
};

template <>
struct Px<int32_t> {
  static constexpr int E = 1;
  static constexpr uint32_t LOW = 0x80000000u, HIGH = 0x7FFFFFFFu, FLIP = 0xFFFFFFFFu, ZERO = 0u;
  static constexpr uint32_t ELEM_FLIP = 0xFFFFFFFFu;
  __device__ static __forceinline__ uint32_t vmax(uint32_t a, uint32_t b) { return (uint32_t)max((int)a, (int)b); }
  __device__ static __forceinline__ uint32_t vmin(uint32_t a, uint32_t b) { return (uint32_t)min((int)a, (int)b); }
  __device__ static __forceinline__ uint32_t from_left(uint32_t prev, uint32_t) { return prev; }
  __device__ static __forceinline__ uint32_t from_right(uint32_t, uint32_t next) { return next; }
  __device__ static __forceinline__ uint32_t elem(uint32_t w, int) { return w; }
  __device__ static __forceinline__ uint32_t pack(uint32_t e0, uint32_t) { return e0; }
  __device__ static __forceinline__ uint32_t as_last(uint32_t e) { return e; }
  __device__ static __forceinline__ uint32_t as_first(uint32_t e) { return e; }
  __device__ static __forceinline__ uint32_t load_elem(const int32_t* p) { return (uint32_t)__ldcg(p); }
  __device__ static __forceinline__ uint32_t load_elem_ro(const int32_t* p) { return (uint32_t)__ldg(p); }
  __device__ static __forceinline__ void store_elem(int32_t* p, uint32_t v) { __stcg(p, (int32_t)v); }
  __device__ static __forceinline__ bool lt(uint32_t a, uint32_t b) { return (int)a < (int)b; }
  __device__ static __forceinline__ uint32_t emax(uint32_t a, uint32_t b) { return vmax(a, b); }
  __device__ static __forceinline__ uint32_t emin(uint32_t a, uint32_t b) { return vmin(a, b); }
};

template <>
struct Px<float> {
  static constexpr int E = 1;
  static constexpr uint32_t LOW = 0xFF800000u, HIGH = 0x7F800000u, FLIP = 0x80000000u, ZERO = 0u;
  static constexpr uint32_t ELEM_FLIP = 0x80000000u;
  __device__ static __forceinline__ uint32_t vmax(uint32_t a, uint32_t b) {
    return __float_as_uint(fmaxf(__uint_as_float(a), __uint_as_float(b)));
  }
  __device__ static __forceinline__ uint32_t vmin(uint32_t a, uint32_t b) {
    return __float_as_uint(fminf(__uint_as_float(a), __uint_as_float(b)));
  }
  __device__ static __forceinline__ uint32_t from_left(uint32_t prev, uint32_t) { return prev; }
  __device__ static __forceinline__ uint32_t from_right(uint32_t, uint32_t next) { return next; }
  __device__ static __forceinline__ uint32_t elem(uint32_t w, int) { return w; }
  __device__ static __forceinline__ uint32_t pack(uint32_t e0, uint32_t) { return e0; }
  __device__ static __forceinline__ uint32_t as_last(uint32_t e) { return e; }
  __device__ static __forceinline__ uint32_t as_first(uint32_t e) { return e; }
  __device__ static __forceinline__ uint32_t load_elem(const float* p) { return __float_as_uint(__ldcg(p)); }
  __device__ static __forceinline__ uint32_t load_elem_ro(const float* p) { return __float_as_uint(__ldg(p)); }
  __device__ static __forceinline__ void store_elem(float* p, uint32_t v) { __stcg(p, __uint_as_float(v)); }
  __device__ static __forceinline__ bool lt(uint32_t a, uint32_t b) { return __uint_as_float(a) < __uint_as_float(b); }
  __device__ static __forceinline__ uint32_t emax(uint32_t a, uint32_t b) { return vmax(a, b); }
  __device__ static __forceinline__ uint32_t emin(uint32_t a, uint32_t b) { return vmin(a, b); }
};

// Argument checks shared by every entry point.  Each dimension is bounded before the product
// is formed, so a wrapped product cannot pass.
inline bool valid_dims(int64_t rows, int64_t cols) {
  return rows > 0 && cols > 0 && rows < INT32_MAX && cols < INT32_MAX && rows * cols < (int64_t)INT32_MAX;
}
inline bool valid_pitch(int64_t pitch, int64_t cols, int esz) {
  return esz > 0 && pitch >= cols * esz && pitch % esz == 0;
}
inline bool valid_conn(int conn) { return conn == 4 || conn == 8; }

inline int elem_size(int dtype) {
  switch (dtype) {
    case NSGB_U8: return 1;
    case NSGB_U16: return 2;
    case NSGB_I32: return 4;
    case NSGB_F32: return 4;
    default: return 0;
  }
}

}  // namespace nsgb
