// Union-find connected-component labelling on GB300 (internal templates).
//
// Reference semantics: ConnComponents::label (fastIA-master/src/segment/ConnComponents.cpp:
// 52-86) joins equal-valued non-zero neighbours (left, up, and up-left / up-right for
// 8-connectivity) and always hooks the larger root under the smaller one (merge, 34-43), so
// every component ends labelled with its smallest raster index; background is bgval.  The GPU
// reference (cuda/ccl_uf.cu:64-157, UF_local / UF_global / UF_final) uses the same
// min-index rule with atomicMin.  This implementation keeps that rule (so labels are
// bit-identical) with its own schedule:
//   1. ccl_local: 32x32 tile per CTA; union-find in shared memory with atomicMin hooking;
//      writes the tile-local root's global index and (optionally) each local root's area.
//   2. ccl_merge: one thread per tile-perimeter pixel joins it with its forward neighbours
//      in other tiles (global atomicMin hooking; a failed hook retries with the new parent).
//   3. ccl_flatten: every foreground pixel points directly at its root; local-root areas are
//      added into the root's area; optional "seed" pixels set a bit on their root.
// Roots are exactly the pixels with L[i] == i.  Classifiers (the `Cls` template argument)
// return a pixel's class (0 = background; equal non-zero classes are joined), so the same
// kernels serve bwlabel (class = pixel value), hole filling (class = "not foreground"),
// binary reconstruction and bwselect (class = "mask non-zero").
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace nsgb {
namespace ccl {

constexpr int kTile = 32;      // tile edge (pixels)
constexpr int kThreads = 256;  // 32 x 8 threads, 4 rows each

// Root of x in a shared-memory forest, halving the path on the way (every node on it is
// re-pointed to its grandparent; a concurrent hook of a root is never overwritten because
// roots are not written here).
__device__ __forceinline__ int s_find(volatile int* s, int x) {
  for (;;) {
    const int p = s[x];
    if (p == x) return x;
    const int g = s[p];
    if (g == p) return p;
    s[x] = g;
    x = g;
  }
}

__device__ __forceinline__ void s_union(int* s, int a, int b) {
  for (;;) {
    a = s_find(s, a);
    b = s_find(s, b);
    if (a == b) return;
    if (a < b) {
      const int t = a;
      a = b;
      b = t;
    }
    const int old = atomicMin(&s[a], b);
    if (old == a) return;
    a = old;
  }
}

// Root of x in the global forest with path halving.  The halving write is an atomicMin: a
// parent link only ever moves to a smaller index (an ancestor), so it can never undo another
// thread's write of the root itself (the smallest index on the path).
__device__ __forceinline__ int g_find(int* L, int x) {
  for (;;) {
    const int p = ld_relaxed(L + x);
    if (p == x) return x;
    const int g = ld_relaxed(L + p);
    if (g == p) return p;
    atomicMin(L + x, g);
    x = g;
  }
}

__device__ __forceinline__ void g_union(int* L, int a, int b) {
  for (;;) {
    a = g_find(L, a);
    b = g_find(L, b);
    if (a == b) return;
    if (a < b) {
      const int t = a;
      a = b;
      b = t;
    }
    const int old = atomicMin(&L[a], b);
    if (old == a) return;
    a = old;
  }
}

// L: dense H x W int32 (index y*W + x).  A (optional): dense int32, receives each local root's
// pixel count at the root and 0 elsewhere.
//
// Each warp owns tile rows (lane = column).  Runs of equal class along a row are found with a
// ballot and start out joined (label = run start), so unions are only needed where runs of
// adjacent rows touch: at a pixel that starts its run or sits under the start of a run above
// (and, for 8-connectivity, diagonally past the two ends of the run).  That is one union per
// touching pair of runs instead of one per pixel pair.
template <class Cls, int CONN>
__global__ void __launch_bounds__(kThreads) ccl_local(Cls cls, int H, int W, int* __restrict__ L,
                                                      int* __restrict__ A) {
  __shared__ int s_lab[kTile * kTile];
  __shared__ int s_cnt[kTile * kTile];
  __shared__ uint8_t s_c[kTile * kTile];
  const int x0 = blockIdx.x * kTile, y0 = blockIdx.y * kTile;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  uint8_t c[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int ly = ty + 8 * k, i = ly * kTile + tx;
    const int gy = y0 + ly, gx = x0 + tx;
    c[k] = (uint8_t)((gy < H && gx < W) ? cls(gy, gx) : 0u);
    s_c[i] = c[k];
    s_cnt[i] = 0;
  }
  __syncwarp();
  unsigned same_left[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int ly = ty + 8 * k, i = ly * kTile + tx;
    const uint8_t left = __shfl_up_sync(NSGB_FULL, c[k], 1);
    same_left[k] = __ballot_sync(NSGB_FULL, tx > 0 && c[k] != 0 && left == c[k]);
    // run start: highest lane <= tx whose pixel does not continue a run from the left
    const unsigned starts = ~same_left[k] & (0xFFFFFFFFu >> (31 - tx));
    const int rs = 31 - __clz(starts);
    s_lab[i] = c[k] ? ly * kTile + rs : -1;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int ly = ty + 8 * k, i = ly * kTile + tx;
    const uint8_t v = c[k];
    if (!v || ly == 0) continue;
    const bool run_start = !((same_left[k] >> tx) & 1u);
    const int u = i - kTile;
    const uint8_t up = s_c[u];
    const bool up_start = up != 0 && !(tx > 0 && s_c[u - 1] == up);
    if (up == v && (run_start || up_start)) s_union(s_lab, i, u);
    if (CONN == 8) {
      if (run_start && tx > 0 && s_c[u - 1] == v) s_union(s_lab, i, u - 1);
      const bool run_end = (tx == kTile - 1) || s_c[i + 1] != v;
      if (run_end && tx < kTile - 1 && s_c[u + 1] == v) s_union(s_lab, i, u + 1);
    }
  }
  __syncthreads();
  int root[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int ly = ty + 8 * k, i = ly * kTile + tx;
    root[k] = c[k] ? s_find(s_lab, i) : -1;
  }
  if (A) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int r = root[k];
      const unsigned peers = __match_any_sync(NSGB_FULL, r);
      if (r >= 0 && (__ffs(peers) - 1) == tx) atomicAdd(&s_cnt[r], __popc(peers));
    }
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int ly = ty + 8 * k, i = ly * kTile + tx;
    const int gy = y0 + ly, gx = x0 + tx;
    if (gy >= H || gx >= W) continue;
    const int64_t g = (int64_t)gy * W + gx;
    const int r = root[k];
    L[g] = r < 0 ? -1 : (int)((int64_t)(y0 + r / kTile) * W + x0 + (r % kTile));
    if (A) A[g] = (r == i) ? s_cnt[i] : 0;
  }
}

// Joins tile-perimeter pixels with their forward neighbours (right, down-left, down,
// down-right) that lie in another tile.  Grid: one CTA of 96 threads per tile.
template <class Cls, int CONN>
__global__ void __launch_bounds__(96) ccl_merge(Cls cls, int H, int W, int* __restrict__ L) {
  const int x0 = blockIdx.x * kTile, y0 = blockIdx.y * kTile;
  const int t = threadIdx.x & 31, part = threadIdx.x >> 5;
  int y, x;
  if (part == 0) {  // bottom row
    y = y0 + kTile - 1;
    x = x0 + t;
  } else if (part == 1) {  // right column
    y = y0 + t;
    x = x0 + kTile - 1;
  } else {  // left column
    y = y0 + t;
    x = x0;
  }
  if (y >= H || x >= W) return;
  const uint32_t c = cls(y, x);
  if (!c) return;
  const int p = y * W + x;
  auto join = [&](int qy, int qx) {
    if (qy < 0 || qy >= H || qx < 0 || qx >= W) return;
    if ((qy / kTile) == (y / kTile) && (qx / kTile) == (x / kTile)) return;
    if (cls(qy, qx) != c) return;
    g_union(L, p, qy * W + qx);
  };
  if (part == 0) {
    join(y + 1, x);
    if (CONN == 8) {
      join(y + 1, x - 1);
      join(y + 1, x + 1);
    }
  } else if (part == 1) {
    join(y, x + 1);
    if (CONN == 8) join(y + 1, x + 1);
  } else {
    if (CONN == 8) join(y + 1, x - 1);
  }
}

// Seed policy used by ccl_flatten: `seed(y, x)` says whether the pixel marks its root.
struct NoSeed {
  __device__ bool operator()(int, int) const { return false; }
};

// L[i] <- root(L[i]); local-root areas move into the root; seed pixels set bit root in `bits`.
template <class Seed>
__global__ void ccl_flatten(int H, int W, int* __restrict__ L, int* __restrict__ A, Seed seed,
                            unsigned* __restrict__ bits) {
  const int64_t n = (int64_t)H * W;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int l = ld_relaxed(L + i);
    if (l < 0) continue;
    const int r = g_find(L, l);
    if (r != l) atomicMin(L + i, r);
    if (A) {
      const int a = A[i];
      if (a > 0 && r != (int)i) atomicAdd(&A[r], a);
    }
    if (bits) {
      const int y = (int)(i / W), x = (int)(i - (int64_t)y * W);
      if (seed(y, x)) {
        const unsigned bit = 1u << (r & 31);
        if (!(ld_relaxed((const int*)&bits[r >> 5]) & bit)) atomicOr(&bits[r >> 5], bit);
      }
    }
  }
}

// Read-only in the kernels that call it, so the L1-cached path is used: a giant component's
// root word is read by every pixel and would otherwise hammer one L2 line.
__device__ __forceinline__ bool test_bit(const unsigned* bits, int r) {
  return (__ldg(&bits[r >> 5]) >> (r & 31)) & 1u;
}

// Host helpers (ccl.cu).
inline dim3 tile_grid(int H, int W) { return dim3((W + kTile - 1) / kTile, (H + kTile - 1) / kTile); }
int flat_grid(int64_t n);

template <class Cls, class Seed>
cudaError_t label(const Cls& cls, int H, int W, int conn, int* L, int* A, const Seed& seed, unsigned* bits,
                  cudaStream_t s) {
  const dim3 g = tile_grid(H, W);
  if (conn == 8) {
    ccl_local<Cls, 8><<<g, kThreads, 0, s>>>(cls, H, W, L, A);
    ccl_merge<Cls, 8><<<g, 96, 0, s>>>(cls, H, W, L);
  } else {
    ccl_local<Cls, 4><<<g, kThreads, 0, s>>>(cls, H, W, L, A);
    ccl_merge<Cls, 4><<<g, 96, 0, s>>>(cls, H, W, L);
  }
  ccl_flatten<Seed><<<flat_grid((int64_t)H * W), 256, 0, s>>>(H, W, L, A, seed, bits);
  return cudaGetLastError();
}

// Raster-order ranks of the roots: rank[r] = number of roots before r (only written at roots),
// total roots and (if A) the number of roots whose area lies in [lo, hi) go to counts[0..1].
cudaError_t rank_roots(const int* L, const int* A, int64_t n, int lo, int hi, int* rank, int* block_tmp,
                       int* counts, cudaStream_t s);
size_t rank_tmp_ints(int64_t n);

}  // namespace ccl
}  // namespace nsgb
