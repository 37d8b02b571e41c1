// Union-find connected-component labelling on GB300 (internal templates).
//
// Reference semantics: ConnComponents::label (fastIA-master/src/segment/ConnComponents.cpp:
// 52-86) joins equal-valued non-zero neighbours (left, up, and up-left / up-right for
// 8-connectivity) and always hooks the larger root under the smaller one (merge, 34-43), so
// every component ends labelled with its smallest raster index; background is bgval.  The GPU
// reference (cuda/ccl_uf.cu:64-157, UF_local / UF_global / UF_final) uses the same
// min-index rule with atomicMin.  This implementation keeps that rule (so labels are
// bit-identical) with its own schedule:
//   1. ccl_local: 32x32 tile per CTA; horizontal runs from warp ballots, union-find on run
//      contacts in shared memory with atomicMin hooking; writes the tile-local root's global
//      index, lists the local roots and (optionally) their areas.
//   2. ccl_merge: one warp per tile edge joins runs that touch across the edge (global
//      atomicMin hooking; a failed hook retries with the new parent).
//   3. ccl_flatten_roots: every local root points directly at its global root and passes its
//      area on, so any pixel's root is L[L[i]]; seed kernels set a bit on the roots.
// Roots are exactly the pixels with L[i] == i.  Classifiers (the `Cls` template argument)
// return a pixel's class (0 = background; equal non-zero classes are joined), so the same
// kernels serve bwlabel (class = pixel value), hole filling (class = "not foreground"),
// binary reconstruction and bwselect (class = "mask non-zero").
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <climits>
#include <type_traits>

#include "batch.cuh"
#include "common.cuh"
#include "launch.cuh"

namespace nsgb {
namespace ccl {

constexpr int kTile = 32;      // tile edge (pixels)

// Connectivity codes.  4 and 8 join every class alike.  The two dual codes label two classes
// in one forest: kConnFg8Bg4 joins class 1 with 8-connectivity and class 2 with 4-connectivity,
// kConnFg4Bg8 the other way round (the pairs for which a binary image's components form a
// tree by enclosure).
constexpr int kConnFg8Bg4 = 84;
constexpr int kConnFg4Bg8 = 48;

// Whether pixels of class c join their diagonal neighbours of the same class.
template <int CONN>
__device__ __forceinline__ bool joins_diagonally(uint32_t c) {
  if constexpr (CONN == 8) return true;
  else if constexpr (CONN == 4) return false;
  else if constexpr (CONN == kConnFg8Bg4) return c == 1u;
  else return c == 2u;
}
constexpr int kThreads = 256;            // threads per labelling tile (32 columns x 8 warps)
constexpr int kRows = kTile / (kThreads / 32);  // tile rows per thread (consecutive)

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
// A background entry (-1) on the path means the forest is inconsistent with the classifier
// (never in a correct labelling); the walk then stops with -1 instead of reading before L.
__device__ __forceinline__ int g_find(int* L, int x) {
  for (;;) {
    const int p = ld_relaxed(L + x);
    if (p == x) return x;
    if (p < 0) return -1;
    const int g = ld_relaxed(L + p);
    if (g == p) return p;
    if (g < 0) return -1;
    atomicMin(L + x, g);
    x = g;
  }
}

__device__ __forceinline__ void g_union(int* L, int a, int b) {
  for (;;) {
    a = g_find(L, a);
    b = g_find(L, b);
    if (a == b || a < 0 || b < 0) return;
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

// Output of a labelling over a batch of images: L (int32, one dense plane per image at
// Img::px_base, pixel index = px_base + y*W + x; -1 = background).  Every foreground pixel
// points at its tile-local root and, after ccl_flatten_roots, every local root points at the
// global root, so root(i) = L[L[i]] (one hop).  Indices are global (px_base included), so a
// root is px_base + the smallest raster index of the component.  A (optional) holds the pixel
// count of each local root, then of each global root.  `roots` lists the local roots,
// `nroots` counts them.
struct Forest {
  int* L;
  int* A;
  int* roots;
  int* nroots;
};

__device__ __forceinline__ int root_of(const int* L, int64_t i) {
  const int l = __ldcg(L + i);
  return l < 0 ? -1 : __ldcg(L + l);
}

// The same, for kernels that do not write L: the second load goes through L1, where the
// pixels of one run (and of one component in a tile) find their shared root.
__device__ __forceinline__ int root_of_ro(const int* L, int64_t i) {
  const int l = __ldg(L + i);
  return l < 0 ? -1 : __ldg(L + l);
}

// Labelling tile of CTA `b`: image, tile origin.
struct TileAt {
  Img m;
  int x0, y0;
};
__device__ __forceinline__ TileAt tile_at(const Imgs& I, int b) {
  TileAt t;
  t.m = img_at(I, img_of_tile(I, b, I.c_img, I.c_per, CTileBase()));
  const int lt = b - t.m.c_tile_base;
  const int ty = lt / t.m.c_tiles_x;
  t.x0 = (lt - ty * t.m.c_tiles_x) * kTile;
  t.y0 = ty * kTile;
  return t;
}

// Width of the class values a classifier produces: 8 bits unless it declares `class_t`
// (the float plateau classifier needs all 32 bits of a value).
template <class Cls, class = void>
struct class_type {
  using type = uint8_t;
};
template <class Cls>
struct class_type<Cls, std::void_t<typename Cls::class_t>> {
  using type = typename Cls::class_t;
};

// Each warp owns kRows consecutive tile rows (lane = column) and joins them top-down, so a
// row's runs hook straight onto the root already found for the row above; only the four
// warps' blocks meet concurrently, which keeps the trees (and every later find) shallow.  Runs of equal class along a row are found with a
// ballot and start out joined (label = run start), so unions are only needed where runs of
// adjacent rows touch: at a pixel that starts its run or sits under the start of a run above
// (and, for 8-connectivity, diagonally past the two ends of the run).  That is one union per
// touching pair of runs instead of one per pixel pair.  One CTA per labelling tile (1-D grid
// over the tiles of all images).
template <class Cls, int CONN>
__global__ void __launch_bounds__(kThreads) ccl_local(Cls cls, Imgs I, Forest f) {
  pdl_wait();
  pdl_release();
  using CT = typename class_type<Cls>::type;
  __shared__ int s_lab[kTile * kTile];
  __shared__ int s_cnt[kTile * kTile];
  __shared__ CT s_c[kTile * kTile];
  __shared__ CT s_wv[kThreads / 32];  // per warp: the class of its first pixel
  const TileAt T = tile_at(I, blockIdx.x);
  const int x0 = T.x0, y0 = T.y0, H = T.m.H, W = T.m.W, pb = T.m.px_base;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  CT c[kRows];
#pragma unroll
  for (int k = 0; k < kRows; ++k) {
    const int ly = kRows * ty + k, i = ly * kTile + tx;
    const int gy = y0 + ly, gx = x0 + tx;
    c[k] = (CT)((gy < H && gx < W) ? cls(T.m, gy, gx) : 0u);
    s_c[i] = c[k];
    if (f.A) s_cnt[i] = 0;
  }
  // Uniform warp (one class in all its rows): one run per row, or none; no ballots needed.
  const CT ref = (CT)__shfl_sync(NSGB_FULL, (uint32_t)c[0], 0);
  bool same = true;
#pragma unroll
  for (int k = 0; k < kRows; ++k) same = same && c[k] == ref;
  const bool wu = __all_sync(NSGB_FULL, same);
  if (tx == 0) s_wv[ty] = ref;
  unsigned same_left[kRows];
  if (wu) {
#pragma unroll
    for (int k = 0; k < kRows; ++k) {
      const int ly = kRows * ty + k;
      same_left[k] = ref ? 0xFFFFFFFEu : 0u;
      s_lab[ly * kTile + tx] = ref ? ly * kTile : -1;
    }
  } else {
#pragma unroll
    for (int k = 0; k < kRows; ++k) {
      const int ly = kRows * ty + k, i = ly * kTile + tx;
      const CT left = (CT)__shfl_up_sync(NSGB_FULL, (uint32_t)c[k], 1);
      same_left[k] = __ballot_sync(NSGB_FULL, tx > 0 && c[k] != 0 && left == c[k]);
      // run start: highest lane <= tx whose pixel does not continue a run from the left
      const unsigned starts = ~same_left[k] & (0xFFFFFFFFu >> (31 - tx));
      const int rs = 31 - __clz(starts);
      s_lab[i] = c[k] ? ly * kTile + rs : -1;
    }
  }
  const bool all_wu = __syncthreads_and(wu) != 0;
  // Uniform tile (one class everywhere, pixels outside the image counting as background): the
  // whole tile is one component rooted at its first pixel, or background.  Common in masks
  // (empty background, solid foreground), and it needs no unions.
  if (all_wu) {
    bool uni = true;
#pragma unroll
    for (int w = 1; w < kThreads / 32; ++w) uni = uni && s_wv[w] == s_wv[0];
    if (uni) {
      const bool fg = s_wv[0] != 0;
      const int g0 = pb + y0 * W + x0;
#pragma unroll
      for (int k = 0; k < kRows; ++k) {
        const int gy = y0 + kRows * ty + k, gx = x0 + tx;
        if (gy < H && gx < W) f.L[pb + gy * W + gx] = fg ? g0 : -1;
      }
      if (fg && threadIdx.x == 0) {
        f.roots[atomicAdd(f.nroots, 1)] = g0;
        if (f.A) f.A[g0] = kTile * kTile;
      }
      return;
    }
  }
#pragma unroll
  for (int k = 0; k < kRows; ++k) {
    const int ly = kRows * ty + k, i = ly * kTile + tx;
    const CT v = c[k];
    if (!v || ly == 0) continue;
    const bool run_start = !((same_left[k] >> tx) & 1u);
    const int u = i - kTile;
    const CT up = s_c[u];
    const bool up_start = up != 0 && !(tx > 0 && s_c[u - 1] == up);
    if (up == v && (run_start || up_start)) s_union(s_lab, i, u);
    if (joins_diagonally<CONN>(v)) {
      if (run_start && tx > 0 && s_c[u - 1] == v) s_union(s_lab, i, u - 1);
      const bool run_end = (tx == kTile - 1) || s_c[i + 1] != v;
      if (run_end && tx < kTile - 1 && s_c[u + 1] == v) s_union(s_lab, i, u + 1);
    }
  }
  __syncthreads();
  int root[kRows];
#pragma unroll
  for (int k = 0; k < kRows; ++k) {
    const int ly = kRows * ty + k, i = ly * kTile + tx;
    root[k] = c[k] ? s_find(s_lab, i) : -1;
  }
  if (f.A) {
#pragma unroll
    for (int k = 0; k < kRows; ++k) {
      const int r = root[k];
      const unsigned peers = __match_any_sync(NSGB_FULL, r);
      if (r >= 0 && (__ffs(peers) - 1) == tx) atomicAdd(&s_cnt[r], __popc(peers));
    }
    __syncthreads();
  }
  unsigned rb[kRows];
  int nr = 0;
#pragma unroll
  for (int k = 0; k < kRows; ++k) {
    const int ly = kRows * ty + k, i = ly * kTile + tx;
    const int gy = y0 + ly, gx = x0 + tx;
    const bool in = gy < H && gx < W;
    const int r = root[k];
    const int g = pb + gy * W + gx;
    if (in) f.L[g] = r < 0 ? -1 : pb + (y0 + r / kTile) * W + x0 + (r % kTile);
    rb[k] = __ballot_sync(NSGB_FULL, in && r == i);
    nr += __popc(rb[k]);
  }
  // The warp's local roots (all four rows) go to the list with one atomic: a tile of singleton
  // components has 1024 roots, and per-row atomics on the one counter would serialise.
  if (nr == 0) return;  // warp-uniform: most warps of a labelling hold no root
  int base = 0;
  if (tx == 0) base = atomicAdd(f.nroots, nr);
  base = __shfl_sync(NSGB_FULL, base, 0);
#pragma unroll
  for (int k = 0; k < kRows; ++k) {
    if ((rb[k] >> tx) & 1u) {
      const int ly = kRows * ty + k, i = ly * kTile + tx;
      const int g = pb + (y0 + ly) * W + x0 + tx;
      f.roots[base + __popc(rb[k] & ((1u << tx) - 1u))] = g;
      if (f.A) f.A[g] = s_cnt[i];
    }
    base += __popc(rb[k]);
  }
}

// Joins runs across tile edges.  Two warps per labelling tile: warp 0 takes the bottom edge
// (row y0+31 against row y0+32), warp 1 the right edge (column x0+31 against column x0+32, the
// same logic transposed).  With `a` = the pixel on this side and `b` its partner across the
// edge, runs of equal class along the edge are found with ballots, and a union is made only
// where a run on the far side starts or where a near-side run starts under a far-side run,
// plus the two diagonal ends of each far-side run for 8-connectivity.
template <class Cls, int CONN>
__global__ void __launch_bounds__(64) ccl_merge(Cls cls, Imgs I, int* __restrict__ L) {
  pdl_wait();
  pdl_release();
  const TileAt T = tile_at(I, blockIdx.x);
  const int x0 = T.x0, y0 = T.y0, H = T.m.H, W = T.m.W, pb = T.m.px_base;
  const int lane = threadIdx.x & 31;
  const bool bottom = (threadIdx.x >> 5) == 0;
  // coordinates of the near pixel (a) and the far pixel (b) for this lane
  int ay, ax, by, bx;
  if (bottom) {
    ay = y0 + kTile - 1;
    ax = x0 + lane;
    by = ay + 1;
    bx = ax;
    if (by >= H) return;  // whole warp: no tile below
  } else {
    ax = x0 + kTile - 1;
    ay = y0 + lane;
    bx = ax + 1;
    by = ay;
    if (bx >= W) return;
  }
  const bool in_a = ay < H && ax < W;
  const bool in_b = by < H && bx < W;
  const uint32_t ca = in_a ? cls(T.m, ay, ax) : 0u;
  const uint32_t cb = in_b ? cls(T.m, by, bx) : 0u;
  // runs along the edge (lane order) on each side
  const uint32_t ca_prev = __shfl_up_sync(NSGB_FULL, ca, 1);
  const uint32_t cb_prev = __shfl_up_sync(NSGB_FULL, cb, 1);
  const uint32_t cb_next = __shfl_down_sync(NSGB_FULL, cb, 1);
  const bool a_start = ca != 0 && !(lane > 0 && ca_prev == ca);
  const bool b_start = cb != 0 && !(lane > 0 && cb_prev == cb);
  const bool b_end = cb != 0 && !(lane < 31 && cb_next == cb);
  if (cb == 0) return;
  const int qb = pb + by * W + bx;
  if (ca == cb && (a_start || b_start)) g_union(L, qb, pb + ay * W + ax);
  // Diagonal partners one step before the start / after the end of the far-side run.  When
  // the near pixel at this lane has the far run's class, the partner (its neighbour along the
  // edge) is joined to it by the near tile's own labelling or by the next tile's edge merge,
  // and the near pixel is joined to the far run here: the diagonal union adds nothing.
  if (ca != cb && joins_diagonally<CONN>(cb)) {
    if (b_start) {
      const int dy = bottom ? ay : ay - 1, dx = bottom ? ax - 1 : ax;
      if (dy >= 0 && dx >= 0 && dy < H && dx < W && cls(T.m, dy, dx) == cb) g_union(L, qb, pb + dy * W + dx);
    }
    if (b_end) {
      const int dy = bottom ? ay : ay + 1, dx = bottom ? ax + 1 : ax;
      if (dy < H && dx < W && cls(T.m, dy, dx) == cb) g_union(L, qb, pb + dy * W + dx);
    }
  }
}

// Every local root points directly at its global root; local-root areas move into the root.
// Four list entries per thread and iteration, their loads issued together: most local roots
// are global roots already (one load to see it), so the kernel is load-latency bound.  The
// area adds of a warp are summed per root first (one atomic per root and warp): the local
// roots of a giant component, one per labelling tile, all add into the same word.
static __global__ void ccl_flatten_roots(Forest f, int max_roots) {
  pdl_wait();
  pdl_release();
  const int n = min(__ldcg(f.nroots), max_roots);
  const int stride = gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  for (int k0 = blockIdx.x * blockDim.x + threadIdx.x; k0 - lane < n; k0 += 4 * stride) {
    int lr[4], p[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) lr[j] = k0 + j * stride < n ? __ldcg(f.roots + k0 + j * stride) : -1;
#pragma unroll
    for (int j = 0; j < 4; ++j) p[j] = lr[j] >= 0 ? __ldcg(f.L + lr[j]) : -1;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      int r = -1, a = 0;
      if (lr[j] >= 0 && p[j] != lr[j]) {
        r = g_find(f.L, lr[j]);
        if (r >= 0 && r != lr[j]) {
          atomicMin(f.L + lr[j], r);
          if (f.A) a = __ldcg(f.A + lr[j]);
        } else {
          r = -1;
        }
      }
      if (f.A) {
        const unsigned peers = __match_any_sync(NSGB_FULL, r);
        const int sum = __reduce_add_sync(peers, a);
        if (r >= 0 && (__ffs(peers) - 1) == lane) atomicAdd(f.A + r, sum);
      }
    }
  }
}

__device__ __forceinline__ void set_root_bit(unsigned* bits, int r) {
  const unsigned bit = 1u << (r & 31);
  if (!(__ldcg(&bits[r >> 5]) & bit)) atomicOr(&bits[r >> 5], bit);
}

// Row walk over the rows of all images: g(image, row within the image) for every row this
// block row owns.  A single image strides its rows by gridDim.y.  A batch gives each block row
// a contiguous range of the concatenated rows, so the image is looked up once per block row
// (a binary search over the table) and then followed across image boundaries, instead of
// searching again for every row.
template <class G>
__device__ __forceinline__ void for_batch_rows(const Imgs& I, int total_rows, G&& g) {
  if (!I.d) {
    for (int gr = blockIdx.y; gr < total_rows; gr += gridDim.y) g(I.one, gr);
    return;
  }
  const int per = (total_rows + (int)gridDim.y - 1) / (int)gridDim.y;
  const int r0 = (int)blockIdx.y * per, r1 = min(total_rows, r0 + per);
  if (r0 >= r1) return;
  int ii = img_of(I, r0, RowBase());
  Img m = I.d[ii];
  int next = ii + 1 < I.n ? I.d[ii + 1].row_base : INT_MAX;
  for (int gr = r0; gr < r1; ++gr) {
    while (gr >= next) {
      ++ii;
      m = I.d[ii];
      next = ii + 1 < I.n ? I.d[ii + 1].row_base : INT_MAX;
    }
    g(m, gr - m.row_base);
  }
}

// Row grid over the rows of all images: x = column (blockIdx.x * blockDim.x + threadIdx.x);
// f(image, y, x) runs for every pixel.
template <class F>
__device__ __forceinline__ void for_batch_pixels(const Imgs& I, int total_rows, F&& f) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  for_batch_rows(I, total_rows, [&](const Img& m, int y) {
    if (x < m.W) f(m, y, x);
  });
}

// The same with four consecutive pixels per thread: f(image, y, x, n) for pixels x .. x+n-1
// (n <= 4) of row y; x grid over max_w / 4.
template <class F>
__device__ __forceinline__ void for_batch_quads(const Imgs& I, int total_rows, F&& f) {
  const int x = 4 * (blockIdx.x * blockDim.x + threadIdx.x);
  for_batch_rows(I, total_rows, [&](const Img& m, int y) {
    if (x < m.W) f(m, y, x, min(4, m.W - x));
  });
}

// Roots of four consecutive pixels (L read-only): one 16-byte load when aligned.
__device__ __forceinline__ void roots4_ro(const int* L, int64_t i, int n, int (&r)[4]) {
  int l[4];
  if (n == 4 && ((i & 3) == 0)) {
    const int4 v = __ldg((const int4*)(L + i));
    l[0] = v.x, l[1] = v.y, l[2] = v.z, l[3] = v.w;
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) l[k] = k < n ? __ldg(L + i + k) : -1;
  }
#pragma unroll
  for (int k = 0; k < 4; ++k) r[k] = l[k] < 0 ? -1 : (k > 0 && l[k] == l[k - 1] ? -2 : __ldg(L + l[k]));
#pragma unroll
  for (int k = 1; k < 4; ++k)
    if (r[k] == -2) r[k] = r[k - 1];
}

// Seed pixels set bit root(p) in `bits`.
template <class Seed>
__global__ void ccl_seed_pixels(Imgs I, int total_rows, const int* __restrict__ L, Seed seed,
                                unsigned* __restrict__ bits) {
  for_batch_pixels(I, total_rows, [&](const Img& m, int y, int x) {
    if (!seed(m, y, x)) return;
    const int r = root_of(L, (int64_t)m.px_base + (int64_t)y * m.W + x);
    if (r >= 0) set_root_bit(bits, r);
  });
}

// The same with four consecutive pixels per thread: their roots come from one 16-byte label
// load where aligned, and a root shared with the seed pixel before it is set once.
template <class Seed>
__global__ void ccl_seed_quads(Imgs I, int total_rows, const int* __restrict__ L, Seed seed,
                               unsigned* __restrict__ bits) {
  for_batch_quads(I, total_rows, [&](const Img& m, int y, int x, int n) {
    bool sd[4];
    bool any = false;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      sd[k] = k < n && seed(m, y, x + k);
      any = any || sd[k];
    }
    if (!any) return;
    int r[4];
    roots4_ro(L, (int64_t)m.px_base + (int64_t)y * m.W + x, n, r);
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (sd[k] && r[k] >= 0 && !(k > 0 && sd[k - 1] && r[k - 1] == r[k])) set_root_bit(bits, r[k]);
  });
}

// Border pixel k of an H x W image (top row, bottom row, left column, right column; 2W + 2H
// positions, corners visited twice).
__device__ __forceinline__ void border_pixel(int k, int H, int W, int& y, int& x) {
  if (k < W) {
    y = 0;
    x = k;
  } else if (k < 2 * W) {
    y = H - 1;
    x = k - W;
  } else if (k < 2 * W + H) {
    y = k - 2 * W;
    x = 0;
  } else {
    y = k - 2 * W - H;
    x = W - 1;
  }
}

// Seed pixels on each image's border only: blockIdx.y = image, x walks its border.
template <class Seed>
__global__ void ccl_seed_border(Imgs I, const int* __restrict__ L, Seed seed, unsigned* __restrict__ bits) {
  const Img m = img_at(I, blockIdx.y);
  const int H = m.H, W = m.W;
  const int per = 2 * W + 2 * H;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < per; k += gridDim.x * blockDim.x) {
    int y, x;
    border_pixel(k, H, W, y, x);
    if (!seed(m, y, x)) continue;
    const int r = root_of(L, (int64_t)m.px_base + (int64_t)y * W + x);
    if (r >= 0) set_root_bit(bits, r);
  }
}

// The same before the roots are flattened (after ccl_merge): the root is found by walking the
// forest.
template <class Seed>
__global__ void ccl_seed_border_walk(Imgs I, int* L, Seed seed, unsigned* __restrict__ bits) {
  pdl_wait();
  pdl_release();
  const Img m = img_at(I, blockIdx.y);
  const int H = m.H, W = m.W;
  const int per = 2 * W + 2 * H;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < per; k += gridDim.x * blockDim.x) {
    int y, x;
    border_pixel(k, H, W, y, x);
    if (!seed(m, y, x)) continue;
    const int r = g_find(L, m.px_base + y * W + x);
    if (r >= 0) set_root_bit(bits, r);
  }
}

// Read-only in the kernels that call it, so the L1-cached path is used: a giant component's
// root word is read by every pixel and would otherwise hammer one L2 line.
__device__ __forceinline__ bool test_bit(const unsigned* bits, int r) {
  return (__ldg(&bits[r >> 5]) >> (r & 31)) & 1u;
}

// Host helpers (ccl.cu).
int flat_grid(int64_t n);
// Grid for kernels that walk a device-side list whose length (unknown on the host) is at most
// max_items.
int list_grid(int64_t max_items);
// Row grids: x covers the widest image (256 columns, or 256 quads of columns, per block), y
// strides the rows (one block row per image row up to the grid limit: batched kernels look
// the image of a row up per row, so they want many short row walks).
inline unsigned row_blocks(int total_rows) { return (unsigned)(total_rows < 65535 ? total_rows : 65535); }
inline dim3 rowcol_grid(int total_rows, int max_w) {
  const unsigned bx = (unsigned)((max_w + 255) / 256);
  return dim3(bx, row_blocks(total_rows));
}
inline dim3 quadrow_grid(int total_rows, int max_w) {
  const unsigned bx = (unsigned)(((max_w + 3) / 4 + 255) / 256);
  return dim3(bx, row_blocks(total_rows));
}

// Labels every image of the batch: local pass, edge merge, root flattening.  Afterwards
// root(i) = L[L[i]].
template <class Cls>
cudaError_t label(const Cls& cls, const Imgs& I, const BatchTotals& t, int conn, const Forest& f, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(f.nroots, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  if (conn == 8) {
    ccl_local<Cls, 8><<<t.c_tiles, kThreads, 0, s>>>(cls, I, f);
    ccl_merge<Cls, 8><<<t.c_tiles, 64, 0, s>>>(cls, I, f.L);
  } else {
    ccl_local<Cls, 4><<<t.c_tiles, kThreads, 0, s>>>(cls, I, f);
    ccl_merge<Cls, 4><<<t.c_tiles, 64, 0, s>>>(cls, I, f.L);
  }
  ccl_flatten_roots<<<list_grid(t.px), 256, 0, s>>>(f, (int)t.px);
  return cudaGetLastError();
}

// Enclosure tree of a two-class labelling (kConnFg8Bg4 / kConnFg4Bg8, before flattening):
// with dual connectivities the components of the two classes form a tree by enclosure, the
// image's outside (the components marked in `outside`, those of the outside class that touch
// the border) at its top, and a component's parent is the component of the pixel directly
// above its first pixel in raster order (its root).  Every component below the top joins its
// parent, so each set that results is one component of "class 1 plus the class-2 components
// it encloses" (class 1 with its holes filled).  One thread per listed local root; a global
// root is hooked only by its own thread (its parent's root index is smaller than its own), so
// the test for a global root at the start holds until the thread itself changes it.
static __global__ void ccl_join_parents(Imgs I, Forest f, int max_roots, const unsigned* __restrict__ outside) {
  pdl_wait();
  pdl_release();
  const int n = min(__ldcg(f.nroots), max_roots);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int r = __ldcg(f.roots + k);
    if (ld_relaxed(f.L + r) != r) continue;
    if ((__ldcg(outside + (r >> 5)) >> (r & 31)) & 1u) continue;
    const Img m = img_at(I, img_of(I, r, PxBase()));
    if (r - m.px_base < m.W) continue;  // first row: its parent is the outside
    const int p = g_find(f.L, r - m.W);
    if (p < 0 || ((__ldcg(outside + (p >> 5)) >> (p & 31)) & 1u)) continue;
    g_union(f.L, r, p);
  }
}

// Up to four word ranges to clear in one launch (n[k] words from p[k]; unused ranges have n 0).
struct ZeroSpans {
  unsigned* p[4];
  int n[4];
  int total() const { return n[0] + n[1] + n[2] + n[3]; }
};

static __global__ void zero_words(ZeroSpans z) {
  pdl_wait();
  pdl_release();
  const int total = z.n[0] + z.n[1] + z.n[2] + z.n[3];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    int j = i, r = 0;
    while (j >= z.n[r]) j -= z.n[r++];
    z.p[r][j] = 0u;
  }
}

// Launches `kernel` the ordinary way, or (pdl) as a programmatic dependent of the kernel before
// it on the stream, which every kernel launched here waits for first thing.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t s,
                            Args&&... args) {
  if (pdl) return launch_dependent(kernel, grid, block, s, std::forward<Args>(args)...);
  kernel<<<grid, block, 0, s>>>(std::forward<Args>(args)...);
  return cudaGetLastError();
}

// Seed test: pixels of class 2.
template <class Cls>
struct Class2 {
  Cls cls;
  __device__ bool operator()(const Img& m, int y, int x) const { return cls(m, y, x) == 2u; }
};

// Labels both classes of a two-class classifier (class 1 = the foreground, class 2 = the rest)
// with dual connectivities and joins every component below the outside to its parent: the
// sets are then the components of the foreground with its holes filled, each rooted at its
// smallest raster index, and A holds their areas (holes included).  The border components of
// class 2 are marked in `outside` (zeroed first; their roots stay roots and are not part of
// the filled image).  Afterwards root(i) = L[L[i]].
template <class Cls>
cudaError_t label_filled(const Cls& cls, const Imgs& I, const BatchTotals& t, int conn, const Forest& f,
                         unsigned* outside, size_t outside_bytes, cudaStream_t s, bool pdl = false,
                         ZeroSpans more = ZeroSpans{{nullptr, nullptr, nullptr, nullptr}, {0, 0, 0, 0}}) {
  // The first launch follows whatever the caller queued last, so it is an ordinary one; the
  // rest may start while their predecessor drains.  It also clears the caller's ranges 2 and 3
  // of `more` (for the ranking that follows, say).
  ZeroSpans z = more;
  z.p[0] = (unsigned*)f.nroots;
  z.n[0] = 1;
  z.p[1] = outside;
  z.n[1] = (int)(outside_bytes / sizeof(unsigned));
  cudaError_t e = launch_k(false, zero_words, dim3(flat_grid(z.total())), dim3(256), s, z);
  if (e != cudaSuccess) return e;
  if (conn == kConnFg8Bg4) {
    e = launch_k(pdl, ccl_local<Cls, kConnFg8Bg4>, dim3(t.c_tiles), dim3(kThreads), s, cls, I, f);
    if (e == cudaSuccess) e = launch_k(pdl, ccl_merge<Cls, kConnFg8Bg4>, dim3(t.c_tiles), dim3(64), s, cls, I, f.L);
  } else {
    e = launch_k(pdl, ccl_local<Cls, kConnFg4Bg8>, dim3(t.c_tiles), dim3(kThreads), s, cls, I, f);
    if (e == cudaSuccess) e = launch_k(pdl, ccl_merge<Cls, kConnFg4Bg8>, dim3(t.c_tiles), dim3(64), s, cls, I, f.L);
  }
  const int gx = (t.perimeter_max + 255) / 256 > 64 ? 64 : (t.perimeter_max + 255) / 256;
  if (e == cudaSuccess)
    e = launch_k(pdl, ccl_seed_border_walk<Class2<Cls>>, dim3(gx > 0 ? gx : 1, t.n), dim3(256), s, I, f.L,
                 Class2<Cls>{cls}, outside);
  if (e == cudaSuccess)
    e = launch_k(pdl, ccl_join_parents, dim3(list_grid(t.px)), dim3(256), s, I, f, (int)t.px, (const unsigned*)outside);
  if (e == cudaSuccess) e = launch_k(pdl, ccl_flatten_roots, dim3(list_grid(t.px)), dim3(256), s, f, (int)t.px);
  return e;
}

// Raster-order ranks of the global roots, from the list of local roots: rank[r] = number of
// roots of r's image before r (written at roots only).  counts[2*i] = roots of image i,
// counts[2*i+1] = roots whose area (A, if given) lies in [lo, hi).  `bits` (one bit per
// pixel, px/32 + 2 words), `block_tmp` (one int per rank block) and `wpre` (32 ints per rank
// block) are scratch.
// Roots marked in `skip` (optional) are left out: not counted and not ranked.
// With pdl, every launch is a programmatic dependent of the kernel before it (the caller's last
// launch must be a kernel); with zeroed, `bits` and `counts` are already clear.
cudaError_t rank_roots(const Imgs& I, const BatchTotals& t, const Forest& f, int lo, int hi, int* rank,
                       unsigned* bits, size_t bits_bytes, int* block_tmp, int* wpre, int* counts, cudaStream_t s,
                       const unsigned* skip = nullptr, bool pdl = false, bool zeroed = false);
// The counts of rank_roots alone (no ranks).  `bits` receives the global roots' bits (scratch,
// not cleared first).
cudaError_t count_roots(const Imgs& I, const BatchTotals& t, const Forest& f, int lo, int hi, unsigned* bits,
                        int* counts, cudaStream_t s, const unsigned* skip = nullptr);
constexpr int kBlockPx = 1024;

// The counting half of rank_roots for any bitmap of the images' pixels: per 1024-px block the
// set bits before it in its image (block_tmp, exclusive scan) and per 32-px word the set bits
// before it in its block (wpre).  A set bit's rank is then bit_rank().
cudaError_t rank_bits(const Imgs& I, const BatchTotals& t, const unsigned* bits, int* block_tmp, int* wpre,
                      cudaStream_t s);

// Bits of pixels p .. p+31 (the bitmap has a spare word at the end).
__device__ __forceinline__ unsigned bits_at(const unsigned* bits, int p) {
  const int w = p >> 5, sh = p & 31;
  const unsigned lo = __ldcg(bits + w);
  return sh ? __funnelshift_r(lo, __ldcg(bits + w + 1), sh) : lo;
}

// Rank of pixel p (a set bit) among the set bits of a single image, after rank_bits.
__device__ __forceinline__ int bit_rank(const unsigned* bits, const int* block_tmp, const int* wpre, int p) {
  const int b = p / kBlockPx, j = (p % kBlockPx) >> 5;
  const int w0 = b * kBlockPx + 32 * j;
  int c = __ldcg(block_tmp + b) + __ldcg(wpre + 32 * b + j);
  if (p > w0) c += __popc(bits_at(bits, w0) & ((1u << (p - w0)) - 1u));
  return c;
}

}  // namespace ccl
}  // namespace nsgb
