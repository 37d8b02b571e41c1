// Euclidean distance transform of a u8 mask: for every pixel the distance to the nearest zero
// pixel (0 on zero pixels), the map the segmentation takes before its watershed
// (HistologicalEntities.cpp:341, OpenCV's CV_DIST_L2 / CV_DIST_MASK_PRECISE; the reference's own
// queue version is nscale::distanceTransform, MorphologicOperations.cpp:197-275, GPU
// nscale::gpu::distanceTransform, cuda/global_queue_dist.cu).  Exact: the squared distance is an
// integer, and the float result is the correctly rounded square root of it.  The reference's
// queue version propagates nearest zero pixels between 8-neighbours, which can settle on a zero
// pixel that is not the nearest; it is never closer than the exact distance.
//
// Two passes (Meijster, Roerdink and Hesselink, 2000):
// (1) per column, the distance in rows to the nearest zero pixel of that column, g (INF when the
//     column has none; INF = rows + cols exceeds every real distance).  Columns are cut into
//     128-row chunks: one launch records each chunk's first and last zero row, the next walks
//     each chunk down and up from the nearest zero rows of the chunks above and below (threads
//     of a warp take adjacent columns, so rows are read coalesced);
// (2) per row, D^2(x) = min over x' of (x - x')^2 + g(x')^2, one CTA per row: each pixel
//     searches outward along the row and stops once the column offset alone reaches its best
//     squared distance (at most g(x) columns each way), which is cheap while the row's mean g is
//     small (objects of tens of pixels).  A row with a large mean g (far from every zero pixel,
//     or crossing columns without one) is done by the whole CTA by divide and conquer: the
//     matrix (x - i)^2 + g(i)^2 is Monge, so the leftmost minimising column A(x) never
//     decreases with x, and the row minimum at the midpoint of two computed positions a < b
//     only needs the columns A(a) .. A(b).  Level by level (log2 W levels) every position's
//     candidate columns are laid end to end and split evenly over the threads, each keeping
//     one running minimum per position it touches (64-bit keys: D^2 above the column, so
//     atomicMin keeps the leftmost minimum).  Rows wider than the shared-memory tables
//     (12288 columns) fall back to the lower envelope of the parabolas (Meijster) on one
//     thread.  All three are exact integer arithmetic.
// Output: the distance (float), or the basins of the watershed step (HistologicalEntities.cpp:
// 347-356): -distance on mask pixels, -FLT_MAX elsewhere.  No zero pixel at all: +inf.
#include <cfloat>
#include <cmath>

#include "common.cuh"
#include "edt.cuh"

namespace nsgb {

namespace {

constexpr int kThreads = 32;  // column passes: 32 adjacent columns per block
constexpr int kChunk = 128;   // rows per column chunk

// First and last zero row of every (column, chunk), -1 when none.
__global__ void __launch_bounds__(kThreads) edt_chunk_zeros(const uint8_t* __restrict__ mask, int64_t pitch, int H,
                                                            int W, int* __restrict__ first0, int* __restrict__ last0) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= W) return;
  const int c = blockIdx.y;
  const int y0 = c * kChunk, y1 = min(H, y0 + kChunk);
  int f = -1, l = -1;
  for (int y = y0; y < y1; ++y)
    if (__ldg(mask + (int64_t)y * pitch + x) == 0) {
      if (f < 0) f = y;
      l = y;
    }
  first0[(int64_t)c * W + x] = f;
  last0[(int64_t)c * W + x] = l;
}

// g for the rows of one (column, chunk): nearest zero row above (from the chunks above, then
// this chunk's rows in order) and below.
__global__ void __launch_bounds__(kThreads) edt_columns(const uint8_t* __restrict__ mask, int64_t pitch, int H, int W,
                                                        const int* __restrict__ first0, const int* __restrict__ last0,
                                                        int* __restrict__ g) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= W) return;
  const int c = blockIdx.y, nc = gridDim.y;
  const int y0 = c * kChunk, y1 = min(H, y0 + kChunk);
  const int inf = H + W;
  int z = -1;  // nearest zero row at or above the current row
  for (int k = c - 1; k >= 0 && z < 0; --k) z = __ldg(last0 + (int64_t)k * W + x);
  for (int y = y0; y < y1; ++y) {
    if (__ldg(mask + (int64_t)y * pitch + x) == 0) z = y;
    g[(int64_t)y * W + x] = z >= 0 ? y - z : inf;
  }
  z = -1;  // nearest zero row at or below
  for (int k = c + 1; k < nc && z < 0; ++k) z = __ldg(first0 + (int64_t)k * W + x);
  for (int y = y1 - 1; y >= y0; --y) {
    if (__ldg(mask + (int64_t)y * pitch + x) == 0) z = y;
    if (z >= 0) {
      int* p = g + (int64_t)y * W + x;
      if (z - y < *p) *p = z - y;
    }
  }
}

__device__ __forceinline__ int64_t sq(int64_t v) { return v * v; }

// floor(a / b) for b > 0.
__device__ __forceinline__ int64_t floor_div(int64_t a, int64_t b) {
  const int64_t q = a / b;
  return (a % b != 0 && a < 0) ? q - 1 : q;
}

__device__ __forceinline__ float root(int64_t d2) {
  return d2 < (1ll << 24) ? sqrtf((float)d2) : (float)sqrt((double)d2);
}

template <bool BASINS>
__device__ __forceinline__ void store_px(float* o, const uint8_t* mrow, int x, int64_t d2, int64_t inf2) {
  const float d = d2 >= inf2 ? INFINITY : root(d2);
  if (BASINS) o[x] = __ldg(mrow + x) != 0 ? -d : -FLT_MAX;
  else o[x] = d;
}

// One row by the lower envelope of its parabolas (one thread; stacks s, t in the workspace).
template <bool BASINS>
__device__ void envelope_row(const int* __restrict__ gr, int* s, int* t, float* o, const uint8_t* mrow, int W,
                             int64_t inf2) {
  int q = 0;
  s[0] = 0;
  t[0] = 0;
  int64_t gs = sq(__ldg(gr));  // g(s[q])^2
  for (int u = 1; u < W; ++u) {
    const int64_t gu = sq(__ldg(gr + u));
    // pop while the top parabola is above u's at the top's start t[q]
    while (q >= 0 && sq((int64_t)t[q] - s[q]) + gs > sq((int64_t)t[q] - u) + gu) {
      --q;
      if (q >= 0) gs = sq(__ldg(gr + s[q]));
    }
    if (q < 0) {
      q = 0;
      s[0] = u;
      t[0] = 0;
      gs = gu;
    } else {
      // first x at which u's parabola is below s[q]'s: 1 + floor(sep)
      const int64_t sep = floor_div(sq((int64_t)u) - sq((int64_t)s[q]) + gu - gs, 2 * ((int64_t)u - s[q]));
      const int64_t w = 1 + sep;
      if (w < W) {
        ++q;
        s[q] = u;
        t[q] = (int)w;
        gs = gu;
      }
    }
  }
  int64_t gq = sq(__ldg(gr + s[q]));
  for (int x = W - 1; x >= 0; --x) {
    store_px<BASINS>(o, mrow, x, sq((int64_t)x - s[q]) + gq, inf2);
    if (x == t[q] && q > 0) {
      --q;
      gq = sq(__ldg(gr + s[q]));
    }
  }
}

constexpr int kRowThreads = 256;
// A row whose mean g exceeds this takes the divide and conquer instead of the per-pixel search.
constexpr int64_t kMeanG = 32;
// Widest row for the divide and conquer's shared-memory tables (8 bytes per column).
constexpr int kDcMaxW = 12288;

__device__ __forceinline__ int dc_levels(int W) {
  int L = 1;
  while ((1 << L) < W + 1) ++L;
  return L;
}

// Exclusive prefix sum of a[0 .. n) in place by the whole CTA; returns the total.
__device__ int block_exclusive_scan(int* a, int n) {
  __shared__ int s_warp[kRowThreads / 32];
  __shared__ int s_total;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int per = (n + kRowThreads - 1) / kRowThreads;
  const int b = min(n, tid * per), e = min(n, b + per);
  int sum = 0;
  for (int k = b; k < e; ++k) sum += a[k];
  int incl = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(NSGB_FULL, incl, o);
    if (lane >= o) incl += v;
  }
  if (lane == 31) s_warp[wid] = incl;
  __syncthreads();
  int base = 0;
  for (int w = 0; w < wid; ++w) base += s_warp[w];
  if (tid == kRowThreads - 1) s_total = base + incl;
  int run = base + incl - sum;
  for (int k = b; k < e; ++k) {
    const int v = a[k];
    a[k] = run;
    run += v;
  }
  __syncthreads();
  return s_total;
}

// Divide and conquer over the row (see the file comment).  Level l computes the positions
// x = (2k + 1) h - 1, h = 2^(L-1-l), whose neighbours x - h and x + h were computed before (or
// lie outside the row: A = 0 on the left, W - 1 on the right).  Shared memory: A (u16 per
// column), the level's keys (u64 per position) and candidate offsets (int per position + 1).
template <bool BASINS>
__device__ void dc_row(const int* __restrict__ gr, float* o, const uint8_t* mrow, int W, int64_t inf2,
                       unsigned char* smem) {
  uint16_t* A = (uint16_t*)smem;
  const int max_nodes = W / 2 + 1;
  unsigned long long* key = (unsigned long long*)(smem + (((size_t)W * 2 + 15) & ~(size_t)15));
  int* off = (int*)(key + max_nodes);
  const int L = dc_levels(W);
  const int tid = threadIdx.x;
  for (int l = 0; l < L; ++l) {
    const int h = 1 << (L - 1 - l);
    const int n = (W / h + 1) / 2;  // positions of this level inside the row
    for (int k = tid; k < n; k += kRowThreads) {
      const int x = (2 * k + 1) * h - 1;
      const int lo = x - h < 0 ? 0 : A[x - h];
      const int hi = x + h >= W ? W - 1 : A[x + h];
      off[k] = hi - lo + 1;
      key[k] = ~0ull;
    }
    __syncthreads();
    const int total = block_exclusive_scan(off, n);
    if (tid == 0) off[n] = total;
    __syncthreads();
    const int chunk = (total + kRowThreads - 1) / kRowThreads;
    int j = tid * chunk;
    const int end = min(total, j + chunk);
    if (j < end) {
      // the position holding candidate j: the last k with off[k] <= j
      int a = 0, b = n - 1;
      while (a < b) {
        const int m = (a + b + 1) >> 1;
        if (off[m] <= j) a = m;
        else b = m - 1;
      }
      int k = a;
      while (j < end) {
        const int x = (2 * k + 1) * h - 1;
        const int lo = x - h < 0 ? 0 : A[x - h];
        const int stop = min(end, off[k + 1]);
        unsigned long long best = ~0ull;
        for (; j < stop; ++j) {
          const int i = lo + (j - off[k]);
          const unsigned long long d2 = (unsigned long long)(sq((int64_t)x - i) + sq(__ldg(gr + i)));
          const unsigned long long kk = (d2 << 24) | (unsigned long long)i;
          best = kk < best ? kk : best;
        }
        atomicMin(&key[k], best);
        ++k;
      }
    }
    __syncthreads();
    for (int k = tid; k < n; k += kRowThreads) {
      const int x = (2 * k + 1) * h - 1;
      const unsigned long long kk = key[k];
      A[x] = (uint16_t)(kk & 0xFFFFFFull);
      store_px<BASINS>(o, mrow, x, (int64_t)(kk >> 24), inf2);
    }
    __syncthreads();
  }
}

// One CTA per row.  D(x) <= g(x), so a pixel's search along the row stops after at most g(x)
// columns each way (once k^2 reaches the best squared distance so far); when the row's g sum
// keeps that work small (mean g <= kMeanG) all threads search their pixels, otherwise the CTA
// runs the divide and conquer (`dc`: the row fits the shared tables and its squared distances
// fit the 40-bit keys), or one thread builds the row's lower envelope.

template <bool BASINS>
__global__ void __launch_bounds__(kRowThreads) edt_rows(const uint8_t* __restrict__ mask, int64_t pitch_in,
                                                        const int* __restrict__ g, int* __restrict__ stack_s,
                                                        int* __restrict__ stack_t, float* __restrict__ out,
                                                        int64_t pitch_out, int H, int W, bool dc) {
  extern __shared__ __align__(16) unsigned char dc_smem[];
  __shared__ long long s_sum[kRowThreads / 32];
  const int64_t inf2 = sq((int64_t)H + W);
  for (int y = blockIdx.x; y < H; y += gridDim.x) {
    const int* gr = g + (int64_t)y * W;
    float* o = (float*)((char*)out + (int64_t)y * pitch_out);
    const uint8_t* mrow = mask + (int64_t)y * pitch_in;
    long long sum = 0;
    for (int x = threadIdx.x; x < W; x += kRowThreads) sum += __ldg(gr + x);
    for (int off = 16; off > 0; off >>= 1) sum += __shfl_down_sync(NSGB_FULL, sum, off);
    if ((threadIdx.x & 31) == 0) s_sum[threadIdx.x >> 5] = sum;
    __syncthreads();
    long long total = 0;
#pragma unroll
    for (int k = 0; k < kRowThreads / 32; ++k) total += s_sum[k];
    if (total <= kMeanG * W) {
      for (int x = threadIdx.x; x < W; x += kRowThreads) {
        const int64_t gx = __ldg(gr + x);
        int64_t best = gx * gx;
        for (int64_t k = 1; k < W && k * k < best; ++k) {
          if (x - k >= 0) best = min(best, k * k + sq(__ldg(gr + x - k)));
          if (x + k < W) best = min(best, k * k + sq(__ldg(gr + x + k)));
        }
        store_px<BASINS>(o, mrow, x, best, inf2);
      }
    } else if (dc) {
      dc_row<BASINS>(gr, o, mrow, W, inf2, dc_smem);
    } else if (threadIdx.x == 0) {
      envelope_row<BASINS>(gr, stack_s + (int64_t)y * W, stack_t + (int64_t)y * W, o, mrow, W, inf2);
    }
    __syncthreads();  // s_sum is rewritten for the next row
  }
}

}  // namespace

size_t edt_workspace_bytes(int64_t rows, int64_t cols) {
  const size_t plane = ((size_t)rows * (size_t)cols * sizeof(int) + 255) & ~(size_t)255;
  const size_t chunks = ((size_t)((rows + kChunk - 1) / kChunk) * (size_t)cols * sizeof(int) + 255) & ~(size_t)255;
  return 256 + 3 * plane + 2 * chunks;
}

cudaError_t edt_launch(const uint8_t* mask, int64_t pitch_in, float* out, int64_t pitch_out, int rows, int cols,
                       bool basins, void* ws, cudaStream_t s) {
  const size_t plane = ((size_t)rows * (size_t)cols * sizeof(int) + 255) & ~(size_t)255;
  const int nchunks = (rows + kChunk - 1) / kChunk;
  const size_t chunks = ((size_t)nchunks * (size_t)cols * sizeof(int) + 255) & ~(size_t)255;
  char* p = (char*)ws + 256;
  int* g = (int*)p;
  int* st_s = (int*)(p + plane);
  int* st_t = (int*)(p + 2 * plane);
  int* first0 = (int*)(p + 3 * plane);
  int* last0 = (int*)(p + 3 * plane + chunks);
  const dim3 cgrid((cols + kThreads - 1) / kThreads, nchunks);
  edt_chunk_zeros<<<cgrid, kThreads, 0, s>>>(mask, pitch_in, rows, cols, first0, last0);
  edt_columns<<<cgrid, kThreads, 0, s>>>(mask, pitch_in, rows, cols, first0, last0, g);
  const int rblocks = rows < (1 << 20) ? rows : (1 << 20);
  // divide and conquer: tables fit (u16 columns, 24-bit column field) and 2 (H + W)^2 < 2^40
  const bool dc = cols <= kDcMaxW && (int64_t)rows + cols < (1 << 19);
  const size_t smem = dc ? (((size_t)cols * 2 + 15) & ~(size_t)15) + (size_t)(cols / 2 + 1) * 8 +
                               (size_t)(cols / 2 + 2) * 4
                         : 0;
  cudaError_t e = cudaSuccess;
  if (basins) {
    if (smem > 48 * 1024) e = cudaFuncSetAttribute(edt_rows<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      edt_rows<true><<<rblocks, kRowThreads, smem, s>>>(mask, pitch_in, g, st_s, st_t, out, pitch_out, rows, cols, dc);
  } else {
    if (smem > 48 * 1024) e = cudaFuncSetAttribute(edt_rows<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess)
      edt_rows<false><<<rblocks, kRowThreads, smem, s>>>(mask, pitch_in, g, st_s, st_t, out, pitch_out, rows, cols, dc);
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

}  // namespace nsgb
