// Root ranking for the raster-order relabel (ConnComponents::relabel, ConnComponents.cpp:
// 89-118: roots numbered 1..n in raster order) and the kept-component count of the area
// filter (areaThresholdLabeled, ConnComponents.cpp:205-239).  Replaces the reference GPU's
// Thrust transform / inclusive_scan / sort passes (cuda/ccl_uf.cu:285-479, 684-794) with a
// three-kernel count / scan / assign over 1024-pixel blocks.
#include "ccl.cuh"

namespace nsgb {
namespace ccl {

namespace {

constexpr int kBlockPx = 1024;
constexpr int kRankThreads = 256;

__device__ __forceinline__ bool in_range(int a, int lo, int hi) { return a >= lo && a < hi; }

__global__ void __launch_bounds__(kRankThreads) count_roots(const int* __restrict__ L, const int* __restrict__ A,
                                                            int64_t n, int lo, int hi, int* __restrict__ cnt,
                                                            int* __restrict__ kept) {
  __shared__ int s[2][kRankThreads / 32];
  const int64_t base = (int64_t)blockIdx.x * kBlockPx;
  int c = 0, k = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int64_t i = base + j * kRankThreads + threadIdx.x;
    if (i < n && __ldcg(&L[i]) == (int)i) {
      ++c;
      if (A && in_range(__ldcg(&A[i]), lo, hi)) ++k;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    c += __shfl_down_sync(NSGB_FULL, c, o);
    k += __shfl_down_sync(NSGB_FULL, k, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s[0][threadIdx.x >> 5] = c;
    s[1][threadIdx.x >> 5] = k;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int tc = 0, tk = 0;
    for (int w = 0; w < kRankThreads / 32; ++w) {
      tc += s[0][w];
      tk += s[1][w];
    }
    cnt[blockIdx.x] = tc;
    kept[blockIdx.x] = tk;
  }
}

// Single CTA: exclusive scan of cnt[0..nb) in place; totals into counts[0] (roots) and
// counts[1] (kept).
__global__ void __launch_bounds__(1024) scan_counts(int* __restrict__ cnt, const int* __restrict__ kept, int nb,
                                                    int* __restrict__ counts) {
  __shared__ int s_warp[32];
  __shared__ int s_carry;
  __shared__ int s_kept[32];
  if (threadIdx.x == 0) s_carry = 0;
  int ksum = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += 1024) {
    const int i = base + threadIdx.x;
    const int v = i < nb ? cnt[i] : 0;
    if (i < nb) ksum += kept[i];
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(NSGB_FULL, x, o);
      if ((threadIdx.x & 31) >= o) x += y;
    }
    if ((threadIdx.x & 31) == 31) s_warp[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
      int w = s_warp[threadIdx.x];
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(NSGB_FULL, w, o);
        if (threadIdx.x >= o) w += y;
      }
      s_warp[threadIdx.x] = w;
    }
    __syncthreads();
    const int warp_off = (threadIdx.x >> 5) ? s_warp[(threadIdx.x >> 5) - 1] : 0;
    if (i < nb) cnt[i] = s_carry + warp_off + x - v;
    __syncthreads();
    if (threadIdx.x == 1023) s_carry += warp_off + x;
    __syncthreads();
  }
  for (int o = 16; o > 0; o >>= 1) ksum += __shfl_down_sync(NSGB_FULL, ksum, o);
  if ((threadIdx.x & 31) == 0) s_kept[threadIdx.x >> 5] = ksum;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < 32; ++w) t += s_kept[w];
    counts[0] = s_carry;
    counts[1] = t;
  }
}

__global__ void __launch_bounds__(kRankThreads) assign_ranks(const int* __restrict__ L, int64_t n,
                                                             const int* __restrict__ off, int* __restrict__ rank) {
  __shared__ int s_warp[kRankThreads / 32 * 4];
  const int64_t base = (int64_t)blockIdx.x * kBlockPx;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // Pixel order inside the block: j-major (j*256 + tid); warp w, chunk j covers
  // [j*256 + 32w, j*256 + 32w + 32).  Rank order follows the raster index.
  bool isroot[4];
  int pre[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int64_t i = base + j * kRankThreads + threadIdx.x;
    isroot[j] = i < n && __ldcg(&L[i]) == (int)i;
    const unsigned b = __ballot_sync(NSGB_FULL, isroot[j]);
    pre[j] = __popc(b & ((1u << lane) - 1u));
    if (lane == 0) s_warp[j * (kRankThreads / 32) + warp] = __popc(b);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int run = 0;
    for (int t = 0; t < 4 * (kRankThreads / 32); ++t) {
      const int c = s_warp[t];
      s_warp[t] = run;
      run += c;
    }
  }
  __syncthreads();
  const int o = off[blockIdx.x];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    if (!isroot[j]) continue;
    const int64_t i = base + j * kRankThreads + threadIdx.x;
    rank[i] = o + s_warp[j * (kRankThreads / 32) + warp] + pre[j];
  }
}

}  // namespace

int flat_grid(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return (int)b;
}

size_t rank_tmp_ints(int64_t n) { return 2 * (size_t)((n + kBlockPx - 1) / kBlockPx) + 2; }

cudaError_t rank_roots(const int* L, const int* A, int64_t n, int lo, int hi, int* rank, int* block_tmp, int* counts,
                       cudaStream_t s) {
  const int nb = (int)((n + kBlockPx - 1) / kBlockPx);
  int* cnt = block_tmp;
  int* kept = block_tmp + nb;
  count_roots<<<nb, kRankThreads, 0, s>>>(L, A, n, lo, hi, cnt, kept);
  scan_counts<<<1, 1024, 0, s>>>(cnt, kept, nb, counts);
  assign_ranks<<<nb, kRankThreads, 0, s>>>(L, n, cnt, rank);
  return cudaGetLastError();
}

}  // namespace ccl
}  // namespace nsgb
