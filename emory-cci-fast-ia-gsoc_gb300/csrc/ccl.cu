// Root ranking for the raster-order relabel (ConnComponents::relabel, ConnComponents.cpp:
// 89-118: roots numbered 1..n in raster order) and the kept-component count of the area
// filter (areaThresholdLabeled, ConnComponents.cpp:205-239).  Replaces the reference GPU's
// Thrust transform / inclusive_scan / sort passes (cuda/ccl_uf.cu:285-479, 684-794) with a
// three-kernel count / scan / assign over 1024-pixel blocks; every image of a batch is ranked
// on its own (one scan CTA per image).
#include "ccl.cuh"

namespace nsgb {
namespace ccl {

namespace {

constexpr int kRankThreads = 256;

__device__ __forceinline__ bool in_range(int a, int lo, int hi) { return a >= lo && a < hi; }

// Pixel range [begin, end) of rank block b (global pixel indices).
struct BlockRange {
  int begin, end;
};
__device__ __forceinline__ BlockRange block_range(const Imgs& I, int b) {
  const Img m = img_at(I, img_of(I, b, BlkBase()));
  BlockRange r;
  r.begin = m.px_base + (b - m.blk_base) * kBlockPx;
  r.end = m.px_base + m.H * m.W;
  return r;
}

__global__ void __launch_bounds__(kRankThreads) count_roots(Imgs I, const int* __restrict__ L,
                                                            const int* __restrict__ A, int lo, int hi,
                                                            int* __restrict__ cnt, int* __restrict__ kept) {
  __shared__ int s[2][kRankThreads / 32];
  const BlockRange br = block_range(I, blockIdx.x);
  int c = 0, k = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int i = br.begin + j * kRankThreads + threadIdx.x;
    if (i < br.end && __ldcg(&L[i]) == i) {
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

// One CTA per image: exclusive scan of the image's block counts in place; totals into
// counts[2*i] (roots) and counts[2*i+1] (kept).
__global__ void __launch_bounds__(1024) scan_counts(Imgs I, int* __restrict__ cnt, const int* __restrict__ kept,
                                                    int* __restrict__ counts) {
  __shared__ int s_warp[32];
  __shared__ int s_carry;
  __shared__ int s_kept[32];
  const Img m = img_at(I, blockIdx.x);
  const int b0 = m.blk_base;
  const int nb = (m.H * m.W + kBlockPx - 1) / kBlockPx;
  if (threadIdx.x == 0) s_carry = 0;
  int ksum = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += 1024) {
    const int i = base + threadIdx.x;
    const int v = i < nb ? cnt[b0 + i] : 0;
    if (i < nb) ksum += kept[b0 + i];
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
    if (i < nb) cnt[b0 + i] = s_carry + warp_off + x - v;
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
    counts[2 * blockIdx.x] = s_carry;
    counts[2 * blockIdx.x + 1] = t;
  }
}

__global__ void __launch_bounds__(kRankThreads) assign_ranks(Imgs I, const int* __restrict__ L,
                                                             const int* __restrict__ off, int* __restrict__ rank) {
  __shared__ int s_warp[kRankThreads / 32 * 4];
  const BlockRange br = block_range(I, blockIdx.x);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // Pixel order inside the block: j-major (j*256 + tid); warp w, chunk j covers
  // [j*256 + 32w, j*256 + 32w + 32).  Rank order follows the raster index.
  bool isroot[4];
  int pre[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int i = br.begin + j * kRankThreads + threadIdx.x;
    isroot[j] = i < br.end && __ldcg(&L[i]) == i;
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
    const int i = br.begin + j * kRankThreads + threadIdx.x;
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

cudaError_t rank_roots(const Imgs& I, const BatchTotals& t, const int* L, const int* A, int lo, int hi, int* rank,
                       int* block_tmp, int* counts, cudaStream_t s) {
  int* cnt = block_tmp;
  int* kept = block_tmp + t.blocks;
  count_roots<<<t.blocks, kRankThreads, 0, s>>>(I, L, A, lo, hi, cnt, kept);
  scan_counts<<<t.n, 1024, 0, s>>>(I, cnt, kept, counts);
  assign_ranks<<<t.blocks, kRankThreads, 0, s>>>(I, L, cnt, rank);
  return cudaGetLastError();
}

}  // namespace ccl
}  // namespace nsgb
