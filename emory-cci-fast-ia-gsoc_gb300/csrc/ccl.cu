// Root ranking for the raster-order relabel (ConnComponents::relabel, ConnComponents.cpp:
// 89-118: roots numbered 1..n in raster order) and the kept-component count of the area
// filter (areaThresholdLabeled, ConnComponents.cpp:205-239).  Replaces the reference GPU's
// Thrust transform / inclusive_scan / sort passes (cuda/ccl_uf.cu:285-479, 684-794): the
// global roots are picked out of the list of local roots into a one-bit-per-pixel map, which
// is counted per 1024-pixel block and scanned (one CTA per image); a root's rank is its
// block's offset plus the set bits before it.  No pass reads the label plane.
#include "ccl.cuh"

namespace nsgb {
namespace ccl {

namespace {

constexpr int kRankThreads = 256;

// Global roots among the local roots: set their bit, count them (and the kept ones) per image.
__global__ void __launch_bounds__(kRankThreads) mark_roots(Imgs I, Forest f, int max_roots, int lo, int hi,
                                                           unsigned* __restrict__ bits, int* __restrict__ counts,
                                                           const unsigned* __restrict__ skip) {
  pdl_wait();
  pdl_release();
  const int n = min(__ldcg(f.nroots), max_roots);
  const int lane = threadIdx.x & 31;
  for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const int k = base + threadIdx.x;
    int img = -1;
    bool keep = false;
    if (k < n) {
      const int lr = __ldcg(f.roots + k);
      if (__ldcg(f.L + lr) == lr && !(skip && test_bit(skip, lr))) {
        atomicOr(bits + (lr >> 5), 1u << (lr & 31));
        img = img_of(I, lr, PxBase());
        if (f.A) {
          const int a = __ldcg(f.A + lr);
          keep = a >= lo && a < hi;
        }
      }
    }
    // one atomic per image present in the warp
    const unsigned peers = __match_any_sync(NSGB_FULL, img);
    const unsigned kept = __ballot_sync(NSGB_FULL, keep) & peers;
    if (img >= 0 && (__ffs(peers) - 1) == lane) {
      atomicAdd(counts + 2 * img, __popc(peers));
      if (kept) atomicAdd(counts + 2 * img + 1, __popc(kept));
    }
  }
}

// Roots per 1024-pixel rank block (one warp per block), and per 32-pixel word of the block the
// number of roots before it in the block (wpre[32 * b + j]).
__global__ void __launch_bounds__(kRankThreads) count_blocks(Imgs I, int nblocks, const unsigned* __restrict__ bits,
                                                             int* __restrict__ cnt, int* __restrict__ wpre) {
  pdl_wait();
  pdl_release();
  const int b = blockIdx.x * (kRankThreads / 32) + (threadIdx.x >> 5);
  if (b >= nblocks) return;
  const int lane = threadIdx.x & 31;
  const Img m = img_at(I, img_of(I, b, BlkBase()));
  const int begin = m.px_base + (b - m.blk_base) * kBlockPx;
  const int end = min(begin + kBlockPx, m.px_base + m.H * m.W);
  const int p = begin + 32 * lane;
  int c = 0;
  if (p < end) {
    unsigned w = bits_at(bits, p);
    if (end - p < 32) w &= (1u << (end - p)) - 1u;
    c = __popc(w);
  }
  int x = c;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(NSGB_FULL, x, o);
    if (lane >= o) x += y;
  }
  wpre[32 * b + lane] = x - c;
  if (lane == 31) cnt[b] = x;
}

// One CTA per image: exclusive scan of the image's block counts in place.  The counts are
// taken in passes of 8 x 1024 (coalesced, all loads of a pass in flight at once); thread t
// holds elements j * 1024 + t of the pass.
__global__ void __launch_bounds__(1024) scan_blocks(Imgs I, int* __restrict__ cnt) {
  pdl_wait();
  pdl_release();
  constexpr int J = 8;
  __shared__ int s_tot[J][32];
  __shared__ int s_chunk[J + 1];
  const Img m = img_at(I, blockIdx.x);
  int* c = cnt + m.blk_base;
  const int nb = (m.H * m.W + kBlockPx - 1) / kBlockPx;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int carry = 0;
  for (int base = 0; base < nb; base += J * 1024) {
    int v[J], x[J];
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const int b = base + j * 1024 + threadIdx.x;
      v[j] = b < nb ? c[b] : 0;
    }
#pragma unroll
    for (int j = 0; j < J; ++j) {
      x[j] = v[j];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(NSGB_FULL, x[j], o);
        if (lane >= o) x[j] += y;
      }
      if (lane == 31) s_tot[j][warp] = x[j];
    }
    __syncthreads();
    if (warp < J) {  // warp j scans the warp totals of chunk j
      int w = s_tot[warp][lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(NSGB_FULL, w, o);
        if (lane >= o) w += y;
      }
      s_tot[warp][lane] = w;  // inclusive over warps
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      int run = carry;
      for (int j = 0; j < J; ++j) {
        s_chunk[j] = run;
        run += s_tot[j][31];
      }
      s_chunk[J] = run;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < J; ++j) {
      const int b = base + j * 1024 + threadIdx.x;
      if (b < nb) c[b] = s_chunk[j] + (warp ? s_tot[j][warp - 1] : 0) + x[j] - v[j];
    }
    carry = s_chunk[J];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kRankThreads) assign_ranks(Imgs I, Forest f, int max_roots,
                                                             const unsigned* __restrict__ bits,
                                                             const int* __restrict__ off, const int* __restrict__ wpre,
                                                             int* __restrict__ rank,
                                                             const unsigned* __restrict__ skip) {
  pdl_wait();
  pdl_release();
  const int n = min(__ldcg(f.nroots), max_roots);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int r = __ldcg(f.roots + k);
    if (__ldcg(f.L + r) != r || (skip && test_bit(skip, r))) continue;
    const Img m = img_at(I, img_of(I, r, PxBase()));
    const int local = r - m.px_base;
    const int b = m.blk_base + local / kBlockPx;
    const int j = (local % kBlockPx) >> 5;
    const int p = m.px_base + (local / kBlockPx) * kBlockPx + 32 * j;
    int c = __ldcg(off + b) + __ldcg(wpre + 32 * b + j);
    if (r > p) c += __popc(bits_at(bits, p) & ((1u << (r - p)) - 1u));
    rank[r] = c;
  }
}

}  // namespace

int list_grid(int64_t max_items) {
  int64_t g = max_items / 65536;
  if (g < 2 * 152) g = 2 * 152;
  if (g > 16 * 152) g = 16 * 152;
  return (int)g;
}

int flat_grid(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  if (b < 1) b = 1;
  return (int)b;
}

cudaError_t rank_bits(const Imgs& I, const BatchTotals& t, const unsigned* bits, int* block_tmp, int* wpre,
                      cudaStream_t s) {
  count_blocks<<<(t.blocks + kRankThreads / 32 - 1) / (kRankThreads / 32), kRankThreads, 0, s>>>(I, t.blocks, bits,
                                                                                                  block_tmp, wpre);
  scan_blocks<<<t.n, 1024, 0, s>>>(I, block_tmp);
  return cudaGetLastError();
}

cudaError_t rank_roots(const Imgs& I, const BatchTotals& t, const Forest& f, int lo, int hi, int* rank,
                       unsigned* bits, size_t bits_bytes, int* block_tmp, int* wpre, int* counts, cudaStream_t s,
                       const unsigned* skip, bool pdl, bool zeroed) {
  cudaError_t e = cudaSuccess;
  if (!zeroed && pdl) {
    const ZeroSpans z{{bits, (unsigned*)counts, nullptr, nullptr}, {(int)(bits_bytes / sizeof(unsigned)), 2 * t.n, 0, 0}};
    e = launch_k(true, zero_words, dim3(flat_grid(z.total())), dim3(256), s, z);
  } else if (!zeroed) {
    e = cudaMemsetAsync(bits, 0, bits_bytes, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, sizeof(int) * 2 * (size_t)t.n, s);
  }
  if (e != cudaSuccess) return e;
  const int g = list_grid(t.px);
  const int cb = (t.blocks + kRankThreads / 32 - 1) / (kRankThreads / 32);
  e = launch_k(pdl, mark_roots, dim3(g), dim3(kRankThreads), s, I, f, (int)t.px, lo, hi, bits, counts, skip);
  if (e == cudaSuccess)
    e = launch_k(pdl, count_blocks, dim3(cb), dim3(kRankThreads), s, I, t.blocks, (const unsigned*)bits, block_tmp,
                 wpre);
  if (e == cudaSuccess) e = launch_k(pdl, scan_blocks, dim3(t.n), dim3(1024), s, I, block_tmp);
  if (e == cudaSuccess)
    e = launch_k(pdl, assign_ranks, dim3(g), dim3(kRankThreads), s, I, f, (int)t.px, (const unsigned*)bits,
                 (const int*)block_tmp, (const int*)wpre, rank, skip);
  return e;
}

cudaError_t count_roots(const Imgs& I, const BatchTotals& t, const Forest& f, int lo, int hi, unsigned* bits,
                        int* counts, cudaStream_t s, const unsigned* skip) {
  cudaError_t e = cudaMemsetAsync(counts, 0, sizeof(int) * 2 * (size_t)t.n, s);
  if (e != cudaSuccess) return e;
  mark_roots<<<list_grid(t.px), kRankThreads, 0, s>>>(I, f, (int)t.px, lo, hi, bits, counts, skip);
  return cudaGetLastError();
}

}  // namespace ccl
}  // namespace nsgb
