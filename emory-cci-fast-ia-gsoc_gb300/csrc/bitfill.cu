// Binary hole filling on bit planes: a flood from outside the image through the open pixels.
//
// imfillHoles<T>(binary) (MorphologicOperations.cpp:1859-1926) fills every region of non-
// foreground pixels that does not touch the image border: the reference pads the image,
// reconstructs the padding ring into the complement and inverts.  Here the open pixels (not
// foreground) are one bit each; the flood starts outside the image (every pixel outside counts
// as flooded) and spreads through open pixels, 4- or 8-connected; the filled image is the set
// of pixels the flood did not reach.
//
// A flood tile is 32 rows x 32 words (1024 pixels across) and lives in registers: lane l holds
// word column l of each row (p = open bits, f = flooded bits).  A visit sweeps the tile to its
// local fixed point:
//   * row pass: in each word, the runs of open bits that hold a flooded bit are flooded whole
//     (one add finds the part of each run from its lowest seed up, the same on the reversed word
//     the part down); runs that continue into the next word are joined across the lanes with
//     three ballots per row: a flood enters lane l from the left if lane l-1 ends flooded, or
//     if lane l-1 is entirely open and a flood entered it, and the same add on the lane masks
//     finds every lane such a chain reaches (and from the right, reversed);
//   * column pass: top-down and bottom-up, each row flooded where the row before it is (or,
//     for 8-connectivity, a diagonal neighbour of it) and the pixel is open: two operations per
//     row and word, so the pass is a short chain; the runs are left to the next row pass.
// It ends on a column pass that changes nothing.  The halo (the rows above and below, the pixel
// columns left and right, each with its open and flooded bits) enters as constants; outside the
// image everything is open and flooded.  Scheduling is the reconstruction's (tilequeue.cuh):
// a persistent kernel drains a work ring of tiles, each tile changing state only by atomic
// read-modify-writes (acquire on taking it, release on marking a neighbour and on letting it
// go).  The ring starts with the tiles on the image border, the only ones the flood can enter
// first; a tile whose flooded pixels can reach an unflooded open pixel of a neighbour marks it.
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "bitfill.cuh"
#include "common.cuh"
#include "tilequeue.cuh"

namespace nsgb {

namespace {

using namespace tq;

constexpr int kFloodWarps = 4;
constexpr int kFloodHdrInts = 192;  // the reconstruction's workspace header layout

struct FloodArgs {
  Imgs I;
  const uint32_t* open;
  uint32_t* flooded;
  int max_iters;
  Ctl c;
};

// Bits of word k of a row of width W that lie outside the image (all of them past the row).
__device__ __forceinline__ uint32_t outside_bits(int k, int W) {
  const int nw = bit_words(W);
  if (k >= nw) return 0xFFFFFFFFu;
  if (k < nw - 1 || (W & 31) == 0) return 0u;
  return ~((1u << (W & 31)) - 1u);
}

// Open runs of `p` that hold a bit of `s`, from the lowest such bit towards bit 31.
__device__ __forceinline__ uint32_t fill_up(uint32_t s, uint32_t p) { return (((p + s) ^ p) & p) | s; }

// Open runs of `p` (whole) that hold a bit of `s`.
__device__ __forceinline__ uint32_t fill_runs(uint32_t s, uint32_t p) {
  s &= p;
  return fill_up(s, p) | __brev(fill_up(__brev(s), __brev(p)));
}

// Row pass of one row: g = the row word after the in-word fill; hl / hr = 1 if the pixel left of
// the tile (right of it) floods into this row.  Joins the runs that cross word boundaries.
__device__ __forceinline__ uint32_t row_spread(uint32_t g, uint32_t p, uint32_t hl, uint32_t hr, int lane) {
  const uint32_t ends_right = __ballot_sync(NSGB_FULL, (g >> 31) & 1u);
  const uint32_t ends_left = __ballot_sync(NSGB_FULL, g & 1u);
  const uint32_t all_open = __ballot_sync(NSGB_FULL, p == 0xFFFFFFFFu);
  // bit l: a flood enters lane l at its first pixel (from lane l-1, or the halo for lane 0)
  const uint32_t gl = (ends_right << 1) | hl;
  const uint32_t in_left = fill_up(gl, (all_open << 1) | gl);
  // bit l: a flood enters lane l at its last pixel (from lane l+1, or the halo for lane 31)
  const uint32_t gr = (ends_left >> 1) | (hr << 31);
  const uint32_t in_right = __brev(fill_up(__brev(gr), __brev((all_open >> 1) | gr)));
  const uint32_t seed = ((in_left >> lane) & 1u) | (((in_right >> lane) & 1u) << 31);
  return fill_runs(g | seed, p);  // branch-free: a data-dependent branch here diverges the warp
}

// What row word `prev` floods into the row next to it (before that row's own runs): the same
// columns, and for 8-connectivity the columns beside them (neighbouring lanes' edge bits).
template <int CONN>
__device__ __forceinline__ uint32_t spread_vertical(uint32_t prev, int lane) {
  if constexpr (CONN == 8) {
    uint32_t l = __shfl_up_sync(NSGB_FULL, prev, 1);
    uint32_t r = __shfl_down_sync(NSGB_FULL, prev, 1);
    if (lane == 0) l = 0;
    if (lane == 31) r = 0;
    return prev | (prev << 1) | (prev >> 1) | (l >> 31) | (r << 31);
  } else {
    return prev;
  }
}

template <int CONN>
__device__ __forceinline__ void flood_visit(const FloodArgs& a, int t, int lane) {
  const Imgs& I = a.I;
  const int ii = I.d ? img_of(I, t, FTileBase()) : 0;
  const Img& m = I.d ? I.d[ii] : I.one;
  const int H = m.H, W = m.W;
  const int nw = bit_words(W);
  const int ntx = flood_tiles_x(W), nty = flood_tiles_y(H);
  const int lt = t - (I.d ? m.f_tile_base : 0);
  const int ty = lt / ntx, tx = lt - ty * ntx;
  const int y0 = ty * 32, wc0 = tx * 32, wc = wc0 + lane;
  const uint32_t* P = a.open + m.b_base;
  uint32_t* F = a.flooded + m.b_base;
  const uint32_t out = outside_bits(wc, W);
  const bool col_in = wc < nw;

  // The caller took the tile with an acquire exchange (lane 0); order every lane after it.
  __syncwarp();
  uint32_t p[32], f[32];
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    const int y = y0 + i;
    if (y < H && col_in) {
      const int64_t o = (int64_t)y * nw + wc;
      p[i] = __ldg(P + o) | out;
      f[i] = __ldcg(F + o) | out;
    } else {
      p[i] = 0xFFFFFFFFu;
      f[i] = 0xFFFFFFFFu;
    }
  }
  // halo rows
  uint32_t pt = 0xFFFFFFFFu, ft = 0xFFFFFFFFu, pb = 0xFFFFFFFFu, fb = 0xFFFFFFFFu;
  if (y0 > 0 && col_in) {
    const int64_t o = (int64_t)(y0 - 1) * nw + wc;
    pt = __ldg(P + o) | out;
    ft = __ldcg(F + o) | out;
  }
  if (y0 + 32 < H && col_in) {
    const int64_t o = (int64_t)(y0 + 32) * nw + wc;
    pb = __ldg(P + o) | out;
    fb = __ldcg(F + o) | out;
  }
  // halo columns: pixel left of the tile (bit 31 of word wc0 - 1) and right of it (bit 0 of word
  // wc0 + 32), rows y0 - 1 .. y0 + 32 (bit k = row y0 - 1 + k); outside the image: open, flooded
  uint32_t hl_f[2], hl_p[2], hr_f[2], hr_p[2];
#pragma unroll
  for (int j = 0; j < 2; ++j) {
    const int k = lane + 32 * j;
    const int y = y0 - 1 + k;
    bool lf = true, lp = true, rf = true, rp = true;
    if (k < 34 && y >= 0 && y < H) {
      if (wc0 > 0) {
        const int64_t o = (int64_t)y * nw + wc0 - 1;
        lp = (__ldg(P + o) >> 31) & 1u;
        lf = (__ldcg(F + o) >> 31) & 1u;
      }
      if (wc0 + 32 < nw) {
        const int64_t o = (int64_t)y * nw + wc0 + 32;
        rp = __ldg(P + o) & 1u;
        rf = __ldcg(F + o) & 1u;
      }
    }
    hl_f[j] = __ballot_sync(NSGB_FULL, lf);
    hl_p[j] = __ballot_sync(NSGB_FULL, lp);
    hr_f[j] = __ballot_sync(NSGB_FULL, rf);
    hr_p[j] = __ballot_sync(NSGB_FULL, rp);
  }
  const uint64_t HLf = (uint64_t)hl_f[0] | ((uint64_t)(hl_f[1] & 3u) << 32);
  const uint64_t HLp = (uint64_t)hl_p[0] | ((uint64_t)(hl_p[1] & 3u) << 32);
  const uint64_t HRf = (uint64_t)hr_f[0] | ((uint64_t)(hr_f[1] & 3u) << 32);
  const uint64_t HRp = (uint64_t)hr_p[0] | ((uint64_t)(hr_p[1] & 3u) << 32);
  // what the halo columns flood into row i's first / last pixel (the same row, and for
  // 8-connectivity the rows above and below)
  const uint64_t HLin = CONN == 8 ? (HLf | (HLf >> 1) | (HLf >> 2)) : (HLf >> 1);
  const uint64_t HRin = CONN == 8 ? (HRf | (HRf >> 1) | (HRf >> 2)) : (HRf >> 1);

  uint32_t any = 0;
  int it = 0;
  for (;;) {
    // row pass
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const uint32_t g = fill_runs(f[i], p[i]);
      const uint32_t n = row_spread(g, p[i], (uint32_t)(HLin >> i) & 1u, (uint32_t)(HRin >> i) & 1u, lane);
      any |= n ^ f[i];
      f[i] = n;
    }
    // column pass
    uint32_t cch = 0;
    uint32_t prev = ft;
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const uint32_t n = f[i] | (spread_vertical<CONN>(prev, lane) & p[i]);
      cch |= n ^ f[i];
      f[i] = n;
      prev = n;
    }
    prev = fb;
#pragma unroll
    for (int i = 31; i >= 0; --i) {
      const uint32_t n = f[i] | (spread_vertical<CONN>(prev, lane) & p[i]);
      cch |= n ^ f[i];
      f[i] = n;
      prev = n;
    }
    any |= cch;
    ++it;
    if (!__any_sync(NSGB_FULL, cch != 0)) break;
    if (it >= a.max_iters) {
      if (lane == 0) set_status(a.c.status, kDevNotConverged);
      break;
    }
  }
  if (lane == 0) {
    atomicAdd(&a.c.stats[0], 1);
    atomicAdd(&a.c.stats[1], it);
  }
  if (__any_sync(NSGB_FULL, any != 0) && col_in) {
#pragma unroll
    for (int i = 0; i < 32; ++i)
      if (y0 + i < H) __stcg(F + (int64_t)(y0 + i) * nw + wc, f[i] & ~out);
  }

  // Which neighbours could the tile's flooded border pixels flood further?
  unsigned dirs = 0;  // bit (dy+1)*3 + (dx+1)
  {
    const uint32_t up = spread_vertical<CONN>(f[0], lane) & pt & ~ft;
    const uint32_t dn = spread_vertical<CONN>(f[31], lane) & pb & ~fb;
    if (__any_sync(NSGB_FULL, up != 0)) dirs |= 1u << 1;
    if (__any_sync(NSGB_FULL, dn != 0)) dirs |= 1u << 7;
    // first / last pixel columns of the tile, bit i = row y0 + i
    uint32_t c0 = 0, c1 = 0;
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      c0 |= (f[i] & 1u) << i;
      c1 |= ((f[i] >> 31) & 1u) << i;
    }
    c0 = __shfl_sync(NSGB_FULL, c0, 0);
    c1 = __shfl_sync(NSGB_FULL, c1, 31);
    // halo column pixels of rows y0 .. y0+31 that are open and not flooded
    const uint32_t l_free = (uint32_t)((HLp & ~HLf) >> 1), r_free = (uint32_t)((HRp & ~HRf) >> 1);
    const uint32_t c0r = CONN == 8 ? (c0 | (c0 << 1) | (c0 >> 1)) : c0;
    const uint32_t c1r = CONN == 8 ? (c1 | (c1 << 1) | (c1 >> 1)) : c1;
    if (c0r & l_free) dirs |= 1u << 3;
    if (c1r & r_free) dirs |= 1u << 5;
    if constexpr (CONN == 8) {
      // corners: rows y0 - 1 and y0 + 32 of the halo columns (bits 0 and 33)
      if ((c0 & 1u) && (HLp & ~HLf & 1ull)) dirs |= 1u << 0;
      if ((c1 & 1u) && (HRp & ~HRf & 1ull)) dirs |= 1u << 2;
      if ((c0 >> 31) && ((HLp & ~HLf) >> 33) & 1ull) dirs |= 1u << 6;
      if ((c1 >> 31) && ((HRp & ~HRf) >> 33) & 1ull) dirs |= 1u << 8;
    }
  }
  // The warp barrier orders every lane's stores before the release atomics below.
  __syncwarp();
  if (lane < 9 && ((dirs >> lane) & 1u)) {
    const int ny = ty + lane / 3 - 1, nx = tx + lane % 3 - 1;
    if (ny >= 0 && ny < nty && nx >= 0 && nx < ntx) mark_tile(a.c, (I.d ? m.f_tile_base : 0) + ny * ntx + nx);
  }
  __syncwarp();
  if (lane == 0) {
    if (atom_cas_acq_rel(&a.c.state[t], kRunning, kIdle) == kRunning) {
      pending_release(a.c);
    } else {
      atom_exch_acq_rel(&a.c.state[t], kQueued);
      atomicAdd(&a.c.stats[2], 1);
      queue_push(a.c, t);
    }
  }
  __syncwarp();
}

template <int CONN>
__global__ void __launch_bounds__(kFloodWarps * 32, 2) flood_kernel(FloodArgs a) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    int t = 0;
    if (lane == 0) t = queue_pop(a.c);
    t = __shfl_sync(NSGB_FULL, t, 0);
    if (t < 0) break;
    if (lane == 0) atom_exch_acquire(&a.c.state[t], kRunning);
    flood_visit<CONN>(a, t, lane);
    if (ld_relaxed(a.c.status) != 0) break;
  }
}

// The ring starts with the tiles on the border of each image (state queued); every other tile
// is idle.
__global__ void flood_seed_kernel(Ctl c, Imgs I, int ntiles, unsigned* counter) {
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < c.cap; i += gridDim.x * blockDim.x) {
    if ((int)i >= ntiles) continue;
    const int t = (int)i;
    const Img& m = I.d ? I.d[img_of(I, t, FTileBase())] : I.one;
    const int ntx = flood_tiles_x(m.W), nty = flood_tiles_y(m.H);
    const int lt = t - (I.d ? m.f_tile_base : 0);
    const int ty = lt / ntx, tx = lt - ty * ntx;
    const bool border = ty == 0 || ty == nty - 1 || tx == 0 || tx == ntx - 1;
    c.state[t] = border ? kQueued : kIdle;
    if (border) {
      const unsigned k = atomicAdd(counter, 1u);
      c.slots[k].val = t;
      c.slots[k].seq = k + 1u;
    }
  }
}

__global__ void flood_seed_finish_kernel(Ctl c, const unsigned* counter) {
  const unsigned n = *counter;
  for (unsigned i = n + blockIdx.x * blockDim.x + threadIdx.x; i < c.cap; i += gridDim.x * blockDim.x) {
    c.slots[i].val = -1;
    c.slots[i].seq = i;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *c.head = 0u;
    *c.tail = n;
    *c.pending = (int)n;
    if (n == 0) *c.done = 1;
  }
}

}  // namespace

cudaError_t flood_launch(const Imgs& I, int ntiles, const uint32_t* open, uint32_t* flooded, int conn, void* ws,
                         cudaStream_t s, long long poll_limit) {
  if (ntiles <= 0) return cudaSuccess;
  FloodArgs a;
  a.I = I;
  a.open = open;
  a.flooded = flooded;
  a.max_iters = 1 << 16;
  int* wi = (int*)ws;
  a.c.status = wi + 0;
  a.c.stats = wi + 1;
  a.c.visit_count = (unsigned long long*)(wi + 6);
  a.c.prof = (unsigned long long*)(wi + 160);
  a.c.head = (unsigned*)(wi + 32);
  a.c.tail = (unsigned*)(wi + 64);
  a.c.pending = wi + 96;
  a.c.done = wi + 128;
  a.c.state = wi + kFloodHdrInts;
  a.c.cap = ring_cap(ntiles);
  a.c.slots = (Slot*)(a.c.state + ((ntiles + 1) & ~1));
  a.c.max_visits = 0;
  a.c.budget_step = 1;
  a.c.spin_limit = poll_limit > 0 ? poll_limit : kSpinLimit;
  // The status word (int 0) is the caller's: it is left alone, so an earlier stage's status
  // survives.  The queue's own words are reset.
  cudaError_t e = cudaMemsetAsync(wi + 1, 0, sizeof(int) * (kFloodHdrInts - 1), s);
  if (e != cudaSuccess) return e;
  unsigned* counter = (unsigned*)(wi + 8);
  const int sgrid = (int)((a.c.cap + 255) / 256);
  flood_seed_kernel<<<sgrid, 256, 0, s>>>(a.c, I, ntiles, counter);
  flood_seed_finish_kernel<<<sgrid, 256, 0, s>>>(a.c, counter);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  constexpr int kOccDevices = 64;
  static std::atomic<int> occ_cache[2][kOccDevices];
  int dev = 0;
  e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const int ci = conn == 8 ? 1 : 0;
  const bool cached = dev >= 0 && dev < kOccDevices;
  int occ = cached ? occ_cache[ci][dev].load(std::memory_order_relaxed) : 0;
  if (occ == 0) {
    int bps = 0;
    e = conn == 8 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, flood_kernel<8>, kFloodWarps * 32, 0)
                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, flood_kernel<4>, kFloodWarps * 32, 0);
    if (e != cudaSuccess) return e;
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    occ = bps * sms;
    if (occ <= 0) return cudaErrorLaunchOutOfResources;
    if (cached) occ_cache[ci][dev].store(occ, std::memory_order_relaxed);
  }
  int grid = (ntiles + kFloodWarps - 1) / kFloodWarps;
  if (grid > occ) grid = occ;
  if (grid < 1) grid = 1;
  void* args[] = {&a};
  return cudaLaunchCooperativeKernel(conn == 8 ? (const void*)flood_kernel<8> : (const void*)flood_kernel<4>, dim3(grid),
                                     dim3(kFloodWarps * 32), args, 0, s);
}

}  // namespace nsgb
