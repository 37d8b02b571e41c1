// Tile work queue of the reconstruction kernel (recon.cu): per-tile states, a bounded
// multi-producer / multi-consumer ring with per-slot sequence numbers (Vyukov's queue),
// neighbour marking, and the initial orders.
// Every wait is bounded; a wait that runs out sets the status word.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace nsgb {
namespace tq {

enum TileState : int { kIdle = 0, kQueued = 1, kRunning = 2, kRunningDirty = 3 };


struct Slot {
  int val;
  unsigned seq;
};

struct Ctl {
  int* state;         // [ntiles] TileState
  Slot* slots;        // [cap] work ring
  unsigned* head;     // consumer ticket counter
  unsigned* tail;     // producer ticket counter
  int* pending;       // queued + running tiles
  int* done;          // set once pending reaches zero
  int* status;
  int* stats;         // [0] visits, [1] sweeps, [2] re-runs
  unsigned long long* visit_count;  // budget counter
  unsigned long long* prof;         // [8] phase cycle counters (profiling builds only)
  unsigned cap;       // ring capacity (power of two >= ntiles)
  long long max_visits;
  long long spin_limit;  // polls before a queue wait gives up (kSpinLimit unless overridden)
  int budget_step;
};

__device__ __forceinline__ void st_release_u(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Producer side of the ring (Vyukov's bounded queue): wait until slot `p` is free for this
// lap, fill it, publish it.
__device__ __forceinline__ bool queue_push(const Ctl& c, int t) {
  const unsigned p = atomicAdd(c.tail, 1u);
  Slot* sl = &c.slots[p & (c.cap - 1)];
  long long spins = 0;
  while (ld_acquire_u(&sl->seq) != p) {
    if (++spins > c.spin_limit || ld_relaxed(c.status) != 0) {
      set_status(c.status, kDevTimeout);
      return false;
    }
    __nanosleep(64);
  }
  sl->val = t;
  st_release_u(&sl->seq, p + 1u);
  return true;
}

// Consumer side: claim a ticket and wait for its item; returns -1 once no tile is queued or
// running any more (the done flag: nothing can be pushed again) or after an error.  A waiting
// warp polls its own slot; the done flag only every second wait and the status word every 64th,
// so that idle warps do not flood the L2 lines that the working warps' atomics use.
__device__ __forceinline__ int queue_pop(const Ctl& c) {
  const unsigned tk = atomicAdd(c.head, 1u);
  Slot* sl = &c.slots[tk & (c.cap - 1)];
  long long spins = 0;
  unsigned ns = 64;
  for (;;) {
    if (ld_acquire_u(&sl->seq) == tk + 1u) {
      const int t = *(volatile int*)&sl->val;
      st_release_u(&sl->seq, tk + c.cap);
      return t;
    }
    ++spins;
    if ((spins & 1) == 0 && ld_relaxed(c.done) != 0) return -1;
    if ((spins & 63) == 0 && ld_relaxed(c.status) != 0) return -1;
    if (spins > c.spin_limit) {
      set_status(c.status, kDevTimeout);
      return -1;
    }
    __nanosleep(ns);
    if (ns < 512) ns <<= 1;
  }
}

// Release of a running or queued tile from the pending count; the call that takes it to zero
// raises the done flag.
__device__ __forceinline__ void pending_release(const Ctl& c) {
  if (atomicSub(c.pending, 1) == 1) atomicExch(c.done, 1);
}

// Tile states and the memory order of tile visits.  Every change of a tile's state is an atomic
// read-modify-write, so all of them are totally ordered per tile.  A visit takes its tile with an
// acquire exchange (QUEUED -> RUNNING) before it reads any pixel; a warp that stored pixels marks
// a neighbour with a release `or 1` (IDLE -> QUEUED, RUNNING -> RUNNING_DIRTY, the others
// unchanged), and releases its own tile with a release compare-and-swap.  For a visit V of tile
// t and a marker U of t, either U's `or` comes before V's exchange in t's order -- then V's
// acquire reads from U's release (or a later read-modify-write of the same sequence) and V's
// loads see U's stores -- or after it, and then U sees RUNNING and the visit is run again.  No
// fence is needed on either side.
__device__ __forceinline__ int atom_or_release(int* p, int v) {
  int old;
  asm volatile("atom.release.gpu.global.or.b32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ int atom_exch_acquire(int* p, int v) {
  int old;
  asm volatile("atom.acquire.gpu.global.exch.b32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ int atom_exch_acq_rel(int* p, int v) {
  int old;
  asm volatile("atom.acq_rel.gpu.global.exch.b32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ int atom_cas_acq_rel(int* p, int cmp, int v) {
  int old;
  asm volatile("atom.acq_rel.gpu.global.cas.b32 %0, [%1], %2, %3;" : "=r"(old) : "l"(p), "r"(cmp), "r"(v) : "memory");
  return old;
}

// A neighbour's values may have become stale: make sure it (re)reads them.  One release `or`:
// an idle neighbour becomes queued (and this call pushes it), a running one becomes
// running-dirty (its owner runs it again), a queued one will load after the stores that the
// release orders before the `or`.  The caller's pixel stores are ordered before it by a warp
// barrier.
__device__ __forceinline__ void mark_tile(const Ctl& c, int nt) {
  if (atom_or_release(&c.state[nt], 1) == kIdle) {
    atomicAdd(c.pending, 1);
    queue_push(c, nt);
  }
}

// Initial queue order.  order 0: raster.  order 1: checkerboard, even tiles first.  order 2:
// four colours by (row parity, column parity) in the sequence (0,0), (1,1), (0,1), (1,0), so
// that no two tiles of one colour touch, not even diagonally.  Tiles taken from the queue at
// the same time are then rarely neighbours, and later colours read finished neighbours.
__device__ __forceinline__ int initial_tile(int i, int ntiles, int tiles_x, int order) {
  const int tiles_y = ntiles / tiles_x;
  if (order == 1) {
    // tiles (ty, tx) with (ty + tx) even first, then the odd ones, each in raster order; row ty
    // holds ceil(tiles_x / 2) of its first colour and floor(tiles_x / 2) of the other
    const int hi = (tiles_x + 1) / 2, lo = tiles_x / 2;
    const int even_total = ((tiles_y + 1) / 2) * hi + (tiles_y / 2) * lo;
    int k = i, parity = 0;
    if (k >= even_total) {
      k -= even_total;
      parity = 1;
    }
    // rows alternate between `a` tiles (ty even for parity 0) and `b` tiles
    const int a = parity ? lo : hi, b = parity ? hi : lo;
    const int pair = a + b;
    int ty = pair ? 2 * (k / pair) : 0;
    k = pair ? k % pair : k;
    if (k >= a) {
      k -= a;
      ++ty;
    }
    const int first = ((ty & 1) ^ parity) ? 1 : 0;
    return ty * tiles_x + first + 2 * k;
  }
  if (order == 2) {
    const int seq_py[4] = {0, 1, 0, 1}, seq_px[4] = {0, 1, 1, 0};
    int k = i;
    for (int c = 0; c < 4; ++c) {
      const int py = seq_py[c], px = seq_px[c];
      const int ny = (tiles_y - py + 1) / 2, nx = (tiles_x - px + 1) / 2;
      if (k < ny * nx) return (py + 2 * (k / nx)) * tiles_x + px + 2 * (k % nx);
      k -= ny * nx;
    }
  }
  return i;
}

inline unsigned ring_cap(int64_t ntiles) {
  unsigned c = 32;
  while ((int64_t)c < ntiles) c <<= 1;
  return c;
}


}  // namespace tq
}  // namespace nsgb
