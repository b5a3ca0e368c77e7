// Device helpers shared by the particle kernel files (FP64, mixed, MCC).
#pragma once

#include "epic_internal.cuh"

namespace epic {

// ------------------------------------------------------------ helpers ---
static __device__ __forceinline__ void set_flag(int* flags, int bit) { atomicOr(flags, bit); }

// Ordered tile scan (decoupled look-back).  Tiles are claimed in increasing
// order through an atomic counter, so every tile a block waits on belongs to a
// block that is already running; each wait is bounded by SPIN_LIMIT polls.
// status[t] = (state << 62) | value, state 1 = tile aggregate, 2 = inclusive
// prefix.  Called by one thread; returns the exclusive prefix of `tile`, or
// ~0 on timeout (FLAG_TIMEOUT set).
static __device__ unsigned long long tile_lookback(unsigned long long* status, int tile, unsigned long long count,
                                            int* flags) {
  const unsigned long long MASK = (1ull << 62) - 1;
  if (tile == 0) {
    __threadfence();
    atomicExch(&status[0], (2ull << 62) | count);
    return 0;
  }
  __threadfence();
  atomicExch(&status[tile], (1ull << 62) | count);
  unsigned long long prefix = 0;
  int t = tile - 1;
  long long spins = 0;
  while (t >= 0) {
    unsigned long long v = *((volatile unsigned long long*)&status[t]);
    unsigned long long st = v >> 62;
    if (st == 0) {
      if (++spins > SPIN_LIMIT) {
        set_flag(flags, FLAG_TIMEOUT);
        return ~0ull;
      }
      __nanosleep(32);
      continue;
    }
    prefix += v & MASK;
    if (st == 2) break;
    t--;
  }
  __threadfence();
  atomicExch(&status[tile], (2ull << 62) | (prefix + count));
  return prefix;
}

// Block-wide exclusive scan of one int per thread (PART_THREADS threads).
static __device__ __forceinline__ int block_exclusive_scan(int v, int* total, int* sm /* >= 33 ints */) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sm[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < (PART_THREADS / 32) ? sm[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < (PART_THREADS / 32)) sm[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  int warp_prefix = wid > 0 ? sm[wid - 1] : 0;
  *total = sm[PART_THREADS / 32 - 1];
  __syncthreads();
  return warp_prefix + x - v;
}

}  // namespace epic
