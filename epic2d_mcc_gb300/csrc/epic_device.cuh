// Device helpers shared by the particle kernel files (FP64, mixed, MCC).
#pragma once

#include "epic_internal.cuh"

namespace epic {

// ------------------------------------------------------------ helpers ---
static __device__ __forceinline__ void set_flag(int* flags, int bit) { atomicOr(flags, bit); }

// Philox-4x32-10 counter-based generator (Salmon et al., SC'11): the stream is
// addressed by a 96-bit counter (c0, c1, c2) and a 64-bit key; draw k uses
// 53 bits of block k/2.
struct Philox {
  uint32_t c0, c1, c2, key0, key1;
  int k;
  uint4 cur;
  __device__ static uint4 round10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
      uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
      uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
      c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    return c;
  }
  // The k-th draw as a 53-bit integer M; the uniform is M * 2^-53 in [0, 1).
  __device__ unsigned long long next53() {
    if ((k & 1) == 0) cur = round10(make_uint4(c0, c1, c2, (uint32_t)(k >> 1)), key0, key1);
    uint32_t a = (k & 1) ? cur.z : cur.x, b = (k & 1) ? cur.w : cur.y;
    k++;
    return ((unsigned long long)(a >> 5) << 26) | (b >> 6);
  }
  __device__ double next() { return (double)next53() * (1.0 / 9007199254740992.0); }
};

// Speed bin (MCC_SPEED_BINS) from the unbiased exponent e and the top two
// fraction bits q of m = max |v_i|.
__device__ __forceinline__ int speed_bin_of(int e, int q) {
  if (e < MCC_BIN_EMIN) return 0;
  if (e > MCC_BIN_EMAX) return MCC_SPEED_BINS - 1;
  return 1 + 4 * (e - MCC_BIN_EMIN) + q;
}

// The speed bin of an FP64 velocity, on the integer pipe.
__device__ __forceinline__ int speed_bin_fp64(double vx, double vy, double vz) {
  const unsigned long long M = 0x7FFFFFFFFFFFFFFFull;
  const unsigned long long a = (unsigned long long)__double_as_longlong(vx) & M;
  const unsigned long long b = (unsigned long long)__double_as_longlong(vy) & M;
  const unsigned long long c = (unsigned long long)__double_as_longlong(vz) & M;
  const unsigned long long m = max(a, max(b, c));
  return speed_bin_of((int)(m >> 52) - 1023, (int)((m >> 50) & 3));
}

// The speed bin of an FP32 velocity (the mixed form), on the integer pipe.
__device__ __forceinline__ int speed_bin_fp32(float vx, float vy, float vz) {
  const unsigned a = __float_as_uint(vx) & 0x7FFFFFFFu, b = __float_as_uint(vy) & 0x7FFFFFFFu;
  const unsigned c = __float_as_uint(vz) & 0x7FFFFFFFu;
  const unsigned m = max(a, max(b, c));
  const int eb = (int)(m >> 23);  // 0: zero or subnormal (below 2^-126), 255: inf / NaN
  return speed_bin_of(eb == 255 ? 1 << 20 : eb - 127, (int)((m >> 21) & 3));
}

// The MCC's first pass for electron q (Philox mode): its first draw against the
// cut of its speed bin (or cut53 for every bin without a table).
__device__ __forceinline__ bool mcc_first_draw_passes(const SelectArgs& s, long long q, unsigned long long step,
                                                      unsigned long long cut) {
  Philox src{(uint32_t)q, (uint32_t)(q >> 32), (uint32_t)step, (uint32_t)s.seed, (uint32_t)(s.seed >> 32), 0,
             make_uint4(0, 0, 0, 0)};
  return src.next53() < cut;
}

__device__ __forceinline__ bool mcc_candidate(const SelectArgs& s, long long q, unsigned long long step, double vx,
                                              double vy, double vz) {
  const unsigned long long cut = s.bin_cut ? __ldg(&s.bin_cut[speed_bin_fp64(vx, vy, vz)]) : s.cut53;
  return mcc_first_draw_passes(s, q, step, cut);
}

__device__ __forceinline__ bool mcc_candidate(const SelectArgs& s, long long q, unsigned long long step, float vx,
                                              float vy, float vz) {
  const unsigned long long cut = s.bin_cut ? __ldg(&s.bin_cut[speed_bin_fp32(vx, vy, vz)]) : s.cut53;
  return mcc_first_draw_passes(s, q, step, cut);
}


// Ordered tile scan (decoupled look-back).  Tiles are claimed in increasing
// order through an atomic counter, so every tile a block waits on belongs to a
// block that is already running; each wait is bounded by `limit` polls.
// status[t] = (state << 62) | value, state 1 = tile aggregate, 2 = inclusive
// prefix.  Called by one thread; returns the exclusive prefix of `tile`, or
// ~0 on timeout (FLAG_TIMEOUT set).
static __device__ unsigned long long tile_lookback(unsigned long long* status, int tile, unsigned long long count,
                                                   int* flags, long long limit) {
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
      if (++spins >= limit) {
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

// Grid::IsGrid of any conductor (src/grid.cpp:11-65, src/electrode.cpp:20-26),
// for the FP64 and the mixed push.
__device__ __forceinline__ bool in_conductor(const CondSet& cs, double x, double y) {
  for (int k = 0; k < cs.nrect; k++) {
    const double4 r = cs.rect[k];
    if (x >= r.x && x <= r.y && y >= r.z && y <= r.w) return true;
  }
  if (cs.ncirc && *cs.live) {
    for (int k = 0; k < cs.ncirc; k++) {
      const double4 e = cs.circ[k];
      const double dx = __dsub_rn(x, e.x), dy = __dsub_rn(y, e.y);
      if (__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)) <= e.z) return true;  // uncontracted in every file
    }
  }
  return false;
}

}  // namespace epic
