// Exact fixed-point sums of doubles with integer arithmetic only.
//
// Why: on GB300 a dependent FP64 instruction costs ~90 cycles, so the
// shuffle-tree reductions of a solver iteration (a few dozen dependent FP64
// adds) and a library division cost more than the iteration's stencil.  The
// integer pipe has none of that latency, and a fixed-point sum is exact, so
// the total does not depend on the order of the terms (deterministic by
// construction).
//
// Format: a sum is a signed 128-bit integer V with a biased exponent anchor A
// (that of the largest term): value = V * 2^(A - 1129).  A double with biased
// exponent e <= A and 53-bit significand m is V = m * 2^(54 + e - A): the
// largest term has its top bit at 2^106, leaving 20 bits of headroom for
// 2^20 terms, and a term more than 2^54 below the largest loses the bits
// under 2^(A - 1129) (truncated toward zero), ~2^-106 of the largest term.
// The total is rounded once, to nearest even, by xsum_to_double.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define XS_HD __host__ __device__ __forceinline__
#else
#define XS_HD inline
#endif

namespace epic {

typedef __int128 xs_int;
typedef unsigned __int128 xs_uint;

XS_HD uint64_t xs_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  __builtin_memcpy(&b, &x, 8);
  return b;
#endif
}

XS_HD double xs_double(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double x;
  __builtin_memcpy(&x, &b, 8);
  return x;
#endif
}

XS_HD int xs_clz64(uint64_t v) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)v);
#else
  return v ? __builtin_clzll(v) : 64;
#endif
}

// Biased exponent used for anchoring: subnormals count as 1, zero as 0.
XS_HD int xs_exponent(double x) {
  const uint64_t b = xs_bits(x);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e) return e;
  return (b << 1) ? 1 : 0;
}

// x as V for anchor A (requires xs_exponent(x) <= A; finite x).
XS_HD xs_int xs_from_double(double x, int A) {
  const uint64_t b = xs_bits(x);
  int e = (int)((b >> 52) & 0x7FF);
  uint64_t m = b & 0xFFFFFFFFFFFFFull;
  if (e) m |= 1ull << 52;
  else e = 1;
  if (!m) return 0;
  const int sh = 54 - (A - e);
  xs_int v;
  if (sh >= 0) v = (xs_int)m << sh;
  else if (sh > -64) v = (xs_int)(m >> (-sh));
  else v = 0;
  return (b >> 63) ? -v : v;
}

// V re-anchored from A to A2 >= A (arithmetic shift: exact unless bits fall
// below 2^(A2 - 1129)).
XS_HD xs_int xs_realign(xs_int v, int A, int A2) {
  const int d = A2 - A;
  if (d <= 0) return v;
  if (d >= 127) return v < 0 ? -1 : 0;
  return v >> d;
}

// The double nearest to V * 2^(A - 1129) (ties to even); results below the
// normal range flush to zero, above it give infinity.  The magnitude's top 64
// bits are rounded to 53 with the bits under them as a sticky bit: a few
// dependent integer operations, no 128-bit shifts by variable amounts.
XS_HD double xs_to_double(xs_int v, int A) {
  if (v == 0) return 0.0;
  const uint64_t sign = v < 0 ? 1u : 0u;
  const xs_uint u = sign ? (xs_uint)(-v) : (xs_uint)v;
  const uint64_t hi = (uint64_t)(u >> 64), lo = (uint64_t)u;
  const int lz = hi ? xs_clz64(hi) : 64 + xs_clz64(lo);
  uint64_t w, rest;
  if (lz >= 64) {
    w = lo << (lz - 64);
    rest = 0;
  } else if (lz == 0) {
    w = hi;
    rest = lo;
  } else {
    w = (hi << lz) | (lo >> (64 - lz));
    rest = lo << lz;
  }
  uint64_t q = w >> 11;  // 53 bits, the top one set
  long E = (long)(127 - lz) + A - 106;
  const bool guard = (w >> 10) & 1, sticky = (w & 0x3FFull) != 0 || rest != 0;
  if (guard && (sticky || (q & 1))) {
    q++;
    if (q >> 53) {
      q >>= 1;
      E++;
    }
  }
  if (E <= 0) return sign ? -0.0 : 0.0;
  if (E >= 2047) return xs_double((sign << 63) | (0x7FFull << 52));
  return xs_double((sign << 63) | ((uint64_t)E << 52) | (q & 0xFFFFFFFFFFFFFull));
}

// v << s and v >> s, 0 for s >= 64 (s is unsigned, so a negative amount
// converted to it is also 0); on the device the PTX shifts, which clamp the
// amount to the width.
XS_HD uint64_t xs_shl(uint64_t v, unsigned s) {
#if defined(__CUDA_ARCH__)
  uint64_t r;
  asm("shl.b64 %0, %1, %2;" : "=l"(r) : "l"(v), "r"(s));
  return r;
#else
  return s >= 64 ? 0 : v << s;
#endif
}
XS_HD uint64_t xs_shr(uint64_t v, unsigned s) {
#if defined(__CUDA_ARCH__)
  uint64_t r;
  asm("shr.b64 %0, %1, %2;" : "=l"(r) : "l"(v), "r"(s));
  return r;
#else
  return s >= 64 ? 0 : v >> s;
#endif
}

#if defined(__CUDACC__)
// Warp total of 128-bit fixed-point values: five 26-bit limbs (the top one
// signed) summed with redux.sync — a limb total of 32 lanes stays below 2^31
// for |v| < 2^122 — and recombined exactly.
__device__ __forceinline__ xs_int xs_warp_sum(xs_int v) {
  const xs_uint u = (xs_uint)v;
  const unsigned M = (1u << 26) - 1;
  const int l0 = __reduce_add_sync(0xffffffffu, (int)((unsigned)u & M));
  const int l1 = __reduce_add_sync(0xffffffffu, (int)((unsigned)(u >> 26) & M));
  const int l2 = __reduce_add_sync(0xffffffffu, (int)((unsigned)(u >> 52) & M));
  const int l3 = __reduce_add_sync(0xffffffffu, (int)((unsigned)(u >> 78) & M));
  const int l4 = __reduce_add_sync(0xffffffffu, (int)(v >> 104));
  const xs_uint s = ((xs_uint)(xs_int)l4 << 104) + ((xs_uint)(unsigned)l3 << 78) + ((xs_uint)(unsigned)l2 << 52) +
                    ((xs_uint)(unsigned)l1 << 26) + (xs_uint)(unsigned)l0;
  return (xs_int)s;
}
#endif

}  // namespace epic

#include <cmath>
#if defined(__CUDACC__)
#define XS_HOST __host__ inline
#else
#define XS_HOST inline
#endif
namespace epic {
// Smallest double T with sqrt(T) >= tol (correctly rounded sqrt), so that for
// r >= 0: sqrt(r) < tol  <=>  bits(r) < bits(T) (non-negative doubles order
// like their bit patterns).  Host only.
XS_HOST double xs_sqrt_threshold(double tol) {
  if (!(tol > 0)) return 0.0;
  if (std::isinf(tol) || std::isinf(tol * tol)) return INFINITY;
  double T = tol * tol;
  while (T > 0 && std::sqrt(T) >= tol) T = std::nextafter(T, 0.0);
  while (std::sqrt(T) < tol) T = std::nextafter(T, INFINITY);
  return T;
}
}  // namespace epic
