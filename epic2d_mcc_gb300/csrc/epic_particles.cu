// Particle kernels of the FP64 plain form: charge deposit, field gather +
// leapfrog push (+ stable in-place compaction for open boundaries), the
// initial half-step rewind, and the energy/momentum reductions.  The
// Monte-Carlo collisions are in epic_mcc.cu.
//
// Built with -fmad=false: every expression keeps the reference's association
// order and rounding (no contracted multiply-adds), so positions and velocities
// match the reference bit for bit given the same field.
//
// Every particle kernel is a fixed-size persistent launch (a multiple of the SM
// count) that reads the live particle count from device memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "epic_internal.cuh"
#include "epic_mixed.cuh"
#include "epic_device.cuh"
#include "epic_emit.cuh"

namespace epic {

// Domain::XtoL / YtoL (src/domain.cpp:257-264).  With a unit cell (dx == 1,
// the normalisation of norm_scheme 1-4) the division is the identity in IEEE
// arithmetic, so the UNIT variant drops it without changing a bit; FP64
// division is costly on GB300.
template <bool UNIT>
__device__ __forceinline__ double to_logical(double x, double x0, double dx) {
  return UNIT ? (x - x0) : (x - x0) / dx;
}

// Domain::Interpolate (src/domain.cpp:231-255) of both field components from
// the interleaved (efx, efy) grid; returns false when the stencil leaves the grid.
template <int SHAPE>
__device__ __forceinline__ bool gather(const Geom& g, const double2* __restrict__ ef, double lx, double ly, double& ex,
                                       double& ey) {
  if (SHAPE == EPIC_NGP) {
    int gx = (int)round(lx), gy = (int)round(ly);
    if (gx < 0 || gx >= g.nx || gy < 0 || gy >= g.ny) return false;
    double2 f = __ldg(&ef[(long)gx * g.ny + gy]);
    ex = f.x;
    ey = f.y;
    return true;
  }
  int i = (int)lx, j = (int)ly;
  if (i < 0 || i + 1 >= g.nx || j < 0 || j + 1 >= g.ny) return false;
  double di = lx - i, dj = ly - j;
  long k = (long)i * g.ny + j;
  double2 f00 = __ldg(&ef[k]), f01 = __ldg(&ef[k + 1]);
  double2 f10 = __ldg(&ef[k + g.ny]), f11 = __ldg(&ef[k + g.ny + 1]);
  ex = f00.x * (1 - di) * (1 - dj) + f10.x * (di) * (1 - dj) + f01.x * (1 - di) * (dj) + f11.x * (di) * (dj);
  ey = f00.y * (1 - di) * (1 - dj) + f10.y * (di) * (1 - dj) + f01.y * (1 - di) * (dj) + f11.y * (di) * (dj);
  return true;
}

// ------------------------------------------------------------ deposit ---
// Fixed-point CIC weights on the integer pipe.  For a logical coordinate
// l in [0, 2^11) held as X = l * 2^52 (the bits of l under 2^-52 dropped:
// below 2^-52 of the cell, far under the weight quantum), the cell is X >> 52
// and the offset d = X mod 2^52 with 1 - d = 2^52 - d exactly; a weight
// (1-di)(1-dj) etc. is the exact 106-bit product rounded once to the quantum
// 2^-k, where the FP64 form rounds 1-d, the product and the scaled value
// (so the two can differ by one quantum).  GB300 issues FP64 at 1/32 of the
// integer rate, and these weights are most of the deposit's arithmetic.
__device__ __forceinline__ bool fx52(double l, uint64_t& X) {
  const uint64_t b = (uint64_t)__double_as_longlong(l);
  const int e = (int)((b >> 52) & 0x7FF);
  if ((b >> 63) || e >= 1023 + 11) return false;  // negative, or 2^11 and above
  const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | ((uint64_t)(e != 0) << 52);
  const int sh = e - 1023;
  X = sh >= 0 ? (m << sh) : (sh > -64 ? m >> (-sh) : 0ull);
  return true;
}

// round(a * b * 2^-s) for a, b <= 2^52 and 43 <= s < 128 (ties up).
__device__ __forceinline__ unsigned long long fx_weight(uint64_t a, uint64_t b, int s) {
  const unsigned __int128 p = ((unsigned __int128)__umul64hi(a, b) << 64) | (a * b);
  return (unsigned long long)((p + ((unsigned __int128)1 << (s - 1))) >> s);
}

// Species::ScatterSpecies_serial's accumulation (src/species.cpp:174-183) with
// Domain::Scatter (src/domain.cpp:205-228).  FIXED accumulates each CIC weight
// rounded to an integer multiple of 2^-k (k chosen from the capacity so no
// node can overflow): integer addition is associative, so the grid is
// identical run to run; the weight is applied at finalisation.  Otherwise
// FP64 atomics add spwt*w into the same accumulator buffer read as doubles.
// One particle's deposit; false when its stencil leaves the grid.  ORIGIN:
// unit cells and x0 = y0 = +0, where the logical coordinate x - x0 is x.
template <int SHAPE, bool FIXED, bool UNIT, bool ORIGIN = false>
__device__ __forceinline__ bool deposit_one(const Geom& g, double x, double y, double spwt,
                                            unsigned long long* __restrict__ acc, double fx_scale, int wshift) {
  double* facc = reinterpret_cast<double*>(acc);
  double lx = ORIGIN ? x : to_logical<UNIT>(x, g.x0, g.dx);
  double ly = ORIGIN ? y : to_logical<UNIT>(y, g.y0, g.dy);
  if (SHAPE == EPIC_NGP) {
    int gx = (int)round(lx), gy = (int)round(ly);
    if (gx < 0 || gx >= g.nx || gy < 0 || gy >= g.ny) return false;
    long k = (long)gx * g.ny + gy;
    if (FIXED) atomicAdd(&acc[k], (unsigned long long)__double2ll_rn(fx_scale));
    else atomicAdd(&facc[k], spwt);
    return true;
  }
  uint64_t X, Y;
  if (FIXED && fx52(lx, X) && fx52(ly, Y)) {
    const int i = (int)(X >> 52), j = (int)(Y >> 52);
    if (i + 1 >= g.nx || j + 1 >= g.ny) return false;
    const uint64_t one = 1ull << 52, di = X & (one - 1), dj = Y & (one - 1);
    const long k = (long)i * g.ny + j;
    atomicAdd(&acc[k], fx_weight(one - di, one - dj, wshift));
    atomicAdd(&acc[k + g.ny], fx_weight(di, one - dj, wshift));
    atomicAdd(&acc[k + 1], fx_weight(one - di, dj, wshift));
    atomicAdd(&acc[k + g.ny + 1], fx_weight(di, dj, wshift));
    return true;
  }
  int i = (int)lx, j = (int)ly;
  if (i < 0 || i + 1 >= g.nx || j < 0 || j + 1 >= g.ny) return false;
  double di = lx - i, dj = ly - j;
  long k = (long)i * g.ny + j;
  if (FIXED) {
    atomicAdd(&acc[k], (unsigned long long)__double2ll_rn((1 - di) * (1 - dj) * fx_scale));
    atomicAdd(&acc[k + g.ny], (unsigned long long)__double2ll_rn((di) * (1 - dj) * fx_scale));
    atomicAdd(&acc[k + 1], (unsigned long long)__double2ll_rn((1 - di) * (dj) * fx_scale));
    atomicAdd(&acc[k + g.ny + 1], (unsigned long long)__double2ll_rn((di) * (dj) * fx_scale));
  } else {
    atomicAdd(&facc[k], spwt * (1 - di) * (1 - dj));
    atomicAdd(&facc[k + g.ny], spwt * (di) * (1 - dj));
    atomicAdd(&facc[k + 1], spwt * (1 - di) * (dj));
    atomicAdd(&facc[k + g.ny + 1], spwt * (di) * (dj));
  }
  return true;
}

// fx_scale = 2^k: a weight product of two 52-bit offsets carries 2^104.
__device__ __forceinline__ int weight_shift(double fx_scale) {
  return 104 - ((int)(((uint64_t)__double_as_longlong(fx_scale) >> 52) & 0x7FF) - 1023);
}

template <int SHAPE, bool UNIT>
__global__ void __launch_bounds__(PART_THREADS) k_deposit_range(Geom g, SoA p, const long long* __restrict__ d_from,
                                                                const long long* __restrict__ d_n,
                                                                unsigned long long* __restrict__ acc, double fx_scale,
                                                                int* flags) {
  const long long n = *d_n;
  const int wshift = weight_shift(fx_scale);
  bool bad = false;
  for (long long q = *d_from + (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x)
    bad |= !deposit_one<SHAPE, true, UNIT>(g, p.x[q], p.y[q], 0.0, acc, fx_scale, wshift);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) set_flag(flags, FLAG_OUT_OF_GRID);
}

template <int SHAPE, bool FIXED, bool UNIT>
__global__ void __launch_bounds__(PART_THREADS) k_deposit(Geom g, SoA p, const long long* __restrict__ d_n,
                                                          double spwt, double* __restrict__ den,
                                                          unsigned long long* __restrict__ acc, double fx_scale,
                                                          int* flags) {
  const long long n = *d_n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const int wshift = weight_shift(fx_scale);
  bool bad = false;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride)
    bad |= !deposit_one<SHAPE, FIXED, UNIT>(g, p.x[q], p.y[q], spwt, acc, fx_scale, wshift);
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) set_flag(flags, FLAG_OUT_OF_GRID);
}

static bool unit_cell(const Geom& g) { return g.dx == 1.0 && g.dy == 1.0; }

void launch_deposit(cudaStream_t st, const Geom& g, int shape, int fixed, const SoA& p, const long long* d_n,
                    double spwt, double* den, unsigned long long* acc, double fx_scale, int* flags, int grid) {
#define DEP(SH, FX, U) k_deposit<SH, FX, U><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, spwt, den, acc, fx_scale, flags)
  const bool u = unit_cell(g);
  if (shape == EPIC_NGP) {
    if (fixed) { if (u) DEP(EPIC_NGP, true, true); else DEP(EPIC_NGP, true, false); }
    else { if (u) DEP(EPIC_NGP, false, true); else DEP(EPIC_NGP, false, false); }
  } else {
    if (fixed) { if (u) DEP(EPIC_CIC, true, true); else DEP(EPIC_CIC, true, false); }
    else { if (u) DEP(EPIC_CIC, false, true); else DEP(EPIC_CIC, false, false); }
  }
#undef DEP
}

void launch_deposit_range(cudaStream_t st, const Geom& g, int shape, const SoA& p, const long long* d_from,
                          const long long* d_n, unsigned long long* acc, double fx_scale, int* flags, int grid) {
#define DR(SH, U) k_deposit_range<SH, U><<<grid, PART_THREADS, 0, st>>>(g, p, d_from, d_n, acc, fx_scale, flags)
  const bool u = unit_cell(g);
  if (shape == EPIC_NGP) { if (u) DR(EPIC_NGP, true); else DR(EPIC_NGP, false); }
  else { if (u) DR(EPIC_CIC, true); else DR(EPIC_CIC, false); }
#undef DR
}

// The cell i = (int)l and offset d = l - i of a logical coordinate l, on the
// integer pipe, giving the doubles of the FP64 forms bit for bit: for |l| < 1
// (either sign) i = 0 and d = l; for 1 <= l < 2^31 the significand m and
// s = exponent - 1023 give i = m >> (52 - s) and d = ((m << s) mod 2^52) 2^-52,
// exact because l's ulp is at least 2^-52 there; for l <= -1, l >= 2^31, or
// NaN, i = -1 (off the grid, as the reference's truncated index is).
__device__ __forceinline__ void split_cell(double l, int& i, double& d) {
  // Branch-free, with d selected as integer bits: a select of doubles can
  // cost FP64 instructions.
  const uint64_t b = (uint64_t)__double_as_longlong(l);
  const int sh = (int)((b >> 52) & 0x7FF) - 1023;
  const bool small = sh < 0, out = !small && ((b >> 63) || sh > 30);
  const int s = min(max(sh, 0), 30);
  const uint64_t m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const uint64_t F = (m << s) & 0xFFFFFFFFFFFFFull;
  const int t = 63 - __clzll((long long)(F | 1));  // F 2^-52, normalised by F's top bit t
  uint64_t db = F ? (((uint64_t)(971 + t) << 52) | ((F << (52 - t)) & 0xFFFFFFFFFFFFFull)) : 0ull;
  db = small ? b : (out ? 0ull : db);
  i = small ? 0 : (out ? -1 : (int)(m >> (52 - s)));
  asm("mov.b64 %0, %1;" : "=d"(d) : "l"(db));
}

// Bilinear coefficients of the node field over each cell, four double2 per
// cell at 4 (i ny + j): E(i + di, j + dj) = a0 + a1 di + a2 dj + a3 di dj with
// a0 = E00, a1 = E10 - E00, a2 = E01 - E00, a3 = (E11 - E10) - (E01 - E00).
// The same function as the reference's weighted sum (src/domain.cpp:231-255)
// up to the roundings of the differences.
__global__ void k_cell_coef(Geom g, const double2* __restrict__ ef, double2* __restrict__ cell) {
  const int ny = g.ny, nc = (g.nx - 1) * (ny - 1);
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    const int i = c / (ny - 1), j = c - i * (ny - 1);
    const long k = (long)i * ny + j;
    const double2 f00 = ef[k], f01 = ef[k + 1], f10 = ef[k + ny], f11 = ef[k + ny + 1];
    double2* a = cell + 4 * k;
    a[0] = f00;
    a[1] = make_double2(f10.x - f00.x, f10.y - f00.y);
    a[2] = make_double2(f01.x - f00.x, f01.y - f00.y);
    a[3] = make_double2((f11.x - f10.x) - (f01.x - f00.x), (f11.y - f10.y) - (f01.y - f00.y));
  }
}

void launch_cell_coef(cudaStream_t st, const Geom& g, const double2* ef, double2* cell) {
  const int nc = (g.nx - 1) * (g.ny - 1);
  k_cell_coef<<<(nc + 255) / 256 > 0 ? (nc + 255) / 256 : 1, 256, 0, st>>>(g, ef, cell);
}

// The contracted CIC gather from the cell coefficients:
// E = fma(dj, fma(di, a3, a2), fma(di, a1, a0)), 6 FP64 operations for both
// components where the reference's expression takes 22 (each result within a
// few ulps of the largest corner value of the reference's).
__device__ __forceinline__ bool gather_cell(const Geom& g, const double2* __restrict__ cell, double lx, double ly,
                                            double& ex, double& ey) {
  int i, j;
  double di, dj;
  split_cell(lx, i, di);
  split_cell(ly, j, dj);
  if (i < 0 || i + 1 >= g.nx || j < 0 || j + 1 >= g.ny) return false;
  const double2* a = cell + 4 * ((long)i * g.ny + j);
  const double2 a0 = __ldg(a), a1 = __ldg(a + 1), a2 = __ldg(a + 2), a3 = __ldg(a + 3);
  ex = fma(dj, fma(di, a3.x, a2.x), fma(di, a1.x, a0.x));
  ey = fma(dj, fma(di, a3.y, a2.y), fma(di, a1.y, a0.y));
  return true;
}

// A signed integer that orders doubles as < does: the sign-magnitude bits as
// two's complement, so -0 and +0 share the key 0.  NaN keys compare some way
// where < is false both ways; the wrap then still leaves a NaN coordinate NaN.
// The bits are taken through an opaque move: a plain reinterpretation lets
// the compiler fold the key back into FP64 arithmetic (two additions per
// particle on GB300's narrow FP64 pipe).
__device__ __forceinline__ long long dkey(double v) {
  long long b;
  asm("mov.b64 %0, %1;" : "=l"(b) : "d"(v));
  return b < 0 ? -(b & 0x7FFFFFFFFFFFFFFFll) : b;
}

// --------------------------------------------------------------- push ---
// The push's logical coordinates: MAP_GENERAL (x - x0) / dx, MAP_UNIT x - x0
// (dx = 1), MAP_ORIGIN x itself (dx = 1 and x0 = y0 = +0, where x - x0 is x
// bit for bit).
enum { MAP_GENERAL = 0, MAP_UNIT = 1, MAP_ORIGIN = 2 };
static int push_map(const Geom& g) {
  if (!unit_cell(g)) return MAP_GENERAL;
  const bool zero = std::signbit(g.x0) == 0 && g.x0 == 0.0 && std::signbit(g.y0) == 0 && g.y0 == 0.0;
  return zero ? MAP_ORIGIN : MAP_UNIT;
}
template <int MAP>
__device__ __forceinline__ double push_logical(double x, double x0, double dx) {
  return MAP == MAP_ORIGIN ? x : to_logical<MAP == MAP_UNIT>(x, x0, dx);
}

__device__ __forceinline__ double add_rn_volatile(double a, double b) {
  double r;
  asm volatile("add.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
  return r;
}

// Per-launch constants of the contracted push, formed once per thread.
struct PushK {
  double kv, kx;         // qmK dt and c dt
  long long lo, hx, hy;  // order keys of x0, x0 + Lx and x0 + Ly
};
__device__ __forceinline__ PushK push_consts(const Geom& g, double qmK, double c, double dtsub) {
  return PushK{qmK * dtsub, c * dtsub, dkey(g.x0), dkey(g.x0 + g.Lx), dkey(g.x0 + g.Ly)};
}

// Species::Push_species_serial (src/species.cpp:29-170):
//   v += (qm*K) * E * (DT*sub);  x += (vel_norm/(L*W)) * v * (DT*sub)
// then the boundary rule.  qmK = (q/m) * (n0*e*L)/(eps0*W*vel_norm) and
// c = vel_norm/(L*W) come from the host, computed exactly as the reference
// evaluates the leading factors of its expressions.  CONTRACT = false keeps the
// reference's operation order (bit for bit); CONTRACT (EPIC_PUSH_CONTRACTED)
// takes E of a CIC particle from the cell coefficients (ef is then the table
// k_cell_coef writes), splits the coordinates on the integer pipe and uses
// multiply-adds, v = fma(qmK dt, E, v) and x = fma(c dt, v, x): about a
// quarter of the FP64 operations, each result within a few ulps of the
// reference's.  k holds the contracted form's per-launch constants.
template <int SHAPE, int BC, int MAP, bool CONTRACT>
__device__ __forceinline__ bool push_one(const Geom& g, const double2* __restrict__ ef, double qmK, double c,
                                         double dtsub, const PushK& k, double& x, double& y, double& vx, double& vy,
                                         bool& bad) {
  double lx = push_logical<MAP>(x, g.x0, g.dx);
  double ly = push_logical<MAP>(y, g.y0, g.dy);
  double ex, ey;
  const bool in = (SHAPE == EPIC_CIC && CONTRACT) ? gather_cell(g, ef, lx, ly, ex, ey)
                                                  : gather<SHAPE>(g, ef, lx, ly, ex, ey);
  if (!in) {
    bad = true;
    return true;  // keep the particle untouched; the host reports FLAG_OUT_OF_GRID
  }
  if (CONTRACT) {
    vx = fma(k.kv, ex, vx);
    vy = fma(k.kv, ey, vy);
    x = fma(k.kx, vx, x);
    y = fma(k.kx, vy, y);
  } else {
    vx += qmK * ex * dtsub;
    vy += qmK * ey * dtsub;
    x += c * vx * dtsub;
    y += c * vy * dtsub;
  }
  if (BC == EPIC_PBC) {
    // y is compared against x0 as in the reference (src/species.cpp:74-79).
    if (CONTRACT) {
      // The same comparisons on order-preserving integer keys; the FP64
      // additions (x + L or x + (-L) = x - L) run only in the few warps that
      // hold a particle to wrap: volatile, so the compiler cannot hoist them
      // out of the branch.
      const long long qx = dkey(x), qy = dkey(y);
      const bool wx = qx < k.lo || qx >= k.hx, wy = qy < k.lo || qy >= k.hy;
      if (__any_sync(__activemask(), wx || wy)) {
        if (wx) x = add_rn_volatile(x, qx < k.lo ? g.Lx : -g.Lx);
        if (wy) y = add_rn_volatile(y, qy < k.lo ? g.Ly : -g.Ly);
      }
      return true;
    }
    if (x < g.x0) x = x + g.Lx;
    else if (x >= g.x0 + g.Lx) x = x - g.Lx;
    if (y < g.x0) y = y + g.Ly;
    else if (y >= g.x0 + g.Ly) y = y - g.Ly;
    return true;
  } else if (BC == EPIC_OPEN) {
    return !(x < g.x0 || x >= g.x0 + g.Lx || y < g.x0 || y >= g.x0 + g.Ly);
  } else {
    if (x < g.x0) { x = g.x0 + (g.x0 - x); vx = -vx; }
    else if (x >= g.x0 + g.Lx) { x = g.x0 + g.Lx - (x - (g.x0 + g.Lx)); vx = -vx; }
    if (y < g.x0) { y = g.x0 + (g.x0 - y); vy = -vy; }
    else if (y >= g.x0 + g.Ly) { y = g.x0 + g.Ly - (y - (g.x0 + g.Ly)); vy = -vy; }
    return true;
  }
}

// SEL: also the MCC's first pass over the pushed electrons (k_mcc_select's
// test on the new velocities, block-aggregated appends to sel.cand), in rounds
// that every thread of the CTA takes.
template <int SHAPE, int BC, int MAP, bool CONTRACT, bool DEP, bool SEL>
__global__ void __launch_bounds__(PART_THREADS) k_push(Geom g, SoA p, const long long* __restrict__ d_n,
                                                       const double2* __restrict__ ef, double qmK, double c,
                                                       double dtsub, int* flags, unsigned long long* __restrict__ acc,
                                                       double fx_scale, SelectArgs sel) {
  const long long n = *d_n;
  const PushK k = push_consts(g, qmK, c, dtsub);
  const int wshift = DEP ? weight_shift(fx_scale) : 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  bool bad = false;
  if (SEL) {
    __shared__ unsigned int s_cnt[PART_THREADS / 32];
    __shared__ unsigned int s_base;
    const unsigned long long step = *sel.d_step;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const long long nround = (n + stride - 1) / stride;
    for (long long rd = 0; rd < nround; rd++) {
      const long long q = rd * stride + (long long)blockIdx.x * blockDim.x + threadIdx.x;
      bool cand = false;
      if (q < n) {
        double x = p.x[q], y = p.y[q], vx = p.vx[q], vy = p.vy[q];
        push_one<SHAPE, BC, MAP, CONTRACT>(g, ef, qmK, c, dtsub, k, x, y, vx, vy, bad);
        p.x[q] = x;
        p.y[q] = y;
        p.vx[q] = vx;
        p.vy[q] = vy;
        if (DEP)
          bad |= !deposit_one<SHAPE, true, MAP != MAP_GENERAL, MAP == MAP_ORIGIN>(g, x, y, 0.0, acc, fx_scale,
                                                                                  wshift);
        cand = mcc_candidate(sel, q, step, vx, vy, p.vz[q]);
      }
      const unsigned int mask = __ballot_sync(0xffffffffu, cand);
      if (lane == 0) s_cnt[wid] = (unsigned int)__popc(mask);
      __syncthreads();
      if (threadIdx.x == 0) {
        unsigned int tot = 0;
#pragma unroll
        for (int w = 0; w < PART_THREADS / 32; w++) {
          const unsigned int cw = s_cnt[w];
          s_cnt[w] = tot;
          tot += cw;
        }
        s_base = tot ? atomicAdd(sel.cand_count, tot) : 0u;
      }
      __syncthreads();
      if (cand) sel.cand[s_base + s_cnt[wid] + __popc(mask & ((1u << lane) - 1))] = (unsigned int)q;
      __syncthreads();
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) set_flag(flags, FLAG_OUT_OF_GRID);
    return;
  }
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
    double x = p.x[q], y = p.y[q], vx = p.vx[q], vy = p.vy[q];
    push_one<SHAPE, BC, MAP, CONTRACT>(g, ef, qmK, c, dtsub, k, x, y, vx, vy, bad);
    p.x[q] = x;
    p.y[q] = y;
    p.vx[q] = vx;
    p.vy[q] = vy;
    if (DEP)
      bad |= !deposit_one<SHAPE, true, MAP != MAP_GENERAL, MAP == MAP_ORIGIN>(g, x, y, 0.0, acc, fx_scale, wshift);
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) set_flag(flags, FLAG_OUT_OF_GRID);
}

// Open boundaries erase leaving particles keeping the order of the rest
// (std::vector::erase, src/species.cpp:95,106).  Each tile of SCAN_TILE
// particles is loaded into registers, pushed, ranked in index order, and its
// survivors written in place at (prefix of earlier tiles) + rank.  A tile's
// writes land only at or below its own range, in slots earlier tiles have
// already loaded before publishing their counts, so no second buffer is needed.

template <int SHAPE, int BC, int MAP, bool COND, bool CONTRACT>
__global__ void __launch_bounds__(PART_THREADS) k_push_compact(Geom g, SoA p, long long* d_n,
                                                               const double2* __restrict__ ef, double qmK, double c,
                                                               double dtsub, unsigned long long* status,
                                                               unsigned int* tile_ctr, int* flags, CondSet cs,
                                                               long long spin) {
  constexpr int ITEMS = SCAN_TILE / PART_THREADS;
  __shared__ int sm[40];
  __shared__ unsigned long long s_prefix;
  __shared__ int s_tile;
  const long long n = *d_n;
  const int num_tiles = (int)((n + SCAN_TILE - 1) / SCAN_TILE);
  const PushK pk = push_consts(g, qmK, c, dtsub);
  bool bad = false;
  for (;;) {
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(tile_ctr, 1u);
    __syncthreads();
    const int tile = s_tile;
    if (tile >= num_tiles) break;
    const long long base = (long long)tile * SCAN_TILE;
    double x[ITEMS], y[ITEMS], vx[ITEMS], vy[ITEMS], vz[ITEMS];
    int keep[ITEMS];
#pragma unroll
    for (int k = 0; k < ITEMS; k++) {
      long long q = base + (long long)k * PART_THREADS + threadIdx.x;
      keep[k] = 0;
      if (q < n) {
        x[k] = p.x[q]; y[k] = p.y[q]; vx[k] = p.vx[q]; vy[k] = p.vy[q]; vz[k] = p.vz[q];
        keep[k] = push_one<SHAPE, BC, MAP, CONTRACT>(g, ef, qmK, c, dtsub, pk, x[k], y[k], vx[k], vy[k], bad) &&
                          !(COND && in_conductor(cs, x[k], y[k]))
                      ? 1
                      : 0;
      }
    }
    int rank[ITEMS];
    int tile_total = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; k++) {
      int row_total;
      rank[k] = tile_total + block_exclusive_scan(keep[k], &row_total, sm);
      tile_total += row_total;
    }
    if (threadIdx.x == 0) s_prefix = tile_lookback(status, tile, (unsigned long long)tile_total, flags, spin);
    __syncthreads();
    const unsigned long long prefix = s_prefix;
    if (prefix != ~0ull) {
#pragma unroll
      for (int k = 0; k < ITEMS; k++) {
        if (keep[k]) {
          long long o = (long long)prefix + rank[k];
          p.x[o] = x[k]; p.y[o] = y[k]; p.vx[o] = vx[k]; p.vy[o] = vy[k]; p.vz[o] = vz[k];
        }
      }
      if (tile == num_tiles - 1 && threadIdx.x == 0) *d_n = (long long)prefix + tile_total;
    }
    __syncthreads();
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) set_flag(flags, FLAG_OUT_OF_GRID);
}

void launch_push(cudaStream_t st, const Geom& g, int shape, int bc, const SoA& p, long long* d_n, const double2* ef,
                 const double2* cell, double qmK, double c, double dtsub, int* flags,
                 unsigned long long* tile_status, unsigned int* tile_ctr, int grid, int contract,
                 unsigned long long* dep_acc, double fx_scale, const SelectArgs* sel) {
  if (shape == EPIC_CIC && contract) ef = cell;
  if (sel && dep_acc && contract && (bc == EPIC_PBC || bc == EPIC_REFLECTIVE)) {
#define SEL3(SH, B, U) \
  k_push<SH, B, U, true, true, true><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, ef, qmK, c, dtsub, flags, dep_acc, \
                                                                    fx_scale, *sel)
#define SEL2(SH, B)                                        \
  do {                                                     \
    const int map = push_map(g);                           \
    if (map == MAP_ORIGIN) SEL3(SH, B, 2);                 \
    else if (map == MAP_UNIT) SEL3(SH, B, 1);              \
    else SEL3(SH, B, 0);                                   \
  } while (0)
    if (shape == EPIC_NGP) { if (bc == EPIC_PBC) SEL2(EPIC_NGP, EPIC_PBC); else SEL2(EPIC_NGP, EPIC_REFLECTIVE); }
    else { if (bc == EPIC_PBC) SEL2(EPIC_CIC, EPIC_PBC); else SEL2(EPIC_CIC, EPIC_REFLECTIVE); }
#undef SEL2
#undef SEL3
    return;
  }
#define PUSH2(SH, B, U, C, D)                                                                                    \
  k_push<SH, B, U, C, D, false><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, ef, qmK, c, dtsub, flags, dep_acc, \
                                                               fx_scale, SelectArgs{})
#define PUSH1(SH, B, U, C) do { if (dep_acc) PUSH2(SH, B, U, C, true); else PUSH2(SH, B, U, C, false); } while (0)
#define PUSH(SH, B, U) do { if (contract) PUSH1(SH, B, U, true); else PUSH1(SH, B, U, false); } while (0)
#define COMPACT1(SH, U, C)                                                                                      \
  k_push_compact<SH, EPIC_OPEN, U, false, C><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, ef, qmK, c, dtsub,      \
                                                                            tile_status, tile_ctr, flags, CondSet{},      \
                                                                            spin_limit())
#define COMPACT(SH, U) do { if (contract) COMPACT1(SH, U, true); else COMPACT1(SH, U, false); } while (0)
#define BOTH(M, ...)                          \
  do {                                        \
    if (map == MAP_ORIGIN) M(__VA_ARGS__, 2); \
    else if (map == MAP_UNIT) M(__VA_ARGS__, 1); \
    else M(__VA_ARGS__, 0);                   \
  } while (0)
  const int map = push_map(g);
  if (bc == EPIC_OPEN) {
    if (shape == EPIC_NGP) BOTH(COMPACT, EPIC_NGP);
    else BOTH(COMPACT, EPIC_CIC);
  } else if (bc == EPIC_PBC) {
    if (shape == EPIC_NGP) BOTH(PUSH, EPIC_NGP, EPIC_PBC);
    else BOTH(PUSH, EPIC_CIC, EPIC_PBC);
  } else {
    if (shape == EPIC_NGP) BOTH(PUSH, EPIC_NGP, EPIC_REFLECTIVE);
    else BOTH(PUSH, EPIC_CIC, EPIC_REFLECTIVE);
  }
#undef BOTH
#undef COMPACT
#undef COMPACT1
#undef PUSH
#undef PUSH1
#undef PUSH2
}

void launch_push_conductors(cudaStream_t st, const Geom& g, int shape, int bc, const SoA& p, long long* d_n,
                            const double2* ef, const double2* cell, double qmK, double c, double dtsub,
                            const CondSet& cs, int* flags, unsigned long long* tile_status, unsigned int* tile_ctr,
                            int grid, int contract) {
  if (shape == EPIC_CIC && contract) ef = cell;
#define PC1(SH, B, U, C)                                                                                        \
  k_push_compact<SH, B, U, true, C><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, ef, qmK, c, dtsub, tile_status, \
                                                                   tile_ctr, flags, cs, spin_limit())
#define PC(SH, B, U) do { if (contract) PC1(SH, B, U, true); else PC1(SH, B, U, false); } while (0)
#define BOTH(SH, B)                            \
  do {                                         \
    if (map == MAP_ORIGIN) PC(SH, B, 2);       \
    else if (map == MAP_UNIT) PC(SH, B, 1);    \
    else PC(SH, B, 0);                         \
  } while (0)
#define SHAPES(B) do { if (shape == EPIC_NGP) BOTH(EPIC_NGP, B); else BOTH(EPIC_CIC, B); } while (0)
  const int map = push_map(g);
  if (bc == EPIC_OPEN) SHAPES(EPIC_OPEN);
  else if (bc == EPIC_PBC) SHAPES(EPIC_PBC);
  else SHAPES(EPIC_REFLECTIVE);
#undef SHAPES
#undef BOTH
#undef PC
#undef PC1
}

__global__ void k_conductor_rho(double* __restrict__ rho, const int* __restrict__ nodes,
                                const double* __restrict__ vals, int n, int* live) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) rho[nodes[k]] = vals[k];
  if (k == 0) *live = 1;
}

void launch_conductor_rho(cudaStream_t st, double* rho, const int* nodes, const double* vals, int n, int* live) {
  k_conductor_rho<<<(n + 255) / 256 > 0 ? (n + 255) / 256 : 1, 256, 0, st>>>(rho, nodes, vals, n, live);
}

// ------------------------------------------------------------- emitters ---
// Emitter::inject (src/emitter.cpp:5-36) into one species: point q's draws
// from emit_point (epic_emit.cuh), written at the live count.
// MIXED: the record goes to the mixed form's layout (cell and FP32 offsets of
// the FP64 position, FP32 velocities), as the upload converts it.
template <bool MIXED>
__global__ void __launch_bounds__(PART_THREADS) k_emit(SoA p, MixedSoA m, Geom g, const long long* __restrict__ d_n,
                                                       long long cap, EmitDev e, unsigned long long seed,
                                                       const unsigned long long* __restrict__ d_inj,
                                                       const double* __restrict__ uniforms, int* flags) {
  const long long n0 = *d_n;
  const unsigned long long inj = *d_inj;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < e.num; q += gridDim.x * blockDim.x) {
    const long long o = n0 + q;
    if (o >= cap) {
      set_flag(flags, FLAG_CAPACITY);
      continue;
    }
    double x, y, vx, vy, vz;
    emit_point(e, q, seed, inj, uniforms, x, y, vx, vy, vz);
    if (MIXED) {
      int i, j;
      float ox, oy;
      const bool in_x = cell_offset((x - g.x0) / g.dx, g.nx - 1, i, ox);
      const bool in_y = cell_offset((y - g.y0) / g.dy, g.ny - 1, j, oy);
      if (!(in_x && in_y)) set_flag(flags, FLAG_OUT_OF_GRID);
      m.cell[o] = i * g.ny + j;
      m.ox[o] = ox;
      m.oy[o] = oy;
      m.vx[o] = (float)vx;
      m.vy[o] = (float)vy;
      m.vz[o] = (float)vz;
    } else {
      p.x[o] = x;
      p.y[o] = y;
      p.vx[o] = vx;
      p.vy[o] = vy;
      p.vz[o] = vz;
    }
  }
}

__global__ void k_emit_commit(long long* d_n, long long num, long long cap, int* flags) {
  long long n = *d_n + num;
  if (n > cap) {
    set_flag(flags, FLAG_CAPACITY);
    n = cap;
  }
  *d_n = n;
}

__global__ void k_inject_tick(unsigned long long* d_inj) { *d_inj += 1; }

void launch_emit(cudaStream_t st, const ParticleRef& p, const Geom& g, const long long* d_n, long long cap,
                 const EmitDev& e, unsigned long long seed, const unsigned long long* d_inj, const double* uniforms,
                 int* flags, int grid) {
  const int blocks = std::max(1, std::min(grid, (e.num + PART_THREADS - 1) / PART_THREADS));
  if (p.mixed) k_emit<true><<<blocks, PART_THREADS, 0, st>>>(p.f, p.m, g, d_n, cap, e, seed, d_inj, uniforms, flags);
  else k_emit<false><<<blocks, PART_THREADS, 0, st>>>(p.f, p.m, g, d_n, cap, e, seed, d_inj, uniforms, flags);
}

void launch_emit_commit(cudaStream_t st, long long* d_n, long long num, long long cap, int* flags) {
  k_emit_commit<<<1, 1, 0, st>>>(d_n, num, cap, flags);
}

void launch_inject_tick(cudaStream_t st, unsigned long long* d_inj) { k_inject_tick<<<1, 1, 0, st>>>(d_inj); }

// Species::Rewind_species (src/species.cpp:229-246): v -= (0.5*qm*K) * E * DT.
template <int SHAPE, bool UNIT>
__global__ void __launch_bounds__(PART_THREADS) k_rewind(Geom g, SoA p, const long long* __restrict__ d_n,
                                                         const double2* __restrict__ ef, double hqmK, double dt,
                                                         int* flags) {
  const long long n = *d_n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  bool bad = false;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
    double lx = to_logical<UNIT>(p.x[q], g.x0, g.dx);
    double ly = to_logical<UNIT>(p.y[q], g.y0, g.dy);
    double ex, ey;
    if (!gather<SHAPE>(g, ef, lx, ly, ex, ey)) {
      bad = true;
      continue;
    }
    p.vx[q] -= hqmK * ex * dt;
    p.vy[q] -= hqmK * ey * dt;
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) set_flag(flags, FLAG_OUT_OF_GRID);
}

void launch_rewind(cudaStream_t st, const Geom& g, int shape, const SoA& p, const long long* d_n, const double2* ef,
                   double hqmK, double dt, int* flags, int grid) {
#define RW(SH, U) k_rewind<SH, U><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, ef, hqmK, dt, flags)
  const bool u = unit_cell(g);
  if (shape == EPIC_NGP) { if (u) RW(EPIC_NGP, true); else RW(EPIC_NGP, false); }
  else { if (u) RW(EPIC_CIC, true); else RW(EPIC_CIC, false); }
#undef RW
}

// -------------------------------------------------------- reductions ---
// Species::Compute_KE / Compute_Momentum sums (src/species.cpp:248-297):
// what 0 -> sum_p (v_c*v_c)*vn*vn, what 1 -> sum_p v_c*vn, c = x, y, z.
// Two fixed-shape stages (per-block tree, then one block over the partials in
// block order), so the result is identical run to run.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(PART_THREADS) k_particle_sums(int what, SoA p, const long long* __restrict__ d_n,
                                                                double vn, double* partials) {
  const long long n = *d_n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  double s0 = 0, s1 = 0, s2 = 0;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
    double a = p.vx[q], b = p.vy[q], c = p.vz[q];
    if (what == 0) {
      s0 += (a * a) * (vn) * (vn);
      s1 += (b * b) * (vn) * (vn);
      s2 += (c * c) * (vn) * (vn);
    } else {
      s0 += (a) * vn;
      s1 += (b) * vn;
      s2 += (c) * vn;
    }
  }
  __shared__ double sm[3][PART_THREADS / 32];
  s0 = warp_sum(s0);
  s1 = warp_sum(s1);
  s2 = warp_sum(s2);
  if ((threadIdx.x & 31) == 0) {
    sm[0][threadIdx.x >> 5] = s0;
    sm[1][threadIdx.x >> 5] = s1;
    sm[2][threadIdx.x >> 5] = s2;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0;
    for (int w = 0; w < PART_THREADS / 32; w++) t += sm[threadIdx.x][w];
    partials[blockIdx.x * 3 + threadIdx.x] = t;
  }
}

__global__ void k_sum_partials3(const double* partials, int nblocks, double* out) {
  // warp c sums component c: lanes take a fixed strided subset, then a fixed tree.
  const int c = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (c >= 3) return;
  double t = 0;
  for (int b = lane; b < nblocks; b += 32) t += partials[b * 3 + c];
  t = warp_sum(t);
  if (lane == 0) out[c] = t;
}

void launch_particle_sums(cudaStream_t st, int what, const SoA& p, const long long* d_n, double vel_norm,
                          double* partials, double* out3, int grid) {
  k_particle_sums<<<grid, PART_THREADS, 0, st>>>(what, p, d_n, vel_norm, partials);
  k_sum_partials3<<<1, 96, 0, st>>>(partials, grid, out3);
}

// ------------------------------------------- host-resident particles ---
// For a caller that keeps its particles in host memory, as the reference
// keeps part_list (epic_step_host): these kernels read and write that memory
// directly (SM loads and stores over the host link, mapped pinned memory),
// staging tiles of HOSTIO_TILE records of {x, y, vx, vy, vz} in shared memory
// so the host side moves as one contiguous run per tile, and do the step's
// own work on the way, so the transfer hides it: the upload fills the device
// arrays and deposits, the push writes the device arrays and the host records.
constexpr int HOSTIO_TILE = PART_THREADS;

template <int SHAPE, bool UNIT>
__global__ void __launch_bounds__(PART_THREADS) k_upload_deposit(const double* __restrict__ host, long long n, SoA p,
                                                                 long long* __restrict__ d_n, Geom g,
                                                                 unsigned long long* __restrict__ acc,
                                                                 double fx_scale, int* flags) {
  __shared__ double tile[HOSTIO_TILE * 5];
  if (blockIdx.x == 0 && threadIdx.x == 0) *d_n = n;
  const int wshift = weight_shift(fx_scale);
  bool bad = false;
  for (long long base = (long long)blockIdx.x * HOSTIO_TILE; base < n;
       base += (long long)gridDim.x * HOSTIO_TILE) {
    const int cnt = (int)min((long long)HOSTIO_TILE, n - base);
    const double* src = host + base * 5;
    for (int k = threadIdx.x; k < cnt * 5; k += PART_THREADS) tile[k] = src[k];
    __syncthreads();
    if (threadIdx.x < cnt) {
      const double* r = tile + threadIdx.x * 5;
      const long long q = base + threadIdx.x;
      p.x[q] = r[0];
      p.y[q] = r[1];
      p.vx[q] = r[2];
      p.vy[q] = r[3];
      p.vz[q] = r[4];
      bad |= !deposit_one<SHAPE, true, UNIT>(g, r[0], r[1], 0.0, acc, fx_scale, wshift);
    }
    __syncthreads();
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) set_flag(flags, FLAG_OUT_OF_GRID);
}

template <int SHAPE, int BC, int MAP, bool CONTRACT>
__global__ void __launch_bounds__(PART_THREADS) k_push_download(Geom g, SoA p, const long long* __restrict__ d_n,
                                                                const double2* __restrict__ ef, double qmK, double c,
                                                                double dtsub, double* __restrict__ host, int* flags) {
  __shared__ double tile[HOSTIO_TILE * 5];
  const long long n = *d_n;
  const PushK pk = push_consts(g, qmK, c, dtsub);
  bool bad = false;
  for (long long base = (long long)blockIdx.x * HOSTIO_TILE; base < n;
       base += (long long)gridDim.x * HOSTIO_TILE) {
    const int cnt = (int)min((long long)HOSTIO_TILE, n - base);
    if (threadIdx.x < cnt) {
      const long long q = base + threadIdx.x;
      double x = p.x[q], y = p.y[q], vx = p.vx[q], vy = p.vy[q];
      const double vz = p.vz[q];
      push_one<SHAPE, BC, MAP, CONTRACT>(g, ef, qmK, c, dtsub, pk, x, y, vx, vy, bad);
      p.x[q] = x;
      p.y[q] = y;
      p.vx[q] = vx;
      p.vy[q] = vy;
      double* r = tile + threadIdx.x * 5;
      r[0] = x;
      r[1] = y;
      r[2] = vx;
      r[3] = vy;
      r[4] = vz;
    }
    __syncthreads();
    double* dst = host + base * 5;
    for (int k = threadIdx.x; k < cnt * 5; k += PART_THREADS) dst[k] = tile[k];
    __syncthreads();
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) set_flag(flags, FLAG_OUT_OF_GRID);
}

// Records [from, min(n, cap)) to host memory (FLAG_CAPACITY if n > cap).
__global__ void __launch_bounds__(PART_THREADS) k_download(SoA p, const long long* __restrict__ d_n, long long from,
                                                           long long cap, double* __restrict__ host, int* flags) {
  __shared__ double tile[HOSTIO_TILE * 5];
  long long n = *d_n;
  if (n > cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) set_flag(flags, FLAG_CAPACITY);
    n = cap;
  }
  for (long long base = from + (long long)blockIdx.x * HOSTIO_TILE; base < n;
       base += (long long)gridDim.x * HOSTIO_TILE) {
    const int cnt = (int)min((long long)HOSTIO_TILE, n - base);
    if (threadIdx.x < cnt) {
      const long long q = base + threadIdx.x;
      double* r = tile + threadIdx.x * 5;
      r[0] = p.x[q];
      r[1] = p.y[q];
      r[2] = p.vx[q];
      r[3] = p.vy[q];
      r[4] = p.vz[q];
    }
    __syncthreads();
    double* dst = host + base * 5;
    for (int k = threadIdx.x; k < cnt * 5; k += PART_THREADS) dst[k] = tile[k];
    __syncthreads();
  }
}

void launch_upload_deposit(cudaStream_t st, const Geom& g, int shape, const double* host, long long n, const SoA& p,
                           long long* d_n, unsigned long long* acc, double fx_scale, int* flags, int grid) {
#define UPD(SH, U) k_upload_deposit<SH, U><<<grid, PART_THREADS, 0, st>>>(host, n, p, d_n, g, acc, fx_scale, flags)
  const bool u = unit_cell(g);
  if (shape == EPIC_NGP) { if (u) UPD(EPIC_NGP, true); else UPD(EPIC_NGP, false); }
  else { if (u) UPD(EPIC_CIC, true); else UPD(EPIC_CIC, false); }
#undef UPD
}

void launch_push_download(cudaStream_t st, const Geom& g, int shape, int bc, const SoA& p, const long long* d_n,
                          const double2* ef, const double2* cell, double qmK, double c, double dtsub, double* host,
                          int* flags, int grid, int contract) {
  if (shape == EPIC_CIC && contract) ef = cell;
#define PD1(SH, B, U, C) \
  k_push_download<SH, B, U, C><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, ef, qmK, c, dtsub, host, flags)
#define PD(SH, B, U) do { if (contract) PD1(SH, B, U, true); else PD1(SH, B, U, false); } while (0)
#define BOTH(...)                              \
  do {                                         \
    if (map == MAP_ORIGIN) PD(__VA_ARGS__, 2); \
    else if (map == MAP_UNIT) PD(__VA_ARGS__, 1); \
    else PD(__VA_ARGS__, 0);                   \
  } while (0)
  const int map = push_map(g);
  if (bc == EPIC_PBC) {
    if (shape == EPIC_NGP) BOTH(EPIC_NGP, EPIC_PBC);
    else BOTH(EPIC_CIC, EPIC_PBC);
  } else {
    if (shape == EPIC_NGP) BOTH(EPIC_NGP, EPIC_REFLECTIVE);
    else BOTH(EPIC_CIC, EPIC_REFLECTIVE);
  }
#undef BOTH
#undef PD
#undef PD1
}

void launch_download(cudaStream_t st, const SoA& p, const long long* d_n, long long from, long long cap, double* host,
                     int* flags, int grid) {
  k_download<<<grid, PART_THREADS, 0, st>>>(p, d_n, from, cap, host, flags);
}

}  // namespace epic
