// Particle kernels of the FP64 plain form: charge deposit, field gather +
// leapfrog push (+ stable in-place compaction for open boundaries), the
// initial half-step rewind, Monte-Carlo collisions with ordered appends, and
// the energy/momentum reductions.
//
// Built with -fmad=false: every expression keeps the reference's association
// order and rounding (no contracted multiply-adds), so positions and velocities
// match the reference bit for bit given the same field.
//
// Every particle kernel is a fixed-size persistent launch (a multiple of the SM
// count) that reads the live particle count from device memory.
#include <cuda_runtime.h>

#include "epic_internal.cuh"

namespace epic {

// ------------------------------------------------------------ helpers ---
__device__ __forceinline__ void set_flag(int* flags, int bit) { atomicOr(flags, bit); }

// Ordered tile scan (decoupled look-back).  Tiles are claimed in increasing
// order through an atomic counter, so every tile a block waits on belongs to a
// block that is already running; each wait is bounded by SPIN_LIMIT polls.
// status[t] = (state << 62) | value, state 1 = tile aggregate, 2 = inclusive
// prefix.  Called by one thread; returns the exclusive prefix of `tile`, or
// ~0 on timeout (FLAG_TIMEOUT set).
__device__ unsigned long long tile_lookback(unsigned long long* status, int tile, unsigned long long count,
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
__device__ __forceinline__ int block_exclusive_scan(int v, int* total, int* sm /* >= 33 ints */) {
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
// Species::ScatterSpecies_serial's accumulation (src/species.cpp:174-183) with
// Domain::Scatter (src/domain.cpp:205-228).  FIXED accumulates each CIC weight
// rounded to an integer multiple of 2^-k (k chosen from the capacity so no
// node can overflow): integer addition is associative, so the grid is
// identical run to run; the weight is applied at finalisation.  Otherwise
// FP64 atomics add spwt*w into the same accumulator buffer read as doubles.
template <int SHAPE, bool FIXED, bool UNIT>
__global__ void __launch_bounds__(PART_THREADS) k_deposit(Geom g, SoA p, const long long* __restrict__ d_n,
                                                          double spwt, double* __restrict__ den,
                                                          unsigned long long* __restrict__ acc, double fx_scale,
                                                          int* flags) {
  const long long n = *d_n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  double* facc = reinterpret_cast<double*>(acc);
  bool bad = false;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
    double lx = to_logical<UNIT>(p.x[q], g.x0, g.dx);
    double ly = to_logical<UNIT>(p.y[q], g.y0, g.dy);
    if (SHAPE == EPIC_NGP) {
      int gx = (int)round(lx), gy = (int)round(ly);
      if (gx < 0 || gx >= g.nx || gy < 0 || gy >= g.ny) {
        bad = true;
        continue;
      }
      long k = (long)gx * g.ny + gy;
      if (FIXED) atomicAdd(&acc[k], (unsigned long long)__double2ll_rn(fx_scale));
      else atomicAdd(&facc[k], spwt);
    } else {
      int i = (int)lx, j = (int)ly;
      if (i < 0 || i + 1 >= g.nx || j < 0 || j + 1 >= g.ny) {
        bad = true;
        continue;
      }
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
    }
  }
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

// --------------------------------------------------------------- push ---
// Species::Push_species_serial (src/species.cpp:29-170):
//   v += (qm*K) * E * (DT*sub);  x += (vel_norm/(L*W)) * v * (DT*sub)
// then the boundary rule.  qmK = (q/m) * (n0*e*L)/(eps0*W*vel_norm) and
// c = vel_norm/(L*W) come from the host, computed exactly as the reference
// evaluates the leading factors of its expressions.
template <int SHAPE, int BC, bool UNIT>
__device__ __forceinline__ bool push_one(const Geom& g, const double2* __restrict__ ef, double qmK, double c,
                                         double dtsub, double& x, double& y, double& vx, double& vy, bool& bad) {
  double lx = to_logical<UNIT>(x, g.x0, g.dx);
  double ly = to_logical<UNIT>(y, g.y0, g.dy);
  double ex, ey;
  if (!gather<SHAPE>(g, ef, lx, ly, ex, ey)) {
    bad = true;
    return true;  // keep the particle untouched; the host reports FLAG_OUT_OF_GRID
  }
  vx += qmK * ex * dtsub;
  vy += qmK * ey * dtsub;
  x += c * vx * dtsub;
  y += c * vy * dtsub;
  if (BC == EPIC_PBC) {
    // y is compared against x0 as in the reference (src/species.cpp:74-79).
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

template <int SHAPE, int BC, bool UNIT>
__global__ void __launch_bounds__(PART_THREADS) k_push(Geom g, SoA p, const long long* __restrict__ d_n,
                                                       const double2* __restrict__ ef, double qmK, double c,
                                                       double dtsub, int* flags) {
  const long long n = *d_n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  bool bad = false;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride) {
    double x = p.x[q], y = p.y[q], vx = p.vx[q], vy = p.vy[q];
    push_one<SHAPE, BC, UNIT>(g, ef, qmK, c, dtsub, x, y, vx, vy, bad);
    p.x[q] = x;
    p.y[q] = y;
    p.vx[q] = vx;
    p.vy[q] = vy;
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) set_flag(flags, FLAG_OUT_OF_GRID);
}

// Open boundaries erase leaving particles keeping the order of the rest
// (std::vector::erase, src/species.cpp:95,106).  Each tile of SCAN_TILE
// particles is loaded into registers, pushed, ranked in index order, and its
// survivors written in place at (prefix of earlier tiles) + rank.  A tile's
// writes land only at or below its own range, in slots earlier tiles have
// already loaded before publishing their counts, so no second buffer is needed.
template <int SHAPE, bool UNIT>
__global__ void __launch_bounds__(PART_THREADS) k_push_compact(Geom g, SoA p, long long* d_n,
                                                               const double2* __restrict__ ef, double qmK, double c,
                                                               double dtsub, unsigned long long* status,
                                                               unsigned int* tile_ctr, int* flags) {
  constexpr int ITEMS = SCAN_TILE / PART_THREADS;
  __shared__ int sm[40];
  __shared__ unsigned long long s_prefix;
  __shared__ int s_tile;
  const long long n = *d_n;
  const int num_tiles = (int)((n + SCAN_TILE - 1) / SCAN_TILE);
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
        keep[k] = push_one<SHAPE, EPIC_OPEN, UNIT>(g, ef, qmK, c, dtsub, x[k], y[k], vx[k], vy[k], bad) ? 1 : 0;
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
    if (threadIdx.x == 0) s_prefix = tile_lookback(status, tile, (unsigned long long)tile_total, flags);
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
                 double qmK, double c, double dtsub, int* flags, unsigned long long* tile_status,
                 unsigned int* tile_ctr, int grid) {
#define PUSH(SH, B, U) k_push<SH, B, U><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, ef, qmK, c, dtsub, flags)
#define COMPACT(SH, U) \
  k_push_compact<SH, U><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, ef, qmK, c, dtsub, tile_status, tile_ctr, flags)
#define BOTH(M, ...) \
  do { if (u) M(__VA_ARGS__, true); else M(__VA_ARGS__, false); } while (0)
  const bool u = unit_cell(g);
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
#undef PUSH
}

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

// ---------------------------------------------------------------- MCC ---
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): counter-based, so the
// k-th draw of electron p at step s is a pure function of (p, s, k, seed).
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

struct Injected {
  const double* u;
  __device__ double next() { return *u++; }
};

// Cross-section lookup: reference linear table (nearest index,
// src/collision.cpp:194-197) or the logarithmic extension.
struct Sigma {
  double tot, ela, exc, ion;
};

__device__ __forceinline__ Sigma sigma_at(const CrossSections& cs, double energy, double velocity_unused) {
  Sigma s;
  if (cs.kind == 0) {
    int idx = (int)(energy / cs.de + 0.5);
    if (idx > (int)cs.n - 1) idx = (int)cs.n - 1;
    s.tot = __ldg(&cs.tot[idx]);
    s.ela = __ldg(&cs.ela[idx]);
    s.exc = __ldg(&cs.exc[idx]);
    s.ion = __ldg(&cs.ion[idx]);
  } else {
    double e = fmin(fmax(energy, cs.e_min), cs.e_max);
    double u = (log(e) - cs.log_emin) * cs.inv_dlog;
    int i = (int)u;
    if (i > (int)cs.n - 2) i = (int)cs.n - 2;
    if (i < 0) i = 0;
    double f = u - i;
    s.ela = __ldg(&cs.ela[i]) * (1 - f) + __ldg(&cs.ela[i + 1]) * f;
    s.exc = __ldg(&cs.exc[i]) * (1 - f) + __ldg(&cs.exc[i + 1]) * f;
    s.ion = __ldg(&cs.ion[i]) * (1 - f) + __ldg(&cs.ion[i + 1]) * f;
    s.tot = __ldg(&cs.tot[i]) * (1 - f) + __ldg(&cs.tot[i + 1]) * f;
  }
  return s;
}

// Init::SampleVel (src/init.cpp:104-114).
template <class D>
__device__ __forceinline__ double sample_vel(D& src, double mass, double temp) {
  double v_th = sqrt(2 * K_B * temp * (QE / K_B) / mass);
  double u1 = src.next();
  double u2 = src.next();
  double u3 = src.next();
  return v_th * sqrt(2.0) * (u1 + u2 + u3 - 1.5);
}

struct MccParams {
  double vn, dt_phys, ion_mass, ion_temp, F1, F2, p_cut;
  unsigned long long cut53;  // ceil(p_cut * 2^53): u < p_cut  <=>  M < cut53 for u = M * 2^-53
  int null_collision;
};

// Products of one ionisation: the secondary electron and the new ion at the
// primary's position.
struct IonEvent {
  double x, y, ev[3], iv[3];
};

// CollisionHandler::handle_collisions for one electron plus collision_electron
// (src/collision.cpp:60-207), after its first draw u0 passed the early-out
// below; later draws come from `src` in the reference's order.  Returns 0
// (none), 1 elastic, 2 excitation, 3 ionisation (products in evt).
//
// Early-out: p_cut bounds the collision probability of every electron from
// above (1 - exp(-nu_max dt), nu_max >= tot(E)*|v| over the table, plus a
// relative margin of 1e-9 for rounding), so u0 >= p_cut means "no collision"
// in the reference's test p_coll > u0 too, and such electrons are rejected
// before their velocity is read.  With Philox the test is an integer compare
// of the draw's 53-bit mantissa.  In null-collision mode p_cut is the
// null-collision probability itself and a second draw accepts with nu/nu_max.
template <class D>
__device__ int mcc_collide(const CrossSections& cs, const MccParams& m, const SoA& e, long long q, D& src, double u0,
                           IonEvent& evt) {
  double* pe = evt.ev;
  double* pi = evt.iv;
  double vx = e.vx[q], vy = e.vy[q], vz = e.vz[q];
  double v_sqr = (vx * vx + vy * vy + vz * vz) * m.vn * m.vn;
  double velocity = sqrt(v_sqr);
  double energy = (0.5 * ME * v_sqr) / EV;
  Sigma s = sigma_at(cs, energy, velocity);
  double nu = s.tot * velocity;
  if (m.null_collision) {
    if (!(src.next() * cs.nu_max < nu)) return 0;
  } else {
    double p_coll = 1 - exp(-nu * m.dt_phys);
    if (!(p_coll > u0)) return 0;
  }
  double gx = vx, gy = vy, gz = vz;
  double g = sqrt(gx * gx + gy * gy + gz * gz);
  double wx = m.F1 * vx, wy = m.F1 * vy, wz = m.F1 * vz;
  double theta, phi, chi, eta;
  if (gx == 0) theta = 0.5 * PI_REF;
  else theta = atan2(sqrt(gy * gy + gz * gz), gx);
  if (gy == 0) phi = gz > 0 ? 0.5 * PI_REF : -0.5 * PI_REF;
  else phi = atan2(gz, gy);
  double st = sin(theta), ct = cos(theta), sp = sin(phi), cp = cos(phi);
  double t0 = s.ela;
  double t1 = t0 + s.exc;
  double t2 = t1 + s.ion;
  int kind;
  if (src.next() < (t0 / t2)) {
    kind = 1;
    chi = acos(1.0 - 2.0 * src.next());
    eta = 2 * PI_REF * src.next();
  } else if (src.next() < (t1 / t2)) {
    kind = 2;
    double en = 0.5 * ME * g * g * m.vn * m.vn;
    en = fabs(en - E_EXC_TH * EV);
    g = sqrt(2.0 * en / ME);
    g = g / m.vn;
    chi = acos(1.0 - 2.0 * src.next());
    eta = 2 * PI_REF * src.next();
  } else {
    kind = 3;
    double en = 0.5 * ME * g * g * m.vn * m.vn;
    en = fabs(en - E_ION_TH * EV);
    double e_ej = 10.0 * tan(src.next() * atan(en / EV / 20.0)) * EV;
    double e_sc = fabs(en - e_ej);
    g = sqrt(2.0 * e_sc / ME);
    double g2 = sqrt(2.0 * e_ej / ME);
    g = g / m.vn;
    g2 = g2 / m.vn;
    chi = acos(sqrt(e_sc / en));
    double chi2 = acos(sqrt(e_ej / en));
    eta = 2 * PI_REF * src.next();
    double eta2 = eta + PI_REF;
    double sc = sin(chi2), cc = cos(chi2), se = sin(eta2), ce = cos(eta2);
    double hx = g2 * (ct * cc - st * sc * ce);
    double hy = g2 * (st * cp * cc + ct * cp * sc * ce - sp * sc * se);
    double hz = g2 * (st * sp * cc + ct * sp * sc * ce + cp * sc * se);
    pe[0] = (wx + m.F2 * hx);
    pe[1] = (wy + m.F2 * hy);
    pe[2] = (wz + m.F2 * hz);
    // The reference builds Particle(x, y, SampleVel, SampleVel, SampleVel)
    // and GCC evaluates those arguments right to left: vz draws first.  The
    // ion keeps its velocity in m/s (not divided by vel_norm), as there.
    pi[2] = sample_vel(src, m.ion_mass, m.ion_temp);
    pi[1] = sample_vel(src, m.ion_mass, m.ion_temp);
    pi[0] = sample_vel(src, m.ion_mass, m.ion_temp);
    evt.x = e.x[q];
    evt.y = e.y[q];
  }
  double sc = sin(chi), cc = cos(chi), se = sin(eta), ce = cos(eta);
  gx = g * (ct * cc - st * sc * ce);
  gy = g * (st * cp * cc + ct * cp * sc * ce - sp * sc * se);
  gz = g * (st * sp * cc + ct * sp * sc * ce + cp * sc * se);
  e.vx[q] = wx + m.F2 * gx;
  e.vy[q] = wy + m.F2 * gy;
  e.vz[q] = wz + m.F2 * gz;
  return kind;
}

// Pass 1a: every electron draws u0 (no ordering, fixed grid); the few below
// the cut are appended, in any order, to a candidate list.  Compacting them
// first keeps whole warps on the FP64 collision path instead of one lane in
// 32 (divergent FP64 work costs full warp throughput).
template <int MODE>
__global__ void __launch_bounds__(PART_THREADS) k_mcc_select(MccParams m, const long long* __restrict__ d_ne,
                                                             const double* __restrict__ uniforms, int ustride,
                                                             uint64_t seed, const unsigned long long* __restrict__ d_step,
                                                             McEvents ev) {
  const long long ne = *d_ne;
  const unsigned long long step = *d_step;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const int lane = threadIdx.x & 31;
  const long long nround = (ne + stride - 1) / stride;
  for (long long rd = 0; rd < nround; rd++) {
    const long long q = rd * stride + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool cand = false;
    if (q < ne) {
      if (MODE == EPIC_MCC_INJECTED) {
        cand = __ldg(&uniforms[q * ustride]) < m.p_cut;
      } else {
        Philox src{(uint32_t)q, (uint32_t)(q >> 32), (uint32_t)step, (uint32_t)seed, (uint32_t)(seed >> 32), 0,
                   make_uint4(0, 0, 0, 0)};
        cand = src.next53() < m.cut53;
      }
    }
    const unsigned int mask = __ballot_sync(0xffffffffu, cand);
    if (mask) {
      unsigned int base = 0;
      if (lane == __ffs(mask) - 1) base = atomicAdd(ev.cand_count, (unsigned int)__popc(mask));
      base = __shfl_sync(0xffffffffu, base, __ffs(mask) - 1);
      if (cand) ev.cand[base + __popc(mask & ((1u << lane) - 1))] = (unsigned int)q;
    }
  }
}

// Pass 1b: the candidates, whole warps at a time.  Each redraws u0 from the
// same stream position and runs the collision; an ionisation stores its
// products in the event buffer and marks the electron (slot) and its tile of
// MCC_TILE electrons (tile_cnt).
template <int MODE>
__global__ void __launch_bounds__(PART_THREADS) k_mcc_collide(CrossSections cs, MccParams m, SoA e,
                                                              const double* __restrict__ uniforms, int ustride,
                                                              uint64_t seed,
                                                              const unsigned long long* __restrict__ d_step,
                                                              McEvents ev, unsigned long long* pending, int* flags) {
  __shared__ unsigned long long s_coll;
  if (threadIdx.x == 0) s_coll = 0;
  __syncthreads();
  const unsigned int nc = *ev.cand_count;
  const unsigned long long step = *d_step;
  unsigned int ncoll = 0;
  for (unsigned int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
    const long long q = ev.cand[c];
    IonEvent evt;
    int kind;
    if (MODE == EPIC_MCC_INJECTED) {
      Injected src{uniforms + q * ustride};
      double u0 = src.next();
      kind = mcc_collide(cs, m, e, q, src, u0, evt);
    } else {
      Philox src{(uint32_t)q, (uint32_t)(q >> 32), (uint32_t)step, (uint32_t)seed, (uint32_t)(seed >> 32), 0,
                 make_uint4(0, 0, 0, 0)};
      unsigned long long M = src.next53();
      kind = mcc_collide(cs, m, e, q, src, (double)M * (1.0 / 9007199254740992.0), evt);
    }
    ncoll += kind != 0;
    if (kind == 3) {
      unsigned int slot = atomicAdd(ev.count, 1u);
      if (slot < ev.cap) {
        ev.buf[slot] = evt;
        ev.slot[q] = (int)slot;
        atomicAdd(&ev.tile_cnt[q / MCC_TILE], 1u);
      } else {
        set_flag(flags, FLAG_CAPACITY);
      }
    }
  }
  if (ncoll) atomicAdd(&s_coll, (unsigned long long)ncoll);
  __syncthreads();
  if (threadIdx.x == 0 && s_coll) atomicAdd(&pending[1], s_coll);
}

// Pass 2 (one block): exclusive scan of the per-tile event counts.
__global__ void __launch_bounds__(1024) k_mcc_scan(const long long* __restrict__ d_ne, McEvents ev,
                                                   unsigned long long* pending) {
  __shared__ unsigned int warp_tot[32];
  __shared__ unsigned int carry;
  const long long ne = *d_ne;
  const int tiles = (int)((ne + MCC_TILE - 1) / MCC_TILE);
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < tiles; base += blockDim.x) {
    const int t = base + threadIdx.x;
    unsigned int v = t < tiles ? ev.tile_cnt[t] : 0u, x = v;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
      unsigned int y = warp_tot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        unsigned int z = __shfl_up_sync(0xffffffffu, y, o);
        if (lane >= o) y += z;
      }
      warp_tot[lane] = y;
    }
    __syncthreads();
    const unsigned int excl = carry + (w ? warp_tot[w - 1] : 0u) + x - v;
    if (t < tiles) ev.tile_off[t] = excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) pending[0] = carry;
}

// Pass 3: tiles that had events append their products in electron order at
// [n_e + tile offset + rank] / [n_i + ...] (the reference appends in loop
// order, src/collision.cpp:163-164), then clear their marks.
__global__ void __launch_bounds__(PART_THREADS) k_mcc_append(SoA e, const long long* __restrict__ d_ne,
                                                             long long e_cap, SoA ion,
                                                             const long long* __restrict__ d_ni, long long i_cap,
                                                             McEvents ev, int* flags) {
  constexpr int ITEMS = MCC_TILE / PART_THREADS;
  __shared__ int sm[40];
  const long long ne = *d_ne, ni = *d_ni;
  const int tiles = (int)((ne + MCC_TILE - 1) / MCC_TILE);
  for (int t = blockIdx.x; t < tiles; t += gridDim.x) {
    if (ev.tile_cnt[t] == 0) continue;  // block-uniform
    const long long base = (long long)t * MCC_TILE;
    int slot[ITEMS], flag[ITEMS];
#pragma unroll
    for (int k = 0; k < ITEMS; k++) {
      const long long q = base + k * PART_THREADS + threadIdx.x;
      slot[k] = q < ne ? ev.slot[q] : -1;
      flag[k] = slot[k] >= 0;
    }
    int run = 0;
#pragma unroll
    for (int k = 0; k < ITEMS; k++) {
      int row_total;
      const int rank = run + block_exclusive_scan(flag[k], &row_total, sm);
      run += row_total;
      if (flag[k]) {
        const IonEvent v = ev.buf[slot[k]];
        const long long oe = ne + ev.tile_off[t] + rank, oi = ni + ev.tile_off[t] + rank;
        if (oe < e_cap && oi < i_cap) {
          e.x[oe] = v.x; e.y[oe] = v.y; e.vx[oe] = v.ev[0]; e.vy[oe] = v.ev[1]; e.vz[oe] = v.ev[2];
          ion.x[oi] = v.x; ion.y[oi] = v.y; ion.vx[oi] = v.iv[0]; ion.vy[oi] = v.iv[1]; ion.vz[oi] = v.iv[2];
        } else {
          set_flag(flags, FLAG_CAPACITY);
        }
        ev.slot[base + k * PART_THREADS + threadIdx.x] = -1;
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) ev.tile_cnt[t] = 0;
  }
}

__global__ void k_mcc_commit(long long* d_ne, long long e_cap, long long* d_ni, long long i_cap,
                             unsigned long long* pending, unsigned long long* ncoll_out,
                             unsigned long long* d_step, McEvents ev, int* flags) {
  long long add = (long long)pending[0];
  long long ne = *d_ne + add, ni = *d_ni + add;
  if (ne > e_cap || ni > i_cap) {
    set_flag(flags, FLAG_CAPACITY);
    ne = ne > e_cap ? e_cap : ne;
    ni = ni > i_cap ? i_cap : ni;
  }
  *d_ne = ne;
  *d_ni = ni;
  *ncoll_out = pending[1];
  pending[0] = 0;
  pending[1] = 0;
  *ev.count = 0;
  *ev.cand_count = 0;
  *d_step += 1;
}

size_t ion_event_bytes() { return sizeof(IonEvent); }

void launch_mcc(cudaStream_t st, int mode, const CrossSections& cs, const SoA& e, long long* d_ne, long long e_cap,
                const SoA& ion, long long* d_ni, long long i_cap, double vel_norm, double dt_phys, double ion_mass,
                double ion_temp, const double* uniforms, int ustride, uint64_t seed, unsigned long long* d_step,
                const McEvents& ev, unsigned long long* d_ncoll, int* flags, int grid) {
  MccParams m;
  m.vn = vel_norm;
  m.dt_phys = dt_phys;
  m.ion_mass = ion_mass;
  m.ion_temp = ion_temp;
  m.F1 = ME / (ME + ion_mass);
  m.F2 = ion_mass / (ME + ion_mass);
  m.null_collision = mode == EPIC_MCC_NULL;
  const double p_null = 1 - exp(-cs.nu_max * dt_phys);
  m.p_cut = m.null_collision ? p_null : fmin(1.0, p_null * (1 + 1e-9) + 1e-300);
  m.cut53 = (unsigned long long)ceil(m.p_cut * 9007199254740992.0);
  unsigned long long* pending = d_ncoll + 1;
  if (mode == EPIC_MCC_INJECTED) {
    k_mcc_select<EPIC_MCC_INJECTED><<<grid, PART_THREADS, 0, st>>>(m, d_ne, uniforms, ustride, seed, d_step, ev);
    k_mcc_collide<EPIC_MCC_INJECTED><<<grid, PART_THREADS, 0, st>>>(cs, m, e, uniforms, ustride, seed, d_step, ev,
                                                                     pending, flags);
  } else {
    k_mcc_select<EPIC_MCC_PHILOX><<<grid, PART_THREADS, 0, st>>>(m, d_ne, uniforms, ustride, seed, d_step, ev);
    k_mcc_collide<EPIC_MCC_PHILOX><<<grid, PART_THREADS, 0, st>>>(cs, m, e, uniforms, ustride, seed, d_step, ev,
                                                                   pending, flags);
  }
  k_mcc_scan<<<1, 1024, 0, st>>>(d_ne, ev, pending);
  k_mcc_append<<<grid, PART_THREADS, 0, st>>>(e, d_ne, e_cap, ion, d_ni, i_cap, ev, flags);
  k_mcc_commit<<<1, 1, 0, st>>>(d_ne, e_cap, d_ni, i_cap, pending, d_ncoll, d_step, ev, flags);
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

}  // namespace epic
