// Particle kernels of the mixed-precision form.
//
// Record: cell (int32 node index i*ny + j of the cell's lower-left node),
// ox, oy (FP32 offsets inside the cell, [0, 1)), vx, vy, vz (FP32) — 24 bytes.
// The push reads and writes 20 of them (40 B per particle-step); the deposit
// reads 12; everything runs on the FP32 and integer pipes.  Offsets keep a
// uniform 2^-24-cell resolution over the whole domain, where FP32 absolute
// positions would lose precision with distance from the origin.
//
// Compiled with contraction (FMA) enabled: this form is checked against the
// FP64 oracle within stated tolerances, not bit for bit.
#include <cuda_runtime.h>

#include "epic_device.cuh"
#include "epic_internal.cuh"
#include "epic_mixed.cuh"

namespace epic {

// ------------------------------------------------------------ layout ---
// Upload: FP64 records {x, y, vx, vy, vz} -> mixed.  Species::AddParticle's
// positions become (cell, offset); a particle outside the grid raises
// FLAG_OUT_OF_GRID (the reference would throw at its first deposit).
__global__ void k_aos_to_mixed(Geom g, const double* __restrict__ aos, MixedSoA p, long long n, int* flags) {
  bool bad = false;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const double* r = aos + 5 * q;
    int i, j;
    float ox, oy;
    const bool in_x = cell_offset((r[0] - g.x0) / g.dx, g.nx - 1, i, ox);
    const bool in_y = cell_offset((r[1] - g.y0) / g.dy, g.ny - 1, j, oy);
    bad |= !(in_x && in_y);
    p.cell[q] = i * g.ny + j;
    p.ox[q] = ox;
    p.oy[q] = oy;
    p.vx[q] = (float)r[2];
    p.vy[q] = (float)r[3];
    p.vz[q] = (float)r[4];
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) set_flag(flags, FLAG_OUT_OF_GRID);
}

__global__ void k_mixed_to_aos(Geom g, double* __restrict__ aos, MixedSoA p, const long long* __restrict__ d_n) {
  const long long n = *d_n;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const int c = p.cell[q];
    const int i = c / g.ny, j = c - i * g.ny;
    double* r = aos + 5 * q;
    // explicit roundings (no contraction): the batch's extraction computes the same
    r[0] = __dadd_rn(g.x0, __dmul_rn(__dadd_rn((double)i, (double)p.ox[q]), g.dx));
    r[1] = __dadd_rn(g.y0, __dmul_rn(__dadd_rn((double)j, (double)p.oy[q]), g.dy));
    r[2] = p.vx[q];
    r[3] = p.vy[q];
    r[4] = p.vz[q];
  }
}

void launch_aos_to_mixed(cudaStream_t st, const Geom& g, const double* aos, const MixedSoA& p, long long n,
                         int* flags, int grid) {
  k_aos_to_mixed<<<grid, PART_THREADS, 0, st>>>(g, aos, p, n, flags);
}

void launch_mixed_to_aos(cudaStream_t st, const Geom& g, double* aos, const MixedSoA& p, const long long* d_n,
                         int grid) {
  k_mixed_to_aos<<<grid, PART_THREADS, 0, st>>>(g, aos, p, d_n);
}

// ----------------------------------------------------------- deposit ---
// CIC / NGP deposit with integer weights (Domain::Scatter, src/domain.cpp:
// 205-228): the offsets are quantised to 2^-20 of a cell and the four CIC
// weights are exact integer products summing to 2^40, accumulated in int64
// (deterministic: integer addition is associative).  No node can overflow
// unless more than 2^23 particles share its four cells.  The finalisation
// multiplies by spwt * 2^-40.
template <int SHAPE>
__global__ void __launch_bounds__(PART_THREADS) k_deposit_mixed(Geom g, MixedSoA p, const long long* __restrict__ d_n,
                                                                unsigned long long* __restrict__ acc) {
  const long long n = *d_n;
  const long long S = 1ll << MIXED_OFFSET_BITS;
  const float fS = (float)S;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const int c = __ldg(&p.cell[q]);
    const float ox = __ldg(&p.ox[q]), oy = __ldg(&p.oy[q]);
    if (SHAPE == EPIC_NGP) {
      // round(lx) with lx = i + ox >= 0: i + (ox >= 0.5)
      const int k = c + (ox >= 0.5f ? g.ny : 0) + (oy >= 0.5f ? 1 : 0);
      atomicAdd(&acc[k], (unsigned long long)(S * S));
    } else {
      const long long a = (long long)(ox * fS), b = (long long)(oy * fS);  // truncation, in [0, 2^20)
      atomicAdd(&acc[c], (unsigned long long)((S - a) * (S - b)));
      atomicAdd(&acc[c + g.ny], (unsigned long long)(a * (S - b)));
      atomicAdd(&acc[c + 1], (unsigned long long)((S - a) * b));
      atomicAdd(&acc[c + g.ny + 1], (unsigned long long)(a * b));
    }
  }
}

void launch_deposit_mixed(cudaStream_t st, const Geom& g, int shape, const MixedSoA& p, const long long* d_n,
                          unsigned long long* acc, int* flags, int grid) {
  (void)flags;
  if (shape == EPIC_NGP) k_deposit_mixed<EPIC_NGP><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, acc);
  else k_deposit_mixed<EPIC_CIC><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, acc);
}

// CIC deposit of the particles [*d_from, *d_n) (the MCC's ionisation
// products, appended after the push deposited the rest).
__global__ void __launch_bounds__(PART_THREADS) k_deposit_mixed_range(Geom g, MixedSoA p,
                                                                      const long long* __restrict__ d_from,
                                                                      const long long* __restrict__ d_n,
                                                                      unsigned long long* __restrict__ acc) {
  const long long from = *d_from, n = *d_n;
  const long long S = 1ll << MIXED_OFFSET_BITS;
  const float fS = (float)S;
  for (long long q = from + (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int c = p.cell[q];
    const long long a = (long long)(p.ox[q] * fS), b = (long long)(p.oy[q] * fS);
    atomicAdd(&acc[c], (unsigned long long)((S - a) * (S - b)));
    atomicAdd(&acc[c + g.ny], (unsigned long long)(a * (S - b)));
    atomicAdd(&acc[c + 1], (unsigned long long)((S - a) * b));
    atomicAdd(&acc[c + g.ny + 1], (unsigned long long)(a * b));
  }
}

void launch_deposit_mixed_range(cudaStream_t st, const Geom& g, const MixedSoA& p, const long long* d_from,
                                const long long* d_n, unsigned long long* acc, int grid) {
  k_deposit_mixed_range<<<grid, PART_THREADS, 0, st>>>(g, p, d_from, d_n, acc);
}

// -------------------------------------------------------------- push ---
// gather32 / advance / push_mixed_one: epic_mixed.cuh (shared with the batch).
template <int SHAPE, int BC>
__global__ void __launch_bounds__(PART_THREADS) k_push_mixed(Geom g, MixedSoA p, const long long* __restrict__ d_n,
                                                             const float2* __restrict__ ef, float qmK_dt, float cx,
                                                             float cy) {
  const long long n = *d_n;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    int c = p.cell[q];
    float ox = p.ox[q], oy = p.oy[q], vx = p.vx[q], vy = p.vy[q];
    push_mixed_one<SHAPE, BC>(g, ef, qmK_dt, cx, cy, c, ox, oy, vx, vy);
    p.cell[q] = c;
    p.ox[q] = ox;
    p.oy[q] = oy;
    p.vx[q] = vx;
    p.vy[q] = vy;
  }
}

// Periodic or reflective walls, CIC: the push, the deposit of the new
// positions into acc (deposit_warp_sorted) and, with SEL, the MCC's first
// pass over the pushed electrons (mcc_candidate on the new velocities,
// CTA-aggregated appends to sel.cand) in one pass over the particles.  Each
// thread takes DEP_PER_THREAD consecutive particles with vector loads and
// stores.  The particles, the integer sums and the candidate set (in another
// order, which the MCC does not depend on) equal those of k_push_mixed +
// k_deposit_mixed_sorted + k_mcc_select.
template <int BC, bool SEL>
__global__ void __launch_bounds__(PART_THREADS, 3) k_push_mixed_dep(Geom g, MixedSoA p, const long long* __restrict__ d_n,
                                                                 const float2* __restrict__ ef, float qmK_dt,
                                                                 float cx, float cy, unsigned long long* __restrict__ acc,
                                                                 SelectArgs sel) {
  constexpr int P = DEP_PER_THREAD;
  __shared__ DepWarp tables[PART_THREADS / 32];
  DepWarp& w = tables[threadIdx.x >> 5];
  const long long n = *d_n;
  const unsigned long long step = SEL ? *sel.d_step : 0ull;
  const int lane = threadIdx.x & 31;
  dep_init(w);
  for (long long chunk = (long long)blockIdx.x * DEP_CHUNK; chunk < n; chunk += (long long)gridDim.x * DEP_CHUNK) {
    const long long q0 = chunk + (long long)threadIdx.x * P;
    const bool full = q0 + P <= n;
    int c[P];
    float ox[P], oy[P], vx[P], vy[P], vz[P];
    if (full) {
#pragma unroll
      for (int h = 0; h < P / 4; h++) {
        const int4 cc = reinterpret_cast<const int4*>(p.cell + q0)[h];
        const float4 a = reinterpret_cast<const float4*>(p.ox + q0)[h];
        const float4 b = reinterpret_cast<const float4*>(p.oy + q0)[h];
        const float4 u = reinterpret_cast<const float4*>(p.vx + q0)[h];
        const float4 v = reinterpret_cast<const float4*>(p.vy + q0)[h];
        c[4 * h] = cc.x; c[4 * h + 1] = cc.y; c[4 * h + 2] = cc.z; c[4 * h + 3] = cc.w;
        ox[4 * h] = a.x; ox[4 * h + 1] = a.y; ox[4 * h + 2] = a.z; ox[4 * h + 3] = a.w;
        oy[4 * h] = b.x; oy[4 * h + 1] = b.y; oy[4 * h + 2] = b.z; oy[4 * h + 3] = b.w;
        vx[4 * h] = u.x; vx[4 * h + 1] = u.y; vx[4 * h + 2] = u.z; vx[4 * h + 3] = u.w;
        vy[4 * h] = v.x; vy[4 * h + 1] = v.y; vy[4 * h + 2] = v.z; vy[4 * h + 3] = v.w;
        if (SEL) {
          const float4 w = reinterpret_cast<const float4*>(p.vz + q0)[h];
          vz[4 * h] = w.x; vz[4 * h + 1] = w.y; vz[4 * h + 2] = w.z; vz[4 * h + 3] = w.w;
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < P; k++) {
        const long long q = q0 + k;
        const bool in = q < n;
        c[k] = in ? p.cell[q] : -1;
        ox[k] = in ? p.ox[q] : 0.f;
        oy[k] = in ? p.oy[q] : 0.f;
        vx[k] = in ? p.vx[q] : 0.f;
        vy[k] = in ? p.vy[q] : 0.f;
        vz[k] = (SEL && in) ? p.vz[q] : 0.f;
      }
    }
    unsigned int cand = 0;
#pragma unroll
    for (int k = 0; k < P; k++)
      if (c[k] >= 0) {
        push_mixed_one<EPIC_CIC, BC>(g, ef, qmK_dt, cx, cy, c[k], ox[k], oy[k], vx[k], vy[k]);
        if (SEL && mcc_candidate(sel, q0 + k, step, vx[k], vy[k], vz[k])) cand |= 1u << k;
      }
    if (full) {
#pragma unroll
      for (int h = 0; h < P / 4; h++) {
        reinterpret_cast<int4*>(p.cell + q0)[h] = make_int4(c[4 * h], c[4 * h + 1], c[4 * h + 2], c[4 * h + 3]);
        reinterpret_cast<float4*>(p.ox + q0)[h] = make_float4(ox[4 * h], ox[4 * h + 1], ox[4 * h + 2], ox[4 * h + 3]);
        reinterpret_cast<float4*>(p.oy + q0)[h] = make_float4(oy[4 * h], oy[4 * h + 1], oy[4 * h + 2], oy[4 * h + 3]);
        reinterpret_cast<float4*>(p.vx + q0)[h] = make_float4(vx[4 * h], vx[4 * h + 1], vx[4 * h + 2], vx[4 * h + 3]);
        reinterpret_cast<float4*>(p.vy + q0)[h] = make_float4(vy[4 * h], vy[4 * h + 1], vy[4 * h + 2], vy[4 * h + 3]);
      }
    } else {
#pragma unroll
      for (int k = 0; k < P; k++)
        if (c[k] >= 0) {
          const long long q = q0 + k;
          p.cell[q] = c[k];
          p.ox[q] = ox[k];
          p.oy[q] = oy[k];
          p.vx[q] = vx[k];
          p.vy[q] = vy[k];
        }
    }
    if (SEL && __any_sync(0xffffffffu, cand != 0)) {  // one atomic per warp with candidates
      const unsigned int mine = __popc(cand);
      unsigned int incl = mine;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      unsigned int base = 0;
      if (lane == 31) base = atomicAdd(sel.cand_count, incl);
      unsigned int o = __shfl_sync(0xffffffffu, base, 31) + incl - mine;
#pragma unroll
      for (int k = 0; k < P; k++)
        if (cand & (1u << k)) sel.cand[o++] = (unsigned int)(q0 + k);
    }
    deposit_warp_sorted(acc, w, ConstNy{g.ny}, c, ox, oy);
  }
}

// Open boundaries or conductors: push + stable in-place compaction with
// ordered tiles (the FP64 form's scheme; see k_push_compact in
// epic_particles.cu).  COND: a particle that ends inside a conductor, its
// position taken as x0 + (i + ox) dx in FP64, is erased too
// (src/species.cpp:80-165).
template <int SHAPE, int BC, bool COND>
__global__ void __launch_bounds__(PART_THREADS) k_push_mixed_compact(Geom g, MixedSoA p, long long* d_n,
                                                                     const float2* __restrict__ ef, float qmK_dt,
                                                                     float cx, float cy, unsigned long long* status,
                                                                     unsigned int* tile_ctr, int* flags,
                                                                     long long spin, CondSet cs) {
  constexpr int ITEMS = SCAN_TILE / PART_THREADS;
  __shared__ int sm[40];
  __shared__ unsigned long long s_prefix;
  __shared__ int s_tile;
  const long long n = *d_n;
  const int num_tiles = (int)((n + SCAN_TILE - 1) / SCAN_TILE);
  for (;;) {
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(tile_ctr, 1u);
    __syncthreads();
    const int tile = s_tile;
    if (tile >= num_tiles) break;
    const long long base = (long long)tile * SCAN_TILE;
    int c[ITEMS], keep[ITEMS];
    float ox[ITEMS], oy[ITEMS], vx[ITEMS], vy[ITEMS], vz[ITEMS];
#pragma unroll
    for (int k = 0; k < ITEMS; k++) {
      const long long q = base + (long long)k * PART_THREADS + threadIdx.x;
      keep[k] = 0;
      if (q < n) {
        c[k] = p.cell[q]; ox[k] = p.ox[q]; oy[k] = p.oy[q]; vx[k] = p.vx[q]; vy[k] = p.vy[q]; vz[k] = p.vz[q];
        keep[k] = push_mixed_one<SHAPE, BC>(g, ef, qmK_dt, cx, cy, c[k], ox[k], oy[k], vx[k], vy[k]);
        if (COND && keep[k]) {
          int i, j;
          split_cell(c[k], g.ny, i, j);
          const double x = __dadd_rn(g.x0, __dmul_rn(__dadd_rn((double)i, (double)ox[k]), g.dx));
          const double y = __dadd_rn(g.y0, __dmul_rn(__dadd_rn((double)j, (double)oy[k]), g.dy));
          keep[k] = !in_conductor(cs, x, y);
        }
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
          const long long o = (long long)prefix + rank[k];
          p.cell[o] = c[k]; p.ox[o] = ox[k]; p.oy[o] = oy[k]; p.vx[o] = vx[k]; p.vy[o] = vy[k]; p.vz[o] = vz[k];
        }
      }
      if (tile == num_tiles - 1 && threadIdx.x == 0) *d_n = (long long)prefix + tile_total;
    }
    __syncthreads();
  }
}

void launch_push_mixed(cudaStream_t st, const Geom& g, int shape, int bc, const MixedSoA& p, long long* d_n,
                       const float2* ef, float qmK_dt, float cx, float cy, int* flags,
                       unsigned long long* tile_status, unsigned int* tile_ctr, int grid,
                       unsigned long long* dep_acc, const SelectArgs* sel, const CondSet* cond) {
  if (cond) {  // the compacting push with the conductor test, for any wall rule
#define PC(SH, B) \
  k_push_mixed_compact<SH, B, true><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, ef, qmK_dt, cx, cy, tile_status, tile_ctr, \
                                                                   flags, spin_limit(), *cond)
#define PCB(SH)                          \
  do {                                   \
    if (bc == EPIC_OPEN) PC(SH, EPIC_OPEN); \
    else if (bc == EPIC_PBC) PC(SH, EPIC_PBC); \
    else PC(SH, EPIC_REFLECTIVE);        \
  } while (0)
    if (shape == EPIC_NGP) PCB(EPIC_NGP);
    else PCB(EPIC_CIC);
#undef PCB
#undef PC
    return;
  }
#define PM(SH, B) k_push_mixed<SH, B><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, ef, qmK_dt, cx, cy)
  if (dep_acc && shape == EPIC_CIC && (bc == EPIC_PBC || bc == EPIC_REFLECTIVE)) {
    const SelectArgs a = sel ? *sel : SelectArgs{};
    // one wave of resident CTAs (the kernel strides over the chunks)
#define PD(B, S)                                                                                       \
  k_push_mixed_dep<B, S><<<resident_grid(k_push_mixed_dep<B, S>, PART_THREADS), PART_THREADS, 0, st>>>( \
      g, p, d_n, ef, qmK_dt, cx, cy, dep_acc, a)
    if (bc == EPIC_PBC) { if (sel) PD(EPIC_PBC, true); else PD(EPIC_PBC, false); }
    else { if (sel) PD(EPIC_REFLECTIVE, true); else PD(EPIC_REFLECTIVE, false); }
#undef PD
    return;
  }
  if (bc == EPIC_OPEN) {
    if (shape == EPIC_NGP)
      k_push_mixed_compact<EPIC_NGP, EPIC_OPEN, false><<<grid, PART_THREADS, 0, st>>>(
          g, p, d_n, ef, qmK_dt, cx, cy, tile_status, tile_ctr, flags, spin_limit(), CondSet{});
    else
      k_push_mixed_compact<EPIC_CIC, EPIC_OPEN, false><<<grid, PART_THREADS, 0, st>>>(
          g, p, d_n, ef, qmK_dt, cx, cy, tile_status, tile_ctr, flags, spin_limit(), CondSet{});
  } else if (bc == EPIC_PBC) {
    if (shape == EPIC_NGP) PM(EPIC_NGP, EPIC_PBC);
    else PM(EPIC_CIC, EPIC_PBC);
  } else {
    if (shape == EPIC_NGP) PM(EPIC_NGP, EPIC_REFLECTIVE);
    else PM(EPIC_CIC, EPIC_REFLECTIVE);
  }
#undef PM
}

// Species::Rewind_species (src/species.cpp:229-246): v -= (0.5*qm*K*DT) E.
template <int SHAPE>
__global__ void __launch_bounds__(PART_THREADS) k_rewind_mixed(Geom g, MixedSoA p, const long long* __restrict__ d_n,
                                                               const float2* __restrict__ ef, float hqmK_dt) {
  const long long n = *d_n;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    float ex, ey;
    gather32<SHAPE>(g, ef, p.cell[q], p.ox[q], p.oy[q], ex, ey);
    p.vx[q] = fmaf(-hqmK_dt, ex, p.vx[q]);
    p.vy[q] = fmaf(-hqmK_dt, ey, p.vy[q]);
  }
}

void launch_rewind_mixed(cudaStream_t st, const Geom& g, int shape, const MixedSoA& p, const long long* d_n,
                         const float2* ef, float hqmK_dt, int* flags, int grid) {
  (void)flags;
  if (shape == EPIC_NGP) k_rewind_mixed<EPIC_NGP><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, ef, hqmK_dt);
  else k_rewind_mixed<EPIC_CIC><<<grid, PART_THREADS, 0, st>>>(g, p, d_n, ef, hqmK_dt);
}

// ------------------------------------------------------- reductions ---
// Energy / momentum sums accumulated in FP64 from the FP32 velocities
// (Species::Compute_KE / Compute_Momentum, src/species.cpp:248-297).
__device__ __forceinline__ double warp_sum_m(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(PART_THREADS) k_particle_sums_mixed(int what, MixedSoA p,
                                                                      const long long* __restrict__ d_n, double vn,
                                                                      double* partials) {
  const long long n = *d_n;
  double s0 = 0, s1 = 0, s2 = 0;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const double a = p.vx[q], b = p.vy[q], c = p.vz[q];
    if (what == 0) {
      s0 += (a * a) * vn * vn;
      s1 += (b * b) * vn * vn;
      s2 += (c * c) * vn * vn;
    } else {
      s0 += a * vn;
      s1 += b * vn;
      s2 += c * vn;
    }
  }
  __shared__ double sm[3][PART_THREADS / 32];
  s0 = warp_sum_m(s0);
  s1 = warp_sum_m(s1);
  s2 = warp_sum_m(s2);
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

__global__ void k_sum_partials3_m(const double* partials, int nblocks, double* out) {
  const int c = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (c >= 3) return;
  double t = 0;
  for (int b = lane; b < nblocks; b += 32) t += partials[b * 3 + c];
  t = warp_sum_m(t);
  if (lane == 0) out[c] = t;
}

void launch_particle_sums_mixed(cudaStream_t st, int what, const MixedSoA& p, const long long* d_n, double vel_norm,
                                double* partials, double* out3, int grid) {
  k_particle_sums_mixed<<<grid, PART_THREADS, 0, st>>>(what, p, d_n, vel_norm, partials);
  k_sum_partials3_m<<<1, 96, 0, st>>>(partials, grid, out3);
}

}  // namespace epic
