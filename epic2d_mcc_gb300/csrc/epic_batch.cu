// A batch of independent runs advanced together (include/epic2d_batch.h):
// the particle kernels, the spectral solve and the loader of the batch, and
// the host side that lays the runs out, tunes the GEMM tiles and captures a
// step.  Compiled like epic_mixed.cu / epic_spectral.cu (FP32 contraction
// allowed), whose per-particle and per-lattice code it calls, so a run rounds
// as it does alone.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/epic2d_batch.h"
#include "epic_batch.cuh"
#include "epic_device.cuh"
#include "epic_emit.cuh"
#include "epic_host.h"
#include "epic_mixed.cuh"
#include "epic_spectral.cuh"

namespace epic {

constexpr int BATCH_STAGES = 6;  // refinement stages of the spectral solve (as a single run)

// ------------------------------------------------------------ loading ---
// AoS records of one run's species (epic_load.cu's loader) into the batch's
// particle array: the single-run conversion (k_aos_to_mixed) with the cell
// moved to the run's place in the node space.
__global__ void k_batch_from_aos(BRun r, const double* __restrict__ aos, MixedSoA p, long long base, long long n,
                                 int* flags) {
  bool bad = false;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const double* a = aos + 5 * q;
    int i, j;
    float ox, oy;
    const bool in_x = cell_offset((a[0] - r.x0) / r.dx, r.nx - 1, i, ox);
    const bool in_y = cell_offset((a[1] - r.y0) / r.dy, r.ny - 1, j, oy);
    bad |= !(in_x && in_y);
    const long long o = base + q;
    p.cell[o] = (int)(r.node_off + i * r.ny + j);
    p.ox[o] = ox;
    p.oy[o] = oy;
    p.vx[o] = (float)a[2];
    p.vy[o] = (float)a[3];
    p.vz[o] = (float)a[4];
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flags, FLAG_OUT_OF_GRID);
}

// One run's particles of a species as {x, y, vx, vy, vz} (k_mixed_to_aos).
__global__ void k_batch_to_aos(BRun r, double* __restrict__ aos, MixedSoA p, long long base, long long n) {
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const long long o = base + q;
    const int c = (int)(p.cell[o] - r.node_off);
    const int i = c / r.ny, j = c - i * r.ny;
    double* a = aos + 5 * q;
    a[0] = __dadd_rn(r.x0, __dmul_rn(__dadd_rn((double)i, (double)p.ox[o]), r.dx));
    a[1] = __dadd_rn(r.y0, __dmul_rn(__dadd_rn((double)j, (double)p.oy[o]), r.dy));
    a[2] = p.vx[o];
    a[3] = p.vy[o];
    a[4] = p.vz[o];
  }
}

// Particles of one run anywhere in a species' array (after MCC appends a
// run's particles need not be contiguous): per tile of EXTRACT_TILE slots the
// count of the run's particles, then an ordered gather at the scanned offsets.
constexpr int EXTRACT_TILE = 1024;

__global__ void k_batch_count_run(const int* __restrict__ node_run, MixedSoA p, const long long* __restrict__ d_n,
                                  int run, unsigned int* counts) {
  __shared__ unsigned int c;
  const long long n = *d_n;
  const long long base = (long long)blockIdx.x * EXTRACT_TILE;
  if (threadIdx.x == 0) c = 0;
  __syncthreads();
  unsigned int mine = 0;
  for (int k = threadIdx.x; k < EXTRACT_TILE; k += blockDim.x) {
    const long long q = base + k;
    mine += q < n && node_run[p.cell[q]] == run;
  }
  atomicAdd(&c, mine);
  __syncthreads();
  if (threadIdx.x == 0) counts[blockIdx.x] = c;
}

__global__ void __launch_bounds__(256) k_batch_gather_run(BRun r, int run, const int* __restrict__ node_run, MixedSoA p,
                                                          const long long* __restrict__ d_n,
                                                          const unsigned int* __restrict__ offsets, double* aos) {
  __shared__ int sm[40];
  const long long n = *d_n;
  const long long base = (long long)blockIdx.x * EXTRACT_TILE;
  int rank0 = 0;
  for (int k0 = 0; k0 < EXTRACT_TILE; k0 += 256) {
    const long long o = base + k0 + threadIdx.x;
    const int flag = o < n && node_run[p.cell[o]] == run;
    int total;
    const int rank = rank0 + block_exclusive_scan(flag, &total, sm);
    rank0 += total;
    if (flag) {
      const int c = (int)(p.cell[o] - r.node_off);
      const int i = c / r.ny, j = c - i * r.ny;
      double* a = aos + 5 * ((long long)offsets[blockIdx.x] + rank);
      a[0] = __dadd_rn(r.x0, __dmul_rn(__dadd_rn((double)i, (double)p.ox[o]), r.dx));
      a[1] = __dadd_rn(r.y0, __dmul_rn(__dadd_rn((double)j, (double)p.oy[o]), r.dy));
      a[2] = p.vx[o];
      a[3] = p.vy[o];
      a[4] = p.vz[o];
    }
  }
}

// ---------------------------------------------------------- particles ---
__device__ __forceinline__ Geom run_geom(const BRun& r) {
  Geom g;
  g.nx = r.nx;
  g.ny = r.ny;
  g.x0 = r.x0;
  g.y0 = r.y0;
  g.dx = r.dx;
  g.dy = r.dy;
  g.Lx = g.Ly = 0;
  return g;
}

// The single-run push (push_mixed_one) of every particle of a species, each
// with its run's grid, field and constants.
__global__ void __launch_bounds__(PART_THREADS) k_batch_push(const BRun* __restrict__ runs,
                                                             const int* __restrict__ node_run, MixedSoA p,
                                                             const long long* __restrict__ d_n,
                                                             const float2* __restrict__ ef32, int s) {
  const long long n = *d_n;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const int cg = p.cell[q];
    const BRun& r = runs[node_run[cg]];
    const Geom g = run_geom(r);
    const float2* ef = ef32 + r.node_off;
    int c = (int)(cg - r.node_off);
    float ox = p.ox[q], oy = p.oy[q], vx = p.vx[q], vy = p.vy[q];
    if (r.bc == EPIC_PBC) push_mixed_one<EPIC_CIC, EPIC_PBC>(g, ef, r.qmK_dt[s], r.cx, r.cy, c, ox, oy, vx, vy);
    else push_mixed_one<EPIC_CIC, EPIC_REFLECTIVE>(g, ef, r.qmK_dt[s], r.cx, r.cy, c, ox, oy, vx, vy);
    p.cell[q] = (int)(r.node_off + c);
    p.ox[q] = ox;
    p.oy[q] = oy;
    p.vx[q] = vx;
    p.vy[q] = vy;
  }
}

__global__ void __launch_bounds__(PART_THREADS) k_batch_rewind(const BRun* __restrict__ runs,
                                                               const int* __restrict__ node_run, MixedSoA p,
                                                               const long long* __restrict__ d_n,
                                                               const float2* __restrict__ ef32, int s) {
  const long long n = *d_n;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const int cg = p.cell[q];
    const BRun& r = runs[node_run[cg]];
    float ex, ey;
    gather32<EPIC_CIC>(run_geom(r), ef32 + r.node_off, (int)(cg - r.node_off), p.ox[q], p.oy[q], ex, ey);
    const float h = r.hqmK_dt[s];
    p.vx[q] = fmaf(-h, ex, p.vx[q]);
    p.vy[q] = fmaf(-h, ey, p.vy[q]);
  }
}

// The batch's step push: the single-run push of every particle with its run's
// grid, field and constants, the CIC deposit of the new positions into acc
// (deposit_warp_sorted with each cell's run's row stride) and, with SEL, the
// MCC's first pass of k_batch_mcc_select on the pushed electrons of colliding
// runs (appended to ev.cand, one atomic per warp with candidates).  Particles,
// integer sums and the candidate set equal k_batch_push + k_batch_deposit +
// k_batch_mcc_select.
struct RunNy {
  const BRun* runs;
  const int* node_run;
  __device__ __forceinline__ int operator()(int cg) const { return runs[__ldg(&node_run[cg])].ny; }
};

// T threads per CTA (128 or 256; the autotuner picks the shape), each taking
// DEP_PER_THREAD consecutive particles per round.
template <bool SEL, int T>
__global__ void __launch_bounds__(T, 768 / T) k_batch_push_dep(const BRun* __restrict__ runs,
                                                                    const int* __restrict__ node_run, MixedSoA p,
                                                                    const long long* __restrict__ d_n,
                                                                    const float2* __restrict__ ef32, int s,
                                                                    unsigned long long* __restrict__ acc,
                                                                    const unsigned long long* __restrict__ d_step,
                                                                    McEvents ev) {
  constexpr int P = DEP_PER_THREAD;
  constexpr int CHUNK = T * P;
  __shared__ DepWarp tables[T / 32];
  DepWarp& w = tables[threadIdx.x >> 5];
  const long long n = *d_n;
  const unsigned long long step = SEL ? *d_step : 0ull;
  const int lane = threadIdx.x & 31;
  const RunNy ny_of{runs, node_run};
  dep_init(w);
  for (long long chunk = (long long)blockIdx.x * CHUNK; chunk < n; chunk += (long long)gridDim.x * CHUNK) {
    const long long q0 = chunk + (long long)threadIdx.x * P;
    const bool full = q0 + P <= n;
    int c[P];
    float ox[P], oy[P], vx[P], vy[P];
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
      }
    }
    unsigned int cand = 0;
    // A thread's particles are consecutive in the cell-sorted array, so they
    // nearly always share a run: its parameters are loaded once and kept
    // while the run stays the same.
    int rid = -1, rbc = 0, rmcc = 0;
    long long roff = 0;
    float rqm = 0.f, rcx = 0.f, rcy = 0.f;
    unsigned long long rcut = 0, rseed = 0;
    Geom g;
#pragma unroll
    for (int k = 0; k < P; k++)
      if (c[k] >= 0) {
        const int ri = __ldg(&node_run[c[k]]);
        if (ri != rid) {
          const BRun& r = runs[ri];
          g = run_geom(r);
          roff = r.node_off;
          rbc = r.bc;
          rqm = r.qmK_dt[s];
          rcx = r.cx;
          rcy = r.cy;
          if (SEL) {
            rmcc = r.mcc;
            rcut = r.cut53;
            rseed = r.seed;
          }
          rid = ri;
        }
        const float2* ef = ef32 + roff;
        int cl = (int)(c[k] - roff);
        if (rbc == EPIC_PBC)
          push_mixed_one<EPIC_CIC, EPIC_PBC>(g, ef, rqm, rcx, rcy, cl, ox[k], oy[k], vx[k], vy[k]);
        else
          push_mixed_one<EPIC_CIC, EPIC_REFLECTIVE>(g, ef, rqm, rcx, rcy, cl, ox[k], oy[k], vx[k], vy[k]);
        c[k] = (int)(roff + cl);
        if (SEL && rmcc) {
          const long long q = q0 + k;
          Philox src{(uint32_t)q, (uint32_t)(q >> 32), (uint32_t)step, (uint32_t)rseed, (uint32_t)(rseed >> 32), 0,
                     make_uint4(0, 0, 0, 0)};
          if (src.next53() < rcut) cand |= 1u << k;
        }
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
    if (SEL && __any_sync(0xffffffffu, cand != 0)) {
      const unsigned int mine = __popc(cand);
      unsigned int incl = mine;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const unsigned int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      unsigned int base = 0;
      if (lane == 31) base = atomicAdd(ev.cand_count, incl);
      unsigned int o = __shfl_sync(0xffffffffu, base, 31) + incl - mine;
#pragma unroll
      for (int k = 0; k < P; k++)
        if (cand & (1u << k)) ev.cand[o++] = (unsigned int)(q0 + k);
    }
    deposit_warp_sorted(acc, w, ny_of, c, ox, oy);
  }
}

// The batch's push when some run has absorbing walls or conductors: each
// particle with its run's constants and wall rule; a particle that leaves an
// open run, or ends inside one of its run's conductors (its position taken as
// x0 + (i + ox) dx in FP64, as k_push_mixed_compact<..., COND>), is erased and
// the rest keep their order (std::vector::erase, src/species.cpp:80-165),
// through the single run's ordered tile scan over the whole shared array, so
// every run's particles stay contiguous and in order.
__global__ void __launch_bounds__(PART_THREADS) k_batch_push_compact(const BRun* __restrict__ runs,
                                                                     const int* __restrict__ node_run, MixedSoA p,
                                                                     long long* d_n, const float2* __restrict__ ef32,
                                                                     int s, unsigned long long* status,
                                                                     unsigned int* tile_ctr, int* flags, long long spin,
                                                                     BatchConductors cd) {
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
        const int cg = p.cell[q];
        ox[k] = p.ox[q]; oy[k] = p.oy[q]; vx[k] = p.vx[q]; vy[k] = p.vy[q]; vz[k] = p.vz[q];
        const int run = __ldg(&node_run[cg]);
        const BRun& r = runs[run];
        const Geom g = run_geom(r);
        const float2* ef = ef32 + r.node_off;
        int cl = (int)(cg - r.node_off);
        if (r.bc == EPIC_OPEN)
          keep[k] = push_mixed_one<EPIC_CIC, EPIC_OPEN>(g, ef, r.qmK_dt[s], r.cx, r.cy, cl, ox[k], oy[k], vx[k], vy[k]);
        else if (r.bc == EPIC_PBC)
          keep[k] = push_mixed_one<EPIC_CIC, EPIC_PBC>(g, ef, r.qmK_dt[s], r.cx, r.cy, cl, ox[k], oy[k], vx[k], vy[k]);
        else
          keep[k] = push_mixed_one<EPIC_CIC, EPIC_REFLECTIVE>(g, ef, r.qmK_dt[s], r.cx, r.cy, cl, ox[k], oy[k], vx[k],
                                                              vy[k]);
        if (keep[k] && (r.nrect | r.ncirc)) {
          int i, j;
          split_cell(cl, r.ny, i, j);
          const double x = __dadd_rn(g.x0, __dmul_rn(__dadd_rn((double)i, (double)ox[k]), g.dx));
          const double y = __dadd_rn(g.y0, __dmul_rn(__dadd_rn((double)j, (double)oy[k]), g.dy));
          const CondSet cs{r.nrect, r.ncirc, cd.rect + r.rect_off, cd.circ + r.circ_off, cd.live + run};
          keep[k] = !in_conductor(cs, x, y);
        }
        c[k] = (int)(r.node_off + cl);
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

// Grid::initialize inside gssolver (src/field.cpp:100-103) for every run that
// solves with SOR and has conductors: their voltages into rho at the listed
// nodes of the batch's node space (a run's later conductors win, as the host
// list is built), and the runs' electrodes marked as existing.
__global__ void k_batch_conductor_rho(double* __restrict__ rho, const int* __restrict__ nodes,
                                      const double* __restrict__ vals, int n, const int* __restrict__ live_runs,
                                      int nlive, int* live) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int k = t; k < n; k += stride) rho[nodes[k]] = vals[k];
  for (int k = t; k < nlive; k += stride) live[live_runs[k]] = 1;
}

// Emitter::inject of every run (src/emitter.cpp:5-36) into one species: CTA
// row y is emitter em[y]; its points are emit_point's draws (the run alone
// writes the same), written past the live count in (run, emitter) order, so
// each run's new particles follow its others in its own emitters' order.
__global__ void __launch_bounds__(PART_THREADS) k_batch_emit(const BRun* __restrict__ runs,
                                                             const BEmit* __restrict__ em, MixedSoA p,
                                                             const long long* __restrict__ d_n, long long cap,
                                                             const unsigned long long* __restrict__ d_inj,
                                                             int* flags) {
  const BEmit b = em[blockIdx.y];
  const BRun& r = runs[b.run];
  const long long n0 = *d_n + b.off;
  const unsigned long long inj = *d_inj;
  bool bad = false, over = false;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < b.e.num; q += gridDim.x * blockDim.x) {
    const long long o = n0 + q;
    if (o >= cap) {
      over = true;
      continue;
    }
    double x, y, vx, vy, vz;
    emit_point(b.e, q, b.seed, inj, nullptr, x, y, vx, vy, vz);
    int i, j;
    float ox, oy;
    const bool in_x = cell_offset((x - r.x0) / r.dx, r.nx - 1, i, ox);
    const bool in_y = cell_offset((y - r.y0) / r.dy, r.ny - 1, j, oy);
    bad |= !(in_x && in_y);
    p.cell[o] = (int)(r.node_off + i * r.ny + j);
    p.ox[o] = ox;
    p.oy[o] = oy;
    p.vx[o] = (float)vx;
    p.vy[o] = (float)vy;
    p.vz[o] = (float)vz;
  }
  if (over) atomicOr(flags, FLAG_CAPACITY);
  if (bad) atomicOr(flags, FLAG_OUT_OF_GRID);
}

// Advances a species' count past one step's injections (capped at the
// capacity, which raises EPIC_ERR_CAPACITY) and keeps the old count as the
// start of the range to deposit.
__global__ void k_batch_emit_commit(long long* d_n, long long* d_from, long long total, long long cap, int* flags) {
  const long long n0 = *d_n;
  long long n = n0 + total;
  if (n > cap) {
    atomicOr(flags, FLAG_CAPACITY);
    n = cap;
  }
  *d_from = n0;
  *d_n = n;
}

// CIC deposit of the particles [*d_from, *d_n) of a species (the MCC's
// ionisation products, appended after the push deposited the rest, or an
// injection's particles).
__global__ void __launch_bounds__(PART_THREADS) k_batch_deposit_range(const BRun* __restrict__ runs,
                                                                      const int* __restrict__ node_run, MixedSoA p,
                                                                      const long long* __restrict__ d_from,
                                                                      const long long* __restrict__ d_n,
                                                                      unsigned long long* __restrict__ acc) {
  const long long from = *d_from, n = *d_n;
  const long long S = 1ll << MIXED_OFFSET_BITS;
  const float fS = (float)S;
  for (long long q = from + (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int c = p.cell[q];
    const int ny = runs[node_run[c]].ny;
    const long long a = (long long)(p.ox[q] * fS), b = (long long)(p.oy[q] * fS);
    atomicAdd(&acc[c], (unsigned long long)((S - a) * (S - b)));
    atomicAdd(&acc[c + ny], (unsigned long long)(a * (S - b)));
    atomicAdd(&acc[c + 1], (unsigned long long)((S - a) * b));
    atomicAdd(&acc[c + ny + 1], (unsigned long long)(a * b));
  }
}

// Integer CIC deposit of a species (the mixed form's weights, exact, so the
// grid is the single runs' bit for bit): deposit_warp_sorted over chunks of
// consecutive particles, each cell with its run's row stride.
template <int T>
__global__ void __launch_bounds__(T) k_batch_deposit(const BRun* __restrict__ runs, const int* __restrict__ node_run,
                                                     MixedSoA p, const long long* __restrict__ d_n,
                                                     unsigned long long* __restrict__ acc) {
  constexpr int CHUNK = T * DEP_PER_THREAD;
  __shared__ DepWarp tables[T / 32];
  DepWarp& w = tables[threadIdx.x >> 5];
  const long long n = *d_n;
  const RunNy ny_of{runs, node_run};
  dep_init(w);
  for (long long chunk = (long long)blockIdx.x * CHUNK; chunk < n; chunk += (long long)gridDim.x * CHUNK) {
    const long long q0 = chunk + (long long)threadIdx.x * DEP_PER_THREAD;
    int c[DEP_PER_THREAD];
    float ox[DEP_PER_THREAD], oy[DEP_PER_THREAD];
#pragma unroll
    for (int k = 0; k < DEP_PER_THREAD; k++) {
      const long long q = q0 + k;
      c[k] = q < n ? __ldg(&p.cell[q]) : -1;
      ox[k] = q < n ? __ldg(&p.ox[q]) : 0.f;
      oy[k] = q < n ? __ldg(&p.oy[q]) : 0.f;
    }
    deposit_warp_sorted(acc, w, ny_of, c, ox, oy);
  }
}

// -------------------------------------------------------------- solve ---
struct BatchSpec {
  const BRun* runs;
  double* phi;
  const double* rho;
  const float* Q;
  const float* D;
  float *t0, *t1;
  double* partials;
  int* state;  // 4 per run
};

__device__ __forceinline__ SpecLattice run_lattice(const BatchSpec& b, int ri) {
  const BRun& r = b.runs[ri];
  SpecLattice L;
  L.nx = r.nx;
  L.ny = r.ny;
  L.I_off = 0;
  L.NY = r.ny;
  L.R = r.R;
  L.C = r.C;
  L.flat = r.flat;
  L.gs_norm = r.gs_norm;
  L.mode = EPIC_POISSON_DIRICHLET;  // batches run the reference's boundary
  L.bmean = nullptr;
  L.dx2 = r.dx * r.dx;
  L.K = r.K;
  L.tol = r.tol;
  L.rho = b.rho + r.node_off;
  L.phi = b.phi + r.node_off;
  L.t0 = b.t0 + r.lat_off;
  L.partials = b.partials + r.chunk_off;
  L.state = b.state + 4 * ri;
  L.info = nullptr;
  L.iter_total = nullptr;
  return L;
}

__global__ void k_batch_spec_init(BatchSpec b, const int* __restrict__ node_run, long long nodes, int nruns) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nodes; k += (long long)gridDim.x * blockDim.x)
    b.phi[k] = 0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nruns; r += gridDim.x * blockDim.x) {
    b.state[4 * r] = 0;
    b.state[4 * r + 1] = 0;
  }
}

__global__ void __launch_bounds__(256) k_batch_spec_residual(BatchSpec b, const int2* __restrict__ sched) {
  const int2 e = sched[blockIdx.x];  // (run, chunk)
  if (b.state[4 * e.x]) return;
  __shared__ double sm[8];
  spec_residual_chunk(run_lattice(b, e.x), e.y, sm);
}

__global__ void k_batch_spec_check(BatchSpec b, int nruns, int final_pass) {
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nruns; r += gridDim.x * blockDim.x)
    spec_check(run_lattice(b, r), final_pass);
}

// One of the four products of a refinement stage for every (run, tile) of
// the schedule: 0 t1 = Q_R t0; 1 t0 = (t1 Q_C) o D; 2 t1 = Q_R t0; 3 phi += t1 Q_C.
// TILE 16 or 32: spec_gemm_tile; 64: the register-blocked spec_gemm_tile64
// (the same k order, so the same results).
template <int PROD, int TILE>
__global__ void __launch_bounds__(256) k_batch_spec_gemm(BatchSpec b, const int4* __restrict__ sched) {
  const int4 e = sched[blockIdx.x];  // (run, tile row, tile col)
  if (b.state[4 * e.x]) return;
  __shared__ float As[TILE == 64 ? 1 : 32][33];
  __shared__ float Bs[TILE == 64 ? 1 : 32][33];
  __shared__ __align__(16) SpecGemmSmem sg[TILE == 64 ? 1 : 1];
  const BRun& r = b.runs[e.x];
  const SpecLattice L = run_lattice(b, e.x);
  float* t0 = b.t0 + r.lat_off;
  float* t1 = b.t1 + r.lat_off;
  const float* QR = b.Q + r.qR_off;
  const float* QC = b.Q + r.qC_off;
  if constexpr (TILE == 64) {
    if (PROD == 0 || PROD == 2) spec_gemm_tile64<0>(r.R, r.C, r.R, QR, t0, t1, nullptr, &L, e.y, e.z, sg[0]);
    else if (PROD == 1) spec_gemm_tile64<1>(r.R, r.C, r.C, t1, QC, t0, b.D + r.lat_off, &L, e.y, e.z, sg[0]);
    else spec_gemm_tile64<2>(r.R, r.C, r.C, t1, QC, nullptr, nullptr, &L, e.y, e.z, sg[0]);
  } else {
    if (PROD == 0 || PROD == 2)
      spec_gemm_tile<0, TILE>(r.R, r.C, r.R, QR, t0, t1, nullptr, &L, e.y, e.z, As, Bs);
    else if (PROD == 1)
      spec_gemm_tile<1, TILE>(r.R, r.C, r.C, t1, QC, t0, b.D + r.lat_off, &L, e.y, e.z, As, Bs);
    else
      spec_gemm_tile<2, TILE>(r.R, r.C, r.C, t1, QC, nullptr, nullptr, &L, e.y, e.z, As, Bs);
  }
}

}  // namespace epic

// ================================================================ host ===
using namespace epic;

namespace {

epic_status bfail(epic_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  set_last_error(buf);
  return st;
}

#define BCK(call)                                                                                       \
  do {                                                                                                  \
    cudaError_t e_ = (call);                                                                            \
    if (e_ != cudaSuccess)                                                                              \
      return bfail(e_ == cudaErrorMemoryAllocation ? EPIC_ERR_NOMEM : EPIC_ERR_CUDA, "%s: %s", #call,  \
                   cudaGetErrorString(e_));                                                             \
  } while (0)

int size_class(int R, int C) {
  const int m = std::max(R, C);
  return m <= 48 ? 0 : m <= 96 ? 1 : m <= 160 ? 2 : 3;
}

}  // namespace

struct epic_batch {
  int nruns = 0, nsp = 0, sort_every = 0;
  long long nodes = 0;
  int num_sms = 0, grid = 0;
  cudaStream_t stream = nullptr;
  std::vector<BRun> runs;
  std::vector<epic_request> reqs;
  std::vector<long long> poff, pn;  // [run * nsp + s]
  BRun* d_runs = nullptr;
  int* d_node_run = nullptr;
  double *phi = nullptr, *rho = nullptr, *efx = nullptr, *efy = nullptr;
  float2* ef32 = nullptr;
  MixedSoA arena[BATCH_MAX_SPECIES];
  long long* d_n[BATCH_MAX_SPECIES];
  long long cap[BATCH_MAX_SPECIES];
  unsigned long long* acc[BATCH_MAX_SPECIES];
  float *Q = nullptr, *D = nullptr, *t0 = nullptr, *t1 = nullptr;
  double* partials = nullptr;
  int* state = nullptr;
  int* flags = nullptr;
  int2* chunk_sched = nullptr;
  int nchunk = 0;
  int4* tile_sched[3] = {nullptr, nullptr, nullptr};  // TILE 16, 32, 64
  int ntile[3] = {0, 0, 0};
  int tiles[4] = {32, 32, 32, 32};
  // Launch shapes of the particle passes (the autotuner's choice): threads
  // per CTA and CTAs of the fused push and of the deposit pass.
  int push_threads = PART_THREADS, push_blocks = 0, dep_threads = PART_THREADS, dep_blocks = 0;
  float push_ms[5] = {0, 0, 0, 0, 0}, dep_ms[6] = {0, 0, 0, 0, 0, 0};
  bool particles_tuned = false;
  // Phase timers (epic_batch_set_profiling): events around each phase of a
  // step launched directly (not while a graph is being captured).
  bool profiling = false;
  std::vector<cudaEvent_t> event_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_pending;
  double prof_ms[7] = {0, 0, 0, 0, 0, 0, 0};
  long long prof_count[7] = {0, 0, 0, 0, 0, 0, 0};

  struct Phase {  // phases as epic_get_profile: 0 deposit .. 6 sort
    epic_batch* b;
    int phase;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    Phase(epic_batch* b_, int p) : b(b_), phase(p) {
      if (!b->profiling) return;
      cudaStreamCaptureStatus cs;
      if (cudaStreamIsCapturing(b->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
      e0 = b->take_event();
      e1 = b->take_event();
      cudaEventRecord(e0, b->stream);
    }
    ~Phase() {
      if (!e0) return;
      cudaEventRecord(e1, b->stream);
      b->prof_pending.push_back({phase, {e0, e1}});
    }
  };
  cudaEvent_t take_event() {
    if (!event_pool.empty()) {
      cudaEvent_t e = event_pool.back();
      event_pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
  void* sort_buf = nullptr;
  double* staging = nullptr;
  int64_t step_index = 0;
  cudaGraphExec_t g_plain = nullptr, g_sort = nullptr;
  // acc holds the deposit of the current positions (the step's push leaves it
  // so); the counts before the MCC, whose products are deposited after it
  bool acc_valid = false;
  long long* d_nold = nullptr;
  // some run has absorbing walls: the compacting push, its ordered tile scan
  bool has_open = false;
  unsigned long long* tile_status = nullptr;
  unsigned int* tile_ctr = nullptr;
  long long tile_status_len = 0;
  std::vector<void*> allocs;
  // Emitters (src/emitter.cpp:5-36): per species the (run, emitter) rows that
  // feed it, its points per step and the largest emitter; the injection count
  // that keys the draws; each species' count before a step's injections
  BEmit* d_emit[BATCH_MAX_SPECIES] = {};
  int nemit[BATCH_MAX_SPECIES] = {};
  int emit_max[BATCH_MAX_SPECIES] = {};
  long long emit_total[BATCH_MAX_SPECIES] = {};
  bool any_emit = false;
  unsigned long long* d_inj = nullptr;
  long long* d_efrom = nullptr;
  // Conductors: every run's rectangles and electrodes, whether its electrodes
  // exist yet, the rho override of the runs that solve with SOR (nodes of the
  // batch's node space) and those runs; each run's list for the host loader
  double4 *d_cond_rect = nullptr, *d_cond_circ = nullptr;
  int* d_cond_live = nullptr;
  int* d_cond_nodes = nullptr;
  double* d_cond_vals = nullptr;
  int* d_cond_runs = nullptr;
  int cond_nnodes = 0, cond_nruns = 0;
  std::vector<std::vector<epic_conductor>> conductors;
  // MCC
  bool any_mcc = false;
  double gas_density = 0;
  CrossSections cs;
  McEvents ev;
  unsigned long long *d_step = nullptr, *d_ncoll = nullptr;

  template <class T>
  epic_status alloc(T** p, size_t count) {
    *p = nullptr;
    BCK(cudaMallocAsync((void**)p, std::max<size_t>(count, 1) * sizeof(T), stream));
    BCK(cudaMemsetAsync(*p, 0, std::max<size_t>(count, 1) * sizeof(T), stream));
    allocs.push_back(*p);
    return EPIC_OK;
  }

  BatchSpec spec() const {
    BatchSpec b;
    b.runs = d_runs;
    b.phi = phi;
    b.rho = rho;
    b.Q = Q;
    b.D = D;
    b.t0 = t0;
    b.t1 = t1;
    b.partials = partials;
    b.state = state;
    return b;
  }

  BatchGrids grids() const {
    BatchGrids g;
    g.nruns = nruns;
    g.nsp = nsp;
    g.nodes = nodes;
    g.runs = d_runs;
    g.node_run = d_node_run;
    g.phi = phi;
    g.rho = rho;
    g.efx = efx;
    g.efy = efy;
    g.ef32 = ef32;
    for (int s = 0; s < BATCH_MAX_SPECIES; s++) g.acc[s] = s < nsp ? acc[s] : nullptr;
    return g;
  }

  void launch_gemms(int prod, int which) {
    const BatchSpec b = spec();
    const int n = ntile[which];
    if (!n) return;
    const int4* sc = tile_sched[which];
    if (which == 0) {
      if (prod == 0 || prod == 2) k_batch_spec_gemm<0, 16><<<n, 256, 0, stream>>>(b, sc);
      else if (prod == 1) k_batch_spec_gemm<1, 16><<<n, 256, 0, stream>>>(b, sc);
      else k_batch_spec_gemm<3, 16><<<n, 256, 0, stream>>>(b, sc);
    } else if (which == 1) {
      if (prod == 0 || prod == 2) k_batch_spec_gemm<0, 32><<<n, 256, 0, stream>>>(b, sc);
      else if (prod == 1) k_batch_spec_gemm<1, 32><<<n, 256, 0, stream>>>(b, sc);
      else k_batch_spec_gemm<3, 32><<<n, 256, 0, stream>>>(b, sc);
    } else {
      if (prod == 0 || prod == 2) k_batch_spec_gemm<0, 64><<<n, 256, 0, stream>>>(b, sc);
      else if (prod == 1) k_batch_spec_gemm<1, 64><<<n, 256, 0, stream>>>(b, sc);
      else k_batch_spec_gemm<3, 64><<<n, 256, 0, stream>>>(b, sc);
    }
  }

  BatchConductors cond_view() const { return BatchConductors{d_cond_rect, d_cond_circ, d_cond_live}; }

  void solve() {
    const BatchSpec b = spec();
    if (cond_nnodes || cond_nruns) {  // the SOR runs' Grid::initialize: the same right-hand side for the spectral solve
      const int m = std::max(cond_nnodes, cond_nruns);
      k_batch_conductor_rho<<<std::max(1, std::min(grid, (m + 255) / 256)), 256, 0, stream>>>(
          rho, d_cond_nodes, d_cond_vals, cond_nnodes, d_cond_runs, cond_nruns, d_cond_live);
    }
    k_batch_spec_init<<<grid, 256, 0, stream>>>(b, d_node_run, nodes, nruns);
    for (int st = 0; st < BATCH_STAGES; st++) {
      k_batch_spec_residual<<<nchunk, 256, 0, stream>>>(b, chunk_sched);
      k_batch_spec_check<<<(nruns + 255) / 256, 256, 0, stream>>>(b, nruns, 0);
      for (int prod = 0; prod < 4; prod++)
        for (int w = 0; w < 3; w++) launch_gemms(prod, w);
    }
    k_batch_spec_residual<<<nchunk, 256, 0, stream>>>(b, chunk_sched);
    k_batch_spec_check<<<(nruns + 255) / 256, 256, 0, stream>>>(b, nruns, 1);
  }

  void deposit_all() {
    for (int s = 0; s < nsp; s++) {
      cudaMemsetAsync(acc[s], 0, nodes * sizeof(unsigned long long), stream);
      launch_deposit(arena[s], d_n[s], acc[s], dep_threads, dep_blocks ? dep_blocks : grid);
    }
    acc_valid = true;
  }

  void launch_deposit(const MixedSoA& a, const long long* dn, unsigned long long* out, int T, int blocks) {
    if (T == 128) k_batch_deposit<128><<<blocks, 128, 0, stream>>>(d_runs, d_node_run, a, dn, out);
    else k_batch_deposit<256><<<blocks, 256, 0, stream>>>(d_runs, d_node_run, a, dn, out);
  }

  template <bool SEL>
  void launch_push(const MixedSoA& a, const long long* dn, const float2* ef, int s, unsigned long long* out, int T,
                   int blocks) {
    if (T == 128)
      k_batch_push_dep<SEL, 128><<<blocks, 128, 0, stream>>>(d_runs, d_node_run, a, dn, ef, s, out, d_step, ev);
    else
      k_batch_push_dep<SEL, 256><<<blocks, 256, 0, stream>>>(d_runs, d_node_run, a, dn, ef, s, out, d_step, ev);
  }

  void deposit_and_solve() {
    if (!acc_valid) {
      Phase ph(this, 0);
      deposit_all();
    }
    {
      Phase ph(this, 1);
      launch_batch_finalize(stream, grids());
    }
    {
      Phase ph(this, 2);
      solve();
    }
    Phase ph(this, 3);
    launch_batch_efield(stream, grids());
  }

  void sort_all() {
    Geom g;
    std::memset(&g, 0, sizeof(g));
    g.nx = 1;
    g.ny = (int)nodes;
    for (int s = 0; s < nsp; s++) {
      ParticleRef p;
      std::memset(&p, 0, sizeof(p));
      p.mixed = 1;
      p.m = arena[s];
      launch_sort(stream, g, p, d_n[s], cap[s], carve_sort_scratch(sort_buf, cap[s]), grid);
    }
  }

  // A step's injections, first in the step as in the run alone
  // (src/main.cpp:397-403): each species' emitters in one launch, its count
  // advanced past them, and their deposit added to the accumulators when these
  // hold the others' (with absorbing walls the step deposits everything).
  void inject() {
    for (int s = 0; s < nsp; s++) {
      if (!nemit[s]) continue;
      const int bx = std::max(1, std::min((emit_max[s] + PART_THREADS - 1) / PART_THREADS, grid / nemit[s]));
      k_batch_emit<<<dim3(bx, nemit[s]), PART_THREADS, 0, stream>>>(d_runs, d_emit[s], arena[s], d_n[s], cap[s],
                                                                   d_inj, flags);
      k_batch_emit_commit<<<1, 1, 0, stream>>>(d_n[s], d_efrom + s, emit_total[s], cap[s], flags);
      if (acc_valid && !has_open)
        k_batch_deposit_range<<<grid, PART_THREADS, 0, stream>>>(d_runs, d_node_run, arena[s], d_efrom + s, d_n[s],
                                                                 acc[s]);
    }
    launch_inject_tick(stream, d_inj);
  }

  // A step: (injections, sort,) field phase from the accumulators, then each
  // species' push deposits its new positions (and the electrons' push selects
  // the MCC's candidates), the MCC, and the deposit of its ionisation products.
  void step(int sort) {
    if (any_emit) {
      Phase ph(this, 0);
      inject();
    }
    if (sort) {
      Phase ph(this, 6);
      sort_all();  // the accumulators do not depend on the order
    }
    if (has_open) {  // erasing pushes: deposit, field, compacting push, MCC with its own selection
      {
        Phase ph(this, 0);
        deposit_all();
      }
      deposit_and_solve();
      {
        Phase ph(this, 4);
        for (int s = 0; s < nsp; s++) {
          cudaMemsetAsync(tile_ctr, 0, sizeof(unsigned int), stream);
          cudaMemsetAsync(tile_status, 0, tile_status_len * sizeof(unsigned long long), stream);
          k_batch_push_compact<<<grid, PART_THREADS, 0, stream>>>(d_runs, d_node_run, arena[s], d_n[s], ef32, s,
                                                                  tile_status, tile_ctr, flags, spin_limit(),
                                                                  cond_view());
        }
      }
      if (any_mcc) {
        Phase ph(this, 5);
        launch_batch_mcc(stream, cs, d_runs, d_node_run, arena[0], d_n[0], cap[0], arena[1], d_n[1], cap[1], d_step,
                         ev, d_ncoll, flags, grid);
      }
      acc_valid = false;
      return;
    }
    deposit_and_solve();
    {
      Phase ph(this, 4);
      const int grid_dep =
          push_blocks ? push_blocks : resident_grid(k_batch_push_dep<true, PART_THREADS>, PART_THREADS);
      for (int s = 0; s < nsp; s++) {
        cudaMemsetAsync(acc[s], 0, nodes * sizeof(unsigned long long), stream);
        if (any_mcc && s == 0) launch_push<true>(arena[s], d_n[s], ef32, s, acc[s], push_threads, grid_dep);
        else launch_push<false>(arena[s], d_n[s], ef32, s, acc[s], push_threads, grid_dep);
      }
    }
    if (any_mcc) {
      {
        Phase ph(this, 5);
        for (int k = 0; k < 2; k++)
          cudaMemcpyAsync(d_nold + k, d_n[k], sizeof(long long), cudaMemcpyDeviceToDevice, stream);
        launch_batch_mcc(stream, cs, d_runs, d_node_run, arena[0], d_n[0], cap[0], arena[1], d_n[1], cap[1], d_step,
                         ev, d_ncoll, flags, grid, 1);
      }
      Phase ph(this, 0);
      for (int k = 0; k < 2; k++)
        k_batch_deposit_range<<<grid, PART_THREADS, 0, stream>>>(d_runs, d_node_run, arena[k], d_nold + k, d_n[k],
                                                                 acc[k]);
    }
    acc_valid = true;
  }
};

namespace {

// Builds the GEMM tile schedules: per size class the tile the autotuner chose.
int tile_index(int t) { return t == 16 ? 0 : t == 32 ? 1 : 2; }

void build_tile_sched(epic_batch* b, std::vector<int4> (&by_tile)[3]) {
  for (auto& v : by_tile) v.clear();
  for (int r = 0; r < b->nruns; r++) {
    const BRun& br = b->runs[r];
    const int t = b->tiles[size_class(br.R, br.C)];
    const int w = tile_index(t);
    for (int tr = 0; tr < (br.R + t - 1) / t; tr++)
      for (int tc = 0; tc < (br.C + t - 1) / t; tc++) by_tile[w].push_back(make_int4(r, tr, tc, 0));
  }
}

epic_status upload_tile_sched(epic_batch* b) {
  std::vector<int4> by_tile[3];
  build_tile_sched(b, by_tile);
  for (int w = 0; w < 3; w++) {
    if (b->tile_sched[w]) cudaFreeAsync(b->tile_sched[w], b->stream);
    b->tile_sched[w] = nullptr;
    b->ntile[w] = (int)by_tile[w].size();
    if (!b->ntile[w]) continue;
    BCK(cudaMallocAsync((void**)&b->tile_sched[w], by_tile[w].size() * sizeof(int4), b->stream));
    BCK(cudaMemcpyAsync(b->tile_sched[w], by_tile[w].data(), by_tile[w].size() * sizeof(int4),
                        cudaMemcpyHostToDevice, b->stream));
  }
  BCK(cudaStreamSynchronize(b->stream));
  return EPIC_OK;
}

// Times one refinement stage's four products for the runs of each size class
// with 16-, 32- and 64-wide tiles and keeps the fastest per class (identical
// results whichever).  Runs before the initial field: it only writes the
// transform scratch and phi, which every solve starts over.
epic_status autotune(epic_batch* b) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best[4][3];
  for (int cls = 0; cls < 4; cls++) best[cls][0] = best[cls][1] = best[cls][2] = 0;
  const int widths[3] = {16, 32, 64};
  for (int w = 0; w < 3; w++) {
    for (int cls = 0; cls < 4; cls++) {
      bool any = false;
      for (int r = 0; r < b->nruns; r++) any |= size_class(b->runs[r].R, b->runs[r].C) == cls;
      if (!any) continue;
      int saved[4];
      std::memcpy(saved, b->tiles, sizeof(saved));
      for (int c = 0; c < 4; c++) b->tiles[c] = 0;  // only this class is scheduled
      b->tiles[cls] = widths[w];
      std::vector<int4> by_tile[3];
      for (int r = 0; r < b->nruns; r++) {
        const BRun& br = b->runs[r];
        if (size_class(br.R, br.C) != cls) continue;
        const int t = b->tiles[cls];
        for (int tr = 0; tr < (br.R + t - 1) / t; tr++)
          for (int tc = 0; tc < (br.C + t - 1) / t; tc++) by_tile[w].push_back(make_int4(r, tr, tc, 0));
      }
      std::memcpy(b->tiles, saved, sizeof(saved));
      int4* sc = nullptr;
      BCK(cudaMallocAsync((void**)&sc, by_tile[w].size() * sizeof(int4), b->stream));
      BCK(cudaMemcpyAsync(sc, by_tile[w].data(), by_tile[w].size() * sizeof(int4), cudaMemcpyHostToDevice,
                          b->stream));
      int4* keep[3] = {b->tile_sched[0], b->tile_sched[1], b->tile_sched[2]};
      const int nkeep[3] = {b->ntile[0], b->ntile[1], b->ntile[2]};
      b->tile_sched[0] = b->tile_sched[1] = b->tile_sched[2] = nullptr;
      b->ntile[0] = b->ntile[1] = b->ntile[2] = 0;
      b->tile_sched[w] = sc;
      b->ntile[w] = (int)by_tile[w].size();
      for (int rep = 0; rep < 2; rep++)
        for (int prod = 0; prod < 4; prod++) b->launch_gemms(prod, w);  // warm-up
      cudaEventRecord(e0, b->stream);
      for (int rep = 0; rep < 5; rep++)
        for (int prod = 0; prod < 4; prod++) b->launch_gemms(prod, w);
      cudaEventRecord(e1, b->stream);
      BCK(cudaEventSynchronize(e1));
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      best[cls][w] = ms;
      cudaFreeAsync(sc, b->stream);
      for (int k = 0; k < 3; k++) {
        b->tile_sched[k] = keep[k];
        b->ntile[k] = nkeep[k];
      }
    }
  }
  for (int cls = 0; cls < 4; cls++) {
    if (!(best[cls][0] > 0)) continue;
    int k = 0;
    for (int w = 1; w < 3; w++)
      if (best[cls][w] > 0 && best[cls][w] < best[cls][k]) k = w;
    b->tiles[cls] = widths[k];
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  BCK(cudaGetLastError());
  return upload_tile_sched(b);
}

// Launch shapes of the particle passes, timed on a sample: a copy of the
// first 2^24 particles of species 0 pushed through a zero field and deposited
// into a scratch accumulator (the batch's own particles, runs and node table;
// the copy is discarded), one warm-up and three timed launches per shape.  The
// shapes change neither the push nor the integer deposit, so results do not
// depend on the choice.  Runs after the particles are loaded.
epic_status tune_particle_passes(epic_batch* b) {
  const long long n0 = b->pn.empty() ? 0 : [&] {
    long long t = 0;
    for (int r = 0; r < b->nruns; r++) t += b->pn[(size_t)r * b->nsp];
    return t;
  }();
  const long long ns = std::min<long long>(n0, 1ll << 24);
  if (ns < 1) return EPIC_OK;
  const int sms = b->num_sms;
  MixedSoA sm;
  std::memset(&sm, 0, sizeof(sm));
  long long* dns = nullptr;
  unsigned long long* sacc = nullptr;
  float2* zef = nullptr;
  BCK(cudaMallocAsync((void**)&sm.cell, ns * sizeof(int), b->stream));
  BCK(cudaMallocAsync((void**)&sm.ox, ns * sizeof(float), b->stream));
  BCK(cudaMallocAsync((void**)&sm.oy, ns * sizeof(float), b->stream));
  BCK(cudaMallocAsync((void**)&sm.vx, ns * sizeof(float), b->stream));
  BCK(cudaMallocAsync((void**)&sm.vy, ns * sizeof(float), b->stream));
  BCK(cudaMallocAsync((void**)&sm.vz, ns * sizeof(float), b->stream));
  BCK(cudaMallocAsync((void**)&dns, sizeof(long long), b->stream));
  BCK(cudaMallocAsync((void**)&sacc, b->nodes * sizeof(unsigned long long), b->stream));
  BCK(cudaMallocAsync((void**)&zef, b->nodes * sizeof(float2), b->stream));
  const MixedSoA& a = b->arena[0];
  BCK(cudaMemcpyAsync(sm.cell, a.cell, ns * sizeof(int), cudaMemcpyDeviceToDevice, b->stream));
  BCK(cudaMemcpyAsync(sm.ox, a.ox, ns * sizeof(float), cudaMemcpyDeviceToDevice, b->stream));
  BCK(cudaMemcpyAsync(sm.oy, a.oy, ns * sizeof(float), cudaMemcpyDeviceToDevice, b->stream));
  BCK(cudaMemcpyAsync(sm.vx, a.vx, ns * sizeof(float), cudaMemcpyDeviceToDevice, b->stream));
  BCK(cudaMemcpyAsync(sm.vy, a.vy, ns * sizeof(float), cudaMemcpyDeviceToDevice, b->stream));
  BCK(cudaMemcpyAsync(sm.vz, a.vz, ns * sizeof(float), cudaMemcpyDeviceToDevice, b->stream));
  BCK(cudaMemcpyAsync(dns, &ns, sizeof(long long), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemsetAsync(zef, 0, b->nodes * sizeof(float2), b->stream));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto time_it = [&](auto&& launch) -> float {
    float tot = 0;
    for (int rep = 0; rep < 4; rep++) {
      cudaMemsetAsync(sacc, 0, b->nodes * sizeof(unsigned long long), b->stream);
      cudaEventRecord(e0, b->stream);
      launch();
      cudaEventRecord(e1, b->stream);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep) tot += ms;  // the first launch warms up
    }
    return tot / 3;
  };
  // push: 128 and 256 threads with every CTA resident, 256 with 1 and 2 CTAs
  // per SM, 128 with 3
  const int pT[5] = {128, 256, 256, 256, 128};
  const int pB[5] = {resident_grid(k_batch_push_dep<false, 128>, 128),
                     resident_grid(k_batch_push_dep<false, 256>, 256), sms, 2 * sms, 3 * sms};
  // A shape replaces the default only if the sample runs it at least 5 %
  // faster: the sample is a few runs' particles, and differences within that
  // margin have not carried over to the whole batch (a 0.2 % gain on the
  // sample measured 18 % slower on the batch).
  auto pick = [](const float* ms, int nv, int def) {
    int best = def;
    for (int v = 0; v < nv; v++)
      if (ms[v] > 0 && ms[v] < ms[best]) best = v;
    return ms[best] < 0.95f * ms[def] ? best : def;
  };
  int best = -1;
  if (!b->has_open) {
    for (int v = 0; v < 5; v++)
      b->push_ms[v] = time_it([&] { b->launch_push<false>(sm, dns, zef, 0, sacc, pT[v], pB[v]); });
    best = pick(b->push_ms, 5, 1);  // default: 256 threads, every CTA resident
    b->push_threads = pT[best];
    b->push_blocks = pB[best];
  }
  // deposit: 128 and 256 threads at full occupancy, 256 with 4, 8 and 16
  // CTAs per SM, 128 with 8
  const int dT[6] = {128, 256, 256, 256, 256, 128};
  const int dB[6] = {resident_grid(k_batch_deposit<128>, 128), resident_grid(k_batch_deposit<256>, 256), 4 * sms,
                     8 * sms, 16 * sms, 8 * sms};
  for (int v = 0; v < 6; v++) b->dep_ms[v] = time_it([&] { b->launch_deposit(sm, dns, sacc, dT[v], dB[v]); });
  best = pick(b->dep_ms, 6, 3);  // default: 256 threads, 8 CTAs per SM
  b->dep_threads = dT[best];
  b->dep_blocks = dB[best];
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  void* bufs[9] = {sm.cell, sm.ox, sm.oy, sm.vx, sm.vy, sm.vz, dns, sacc, zef};
  for (void* q : bufs) cudaFreeAsync(q, b->stream);
  BCK(cudaStreamSynchronize(b->stream));
  BCK(cudaGetLastError());
  return EPIC_OK;
}

// Transforms of side n (orthonormal DST-I) and eigenvalues, as the single run.
void sine_transform_h(int n, std::vector<float>& Q, std::vector<double>& lam) {
  const double pi = 3.14159265358979323846;
  const double c = std::sqrt(2.0 / (n + 1));
  Q.assign((size_t)n * n, 0.f);
  lam.assign(n, 0.0);
  for (int j = 0; j < n; j++) {
    for (int k = 0; k < n; k++) Q[(size_t)j * n + k] = (float)(c * std::sin(pi * (j + 1) * (double)(k + 1) / (n + 1)));
    const double sn = std::sin(pi * (j + 1) / (2.0 * (n + 1)));
    lam[j] = -4.0 * sn * sn;
  }
}

epic_status build(epic_batch* b, const epic_request* reqs, int nruns) {
  if (nruns < 1) return bfail(EPIC_ERR_INVALID, "empty batch");
  b->nruns = nruns;
  b->reqs.assign(reqs, reqs + nruns);
  b->nsp = reqs[0].num_species;
  if (b->nsp < 1 || b->nsp > BATCH_MAX_SPECIES)
    return bfail(EPIC_ERR_INVALID, "a batch holds 1 to %d species per run", BATCH_MAX_SPECIES);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, dev);
  b->grid = b->num_sms * 8;
  BCK(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  // Lay out runs, lattices, transforms.
  b->runs.resize(nruns);
  b->poff.assign((size_t)nruns * b->nsp, 0);
  b->pn.assign((size_t)nruns * b->nsp, 0);
  long long node_off = 0, lat_off = 0, qpool = 0;
  int chunk_off = 0;
  std::vector<long long> q_off_of_side(4096, -1);
  std::vector<std::pair<int, long long>> sides;  // (side, offset) of each transform
  std::vector<int2> chunks;
  for (int r = 0; r < nruns; r++) {
    const epic_config& c = reqs[r].cfg;
    if (reqs[r].num_species != b->nsp) return bfail(EPIC_ERR_INVALID, "run %d: every run needs %d species", r, b->nsp);
    if (c.precision != EPIC_PRECISION_MIXED) return bfail(EPIC_ERR_INVALID, "run %d: batches run the mixed form", r);
    if (reqs[r].num_conductors < 0 || reqs[r].num_conductors > EPIC_REQUEST_MAX_CONDUCTORS)
      return bfail(EPIC_ERR_INVALID, "run %d: bad conductor count", r);
    for (int k = 0; k < reqs[r].num_conductors; k++) {  // epic_add_conductor's checks
      const epic_conductor& g = reqs[r].conductors[k];
      if (g.type != EPIC_CONDUCTOR_RECT && g.type != EPIC_CONDUCTOR_CIRCULAR)
        return bfail(EPIC_ERR_INVALID, "run %d: unknown conductor type %d", r, g.type);
      if (g.type == EPIC_CONDUCTOR_CIRCULAR && (g.electrode_number < 1 || g.electrode_number > 4096))
        return bfail(EPIC_ERR_INVALID, "run %d: electrode_number must be in [1, 4096]", r);
    }
    // conductors erase particles: the batch's push is then the compacting one
    if (reqs[r].num_conductors) b->has_open = true;
    if (reqs[r].num_emitters < 0 || reqs[r].num_emitters > EPIC_REQUEST_MAX_EMITTERS)
      return bfail(EPIC_ERR_INVALID, "run %d: bad emitter count", r);
    for (int k = 0; k < reqs[r].num_emitters; k++) {
      const epic_emitter& m = reqs[r].emitters[k];
      if (m.species_idx1 < 0 || m.species_idx1 >= b->nsp || m.species_idx2 < 0 || m.species_idx2 >= b->nsp)
        return bfail(EPIC_ERR_INVALID, "run %d: emitter %d: species index out of range", r, k);
      if (m.numparticle < 0 || m.numparticle > (1 << 28))
        return bfail(EPIC_ERR_INVALID, "run %d: emitter %d: bad numparticle", r, k);
    }
    if (c.shape != EPIC_CIC) return bfail(EPIC_ERR_INVALID, "run %d: batches deposit with CIC", r);
    if (c.bc != EPIC_PBC && c.bc != EPIC_REFLECTIVE && c.bc != EPIC_OPEN)
      return bfail(EPIC_ERR_INVALID, "run %d: bad wall rule", r);
    if (c.bc == EPIC_OPEN) b->has_open = true;
    if (reqs[r].collisions) {
      if (b->nsp < 2) return bfail(EPIC_ERR_INVALID, "run %d: MCC needs electrons (species 0) and ions (1)", r);
      if (b->any_mcc && c.gas_density != b->gas_density)
        return bfail(EPIC_ERR_INVALID, "run %d: the MCC runs of a batch share one gas density", r);
      b->any_mcc = true;
      b->gas_density = c.gas_density;
    }
    const Geom g{c.nx, c.ny, c.x0, c.y0, c.dx, c.dy, 0, 0};
    if (c.poisson_bc != EPIC_POISSON_DIRICHLET || !spectral_supported(g, c.solver, c.poisson_bc)) return bfail(EPIC_ERR_INVALID, "run %d: grid not supported", r);
    if (c.nx > 4095 || c.ny > 4095) return bfail(EPIC_ERR_INVALID, "run %d: grid too large for a batch", r);
    BRun& br = b->runs[r];
    std::memset(&br, 0, sizeof(br));
    br.nx = c.nx;
    br.ny = c.ny;
    br.bc = c.bc;
    br.node_off = node_off;
    br.x0 = c.x0;
    br.y0 = c.y0;
    br.dx = c.dx;
    br.dy = c.dy;
    const double K = (c.density * QE * c.L) / (EPS_0 * c.W * c.vel_norm);
    const double cc = c.vel_norm / (c.L * c.W);
    const double dtsub = c.DT * 1;
    br.cx = (float)(cc * dtsub / c.dx);
    br.cy = (float)(cc * dtsub / c.dy);
    for (int s = 0; s < b->nsp; s++) {
      const epic_species_desc& d = reqs[r].species[s];
      const double qm = d.charge / d.mass;
      const double qmK = qm * K;
      br.qmK_dt[s] = (float)(qmK * dtsub);
      const double hqmK = 0.5 * qm * K;
      br.hqmK_dt[s] = (float)(hqmK * c.DT);
      br.spwt[s] = d.spwt;
      br.charge_over_qe[s] = d.charge * (1 / QE);
    }
    const double cell_area = c.dx * c.dy;
    const double L2 = c.L * c.L;
    br.div = cell_area * L2 * c.density;
    br.inv_scale = std::ldexp(1.0, -2 * MIXED_OFFSET_BITS);
    br.K = (c.L * c.L) / (c.LDe * c.LDe);
    br.tol = c.tolerance;
    const bool gs = c.solver == EPIC_SOLVER_GS;
    br.flat = !gs;
    br.gs_norm = gs;
    br.R = gs ? c.nx - 2 : c.ny;
    br.C = gs ? c.ny - 2 : c.nx;
    // a single run solves lattices with a side of 512 or more unknowns by FFT
    // passes (where its sides allow), the batch by the dense products: such a
    // run would not equal its single run bit for bit, so it runs alone
    if (std::max(br.R, br.C) >= 512)
      return bfail(EPIC_ERR_INVALID, "run %d: lattices with a side of 512 or more unknowns run alone", r);
    br.lat_off = lat_off;
    for (int side : {br.R, br.C}) {
      if (q_off_of_side[side] < 0) {
        q_off_of_side[side] = qpool;
        sides.push_back({side, qpool});
        qpool += (long long)side * side;
      }
    }
    br.qR_off = q_off_of_side[br.R];
    br.qC_off = q_off_of_side[br.C];
    br.mcc = reqs[r].collisions;
    br.vn = c.vel_norm;
    br.dt_phys = c.DT / c.W;
    if (b->nsp >= 2) {
      br.ion_mass = reqs[r].species[1].mass;
      br.ion_temp = reqs[r].species[1].temp;
      br.F1 = ME / (ME + br.ion_mass);
      br.F2 = br.ion_mass / (ME + br.ion_mass);
    }
    br.seed = c.seed ^ (reqs[r].load_seed * 0x9E3779B97F4A7C15ull);
    br.chunk_off = chunk_off;
    const int nch = (br.R * br.C + SPEC_CHUNK - 1) / SPEC_CHUNK;
    for (int k = 0; k < nch; k++) chunks.push_back(make_int2(r, k));
    chunk_off += nch;
    lat_off += (long long)br.R * br.C;
    node_off += (long long)c.nx * c.ny;
  }
  b->nodes = node_off;
  if (b->nodes >= INT_MAX) return bfail(EPIC_ERR_INVALID, "batch node space above 2^31");
  // Particle arrays: run r's species s at poff, in run order.
  for (int s = 0; s < b->nsp; s++) {
    long long off = 0;
    for (int r = 0; r < nruns; r++) {
      b->poff[(size_t)r * b->nsp + s] = off;
      b->pn[(size_t)r * b->nsp + s] = reqs[r].species[s].numparticle;
      off += reqs[r].species[s].numparticle;
    }
    // room for ionisation products: +10 % + 4096 per run, and for a run's
    // injections over its request's steps (overflow raises EPIC_ERR_CAPACITY,
    // as in a single run)
    long long slack = 0;
    for (int r = 0; r < nruns; r++) {
      if (b->any_mcc) slack += reqs[r].species[s].numparticle / 10 + 4096;
      for (int k = 0; k < reqs[r].num_emitters; k++) {
        const epic_emitter& m = reqs[r].emitters[k];
        if (m.species_idx1 == s || m.species_idx2 == s)
          slack += (long long)m.numparticle * std::max(reqs[r].steps, 0);
      }
    }
    b->cap[s] = std::max<long long>(off + slack, 1);
  }
  epic_status st;
  if ((st = b->alloc(&b->d_runs, nruns))) return st;
  if ((st = b->alloc(&b->d_node_run, b->nodes))) return st;
  if ((st = b->alloc(&b->phi, b->nodes))) return st;
  if ((st = b->alloc(&b->rho, b->nodes))) return st;
  if ((st = b->alloc(&b->efx, b->nodes))) return st;
  if ((st = b->alloc(&b->efy, b->nodes))) return st;
  if ((st = b->alloc(&b->ef32, b->nodes))) return st;
  if ((st = b->alloc(&b->Q, qpool))) return st;
  if ((st = b->alloc(&b->D, lat_off))) return st;
  if ((st = b->alloc(&b->t0, lat_off))) return st;
  if ((st = b->alloc(&b->t1, lat_off))) return st;
  if ((st = b->alloc(&b->partials, chunk_off))) return st;
  if ((st = b->alloc(&b->state, 4 * (size_t)nruns))) return st;
  if ((st = b->alloc(&b->flags, 1))) return st;
  if ((st = b->alloc(&b->d_nold, 2))) return st;
  if ((st = b->alloc(&b->chunk_sched, chunks.size()))) return st;
  b->nchunk = (int)chunks.size();
  for (int s = 0; s < b->nsp; s++) {
    const size_t cap = (size_t)b->cap[s];
    MixedSoA& m = b->arena[s];
    if ((st = b->alloc(&m.cell, cap)) || (st = b->alloc(&m.ox, cap)) || (st = b->alloc(&m.oy, cap)) ||
        (st = b->alloc(&m.vx, cap)) || (st = b->alloc(&m.vy, cap)) || (st = b->alloc(&m.vz, cap)))
      return st;
    if ((st = b->alloc(&b->d_n[s], 1))) return st;
    if ((st = b->alloc(&b->acc[s], b->nodes))) return st;
  }
  long long cmax = 0, nmax = 1;
  for (int s = 0; s < b->nsp; s++) cmax = std::max(cmax, b->cap[s]);
  if (b->has_open) {
    b->tile_status_len = cmax / SCAN_TILE + 2;
    if ((st = b->alloc(&b->tile_status, (size_t)b->tile_status_len)) || (st = b->alloc(&b->tile_ctr, 1))) return st;
  }
  for (long long v : b->pn) nmax = std::max(nmax, v);
  if (b->sort_every > 0) {
    BCK(cudaMallocAsync(&b->sort_buf, sort_scratch_bytes(cmax, 24), b->stream));
    b->allocs.push_back(b->sort_buf);
  }
  if ((st = b->alloc(&b->staging, (size_t)nmax * 5))) return st;
  std::memset(&b->cs, 0, sizeof(b->cs));
  std::memset(&b->ev, 0, sizeof(b->ev));
  if ((st = b->alloc(&b->d_step, 1)) || (st = b->alloc(&b->d_ncoll, 4))) return st;
  if (b->any_mcc) {
    const long long ecap = b->cap[0];
    McEvents& ev = b->ev;
    ev.cap = (unsigned int)std::min<long long>(std::max<long long>(ecap / 8, 65536), 1LL << 30);
    const size_t tiles = (size_t)(ecap / MCC_TILE + 2);
    char* buf = nullptr;
    if ((st = b->alloc(&buf, (size_t)ev.cap * ion_event_bytes()))) return st;
    ev.buf = reinterpret_cast<IonEvent*>(buf);
    if ((st = b->alloc(&ev.cand, (size_t)ecap)) || (st = b->alloc(&ev.cand_count, 1)) ||
        (st = b->alloc(&ev.count, 1)) || (st = b->alloc(&ev.slot, (size_t)ecap)) ||
        (st = b->alloc(&ev.tile_cnt, tiles)) || (st = b->alloc(&ev.tile_off, tiles)))
      return st;
    BCK(cudaMemsetAsync(ev.slot, 0xff, (size_t)ecap * sizeof(int), b->stream));
  }
  // Emitter rows: per species, its (run, emitter) rows in run order, each
  // emitter's slot for that species (Emitter::inject's two species), with the
  // single run's parameters (do_inject_range).
  std::vector<BEmit> em[BATCH_MAX_SPECIES];
  for (int r = 0; r < nruns; r++) {
    const epic_config& c = reqs[r].cfg;
    for (int k = 0; k < reqs[r].num_emitters; k++) {
      const epic_emitter& m = reqs[r].emitters[k];
      const int sp_of[2] = {m.species_idx1, m.species_idx2};
      const int slots = m.species_idx1 != m.species_idx2 ? 2 : 1;
      for (int slot = 0; slot < slots; slot++) {
        const int s = sp_of[slot];
        BEmit e;
        std::memset(&e, 0, sizeof(e));
        e.e.x0 = m.x0;
        e.e.y0 = m.y0;
        e.e.x1 = m.x1;
        e.e.y1 = m.y1;
        e.e.vth = sqrt(2 * K_B * m.temp * (QE / K_B) / reqs[r].species[s].mass);  // Init::SampleVel (src/init.cpp:112)
        e.e.vdx = m.vdx * c.vel_norm;
        e.e.vdy = m.vdy * c.vel_norm;
        e.e.vel_norm = c.vel_norm;
        e.e.num = m.numparticle;
        e.e.slot = slot;
        e.e.emitter = k;
        e.seed = c.seed;
        e.off = b->emit_total[s];
        e.run = r;
        b->emit_total[s] += m.numparticle;
        b->emit_max[s] = std::max(b->emit_max[s], m.numparticle);
        em[s].push_back(e);
      }
    }
  }
  for (int s = 0; s < b->nsp; s++) {
    if (em[s].empty()) continue;
    if (em[s].size() > 65535) return bfail(EPIC_ERR_INVALID, "more than 65535 emitters feed species %d", s);
    b->nemit[s] = (int)em[s].size();
    b->any_emit = true;
    if ((st = b->alloc(&b->d_emit[s], em[s].size()))) return st;
    BCK(cudaMemcpyAsync(b->d_emit[s], em[s].data(), em[s].size() * sizeof(BEmit), cudaMemcpyHostToDevice,
                        b->stream));
  }
  if ((st = b->alloc(&b->d_inj, 1)) || (st = b->alloc(&b->d_efrom, BATCH_MAX_SPECIES))) return st;
  // Conductor tables (conductor_geometry, as epic_add_conductor builds them per run).
  std::vector<double> all_rect, all_circ, all_vals;
  std::vector<int> all_nodes, live_runs;
  b->conductors.assign(nruns, {});
  for (int r = 0; r < nruns; r++) {
    const epic_request& q = reqs[r];
    if (!q.num_conductors) continue;
    std::vector<epic_conductor> cv(q.conductors, q.conductors + q.num_conductors);
    std::vector<double> rects, circles, vals;
    std::vector<int> cnodes;
    conductor_geometry(q.cfg, cv, rects, circles, cnodes, vals);
    BRun& br = b->runs[r];
    br.nrect = (int)(rects.size() / 4);
    br.ncirc = (int)(circles.size() / 4);
    br.rect_off = (int)(all_rect.size() / 4);
    br.circ_off = (int)(all_circ.size() / 4);
    all_rect.insert(all_rect.end(), rects.begin(), rects.end());
    all_circ.insert(all_circ.end(), circles.begin(), circles.end());
    if (q.cfg.solver == EPIC_SOLVER_GS) {  // gssolver calls Grid::initialize (src/field.cpp:100-103), pcgsolver not
      for (size_t k = 0; k < cnodes.size(); k++) {
        all_nodes.push_back((int)(br.node_off + cnodes[k]));
        all_vals.push_back(vals[k]);
      }
      live_runs.push_back(r);
    }
    b->conductors[r] = std::move(cv);
  }
  b->cond_nnodes = (int)all_nodes.size();
  b->cond_nruns = (int)live_runs.size();
  if ((st = b->alloc(&b->d_cond_rect, all_rect.size() / 4)) || (st = b->alloc(&b->d_cond_circ, all_circ.size() / 4)) ||
      (st = b->alloc(&b->d_cond_live, nruns)) || (st = b->alloc(&b->d_cond_nodes, all_nodes.size())) ||
      (st = b->alloc(&b->d_cond_vals, all_vals.size())) || (st = b->alloc(&b->d_cond_runs, live_runs.size())))
    return st;
  auto up = [&](void* dst, const void* src, size_t bytes) -> epic_status {
    if (bytes) BCK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, b->stream));
    return EPIC_OK;
  };
  if ((st = up(b->d_cond_rect, all_rect.data(), all_rect.size() * sizeof(double))) ||
      (st = up(b->d_cond_circ, all_circ.data(), all_circ.size() * sizeof(double))) ||
      (st = up(b->d_cond_nodes, all_nodes.data(), all_nodes.size() * sizeof(int))) ||
      (st = up(b->d_cond_vals, all_vals.data(), all_vals.size() * sizeof(double))) ||
      (st = up(b->d_cond_runs, live_runs.data(), live_runs.size() * sizeof(int))))
    return st;
  // Host tables to the device.
  std::vector<int> node_run(b->nodes);
  for (int r = 0; r < nruns; r++)
    std::fill(node_run.begin() + b->runs[r].node_off,
              node_run.begin() + b->runs[r].node_off + (long long)b->runs[r].nx * b->runs[r].ny, r);
  std::vector<float> Qh(std::max<long long>(qpool, 1)), Dh(std::max<long long>(lat_off, 1));
  std::vector<std::vector<double>> lam_of_side(4096);
  for (auto& sd : sides) {
    std::vector<float> q;
    sine_transform_h(sd.first, q, lam_of_side[sd.first]);
    std::copy(q.begin(), q.end(), Qh.begin() + sd.second);
  }
  for (int r = 0; r < nruns; r++) {
    const BRun& br = b->runs[r];
    const std::vector<double>& lR = lam_of_side[br.R];
    const std::vector<double>& lC = lam_of_side[br.C];
    for (int p = 0; p < br.R; p++)
      for (int q = 0; q < br.C; q++) Dh[br.lat_off + (long long)p * br.C + q] = (float)(1.0 / (lR[p] + lC[q]));
  }
  BCK(cudaMemcpyAsync(b->d_runs, b->runs.data(), nruns * sizeof(BRun), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemcpyAsync(b->d_node_run, node_run.data(), node_run.size() * sizeof(int), cudaMemcpyHostToDevice,
                      b->stream));
  BCK(cudaMemcpyAsync(b->Q, Qh.data(), qpool * sizeof(float), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemcpyAsync(b->D, Dh.data(), lat_off * sizeof(float), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemcpyAsync(b->chunk_sched, chunks.data(), chunks.size() * sizeof(int2), cudaMemcpyHostToDevice,
                      b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return autotune(b);
}

epic_status take_flags(epic_batch* b) {
  int f = 0;
  BCK(cudaMemcpyAsync(&f, b->flags, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  if (!f) return EPIC_OK;
  cudaMemsetAsync(b->flags, 0, sizeof(int), b->stream);
  if (f & FLAG_TIMEOUT) return bfail(EPIC_ERR_TIMEOUT, "a device-side wait gave up (flags 0x%x)", f);
  if (f & FLAG_CAPACITY) return bfail(EPIC_ERR_CAPACITY, "a species outgrew the batch's capacity (flags 0x%x)", f);
  if (f & FLAG_OUT_OF_GRID) return bfail(EPIC_ERR_DOMAIN, "a particle was loaded outside its run's grid");
  return bfail(EPIC_ERR_CUDA, "device flags 0x%x", f);
}

}  // namespace

extern "C" {

epic_status epic_batch_create(const epic_request* runs, int nruns, int sort_every, epic_batch** out) {
  if (!runs || !out || sort_every < 0) return bfail(EPIC_ERR_INVALID, "bad argument");
  epic_batch* b = new epic_batch();
  std::memset(b->arena, 0, sizeof(b->arena));
  std::memset(b->d_n, 0, sizeof(b->d_n));
  std::memset(b->acc, 0, sizeof(b->acc));
  b->sort_every = sort_every;
  epic_status st = build(b, runs, nruns);
  if (st) {
    epic_batch_destroy(b);
    return st;
  }
  *out = b;
  return EPIC_OK;
}

void epic_batch_destroy(epic_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (auto& pe : b->prof_pending) {
    cudaEventDestroy(pe.second.first);
    cudaEventDestroy(pe.second.second);
  }
  for (cudaEvent_t e : b->event_pool) cudaEventDestroy(e);
  if (b->g_plain) cudaGraphExecDestroy(b->g_plain);
  if (b->g_sort) cudaGraphExecDestroy(b->g_sort);
  for (void* p : b->allocs) cudaFreeAsync(p, b->stream);
  void* tables[4] = {b->cs.tot, b->cs.ela, b->cs.exc, b->cs.ion};
  for (void* p : tables)
    if (p) cudaFreeAsync(p, b->stream);
  for (int w = 0; w < 3; w++)
    if (b->tile_sched[w]) cudaFreeAsync(b->tile_sched[w], b->stream);
  if (b->stream) {
    cudaStreamSynchronize(b->stream);
    cudaStreamDestroy(b->stream);
  }
  delete b;
}

epic_status epic_batch_initial_field(epic_batch* b) {
  if (!b) return bfail(EPIC_ERR_INVALID, "null batch");
  for (int r = 0; r < b->nruns; r++) {
    const epic_request& q = b->reqs[r];
    const Geom g{q.cfg.nx, q.cfg.ny, q.cfg.x0, q.cfg.y0, q.cfg.dx, q.cfg.dy, 0, 0};
    if (q.num_conductors) {
      // the host loader, as epic_load_particles with load_seed: Init's mt19937
      // stream continued across the species, positions inside a conductor
      // drawn again (the device loader does not place particles around them)
      RefStream* rs = ref_stream_create((uint32_t)q.load_seed);
      epic_status st = EPIC_OK;
      for (int s = 0; s < b->nsp && !st; s++) {
        std::vector<double> parts;
        std::string err;
        const long long n = b->pn[(size_t)r * b->nsp + s];
        if (int e = load_species(q.cfg, q.species[s], parts, rs, err, b->conductors[r])) {
          st = bfail((epic_status)e, "run %d: %s", r, err.c_str());
        } else if ((long long)(parts.size() / 5) != n) {
          st = bfail(EPIC_ERR_INVALID, "run %d: the loader gave %lld particles", r, (long long)(parts.size() / 5));
        } else if (n) {
          cudaError_t ce = cudaMemcpyAsync(b->staging, parts.data(), (size_t)n * 5 * sizeof(double),
                                           cudaMemcpyHostToDevice, b->stream);
          if (ce == cudaSuccess) {
            k_batch_from_aos<<<b->grid, PART_THREADS, 0, b->stream>>>(b->runs[r], b->staging, b->arena[s],
                                                                       b->poff[(size_t)r * b->nsp + s], n, b->flags);
            ce = cudaStreamSynchronize(b->stream);  // parts goes out of scope
          }
          if (ce != cudaSuccess) st = bfail(EPIC_ERR_CUDA, "run %d: load: %s", r, cudaGetErrorString(ce));
        }
      }
      ref_stream_destroy(rs);
      if (st) return st;
      continue;
    }
    for (int s = 0; s < b->nsp; s++) {
      int kind = 0, narg = 0;
      std::string err;
      if (parse_load_type(q.species[s].load, &kind, &narg, err)) return bfail(EPIC_ERR_INVALID, "%s", err.c_str());
      const long long n = b->pn[(size_t)r * b->nsp + s];
      launch_load(b->stream, g, q.species[s], q.cfg, s, kind, narg, b->staging, q.load_seed, b->grid);
      if (n)
        k_batch_from_aos<<<b->grid, PART_THREADS, 0, b->stream>>>(b->runs[r], b->staging, b->arena[s],
                                                                   b->poff[(size_t)r * b->nsp + s], n, b->flags);
    }
  }
  for (int s = 0; s < b->nsp; s++) {
    long long total = 0;
    for (int r = 0; r < b->nruns; r++) total += b->pn[(size_t)r * b->nsp + s];
    launch_set_count(b->stream, b->d_n[s], total);
  }
  epic_status tst = take_flags(b);
  if (tst) return tst;
  if (!b->particles_tuned) {
    if ((tst = tune_particle_passes(b))) return tst;
    b->particles_tuned = true;
  }
  b->deposit_and_solve();
  for (int s = 0; s < b->nsp; s++)
    k_batch_rewind<<<b->grid, PART_THREADS, 0, b->stream>>>(b->d_runs, b->d_node_run, b->arena[s], b->d_n[s],
                                                             b->ef32, s);
  BCK(cudaGetLastError());
  b->step_index = 0;
  return take_flags(b);
}

epic_status epic_batch_run(epic_batch* b, int steps, int use_graph) {
  if (!b || steps < 0) return bfail(EPIC_ERR_INVALID, "bad argument");
  if (b->any_mcc && !b->cs.tot)
    return bfail(EPIC_ERR_INVALID, "cross sections not set (epic_batch_set_log_cross_sections)");
  const bool sorting = b->sort_every > 0;
  if (!use_graph) {
    for (int k = 0; k < steps; k++) {
      b->step(sorting && b->step_index % b->sort_every == 0);
      b->step_index++;
    }
    BCK(cudaGetLastError());
    return take_flags(b);
  }
  auto capture = [&](int sort, cudaGraphExec_t* exec) -> epic_status {
    cudaGraph_t graph;
    BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    b->step(sort);
    cudaError_t ce = cudaStreamEndCapture(b->stream, &graph);
    if (ce != cudaSuccess) {
      cudaGetLastError();
      return bfail(EPIC_ERR_CUDA, "batch graph capture: %s", cudaGetErrorString(ce));
    }
    ce = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return bfail(EPIC_ERR_CUDA, "batch graph instantiate: %s", cudaGetErrorString(ce));
    return EPIC_OK;
  };
  epic_status st;
  if (!b->acc_valid) b->deposit_all();  // the captured steps take the accumulators as deposited
  if (!b->g_plain && (st = capture(0, &b->g_plain))) return st;
  if (sorting && !b->g_sort && (st = capture(1, &b->g_sort))) return st;
  for (int k = 0; k < steps; k++) {
    const bool srt = sorting && b->step_index % b->sort_every == 0;
    b->step_index++;
    BCK(cudaGraphLaunch(srt ? b->g_sort : b->g_plain, b->stream));
  }
  return take_flags(b);
}

epic_status epic_batch_get_particles(epic_batch* b, int run, int s, double* out, int64_t capacity, int64_t* n) {
  if (!b || run < 0 || run >= b->nruns || s < 0 || s >= b->nsp || !out)
    return bfail(EPIC_ERR_INVALID, "bad argument");
  if (!b->any_mcc && !b->has_open && !b->any_emit) {  // counts never change: each run's particles stay where loaded
    const long long cnt = b->pn[(size_t)run * b->nsp + s];
    if (n) *n = cnt;
    if (cnt > capacity)
      return bfail(EPIC_ERR_CAPACITY, "%lld particles do not fit %lld records", cnt, (long long)capacity);
    if (cnt) {
      k_batch_to_aos<<<b->grid, PART_THREADS, 0, b->stream>>>(b->runs[run], b->staging, b->arena[s],
                                                               b->poff[(size_t)run * b->nsp + s], cnt);
      BCK(cudaGetLastError());
      BCK(cudaMemcpyAsync(out, b->staging, (size_t)cnt * 5 * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    }
    BCK(cudaStreamSynchronize(b->stream));
    return EPIC_OK;
  }
  const int tiles = (int)((b->cap[s] + EXTRACT_TILE - 1) / EXTRACT_TILE);
  unsigned int* d_counts = nullptr;
  BCK(cudaMallocAsync((void**)&d_counts, (size_t)tiles * sizeof(unsigned int), b->stream));
  k_batch_count_run<<<tiles, 256, 0, b->stream>>>(b->d_node_run, b->arena[s], b->d_n[s], run, d_counts);
  std::vector<unsigned int> counts(tiles);
  BCK(cudaMemcpyAsync(counts.data(), d_counts, (size_t)tiles * sizeof(unsigned int), cudaMemcpyDeviceToHost,
                      b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  long long total = 0;
  for (auto& c : counts) {
    const unsigned int v = c;
    c = (unsigned int)total;
    total += v;
  }
  if (n) *n = total;
  if (total > capacity) {
    cudaFreeAsync(d_counts, b->stream);
    return bfail(EPIC_ERR_CAPACITY, "%lld particles do not fit %lld records", total, (long long)capacity);
  }
  double* d_out = nullptr;
  BCK(cudaMallocAsync((void**)&d_out, (size_t)std::max<long long>(total, 1) * 5 * sizeof(double), b->stream));
  BCK(cudaMemcpyAsync(d_counts, counts.data(), (size_t)tiles * sizeof(unsigned int), cudaMemcpyHostToDevice,
                      b->stream));
  k_batch_gather_run<<<tiles, 256, 0, b->stream>>>(b->runs[run], run, b->d_node_run, b->arena[s], b->d_n[s], d_counts,
                                                   d_out);
  BCK(cudaGetLastError());
  if (total) BCK(cudaMemcpyAsync(out, d_out, (size_t)total * 5 * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  cudaFreeAsync(d_out, b->stream);
  cudaFreeAsync(d_counts, b->stream);
  BCK(cudaStreamSynchronize(b->stream));
  return EPIC_OK;
}

epic_status epic_batch_get_grid(epic_batch* b, int run, int which, double* out) {
  if (!b || run < 0 || run >= b->nruns || !out) return bfail(EPIC_ERR_INVALID, "bad argument");
  const double* src = which == EPIC_GRID_PHI ? b->phi : which == EPIC_GRID_RHO ? b->rho : nullptr;
  if (!src) return bfail(EPIC_ERR_INVALID, "batches keep phi and rho");
  const BRun& r = b->runs[run];
  BCK(cudaMemcpyAsync(out, src + r.node_off, (size_t)r.nx * r.ny * sizeof(double), cudaMemcpyDeviceToHost,
                      b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return EPIC_OK;
}

epic_status epic_batch_num_particles(epic_batch* b, int64_t* total) {
  if (!b || !total) return bfail(EPIC_ERR_INVALID, "bad argument");
  int64_t t = 0;
  for (int s = 0; s < b->nsp; s++) {
    long long v = 0;
    BCK(cudaMemcpyAsync(&v, b->d_n[s], sizeof(v), cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaStreamSynchronize(b->stream));
    t += v;
  }
  *total = t;
  return EPIC_OK;
}

epic_status epic_batch_set_log_cross_sections(epic_batch* b, const double* ela, const double* exc, const double* ion,
                                              int64_t n, double e_min, double e_max) {
  if (!b || !ela || !exc || !ion || n < 2 || !(e_min > 0) || !(e_max > e_min))
    return bfail(EPIC_ERR_INVALID, "bad argument");
  // The single run's table (epic_set_log_cross_sections) for the batch's gas density.
  std::vector<double> tot(n);
  for (int64_t i = 0; i < n; i++) tot[i] = (ela[i] + exc[i] + ion[i]) * b->gas_density;
  double** dst[4] = {&b->cs.tot, &b->cs.ela, &b->cs.exc, &b->cs.ion};
  const double* src[4] = {tot.data(), ela, exc, ion};
  for (int k = 0; k < 4; k++) {
    if (*dst[k]) cudaFreeAsync(*dst[k], b->stream);
    *dst[k] = nullptr;
    BCK(cudaMallocAsync((void**)dst[k], (size_t)n * sizeof(double), b->stream));
    BCK(cudaMemcpyAsync(*dst[k], src[k], (size_t)n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  }
  CrossSections& cs = b->cs;
  cs.n = n;
  cs.kind = 1;
  cs.e_min = e_min;
  cs.e_max = e_max;
  cs.log_emin = log(e_min);
  cs.inv_dlog = (n - 1) / (log(e_max) - log(e_min));
  double mx = 0;
  for (int64_t i = 0; i + 1 < n; i++) {
    double e1 = exp(log(e_min) + (i + 1) / cs.inv_dlog);
    mx = std::max(mx, std::max(tot[i], tot[i + 1]) * sqrt(2.0 * e1 * EV / ME));
  }
  mx = std::max(mx, tot[n - 1] * sqrt(2.0 * 4 * e_max * EV / ME));
  cs.nu_max = mx;
  for (BRun& r : b->runs) {  // the single run's early-out bound (launch_mcc)
    const double p_null = 1 - exp(-cs.nu_max * r.dt_phys);
    r.p_cut = fmin(1.0, p_null * (1 + 1e-9) + 1e-300);
    r.cut53 = (unsigned long long)ceil(r.p_cut * 9007199254740992.0);
  }
  BCK(cudaMemcpyAsync(b->d_runs, b->runs.data(), b->runs.size() * sizeof(BRun), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  // captured steps hold the old table
  if (b->g_plain) cudaGraphExecDestroy(b->g_plain);
  if (b->g_sort) cudaGraphExecDestroy(b->g_sort);
  b->g_plain = b->g_sort = nullptr;
  return EPIC_OK;
}

epic_status epic_batch_tuning(epic_batch* b, int tiles[4]) {
  if (!b || !tiles) return bfail(EPIC_ERR_INVALID, "bad argument");
  std::memcpy(tiles, b->tiles, sizeof(b->tiles));
  return EPIC_OK;
}

epic_status epic_batch_set_profiling(epic_batch* b, int enable) {
  if (!b) return bfail(EPIC_ERR_INVALID, "null batch");
  b->profiling = enable != 0;
  return EPIC_OK;
}

epic_status epic_batch_get_profile(epic_batch* b, double ms[7], int64_t counts[7]) {
  if (!b) return bfail(EPIC_ERR_INVALID, "null batch");
  BCK(cudaStreamSynchronize(b->stream));
  for (auto& pe : b->prof_pending) {
    float t = 0;
    BCK(cudaEventElapsedTime(&t, pe.second.first, pe.second.second));
    b->prof_ms[pe.first] += t;
    b->prof_count[pe.first] += 1;
    b->event_pool.push_back(pe.second.first);
    b->event_pool.push_back(pe.second.second);
  }
  b->prof_pending.clear();
  for (int k = 0; k < 7; k++) {
    if (ms) ms[k] = b->prof_ms[k];
    if (counts) counts[k] = b->prof_count[k];
    b->prof_ms[k] = 0;
    b->prof_count[k] = 0;
  }
  return EPIC_OK;
}

epic_status epic_batch_particle_tuning(epic_batch* b, int shapes[4], float push_ms[5], float deposit_ms[6]) {
  if (!b || !shapes) return bfail(EPIC_ERR_INVALID, "bad argument");
  shapes[0] = b->push_threads;
  shapes[1] = b->push_blocks;
  shapes[2] = b->dep_threads;
  shapes[3] = b->dep_blocks;
  if (push_ms) std::memcpy(push_ms, b->push_ms, sizeof(b->push_ms));
  if (deposit_ms) std::memcpy(deposit_ms, b->dep_ms, sizeof(b->dep_ms));
  return EPIC_OK;
}

void* epic_batch_stream(epic_batch* b) { return b ? (void*)b->stream : nullptr; }

}  // extern "C"
