// Per-particle arithmetic of the mixed-precision form (gather, push, boundary
// rules), shared by the single-run kernels (epic_mixed.cu) and the batched
// kernels (epic_batch.cu), which must compute bit-identical particles.  Both
// files are compiled with the same flags (FP32 contraction allowed).  Also the
// chunked deposit of cell-sorted particles (epic_mixed.cu, epic_sort.cu).
#pragma once

#include <climits>

#include "epic_internal.cuh"

namespace epic {

// Species::Push_species_serial (src/species.cpp:29-170) in cell units:
//   v += (qm*K*DT) E;  offset += (vel_norm/(L*W)) * DT / dx * v;
// then whole cells are carried from the offset into the cell index and the
// boundary rule applied to the cell.  Periodic wrap is a modulo, so a
// particle may cross any number of cells in a step.
template <int SHAPE>
__device__ __forceinline__ void gather32(const Geom& g, const float2* __restrict__ ef, int c, float ox, float oy,
                                         float& ex, float& ey) {
  if (SHAPE == EPIC_NGP) {
    const int k = c + (ox >= 0.5f ? g.ny : 0) + (oy >= 0.5f ? 1 : 0);
    const float2 f = __ldg(&ef[k]);
    ex = f.x;
    ey = f.y;
    return;
  }
  const float2 f00 = __ldg(&ef[c]), f01 = __ldg(&ef[c + 1]);
  const float2 f10 = __ldg(&ef[c + g.ny]), f11 = __ldg(&ef[c + g.ny + 1]);
  const float w00 = (1.f - ox) * (1.f - oy), w10 = ox * (1.f - oy), w01 = (1.f - ox) * oy, w11 = ox * oy;
  ex = f00.x * w00 + f10.x * w10 + f01.x * w01 + f11.x * w11;
  ey = f00.y * w00 + f10.y * w10 + f01.y * w01 + f11.y * w11;
}

// The largest FP32 offset below 1: a particle inside the domain whose offset
// in the last cell rounds up to 1 stays there, 2^-24 cell from the wall.
constexpr float MAX_OFFSET = 0x1.fffffep-1f;

// A position in cell units (FP64, from the domain's origin) as a cell index and
// an FP32 offset in [0, 1).  An offset that rounds up to 1 carries into the
// next cell, except in the last cell.  Returns false for a position outside
// [0, ncell); the index is then clamped into the grid.
__device__ __forceinline__ bool cell_offset(double l, int ncell, int& idx, float& o) {
  const double f = floor(l);
  int i = (int)f;
  o = (float)(l - f);
  if (o >= 1.f) {
    if (i + 1 < ncell) {
      o = 0.f;
      i++;
    } else {
      o = MAX_OFFSET;
    }
  }
  const bool in = i >= 0 && i < ncell;
  idx = min(max(i, 0), ncell - 1);
  return in;
}

// c = i * ny + j, 0 <= c < 2^31, 0 < ny: (i, j) with a multiply-high
// (m = floor((2^32 - 1) / ny) underestimates 1/ny by less than 2^-32, so the
// quotient is exact or one short) in place of an integer division.
__device__ __forceinline__ void split_cell(int c, int ny, int& i, int& j) {
  const unsigned m = 0xFFFFFFFFu / (unsigned)ny;  // loop-invariant
  unsigned q = __umulhi((unsigned)c, m);
  int r = c - (int)q * ny;
  if (r >= ny) {
    q++;
    r -= ny;
  }
  i = (int)q;
  j = r;
}

// Moves (cell index, offset) along one axis by `d` cells and applies the
// boundary rule.  Returns false if the particle leaves an open boundary.
template <int BC>
__device__ __forceinline__ bool advance(int& idx, float& o, float& v, float d, int ncell) {
  o += d;
  const float f = floorf(o);
  o -= f;
  idx += (int)f;
  if (o >= 1.f) {  // o was a tiny negative number
    o = 0.f;
    idx += 1;
  }
  if (BC == EPIC_PBC) {
    if (idx < 0 || idx >= ncell) {
      idx %= ncell;
      if (idx < 0) idx += ncell;
    }
    return true;
  } else if (BC == EPIC_OPEN) {
    return idx >= 0 && idx < ncell;
  } else {
    if (idx < 0 || idx >= ncell) {
      // mirror the position about the wall it crossed, flip the velocity
      float pos = (float)idx + o;
      pos = idx < 0 ? -pos : 2.f * ncell - pos;
      const float fl = floorf(pos);
      idx = (int)fl;
      o = pos - fl;
      if (o >= 1.f) {
        o = 0.f;
        idx += 1;
      }
      if (idx >= ncell) {  // mirrored onto the far wall itself: the last offset inside
        idx = ncell - 1;
        o = MAX_OFFSET;
      }
      idx = max(idx, 0);
      v = -v;
    }
    return true;
  }
}

template <int SHAPE, int BC>
__device__ __forceinline__ bool push_mixed_one(const Geom& g, const float2* __restrict__ ef, float qmK_dt, float cx,
                                               float cy, int& c, float& ox, float& oy, float& vx, float& vy) {
  float ex, ey;
  gather32<SHAPE>(g, ef, c, ox, oy, ex, ey);
  vx = fmaf(qmK_dt, ex, vx);
  vy = fmaf(qmK_dt, ey, vy);
  int i, j;
  split_cell(c, g.ny, i, j);
  bool keep = advance<BC>(i, ox, vx, cx * vx, g.nx - 1);
  keep = advance<BC>(j, oy, vy, cy * vy, g.ny - 1) && keep;
  c = i * g.ny + j;
  return keep;
}

// ------------------------------------------ deposit of a sorted chunk ---
// CIC deposit (integer weights, Domain::Scatter, src/domain.cpp:205-228) of a
// warp's DEP_WARP_CHUNK consecutive particles, sorted by cell (or nearly so,
// between sorts), DEP_PER_THREAD consecutive particles per lane.
//
// A particle's weights come from its offsets quantised to 2^-20 of a cell,
// a, b in [0, S), S = 2^20: (S-a)(S-b), a(S-b), (S-a)b, ab on the cell's four
// nodes.  Summed over the particles of one cell they are fixed by five exact
// integer moments — count N, A = sum a, B = sum b and AB = sum ab (two 20-bit
// limbs) — as
//   w00 = N S^2 - S (A + B) + AB,  w10 = S A - AB,  w01 = S B - AB,  w11 = AB.
// Each lane merges runs of equal cells among its particles in registers and
// adds each run's moments with 32-bit shared-memory atomics to a slot of the
// warp's own table (a hash of the cell), which the first run in that cell
// claims (a tag) and lists; a run whose slot another cell holds adds its node
// weights straight to the grid.  Then the lanes add each listed cell's four
// node weights to the grid and free the slots.  The warp's sums stay below
// 2^31.  Only the warp synchronises.  Integer sums: the result does not depend
// on the grouping and equals the per-particle deposit.
constexpr int DEP_PER_THREAD = 8;
constexpr int DEP_WARP_CHUNK = 32 * DEP_PER_THREAD;
constexpr int DEP_CHUNK = PART_THREADS * DEP_PER_THREAD;  // a CTA's particles per round
constexpr int DEP_SLOTS = 128;                            // per warp
constexpr unsigned DEP_LIMB = (1u << 20) - 1;

struct DepWarp {
  unsigned n[DEP_SLOTS], a[DEP_SLOTS], b[DEP_SLOTS], ab_lo[DEP_SLOTS], ab_hi[DEP_SLOTS];
  int tag[DEP_SLOTS];                  // cell held by the slot, -1 free
  unsigned char list[DEP_SLOTS];       // slots claimed in this chunk
  int count;                           // list length
};

// Before the warp's first chunk.
__device__ __forceinline__ void dep_init(DepWarp& w) {
  const int lane = threadIdx.x & 31;
  for (int m = lane; m < DEP_SLOTS; m += 32) {
    w.n[m] = w.a[m] = w.b[m] = w.ab_lo[m] = w.ab_hi[m] = 0;
    w.tag[m] = -1;
  }
  if (lane == 0) w.count = 0;
  __syncwarp();
}

__device__ __forceinline__ void dep_node_weights(unsigned long long* __restrict__ acc, int ny, int c, unsigned N,
                                                 unsigned A, unsigned B, unsigned ab_lo, unsigned ab_hi) {
  constexpr unsigned long long S = 1ull << MIXED_OFFSET_BITS;
  const unsigned long long AB = ((unsigned long long)ab_hi << 20) + ab_lo;
  atomicAdd(&acc[c], (unsigned long long)N * S * S - S * ((unsigned long long)A + B) + AB);  // modulo 2^64
  atomicAdd(&acc[c + ny], S * A - AB);
  atomicAdd(&acc[c + 1], S * B - AB);
  atomicAdd(&acc[c + ny + 1], AB);
}

// The row stride (nodes per grid row) of a cell's grid: one grid, or a batch's
// runs laid end to end (the stride of the run that holds the cell).
struct ConstNy {
  int ny;
  __device__ __forceinline__ int operator()(int) const { return ny; }
};

template <class NY>
__device__ __forceinline__ void dep_run(unsigned long long* __restrict__ acc, DepWarp& w, const NY& ny_of, int c,
                                        unsigned N, unsigned A, unsigned B, unsigned ab_lo, unsigned ab_hi) {
  if (c < 0) return;
  const int m = (int)(((unsigned)c * 0x9E3779B1u) >> 25);  // 7-bit multiplicative hash
  int t = *(volatile int*)&w.tag[m];
  if (t != c) {
    if (t == -1) {
      t = atomicCAS(&w.tag[m], -1, c);
      if (t == -1) {
        w.list[atomicAdd(&w.count, 1)] = (unsigned char)m;
        t = c;
      }
    }
    if (t != c) {
      dep_node_weights(acc, ny_of(c), c, N, A, B, ab_lo, ab_hi);
      return;
    }
  }
  atomicAdd(&w.n[m], N);
  atomicAdd(&w.a[m], A);
  atomicAdd(&w.b[m], B);
  atomicAdd(&w.ab_lo[m], ab_lo);
  atomicAdd(&w.ab_hi[m], ab_hi);
}

// Every lane of the warp calls this once per chunk with its particles
// (c[k] < 0: no particle); ny_of(cell) gives the cell's row stride.
template <class NY>
__device__ __forceinline__ void deposit_warp_sorted(unsigned long long* __restrict__ acc, DepWarp& w, const NY& ny_of,
                                                    const int (&c)[DEP_PER_THREAD],
                                                    const float (&ox)[DEP_PER_THREAD],
                                                    const float (&oy)[DEP_PER_THREAD]) {
  static_assert(DEP_SLOTS == 128, "the hash yields 7 bits");
  const float fS = (float)(1 << MIXED_OFFSET_BITS);
  const int lane = threadIdx.x & 31;
  int cur = -1;
  unsigned N = 0, A = 0, B = 0, L = 0, H = 0;
#pragma unroll
  for (int k = 0; k < DEP_PER_THREAD; k++) {
    if (c[k] < 0) continue;
    const unsigned a = (unsigned)(int)(ox[k] * fS), b = (unsigned)(int)(oy[k] * fS);
    const unsigned long long ab = (unsigned long long)a * b;
    if (c[k] != cur) {
      dep_run(acc, w, ny_of, cur, N, A, B, L, H);
      cur = c[k];
      N = 0; A = 0; B = 0; L = 0; H = 0;
    }
    N += 1;
    A += a;
    B += b;
    L += (unsigned)ab & DEP_LIMB;
    H += (unsigned)(ab >> 20);
  }
  dep_run(acc, w, ny_of, cur, N, A, B, L, H);
  __syncwarp();
  const int cnt = *(volatile int*)&w.count;
  __syncwarp();
  if (lane == 0) w.count = 0;  // every lane has read it; the next appends follow the last __syncwarp
  for (int e = lane; e < cnt; e += 32) {
    const int m = w.list[e];
    const int cm = w.tag[m];
    dep_node_weights(acc, ny_of(cm), cm, w.n[m], w.a[m], w.b[m], w.ab_lo[m], w.ab_hi[m]);
    w.n[m] = w.a[m] = w.b[m] = w.ab_lo[m] = w.ab_hi[m] = 0;
    w.tag[m] = -1;
  }
  __syncwarp();
}

}  // namespace epic
