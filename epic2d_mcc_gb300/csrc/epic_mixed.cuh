// Per-particle arithmetic of the mixed-precision form (gather, push, boundary
// rules), shared by the single-run kernels (epic_mixed.cu) and the batched
// kernels (epic_batch.cu), which must compute bit-identical particles.  Both
// files are compiled with the same flags (FP32 contraction allowed).
#pragma once

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
      idx = min(max(idx, 0), ncell - 1);
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
  int i = c / g.ny, j = c - i * g.ny;
  bool keep = advance<BC>(i, ox, vx, cx * vx, g.nx - 1);
  keep = advance<BC>(j, oy, vy, cy * vy, g.ny - 1) && keep;
  c = i * g.ny + j;
  return keep;
}


}  // namespace epic
