// Per-node arithmetic of the density finalisation and the E-field, shared by
// the single-run kernels (epic_field.cu) and the batched ones
// (epic_batch_grid.cu); both files are compiled with -fmad=false, so the two
// round identically.
#pragma once

#include "epic_internal.cuh"

namespace epic {

// The tail of Species::ScatterSpecies_serial (src/species.cpp:188-225) at node
// (i, j): raw(i, j) is the normalised deposit D = raw/div; pbc folds
// Y(i,j) = D(i,0)+D(i,ny-1) on j edges, then X(i,j) = Y(0,j)+Y(nx-1,j) on i
// edges; open/reflective scale edges by 0.5 and corners by 0.25.
template <class Raw>
__device__ __forceinline__ double fold_density(int bc, int nx, int ny, const Raw& raw, int i, int j) {
  auto fold_y = [&](int ii, int jj) {
    if (jj == 0 || jj == ny - 1) return raw(ii, 0) + raw(ii, ny - 1);
    return raw(ii, jj);
  };
  double v;
  if (bc == EPIC_PBC) {
    if (i == 0 || i == nx - 1) v = fold_y(0, j) + fold_y(nx - 1, j);
    else v = fold_y(i, j);
  } else {
    v = raw(i, j);
    const bool ei = (i == 0 || i == nx - 1), ej = (j == 0 || j == ny - 1);
    if (ei && ej) v *= 0.25;
    else if (ei || ej) v *= 0.5;
  }
  return v;
}

// Edge rule of the E-field per direction: EPIC_PBC (periodic central
// difference through node n-2), EPIC_OPEN (one-sided), or none.  The
// reference takes both from bc (src/field.cpp:289-329); with a Poisson
// extension they follow the field's boundary: periodic directions take the
// periodic rule, the x walls of DIRICHLET_X the one-sided one.
__host__ __device__ inline void efield_edges(int bc, int poisson_bc, int* xr, int* yr) {
  const int ref = bc == EPIC_PBC ? EPIC_PBC : (bc == EPIC_OPEN || bc == EPIC_REFLECTIVE) ? EPIC_OPEN : -1;
  *xr = *yr = ref;
  if (poisson_bc == EPIC_POISSON_PERIODIC) *xr = *yr = EPIC_PBC;
  else if (poisson_bc == EPIC_POISSON_DIRICHLET_X) {
    *xr = EPIC_OPEN;
    *yr = EPIC_PBC;
  }
}

// FieldSolve::CalculateEfield (src/field.cpp:276-330) at node (i, j) with the
// edge rules xr, yr (efield_edges); phi(a, b) reads the potential; ex, ey
// come in holding the previous values (kept where no rule applies).
template <class Phi>
__device__ __forceinline__ void efield_node(int xr, int yr, int nx, int ny, double dx, double dy, const Phi& PHI, int i,
                                            int j, double& ex, double& ey) {
  if (i >= 1 && i < nx - 1) ex = -(PHI(i + 1, j) - PHI(i - 1, j)) / (2 * dx);
  else if (xr == EPIC_OPEN) {
    if (i == 0) ex = -(PHI(1, j) - PHI(0, j)) / dx;
    else ex = -(PHI(nx - 1, j) - PHI(nx - 2, j)) / dx;
  } else if (xr == EPIC_PBC) {
    ex = -(PHI(1, j) - PHI(nx - 2, j)) / (2 * dx);
  }
  if (j >= 1 && j < ny - 1) ey = -(PHI(i, j + 1) - PHI(i, j - 1)) / (2 * dy);
  else if (yr == EPIC_OPEN) {
    if (j == 0) ey = -(PHI(i, 1) - PHI(i, 0)) / dy;
    else ey = -(PHI(i, ny - 1) - PHI(i, ny - 2)) / dy;
  } else if (yr == EPIC_PBC) {
    ey = -(PHI(i, 1) - PHI(i, ny - 2)) / (2 * dy);
  }
}

}  // namespace epic
