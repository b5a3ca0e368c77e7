// Device descriptors of a batch of runs (include/epic2d_batch.h), shared by
// the batch's kernel files.
#pragma once

#include "epic_internal.cuh"

namespace epic {

constexpr int BATCH_MAX_SPECIES = 4;

// One run of the batch: its grid lives at node_off .. node_off + nx*ny of the
// batch's node arrays (node (i, j) at node_off + i*ny + j).
struct BRun {
  int nx, ny, bc;
  long long node_off;
  double x0, y0, dx, dy;
  float qmK_dt[BATCH_MAX_SPECIES], hqmK_dt[BATCH_MAX_SPECIES], cx, cy;
  double spwt[BATCH_MAX_SPECIES], charge_over_qe[BATCH_MAX_SPECIES];
  double div, inv_scale, K, tol;
  // spectral lattice: R x C entries at lat_off of the lattice pools, its
  // transforms at qR_off / qC_off of the transform pool, D at lat_off
  int R, C, flat, gs_norm;
  long long lat_off, qR_off, qC_off;
  int chunk_off;  // first residual chunk slot
};

struct BatchGrids {
  int nruns, nsp;
  long long nodes;
  const BRun* runs;
  const int* node_run;  // run of every node
  double *phi, *rho, *efx, *efy;
  float2* ef32;
  const unsigned long long* acc[BATCH_MAX_SPECIES];
};

void launch_batch_finalize(cudaStream_t st, const BatchGrids& b);
void launch_batch_efield(cudaStream_t st, const BatchGrids& b);

}  // namespace epic
