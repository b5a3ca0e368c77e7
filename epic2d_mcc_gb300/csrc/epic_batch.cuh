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
  // MCC (species 0 against the gas, ions into species 1) when mcc != 0: the
  // single run's parameters (launch_mcc), Philox keyed by this run's seed
  int mcc;
  double vn, dt_phys, ion_mass, ion_temp, F1, F2, p_cut;
  unsigned long long cut53, seed;
  // conductors (src/grid.cpp, src/electrode.cpp): rectangles and electrodes
  // at rect_off / circ_off of the batch's conductor tables (BatchConductors)
  int nrect, ncirc, rect_off, circ_off;
};

// The conductors of every run: rectangles {min_x, max_x, min_y, max_y},
// electrodes {x, y, r*r, 0}, and per run whether its electrodes exist yet (a
// CircularGrid has none until the first SOR solve's Grid::initialize).
struct BatchConductors {
  const double4* rect;
  const double4* circ;
  const int* live;
};

// One emitter of one run feeding one species (e.slot 0: its species_idx1, 1:
// species_idx2): its points go to records off .. off + e.num past the
// species' live count, Philox keyed by the run's configuration seed (as the
// run alone).
struct BEmit {
  EmitDev e;
  unsigned long long seed;
  long long off;
  int run;
};

struct McEvents;
struct CrossSections;
// Electron-neutral MCC of every run with mcc != 0, one launch sequence for the
// batch (epic_mcc.cu).
void launch_batch_mcc(cudaStream_t st, const CrossSections& cs, const BRun* runs, const int* node_run,
                      const MixedSoA& e, long long* d_ne, long long e_cap, const MixedSoA& ion, long long* d_ni,
                      long long i_cap, unsigned long long* d_step, const McEvents& ev, unsigned long long* d_ncoll,
                      int* flags, int grid, int skip_select = 0);

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
