// Grid kernels of a batch (density finalisation + charge density, E-field):
// one thread per node of the batch's node space, each node computed with its
// run's geometry and constants by the single-run formulas (epic_grid.cuh).
// Built with -fmad=false like epic_field.cu, so each run's grids round as they
// would alone.
#include <cuda_runtime.h>

#include "epic_batch.cuh"
#include "epic_grid.cuh"

namespace epic {

__global__ void k_batch_finalize(BatchGrids b) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < b.nodes;
       k += (long long)gridDim.x * blockDim.x) {
    const BRun& r = b.runs[b.node_run[k]];
    const int nx = r.nx, ny = r.ny;
    const int kl = (int)(k - r.node_off);
    const int i = kl / ny, j = kl - i * ny;
    double rho = 0;
    for (int s = 0; s < b.nsp; s++) {
      const unsigned long long* acc = b.acc[s] + r.node_off;
      auto raw = [&](int ii, int jj) {
        const double v = ((double)(long long)acc[ii * ny + jj] * r.inv_scale) * r.spwt[s];
        return v / r.div;
      };
      const double v = fold_density(r.bc, nx, ny, raw, i, j);
      const double t = v * r.charge_over_qe[s];
      rho = rho + t;
    }
    b.rho[k] = rho;
  }
}

__global__ void k_batch_efield(BatchGrids b) {
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < b.nodes;
       k += (long long)gridDim.x * blockDim.x) {
    const BRun& r = b.runs[b.node_run[k]];
    const int nx = r.nx, ny = r.ny;
    const int kl = (int)(k - r.node_off);
    const int i = kl / ny, j = kl - i * ny;
    const double* phi = b.phi + r.node_off;
    double ex = b.efx[k], ey = b.efy[k];
    auto PHI = [&](int a_, int b_) { return phi[a_ * ny + b_]; };
    int xr, yr;
    efield_edges(r.bc, EPIC_POISSON_DIRICHLET, &xr, &yr);
    efield_node(xr, yr, nx, ny, r.dx, r.dy, PHI, i, j, ex, ey);
    b.efx[k] = ex;
    b.efy[k] = ey;
    b.ef32[k] = make_float2((float)ex, (float)ey);
  }
}

void launch_batch_finalize(cudaStream_t st, const BatchGrids& b) {
  k_batch_finalize<<<(int)((b.nodes + 255) / 256), 256, 0, st>>>(b);
}

void launch_batch_efield(cudaStream_t st, const BatchGrids& b) {
  k_batch_efield<<<(int)((b.nodes + 255) / 256), 256, 0, st>>>(b);
}

}  // namespace epic
