// Grid kernels of the FP64 plain form: density finalisation + charge density,
// the two SOR solvers and the PCG solver of FieldSolve, the E-field, and the
// potential-energy / max-phi reductions.
//
// Built with -fmad=false so every expression rounds as the reference's does.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "epic_internal.cuh"

namespace epic {

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// ------------------------------------------------------- finalisation ---
// The tail of Species::ScatterSpecies_serial (src/species.cpp:188-225) for
// every species, then Domain::ComputeRho (src/domain.cpp:194-202), one thread
// per node, reading the deposit accumulators and writing the density grids.  A node on an edge recomputes the (identical) values of the nodes
// it is folded with, so the fold needs no second pass:
//   D = raw/div;  pbc: Y(i,j) = D(i,0)+D(i,ny-1) on j edges, then
//   X(i,j) = Y(0,j)+Y(nx-1,j) on i edges;  open/reflective: edges x0.5,
//   corners x0.25.
__device__ __forceinline__ double raw_den(const FinalizeArgs& a, int s, int i, int j) {
  long k = (long)i * a.g.ny + j;
  double v;
  if (a.fixed) v = ((double)(long long)a.acc[s][k] * a.inv_scale[s]) * a.spwt[s];
  else v = reinterpret_cast<const double*>(a.acc[s])[k];
  return v / a.div;
}

__device__ __forceinline__ double fold_y(const FinalizeArgs& a, int s, int i, int j) {
  const int ny = a.g.ny;
  if (j == 0 || j == ny - 1) return raw_den(a, s, i, 0) + raw_den(a, s, i, ny - 1);
  return raw_den(a, s, i, j);
}

__global__ void k_finalize(FinalizeArgs a) {
  const int nx = a.g.nx, ny = a.g.ny;
  const long nn = (long)nx * ny;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += (long)gridDim.x * blockDim.x) {
    const int i = (int)(k / ny), j = (int)(k % ny);
    double vals[8];
    for (int s = 0; s < a.nsp; s++) {
      double v;
      if (a.stage == RHO_FROM_DEN || !a.active[s]) {
        vals[s] = a.den[s][k];
        continue;
      }
      if (a.bc == EPIC_PBC) {
        if (i == 0 || i == nx - 1) v = fold_y(a, s, 0, j) + fold_y(a, s, nx - 1, j);
        else v = fold_y(a, s, i, j);
      } else {
        v = raw_den(a, s, i, j);
        bool ei = (i == 0 || i == nx - 1), ej = (j == 0 || j == ny - 1);
        if (ei && ej) v *= 0.25;
        else if (ei || ej) v *= 0.5;
      }
      vals[s] = v;
    }
    double rho = 0;
    for (int s = 0; s < a.nsp; s++) {
      if (a.stage != RHO_FROM_DEN && a.active[s]) a.den[s][k] = vals[s];
      double t = vals[s] * a.charge_over_qe[s];
      rho = rho + t;
    }
    if (a.stage != FINALIZE_ONLY) a.rho[k] = rho;
  }
}

void launch_finalize(cudaStream_t st, const FinalizeArgs& a) {
  // Reads only the accumulators (int64 fixed point, or FP64 sums stored in the
  // same buffer) and writes the density grids, so every node is independent.
  long nn = (long)a.g.nx * a.g.ny;
  int blocks = (int)((nn + 255) / 256);
  k_finalize<<<blocks, 256, 0, st>>>(a);
}

// ------------------------------------------------------------ E-field ---
// FieldSolve::CalculateEfield (src/field.cpp:276-330).
__global__ void k_efield(Geom g, int bc, const double* __restrict__ phi, double* efx, double* efy, double2* ef) {
  const int nx = g.nx, ny = g.ny;
  const long nn = (long)nx * ny;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += (long)gridDim.x * blockDim.x) {
    const int i = (int)(k / ny), j = (int)(k % ny);
    double ex = efx[k], ey = efy[k];
#define PHI(a, b) phi[(long)(a) * ny + (b)]
    if (i >= 1 && i < nx - 1) ex = -(PHI(i + 1, j) - PHI(i - 1, j)) / (2 * g.dx);
    else if (bc == EPIC_OPEN || bc == EPIC_REFLECTIVE) {
      if (i == 0) ex = -(PHI(1, j) - PHI(0, j)) / g.dx;
      else ex = -(PHI(nx - 1, j) - PHI(nx - 2, j)) / g.dx;
    } else if (bc == EPIC_PBC) {
      ex = -(PHI(1, j) - PHI(nx - 2, j)) / (2 * g.dx);
    }
    if (j >= 1 && j < ny - 1) ey = -(PHI(i, j + 1) - PHI(i, j - 1)) / (2 * g.dy);
    else if (bc == EPIC_OPEN || bc == EPIC_REFLECTIVE) {
      if (j == 0) ey = -(PHI(i, 1) - PHI(i, 0)) / g.dy;
      else ey = -(PHI(i, ny - 1) - PHI(i, ny - 2)) / g.dy;
    } else if (bc == EPIC_PBC) {
      ey = -(PHI(i, 1) - PHI(i, ny - 2)) / (2 * g.dy);
    }
#undef PHI
    efx[k] = ex;
    efy[k] = ey;
    ef[k] = make_double2(ex, ey);
  }
}

void launch_efield(cudaStream_t st, const Geom& g, int bc, const double* phi, double* efx, double* efy, double2* ef) {
  long nn = (long)g.nx * g.ny;
  int blocks = (int)((nn + 255) / 256);
  k_efield<<<blocks, 256, 0, st>>>(g, bc, phi, efx, efy, ef);
}

// ------------------------------------------------- lexicographic SOR ---
// FieldSolve::gssolver (src/field.cpp:70-139) with its exact iterates.
// Lexicographic Gauss-Seidel (i outer, j inner) updates node (i,j) from the
// new (i-1,j), (i,j-1) and the old (i+1,j), (i,j+1); all interior nodes on
// one anti-diagonal d = (i-1)+(j-1) are independent.  Sweep s of a chunk
// handles diagonal d at time t = d + 2s, so up to S sweeps run as one
// pipelined wavefront: at any time step the active diagonals are two apart
// and no active node reads another active node.  Residual checks follow the
// reference: after sweeps 0, 25, 50, ... (iter % 25 == 0).
//
// One CTA; phi lives in shared memory when it fits, otherwise in global memory.
constexpr int SOR_THREADS = 1024;

__device__ double block_sum_1024(double v, double* sm) {
  v = warp_sum_d(v);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0;
  if (threadIdx.x < 32) {
    t = sm[threadIdx.x];
    t = warp_sum_d(t);
  }
  __syncthreads();
  if (threadIdx.x == 0) sm[32] = t;
  __syncthreads();
  t = sm[32];
  __syncthreads();
  return t;
}

// Residual of src/field.cpp:121-134 over the interior (one block).
__device__ double sor_residual(const SolverArgs& a, const double* phi, double* red) {
  const int nx = a.g.nx, ny = a.g.ny;
  const double dx2 = a.g.dx * a.g.dx, dy2 = a.g.dy * a.g.dy;
  double sum = 0;
  const long ni = (long)(nx - 2) * (ny - 2);
  for (long q = threadIdx.x; q < ni; q += blockDim.x) {
    int i = 1 + (int)(q / (ny - 2)), j = 1 + (int)(q % (ny - 2));
    long k = (long)i * ny + j;
    double R = ((phi[k + ny] - 2 * phi[k] + phi[k - ny]) / dx2) + ((phi[k + 1] - 2 * phi[k] + phi[k - 1]) / dy2) +
               (a.rho[k]) * a.K;
    sum += R * R;
  }
  sum = block_sum_1024(sum, red);
  return sqrt(sum / (nx * ny));
}

__global__ void __launch_bounds__(SOR_THREADS) k_sor_lex(SolverArgs a, int use_smem) {
  extern __shared__ double smem[];
  __shared__ double red[40];
  const int nx = a.g.nx, ny = a.g.ny;
  const long nn = (long)nx * ny;
  double* phi = use_smem ? smem : a.phi;
  const double dx2 = a.g.dx * a.g.dx, dy2 = a.g.dy * a.g.dy;
  const double coeff = (2 / dx2) + (2 / dy2);
  const double inv_coeff = 1 / coeff;
  for (long k = threadIdx.x; k < nn; k += blockDim.x) phi[k] = 0;  // cold start, zero edges (src/field.cpp:78-98)
  __syncthreads();
  const int nxi = nx - 2, nyi = ny - 2;
  const int D = nxi + nyi - 1;
  const int Lmax = nxi < nyi ? nxi : nyi;
  int iter = 0, converged = 0;
  double L2 = 0;
  if (nxi > 0 && nyi > 0) {
    while (iter < a.max_iter) {
      int S = iter == 0 ? 1 : 25;
      if (S > a.max_iter - iter) S = a.max_iter - iter;
      const int T = D + 2 * (S - 1);
      for (int t = 0; t < T; t++) {
        int s_lo = t - D + 1 > 0 ? (t - D + 2) >> 1 : 0;
        int s_hi = (t >> 1) < S - 1 ? (t >> 1) : S - 1;
        int items = (s_hi - s_lo + 1) * Lmax;
        for (int it = threadIdx.x; it < items; it += blockDim.x) {
          int s = s_lo + it / Lmax, q = it % Lmax;
          int d = t - 2 * s;
          int a0 = d - (nyi - 1) > 0 ? d - (nyi - 1) : 0;
          int a1 = d < nxi - 1 ? d : nxi - 1;
          int ai = a0 + q;
          if (ai > a1) continue;
          int i = ai + 1, j = d - ai + 1;
          long k = (long)i * ny + j;
          double phi_new = inv_coeff * (a.rho[k] * a.K + ((phi[k + ny] + phi[k - ny]) / dx2) +
                                        ((phi[k + 1] + phi[k - 1]) / dy2));
          phi[k] = phi[k] + a.omega * (phi_new - phi[k]);
        }
        __syncthreads();
      }
      const int last = iter + S - 1;
      iter += S;
      if (last % 25 == 0) {
        L2 = sor_residual(a, phi, red);
        if (L2 < a.tol) {
          converged = 1;
          break;
        }
      }
    }
  }
  if (use_smem)
    for (long k = threadIdx.x; k < nn; k += blockDim.x) a.phi[k] = phi[k];
  if (threadIdx.x == 0) {
    a.info->iterations = iter;
    a.info->converged = converged;
    a.info->error = L2;
    atomicAdd(a.iter_total, (unsigned long long)iter);
  }
}

constexpr size_t SOR_SMEM_MAX = 200 * 1024;

void init_field_kernels() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(k_sor_lex, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SOR_SMEM_MAX);
  done = true;
}

void launch_sor_lex(cudaStream_t st, const SolverArgs& a) {
  size_t bytes = (size_t)a.g.nx * a.g.ny * sizeof(double);
  int use_smem = bytes <= SOR_SMEM_MAX;
  k_sor_lex<<<1, SOR_THREADS, use_smem ? bytes : 0, st>>>(a, use_smem);
}

// ------------------------------------------------------ grid barrier ---
// Cooperative launches guarantee that all blocks are resident; the barrier is
// a counter plus a generation word, and every wait gives up after SPIN_LIMIT
// polls (FLAG_TIMEOUT) so a fault can never hang the GPU.
__device__ bool grid_sync(unsigned int* bar, int* flags) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = bar + 1;
    unsigned int g0 = *gen;
    __threadfence();
    unsigned int arrived = atomicAdd(bar, 1u);
    int ok = 1;
    if (arrived == gridDim.x - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long spins = 0;
      while (*gen == g0) {
        if (++spins > SPIN_LIMIT) {
          atomicOr(flags, FLAG_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(20);
      }
    }
    __threadfence();
    s_ok = ok && !(*(volatile int*)flags & FLAG_TIMEOUT);
  }
  __syncthreads();
  return s_ok;
}

// Deterministic grid sum: each block writes a partial, then every block adds
// the partials in the same fixed order and gets the same value.
__device__ double block_sum_256(double v, double* sm) {
  v = warp_sum_d(v);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sm[w];
  __syncthreads();
  return t;  // valid in thread 0
}

__device__ double sum_partials(const double* partials, int n, int stride, int off, double* sm) {
  double t = 0;
  if (threadIdx.x < 32) {
    for (int b = threadIdx.x; b < n; b += 32) t += ((volatile const double*)partials)[b * stride + off];
    t = warp_sum_d(t);
    if (threadIdx.x == 0) sm[0] = t;
  }
  __syncthreads();
  t = sm[0];
  __syncthreads();
  return t;
}

// ------------------------------------------------------------- PCG ---
// FieldSolve::pcgsolver (src/field.cpp:212-264) with pcg()
// (linearalgebra/solvers.h:73-100) and the Jacobi preconditioner 1/(-4),
// matrix-free.  The reference's dense row k of A (src/field.cpp:221-232, row
// = k/nx, col = k%nx) summed in column order is, term for term,
//   u_k = ((v[k-nx] + v[k-1]) + (-4 v[k])) + v[k+1]) + v[k+nx]
// with missing neighbours skipped.  Solution x lives in phi (unflatten keeps
// the index i*ny + j).
//
// One cooperative launch runs the whole solve with two grid barriers per
// iteration: the direction update v <- w + s v is fused into the next SpMV,
// which recomputes the updated neighbour values from r and the previous v
// (double-buffered).  Each barrier is preceded by one block reduction of two
// values and followed by one parallel load of the per-block partials summed
// in a fixed tree, so every block derives identical scalars and the solve is
// deterministic.  The dot products are summed in another order than the
// reference's serial loops and the updates use fused multiply-adds; on the
// CPU such perturbations leave the iterates within ~1e-14 of the reference's
// up to 257x257 and ~1000 iterations.  Data written by other blocks within
// the launch is read with ld.global.cg (L2), never from a possibly stale L1.

// (a, b) summed over the block; the result is returned to every thread.
__device__ double2 block_sum2(double a, double b, double* sm /* >= 18 */) {
  a = warp_sum_d(a);
  b = warp_sum_d(b);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sm[w] = a;
    sm[8 + w] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0, tb = 0;
    for (int k = 0; k < nw; k++) {
      ta += sm[k];
      tb += sm[8 + k];
    }
    sm[16] = ta;
    sm[17] = tb;
  }
  __syncthreads();
  double2 r = make_double2(sm[16], sm[17]);
  __syncthreads();
  return r;
}

// Grid total of per-block (a, b) partials, identical in every block.
__device__ double2 grid_total2(const double2* P, int nb, double* sm) {
  double a = 0, b = 0;
  for (int k = threadIdx.x; k < nb; k += blockDim.x) {
    double2 v = __ldcg(&P[k]);
    a += v.x;
    b += v.y;
  }
  return block_sum2(a, b, sm);
}

__device__ __forceinline__ double stencil_row(long k, int nx, int ny, const double* v) {
  long row = k / nx, col = k % nx;
  double sum = 0;
  if (row > 0) sum += __ldcg(&v[k - nx]);
  if (col > 0) sum += __ldcg(&v[k - 1]);
  sum = fma(-4.0, __ldcg(&v[k]), sum);
  if (col < nx - 1) sum += __ldcg(&v[k + 1]);
  if (row < ny - 1) sum += __ldcg(&v[k + nx]);
  return sum;
}

__device__ __forceinline__ double vnext(long k, const double* r, const double* vp, double minv, double s) {
  return fma(__ldcg(&vp[k]), s, minv * __ldcg(&r[k]));
}

__device__ __forceinline__ double stencil_next(long k, int nx, int ny, const double* r, const double* vp, double minv,
                                               double s, double vk) {
  long row = k / nx, col = k % nx;
  double sum = 0;
  if (row > 0) sum += vnext(k - nx, r, vp, minv, s);
  if (col > 0) sum += vnext(k - 1, r, vp, minv, s);
  sum = fma(-4.0, vk, sum);
  if (col < nx - 1) sum += vnext(k + 1, r, vp, minv, s);
  if (row < ny - 1) sum += vnext(k + nx, r, vp, minv, s);
  return sum;
}

__global__ void __launch_bounds__(256) k_pcg(SolverArgs a) {
  __shared__ double sm[20];
  const int nx = a.g.nx, ny = a.g.ny;
  const long n = (long)nx * ny;
  const long tid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long stride = (long)gridDim.x * blockDim.x;
  const int nb = gridDim.x;
  double* x = a.phi;
  double* b = a.b;
  double* r = a.r;
  double* u = a.u;
  double2* PA = reinterpret_cast<double2*>(a.partials);  // [nb] (v.u, -)
  double2* PB = PA + nb;                                  // [nb] (w.r, r.r)
  const double minv = 1.0 / -4.0;
  const double dx2 = a.g.dx * a.g.dx;
  // set-up: b (src/field.cpp:234-252), x = 0, r = b - A*0, w = M^-1 r, v = w.
  double pa = 0, pr = 0;
  for (long k = tid; k < n; k += stride) {
    int i = (int)(k / ny), j = (int)(k % ny);
    double bk = -a.rho[k] * dx2 * a.K;
    if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1) bk = 0;
    b[k] = bk;
    x[k] = 0;
    double rk = bk - 0.0;
    r[k] = rk;
    double wk = minv * rk;
    a.va[k] = wk;
    pa = fma(wk, rk, pa);
    pr = fma(rk, rk, pr);
  }
  double2 bs = block_sum2(pa, pr, sm);
  if (threadIdx.x == 0) PB[blockIdx.x] = bs;
  if (!grid_sync(a.bar, a.flags)) return;
  double2 tot = grid_total2(PB, nb, sm);
  double alpha = tot.x, rr = tot.y;
  unsigned int cap32 = (unsigned int)n * (unsigned int)n;
  int maxit = (int)cap32 < a.max_iter ? (int)cap32 : a.max_iter;
  double* vp = a.va;  // direction of the previous iteration
  double* vc = a.vb;
  double s = 0;
  int it = 0;
  for (it = 0; it < maxit; it++) {
    if (sqrt(rr) < a.tol) break;
    // u = A v, with v = w + s*v_prev folded in after the first iteration.
    double pvu = 0;
    for (long k = tid; k < n; k += stride) {
      double vk, uk;
      if (it == 0) {
        vk = __ldcg(&vp[k]);
        uk = stencil_row(k, nx, ny, vp);
      } else {
        vk = vnext(k, r, vp, minv, s);
        uk = stencil_next(k, nx, ny, r, vp, minv, s, vk);
      }
      vc[k] = vk;
      u[k] = uk;
      pvu = fma(vk, uk, pvu);
    }
    bs = block_sum2(pvu, 0.0, sm);
    if (threadIdx.x == 0) PA[blockIdx.x] = bs;
    if (!grid_sync(a.bar, a.flags)) return;
    double t = alpha / grid_total2(PA, nb, sm).x;
    double pb = 0, prr = 0;
    for (long k = tid; k < n; k += stride) {
      double xk = fma(vc[k], t, x[k]);
      double rk = fma(-u[k], t, r[k]);
      x[k] = xk;
      r[k] = rk;
      double wk = minv * rk;
      pb = fma(wk, rk, pb);
      prr = fma(rk, rk, prr);
    }
    bs = block_sum2(pb, prr, sm);
    if (threadIdx.x == 0) PB[blockIdx.x] = bs;
    if (!grid_sync(a.bar, a.flags)) return;
    tot = grid_total2(PB, nb, sm);
    double beta = tot.x;
    rr = tot.y;
    s = beta / alpha;
    alpha = beta;
    double* tmp = vp;
    vp = vc;
    vc = tmp;
  }
  // domain.error = |A x - b| / n (src/field.cpp:258-259)
  double pe = 0;
  for (long k = tid; k < n; k += stride) {
    double e = stencil_row(k, nx, ny, x) - b[k];
    pe = fma(e, e, pe);
  }
  bs = block_sum2(pe, 0.0, sm);
  if (threadIdx.x == 0) PA[blockIdx.x] = bs;
  if (!grid_sync(a.bar, a.flags)) return;
  double e2 = grid_total2(PA, nb, sm).x;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.info->iterations = it;
    a.info->converged = it < maxit;
    a.info->error = sqrt(e2) / n;
    atomicAdd(a.iter_total, (unsigned long long)it);
  }
}

static int g_pcg_max_blocks = 0;

int solver_max_blocks() {
  if (!g_pcg_max_blocks) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg, 256, 0);
    if (per_sm < 1) per_sm = 1;
    g_pcg_max_blocks = sms * (per_sm < 2 ? per_sm : 2);
  }
  return g_pcg_max_blocks;
}

void launch_pcg(cudaStream_t st, const SolverArgs& a, int blocks) {
  SolverArgs args = a;
  void* params[] = {&args};
  cudaMemsetAsync(a.bar, 0, 2 * sizeof(unsigned int), st);
  cudaLaunchCooperativeKernel((const void*)k_pcg, dim3(blocks), dim3(256), params, 0, st);
}

// -------------------------------------------------- red-black SOR ---
// Fast-mode alternative to the lexicographic sweep: same update formula,
// same cold start, zero edges and residual checks (after sweeps 0, 25, ...),
// but red nodes ((i+j) even) then black nodes per sweep.  It converges to the
// same fixed point with different iterates.
__global__ void __launch_bounds__(256) k_sor_rb(SolverArgs a) {
  __shared__ double sm[40];
  const int nx = a.g.nx, ny = a.g.ny;
  const long n = (long)nx * ny;
  const long tid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long stride = (long)gridDim.x * blockDim.x;
  const int nb = gridDim.x;
  double* phi = a.phi;
  const double dx2 = a.g.dx * a.g.dx, dy2 = a.g.dy * a.g.dy;
  const double coeff = (2 / dx2) + (2 / dy2);
  const double inv_coeff = 1 / coeff;
  if (!a.warm)
    for (long k = tid; k < n; k += stride) phi[k] = 0;
  else
    for (long k = tid; k < n; k += stride) {
      int i = (int)(k / ny), j = (int)(k % ny);
      if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1) phi[k] = 0;
    }
  if (!grid_sync(a.bar, a.flags)) return;
  const long ni = (long)(nx - 2) * (ny - 2);
  int iter = 0, converged = 0;
  double L2 = 0;
  for (iter = 0; iter < a.max_iter && ni > 0;) {
    for (int color = 0; color < 2; color++) {
      for (long q = tid; q < ni; q += stride) {
        int i = 1 + (int)(q / (ny - 2)), j = 1 + (int)(q % (ny - 2));
        if (((i + j) & 1) != color) continue;
        long k = (long)i * ny + j;
        double pE = __ldcg(&phi[k + ny]), pW = __ldcg(&phi[k - ny]);
        double pN = __ldcg(&phi[k + 1]), pS = __ldcg(&phi[k - 1]), pk = __ldcg(&phi[k]);
        double phi_new = inv_coeff * (a.rho[k] * a.K + ((pE + pW) / dx2) + ((pN + pS) / dy2));
        phi[k] = pk + a.omega * (phi_new - pk);
      }
      if (!grid_sync(a.bar, a.flags)) return;
    }
    int last = iter;
    iter++;
    if (last % 25 == 0) {
      double sum = 0;
      for (long q = tid; q < ni; q += stride) {
        int i = 1 + (int)(q / (ny - 2)), j = 1 + (int)(q % (ny - 2));
        long k = (long)i * ny + j;
        double pE = __ldcg(&phi[k + ny]), pW = __ldcg(&phi[k - ny]);
        double pN = __ldcg(&phi[k + 1]), pS = __ldcg(&phi[k - 1]), pk = __ldcg(&phi[k]);
        double R = ((pE - 2 * pk + pW) / dx2) + ((pN - 2 * pk + pS) / dy2) + (a.rho[k]) * a.K;
        sum += R * R;
      }
      sum = block_sum_256(sum, sm);
      if (threadIdx.x == 0) a.partials[blockIdx.x] = sum;
      if (!grid_sync(a.bar, a.flags)) return;
      double tot = sum_partials(a.partials, nb, 1, 0, sm);
      L2 = sqrt(tot / (nx * ny));
      if (!grid_sync(a.bar, a.flags)) return;  // partials are rewritten at the next check
      if (L2 < a.tol) {
        converged = 1;
        break;
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.info->iterations = iter;
    a.info->converged = converged;
    a.info->error = L2;
    atomicAdd(a.iter_total, (unsigned long long)iter);
  }
}

void launch_sor_redblack(cudaStream_t st, const SolverArgs& a, int blocks) {
  SolverArgs args = a;
  void* params[] = {&args};
  cudaMemsetAsync(a.bar, 0, 2 * sizeof(unsigned int), st);
  cudaLaunchCooperativeKernel((const void*)k_sor_rb, dim3(blocks), dim3(256), params, 0, st);
}

// ----------------------------------------------------- grid reductions ---
// what 0: sum ef2*(L*L) with ef2 = efx^2+efy^2 (Domain::Compute_PE,
// src/domain.cpp:266-286); what 1: max(phi) (Output::diagnostics, src/output.cpp:320-332).
__global__ void k_grid_sums(int what, long nn, const double* a, const double* b, double L, double* partials) {
  __shared__ double sm[8];
  double acc = what == 0 ? 0.0 : -1.0 / 0.0;
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += (long)gridDim.x * blockDim.x) {
    if (what == 0) {
      double ef2 = a[k] * a[k] + b[k] * b[k];
      acc += ef2 * (L * L);
    } else {
      acc = fmax(acc, a[k]);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double y = __shfl_down_sync(0xffffffffu, acc, o);
    acc = what == 0 ? acc + y : fmax(acc, y);
  }
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = sm[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) t = what == 0 ? t + sm[w] : fmax(t, sm[w]);
    partials[blockIdx.x] = t;
  }
}

__global__ void k_grid_final(int what, const double* partials, int nb, double* out) {
  double t = what == 0 ? 0.0 : -1.0 / 0.0;
  if (threadIdx.x == 0) {
    for (int i = 0; i < nb; i++) t = what == 0 ? t + partials[i] : fmax(t, partials[i]);
    out[0] = t;
  }
}

void launch_grid_sums(cudaStream_t st, int what, const Geom& g, const double* a, const double* b, double L,
                      double* partials, double* out) {
  long nn = (long)g.nx * g.ny;
  int nb = (int)((nn + 255) / 256);
  if (nb > 256) nb = 256;
  k_grid_sums<<<nb, 256, 0, st>>>(what, nn, a, b, L, partials);
  k_grid_final<<<1, 32, 0, st>>>(what, partials, nb, out);
}

}  // namespace epic
