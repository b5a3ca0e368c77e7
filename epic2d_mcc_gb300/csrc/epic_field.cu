// Grid kernels of the FP64 plain form: density finalisation + charge density,
// the two SOR solvers and the PCG solver of FieldSolve, the E-field, and the
// potential-energy / max-phi reductions.
//
// Built with -fmad=false so every expression rounds as the reference's does;
// the PCG kernel uses explicit fma() where it is documented to.
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
// per node, reading the deposit accumulators and writing the density grids.
// A node on an edge recomputes the (identical) values of the nodes it is
// folded with, so the fold needs no second pass:
//   D = raw/div;  pbc: Y(i,j) = D(i,0)+D(i,ny-1) on j edges, then
//   X(i,j) = Y(0,j)+Y(nx-1,j) on i edges;  open/reflective: edges x0.5,
//   corners x0.25.
__device__ __forceinline__ double raw_den(const FinalizeArgs& a, int s, int i, int j) {
  int k = i * a.g.ny + j;
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
  const int nn = nx * ny;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const int i = k / ny, j = k - i * ny;
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
  int nn = a.g.nx * a.g.ny;
  k_finalize<<<(nn + 255) / 256, 256, 0, st>>>(a);
}

// ------------------------------------------------------------ E-field ---
// FieldSolve::CalculateEfield (src/field.cpp:276-330).
__global__ void k_efield(Geom g, int bc, const double* __restrict__ phi, double* efx, double* efy, double2* ef,
                         float2* ef32) {
  const int nx = g.nx, ny = g.ny;
  const int nn = nx * ny;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const int i = k / ny, j = k - i * ny;
    double ex = efx[k], ey = efy[k];
#define PHI(a, b) phi[(a) * ny + (b)]
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
    if (ef32) ef32[k] = make_float2((float)ex, (float)ey);
  }
}

void launch_efield(cudaStream_t st, const Geom& g, int bc, const double* phi, double* efx, double* efy, double2* ef,
                   float2* ef32) {
  int nn = g.nx * g.ny;
  k_efield<<<(nn + 255) / 256, 256, 0, st>>>(g, bc, phi, efx, efy, ef, ef32);
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
  const int ni = (nx - 2) * (ny - 2);
  for (int q = threadIdx.x; q < ni; q += blockDim.x) {
    int i = 1 + q / (ny - 2), j = 1 + q % (ny - 2);
    int k = i * ny + j;
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
  const int nn = nx * ny;
  double* phi = use_smem ? smem : a.phi;
  const double dx2 = a.g.dx * a.g.dx, dy2 = a.g.dy * a.g.dy;
  const double coeff = (2 / dx2) + (2 / dy2);
  const double inv_coeff = 1 / coeff;
  for (int k = threadIdx.x; k < nn; k += blockDim.x) phi[k] = 0;  // cold start, zero edges (src/field.cpp:78-98)
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
          int k = i * ny + j;
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
    for (int k = threadIdx.x; k < nn; k += blockDim.x) a.phi[k] = phi[k];
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
// Cooperative launches guarantee that all blocks are resident.  bar[0] counts
// arrivals since the launch (zeroed before it): the blocks of barrier episode
// e draw tickets in [e*nb, (e+1)*nb) and wait until the count reaches
// (e+1)*nb.  Every wait gives up after SPIN_LIMIT polls (FLAG_TIMEOUT), so a
// fault can never hang the GPU.
// The arrival is an atom.add with release semantics and the wait polls with
// ld.acquire at GPU scope: the block's writes (ordered before thread 0 by
// __syncthreads) become visible to every block that observes the count, with
// no separate full fences (measured ~1.5 us per barrier on GB300 at 152 CTAs
// against ~1.9 us with __threadfence on both sides).
__device__ __forceinline__ unsigned int atom_add_release_gpu(unsigned int* p, unsigned int v) {
  unsigned int old;
  asm volatile("atom.add.release.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
  unsigned int v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ bool grid_sync(unsigned int* bar, int* flags) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int ticket = atom_add_release_gpu(bar, 1u);
    const unsigned int target = (ticket / gridDim.x + 1) * gridDim.x;
    int ok = 1;
    long long spins = 0;
    while ((int)(ld_acquire_gpu(bar) - target) < 0) {
      if (++spins > SPIN_LIMIT) {
        atomicOr(flags, FLAG_TIMEOUT);
        ok = 0;
        break;
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok;
}

// Block reduction of (a, b) whose totals thread 0 stores as this block's
// partial.  Partials are summed after the next barrier by grid_total2_t0 in a
// fixed order, so every block derives identical totals (deterministic).
__device__ void block_partial2(double a, double b, double2* P, double* sw /* >= 16 */) {
  a = warp_sum_d(a);
  b = warp_sum_d(b);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sw[w] = a;
    sw[8 + w] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double ta = 0, tb = 0;
    for (int k = 0; k < nw; k++) {
      ta += sw[k];
      tb += sw[8 + k];
    }
    P[blockIdx.x] = make_double2(ta, tb);
  }
}

// Totals of the nb partials; valid in thread 0 (the caller broadcasts).
__device__ double2 grid_total2_t0(const double2* P, int nb, double* sw) {
  double a = 0, b = 0;
  for (int k = threadIdx.x; k < nb; k += blockDim.x) {
    double2 v = __ldcg(&P[k]);
    a += v.x;
    b += v.y;
  }
  a = warp_sum_d(a);
  b = warp_sum_d(b);
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sw[w] = a;
    sw[8 + w] = b;
  }
  __syncthreads();
  double2 r = make_double2(0.0, 0.0);
  if (threadIdx.x == 0)
    for (int k = 0; k < nw; k++) {
      r.x += sw[k];
      r.y += sw[8 + k];
    }
  return r;
}

// ------------------------------------------------------------- PCG ---
// FieldSolve::pcgsolver (src/field.cpp:212-264) with pcg()
// (linearalgebra/solvers.h:73-100) and the Jacobi preconditioner M = 1/(-4),
// matrix-free: the reference's dense row k of A (src/field.cpp:221-232,
// row = k/nx, col = k%nx, diagonal -4, off-diagonals 1) as a 5-point stencil
// with missing neighbours skipped.  x lives in phi (unflatten keeps the
// index i*ny + j); x0 = 0, the stopping test |r|_2 < tol precedes every
// update and the cap is min(n*n in 32-bit int, max_iteration), as there.
//
// The iteration is the Chronopoulos-Gear form of the same preconditioned CG
// (u = M r, w = A u; gamma = (r,u), delta = (w,u); beta = gamma/gamma_prev,
// eta = delta - beta*gamma/alpha, alpha = gamma/eta; p = u + beta p,
// s = w + beta s, x += alpha p, r -= alpha s): mathematically the reference's
// iterates, with all three dot products of an iteration (gamma, delta, r.r)
// in one grid reduction.  The SpMV of the next iteration needs the neighbours'
// new u = M(r - alpha(w + beta s)), which each thread recomputes from the
// neighbours' previous r, w, s (double-buffered), so one grid barrier per
// iteration suffices.  On the CPU this form reproduces the reference's
// iteration counts and stays within ~6e-15 of its solution up to 257x257
// (~1000 iterations).  The scalars are computed by thread 0 of each block
// from identically ordered partial sums (deterministic), and data written by
// other blocks within the launch is read with ld.global.cg (L2), never from a
// possibly stale L1.
__device__ __forceinline__ double rhs_at(const SolverArgs& a, int k, int i, int j, double dx2) {
  // src/field.cpp:234-252: -rho * dx^2 * (L^2/LDe^2), zero on the edges.
  if (i == 0 || i == a.g.nx - 1 || j == 0 || j == a.g.ny - 1) return 0.0;
  return -a.rho[k] * dx2 * a.K;
}

// Block partial of three values.  Every thread parks its values in shared
// memory and warp 0 alone adds them (eight each, then a shuffle tree): on
// GB300 each FP64 warp-instruction holds the SM's FP64 pipe for ~16 cycles,
// so a shuffle tree in all eight warps cost ~4k cycles against ~1k for this.
__device__ void block_partial3(double a0, double a1, double a2, double* P, double* sw /* >= 3*256 */) {
  sw[threadIdx.x] = a0;
  sw[256 + threadIdx.x] = a1;
  sw[512 + threadIdx.x] = a2;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t0 = 0, t1 = 0, t2 = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const int m = threadIdx.x + 32 * k;
      t0 += sw[m];
      t1 += sw[256 + m];
      t2 += sw[512 + m];
    }
    t0 = warp_sum_d(t0);
    t1 = warp_sum_d(t1);
    t2 = warp_sum_d(t2);
    if (threadIdx.x == 0) {
      P[4 * blockIdx.x + 0] = t0;
      P[4 * blockIdx.x + 1] = t1;
      P[4 * blockIdx.x + 2] = t2;
    }
  }
}

// Totals of the nb partials in a fixed order, computed by warp 0 alone (no
// block barrier); valid in thread 0.
__device__ double3 grid_total3_t0(const double* P, int nb) {
  double3 r = make_double3(0.0, 0.0, 0.0);
  if (threadIdx.x < 32) {
    double t0 = 0, t1 = 0, t2 = 0;
#pragma unroll 4
    for (int k = threadIdx.x; k < nb; k += 32) {
      const double2 v01 = __ldcg(reinterpret_cast<const double2*>(P + 4 * k));
      t0 += v01.x;
      t1 += v01.y;
      t2 += __ldcg(P + 4 * k + 2);
    }
    r.x = warp_sum_d(t0);
    r.y = warp_sum_d(t1);
    r.z = warp_sum_d(t2);
  }
  return r;
}

__global__ void __launch_bounds__(256) k_pcg(SolverArgs a) {
  __shared__ double sw[3 * 256];
  __shared__ double s_alpha, s_beta;
  __shared__ int s_done;
  const int nx = a.g.nx, ny = a.g.ny;
  const int n = nx * ny;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  const int nb = gridDim.x;
  double* x = a.phi;
  double* b = a.work[0];
  double* R[2] = {a.work[1], a.work[2]};
  double* S[2] = {a.work[3], a.work[4]};
  double* W[2] = {a.work[5], a.work[6]};
  double* Pd = a.work[7];
  double* P = a.partials;  // [nb][4]
  const double minv = 1.0 / -4.0;
  const double dx2 = a.g.dx * a.g.dx;

  // set-up: x = 0, r = b - A*0, u = M r, w = A u, p = s = 0.
  double pg = 0, pd = 0, pr = 0;
  for (int k = tid; k < n; k += stride) {
    const int i = k / ny, j = k - i * ny;
    const int row = k / nx, col = k - row * nx;
    const double bk = rhs_at(a, k, i, j, dx2);
    b[k] = bk;
    x[k] = 0;
    const double rk = bk - 0.0;
    const double uk = minv * rk;
    double sum = 0;
    if (row > 0) { int m = k - nx, mi = m / ny; sum += minv * rhs_at(a, m, mi, m - mi * ny, dx2); }
    if (col > 0) { int m = k - 1, mi = m / ny; sum += minv * rhs_at(a, m, mi, m - mi * ny, dx2); }
    sum = fma(-4.0, uk, sum);
    if (col < nx - 1) { int m = k + 1, mi = m / ny; sum += minv * rhs_at(a, m, mi, m - mi * ny, dx2); }
    if (row < ny - 1) { int m = k + nx, mi = m / ny; sum += minv * rhs_at(a, m, mi, m - mi * ny, dx2); }
    R[0][k] = rk;
    W[0][k] = sum;
    S[0][k] = 0;
    Pd[k] = 0;
    pg = fma(rk, uk, pg);
    pd = fma(sum, uk, pd);
    pr = fma(rk, rk, pr);
  }
  block_partial3(pg, pd, pr, P, sw);
  if (!grid_sync(a.bar, a.flags)) return;
  unsigned int cap32 = (unsigned int)n * (unsigned int)n;
  const int maxit = (int)cap32 < a.max_iter ? (int)cap32 : a.max_iter;
  double alpha = 0, gamma_prev = 0;  // thread 0 only
  int it = 0, cur = 0;
  // Thread 0, after each reduction: the stopping test on r.r and the scalars
  // of the next update, then one __syncthreads broadcasts them.
  auto scalars = [&](double3 t) {
    const double gamma = t.x, delta = t.y;
    s_done = sqrt(t.z) < a.tol;
    double beta, eta;
    if (it == 0) {
      beta = 0;
      eta = delta;
    } else {
      beta = gamma / gamma_prev;
      eta = delta - beta * gamma / alpha;
    }
    alpha = gamma / eta;
    gamma_prev = gamma;
    s_alpha = alpha;
    s_beta = beta;
  };
  {
    double3 t = grid_total3_t0(P, nb);
    if (threadIdx.x == 0) scalars(t);
    __syncthreads();
  }
  while (it < maxit && !s_done) {
    const double al = s_alpha, be = s_beta;
    const double* Rc = R[cur];
    const double* Sc = S[cur];
    const double* Wc = W[cur];
    double* Rn = R[cur ^ 1];
    double* Sn = S[cur ^ 1];
    double* Wn = W[cur ^ 1];
    pg = pd = pr = 0;
    for (int k = tid; k < n; k += stride) {
      const int row = k / nx, col = k - row * nx;
      const double rc = __ldcg(&Rc[k]);
      const double sk = fma(be, __ldcg(&Sc[k]), __ldcg(&Wc[k]));
      const double pk = fma(be, Pd[k], minv * rc);
      x[k] = fma(al, pk, x[k]);
      const double rk = fma(-al, sk, rc);
      const double uk = minv * rk;
      // w_new = A u_new; a neighbour's u_new from its previous r, w, s.  The
      // loads use clamped indices so all of them issue before the first
      // use; missing neighbours are then skipped as in the reference.
#define UNEW(m) (minv * fma(-al, fma(be, __ldcg(&Sc[m]), __ldcg(&Wc[m])), __ldcg(&Rc[m])))
      const double uN = UNEW(row > 0 ? k - nx : k);
      const double uW = UNEW(col > 0 ? k - 1 : k);
      const double uE = UNEW(col < nx - 1 ? k + 1 : k);
      const double uS = UNEW(row < ny - 1 ? k + nx : k);
#undef UNEW
      double sum = 0;
      if (row > 0) sum += uN;
      if (col > 0) sum += uW;
      sum = fma(-4.0, uk, sum);
      if (col < nx - 1) sum += uE;
      if (row < ny - 1) sum += uS;
      Pd[k] = pk;
      Sn[k] = sk;
      Rn[k] = rk;
      Wn[k] = sum;
      pg = fma(rk, uk, pg);
      pd = fma(sum, uk, pd);
      pr = fma(rk, rk, pr);
    }
    block_partial3(pg, pd, pr, P, sw);
    if (!grid_sync(a.bar, a.flags)) return;
    cur ^= 1;
    it++;
    {
      double3 t = grid_total3_t0(P, nb);
      if (threadIdx.x == 0) scalars(t);
      __syncthreads();
    }
  }
  // domain.error = |A x - b| / n (src/field.cpp:258-259); x is complete
  // everywhere after the last barrier.
  double pe = 0;
  for (int k = tid; k < n; k += stride) {
    const int row = k / nx, col = k - row * nx;
    double sum = 0;
    if (row > 0) sum += __ldcg(&x[k - nx]);
    if (col > 0) sum += __ldcg(&x[k - 1]);
    sum = fma(-4.0, __ldcg(&x[k]), sum);
    if (col < nx - 1) sum += __ldcg(&x[k + 1]);
    if (row < ny - 1) sum += __ldcg(&x[k + nx]);
    const double e = sum - b[k];
    pe = fma(e, e, pe);
  }
  block_partial3(pe, 0.0, 0.0, P, sw);
  if (!grid_sync(a.bar, a.flags)) return;
  double3 e2 = grid_total3_t0(P, nb);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.info->iterations = it;
    a.info->converged = it < maxit;
    a.info->error = sqrt(e2.x) / n;
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
  __shared__ double sw[16];
  __shared__ int s_done;
  __shared__ double s_l2;
  const int nx = a.g.nx, ny = a.g.ny;
  const int n = nx * ny;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  const int nb = gridDim.x;
  double* phi = a.phi;
  double2* P = reinterpret_cast<double2*>(a.partials);
  const double dx2 = a.g.dx * a.g.dx, dy2 = a.g.dy * a.g.dy;
  const double coeff = (2 / dx2) + (2 / dy2);
  const double inv_coeff = 1 / coeff;
  for (int k = tid; k < n; k += stride) {
    const int i = k / ny, j = k - i * ny;
    if (!a.warm || i == 0 || i == nx - 1 || j == 0 || j == ny - 1) phi[k] = 0;
  }
  if (!grid_sync(a.bar, a.flags)) return;
  const int ni = (nx - 2) * (ny - 2);
  int iter = 0, converged = 0;
  double L2 = 0;
  for (iter = 0; iter < a.max_iter && ni > 0;) {
    for (int color = 0; color < 2; color++) {
      for (int q = tid; q < ni; q += stride) {
        const int i = 1 + q / (ny - 2), j = 1 + q % (ny - 2);
        if (((i + j) & 1) != color) continue;
        const int k = i * ny + j;
        double pE = __ldcg(&phi[k + ny]), pW = __ldcg(&phi[k - ny]);
        double pN = __ldcg(&phi[k + 1]), pS = __ldcg(&phi[k - 1]), pk = __ldcg(&phi[k]);
        double phi_new = inv_coeff * (a.rho[k] * a.K + ((pE + pW) / dx2) + ((pN + pS) / dy2));
        phi[k] = pk + a.omega * (phi_new - pk);
      }
      if (!grid_sync(a.bar, a.flags)) return;
    }
    const int last = iter;
    iter++;
    if (last % 25 == 0) {
      double sum = 0;
      for (int q = tid; q < ni; q += stride) {
        const int i = 1 + q / (ny - 2), j = 1 + q % (ny - 2);
        const int k = i * ny + j;
        double pE = __ldcg(&phi[k + ny]), pW = __ldcg(&phi[k - ny]);
        double pN = __ldcg(&phi[k + 1]), pS = __ldcg(&phi[k - 1]), pk = __ldcg(&phi[k]);
        double R = ((pE - 2 * pk + pW) / dx2) + ((pN - 2 * pk + pS) / dy2) + (a.rho[k]) * a.K;
        sum += R * R;
      }
      block_partial2(sum, 0.0, P, sw);
      if (!grid_sync(a.bar, a.flags)) return;
      double2 tot = grid_total2_t0(P, nb, sw);
      if (threadIdx.x == 0) {
        s_l2 = sqrt(tot.x / (nx * ny));
        s_done = s_l2 < a.tol;
      }
      __syncthreads();
      L2 = s_l2;
      if (!grid_sync(a.bar, a.flags)) return;  // partials are rewritten at the next check
      if (s_done) {
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
__global__ void k_grid_sums(int what, int nn, const double* a, const double* b, double L, double* partials) {
  __shared__ double sm[8];
  double acc = what == 0 ? 0.0 : -1.0 / 0.0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
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
  int nn = g.nx * g.ny;
  int nb = (nn + 255) / 256;
  if (nb > 256) nb = 256;
  k_grid_sums<<<nb, 256, 0, st>>>(what, nn, a, b, L, partials);
  k_grid_final<<<1, 32, 0, st>>>(what, partials, nb, out);
}

}  // namespace epic
