// Grid kernels of the FP64 plain form: density finalisation + charge density,
// the two SOR solvers and the PCG solver of FieldSolve, the E-field, and the
// potential-energy / max-phi reductions.
//
// Built with -fmad=false so every expression rounds as the reference's does;
// the PCG kernel uses explicit fma() where it is documented to.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <atomic>
#include <map>
#include <mutex>
#include <tuple>

#include <algorithm>

#include "epic_grid.cuh"
#include "epic_internal.cuh"
#include "epic_xsum.cuh"

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


__global__ void k_finalize(FinalizeArgs a) {
  const int nx = a.g.nx, ny = a.g.ny;
  const int nn = nx * ny;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const int i = k / ny, j = k - i * ny;
    // One pass over the species: each density, then its charge added to rho
    // in species order (no per-thread array, which would live in local memory).
    double rho = 0;
    for (int s = 0; s < a.nsp; s++) {
      double v;
      if (a.stage == RHO_FROM_DEN || !a.active[s]) {
        v = a.den[s][k];
      } else {
        auto raw = [&](int ii, int jj) { return raw_den(a, s, ii, jj); };
        v = fold_density(a.bc, nx, ny, raw, i, j);
        a.den[s][k] = v;
      }
      double t = v * a.charge_over_qe[s];
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
// FieldSolve::CalculateEfield (src/field.cpp:276-330), edge rules xr, yr
// (efield_edges).
__global__ void k_efield(Geom g, int xr, int yr, const double* __restrict__ phi, double* efx, double* efy,
                         double2* ef, float2* ef32) {
  const int nx = g.nx, ny = g.ny;
  const int nn = nx * ny;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nn; k += gridDim.x * blockDim.x) {
    const int i = k / ny, j = k - i * ny;
    double ex = efx[k], ey = efy[k];
    auto PHI = [&](int a_, int b_) { return phi[a_ * ny + b_]; };
    efield_node(xr, yr, nx, ny, g.dx, g.dy, PHI, i, j, ex, ey);
    efx[k] = ex;
    efy[k] = ey;
    ef[k] = make_double2(ex, ey);
    if (ef32) ef32[k] = make_float2((float)ex, (float)ey);
  }
}

void launch_efield(cudaStream_t st, const Geom& g, int bc, int poisson_bc, const double* phi, double* efx,
                   double* efy, double2* ef, float2* ef32) {
  int nn = g.nx * g.ny;
  int xr, yr;
  efield_edges(bc, poisson_bc, &xr, &yr);
  k_efield<<<(nn + 255) / 256, 256, 0, st>>>(g, xr, yr, phi, efx, efy, ef, ef32);
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

// ---- exact dot-product reductions (integer pipe, epic_xsum.cuh) ----
// Exact sum of term(q), q in [0, count), over the block (each thread takes a
// strided share), anchored on the largest exponent and rounded once
// (epic_xsum.cuh); valid in every thread.
template <class F>
__device__ double block_exact_sum(int count, const F& term, double* red) {
  __shared__ int s_e[32];
  __shared__ unsigned long long s_v[32][2];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int e = 0;
  for (int q = threadIdx.x; q < count; q += blockDim.x) e = max(e, xs_exponent(term(q)));
  e = (int)__reduce_max_sync(0xffffffffu, (unsigned)e);
  if (lane == 0) s_e[wid] = e;
  __syncthreads();
  int A = 0;
  for (int w = 0; w < nw; w++) A = max(A, s_e[w]);
  xs_int v = 0;
  for (int q = threadIdx.x; q < count; q += blockDim.x) v += xs_from_double(term(q), A);
  v = xs_warp_sum(v);
  if (lane == 0) {
    s_v[wid][0] = (unsigned long long)(xs_uint)v;
    s_v[wid][1] = (unsigned long long)((xs_uint)v >> 64);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    xs_uint tot = 0;
    for (int w = 0; w < nw; w++) tot += ((xs_uint)s_v[w][1] << 64) | s_v[w][0];
    red[33] = xs_to_double((xs_int)tot, A);
  }
  __syncthreads();
  const double r = red[33];
  __syncthreads();
  return r;
}

// The unknowns of gssolver: the interior i in [1, nx-2], j in [1, ny-2]
// (the reference), or an extension lattice (EPIC_POISSON_*): i from i0 = 0
// (PERIODIC) or 1 (DIRICHLET_X) to nx-2, j in [0, ny-2], with wrapped
// neighbours.  Node indices of the four neighbours of unknown (i, j).
struct SorLat {
  int i0, j0, nxi, nyi, wrap_x, wrap_y;
};
__device__ __forceinline__ SorLat sor_lattice(int nx, int ny, int poisson_bc) {
  SorLat l;
  if (poisson_bc == EPIC_POISSON_DIRICHLET) {
    l.i0 = 1; l.j0 = 1; l.nxi = nx - 2; l.nyi = ny - 2; l.wrap_x = 0; l.wrap_y = 0;
  } else {
    l.wrap_x = poisson_bc == EPIC_POISSON_PERIODIC;
    l.wrap_y = 1;
    l.i0 = l.wrap_x ? 0 : 1; l.j0 = 0; l.nxi = nx - 1 - l.i0; l.nyi = ny - 1;
  }
  return l;
}
template <bool EXT>
__device__ __forceinline__ void sor_nbrs(const SorLat& l, int nx, int ny, int i, int j, int& kE, int& kW, int& kN,
                                         int& kS) {
  const int k = i * ny + j;
  if (!EXT) {
    kE = k + ny; kW = k - ny; kN = k + 1; kS = k - 1;
    return;
  }
  kE = (i + 1 < nx - 1 || !l.wrap_x) ? k + ny : j;  // wraps to node (0, j)
  kW = i > 0 ? k - ny : (nx - 2) * ny + j;
  kN = j + 1 < ny - 1 ? k + 1 : i * ny;          // wraps to node (i, 0)
  kS = j > 0 ? k - 1 : i * ny + ny - 2;
}

// Residual of src/field.cpp:121-134 over the unknowns (one block); src(k) is
// the source term rho*K (minus its mean when periodic).
template <bool FLUID, bool UNIT, bool EXT, class Src>
__device__ double sor_residual(const SolverArgs& a, const SorLat& l, const double* phi, const Src& src, double* red) {
  const int nx = a.g.nx, ny = a.g.ny;
  const double dx2 = a.g.dx * a.g.dx, dy2 = a.g.dy * a.g.dy;
  double sum = 0;
  const int ni = l.nxi * l.nyi;
  for (int q = threadIdx.x; q < ni; q += blockDim.x) {
    int i = l.i0 + q / l.nyi, j = l.j0 + q % l.nyi;
    int k = i * ny + j;
    int kE, kW, kN, kS;
    sor_nbrs<EXT>(l, nx, ny, i, j, kE, kW, kN, kS);
    double tx = phi[kE] - 2 * phi[k] + phi[kW], ty = phi[kN] - 2 * phi[k] + phi[kS];
    if (!UNIT) {  // x / 1 is x: unit cells skip the divisions, bit for bit
      tx = tx / dx2;
      ty = ty / dy2;
    }
    double R = (tx + ty) + (FLUID ? (a.rho[k] - exp(phi[k])) * a.K : src(k));
    sum += R * R;
  }
  sum = block_sum_1024(sum, red);
  return sqrt(sum / (nx * ny));
}

// FLUID: gsfluidsolver (src/field.cpp:7-68), Boltzmann electrons: the source
// is (rho - exp(phi)) K and the residual is checked every 50 sweeps.
// UNIT: dx = dy = 1 (every normalisation of the reference), where the
// divisions by dx^2 and dy^2 are identities and are skipped - bit for bit the
// same iterates, without the two FP64 divisions per node update that bound
// this one-SM kernel.  use_smem: phi in shared memory; 2: rho K as well,
// formed once per solve (the same product as in every sweep).
// EXT: an extension lattice (sor_lattice).  Its wrapped neighbours couple
// the first and last node of a periodic row or column, so sweep s may start
// node (i, 0) only after sweep s-1 has passed node (i, nyi-1): sweeps are
// spaced c = max(nxi or nyi of each periodic direction, 2) diagonals apart
// instead of 2, which keeps every read at the same sweep as the
// lexicographic order.  PERIODIC removes the source's mean before and phi's
// mean after the sweeps (exact sums, rounded once).
template <bool FLUID, bool UNIT, bool EXT>
__global__ void __launch_bounds__(SOR_THREADS) k_sor_lex(SolverArgs a, int use_smem) {
  extern __shared__ double smem[];
  __shared__ double red[40];
  const int nx = a.g.nx, ny = a.g.ny;
  const int nn = nx * ny;
  const SorLat l = sor_lattice(nx, ny, EXT ? a.poisson_bc : EPIC_POISSON_DIRICHLET);
  double* phi = use_smem ? smem : a.phi;
  double* const rK = !FLUID && use_smem == 2 ? smem + nn : nullptr;
  if (rK)
    for (int k = threadIdx.x; k < nn; k += blockDim.x) rK[k] = a.rho[k] * a.K;
  // PERIODIC: the mean of rho K over the unknowns, removed from the source.
  const int ni = l.nxi * l.nyi;
  auto unknown = [&](int q) { return (l.i0 + q / l.nyi) * ny + l.j0 + q % l.nyi; };
  double smean = 0.0;
  if (EXT && !FLUID && l.wrap_x) {
    __syncthreads();
    smean = block_exact_sum(ni, [&](int q) { const int k = unknown(q); return rK ? rK[k] : a.rho[k] * a.K; }, red) /
            (double)ni;
  }
  auto src = [&](int k) -> double { return (rK ? rK[k] : a.rho[k] * a.K) - smean; };
  const double dx2 = a.g.dx * a.g.dx, dy2 = a.g.dy * a.g.dy;
  const double coeff = (2 / dx2) + (2 / dy2);
  const double inv_coeff = 1 / coeff;
  for (int k = threadIdx.x; k < nn; k += blockDim.x) phi[k] = 0;  // cold start, zero edges (src/field.cpp:78-98)
  __syncthreads();
  const int nxi = l.nxi, nyi = l.nyi;
  const int D = nxi + nyi - 1;
  const int Lmax = nxi < nyi ? nxi : nyi;
  int cp = 2;  // diagonals between consecutive sweeps
  if (EXT) {
    if (l.wrap_x && nxi > cp) cp = nxi;
    if (l.wrap_y && nyi > cp) cp = nyi;
  }
  int iter = 0, converged = 0;
  double L2 = 0;
  if (nxi > 0 && nyi > 0) {
    while (iter < a.max_iter) {
      constexpr int P = FLUID ? 50 : 25;
      int S = iter == 0 ? 1 : P;
      if (S > a.max_iter - iter) S = a.max_iter - iter;
      const int T = D + cp * (S - 1);
      for (int t = 0; t < T; t++) {
        int s_lo = t - D + 1 > 0 ? (t - D + cp) / cp : 0;
        int s_hi = t / cp < S - 1 ? t / cp : S - 1;
        int items = (s_hi - s_lo + 1) * Lmax;
        for (int it = threadIdx.x; it < items; it += blockDim.x) {
          int s = s_lo + it / Lmax, q = it % Lmax;
          int d = t - cp * s;
          int a0 = d - (nyi - 1) > 0 ? d - (nyi - 1) : 0;
          int a1 = d < nxi - 1 ? d : nxi - 1;
          int ai = a0 + q;
          if (ai > a1) continue;
          int i = ai + l.i0, j = d - ai + l.j0;
          int k = i * ny + j;
          int kE, kW, kN, kS;
          sor_nbrs<EXT>(l, nx, ny, i, j, kE, kW, kN, kS);
          double tx = phi[kE] + phi[kW], ty = phi[kN] + phi[kS];
          if (!UNIT) {
            tx = tx / dx2;
            ty = ty / dy2;
          }
          const double sk = FLUID ? (a.rho[k] - exp(phi[k])) * a.K : src(k);
          double phi_new = inv_coeff * ((sk + tx) + ty);
          phi[k] = phi[k] + a.omega * (phi_new - phi[k]);
        }
        __syncthreads();
      }
      const int last = iter + S - 1;
      iter += S;
      if (last % P == 0) {
        L2 = sor_residual<FLUID, UNIT, EXT>(a, l, phi, src, red);
        if (L2 < a.tol) {
          converged = 1;
          break;
        }
      }
    }
  }
  if (EXT && l.wrap_x) {  // zero-mean gauge over the unknowns
    __syncthreads();
    const double m = block_exact_sum(ni, [&](int q) { return phi[unknown(q)]; }, red) / (double)ni;
    for (int q = threadIdx.x; q < ni; q += blockDim.x) {
      const int k = unknown(q);
      phi[k] = phi[k] - m;
    }
    __syncthreads();
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

// ---- lexicographic SOR over a thread-block cluster ----
// The pipelined wavefront of k_sor_lex spread over the C CTAs of one cluster
// (C <= 16): CTA c owns node rows [c R, c R + R) and keeps their phi (and
// rho K) in its shared memory.  At time step t every CTA updates the active
// nodes of its own rows; the rows beside its band, and the wrapped rows of a
// periodic lattice, are read from the owning CTA's shared memory through the
// cluster's distributed shared memory, and a cluster barrier (release /
// acquire) separates the time steps.  A node update is the same arithmetic
// as in k_sor_lex, in the same wavefront order, so the iterates are the same
// bit for bit.  The residual and the periodic means are exact sums over the
// cluster, rounded once, so every CTA takes the same convergence decision.
// The barrier is the hardware's cluster barrier: all CTAs of a cluster are
// resident together and run the same number of time steps.
constexpr int SORC_THREADS = 512;
constexpr int SORC_MAX = 16;
namespace cgx = cooperative_groups;

struct SorcXs {  // a CTA's share of an exact cluster sum
  int e;
  unsigned long long v[2];
};

// Exact sum of term(q), q in [0, count) of this CTA, over the cluster;
// the same value in every thread of every CTA.  Three cluster barriers.
template <class F>
__device__ double cluster_exact_sum(const cgx::cluster_group& cl, int count, const F& term, SorcXs* mine,
                                    double* red) {
  __shared__ int s_e[32];
  __shared__ unsigned long long s_v[32][2];
  __shared__ int s_A;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int C = (int)cl.num_blocks();
  int e = 0;
  for (int q = threadIdx.x; q < count; q += blockDim.x) e = max(e, xs_exponent(term(q)));
  e = (int)__reduce_max_sync(0xffffffffu, (unsigned)e);
  if (lane == 0) s_e[wid] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    int m = 0;
    for (int w = 0; w < nw; w++) m = max(m, s_e[w]);
    mine->e = m;
  }
  cl.sync();
  if (threadIdx.x == 0) {
    int m = 0;
    for (int r = 0; r < C; r++) m = max(m, cl.map_shared_rank(mine, r)->e);
    s_A = m;
  }
  __syncthreads();
  const int A = s_A;
  xs_int v = 0;
  for (int q = threadIdx.x; q < count; q += blockDim.x) v += xs_from_double(term(q), A);
  v = xs_warp_sum(v);
  if (lane == 0) {
    s_v[wid][0] = (unsigned long long)(xs_uint)v;
    s_v[wid][1] = (unsigned long long)((xs_uint)v >> 64);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    xs_uint tot = 0;
    for (int w = 0; w < nw; w++) tot += ((xs_uint)s_v[w][1] << 64) | s_v[w][0];
    mine->v[0] = (unsigned long long)tot;
    mine->v[1] = (unsigned long long)(tot >> 64);
  }
  cl.sync();
  if (threadIdx.x == 0) {
    xs_uint tot = 0;
    for (int r = 0; r < C; r++) {
      const SorcXs* o = cl.map_shared_rank(mine, r);
      tot += ((xs_uint)o->v[1] << 64) | o->v[0];
    }
    red[33] = xs_to_double((xs_int)tot, A);
  }
  cl.sync();  // the shares are read before they are rewritten; red[33] visible
  return red[33];
}

// with_rk: rho K of the band kept in shared memory after phi (not FLUID).
template <bool FLUID, bool UNIT, bool EXT>
__global__ void __launch_bounds__(SORC_THREADS) k_sor_cluster(SolverArgs a, int R, int with_rk, int K) {
  extern __shared__ double smem[];
  __shared__ double red[40];
  __shared__ double* s_row0[SORC_MAX];  // phi of each CTA's band (distributed shared memory)
  __shared__ SorcXs s_xs;
  const cgx::cluster_group cl = cgx::this_cluster();
  const int me = (int)cl.block_rank(), C = (int)cl.num_blocks();
  const int nx = a.g.nx, ny = a.g.ny;
  const SorLat l = sor_lattice(nx, ny, EXT ? a.poisson_bc : EPIC_POISSON_DIRICHLET);
  const int r_lo = me * R, r_hi = min(nx, r_lo + R);
  const int nloc = max(r_hi - r_lo, 0) * ny;
  const size_t band = (size_t)R * ny;
  double* const phi = smem;  // rows [r_lo, r_hi)
  double* const rK = with_rk ? smem + band : nullptr;
  double* const snaps = smem + band * (with_rk ? 2 : 1);  // K snapshot bands (undrained pipeline)
  if (threadIdx.x < C) s_row0[threadIdx.x] = threadIdx.x == me ? phi : cl.map_shared_rank(phi, (int)threadIdx.x);
  for (int q = threadIdx.x; q < nloc; q += blockDim.x) {
    phi[q] = 0;  // cold start, zero edges (src/field.cpp:78-98)
    if (rK) rK[q] = a.rho[(size_t)r_lo * ny + q] * a.K;
    for (int k = 0; k < K; k++) snaps[k * band + q] = 0;
  }
  // this CTA's unknowns: lattice rows ai in [u_lo, u_hi)
  const int u_lo = max(r_lo, l.i0) - l.i0, u_hi = min(r_hi, l.i0 + l.nxi) - l.i0;
  const int Ru = max(u_hi - u_lo, 0);
  const int nu = Ru * l.nyi;
  auto unknown_local = [&](int q) { return (u_lo + l.i0 - r_lo + q / l.nyi) * ny + l.j0 + q % l.nyi; };
  cl.sync();  // every band initialised (and every CTA running) before remote reads
  auto row_of = [&](int i) -> const double* {
    if (i >= r_lo && i < r_hi) return phi + (size_t)(i - r_lo) * ny;
    const int o = i / R;
    return s_row0[o] + (size_t)(i - o * R) * ny;
  };
  double smean = 0.0;
  if (EXT && !FLUID && l.wrap_x)
    smean = cluster_exact_sum(
                cl, nu,
                [&](int q) {
                  const int kl = unknown_local(q);
                  return rK ? rK[kl] : a.rho[(size_t)r_lo * ny + kl] * a.K;
                },
                &s_xs, red) /
            (double)(l.nxi * l.nyi);
  // the source at node (i, j) whose potential is v
  auto src = [&](int i, int j, int kl, double v) -> double {
    if (FLUID) return (a.rho[(size_t)i * ny + j] - exp(v)) * a.K;
    return (rK ? rK[kl] : a.rho[(size_t)i * ny + j] * a.K) - smean;
  };
  // neighbours of unknown (i, j): rows iE, iW and columns jN, jS (sor_nbrs)
  auto nbrs = [&](int i, int j, int& iE, int& iW, int& jN, int& jS) {
    iE = i + 1; iW = i - 1; jN = j + 1; jS = j - 1;
    if (EXT) {
      if (!(i + 1 < nx - 1 || !l.wrap_x)) iE = 0;
      if (i <= 0) iW = nx - 2;
      if (!(j + 1 < ny - 1)) jN = 0;
      if (j <= 0) jS = ny - 2;
    }
  };
  const double dx2 = a.g.dx * a.g.dx, dy2 = a.g.dy * a.g.dy;
  const double coeff = (2 / dx2) + (2 / dy2);
  const double inv_coeff = 1 / coeff;
  // L2 residual (src/field.cpp:121-134) of the band array buf (phi or a
  // snapshot; the other CTAs' bands at the same offset of their shared memory)
  auto residual = [&](double* buf) -> double {
    auto brow = [&](int i) -> const double* {
      if (i >= r_lo && i < r_hi) return buf + (size_t)(i - r_lo) * ny;
      const int o = i / R;
      return cl.map_shared_rank(buf, o) + (size_t)(i - o * R) * ny;
    };
    const double sum = cluster_exact_sum(
        cl, nu,
        [&](int q) {
          const int i = u_lo + l.i0 + q / l.nyi, j = l.j0 + q % l.nyi;
          const int kl = (i - r_lo) * ny + j;
          int iE, iW, jN, jS;
          nbrs(i, j, iE, iW, jN, jS);
          double tx = brow(iE)[j] - 2 * buf[kl] + brow(iW)[j];
          double ty = buf[kl - j + jN] - 2 * buf[kl] + buf[kl - j + jS];
          if (!UNIT) {
            tx = tx / dx2;
            ty = ty / dy2;
          }
          const double Rv = (tx + ty) + src(i, j, kl, buf[kl]);
          return Rv * Rv;
        },
        &s_xs, red);
    return sqrt(sum / (nx * ny));
  };
  const int nxi = l.nxi, nyi = l.nyi;
  const int D = nxi + nyi - 1;
  int cp = 2;
  if (EXT) {
    if (l.wrap_x && nxi > cp) cp = nxi;
    if (l.wrap_y && nyi > cp) cp = nyi;
  }
  constexpr int P = FLUID ? 50 : 25;  // residual after sweeps 0, P, 2P, ... (src/field.cpp:118)
  // sweep g's update of the node at lattice row ai on diagonal d (snap: also
  // store the new value there)
  auto update = [&](int d, int ai, double* snap) {
    const int i = ai + l.i0, j = d - ai + l.j0;
    const int kl = (i - r_lo) * ny + j;
    int iE, iW, jN, jS;
    nbrs(i, j, iE, iW, jN, jS);
    double tx = row_of(iE)[j] + row_of(iW)[j], ty = phi[kl - j + jN] + phi[kl - j + jS];
    if (!UNIT) {
      tx = tx / dx2;
      ty = ty / dy2;
    }
    const double sk = src(i, j, kl, phi[kl]);
    double phi_new = inv_coeff * ((sk + tx) + ty);
    const double v = phi[kl] + a.omega * (phi_new - phi[kl]);
    phi[kl] = v;
    if (snap) snap[kl] = v;
  };
  int iter = 0, converged = 0;
  double L2 = 0;
  double* out = phi;
  if (nxi > 0 && nyi > 0 && K > 0 && a.max_iter > 0) {
    // Undrained: one wavefront over all sweeps g < max_iter (sweep g on
    // diagonal d at step d + cp g).  The sweeps the reference checks write
    // their values into snapshot (g / P) % K as well; a checked sweep's
    // residual is taken from its snapshot at the step after its last
    // diagonal, and if it converged the snapshot is the result.  A snapshot
    // is rewritten cp K P >= D steps after its sweep started, i.e. after it
    // was checked.
    const long long G = a.max_iter;
    const long long t_end = (long long)D - 1 + (long long)cp * (G - 1);
    long long chk = 0;  // next checked sweep
    for (long long t = 0; t <= t_end + 1; t++) {
      if (chk < G && t == (long long)D + cp * chk) {
        double* sn = snaps + (size_t)((chk / P) % K) * band;
        L2 = residual(sn);
        iter = (int)(chk + 1);
        if (L2 < a.tol) {
          converged = 1;
          out = sn;
          break;
        }
        chk += P;
      }
      if (t > t_end) break;
      const long long g_lo = t - D + 1 > 0 ? (t - D + cp) / cp : 0;
      const long long g_hi = t / cp < G - 1 ? t / cp : G - 1;
      const int items = (int)(g_hi - g_lo + 1) * Ru;
      for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const long long g = g_lo + it / Ru;
        const int ai = u_lo + it % Ru;
        const int d = (int)(t - cp * g);
        const int a0 = d - (nyi - 1) > 0 ? d - (nyi - 1) : 0;
        const int a1 = d < nxi - 1 ? d : nxi - 1;
        if (ai < a0 || ai > a1) continue;
        update(d, ai, g % P == 0 ? snaps + (size_t)((g / P) % K) * band : nullptr);
      }
      cl.sync();
    }
    if (!converged) iter = (int)G;
  } else if (nxi > 0 && nyi > 0 && K == 0) {
    // Drained: chunks of sweeps up to the next check, each chunk's wavefront
    // emptied before its residual
    while (iter < a.max_iter) {
      int S = iter == 0 ? 1 : P;
      if (S > a.max_iter - iter) S = a.max_iter - iter;
      const int T = D + cp * (S - 1);
      for (int t = 0; t < T; t++) {
        const int s_lo = t - D + 1 > 0 ? (t - D + cp) / cp : 0;
        const int s_hi = t / cp < S - 1 ? t / cp : S - 1;
        const int items = (s_hi - s_lo + 1) * Ru;
        for (int it = threadIdx.x; it < items; it += blockDim.x) {
          const int s = s_lo + it / Ru, ai = u_lo + it % Ru;
          const int d = t - cp * s;
          const int a0 = d - (nyi - 1) > 0 ? d - (nyi - 1) : 0;
          const int a1 = d < nxi - 1 ? d : nxi - 1;
          if (ai < a0 || ai > a1) continue;
          update(d, ai, nullptr);
        }
        cl.sync();
      }
      const int last = iter + S - 1;
      iter += S;
      if (last % P == 0) {
        L2 = residual(phi);
        if (L2 < a.tol) {
          converged = 1;
          break;
        }
      }
    }
  }
  if (EXT && l.wrap_x) {  // zero-mean gauge over the unknowns
    const double m =
        cluster_exact_sum(cl, nu, [&](int q) { return out[unknown_local(q)]; }, &s_xs, red) / (double)(nxi * nyi);
    for (int q = threadIdx.x; q < nu; q += blockDim.x) {
      const int kl = unknown_local(q);
      out[kl] = out[kl] - m;
    }
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nloc; q += blockDim.x) a.phi[(size_t)r_lo * ny + q] = out[q];
  if (me == 0 && threadIdx.x == 0) {
    a.info->iterations = iter;
    a.info->converged = converged;
    a.info->error = L2;
    atomicAdd(a.iter_total, (unsigned long long)iter);
  }
  cl.sync();  // no CTA leaves while another may still read its band
}

// Whether the device can co-schedule a cluster of C CTAs of this kernel with
// this shared memory (asked once per kernel, size and shared memory).
static bool cluster_fits(const void* kern, int C, int threads, size_t smem) {
  static std::mutex mu;
  static std::map<std::tuple<const void*, int, size_t>, bool> known;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_tuple(kern, C, smem);
  const auto f = known.find(key);
  if (f != known.end()) return f->second;
  cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SOR_SMEM_MAX);
  cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(C);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int nclusters = 0;
  const bool ok = cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg) == cudaSuccess && nclusters >= 1;
  if (!ok) cudaGetLastError();
  known[key] = ok;
  return ok;
}

// The cluster for a lattice: about min(16, nx / 4) CTAs of R rows each, phi (and rho K when it fits) in shared memory; 0 when the lattice is
// too small, too large for the cluster's shared memory, or the device cannot
// co-schedule the cluster (k_sor_lex then runs it on one CTA).
struct SorCluster {
  int C, R, with_rk, K;
  size_t smem;
};

template <bool FLUID, bool UNIT, bool EXT>
static SorCluster sor_cluster_shape(const SolverArgs& a) {
  SorCluster c{0, 0, 0, 0, 0};
  const int nx = a.g.nx, ny = a.g.ny;
  int C = std::min(SORC_MAX, nx / 4);
  if (C < 2 || ny < 3) return c;
  const int R = (nx + C - 1) / C;
  C = (nx + R - 1) / R;  // no CTA without rows
  const size_t band = (size_t)R * ny * sizeof(double);
  if (band > SOR_SMEM_MAX) return c;
  // the lattice's wavefront (sor_lattice): D diagonals, sweeps cp apart
  const int pbc = EXT ? a.poisson_bc : EPIC_POISSON_DIRICHLET;
  const bool ext = pbc != EPIC_POISSON_DIRICHLET, wrap_x = pbc == EPIC_POISSON_PERIODIC;
  const int nxi = ext ? nx - 1 - (wrap_x ? 0 : 1) : nx - 2, nyi = ext ? ny - 1 : ny - 2;
  const int D = nxi + nyi - 1;
  int cp = 2;
  if (ext) {
    if (wrap_x && nxi > cp) cp = nxi;
    if (nyi > cp) cp = nyi;
  }
  const int P = FLUID ? 50 : 25;
  // snapshots for the undrained pipeline: a checked sweep's snapshot must
  // outlive the D steps until its check, cp K P >= D
  const int K = std::max(1, (D + cp * P - 1) / (cp * P));
  int with_rk = !FLUID && 2 * band <= SOR_SMEM_MAX;
  int k = 0;
  if (band * (1 + with_rk + K) <= SOR_SMEM_MAX) {
    k = K;
  } else if (band * (1 + K) <= SOR_SMEM_MAX) {
    k = K;
    with_rk = 0;
  }
  const size_t smem = band * (1 + with_rk + k);
  if (!cluster_fits((const void*)k_sor_cluster<FLUID, UNIT, EXT>, C, SORC_THREADS, smem)) return c;
  c.C = C;
  c.R = R;
  c.with_rk = with_rk;
  c.K = k;
  c.smem = smem;
  return c;
}

// Launches the cluster form when the lattice suits it; false otherwise.
template <bool FLUID, bool UNIT, bool EXT>
static bool launch_sor_cluster(cudaStream_t st, const SolverArgs& a) {
  const SorCluster c = sor_cluster_shape<FLUID, UNIT, EXT>(a);
  if (!c.C) return false;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = c.C;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.gridDim = dim3(c.C);
  cfg.blockDim = dim3(SORC_THREADS);
  cfg.dynamicSmemBytes = c.smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_sor_cluster<FLUID, UNIT, EXT>, a, c.R, c.with_rk, c.K) == cudaSuccess;
}

void init_field_kernels() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(k_sor_lex<false, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SOR_SMEM_MAX);
  cudaFuncSetAttribute(k_sor_lex<false, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SOR_SMEM_MAX);
  cudaFuncSetAttribute(k_sor_lex<true, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SOR_SMEM_MAX);
  cudaFuncSetAttribute(k_sor_lex<true, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SOR_SMEM_MAX);
  cudaFuncSetAttribute(k_sor_lex<false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SOR_SMEM_MAX);
  cudaFuncSetAttribute(k_sor_lex<false, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SOR_SMEM_MAX);
  done = true;
}

static bool sor_unit(const SolverArgs& a) { return a.g.dx == 1.0 && a.g.dy == 1.0; }

void launch_sor_lex(cudaStream_t st, const SolverArgs& a) {
  const size_t bytes = (size_t)a.g.nx * a.g.ny * sizeof(double);
  const int use_smem = 2 * bytes <= SOR_SMEM_MAX ? 2 : bytes <= SOR_SMEM_MAX ? 1 : 0;
  const size_t smem = use_smem * bytes;
  if (a.poisson_bc != EPIC_POISSON_DIRICHLET) {
    const bool cl = sor_unit(a) ? launch_sor_cluster<false, true, true>(st, a)
                                : launch_sor_cluster<false, false, true>(st, a);
    if (!cl) {
      if (sor_unit(a)) k_sor_lex<false, true, true><<<1, SOR_THREADS, smem, st>>>(a, use_smem);
      else k_sor_lex<false, false, true><<<1, SOR_THREADS, smem, st>>>(a, use_smem);
    }
    launch_fill_poisson_nodes(st, a.g, a.poisson_bc, a.phi);
    return;
  }
  if (sor_unit(a) ? launch_sor_cluster<false, true, false>(st, a) : launch_sor_cluster<false, false, false>(st, a))
    return;
  if (sor_unit(a)) k_sor_lex<false, true, false><<<1, SOR_THREADS, smem, st>>>(a, use_smem);
  else k_sor_lex<false, false, false><<<1, SOR_THREADS, smem, st>>>(a, use_smem);
}

// gsfluidsolver's edge values of rho (src/field.cpp:22-32): bottom 0, top
// 10000 eV/(k_B EV_to_K), then left and right 0 (so the top corners end 0).
__global__ void k_gsfluid_edges(Geom g, double* rho, double top) {
  const int nx = g.nx, ny = g.ny;
  for (int i = threadIdx.x; i < nx; i += blockDim.x) {
    rho[i * ny] = 0;
    rho[i * ny + ny - 1] = top;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < ny; j += blockDim.x) {
    rho[j] = 0;
    rho[(nx - 1) * ny + j] = 0;
  }
}

void launch_gsfluid(cudaStream_t st, const SolverArgs& a, double* rho) {
  k_gsfluid_edges<<<1, 256, 0, st>>>(a.g, rho, 10000 * (QE / (K_B * (QE / K_B))));
  const size_t bytes = (size_t)a.g.nx * a.g.ny * sizeof(double);
  const int use_smem = bytes <= SOR_SMEM_MAX;
  if (sor_unit(a) ? launch_sor_cluster<true, true, false>(st, a) : launch_sor_cluster<true, false, false>(st, a))
    return;
  if (sor_unit(a)) k_sor_lex<true, true, false><<<1, SOR_THREADS, use_smem ? bytes : 0, st>>>(a, use_smem);
  else k_sor_lex<true, false, false><<<1, SOR_THREADS, use_smem ? bytes : 0, st>>>(a, use_smem);
}

// ------------------------------------------------------ Newton hybrid ---
// FieldSolve::nrpcgsolver (src/field.cpp:141-210): ten Newton steps on
// A x - rhovec = 0 with rhovec += exp(x) K each step (the reference
// accumulates it) and J = A - diag(exp(x)), each solved by the dense cg of
// linearalgebra/solvers.h:33-69 (from 0, |r| < 1e-4, at most min(n, 10000)
// iterations).  A is pcgsolver's 5-point matrix on the flattened vector (row
// k / nx, column k % nx); the matrix-vector products sum the five entries in
// ascending column order, which is the dense product's sum (its zero entries
// leave it unchanged).  vec::operator* sums its rounded products serially in
// index order; here the same rounded products are summed exactly over the
// CTA and rounded once (block_exact_sum), which differs from the serial sum
// only by that sum's own rounding errors - a serial chain of dependent FP64
// additions, one per node, would bound every CG iteration.  One CTA; vectors
// in the solver workspace.
__device__ __forceinline__ double nr_row(int nx, int ny, int k, double diag, const double* v) {
  const int row = k / nx, col = k - row * nx;
  double sum = 0;
  if (row > 0) sum += 1.0 * v[k - nx];
  if (col > 0) sum += 1.0 * v[k - 1];
  sum += diag * v[k];
  if (col < nx - 1) sum += 1.0 * v[k + 1];
  if (row < ny - 1) sum += 1.0 * v[k + nx];
  return sum;
}

// (u, v): the rounded products u[i] * v[i] (the kernel is built without
// contraction), summed exactly and rounded once.
__device__ __forceinline__ double nr_dot(const double* u, const double* v, int n, double* red) {
  return block_exact_sum(n, [&](int k) { return u[k] * v[k]; }, red);
}

__global__ void __launch_bounds__(1024) k_nrpcg(SolverArgs a) {
  __shared__ double red[40];
  const int nx = a.g.nx, ny = a.g.ny, n = nx * ny;
  const double dx2 = a.g.dx * a.g.dx;
  const double K = a.K;
  double *rhovec = a.work[0], *x = a.work[1], *F = a.work[2], *J = a.work[3];
  double *y = a.work[4], *r = a.work[5], *p = a.work[6], *Ap = a.work[7];
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int i = k / ny, j = k - i * ny;
    rhovec[k] = (j == 0 || j == ny - 1 || i == 0 || i == nx - 1) ? 0.0 : -a.rho[k] * dx2 * K;
    x[k] = 0;
  }
  __syncthreads();
  const int maxit = n < 10000 ? n : 10000;
  long long total = 0;
  for (int it = 0; it < 10; it++) {
    for (int k = threadIdx.x; k < n; k += blockDim.x) rhovec[k] = rhovec[k] + exp(x[k]) * K;
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      F[k] = nr_row(nx, ny, k, -4.0, x) - rhovec[k];
      J[k] = -4 - exp(x[k]);
      y[k] = 0;
      r[k] = F[k] - 0.0;
      p[k] = r[k];
    }
    __syncthreads();
    double r02 = nr_dot(r, r, n, red);
    for (int i = 0; i < maxit; i++) {
      if (sqrt(r02) < 1e-4) break;
      for (int k = threadIdx.x; k < n; k += blockDim.x) Ap[k] = nr_row(nx, ny, k, J[k], p);
      __syncthreads();
      const double pAp = nr_dot(p, Ap, n, red);
      const double alpha = r02 / pAp;
      for (int k = threadIdx.x; k < n; k += blockDim.x) {
        y[k] = y[k] + p[k] * alpha;
        r[k] = r[k] - Ap[k] * alpha;
      }
      __syncthreads();
      const double r12 = nr_dot(r, r, n, red);
      const double beta = r12 / r02;
      for (int k = threadIdx.x; k < n; k += blockDim.x) p[k] = r[k] + p[k] * beta;
      __syncthreads();
      r02 = r12;
      total++;
    }
    for (int k = threadIdx.x; k < n; k += blockDim.x) x[k] = x[k] - y[k];
    __syncthreads();
  }
  for (int k = threadIdx.x; k < n; k += blockDim.x) a.phi[k] = x[k];
  if (threadIdx.x == 0) {
    a.info->iterations = (int)total;
    a.info->converged = 1;
    a.info->error = 0;  // domain.error = 0 (src/field.cpp:205)
    atomicAdd(a.iter_total, (unsigned long long)total);
  }
}

// The same solve over a thread-block cluster: CTA c owns the nodes
// [c per, c per + per) of the flattened vector and updates them; the
// matrix-vector products read the neighbours' p (and x) from L2 after a
// cluster barrier.  A dot product is summed exactly per CTA against the
// CTA's own anchor, and the C CTA totals are aligned to the largest anchor
// (bits below 2^-106 of the largest term dropped, a fixed rule) and added in
// every warp after one cluster barrier: each CTA obtains the same value, so
// every CTA takes the same CG and Newton decisions.
constexpr int NRC_THREADS = 128;
struct NrSlot {
  int e;
  unsigned long long v[2];
};

// mine: this call's slot; successive calls alternate between two slots, so a
// slot is rewritten only after every CTA has passed the barrier of the call
// in between, i.e. after every CTA has read it.
template <class F>
__device__ __forceinline__ double nrc_sum(const cgx::cluster_group& cl, int lo, int hi, const F& term, NrSlot* mine) {
  __shared__ int s_e[NRC_THREADS / 32];
  __shared__ unsigned long long s_v[NRC_THREADS / 32][2];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int C = (int)cl.num_blocks();
  int e = 0;
  for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) e = max(e, xs_exponent(term(k)));
  e = (int)__reduce_max_sync(0xffffffffu, (unsigned)e);
  if (lane == 0) s_e[wid] = e;
  __syncthreads();
  int Ac = 0;
  for (int w = 0; w < NRC_THREADS / 32; w++) Ac = max(Ac, s_e[w]);
  xs_int v = 0;
  for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) v += xs_from_double(term(k), Ac);
  v = xs_warp_sum(v);
  if (lane == 0) {
    s_v[wid][0] = (unsigned long long)(xs_uint)v;
    s_v[wid][1] = (unsigned long long)((xs_uint)v >> 64);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    xs_uint tot = 0;
    for (int w = 0; w < NRC_THREADS / 32; w++) tot += ((xs_uint)s_v[w][1] << 64) | s_v[w][0];
    mine->e = Ac;
    mine->v[0] = (unsigned long long)tot;
    mine->v[1] = (unsigned long long)(tot >> 64);
  }
  cl.sync();
  int er = 0;
  xs_int vr = 0;
  if (lane < C) {
    const NrSlot* o = cl.map_shared_rank(mine, lane);
    er = o->e;
    vr = (xs_int)(((xs_uint)o->v[1] << 64) | o->v[0]);
  }
  const int A = (int)__reduce_max_sync(0xffffffffu, (unsigned)er);
  vr >>= min(A - er, 127);
  const xs_int tot = xs_warp_sum(vr);
  return xs_to_double(tot, A);
}

// Row k of the matrix-vector product with v distributed over the cluster's
// shared memory: node q lives in CTA q / per at index q % per (base[] holds
// each CTA's array in the distributed shared memory window).
__device__ __forceinline__ double nr_row_dsm(int nx, int ny, int k, double diag, double* const* base, int per,
                                             int lo, int hi, const double* own) {
  auto at = [&](int q) -> double {
    if (q >= lo && q < hi) return own[q - lo];
    const int o = q / per;
    return base[o][q - o * per];
  };
  const int row = k / nx, col = k - row * nx;
  double sum = 0;
  if (row > 0) sum += 1.0 * at(k - nx);
  if (col > 0) sum += 1.0 * at(k - 1);
  sum += diag * own[k - lo];
  if (col < nx - 1) sum += 1.0 * at(k + 1);
  if (row < ny - 1) sum += 1.0 * at(k + nx);
  return sum;
}

// Shared memory of a CTA: seven arrays of per doubles (rhovec, x, J, y, r,
// p, Ap); x and p are read by the other CTAs for their products.
constexpr int NRC_ARRAYS = 7;

__global__ void __launch_bounds__(NRC_THREADS) k_nrpcg_cluster(SolverArgs a, int per) {
  extern __shared__ double sv[];
  __shared__ NrSlot s_slots[2];
  __shared__ double* s_xb[SORC_MAX];
  __shared__ double* s_pb[SORC_MAX];
  const cgx::cluster_group cl = cgx::this_cluster();
  const int me = (int)cl.block_rank(), C = (int)cl.num_blocks();
  const int nx = a.g.nx, ny = a.g.ny, n = nx * ny;
  const int lo = me * per, hi = min(n, lo + per);
  const double dx2 = a.g.dx * a.g.dx;
  const double K = a.K;
  double *rhovec = sv, *x = sv + per, *J = sv + 2 * per, *y = sv + 3 * per;
  double *r = sv + 4 * per, *p = sv + 5 * per, *Ap = sv + 6 * per;
  if (threadIdx.x < C) {
    s_xb[threadIdx.x] = cl.map_shared_rank(x, (int)threadIdx.x);
    s_pb[threadIdx.x] = cl.map_shared_rank(p, (int)threadIdx.x);
  }
  int parity = 0;
  // every thread touches the same nodes k = lo + threadIdx.x + m blockDim in
  // every loop, so an array read only at its own nodes needs no barrier
  for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) {
    const int i = k / ny, j = k - i * ny;
    rhovec[k - lo] = (j == 0 || j == ny - 1 || i == 0 || i == nx - 1) ? 0.0 : -a.rho[k] * dx2 * K;
    x[k - lo] = 0;
  }
  cl.sync();
  const int maxit = n < 10000 ? n : 10000;
  long long total = 0;
  for (int it = 0; it < 10; it++) {
    for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) {
      const int q = k - lo;
      const double xk = x[q];
      rhovec[q] = rhovec[q] + exp(xk) * K;
      const double F = nr_row_dsm(nx, ny, k, -4.0, s_xb, per, lo, hi, x) - rhovec[q];
      J[q] = -4 - exp(xk);
      y[q] = 0;
      r[q] = F - 0.0;
    }
    // p = r: the other CTAs last read p before the barrier of the previous
    // step's last sum
    for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) p[k - lo] = r[k - lo];
    double r02 = nrc_sum(cl, lo, hi, [&](int k) { return r[k - lo] * r[k - lo]; }, s_slots + parity);
    parity ^= 1;  // the barrier above: p visible, x reads done
    for (int i = 0; i < maxit; i++) {
      if (xs_bits(r02) < a.tol_bits) break;  // sqrt(r02) < 1e-4 (r02 >= 0: bit order is value order)
      for (int k = lo + threadIdx.x; k < hi; k += blockDim.x)
        Ap[k - lo] = nr_row_dsm(nx, ny, k, J[k - lo], s_pb, per, lo, hi, p);
      const double pAp = nrc_sum(cl, lo, hi, [&](int k) { return p[k - lo] * Ap[k - lo]; }, s_slots + parity);
      parity ^= 1;  // the barrier above: every CTA's reads of p done
      const double alpha = r02 / pAp;
      for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) {
        const int q = k - lo;
        y[q] = y[q] + p[q] * alpha;
        r[q] = r[q] - Ap[q] * alpha;
      }
      const double r12 = nrc_sum(cl, lo, hi, [&](int k) { return r[k - lo] * r[k - lo]; }, s_slots + parity);
      parity ^= 1;
      const double beta = r12 / r02;
      for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) p[k - lo] = r[k - lo] + p[k - lo] * beta;
      cl.sync();  // p of every CTA visible to the next product
      r02 = r12;
      total++;
    }
    for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) x[k - lo] = x[k - lo] - y[k - lo];
    cl.sync();  // x of every CTA visible to the next Newton step
  }
  for (int k = lo + threadIdx.x; k < hi; k += blockDim.x) a.phi[k] = x[k - lo];
  if (me == 0 && threadIdx.x == 0) {
    a.info->iterations = (int)total;
    a.info->converged = 1;
    a.info->error = 0;  // domain.error = 0 (src/field.cpp:205)
    atomicAdd(a.iter_total, (unsigned long long)total);
  }
  cl.sync();  // no CTA leaves while another may still read its arrays
}

// Cluster of about n / 40 CTAs (2 to 16) when its arrays fit the CTAs'
// shared memory and the device can co-schedule it; one CTA otherwise.
void launch_nrpcg(cudaStream_t st, const SolverArgs& a) {
  const int n = a.g.nx * a.g.ny;
  int C = std::min(SORC_MAX, n / 40);
  const int per = C >= 2 ? (n + C - 1) / C : 0;
  const size_t smem = (size_t)NRC_ARRAYS * per * sizeof(double);
  if (C >= 2 && smem <= SOR_SMEM_MAX) {
    C = (n + per - 1) / per;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(C);
    cfg.blockDim = dim3(NRC_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    SolverArgs an = a;
    an.tol_bits = xs_bits(xs_sqrt_threshold(1e-4));  // the cg's stop test, |r| < 1e-4
    if (cluster_fits((const void*)k_nrpcg_cluster, C, NRC_THREADS, smem) &&
        cudaLaunchKernelEx(&cfg, k_nrpcg_cluster, an, per) == cudaSuccess)
      return;
    cudaGetLastError();
  }
  k_nrpcg<<<1, 1024, 0, st>>>(a);
}

// ------------------------------------------------------ grid barrier ---
// Cooperative launches guarantee that all blocks are resident.  bar[0] counts
// arrivals since the launch (zeroed before it): the blocks of barrier episode
// e draw tickets in [e*nb, (e+1)*nb) and wait until the count reaches
// (e+1)*nb.  Every wait gives up after a bounded number of polls (the
// launch's SolverArgs::spin; FLAG_TIMEOUT), so a fault can never hang the GPU.
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

__device__ bool grid_sync(unsigned int* bar, int* flags, long long limit) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int ticket = atom_add_release_gpu(bar, 1u);
    const unsigned int target = (ticket / gridDim.x + 1) * gridDim.x;
    int ok = 1;
    long long spins = 0;
    while ((int)(ld_acquire_gpu(bar) - target) < 0) {
      if (++spins >= limit) {
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
  __shared__ double s_alpha, s_beta, s_mean;
  __shared__ int s_done;
  // The unknowns as a lattice (Lattice): vectors are indexed by lattice
  // position q = row * C + col, x lives in phi at the node of q.  For the
  // reference's lattice q is the node index itself.
  const Lattice lat = make_lattice(a.g.nx, a.g.ny, a.poisson_bc);
  const int R = lat.R, C = lat.C;
  const int n = R * C;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int stride = gridDim.x * blockDim.x;
  const int nb = gridDim.x;
  const long long spin = spin_or_default(a.spin);
  double* x = a.phi;
  double* b = a.work[0];
  double* R_[2] = {a.work[1], a.work[2]};
  double* S[2] = {a.work[3], a.work[4]};
  double* W[2] = {a.work[5], a.work[6]};
  double* Pd = a.work[7];
  // Partials [2][nb][4], alternating by reduction episode: a block can run
  // at most one reduction ahead of the slowest reader.
  int ep = 0;
  auto Pb = [&](int e) { return a.partials + (e & 1) * 4 * nb; };
  const double minv = 1.0 / -4.0;
  const double dx2 = a.g.dx * a.g.dx;
  auto node = [&](int q) { const int row = q / C; return lattice_node(lat, row, q - row * C); };
  // Lattice neighbours of q (row - 1, col - 1, col + 1, row + 1), or -1.
  auto nbrs = [&](int q, int& up, int& lf, int& rt, int& dn) {
    const int row = q / C, col = q - row * C;
    const int ru = lattice_wrap(row - 1, R, lat.wrap_r), rd = lattice_wrap(row + 1, R, lat.wrap_r);
    const int cl = lattice_wrap(col - 1, C, lat.wrap_c), cr = lattice_wrap(col + 1, C, lat.wrap_c);
    up = ru < 0 ? -1 : ru * C + col;
    dn = rd < 0 ? -1 : rd * C + col;
    lf = cl < 0 ? -1 : row * C + cl;
    rt = cr < 0 ? -1 : row * C + cr;
  };

  // b: the reference's right-hand side (zero on the grid edges) or -rho dx^2 K
  // on every unknown of an extension lattice; PERIODIC projects it onto zero
  // mean.
  double pb = 0;
  for (int q = tid; q < n; q += stride) {
    const int k = node(q);
    double bk;
    if (lat.mode == EPIC_POISSON_DIRICHLET) {
      const int i = k / a.g.ny;
      bk = rhs_at(a, k, i, k - i * a.g.ny, dx2);
    } else {
      bk = -a.rho[k] * dx2 * a.K;
    }
    b[q] = bk;
    pb += bk;
  }
  if (lat.mode == EPIC_POISSON_PERIODIC) {
    block_partial3(pb, 0.0, 0.0, Pb(ep), sw);
    if (!grid_sync(a.bar, a.flags, spin)) return;
    double3 t = grid_total3_t0(Pb(ep++), nb);
    if (threadIdx.x == 0) s_mean = t.x / (double)n;
    __syncthreads();
    const double bm = s_mean;
    for (int q = tid; q < n; q += stride) b[q] = b[q] - bm;
  }
  if (!grid_sync(a.bar, a.flags, spin)) return;

  // set-up: x = 0, r = b - A*0, u = M r, w = A u, p = s = 0.
  double pg = 0, pd = 0, pr = 0;
  for (int q = tid; q < n; q += stride) {
    x[node(q)] = 0;
    const double rk = __ldcg(&b[q]) - 0.0;
    const double uk = minv * rk;
    int up, lf, rt, dn;
    nbrs(q, up, lf, rt, dn);
    double sum = 0;
    if (up >= 0) sum += minv * __ldcg(&b[up]);
    if (lf >= 0) sum += minv * __ldcg(&b[lf]);
    sum = fma(-4.0, uk, sum);
    if (rt >= 0) sum += minv * __ldcg(&b[rt]);
    if (dn >= 0) sum += minv * __ldcg(&b[dn]);
    R_[0][q] = rk;
    W[0][q] = sum;
    S[0][q] = 0;
    Pd[q] = 0;
    pg = fma(rk, uk, pg);
    pd = fma(sum, uk, pd);
    pr = fma(rk, rk, pr);
  }
  block_partial3(pg, pd, pr, Pb(ep), sw);
  if (!grid_sync(a.bar, a.flags, spin)) return;
  // min(n*n, max_iteration) as pcg() caps it: n*n in 32-bit int arithmetic for
  // the reference's lattice (it wraps, as there), in 64 bits for the extensions.
  unsigned int cap32 = (unsigned int)n * (unsigned int)n;
  const long long cap = lat.mode == EPIC_POISSON_DIRICHLET ? (long long)(int)cap32 : (long long)n * n;
  const int maxit = cap < a.max_iter ? (int)cap : a.max_iter;
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
    double3 t = grid_total3_t0(Pb(ep++), nb);
    if (threadIdx.x == 0) scalars(t);
    __syncthreads();
  }
  while (it < maxit && !s_done) {
    const double al = s_alpha, be = s_beta;
    const double* Rc = R_[cur];
    const double* Sc = S[cur];
    const double* Wc = W[cur];
    double* Rn = R_[cur ^ 1];
    double* Sn = S[cur ^ 1];
    double* Wn = W[cur ^ 1];
    pg = pd = pr = 0;
    for (int q = tid; q < n; q += stride) {
      const int k = node(q);
      const double rc = __ldcg(&Rc[q]);
      const double sk = fma(be, __ldcg(&Sc[q]), __ldcg(&Wc[q]));
      const double pk = fma(be, Pd[q], minv * rc);
      x[k] = fma(al, pk, x[k]);
      const double rk = fma(-al, sk, rc);
      const double uk = minv * rk;
      // w_new = A u_new; a neighbour's u_new from its previous r, w, s.  The
      // loads use clamped indices so all of them issue before the first
      // use; missing neighbours are then skipped as in the reference.
      int up, lf, rt, dn;
      nbrs(q, up, lf, rt, dn);
#define UNEW(m) (minv * fma(-al, fma(be, __ldcg(&Sc[m]), __ldcg(&Wc[m])), __ldcg(&Rc[m])))
      const double uN = UNEW(up >= 0 ? up : q);
      const double uW = UNEW(lf >= 0 ? lf : q);
      const double uE = UNEW(rt >= 0 ? rt : q);
      const double uS = UNEW(dn >= 0 ? dn : q);
#undef UNEW
      double sum = 0;
      if (up >= 0) sum += uN;
      if (lf >= 0) sum += uW;
      sum = fma(-4.0, uk, sum);
      if (rt >= 0) sum += uE;
      if (dn >= 0) sum += uS;
      Pd[q] = pk;
      Sn[q] = sk;
      Rn[q] = rk;
      Wn[q] = sum;
      pg = fma(rk, uk, pg);
      pd = fma(sum, uk, pd);
      pr = fma(rk, rk, pr);
    }
    block_partial3(pg, pd, pr, Pb(ep), sw);
    if (!grid_sync(a.bar, a.flags, spin)) return;
    cur ^= 1;
    it++;
    {
      double3 t = grid_total3_t0(Pb(ep++), nb);
      if (threadIdx.x == 0) scalars(t);
      __syncthreads();
    }
  }
  // domain.error = |A x - b| / n (src/field.cpp:258-259, n = nx ny); x is
  // complete everywhere after the last barrier.  PERIODIC also totals x for
  // the zero-mean gauge (the error is that of x before the shift).
  double pe = 0, px = 0;
  for (int q = tid; q < n; q += stride) {
    int up, lf, rt, dn;
    nbrs(q, up, lf, rt, dn);
    const int k = node(q);
    double sum = 0;
    if (up >= 0) sum += __ldcg(&x[node(up)]);
    if (lf >= 0) sum += __ldcg(&x[node(lf)]);
    sum = fma(-4.0, __ldcg(&x[k]), sum);
    if (rt >= 0) sum += __ldcg(&x[node(rt)]);
    if (dn >= 0) sum += __ldcg(&x[node(dn)]);
    const double e = sum - b[q];
    pe = fma(e, e, pe);
    px += __ldcg(&x[k]);
  }
  block_partial3(pe, px, 0.0, Pb(ep), sw);
  if (!grid_sync(a.bar, a.flags, spin)) return;
  double3 e2 = grid_total3_t0(Pb(ep++), nb);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.info->iterations = it;
    a.info->converged = it < maxit;
    a.info->error = sqrt(e2.x) / (a.g.nx * a.g.ny);
    atomicAdd(a.iter_total, (unsigned long long)it);
  }
  if (lat.mode == EPIC_POISSON_PERIODIC) {
    if (threadIdx.x == 0) s_mean = e2.y / (double)n;
    __syncthreads();
    const double xm = s_mean;
    for (int q = tid; q < n; q += stride) {
      const int k = node(q);
      x[k] = x[k] - xm;
    }
  }
}

// Computed on first use (several host threads may race to do it; they all
// store the same value).
static std::atomic<int> g_pcg_max_blocks{0};

int solver_max_blocks() {
  int v = g_pcg_max_blocks.load(std::memory_order_relaxed);
  if (!v) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg, 256, 0);
    if (per_sm < 1) per_sm = 1;
    v = sms * (per_sm < 2 ? per_sm : 2);
    g_pcg_max_blocks.store(v, std::memory_order_relaxed);
  }
  return v;
}

// ------------------------------------------------------ tiled PCG ---
// The same Chronopoulos-Gear iteration as k_pcg, with the unknowns held in
// registers for the whole solve.  The lattice of unknowns (R = ny rows of
// C = nx columns, row = k / nx as in the reference's dense A) is cut into
// one tr x tc tile per CTA; each thread owns up to NPT nodes of its tile and
// keeps their x, r, w, p, s in registers.  The stencil reads r from a
// shared-memory copy of the tile with a one-node halo ring: halo nodes belong
// to neighbouring tiles, whose owners publish r, w, s of their edge nodes
// (double-buffered by iteration parity) before the grid barrier, so after it
// each CTA recomputes the halo's new r - alpha(w + beta s) from them.
//
// Exact identities of the constant Jacobi diagonal -4 remove M from the
// loop: with u = M r = -r/4 every product with u is an exact power-of-two
// scaling, so w = A u = fma(-1/4, sum of the neighbours' r, r), (w, u) =
// -(w, r)/4, gamma = (r, u) = -(r, r)/4, and p is kept as p' = -4p (p' = r +
// beta p', x += (-alpha/4) p').  All of these round exactly as the unscaled
// forms do.  That leaves 10 FP64 operations per node and iteration, and the
// p'/x updates (needed only for the answer) run while the CTA waits at the
// grid barrier, so 8 are on the critical path.  The iteration's scalars need
// one division there: beta = gamma * (1/gamma_prev), with the reciprocal
// formed while waiting, and eta = delta - beta*gamma/alpha_prev =
// delta - beta^2 eta_prev (alpha_prev = gamma_prev/eta_prev), formed as
// delta - gamma^2 (eta_prev/gamma_prev^2) with the second factor also formed
// while waiting; alpha = gamma/eta by div_nr.
//
// One grid-wide synchronisation per iteration carries both dot products: the
// CTAs add their fixed-point partials into counted words of a slot (see
// PCG_SLOT_WORDS), so the poll that ends the barrier also returns the totals.
// The first iteration, and any whose terms outgrow the anchors, reduce
// through block-anchored partials and the counter barrier instead.
struct PcgTiling {
  int tr, tc;          // tile rows, columns
  int tiles_c;         // tiles per lattice row
  int blocks;          // CTAs (tiles)
  int npt;             // owned-node slots per thread
};

constexpr int PCG_T = 256;
constexpr int PCG_HALO_SLOTS = 2;    // halo nodes per thread (the halo ring holds <= 512)
constexpr int PCG_MAX_BLOCKS = 160;  // partial records read per lane: PCG_MAX_BLOCKS / 32

// Split grid barrier: each CTA counts its own barrier episodes, so arriving
// needs no returned ticket (a fire-and-forget red.release by thread 0 after a
// __syncthreads that orders the block's writes before it), and work that no
// other CTA needs can run between arriving and waiting.
__device__ __forceinline__ void bar_arrive(unsigned int* bar) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(bar), "r"(1u) : "memory");
}

// Waits until `target` arrivals are in (bounded: FLAG_TIMEOUT and false on
// giving up).  Ends with a __syncthreads.
__device__ __forceinline__ bool bar_wait(unsigned int* bar, int* flags, unsigned int target, int* s_ok,
                                         long long limit) {
  if (threadIdx.x == 0) {
    int ok = 1;
    long long spins = 0;
    while ((int)(ld_acquire_gpu(bar) - target) < 0) {
      if (++spins >= limit) {
        atomicOr(flags, FLAG_TIMEOUT);
        ok = 0;
        break;
      }
    }
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok;
}

// One CTA's exact partial of two dot products: V = sum * 2^(1129 - a).
struct XPartial {
  unsigned long long lo[2];
  long long hi[2];
  int a[2];
  int pad[2];
};

struct XScratch {
  int e[2][PCG_T / 32];
  unsigned long long v[2][PCG_T / 32][2];
};

// Block partial of the terms t0[j], t1[j] (j < NT) of every thread; thread 0
// stores it to *out.  Two __syncthreads (anchor exponents, warp totals).
template <int NT>
__device__ __forceinline__ void xs_block_partial(const double (&t0)[NT], const double (&t1)[NT], XScratch& sx,
                                                 XPartial* out) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int e0 = 0, e1 = 0;
#pragma unroll
  for (int j = 0; j < NT; j++) {
    e0 = max(e0, xs_exponent(t0[j]));
    e1 = max(e1, xs_exponent(t1[j]));
  }
  e0 = (int)__reduce_max_sync(0xffffffffu, (unsigned)e0);
  e1 = (int)__reduce_max_sync(0xffffffffu, (unsigned)e1);
  if (lane == 0) {
    sx.e[0][wid] = e0;
    sx.e[1][wid] = e1;
  }
  __syncthreads();
  int A0 = 0, A1 = 0;
#pragma unroll
  for (int w = 0; w < PCG_T / 32; w++) {
    A0 = max(A0, sx.e[0][w]);
    A1 = max(A1, sx.e[1][w]);
  }
  xs_int v0 = 0, v1 = 0;
#pragma unroll
  for (int j = 0; j < NT; j++) {
    v0 += xs_from_double(t0[j], A0);
    v1 += xs_from_double(t1[j], A1);
  }
  v0 = xs_warp_sum(v0);
  v1 = xs_warp_sum(v1);
  if (lane == 0) {
    sx.v[0][wid][0] = (unsigned long long)(xs_uint)v0;
    sx.v[0][wid][1] = (unsigned long long)((xs_uint)v0 >> 64);
    sx.v[1][wid][0] = (unsigned long long)(xs_uint)v1;
    sx.v[1][wid][1] = (unsigned long long)((xs_uint)v1 >> 64);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    xs_uint s0 = 0, s1 = 0;
#pragma unroll
    for (int w = 0; w < PCG_T / 32; w++) {
      s0 += ((xs_uint)sx.v[0][w][1] << 64) | sx.v[0][w][0];
      s1 += ((xs_uint)sx.v[1][w][1] << 64) | sx.v[1][w][0];
    }
    XPartial p;
    p.lo[0] = (unsigned long long)s0;
    p.hi[0] = (long long)(s0 >> 64);
    p.lo[1] = (unsigned long long)s1;
    p.hi[1] = (long long)(s1 >> 64);
    p.a[0] = A0;
    p.a[1] = A1;
    p.pad[0] = p.pad[1] = 0;
    *out = p;
  }
}

// Grid totals of the nb partials, by warp 0 (all loads issued first); the
// doubles are valid in thread 0.
__device__ __forceinline__ void xs_grid_totals_w0(const XPartial* Pc, int nb, double* out0, double* out1) {
  constexpr int Q = PCG_MAX_BLOCKS / 32;
  ulonglong2 r01[Q], r23[Q];
  int2 ra[Q];
#pragma unroll
  for (int q = 0; q < Q; q++) {
    const int k = threadIdx.x + 32 * q;
    if (k < nb) {
      const ulonglong2* rec = reinterpret_cast<const ulonglong2*>(Pc + k);
      r01[q] = __ldcg(rec);
      r23[q] = __ldcg(rec + 1);
      ra[q] = __ldcg(reinterpret_cast<const int2*>(rec + 2));
    } else {
      r01[q] = make_ulonglong2(0, 0);
      r23[q] = make_ulonglong2(0, 0);
      ra[q] = make_int2(0, 0);
    }
  }
  int a0 = 0, a1 = 0;
#pragma unroll
  for (int q = 0; q < Q; q++) {
    a0 = max(a0, ra[q].x);
    a1 = max(a1, ra[q].y);
  }
  const int A0 = (int)__reduce_max_sync(0xffffffffu, (unsigned)a0);
  const int A1 = (int)__reduce_max_sync(0xffffffffu, (unsigned)a1);
  xs_int s0 = 0, s1 = 0;
#pragma unroll
  for (int q = 0; q < Q; q++) {
    // record layout: lo[0], lo[1] | hi[0], hi[1] | a[0], a[1]
    const xs_int v0 = (xs_int)(((xs_uint)r23[q].x << 64) | r01[q].x);
    const xs_int v1 = (xs_int)(((xs_uint)r23[q].y << 64) | r01[q].y);
    s0 += xs_realign(v0, ra[q].x, A0);
    s1 += xs_realign(v1, ra[q].y, A1);
  }
  s0 = xs_warp_sum(s0);
  s1 = xs_warp_sum(s1);
  // Lanes 0 and 1 round one total each, side by side.
  const double d = xs_to_double(threadIdx.x == 0 ? s0 : s1, threadIdx.x == 0 ? A0 : A1);
  const double d1 = __shfl_sync(0xffffffffu, d, 1);
  if (threadIdx.x == 0) {
    *out0 = d;
    *out1 = d1;
  }
}

// 1/x by Newton-Raphson (y <- y + y(1 - m y), two steps) on the significand m
// of x, seeded with the FP32 reciprocal of m's leading 24 bits: the ~2^-23
// seed error squares to below FP64 rounding, so the result is within about
// one ulp of 1/x (not correctly rounded).  The exponent is applied in the
// integer domain.  Four dependent FP64 operations in all, against a library
// division's longer sequence; for x and 1/x in the normal range (otherwise
// the library division is used).
__device__ __forceinline__ double recip_nr(double x) {
  const uint64_t b = xs_bits(x);
  const int e = (int)((b >> 52) & 0x7FF);
  const uint64_t sign = b & (1ull << 63);
  if (e == 0 || e >= 2046) return 1.0 / x;
  const double m = xs_double((b & 0xFFFFFFFFFFFFFull) | (1023ull << 52));  // |x| scaled to [1, 2)
  const float mf = __int_as_float(0x3F800000 | (int)((b >> 29) & 0x7FFFFF));
  const float yf = __frcp_rn(mf);  // in (0.5, 1]
  const unsigned yb = (unsigned)__float_as_int(yf);
  double y = xs_double(((uint64_t)(((yb >> 23) & 0xFF) - 127 + 1023) << 52) | ((uint64_t)(yb & 0x7FFFFF) << 29));
  double t = fma(-m, y, 1.0);
  y = fma(y, t, y);
  t = fma(-m, y, 1.0);
  y = fma(y, t, y);
  const uint64_t rb = xs_bits(y);
  const long er = (long)((rb >> 52) & 0x7FF) + 1023 - e;
  if (er <= 0 || er >= 2047) return 1.0 / x;
  return xs_double(sign | ((uint64_t)er << 52) | (rb & 0xFFFFFFFFFFFFFull));
}

// ---- fused grid barrier and reduction ----
// A slot is PCG_SLOT_WORDS 64-bit words, each on its own 128-byte line so that
// the CTAs' additions to different words proceed in parallel in L2 instead of
// queueing on one line.  Every CTA adds
// (payload << 8) + 1 to each word, so a word whose low byte has reached the
// CTA count is complete and its upper bits hold the payload total: polling a
// slot is the barrier and returns the reduction in the same load.  Payloads:
// the 26-bit limb totals of the CTA's fixed-point partials of (w, r) (words
// 0-4) and (r, r) (words 5-9) against grid-wide anchors, and whether the CTA
// had a term beyond the anchors' range (word 10).  Slots rotate over three:
// iteration k adds to slot k % 3, and once CTA 0 has seen it complete it
// clears slot (k - 1) % 3 (every CTA read that one before adding to slot k);
// it is next written in iteration k + 2, after the adders have seen slot
// k + 1 complete, which includes CTA 0's addition after the clearing.
constexpr int PCG_SLOT_WORDS = 11;
constexpr int PCG_WORD_STRIDE = 16;  // 64-bit words: one 128-byte line per slot word
constexpr int PCG_SLOT_U64 = PCG_SLOT_WORDS * PCG_WORD_STRIDE;
constexpr int PCG_SLOTS = 3;
// Byte offset of the slots in the partials buffer (after two parities of
// XPartial records).
constexpr size_t PCG_SLOT_OFFSET = 2 * PCG_MAX_BLOCKS * sizeof(XPartial);
static_assert(PCG_MAX_BLOCKS < 256, "the CTA count must fit the low byte of a slot word");
static_assert(PCG_SLOT_OFFSET % 128 == 0, "slots are 128-byte lines");
// The partials buffer holds at least 16 x 320 doubles (epic_create) and the
// allocation-free entry's 8 x 1024.
static_assert(PCG_SLOT_OFFSET + PCG_SLOTS * PCG_SLOT_U64 * sizeof(unsigned long long) <= 16 * 320 * sizeof(double),
              "slots must fit the solver partials buffer");
// Anchors: (r, r) terms of iteration k+1 are converted against the exponent
// of (r, r) of iteration k plus this headroom, (w, r) terms one higher
// (|w_i r_i| <= 2 max r_i^2 for the diagonal -4 stencil).  A term more than
// one binade above its anchor (a residual component that grew past about
// 2^4 x the previous (r, r)) sends the iteration through the block-anchored
// reduction instead.  Below the anchor, bits under 2^(A - 1129) are dropped:
// about 2^-80 of (r, r) for 2^19 terms, far below FP64 rounding.
constexpr int PCG_ANCHOR_HEADROOM = 3;

__device__ __forceinline__ void red_add_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("red.relaxed.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void red_release_add_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// acc += x * 2^(1129 - A) (the fixed-point value of xs_from_double, bits
// under 2^0 truncated toward zero) for x with biased exponent <= A + 1, branch
// free; a term above that range adds nothing and returns false.  NONNEG: x is
// known to be >= 0 (squares), so no conditional negation.
template <bool NONNEG>
__device__ __forceinline__ bool xs_add_anchored(xs_uint& acc, double x, int A) {
  const uint64_t b = xs_bits(x);
  const int eb = (int)((b >> 52) & 0x7FF);
  const bool ok = eb <= A + 1;
  const uint64_t m = ok ? ((b & 0xFFFFFFFFFFFFFull) | ((uint64_t)(eb != 0) << 52)) : 0ull;
  const int sh = 54 + (eb ? eb : 1) - A;  // <= 55 when ok
  const unsigned up = (unsigned)max(sh, 0), dn = (unsigned)max(-sh, 0);
  const uint64_t lo = sh >= 0 ? xs_shl(m, up) : xs_shr(m, dn);
  const uint64_t hi = xs_shr(m, 64u - up);  // m >> (64 - sh), 0 for sh <= 0
  xs_uint v = ((xs_uint)hi << 64) | lo;
  if (!NONNEG) {
    const xs_uint neg = (xs_uint)(xs_int)(-(int64_t)(b >> 63));  // all ones for a negative x
    v = (v ^ neg) - neg;
  }
  acc += v;
  return ok;
}

// Warp totals of the five 26-bit limbs of v (top limb signed), in every lane:
// v = sum l[k] 2^(26k).  Each limb total of 32 lanes stays below 2^31.
__device__ __forceinline__ void xs_warp_limbs(xs_int v, int (&l)[5]) {
  const xs_uint u = (xs_uint)v;
  const unsigned M = (1u << 26) - 1;
  l[0] = __reduce_add_sync(0xffffffffu, (int)((unsigned)u & M));
  l[1] = __reduce_add_sync(0xffffffffu, (int)((unsigned)(u >> 26) & M));
  l[2] = __reduce_add_sync(0xffffffffu, (int)((unsigned)(u >> 52) & M));
  l[3] = __reduce_add_sync(0xffffffffu, (int)((unsigned)(u >> 78) & M));
  l[4] = __reduce_add_sync(0xffffffffu, (int)(v >> 104));
}

// num / den (den normal, finite) from the FP32 reciprocal y0 of den's
// significand m: with e = 1 - m y0 (|e| < 2^-22), num/m = num y0 (1 + e + e^2)
// to a relative 2^-66, formed as fma(q0, fma(e, e, e), q0), q0 = num y0:
// three dependent FP64 operations after the seed, within about two ulps.
// The exponent is applied in the integer domain; outside the normal range (or
// for den not normal) the library division is used.
__device__ __forceinline__ double div_nr(double num, double den) {
  const uint64_t b = xs_bits(den);
  const int e = (int)((b >> 52) & 0x7FF);
  if (e == 0 || e >= 2046) return num / den;
  const double m = xs_double((b & 0xFFFFFFFFFFFFFull) | (1023ull << 52));  // |den| scaled to [1, 2)
  const float yf = __frcp_rn(__int_as_float(0x3F800000 | (int)((b >> 29) & 0x7FFFFF)));
  const unsigned yb = (unsigned)__float_as_int(yf);
  const double y0 =
      xs_double(((uint64_t)(((yb >> 23) & 0xFF) - 127 + 1023) << 52) | ((uint64_t)(yb & 0x7FFFFF) << 29));
  const double er = fma(-m, y0, 1.0);
  const double q0 = num * y0;
  const double q = fma(q0, fma(er, er, er), q0);
  const uint64_t qb = xs_bits(q);
  const long eq = (long)((qb >> 52) & 0x7FF);
  const long en = eq - (e - 1023);
  if (eq == 0 || eq == 0x7FF || en <= 0 || en >= 2047) return num / den;
  return xs_double(((qb ^ b) & (1ull << 63)) | ((uint64_t)en << 52) | (qb & 0xFFFFFFFFFFFFFull));
}

template <int NPT>
__global__ void __launch_bounds__(PCG_T) k_pcg_tiled(SolverArgs a, PcgTiling t) {
  extern __shared__ double sr[];  // r of the tile and its halo ring, (tr + 2) x (tc + 2)
  __shared__ XScratch sx;
  __shared__ double s_alpha, s_beta;
  __shared__ int s_done, s_ok;
  __shared__ double s_mean;
  const Lattice lat = make_lattice(a.g.nx, a.g.ny, a.poisson_bc);
  const int C = lat.C, R = lat.R;
  const int n = C * R;
  const int tr = t.tr, tc = t.tc, ldu = tc + 2;
  const int br = blockIdx.x / t.tiles_c, bc = blockIdx.x - br * t.tiles_c;
  const int r0 = br * tr, c0 = bc * tc;
  // Valid extent of this tile (the last tile row and column may be partial).
  const int vr = min(tr, R - r0), vc = min(tc, C - c0);
  const int nb = gridDim.x;
  const double dx2 = a.g.dx * a.g.dx;
  const long long spin = spin_or_default(a.spin);
  // Partials [2][nb] alternate by reduction parity (a CTA can run at most one
  // reduction ahead of the slowest reader); published edge values likewise:
  // work[1|2] = r, work[3|4] = w, work[5|6] = s.
  XPartial* const P = reinterpret_cast<XPartial*>(a.partials);
  unsigned int target = 0;
  int ep = 0;  // episodes of the block-anchored reduction (partials parity)
  // The right-hand side at node k: the reference's (zero on the grid edges),
  // or -rho dx^2 K on every unknown of an extension lattice.
  auto rhs = [&](int k) -> double {
    if (lat.mode == EPIC_POISSON_DIRICHLET) {
      const int i = k / a.g.ny;
      return rhs_at(a, k, i, k - i * a.g.ny, dx2);
    }
    return -a.rho[k] * dx2 * a.K;
  };

  for (int m = threadIdx.x; m < (tr + 2) * ldu; m += PCG_T) sr[m] = 0.0;

  // Edge publication: each tile writes its boundary to an edge buffer of
  // 2 (tc + tr) slots per tile - top row at 0, bottom row at tc, left column
  // at 2 tc, right column at 2 tc + tr, the bottom row and right column being
  // the last valid ones - so that a neighbour reads each side of its halo
  // ring as one contiguous run (a column of the lattice would be one
  // scattered load per node).  Tiles span at least 2 x 2 valid nodes where a
  // neighbour can lie beyond them (pcg_tiling), so a node lies on at most one
  // row side and one column side.
  const int ebase = blockIdx.x * 2 * (tc + tr);
  // Owned slots: tile-local q = threadIdx.x + PCG_T*j, row-major in the tile.
  int kk[NPT], si[NPT], pe0[NPT], pe1[NPT];
#pragma unroll
  for (int j = 0; j < NPT; j++) {
    const int q = threadIdx.x + PCG_T * j;
    const int lr = q / tc, lc = q - lr * tc;
    const int row = r0 + lr, col = c0 + lc;
    const bool valid = q < tr * tc && row < R && col < C;
    kk[j] = valid ? lattice_node(lat, row, col) : -1;
    si[j] = (lr + 1) * ldu + lc + 1;
    const int er = lr == 0 ? ebase + lc : lr == vr - 1 ? ebase + tc + lc : -1;
    const int ec = lc == 0 ? ebase + 2 * tc + lr : lc == vc - 1 ? ebase + 2 * tc + tr + lr : -1;
    pe0[j] = !valid ? -1 : er >= 0 ? er : ec;
    pe1[j] = !valid || er < 0 ? -1 : ec;
  }
  // Halo slots: the ring around the valid extent - above, below, left, right
  // - with the node (hk, for the set-up) and the neighbour tile's edge slot
  // (he): the neighbour above publishes its bottom row, the one below its top
  // row, and so on.  Neighbours wrap around where the lattice is periodic.
  int hk[PCG_HALO_SLOTS], hs[PCG_HALO_SLOTS], he[PCG_HALO_SLOTS];
#pragma unroll
  for (int j = 0; j < PCG_HALO_SLOTS; j++) {
    const int h = threadIdx.x + PCG_T * j;
    int row = -1, col = -1, side = -1, sr_ = 0, sc = 0;
    if (h < vc) {
      side = 0; row = r0 - 1; col = c0 + h; sr_ = 0; sc = h + 1;
    } else if (h < 2 * vc) {
      side = 1; row = r0 + vr; col = c0 + h - vc; sr_ = vr + 1; sc = h - vc + 1;
    } else if (h < 2 * vc + vr) {
      side = 2; row = r0 + h - 2 * vc; col = c0 - 1; sr_ = h - 2 * vc + 1; sc = 0;
    } else if (h < 2 * vc + 2 * vr) {
      side = 3; row = r0 + h - 2 * vc - vr; col = c0 + vc; sr_ = h - 2 * vc - vr + 1; sc = vc + 1;
    }
    if (side >= 0) {
      row = lattice_wrap(row, R, lat.wrap_r);
      col = lattice_wrap(col, C, lat.wrap_c);
    }
    const bool valid = side >= 0 && row >= 0 && col >= 0;
    int e = -1;
    if (valid) {
      const int nbr = row / tr, nbc = col / tc;
      const int nlr = row - nbr * tr, nlc = col - nbc * tc;
      const int eslot = side == 0 ? tc + nlc : side == 1 ? nlc : side == 2 ? 2 * tc + tr + nlr : 2 * tc + nlr;
      e = (nbr * t.tiles_c + nbc) * 2 * (tc + tr) + eslot;
    }
    hk[j] = valid ? lattice_node(lat, row, col) : -1;
    he[j] = e;
    hs[j] = sr_ * ldu + sc;
  }

  // set-up: x = 0, r = b, w = A(M r), p' = s = 0.
  double x[NPT], r[NPT], w[NPT], p[NPT], s[NPT], r_old[NPT];
#pragma unroll
  for (int j = 0; j < NPT; j++) {
    x[j] = r[j] = w[j] = p[j] = s[j] = r_old[j] = 0.0;
    if (kk[j] >= 0) r[j] = rhs(kk[j]);
  }
  // PERIODIC: b projected onto zero mean (the mean of the exact total,
  // rounded once; the singular system is then consistent).
  double bmean = 0.0;
  if (lat.mode == EPIC_POISSON_PERIODIC) {
    double t0[NPT], t1[NPT];
#pragma unroll
    for (int j = 0; j < NPT; j++) {
      t0[j] = kk[j] >= 0 ? r[j] : 0.0;
      t1[j] = 0.0;
    }
    XPartial* const Pc = P + (ep & 1) * nb;
    xs_block_partial<NPT>(t0, t1, sx, Pc + blockIdx.x);
    if (threadIdx.x == 0) bar_arrive(a.bar);
    target += nb;
    if (!bar_wait(a.bar, a.flags, target, &s_ok, spin)) return;
    if (threadIdx.x < 32) {
      double tot = 0, unused = 0;
      xs_grid_totals_w0(Pc, nb, &tot, &unused);
      if (threadIdx.x == 0) s_mean = tot / (double)n;
    }
    ep++;
    __syncthreads();
    bmean = s_mean;
#pragma unroll
    for (int j = 0; j < NPT; j++)
      if (kk[j] >= 0) r[j] = r[j] - bmean;
  }
#pragma unroll
  for (int j = 0; j < NPT; j++)
    if (kk[j] >= 0) sr[si[j]] = r[j];
#pragma unroll
  for (int j = 0; j < PCG_HALO_SLOTS; j++)
    if (hk[j] >= 0) sr[hs[j]] = rhs(hk[j]) - bmean;
  __syncthreads();
  // Dot-product terms of this thread's nodes: (w, r) and (r, r).
  double td[NPT], tq[NPT];
#pragma unroll
  for (int j = 0; j < NPT; j++) {
    td[j] = tq[j] = 0.0;
    if (kk[j] >= 0) {
      const double* c = sr + si[j];
      w[j] = fma(-0.25, (c[-ldu] + c[-1]) + (c[1] + c[ldu]), r[j]);
      td[j] = w[j] * r[j];
      tq[j] = r[j] * r[j];
      if (pe0[j] >= 0) {
        a.work[1][pe0[j]] = r[j];
        a.work[3][pe0[j]] = w[j];
        a.work[5][pe0[j]] = 0.0;
      }
      if (pe1[j] >= 0) {
        a.work[1][pe1[j]] = r[j];
        a.work[3][pe1[j]] = w[j];
        a.work[5][pe1[j]] = 0.0;
      }
    }
  }

  // min(n*n, max_iteration) as pcg() caps it: n*n in 32-bit int arithmetic for
  // the reference's lattice (it wraps, as there), in 64 bits for the extensions.
  unsigned int cap32 = (unsigned int)n * (unsigned int)n;
  const long long cap = lat.mode == EPIC_POISSON_DIRICHLET ? (long long)(int)cap32 : (long long)n * n;
  const int maxit = cap < a.max_iter ? (int)cap : a.max_iter;
  unsigned long long* const slots =
      reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(a.partials) + PCG_SLOT_OFFSET);
  // The counted sums hold up to 2^19 terms (the fixed-point headroom).
  const bool fused = n < (1 << 19);
  if (blockIdx.x == 0)
    for (int m = threadIdx.x; m < PCG_SLOTS * PCG_SLOT_U64; m += PCG_T) slots[m] = 0ull;
  __shared__ int s_limb[PCG_T / 32][PCG_SLOT_WORDS];
  __shared__ int s_aq, s_exact;
  // Thread 0's scalars, in the scaled form: rr = (r, r) = -4 gamma,
  // dr = (w, r) = -4 delta, eta_r = -4 eta; then beta = rr / rr_prev,
  // eta_r = dr - beta^2 eta_r_prev = dr - rr^2 g with g = eta_r_prev / rr_prev^2,
  // alpha = rr / eta_r.  Thread 32 forms 1/rr_prev and g while the CTA waits.
  __shared__ double s_rr, s_eta, s_rrinv, s_g;
  if (threadIdx.x == 0) s_rr = s_eta = s_rrinv = s_g = 0.0;
  double be = 0, alq = 0;  // this iteration's beta and -alpha/4
  int aq = 0;              // anchor of the (r, r) terms (grid-wide); (w, r) one higher
  int it = 0;
  // This thread's fixed-point sums of its (w, r) and (r, r) terms against the
  // anchors, accumulated as the stencil forms the terms.
  xs_uint v0 = 0, v1 = 0;
  bool in = true;
  for (;;) {
    const int cur = it & 1;
    double dr = 0, rr = 0;  // valid in thread 0
    bool exact = it == 0 || !fused;
    if (!exact) {
      // Counted sums against the anchors aq (r, r) and aq + 1 (w, r).
      const int ad = aq + 1;
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      const bool out = !in;
      int l0[5], l1[5];
      xs_warp_limbs((xs_int)v0, l0);
      xs_warp_limbs((xs_int)v1, l1);
      const unsigned outw = __ballot_sync(0xffffffffu, out);
      if (lane == 0) {
#pragma unroll
        for (int k = 0; k < 5; k++) {
          s_limb[wid][k] = l0[k];
          s_limb[wid][5 + k] = l1[k];
        }
        s_limb[wid][10] = outw != 0;
      }
      __syncthreads();  // also orders this CTA's published edge values before the release below
      unsigned long long* const slot = slots + (it % PCG_SLOTS) * PCG_SLOT_U64;
      if (wid == 0 && lane >= 1 && lane < PCG_SLOT_WORDS) {
        long long S = 0;
#pragma unroll
        for (int w = 0; w < PCG_T / 32; w++) S += s_limb[w][lane];
        red_add_u64(slot + lane * PCG_WORD_STRIDE, ((unsigned long long)S << 8) + 1ull);
      } else if (threadIdx.x == 64) {
        long long S = 0;
#pragma unroll
        for (int w = 0; w < PCG_T / 32; w++) S += s_limb[w][0];
        red_release_add_u64(slot, ((unsigned long long)S << 8) + 1ull);
      }
      // Warp 0 polls: lanes 0-4 the (w, r) limb words 0-4, lanes 8-12 the
      // (r, r) words 5-9, lane 16 word 10 (so that each total gathers in an
      // 8-lane group).
      const int pword = lane < 5 ? lane : (lane >= 8 && lane < 13) ? lane - 3 : lane == 16 ? 10 : -1;
      unsigned long long wv0 = 0;
      if (wid == 0 && pword >= 0)
        wv0 = lane == 0 ? ld_acquire_u64(slot) : ld_relaxed_u64(slot + pword * PCG_WORD_STRIDE);
      // Deferred update of the previous iteration (no other CTA needs p' or
      // x), and the scalars the next step needs from the previous ones.
#pragma unroll
      for (int j = 0; j < NPT; j++)
        if (kk[j] >= 0) {
          p[j] = fma(be, p[j], r_old[j]);
          x[j] = fma(alq, p[j], x[j]);
        }
      if (threadIdx.x == 32) {
        const double ri = recip_nr(s_rr);
        s_rrinv = ri;
        s_g = s_eta * (ri * ri);
      }
      if (wid == 0) {
        unsigned long long wv = 0;
        int good = 1;
        if (pword >= 0) {
          long long spins = 0;
          wv = wv0;
          for (;;) {
            if ((wv & 255ull) == (unsigned long long)nb) break;
            if (++spins >= spin) {
              atomicOr(a.flags, FLAG_TIMEOUT);
              good = 0;
              break;
            }
            wv = lane == 0 ? ld_acquire_u64(slot) : ld_relaxed_u64(slot + pword * PCG_WORD_STRIDE);
          }
        }
        good = __all_sync(0xffffffffu, good);
        if (blockIdx.x == 0 && pword >= 0)
          slots[((it + PCG_SLOTS - 1) % PCG_SLOTS) * PCG_SLOT_U64 + pword * PCG_WORD_STRIDE] = 0ull;
        const long long S = pword >= 0 ? (long long)(wv - (unsigned long long)nb) >> 8 : 0;
        const long long outc = __shfl_sync(0xffffffffu, S, 16);
        // Each 8-lane group sums its limbs shifted to their weights (a
        // butterfly of 128-bit adds): lane 0 holds (w, r), lane 8 (r, r);
        // both round their totals at once.
        xs_int V = (lane & 7) < 5 && lane < 16 ? (xs_int)S << (26 * (lane & 7)) : (xs_int)0;
#pragma unroll
        for (int o = 4; o >= 1; o >>= 1) {
          const uint64_t vlo = (uint64_t)(xs_uint)V, vhi = (uint64_t)((xs_uint)V >> 64);
          const uint64_t olo = __shfl_xor_sync(0xffffffffu, vlo, o), ohi = __shfl_xor_sync(0xffffffffu, vhi, o);
          V += (xs_int)(((xs_uint)ohi << 64) | olo);
        }
        const double d = xs_to_double(V, lane == 0 ? ad : aq);
        const double d1 = __shfl_sync(0xffffffffu, d, 8);
        if (lane == 0) {
          dr = d;
          rr = d1;
          s_ok = good;
          s_exact = outc != 0;
        }
      }
      __syncthreads();
      if (!s_ok) return;
      exact = s_exact;
    }
    if (exact) {
      // Block-anchored reduction: partials of this episode's parity, then
      // the grid totals after the counter barrier.
      XPartial* const Pc = P + (ep & 1) * nb;
      xs_block_partial<NPT>(td, tq, sx, Pc + blockIdx.x);
      if (threadIdx.x == 0) bar_arrive(a.bar);
      target += nb;
      if (it > 0 && !fused) {
#pragma unroll
        for (int j = 0; j < NPT; j++)
          if (kk[j] >= 0) {
            p[j] = fma(be, p[j], r_old[j]);
            x[j] = fma(alq, p[j], x[j]);
          }
        if (threadIdx.x == 32) {
          const double ri = recip_nr(s_rr);
          s_rrinv = ri;
          s_g = s_eta * (ri * ri);
        }
      }
      if (!bar_wait(a.bar, a.flags, target, &s_ok, spin)) return;
      if (threadIdx.x < 32) xs_grid_totals_w0(Pc, nb, &dr, &rr);
      ep++;
    }
    // Halo inputs published before the barrier, loaded while thread 0 forms
    // the scalars.
    const double* const pr_c = cur ? a.work[2] : a.work[1];
    const double* const pw_c = cur ? a.work[4] : a.work[3];
    const double* const ps_c = cur ? a.work[6] : a.work[5];
    double hr[PCG_HALO_SLOTS], hw[PCG_HALO_SLOTS], hsv[PCG_HALO_SLOTS];
#pragma unroll
    for (int j = 0; j < PCG_HALO_SLOTS; j++)
      if (he[j] >= 0) {
        hr[j] = __ldcg(&pr_c[he[j]]);
        hw[j] = __ldcg(&pw_c[he[j]]);
        hsv[j] = __ldcg(&ps_c[he[j]]);
      }
    if (threadIdx.x == 0) {
      s_rr = rr;
      s_done = xs_bits(rr) < a.tol_bits || it >= maxit;  // sqrt(r.r) < tol
      double beta, eta_r;
      if (it == 0) {
        beta = 0;
        eta_r = dr;
      } else {
        beta = rr * s_rrinv;
        eta_r = fma(-(rr * rr), s_g, dr);
      }
      s_eta = eta_r;
      s_alpha = div_nr(rr, eta_r);
      s_beta = beta;
      s_aq = xs_exponent(rr) + PCG_ANCHOR_HEADROOM;
    }
    __syncthreads();
    if (s_done) break;
    const double al = s_alpha;
    be = s_beta;
    alq = -0.25 * al;
    aq = s_aq;
#pragma unroll
    for (int j = 0; j < NPT; j++)
      if (kk[j] >= 0) {
        r_old[j] = r[j];
        s[j] = fma(be, s[j], w[j]);
        r[j] = fma(-al, s[j], r[j]);
        sr[si[j]] = r[j];
      }
#pragma unroll
    for (int j = 0; j < PCG_HALO_SLOTS; j++)
      if (he[j] >= 0) sr[hs[j]] = fma(-al, fma(be, hsv[j], hw[j]), hr[j]);
    __syncthreads();
    double* const pr_n = cur ? a.work[1] : a.work[2];
    double* const pw_n = cur ? a.work[3] : a.work[4];
    double* const ps_n = cur ? a.work[5] : a.work[6];
    v0 = v1 = 0;
    in = true;
#pragma unroll
    for (int j = 0; j < NPT; j++)
      if (kk[j] >= 0) {
        const double* c = sr + si[j];
        w[j] = fma(-0.25, (c[-ldu] + c[-1]) + (c[1] + c[ldu]), r[j]);
        td[j] = w[j] * r[j];
        tq[j] = r[j] * r[j];
        if (fused) {
          in &= xs_add_anchored<false>(v0, td[j], aq + 1);
          in &= xs_add_anchored<true>(v1, tq[j], aq);
        }
        if (pe0[j] >= 0) {
          pr_n[pe0[j]] = r[j];
          pw_n[pe0[j]] = w[j];
          ps_n[pe0[j]] = s[j];
        }
        if (pe1[j] >= 0) {
          pr_n[pe1[j]] = r[j];
          pw_n[pe1[j]] = w[j];
          ps_n[pe1[j]] = s[j];
        }
      }
    it++;
  }
  // domain.error = |A x - b| / n (src/field.cpp:258-259), n = nx ny.  With
  // PERIODIC the same reduction also totals x, whose mean is then removed
  // (the zero-mean gauge; the error is that of x before the shift).
#pragma unroll
  for (int j = 0; j < NPT; j++)
    if (kk[j] >= 0) a.phi[kk[j]] = x[j];
  __syncthreads();
  if (threadIdx.x == 0) bar_arrive(a.bar);
  target += nb;
  if (!bar_wait(a.bar, a.flags, target, &s_ok, spin)) return;
  const bool gauge = lat.mode == EPIC_POISSON_PERIODIC;
#pragma unroll
  for (int j = 0; j < NPT; j++) {
    td[j] = tq[j] = 0.0;
    if (kk[j] >= 0) {
      const int q = threadIdx.x + PCG_T * j, lr = q / tc, lc = q - lr * tc;
      const int row = r0 + lr, col = c0 + lc;
      const int up = lattice_wrap(row - 1, R, lat.wrap_r), dn = lattice_wrap(row + 1, R, lat.wrap_r);
      const int lf = lattice_wrap(col - 1, C, lat.wrap_c), rt = lattice_wrap(col + 1, C, lat.wrap_c);
      double sum = 0;
      if (up >= 0) sum += __ldcg(&a.phi[lattice_node(lat, up, col)]);
      if (lf >= 0) sum += __ldcg(&a.phi[lattice_node(lat, row, lf)]);
      sum = fma(-4.0, x[j], sum);
      if (rt >= 0) sum += __ldcg(&a.phi[lattice_node(lat, row, rt)]);
      if (dn >= 0) sum += __ldcg(&a.phi[lattice_node(lat, dn, col)]);
      const double e = sum - (rhs(kk[j]) - bmean);
      td[j] = e * e;
      if (gauge) tq[j] = x[j];
    }
  }
  XPartial* const Pe = P + (ep & 1) * nb;
  xs_block_partial<NPT>(td, tq, sx, Pe + blockIdx.x);
  if (threadIdx.x == 0) bar_arrive(a.bar);
  target += nb;
  if (!bar_wait(a.bar, a.flags, target, &s_ok, spin)) return;
  if ((gauge || blockIdx.x == 0) && threadIdx.x < 32) {
    double e2 = 0, xsum = 0;
    xs_grid_totals_w0(Pe, nb, &e2, &xsum);
    if (threadIdx.x == 0) {
      s_mean = xsum / (double)n;
      if (blockIdx.x == 0) {
        a.info->iterations = it;
        a.info->converged = it < maxit;
        a.info->error = sqrt(e2) / (a.g.nx * a.g.ny);
        atomicAdd(a.iter_total, (unsigned long long)it);
      }
    }
  }
  if (gauge) {
    __syncthreads();
    const double xm = s_mean;
#pragma unroll
    for (int j = 0; j < NPT; j++)
      if (kk[j] >= 0) a.phi[kk[j]] = x[j] - xm;
  }
}

// Tile shape for at most max_blocks CTAs: the fewest FP64 operations on the
// busiest CTA (11 per owned node, 3 per halo node), ties to fewer CTAs.
// Returns false when no tile fits PCG_T * 8 owned nodes and a halo ring of
// PCG_T * PCG_HALO_SLOTS nodes (then the global-memory k_pcg runs).
static bool pcg_tiling(int R, int C, int wrap_r, int wrap_c, int max_blocks, PcgTiling* out) {
  long long best = -1;
  PcgTiling b{};
  for (int tcb = 1; tcb <= C && tcb <= max_blocks; tcb++) {
    const int tc = (C + tcb - 1) / tcb;
    const int ncb = (C + tc - 1) / tc;
    const int rb_max = max_blocks / ncb;
    if (rb_max < 1) continue;
    const int tr = (R + rb_max - 1) / rb_max;
    const int nrb = (R + tr - 1) / tr;
    const long long nodes = (long long)tr * tc;
    if (nodes > PCG_T * 8 || 2LL * (tr + tc) > PCG_T * PCG_HALO_SLOTS) continue;
    if (ncb * nrb > PCG_MAX_BLOCKS) continue;
    // Where the lattice wraps, the last tile's valid extent has a neighbour
    // beyond both of its sides and must span two nodes (so that its first
    // and last rows / columns are different nodes).
    if ((wrap_r && R - (nrb - 1) * tr < 2) || (wrap_c && C - (ncb - 1) * tc < 2)) continue;
    // The edge buffers (2 (tr + tc) slots per tile) live in node-sized vectors.
    if (tr < 2 || tc < 2 || (long long)ncb * nrb * 2 * (tr + tc) > (long long)R * C) continue;
    const long long cost = 11 * nodes + 3 * 2LL * (tr + tc);
    const int blocks = ncb * nrb;
    if (best < 0 || cost < best || (cost == best && blocks < b.blocks)) {
      best = cost;
      b.tr = tr;
      b.tc = tc;
      b.tiles_c = ncb;
      b.blocks = blocks;
      const int npt = (int)((nodes + PCG_T - 1) / PCG_T);
      b.npt = npt <= 1 ? 1 : npt <= 2 ? 2 : npt <= 4 ? 4 : 8;
    }
  }
  if (best < 0) return false;
  *out = b;
  return true;
}

int pcg_default_blocks(long long nodes, int sms) {
  // One CTA per SM at most (FP64 throughput is per SM; more CTAs only add
  // barrier arrivals), and no fewer than ~384 nodes per CTA on small grids.
  long long want = (nodes + 383) / 384;
  return (int)std::max(1LL, std::min<long long>(want, std::min(solver_max_blocks(), sms)));
}

// Launches the tiled solve if all its CTAs can be resident at once (the
// cooperative-launch condition); returns false otherwise.
template <int NPT>
static bool launch_tiled(cudaStream_t st, const SolverArgs& a, const PcgTiling& t) {
  const int smem = (t.tr + 2) * (t.tc + 2) * (int)sizeof(double);
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pcg_tiled<NPT>, PCG_T, smem);
  if (t.blocks > per_sm * sms) return false;
  SolverArgs args = a;
  PcgTiling tl = t;
  void* params[] = {&args, &tl};
  cudaLaunchCooperativeKernel((const void*)k_pcg_tiled<NPT>, dim3(t.blocks), dim3(PCG_T), params, smem, st);
  return true;
}

void launch_pcg(cudaStream_t st, const SolverArgs& a_in, int blocks) {
  cudaMemsetAsync(a_in.bar, 0, 2 * sizeof(unsigned int), st);
  SolverArgs a = a_in;
  a.spin = spin_limit();
  const Lattice lat = make_lattice(a.g.nx, a.g.ny, a.poisson_bc);
  PcgTiling t;
  if (pcg_tiling(lat.R, lat.C, lat.wrap_r, lat.wrap_c, blocks, &t)) {
    SolverArgs at = a;
    at.tol_bits = xs_bits(xs_sqrt_threshold(a.tol));
    bool ok;
    switch (t.npt) {
      case 1: ok = launch_tiled<1>(st, at, t); break;
      case 2: ok = launch_tiled<2>(st, at, t); break;
      case 4: ok = launch_tiled<4>(st, at, t); break;
      default: ok = launch_tiled<8>(st, at, t); break;
    }
    if (ok) {
      if (a.poisson_bc != EPIC_POISSON_DIRICHLET) launch_fill_poisson_nodes(st, a.g, a.poisson_bc, a.phi);
      return;
    }
  }
  SolverArgs args = a;
  void* params[] = {&args};
  cudaLaunchCooperativeKernel((const void*)k_pcg, dim3(blocks), dim3(256), params, 0, st);
  if (a.poisson_bc != EPIC_POISSON_DIRICHLET) launch_fill_poisson_nodes(st, a.g, a.poisson_bc, a.phi);
}

__global__ void k_fill_poisson_nodes(Geom g, int mode, double* phi) {
  const int nx = g.nx, ny = g.ny;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nx * ny; k += gridDim.x * blockDim.x) {
    const int i = k / ny, j = k - i * ny;
    if (mode == EPIC_POISSON_DIRICHLET_X && (i == 0 || i == nx - 1)) {
      phi[k] = 0.0;
    } else if (j == ny - 1 || (mode == EPIC_POISSON_PERIODIC && i == nx - 1)) {
      const int si = mode == EPIC_POISSON_PERIODIC && i == nx - 1 ? 0 : i;
      phi[k] = phi[si * ny + (j == ny - 1 ? 0 : j)];  // an unknown: never written here
    }
  }
}

void launch_fill_poisson_nodes(cudaStream_t st, const Geom& g, int poisson_bc, double* phi) {
  const int nn = g.nx * g.ny;
  k_fill_poisson_nodes<<<(nn + 255) / 256, 256, 0, st>>>(g, poisson_bc, phi);
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
  if (!grid_sync(a.bar, a.flags, spin_or_default(a.spin))) return;
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
      if (!grid_sync(a.bar, a.flags, spin_or_default(a.spin))) return;
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
      if (!grid_sync(a.bar, a.flags, spin_or_default(a.spin))) return;
      double2 tot = grid_total2_t0(P, nb, sw);
      if (threadIdx.x == 0) {
        s_l2 = sqrt(tot.x / (nx * ny));
        s_done = s_l2 < a.tol;
      }
      __syncthreads();
      L2 = s_l2;
      if (!grid_sync(a.bar, a.flags, spin_or_default(a.spin))) return;  // partials are rewritten at the next check
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
  args.spin = spin_limit();
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
