// Poisson solve of the mixed-precision form: FP64 defect correction around an
// FP32 inner solve.
//
// The operator is the reference's: the 5-point Laplacian with diagonal -4 and
// zero exterior, on every node for pcgsolver (src/field.cpp:212-264) or on
// the interior nodes with phi = 0 on the edges for gssolver
// (src/field.cpp:70-139); b = -rho * dx^2 * (L/LDe)^2, zero on grid edges.
// The unknowns form an R x C lattice on which the operator is separable,
// A = T_R (x) I + I (x) T_C with T = tridiag(1, -2, 1): for pcgsolver the
// reference's own lattice of the flattened vector (R = ny rows of C = nx,
// neighbours k +- 1 and k +- nx, src/field.cpp:221-232 — the physical grid
// when nx = ny), for gssolver the interior nodes (R = nx - 2 by C = ny - 2,
// the physical neighbours).  T_n is diagonalised by the orthonormal, symmetric
// sine transform Q_jk = sqrt(2/(n+1)) sin(pi (j+1)(k+1)/(n+1)) with
// eigenvalues lambda_k = -4 sin^2(pi (k+1)/(2(n+1))), so
// A^-1 X = Q_R ((Q_R X Q_C) o D) Q_C with D_pq = 1/(lambda_p + mu_q): four dense
// products, done here in FP32 (each inner solve is accurate to ~1e-6
// relative); on large lattices whose sides allow it (SpecFFT) the four
// products are FFT passes instead, O(n^2 log n) against O(n^3).  Each stage computes the FP64 residual r = b - A x, stops
// once the reference's own stopping norm is below its tolerance (|r|_2 for
// pcgsolver; the SOR residual L2 = sqrt(sum R^2 / (nx ny)), R = r/dx^2, for
// gssolver), and otherwise adds the FP32 correction A^-1 r to x in FP64.
// The stages run in one cooperative launch (k_spec_solve) that stops as soon
// as the test passes, so one fixed launch sequence (graph-capturable) serves
// any number of stages up to the cap.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "epic_internal.cuh"
#include "epic_spectral.cuh"

namespace epic {

int spectral_supported(const Geom& g, int solver, int poisson_bc) {
  if (g.nx < 3 || g.ny < 3) return 0;
  if (solver != EPIC_SOLVER_PCG && solver != EPIC_SOLVER_GS) return 0;  // the Boltzmann solvers are nonlinear
  // The extension lattices (both solvers' unknowns are the same there) are
  // isotropic only for dx = dy.
  if (poisson_bc != EPIC_POISSON_DIRICHLET) return g.dx == g.dy;
  return solver == EPIC_SOLVER_PCG || g.dx == g.dy;  // the SOR lattice is isotropic only for dx = dy
}

static SpecLattice lattice_of(const SpectralSolver& sp, const SolverArgs& a) {
  SpecLattice L;
  L.nx = a.g.nx;
  L.ny = a.g.ny;
  L.I_off = 0;
  L.NY = a.g.ny;
  L.R = sp.R;
  L.C = sp.C;
  L.flat = sp.flat;
  L.gs_norm = sp.gs_norm;
  L.mode = sp.mode;
  L.bmean = nullptr;  // PERIODIC: set inside the solve
  L.dx2 = a.g.dx * a.g.dx;
  L.K = a.K;
  L.tol = a.tol;
  L.rho = a.rho;
  L.phi = a.phi;
  L.t0 = sp.t0;
  L.partials = sp.partials;
  L.state = sp.state;
  L.info = a.info;
  L.iter_total = a.iter_total;
  return L;
}

// x = 0 on all nodes (cold start, as both reference solvers), or for a warm
// start zero only the nodes that are not unknowns (the edges under gssolver).
__global__ void k_spec_init(SpecLattice L, int warm) {
  const int nx = L.nx, ny = L.ny;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nx * ny; k += gridDim.x * blockDim.x) {
    const int i = k / ny, j = k - i * ny;
    const bool unknown = L.mode == EPIC_POISSON_PERIODIC   ? i < nx - 1 && j < ny - 1
                         : L.mode == EPIC_POISSON_DIRICHLET_X ? i >= 1 && i < nx - 1 && j < ny - 1
                         : L.flat || (i >= 1 && i < nx - 1 && j >= 1 && j < ny - 1);
    if (!warm || !unknown) spec_init_node(L, k);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    L.state[0] = 0;
    L.state[1] = 0;
    L.state[2] = 0;
  }
}

int spectral_chunks(const SpectralSolver& sp) { return (sp.R * sp.C + SPEC_CHUNK - 1) / SPEC_CHUNK; }

// Grid barrier of a cooperative launch (counter zeroed before the launch):
// the CTA barrier orders the CTA's writes before thread 0's release add, and
// the acquire poll followed by the CTA barrier orders every later read after
// the other CTAs' writes; bounded by `limit` polls (FLAG_TIMEOUT).
__device__ bool spec_grid_sync(unsigned int* bar, int* flags, long long limit) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int ticket;
    asm volatile("atom.add.release.gpu.global.u32 %0, [%1], 1;" : "=r"(ticket) : "l"(bar) : "memory");
    const unsigned int target = (ticket / gridDim.x + 1) * gridDim.x;
    int ok = 1;
    long long spins = 0;
    for (;;) {
      unsigned int v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
      if ((int)(v - target) >= 0) break;
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

// The whole defect-correction loop in one cooperative launch: the CTAs take
// the residual chunks in turn; after a grid barrier every CTA forms the
// stopping norm from the exact sum of the chunk sums (so every CTA decides
// alike, and as spec_check; CTA 0 records it); then the four products, the CTAs
// taking TILE x TILE output tiles in turn, with a grid barrier after each.
// Each output accumulates over k in order whatever the tile, so the
// potentials equal those of the batched solve bit for bit.
// PERIODIC: a fixed-order sum over the lattice entries [ch * SPEC_CHUNK, ...)
// of b = -rho dx^2 K (what = 0) or of phi (what = 1); entry (r, c) is node
// (r, c).  Called by a whole CTA of 256 threads; the sum goes to out[ch].
__device__ void spec_chunk_sum(const SpecLattice& L, int what, int ch, double* out, double* sm8) {
  const int total = L.R * L.C;
  double acc = 0;
#pragma unroll
  for (int u = 0; u < SPEC_CHUNK / 256; u++) {
    const int q = ch * SPEC_CHUNK + u * 256 + threadIdx.x;
    if (q < total) {
      const int r = q / L.C, c = q - r * L.C;
      const int k = spec_node(L, r, c);
      acc += what ? __ldcg(&L.phi[k]) : -L.rho[k] * L.dx2 * L.K;
    }
  }
  acc = spec_warp_sum(acc);
  if ((threadIdx.x & 31) == 0) sm8[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < 8; w++) t += sm8[w];
    out[ch] = t;
  }
  __syncthreads();
}

// The mean over the lattice from the chunk sums, added exactly by the whole
// CTA (every CTA forms the same value).
__device__ double spec_chunk_mean(const SpecLattice& L, const double* sums, int nch, int* s_e,
                                  unsigned long long (*s_v)[2], double* s_out) {
  return spec_exact_sum_cta(sums, nch, s_e, s_v, s_out) / ((double)L.R * L.C);
}

// TILE 16, 32, 64: the dense products in output tiles of that side; TILE 0:
// FFT passes (F), units of SPEC_FFT_LINES lines, the sequences in dynamic
// shared memory.
template <int TILE>
__global__ void __launch_bounds__(256) k_spec_solve(SpecLattice L, const float* __restrict__ QR,
                                                    const float* __restrict__ QC, const float* __restrict__ D,
                                                    float* t1, int stages, unsigned int* bar, int* flags,
                                                    long long spin, SpecFFT F) {
  extern __shared__ float2 fbuf[];
  __shared__ __align__(16) float As[TILE == 64 || TILE == 0 ? 1 : 32][33];
  __shared__ float Bs[TILE == 64 || TILE == 0 ? 1 : 32][33];
  __shared__ __align__(16) SpecGemmSmem sg[TILE == 64 ? 1 : 0 + 1];
  __shared__ double sm8[8];
  __shared__ double s_mean, s_sum;
  __shared__ int s_stop;
  __shared__ int s_xe[8];
  __shared__ unsigned long long s_xv[8][2];
  const int R = L.R, C = L.C;
  const int nch = (R * C + SPEC_CHUNK - 1) / SPEC_CHUNK;
  const int TL = TILE ? TILE : 1;
  const int tiles_c = (C + TL - 1) / TL, ntiles = tiles_c * ((R + TL - 1) / TL);
  const int ucols = (C + SPEC_FFT_LINES - 1) / SPEC_FFT_LINES, urows = (R + SPEC_FFT_LINES - 1) / SPEC_FFT_LINES;
  // PERIODIC: the chunk sums of b and of phi go after the residual's.
  double* const sums = L.partials + nch;
  const bool periodic = L.mode == EPIC_POISSON_PERIODIC;
  // FFT: the twiddle tables in shared memory after the sequences
  float2* const s_twR = fbuf + (TILE == 0 ? (SPEC_FFT_LINES / 2) * spec_fft_seq(max(F.mR, F.mC)) : 0);
  float2* const s_twC = s_twR + (TILE == 0 ? F.mR / 2 : 0);
  if (TILE == 0) {
    for (int k = threadIdx.x; k < F.mR / 2; k += blockDim.x) s_twR[k] = F.twR[k];
    for (int k = threadIdx.x; k < F.mC / 2; k += blockDim.x) s_twC[k] = F.twC[k];
    __syncthreads();
  }
  if (periodic) {  // b projected onto zero mean: the mean of b over the unknowns
    for (int ch = blockIdx.x; ch < nch; ch += gridDim.x) spec_chunk_sum(L, 0, ch, sums, sm8);
    if (!spec_grid_sync(bar, flags, spin)) return;
    const double m = spec_chunk_mean(L, sums, nch, s_xe, s_xv, &s_sum);
    if (threadIdx.x == 0) s_mean = m;
    __syncthreads();
    L.bmean = &s_mean;
  }
  for (int s = 0;; s++) {
    for (int ch = blockIdx.x; ch < nch; ch += gridDim.x) {
      spec_residual_chunk(L, ch, sm8);
      __syncthreads();
    }
    if (!spec_grid_sync(bar, flags, spin)) return;
    const double sum = spec_exact_sum_cta(L.partials, nch, s_xe, s_xv, &s_sum);
    if (threadIdx.x == 0) {
      double norm, err;
      spec_norm(L, sum, norm, err);
      const int done = norm < L.tol;
      if (blockIdx.x == 0) spec_record(L, done, s == stages, err);
      s_stop = done || s == stages;
    }
    __syncthreads();
    if (s_stop) break;
#define SPEC_PASS(EPI, K_, A_, B_, C_, D_)                                                                    \
  for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {                                                       \
    if (TILE == 64)                                                                                          \
      spec_gemm_tile64<EPI>(R, C, K_, A_, B_, C_, D_, &L, t / tiles_c, t - (t / tiles_c) * tiles_c, sg[0]);  \
    else                                                                                                     \
      spec_gemm_tile<EPI, TILE == 64 ? 32 : TILE>(R, C, K_, A_, B_, C_, D_, &L, t / tiles_c,                 \
                                                  t - (t / tiles_c) * tiles_c, As, Bs);                      \
  }                                                                                                          \
  if (!spec_grid_sync(bar, flags, spin)) return;
#define SPEC_FFT(EPI, DIR, IN_, OUT_, D_)                                                         \
  for (int u = blockIdx.x; u < (DIR == 0 ? ucols : urows); u += gridDim.x)                          \
    spec_fft_unit<EPI>(L, F, DIR, u * SPEC_FFT_LINES, IN_, OUT_, D_, fbuf, s_twR, s_twC);           \
  if (!spec_grid_sync(bar, flags, spin)) return;
    if constexpr (TILE == 0) {  // the same four products as FFT passes: along r, along c (o D), along r, along c (+= phi)
      SPEC_FFT(0, 0, L.t0, t1, nullptr)
      SPEC_FFT(1, 1, t1, L.t0, D)
      SPEC_FFT(0, 0, L.t0, t1, nullptr)
      SPEC_FFT(2, 1, t1, nullptr, nullptr)
    } else {
      SPEC_PASS(0, R, QR, L.t0, t1, nullptr)
      SPEC_PASS(1, C, t1, QC, L.t0, D)
      SPEC_PASS(0, R, QR, L.t0, t1, nullptr)
      SPEC_PASS(2, C, t1, QC, nullptr, nullptr)
    }
#undef SPEC_PASS
#undef SPEC_FFT
  }
  if (periodic) {  // phi shifted to zero mean over the unknowns (the FP64 solver's gauge)
    for (int ch = blockIdx.x; ch < nch; ch += gridDim.x) spec_chunk_sum(L, 1, ch, sums, sm8);
    if (!spec_grid_sync(bar, flags, spin)) return;
    const double m = spec_chunk_mean(L, sums, nch, s_xe, s_xv, &s_sum);
    for (int ch = blockIdx.x; ch < nch; ch += gridDim.x)
      for (int u = 0; u < SPEC_CHUNK / 256; u++) {
        const int q = ch * SPEC_CHUNK + u * 256 + threadIdx.x;
        if (q < R * C) {
          const int r = q / C, c = q - r * C;
          L.phi[spec_node(L, r, c)] -= m;
        }
      }
  }
}

void launch_spectral(cudaStream_t st, const SpectralSolver& sp, const SolverArgs& a, int stages) {
  const int R = sp.R, C = sp.C;
  const SpecLattice L = lattice_of(sp, a);
  k_spec_init<<<(a.g.nx * a.g.ny + 255) / 256, 256, 0, st>>>(L, a.warm);
  // One wave of co-resident CTAs, at most one per output tile.
  // Output tiles: 64 x 64 (register-blocked) once there are enough of them
  // for every SM, else 32 x 32 with two per SM, else 16 x 16.
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long t64 = (long long)((R + 63) / 64) * ((C + 63) / 64);
  const long long t32 = (long long)((R + 31) / 32) * ((C + 31) / 32);
  const long long t16 = (long long)((R + 15) / 16) * ((C + 15) / 16);
  // FFT passes (sp.fft.on): units of SPEC_FFT_LINES lines per direction.
  const int tile = sp.fft.on ? 0 : t64 >= sms ? 64 : t32 >= 2LL * sms ? 32 : 16;
  const void* kern = tile == 0    ? (const void*)k_spec_solve<0>
                     : tile == 64 ? (const void*)k_spec_solve<64>
                     : tile == 32 ? (const void*)k_spec_solve<32> : (const void*)k_spec_solve<16>;
  const int fft_smem =
      tile == 0 ? (int)(((SPEC_FFT_LINES / 2) * spec_fft_seq(std::max(sp.fft.mR, sp.fft.mC)) + sp.fft.mR / 2 +
                         sp.fft.mC / 2) *
                        sizeof(float2))
                : 0;
  if (fft_smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, fft_smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, 256, fft_smem);
  per = std::max(1, std::min(2, per));
  const long long units =
      (long long)std::max((C + SPEC_FFT_LINES - 1) / SPEC_FFT_LINES, (R + SPEC_FFT_LINES - 1) / SPEC_FFT_LINES);
  const long long tiles = tile == 0 ? units : tile == 64 ? t64 : tile == 32 ? t32 : t16;
  const int grid = (int)std::max(1LL, std::min<long long>(tiles, (long long)per * sms));
  cudaMemsetAsync(a.bar, 0, sizeof(unsigned int), st);
  SpecLattice Lk = L;
  const float *qr = sp.QR, *qc = sp.QC, *d = sp.D;
  float* t1 = sp.t1;
  int stg = stages;
  unsigned int* bar = a.bar;
  int* flags = a.flags;
  long long spin = spin_limit();
  SpecFFT F = sp.fft;
  void* params[] = {&Lk, &qr, &qc, &d, &t1, &stg, &bar, &flags, &spin, &F};
  cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(256), params, fft_smem, st);
  if (sp.mode != EPIC_POISSON_DIRICHLET) launch_fill_poisson_nodes(st, a.g, sp.mode, a.phi);
}

}  // namespace epic
