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
// relative).  Each stage computes the FP64 residual r = b - A x, stops
// once the reference's own stopping norm is below its tolerance (|r|_2 for
// pcgsolver; the SOR residual L2 = sqrt(sum R^2 / (nx ny)), R = r/dx^2, for
// gssolver), and otherwise adds the FP32 correction A^-1 r to x in FP64.
// Every kernel reads a device-side done flag and returns at once after
// convergence, so a fixed launch sequence (graph-capturable) serves any
// number of stages up to the cap.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "epic_internal.cuh"

namespace epic {

int spectral_supported(const Geom& g, int solver) {
  if (g.nx < 3 || g.ny < 3) return 0;
  return solver == EPIC_SOLVER_PCG || g.dx == g.dy;  // the SOR lattice is isotropic only for dx = dy
}

__device__ __forceinline__ double warp_sum_s(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// x = 0 on all nodes (cold start, as both reference solvers), or for a warm
// start zero only the nodes that are not unknowns (the edges under gssolver).
__global__ void k_spec_init(SolverArgs a, SpectralSolver sp) {
  const int nx = a.g.nx, ny = a.g.ny;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nx * ny; k += gridDim.x * blockDim.x) {
    const int i = k / ny, j = k - i * ny;
    const bool unknown = sp.flat || (i >= 1 && i < nx - 1 && j >= 1 && j < ny - 1);
    if (!a.warm || !unknown) a.phi[k] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    sp.state[0] = 0;
    sp.state[1] = 0;
    sp.state[2] = 0;
  }
}

// r = b - A x in FP64 on the unknowns; r (FP32) to t0 in transform layout;
// per-block partial of r^2.
__global__ void __launch_bounds__(256) k_spec_residual(SolverArgs a, SpectralSolver sp) {
  if (sp.state[0]) return;
  __shared__ double sm[8];
  const int nx = a.g.nx, ny = a.g.ny, R = sp.R, C = sp.C;
  const double dx2 = a.g.dx * a.g.dx;
  double acc = 0;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < R * C; q += gridDim.x * blockDim.x) {
    const int ri = q / C, cj = q - ri * C;
    const double* x = a.phi;
    int k, i, j;
    double ax;
    if (sp.flat) {  // pcgsolver: rows of C = nx nodes of the flattened vector
      k = q;
      i = k / ny;
      j = k - i * ny;
      ax = -4 * x[k];
      if (ri > 0) ax += x[k - C];
      if (ri < R - 1) ax += x[k + C];
      if (cj > 0) ax += x[k - 1];
      if (cj < C - 1) ax += x[k + 1];
    } else {  // gssolver: interior nodes, physical neighbours
      i = ri + 1;
      j = cj + 1;
      k = i * ny + j;
      ax = -4 * x[k];
      if (i > 0) ax += x[k - ny];
      if (i < nx - 1) ax += x[k + ny];
      if (j > 0) ax += x[k - 1];
      if (j < ny - 1) ax += x[k + 1];
    }
    const bool edge = i == 0 || i == nx - 1 || j == 0 || j == ny - 1;
    const double b = edge ? 0.0 : -a.rho[k] * dx2 * a.K;
    const double r = b - ax;
    sp.t0[q] = (float)r;
    acc += r * r;
  }
  acc = warp_sum_s(acc);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sm[w];
    sp.partials[blockIdx.x] = t;
  }
}

// Stopping test of the reference solver on the residual just computed.
__global__ void k_spec_check(SolverArgs a, SpectralSolver sp, int nb, int final_pass) {
  if (sp.state[0] && !final_pass) return;
  double s = 0;
  for (int b = 0; b < nb; b++) s += sp.partials[b];
  if (sp.state[0] && final_pass) return;  // converged earlier; info already set
  const int nx = a.g.nx, ny = a.g.ny;
  const double dx2 = a.g.dx * a.g.dx;
  double norm, err;
  if (sp.gs_norm) {
    norm = sqrt(s / (dx2 * dx2) / (nx * ny));
    err = norm;
  } else {
    norm = sqrt(s);
    err = sqrt(s) / (nx * ny);
  }
  const int done = norm < a.tol;
  a.info->iterations = sp.state[1];
  a.info->error = err;
  a.info->converged = done;
  if (done || final_pass) {
    sp.state[0] = 1;
    atomicAdd(a.iter_total, (unsigned long long)sp.state[1]);
  } else {
    sp.state[1] += 1;
  }
}

// C = A B for an M x K by K x N product of row-major FP32 matrices, 32x32
// tiles, 2x2 outputs per thread.  EPI 0: store; 1: store C o D;
// 2: x[(r+off)*ldx + (c+off)] += C (FP64).
template <int EPI>
__global__ void __launch_bounds__(256) k_spec_gemm(int M, int N, int K, const float* __restrict__ A,
                                                   const float* __restrict__ B, float* __restrict__ C,
                                                   const float* __restrict__ D, double* __restrict__ x, int ldx,
                                                   int off, const int* __restrict__ state) {
  if (state[0]) return;
  __shared__ float As[32][33];
  __shared__ float Bs[32][33];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int row0 = blockIdx.y * 32, col0 = blockIdx.x * 32;
  float c00 = 0, c01 = 0, c10 = 0, c11 = 0;
  for (int k0 = 0; k0 < K; k0 += 32) {
    for (int e = threadIdx.x; e < 1024; e += 256) {
      const int r = e >> 5, c = e & 31;
      As[r][c] = (row0 + r < M && k0 + c < K) ? A[(row0 + r) * K + k0 + c] : 0.f;
      Bs[r][c] = (k0 + r < K && col0 + c < N) ? B[(k0 + r) * N + col0 + c] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < 32; kk++) {
      const float a0 = As[2 * ty][kk], a1 = As[2 * ty + 1][kk];
      const float b0 = Bs[kk][2 * tx], b1 = Bs[kk][2 * tx + 1];
      c00 = fmaf(a0, b0, c00);
      c01 = fmaf(a0, b1, c01);
      c10 = fmaf(a1, b0, c10);
      c11 = fmaf(a1, b1, c11);
    }
    __syncthreads();
  }
  const float cv[2][2] = {{c00, c01}, {c10, c11}};
#pragma unroll
  for (int a = 0; a < 2; a++)
#pragma unroll
    for (int b = 0; b < 2; b++) {
      const int r = row0 + 2 * ty + a, c = col0 + 2 * tx + b;
      if (r >= M || c >= N) continue;
      if (EPI == 0) C[r * N + c] = cv[a][b];
      else if (EPI == 1) C[r * N + c] = cv[a][b] * D[r * N + c];
      else x[(r + off) * ldx + (c + off)] += (double)cv[a][b];
    }
}

void launch_spectral(cudaStream_t st, const SpectralSolver& sp, const SolverArgs& a, int stages) {
  const int R = sp.R, C = sp.C;
  const int nb = 152;
  // x lattice (r, c) -> node: flat r*C + c (pcgsolver) or (r+1)*ny + (c+1) (gssolver)
  const int ldx = sp.flat ? C : a.g.ny, off = sp.flat ? 0 : 1;
  k_spec_init<<<(a.g.nx * a.g.ny + 255) / 256, 256, 0, st>>>(a, sp);
  dim3 g2((C + 31) / 32, (R + 31) / 32);
  for (int s = 0; s < stages; s++) {
    k_spec_residual<<<nb, 256, 0, st>>>(a, sp);
    k_spec_check<<<1, 1, 0, st>>>(a, sp, nb, 0);
    k_spec_gemm<0><<<g2, 256, 0, st>>>(R, C, R, sp.QR, sp.t0, sp.t1, nullptr, nullptr, 0, 0, sp.state);
    k_spec_gemm<1><<<g2, 256, 0, st>>>(R, C, C, sp.t1, sp.QC, sp.t0, sp.D, nullptr, 0, 0, sp.state);
    k_spec_gemm<0><<<g2, 256, 0, st>>>(R, C, R, sp.QR, sp.t0, sp.t1, nullptr, nullptr, 0, 0, sp.state);
    k_spec_gemm<2><<<g2, 256, 0, st>>>(R, C, C, sp.t1, sp.QC, nullptr, nullptr, a.phi, ldx, off, sp.state);
  }
  k_spec_residual<<<nb, 256, 0, st>>>(a, sp);
  k_spec_check<<<1, 1, 0, st>>>(a, sp, nb, 1);
}

}  // namespace epic
