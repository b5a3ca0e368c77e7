// C ABI of include/epic2d.h: handle lifetime, device memory, and the
// orchestration of the time-step loop on the handle's CUDA stream.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "epic_host.h"
#include "epic_internal.cuh"

using namespace epic;

namespace {

thread_local std::string g_err;

epic_status fail(epic_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return st;
}

#define CK(call)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess) return fail(e_ == cudaErrorMemoryAllocation ? EPIC_ERR_NOMEM : EPIC_ERR_CUDA, \
                                       "%s: %s", #call, cudaGetErrorString(e_));                 \
  } while (0)

#define CKL()                                                                                     \
  do {                                                                                            \
    cudaError_t e_ = cudaGetLastError();                                                          \
    if (e_ != cudaSuccess) return fail(EPIC_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e_)); \
  } while (0)

// Device allocations are stream-ordered on the handle's stream (and freed
// the same way): a plain cudaMalloc, cudaFree or cudaMemset would serialise
// the work of every other stream on the device, which stalls the other runs a
// server keeps in flight.
template <class T>
epic_status dalloc(epic_sim* s, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  CK(cudaMallocAsync((void**)p, count * sizeof(T), s->stream));
  CK(cudaMemsetAsync(*p, 0, count * sizeof(T), s->stream));
  return EPIC_OK;
}

void dfree(epic_sim* s, void* p) {
  if (p) cudaFreeAsync(p, s->stream);
}

long long nnodes(const epic_sim* s) { return (long long)s->cfg.nx * s->cfg.ny; }

// Reads and clears the device error flags (the stream must be idle).
epic_status take_flags(epic_sim* s) {
  int f = 0;
  CK(cudaMemcpyAsync(&f, s->d_flags, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (!f) return EPIC_OK;
  CK(cudaMemsetAsync(s->d_flags, 0, sizeof(int), s->stream));
  if (f & FLAG_TIMEOUT) return fail(EPIC_ERR_TIMEOUT, "a device-side wait gave up (flags 0x%x)", f);
  if (f & FLAG_CAPACITY) return fail(EPIC_ERR_CAPACITY, "a species outgrew its particle capacity (flags 0x%x)", f);
  if (f & FLAG_LOAD_IN_CONDUCTOR)
    return fail(EPIC_ERR_INVALID, "the load type places a particle inside a conductor (the reference loops forever)");
  if (f & FLAG_OUT_OF_GRID)
    return fail(EPIC_ERR_DOMAIN, "a particle left the grid (the reference raises std::out_of_range here)");
  return fail(EPIC_ERR_CUDA, "device flags 0x%x", f);
}

epic_status sync(epic_sim* s) {
  CK(cudaStreamSynchronize(s->stream));
  return take_flags(s);
}

bool valid_species(epic_sim* s, int i) { return s && i >= 0 && i < (int)s->sp.size(); }

epic_status ensure_tile_status(epic_sim* s, long long cap) {
  long long need = cap / SCAN_TILE + 2;
  if (need <= s->tile_status_len) return EPIC_OK;
  if (s->tile_status) dfree(s, s->tile_status);
  s->tile_status = nullptr;
  epic_status st = dalloc(s, &s->tile_status, (size_t)need);
  if (st) return st;
  s->tile_status_len = need;
  return EPIC_OK;
}

epic_status ensure_staging(epic_sim* s, size_t bytes) {
  if (bytes <= s->staging_bytes) return EPIC_OK;
  if (s->staging) dfree(s, s->staging);
  s->staging = nullptr;
  s->staging_bytes = 0;
  CK(cudaMallocAsync(&s->staging, bytes, s->stream));
  s->staging_bytes = bytes;
  return EPIC_OK;
}

void free_species(epic_sim* s, epic_species_state& sp) {
  void* ptrs[] = {sp.soa.x, sp.soa.y, sp.soa.vx, sp.soa.vy, sp.soa.vz, sp.mx.cell, sp.mx.ox, sp.mx.oy,
                  sp.mx.vx, sp.mx.vy, sp.mx.vz, sp.d_n, sp.den, sp.acc};
  for (void* p : ptrs) dfree(s, p);
}

// Refinement stages of the mixed-precision Poisson solve (each gains ~6
// digits; the loop stops on the reference's tolerance, usually after 2-3).
constexpr int SPECTRAL_STAGES = 6;
// Lattices with a side of at least this many unknowns use FFT passes where
// their sides allow (SpecFFT); a batch holds only smaller ones.
constexpr int SPECTRAL_FFT_MIN = 512;

// Sine transforms and inverse eigenvalues of the reference operator for the
// mixed-precision solve: computed in FP64 on the host, stored in FP32.
static void sine_transform(int n, std::vector<float>& Q, std::vector<double>& lam) {
  const double pi = 3.14159265358979323846;
  const double c = std::sqrt(2.0 / (n + 1));
  Q.assign((size_t)n * n, 0.f);
  lam.assign(n, 0.0);
  for (int j = 0; j < n; j++) {
    for (int k = 0; k < n; k++) Q[(size_t)j * n + k] = (float)(c * std::sin(pi * (j + 1) * (double)(k + 1) / (n + 1)));
    const double sn = std::sin(pi * (j + 1) / (2.0 * (n + 1)));
    lam[j] = -4.0 * sn * sn;
  }
}

// The periodic counterpart: the orthonormal, symmetric Hartley transform
// H_jk = (cos(2 pi j k / n) + sin(2 pi j k / n)) / sqrt(n), which diagonalises
// the circulant tridiag(1, -2, 1) with eigenvalues -4 sin^2(pi k / n) (cos
// and sin modes of wavenumber k share the eigenvalue, so their sum is an
// eigenvector).
static void hartley_transform(int n, std::vector<float>& Q, std::vector<double>& lam) {
  const double pi = 3.14159265358979323846;
  const double c = 1.0 / std::sqrt((double)n);
  Q.assign((size_t)n * n, 0.f);
  lam.assign(n, 0.0);
  for (int j = 0; j < n; j++) {
    for (int k = 0; k < n; k++) {
      const double t = 2.0 * pi * (double)(((long long)j * k) % n) / n;
      Q[(size_t)j * n + k] = (float)(c * (std::cos(t) + std::sin(t)));
    }
    const double sn = std::sin(pi * j / n);
    lam[j] = -4.0 * sn * sn;
  }
}

epic_status setup_spectral(epic_sim* s) {
  SpectralSolver& sp = s->spec;
  const bool gs = s->cfg.solver == EPIC_SOLVER_GS;
  const int mode = s->cfg.poisson_bc;
  sp.mode = mode;
  sp.flat = !gs;
  sp.gs_norm = gs;
  sp.R = gs ? s->cfg.nx - 2 : s->cfg.ny;
  sp.C = gs ? s->cfg.ny - 2 : s->cfg.nx;
  if (mode != EPIC_POISSON_DIRICHLET) {  // the extension lattice (Lattice), the same for both solvers
    sp.flat = 0;
    sp.R = mode == EPIC_POISSON_PERIODIC ? s->cfg.nx - 1 : s->cfg.nx - 2;
    sp.C = s->cfg.ny - 1;
  }
  const int R = sp.R, C = sp.C;
  std::vector<float> QR, QC, D((size_t)R * C);
  std::vector<double> lamR, lamC;
  if (mode == EPIC_POISSON_PERIODIC) hartley_transform(R, QR, lamR);
  else sine_transform(R, QR, lamR);
  if (mode == EPIC_POISSON_DIRICHLET) sine_transform(C, QC, lamC);
  else hartley_transform(C, QC, lamC);
  for (int p = 0; p < R; p++)
    for (int q = 0; q < C; q++) {
      const double l = lamR[p] + lamC[q];
      // The constant mode of the periodic lattice is the operator's null space:
      // the right-hand side has none (projected), the correction gets none.
      D[(size_t)p * C + q] = l == 0.0 ? 0.f : (float)(1.0 / l);
    }
  // FFT passes for large lattices whose sides allow them: the Hartley
  // direction (periodic) of n a power of two, FFT length n; the sine
  // direction of n + 1 a power of two, FFT length 2 (n + 1).  Smaller lattices
  // keep the dense products, whose cost there is the grid barriers' anyway.
  std::memset(&sp.fft, 0, sizeof(sp.fft));
  {
    auto pow2 = [](long long v) { return v >= 2 && (v & (v - 1)) == 0; };
    const int sineR = mode != EPIC_POISSON_PERIODIC, sineC = mode == EPIC_POISSON_DIRICHLET;
    const long long mR = sineR ? 2LL * (R + 1) : R, mC = sineC ? 2LL * (C + 1) : C;
    if (std::max(R, C) >= SPECTRAL_FFT_MIN && pow2(mR) && pow2(mC) && mR <= 4096 && mC <= 4096) {
      SpecFFT& F = sp.fft;
      F.on = 1;
      F.mR = (int)mR;
      F.mC = (int)mC;
      F.lgR = __builtin_ctzll(mR);
      F.lgC = __builtin_ctzll(mC);
      F.sineR = sineR;
      F.sineC = sineC;
      F.scaleR = (float)(sineR ? std::sqrt(2.0 / (R + 1)) : 1.0 / std::sqrt((double)R));
      F.scaleC = (float)(sineC ? std::sqrt(2.0 / (C + 1)) : 1.0 / std::sqrt((double)C));
      const double pi = 3.14159265358979323846;
      for (int d = 0; d < 2; d++) {
        const long long m = d ? mC : mR;
        std::vector<float2> tw((size_t)m / 2);
        for (long long k = 0; k < m / 2; k++)
          tw[(size_t)k] = make_float2((float)std::cos(2.0 * pi * (double)k / (double)m),
                                      (float)-std::sin(2.0 * pi * (double)k / (double)m));
        float2* dt = nullptr;
        CK(cudaMallocAsync((void**)&dt, tw.size() * sizeof(float2), s->stream));
        CK(cudaMemcpyAsync(dt, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice, s->stream));
        CK(cudaStreamSynchronize(s->stream));  // tw is a host temporary
        (d ? F.twC : F.twR) = dt;
      }
    }
  }
  CK(cudaMallocAsync((void**)&sp.QR, QR.size() * sizeof(float), s->stream));
  if (C == R && mode != EPIC_POISSON_DIRICHLET_X) sp.QC = sp.QR;
  else CK(cudaMallocAsync((void**)&sp.QC, QC.size() * sizeof(float), s->stream));
  CK(cudaMallocAsync((void**)&sp.D, D.size() * sizeof(float), s->stream));
  CK(cudaMallocAsync((void**)&sp.t0, D.size() * sizeof(float), s->stream));
  CK(cudaMallocAsync((void**)&sp.t1, D.size() * sizeof(float), s->stream));
  // the residual's chunk sums, then (periodic) those of b and of phi
  CK(cudaMallocAsync((void**)&sp.partials, std::max(256, 2 * spectral_chunks(sp)) * sizeof(double), s->stream));
  CK(cudaMallocAsync((void**)&sp.state, 4 * sizeof(int), s->stream));
  CK(cudaMemcpyAsync(sp.QR, QR.data(), QR.size() * sizeof(float), cudaMemcpyHostToDevice, s->stream));
  if (sp.QC != sp.QR)
    CK(cudaMemcpyAsync(sp.QC, QC.data(), QC.size() * sizeof(float), cudaMemcpyHostToDevice, s->stream));
  CK(cudaMemcpyAsync(sp.D, D.data(), D.size() * sizeof(float), cudaMemcpyHostToDevice, s->stream));
  CK(cudaMemsetAsync(sp.state, 0, 4 * sizeof(int), s->stream));
  CK(cudaStreamSynchronize(s->stream));  // host temporaries
  return EPIC_OK;
}

__global__ void k_aos_to_soa(const double* __restrict__ aos, SoA p, long long n) {
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const double* r = aos + 5 * q;
    p.x[q] = r[0]; p.y[q] = r[1]; p.vx[q] = r[2]; p.vy[q] = r[3]; p.vz[q] = r[4];
  }
}

__global__ void k_soa_to_aos(double* __restrict__ aos, SoA p, const long long* d_n) {
  const long long n = *d_n;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    double* r = aos + 5 * q;
    r[0] = p.x[q]; r[1] = p.y[q]; r[2] = p.vx[q]; r[3] = p.vy[q]; r[4] = p.vz[q];
  }
}

// Per-phase CUDA events on the handle's stream (epic_set_profiling), and an
// NVTX range per phase on the calling thread (always; free without a tool
// attached), so that profilers can attribute and filter the phases.
static const char* const kPhaseNames[EPIC_NUM_PHASES] = {"epic deposit", "epic finalize", "epic solve",
                                                         "epic efield",  "epic push",     "epic mcc",
                                                         "epic sort"};
struct PhaseTimer {
  epic_sim* s;
  int phase;
  cudaEvent_t a = nullptr, b = nullptr;
  struct Nvtx {
    explicit Nvtx(int p) { nvtxRangePushA(kPhaseNames[p]); }
    ~Nvtx() { nvtxRangePop(); }
  } nvtx;
  static cudaEvent_t take(epic_sim* s) {
    if (!s->event_pool.empty()) {
      cudaEvent_t e = s->event_pool.back();
      s->event_pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
  PhaseTimer(epic_sim* s_, int p) : s(s_), phase(p), nvtx(p) {
    if (!s->profiling) return;
    cudaStreamCaptureStatus cs;
    if (cudaStreamIsCapturing(s->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return;
    a = take(s);
    b = take(s);
    cudaEventRecord(a, s->stream);
  }
  ~PhaseTimer() {
    if (!a) return;
    cudaEventRecord(b, s->stream);
    s->prof_pending.push_back({phase, {a, b}});
  }
};

// ---- phase launchers (no synchronisation; usable inside stream capture) ----
// The step deposits each pushed species while it moves it (the push kernel
// with an accumulator) and the MCC's products after the MCC, so the next
// step's deposit is already in the accumulators: the same integer sums,
// without a second pass over the positions.  Periodic or reflective walls, no
// conductors or emitters; the FP64 form with the fixed-point deposit, the
// mixed form with CIC.
static bool fused_deposit(const epic_sim* s) {
  if (!s->conductors.empty() || !s->emitters.empty() || (s->cfg.bc != EPIC_PBC && s->cfg.bc != EPIC_REFLECTIVE))
    return false;
  return s->mixed ? s->cfg.shape == EPIC_CIC : s->cfg.deposit_mode == EPIC_DEPOSIT_FIXED;
}

static void invalidate_acc(epic_sim* s) {
  for (auto& sp : s->sp) sp.acc_valid = false;
}

epic_status do_deposit(epic_sim* s, int i) {
  PhaseTimer t(s, 0);
  epic_species_state& sp = s->sp[i];
  sp.acc_valid = true;
  CK(cudaMemsetAsync(sp.acc, 0, nnodes(s) * sizeof(unsigned long long), s->stream));
  if (s->mixed && s->cfg.shape == EPIC_CIC)
    launch_deposit_mixed_sorted(s->stream, s->g, sp.mx, sp.d_n, sp.acc, s->part_grid);
  else if (s->mixed)
    launch_deposit_mixed(s->stream, s->g, s->cfg.shape, sp.mx, sp.d_n, sp.acc, s->d_flags, s->part_grid);
  else
    launch_deposit(s->stream, s->g, s->cfg.shape, s->cfg.deposit_mode == EPIC_DEPOSIT_FIXED, sp.soa, sp.d_n,
                   sp.desc.spwt, sp.den, sp.acc, sp.fx_scale, s->d_flags, s->part_grid);
  s->launches += 1;
  CKL();
  return EPIC_OK;
}

FinalizeArgs finalize_args(epic_sim* s, int stage, int only) {
  FinalizeArgs a;
  std::memset(&a, 0, sizeof(a));
  a.g = s->g;
  a.bc = s->cfg.bc;
  a.fixed = s->mixed || s->cfg.deposit_mode == EPIC_DEPOSIT_FIXED;
  a.stage = stage;
  double cell_area = s->cfg.dx * s->cfg.dy;
  double L2 = s->cfg.L * s->cfg.L;
  a.div = cell_area * L2 * s->cfg.density;
  a.nsp = (int)s->sp.size();
  for (int k = 0; k < a.nsp; k++) {
    epic_species_state& sp = s->sp[k];
    a.acc[k] = sp.acc;
    a.den[k] = sp.den;
    a.spwt[k] = sp.desc.spwt;
    a.inv_scale[k] = s->mixed ? std::ldexp(1.0, -2 * MIXED_OFFSET_BITS) : sp.fx_inv_scale;
    a.charge_over_qe[k] = sp.desc.charge * (1 / QE);
    a.active[k] = only < 0 || only == k;
  }
  a.rho = s->rho;
  return a;
}

epic_status do_finalize(epic_sim* s, int stage, int only) {
  PhaseTimer t(s, 1);
  launch_finalize(s->stream, finalize_args(s, stage, only));
  s->launches += 1;
  CKL();
  return EPIC_OK;
}

SolverArgs solver_args(epic_sim* s) {
  SolverArgs a;
  std::memset(&a, 0, sizeof(a));
  a.g = s->g;
  a.tol = s->cfg.tolerance;
  a.max_iter = s->cfg.max_iteration;
  a.omega = s->cfg.sor_omega;
  a.K = (s->cfg.L * s->cfg.L) / (s->cfg.LDe * s->cfg.LDe);
  a.rho = s->rho;
  a.phi = s->phi;
  a.info = s->d_info;
  a.iter_total = s->d_iter_total;
  a.flags = s->d_flags;
  for (int k = 0; k < 8; k++) a.work[k] = s->work[k];
  a.partials = s->partials;
  a.bar = s->bar;
  a.warm = s->cfg.warm_start;
  a.poisson_bc = s->cfg.poisson_bc;
  return a;
}

int solver_blocks(epic_sim* s, long long nodes_per_block) {
  int mx = solver_max_blocks();
  if (s->cfg.solver_blocks > 0) return std::min(s->cfg.solver_blocks, mx);
  // One CTA per SM at most: a sweep over 16..304 CTAs on 65^2..257^2 grids
  // found the per-iteration time lowest between 130 and 152 CTAs and worse
  // at two per SM (more barrier arrivals, no more FP64 throughput per SM).
  long long want = (nnodes(s) + nodes_per_block - 1) / nodes_per_block;
  return (int)std::max(1LL, std::min<long long>(want, std::min(mx, s->num_sms)));
}

epic_status do_solve(epic_sim* s) {
  PhaseTimer t(s, 2);
  SolverArgs a = solver_args(s);
  if (s->mixed && s->spec.QR) {
    if (s->cfg.solver == EPIC_SOLVER_GS && !s->conductors.empty()) {
      // Grid::initialize inside gssolver (src/field.cpp:100-103): the same
      // right-hand side for the spectral solve of the same operator
      launch_conductor_rho(s->stream, s->rho, s->d_cond_nodes, s->d_cond_vals, s->cond_nnodes, s->d_cond_live);
      s->launches += 1;
    }
    launch_spectral(s->stream, s->spec, a, SPECTRAL_STAGES);
    // set-up, the cooperative solve, the duplicated nodes (extensions)
    s->launches += 2 + (s->spec.mode != EPIC_POISSON_DIRICHLET ? 1 : 0);
    CKL();
    return EPIC_OK;
  }
  if (s->cfg.solver == EPIC_SOLVER_GSHYBRID) {
    launch_gsfluid(s->stream, a, s->rho);
  } else if (s->cfg.solver == EPIC_SOLVER_HYBRID) {
    launch_nrpcg(s->stream, a);
  } else if (s->cfg.solver == EPIC_SOLVER_GS) {
    if (!s->conductors.empty()) {  // Grid::initialize inside gssolver (src/field.cpp:100-103)
      launch_conductor_rho(s->stream, s->rho, s->d_cond_nodes, s->d_cond_vals, s->cond_nnodes, s->d_cond_live);
      s->launches += 1;
    }
    if (s->cfg.sor_mode == EPIC_SOR_LEXICOGRAPHIC) launch_sor_lex(s->stream, a);
    else launch_sor_redblack(s->stream, a, solver_blocks(s, 1024));
  } else {
    const int nb = s->cfg.solver_blocks > 0 ? std::min(s->cfg.solver_blocks, solver_max_blocks())
                                            : pcg_default_blocks(nnodes(s), s->num_sms);
    launch_pcg(s->stream, a, nb);
  }
  s->launches += s->cfg.poisson_bc != EPIC_POISSON_DIRICHLET ? 2 : 1;  // + the duplicated nodes' fill
  CKL();
  return EPIC_OK;
}

epic_status do_efield(epic_sim* s) {
  PhaseTimer t(s, 3);
  launch_efield(s->stream, s->g, s->cfg.bc, s->cfg.poisson_bc, s->phi, s->efx, s->efy, s->ef,
                s->mixed ? s->ef32 : nullptr);
  s->launches += 1;
  if (s->ef_cell) {
    launch_cell_coef(s->stream, s->g, s->ef, s->ef_cell);
    s->launches += 1;
  }
  CKL();
  return EPIC_OK;
}

epic_status do_push(epic_sim* s, int i, int sub_cycle, const SelectArgs* sel = nullptr) {
  PhaseTimer t(s, 4);
  epic_species_state& sp = s->sp[i];
  const epic_config& c = s->cfg;
  double qm = sp.desc.charge / sp.desc.mass;
  double K = (c.density * QE * c.L) / (EPS_0 * c.W * c.vel_norm);
  double qmK = qm * K;
  double cc = (c.vel_norm) / (c.L * c.W);
  double dtsub = c.DT * sub_cycle;
  const bool cond = !s->conductors.empty();
  if (c.bc == EPIC_OPEN || cond) {
    CK(cudaMemsetAsync(s->tile_ctr, 0, sizeof(unsigned int), s->stream));
    CK(cudaMemsetAsync(s->tile_status, 0, s->tile_status_len * sizeof(unsigned long long), s->stream));
  }
  sp.acc_valid = false;
  if (cond && !s->mixed) {
    const CondSet cs{s->cond_nrect, s->cond_ncirc, s->d_cond_rect, s->d_cond_circ, s->d_cond_live};
    launch_push_conductors(s->stream, s->g, c.shape, c.bc, sp.soa, sp.d_n, s->ef, s->ef_cell, qmK, cc, dtsub, cs,
                           s->d_flags,
                           s->tile_status, s->tile_ctr, s->part_grid, c.push_order == EPIC_PUSH_CONTRACTED);
  } else if (s->mixed) {
    const bool dep = fused_deposit(s);
    if (dep) CK(cudaMemsetAsync(sp.acc, 0, nnodes(s) * sizeof(unsigned long long), s->stream));
    const CondSet cs{s->cond_nrect, s->cond_ncirc, s->d_cond_rect, s->d_cond_circ, s->d_cond_live};
    launch_push_mixed(s->stream, s->g, c.shape, c.bc, sp.mx, sp.d_n, s->ef32, (float)(qmK * dtsub),
                      (float)(cc * dtsub / c.dx), (float)(cc * dtsub / c.dy), s->d_flags, s->tile_status,
                      s->tile_ctr, s->part_grid, dep ? sp.acc : nullptr, dep ? sel : nullptr, cond ? &cs : nullptr);
    sp.acc_valid = dep;
  } else {
    const bool dep = fused_deposit(s);
    if (dep) CK(cudaMemsetAsync(sp.acc, 0, nnodes(s) * sizeof(unsigned long long), s->stream));
    launch_push(s->stream, s->g, c.shape, c.bc, sp.soa, sp.d_n, s->ef, s->ef_cell, qmK, cc, dtsub, s->d_flags,
                s->tile_status, s->tile_ctr, s->part_grid, c.push_order == EPIC_PUSH_CONTRACTED,
                dep ? sp.acc : nullptr, sp.fx_scale, dep ? sel : nullptr);
    sp.acc_valid = dep;
  }
  s->launches += 1;
  CKL();
  return EPIC_OK;
}

// Event scratch of the MCC for an electron capacity: marks (-1 = none) for
// every slot, per-tile counts, and products for up to cap/8 ionisations per
// call (more raise EPIC_ERR_CAPACITY).  Allocates, so it must run outside
// stream capture; epic_run calls it before capturing.
epic_status ensure_mcc_events(epic_sim* s, long long e_cap) {
  if (s->mcc_ev_for_cap >= e_cap) return EPIC_OK;
  cudaStreamCaptureStatus cs;
  if (cudaStreamIsCapturing(s->stream, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone)
    return fail(EPIC_ERR_INVALID, "MCC scratch must be allocated before stream capture");
  McEvents& ev = s->mcc_ev;
  dfree(s, ev.buf); dfree(s, ev.count); dfree(s, ev.slot); dfree(s, ev.tile_cnt); dfree(s, ev.tile_off);
  dfree(s, ev.cand); dfree(s, ev.cand_count);
  std::memset(&ev, 0, sizeof(ev));
  s->mcc_ev_for_cap = 0;
  const size_t tiles = (size_t)(e_cap / MCC_TILE + 2);
  ev.cap = (unsigned int)std::min<long long>(std::max<long long>(e_cap / 8, 65536), 1LL << 30);
  CK(cudaMallocAsync((void**)&ev.buf, (size_t)ev.cap * ion_event_bytes(), s->stream));
  CK(cudaMallocAsync((void**)&ev.cand, (size_t)e_cap * sizeof(unsigned int), s->stream));
  CK(cudaMallocAsync((void**)&ev.cand_count, sizeof(unsigned int), s->stream));
  CK(cudaMemsetAsync(ev.cand_count, 0, sizeof(unsigned int), s->stream));
  CK(cudaMallocAsync((void**)&ev.count, sizeof(unsigned int), s->stream));
  CK(cudaMallocAsync((void**)&ev.slot, (size_t)e_cap * sizeof(int), s->stream));
  CK(cudaMallocAsync((void**)&ev.tile_cnt, tiles * sizeof(unsigned int), s->stream));
  CK(cudaMallocAsync((void**)&ev.tile_off, tiles * sizeof(unsigned int), s->stream));
  CK(cudaMemsetAsync(ev.count, 0, sizeof(unsigned int), s->stream));
  CK(cudaMemsetAsync(ev.slot, 0xff, (size_t)e_cap * sizeof(int), s->stream));
  CK(cudaMemsetAsync(ev.tile_cnt, 0, tiles * sizeof(unsigned int), s->stream));
  s->mcc_ev_for_cap = e_cap;
  return EPIC_OK;
}

epic_status do_mcc(epic_sim* s, int e, int ion, const double* d_uniforms, int ustride, int skip_select = 0) {
  PhaseTimer t(s, 5);
  if (!s->cs.tot) return fail(EPIC_ERR_INVALID, "cross sections not set (epic_set_reference_cross_sections)");
  epic_species_state& E = s->sp[e];
  epic_species_state& I = s->sp[ion];
  const epic_config& c = s->cfg;
  if (s->mcc_ev_for_cap < E.cap) {
    epic_status st = ensure_mcc_events(s, E.cap);
    if (st) return st;
  }
  int mode = c.mcc_mode;
  if (mode == EPIC_MCC_INJECTED && !d_uniforms) mode = EPIC_MCC_PHILOX;
  const ParticleRef er{s->mixed, E.soa, E.mx}, ir{s->mixed, I.soa, I.mx};
  launch_mcc(s->stream, mode, s->cs, er, E.d_n, E.cap, ir, I.d_n, I.cap, c.vel_norm, c.DT / c.W, I.desc.mass,
             I.desc.temp, d_uniforms, ustride, c.seed, s->d_step, s->mcc_ev, s->d_ncoll, s->d_flags, s->part_grid,
             skip_select);
  s->launches += skip_select ? 4 : 5;
  CKL();
  return EPIC_OK;
}

// The loop body of src/main.cpp:405-423 as a launch sequence.
// Scratch of the cell sort, sized for the largest species (allocated before
// any graph capture).
epic_status ensure_sort_scratch(epic_sim* s) {
  long long cap = 0;
  for (auto& sp : s->sp) cap = std::max(cap, sp.cap);
  if (s->sort_buf && s->sort_cap >= cap) return EPIC_OK;
  if (s->sort_buf) dfree(s, s->sort_buf);
  s->sort_buf = nullptr;
  if (cudaMallocAsync(&s->sort_buf, sort_scratch_bytes(cap, s->mixed ? 24 : 40), s->stream) != cudaSuccess) {
    cudaGetLastError();
    return fail(EPIC_ERR_NOMEM, "cell sort scratch (%lld particles)", cap);
  }
  s->sort_cap = cap;
  return EPIC_OK;
}

epic_status do_sort(epic_sim* s, int i) {
  PhaseTimer t(s, 6);
  epic_status st = ensure_sort_scratch(s);
  if (st) return st;
  epic_species_state& sp = s->sp[i];
  ParticleRef p;
  p.mixed = s->mixed;
  p.f = sp.soa;
  p.m = sp.mx;
  s->launches += launch_sort(s->stream, s->g, p, sp.d_n, sp.cap, carve_sort_scratch(s->sort_buf, sp.cap),
                             s->part_grid);
  CKL();
  return EPIC_OK;
}

// Emitter::inject of every emitter (src/emitter.cpp:5-36); d_uniforms: null
// for Philox, else device rows of 14 per point, emitters in order.
// Emitters [k0, k1) in order; tick: advance the injection counter that keys
// their Philox streams (once per loop iteration, after the last emitter).
epic_status do_inject_range(epic_sim* s, size_t k0, size_t k1, const double* d_uniforms, bool tick) {
  const epic_config& c = s->cfg;
  const double* u = d_uniforms;
  for (size_t k = k0; k < k1; k++) {
    const epic_emitter& m = s->emitters[k];
    const int sp_of[2] = {m.species_idx1, m.species_idx2};
    const int slots = m.species_idx1 != m.species_idx2 ? 2 : 1;
    for (int slot = 0; slot < slots; slot++) {
      epic_species_state& sp = s->sp[sp_of[slot]];
      EmitDev e;
      e.x0 = m.x0;
      e.y0 = m.y0;
      e.x1 = m.x1;
      e.y1 = m.y1;
      e.vth = sqrt(2 * K_B * m.temp * (QE / K_B) / sp.desc.mass);  // Init::SampleVel (src/init.cpp:112)
      e.vdx = m.vdx * c.vel_norm;
      e.vdy = m.vdy * c.vel_norm;
      e.vel_norm = c.vel_norm;
      e.num = m.numparticle;
      e.slot = slot;
      e.emitter = (int)k;
      launch_emit(s->stream, ParticleRef{s->mixed, sp.soa, sp.mx}, s->g, sp.d_n, sp.cap, e, c.seed, s->d_inj, u,
                  s->d_flags, s->part_grid);
    }
    for (int slot = 0; slot < slots; slot++) {
      epic_species_state& sp = s->sp[sp_of[slot]];
      launch_emit_commit(s->stream, sp.d_n, m.numparticle, sp.cap, s->d_flags);
    }
    s->launches += 2 * slots;
    if (u) u += (size_t)m.numparticle * 14;
  }
  if (tick) {
    launch_inject_tick(s->stream, s->d_inj);
    s->launches += 1;
  }
  CKL();
  return EPIC_OK;
}

epic_status do_inject(epic_sim* s, const double* d_uniforms) {
  return do_inject_range(s, 0, s->emitters.size(), d_uniforms, true);
}

// sort: -1 by the step counter and cfg.sort_every, 0 never, 1 always.
// A step is do_step_field (emitters, cell sort, deposit, rho, solve, E-field)
// then do_step_move (push, MCC, deposit of the MCC's products).
epic_status do_step_field(epic_sim* s, int sort = -1) {
  epic_status st;
  const int nsp = (int)s->sp.size();
  if (!s->emitters.empty() && (st = do_inject(s, nullptr))) return st;  // src/main.cpp:397-403
  if (sort < 0) sort = s->cfg.sort_every > 0 && s->step_index % s->cfg.sort_every == 0;
  s->step_index++;
  if (sort)
    for (int i = 0; i < nsp; i++)
      if ((st = do_sort(s, i))) return st;
  const bool fused = fused_deposit(s);
  for (int i = 0; i < nsp; i++)
    if (!(fused && (s->steady_capture || s->sp[i].acc_valid)))
      if ((st = do_deposit(s, i))) return st;
  if ((st = do_finalize(s, FINALIZE_AND_RHO, -1))) return st;
  if ((st = do_solve(s))) return st;
  return do_efield(s);
}

epic_status do_step_move(epic_sim* s, int with_collisions) {
  epic_status st;
  const int nsp = (int)s->sp.size();
  const bool fused = fused_deposit(s);
  // The MCC's selection pass folded into the electrons' push (the same test on
  // the same post-push velocities, one pass over them fewer).
  const bool coll = with_collisions && nsp >= 2;
  const bool presel = coll && fused && (s->mixed || s->cfg.push_order == EPIC_PUSH_CONTRACTED) && s->cs.tot &&
                      !(s->cfg.ionfixed == 1 && s->sp[0].name == "ion");
  SelectArgs sel{};
  if (presel) {
    if (s->mcc_ev_for_cap < s->sp[0].cap && (st = ensure_mcc_events(s, s->sp[0].cap))) return st;
    const int mode = s->cfg.mcc_mode == EPIC_MCC_INJECTED ? EPIC_MCC_PHILOX : s->cfg.mcc_mode;
    mcc_select_cut(s->cs, mode, s->cfg.DT / s->cfg.W, &sel.cut53, &sel.bin_cut);
    sel.seed = s->cfg.seed;
    sel.d_step = s->d_step;
    sel.cand = s->mcc_ev.cand;
    sel.cand_count = s->mcc_ev.cand_count;
  }
  for (int i = 0; i < nsp; i++) {
    if (s->cfg.ionfixed == 1 && s->sp[i].name == "ion") continue;
    if ((st = do_push(s, i, 1, presel && i == 0 ? &sel : nullptr))) return st;
  }
  if (coll) {
    if (fused)  // counts before the MCC: its ionisation products are deposited after it
      for (int k = 0; k < 2; k++)
        CK(cudaMemcpyAsync(s->d_nold + k, s->sp[k].d_n, sizeof(long long), cudaMemcpyDeviceToDevice, s->stream));
    if ((st = do_mcc(s, 0, 1, nullptr, 0, presel))) return st;
    if (fused) {
      PhaseTimer t(s, 0);
      for (int k = 0; k < 2; k++) {
        epic_species_state& sp = s->sp[k];
        if (s->mixed)
          launch_deposit_mixed_range(s->stream, s->g, sp.mx, s->d_nold + k, sp.d_n, sp.acc, s->part_grid);
        else
          launch_deposit_range(s->stream, s->g, s->cfg.shape, sp.soa, s->d_nold + k, sp.d_n, sp.acc, sp.fx_scale,
                               s->d_flags, s->part_grid);
        s->launches += 1;
      }
      CKL();
    }
  }
  return EPIC_OK;
}

epic_status do_step(epic_sim* s, int with_collisions, int sort = -1) {
  epic_status st = do_step_field(s, sort);
  if (st) return st;
  return do_step_move(s, with_collisions);
}

}  // namespace

namespace epic {
void set_last_error(const char* msg) { g_err = msg; }

static std::atomic<long long> g_spin_limit{SPIN_LIMIT};
long long spin_limit() { return g_spin_limit.load(std::memory_order_relaxed); }
}  // namespace epic

extern "C" {

const char* epic_last_error(void) { return g_err.c_str(); }

epic_status epic_set_spin_limit(long long polls) {
  g_spin_limit.store(polls > 0 ? polls : SPIN_LIMIT, std::memory_order_relaxed);
  return EPIC_OK;
}

void epic_config_defaults(epic_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->dx = c->dy = 1.0;
  c->shape = EPIC_CIC;
  c->bc = EPIC_PBC;
  c->solver = EPIC_SOLVER_GS;
  c->tolerance = 1e-3;
  c->max_iteration = 4000;
  c->sor_omega = 1.4;
  c->sor_mode = EPIC_SOR_LEXICOGRAPHIC;
  c->deposit_mode = EPIC_DEPOSIT_FIXED;
  c->mcc_mode = EPIC_MCC_PHILOX;
  c->seed = 0;
  c->warm_start = 0;
}

epic_status epic_config_from_ini(const char* path, epic_config* cfg, epic_species_desc* species, int max_species,
                                 int* num_species, int* num_ts) {
  if (!path || !cfg || !num_species) return fail(EPIC_ERR_INVALID, "null argument");
  std::string err;
  int st = config_from_ini(path, cfg, species, max_species, num_species, num_ts, err);
  if (st) return fail((epic_status)st, "%s", err.c_str());
  return EPIC_OK;
}

epic_status epic_conductors_from_ini(const char* path, epic_conductor* out, int max, int* count) {
  if (!path || !count || (max > 0 && !out)) return fail(EPIC_ERR_INVALID, "bad argument");
  std::vector<epic_conductor> v;
  std::string err;
  int st = conductors_from_ini(path, v, err);
  if (st) return fail((epic_status)st, "%s", err.c_str());
  *count = (int)v.size();
  for (int k = 0; k < (int)v.size() && k < max; k++) out[k] = v[k];
  return EPIC_OK;
}

epic_status epic_add_conductor(epic_sim* s, const epic_conductor* c) {
  if (!s || !c) return fail(EPIC_ERR_INVALID, "bad argument");
  if (s->cfg.poisson_bc != EPIC_POISSON_DIRICHLET)
    return fail(EPIC_ERR_INVALID, "conductors are supported with the reference's Poisson boundary");
  if (c->type != EPIC_CONDUCTOR_RECT && c->type != EPIC_CONDUCTOR_CIRCULAR)
    return fail(EPIC_ERR_INVALID, "unknown conductor type %d", c->type);
  if (c->type == EPIC_CONDUCTOR_CIRCULAR && (c->electrode_number < 1 || c->electrode_number > 4096))
    return fail(EPIC_ERR_INVALID, "electrode_number must be in [1, 4096]");
  s->conductors.push_back(*c);
  std::vector<double> rects, circles, vals;
  std::vector<int> nodes;
  conductor_geometry(s->cfg, s->conductors, rects, circles, nodes, vals);
  void* old[] = {s->d_cond_rect, s->d_cond_circ, s->d_cond_nodes, s->d_cond_vals};
  for (void* p : old)
    if (p) dfree(s, p);
  s->d_cond_rect = nullptr;
  s->d_cond_circ = nullptr;
  s->d_cond_nodes = nullptr;
  s->d_cond_vals = nullptr;
  s->cond_nrect = (int)(rects.size() / 4);
  s->cond_ncirc = (int)(circles.size() / 4);
  s->cond_nnodes = (int)nodes.size();
  auto up = [&](void** dst, const void* src, size_t bytes) -> epic_status {
    CK(cudaMallocAsync(dst, std::max<size_t>(bytes, 16), s->stream));
    if (bytes) CK(cudaMemcpyAsync(*dst, src, bytes, cudaMemcpyHostToDevice, s->stream));
    return EPIC_OK;
  };
  epic_status st;
  if ((st = up((void**)&s->d_cond_rect, rects.data(), rects.size() * sizeof(double))) ||
      (st = up((void**)&s->d_cond_circ, circles.data(), circles.size() * sizeof(double))) ||
      (st = up((void**)&s->d_cond_nodes, nodes.data(), nodes.size() * sizeof(int))) ||
      (st = up((void**)&s->d_cond_vals, vals.data(), vals.size() * sizeof(double))))
    return st;
  if (!s->d_cond_live) CK(cudaMallocAsync((void**)&s->d_cond_live, sizeof(int), s->stream));
  CK(cudaMemsetAsync(s->d_cond_live, 0, sizeof(int), s->stream));
  // A captured step holds the old geometry.
  if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
  if (s->graph_exec_sort) cudaGraphExecDestroy(s->graph_exec_sort);
  s->graph_exec = s->graph_exec_sort = nullptr;
  return sync(s);  // the host vectors go out of scope
}

epic_status epic_emitters_from_ini(const char* path, epic_emitter* out, int max, int* count) {
  if (!path || !count || (max > 0 && !out)) return fail(EPIC_ERR_INVALID, "bad argument");
  std::vector<epic_emitter> v;
  std::string err;
  int st = emitters_from_ini(path, v, err);
  if (st) return fail((epic_status)st, "%s", err.c_str());
  *count = (int)v.size();
  for (int k = 0; k < (int)v.size() && k < max; k++) out[k] = v[k];
  return EPIC_OK;
}

epic_status epic_add_emitter(epic_sim* s, const epic_emitter* e) {
  if (!s || !e) return fail(EPIC_ERR_INVALID, "bad argument");
  const int nsp = (int)s->sp.size();
  if (e->species_idx1 < 0 || e->species_idx1 >= nsp || e->species_idx2 < 0 || e->species_idx2 >= nsp)
    return fail(EPIC_ERR_INVALID, "emitter species index out of range (add the species first)");
  if (e->numparticle < 0 || e->numparticle > (1 << 28)) return fail(EPIC_ERR_INVALID, "bad numparticle");
  if (!s->d_inj) {
    CK(cudaMallocAsync((void**)&s->d_inj, sizeof(unsigned long long), s->stream));
    CK(cudaMemsetAsync(s->d_inj, 0, sizeof(unsigned long long), s->stream));
  }
  s->emitters.push_back(*e);
  // A captured step has no injection for it.
  if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
  if (s->graph_exec_sort) cudaGraphExecDestroy(s->graph_exec_sort);
  s->graph_exec = s->graph_exec_sort = nullptr;
  return sync(s);
}

epic_status epic_inject(epic_sim* s, const double* uniforms) {
  if (!s) return fail(EPIC_ERR_INVALID, "null handle");
  if (s->emitters.empty()) return EPIC_OK;
  invalidate_acc(s);
  const double* d_u = nullptr;
  if (uniforms) {
    size_t rows = 0;
    for (const epic_emitter& m : s->emitters) rows += (size_t)m.numparticle;
    epic_status st = ensure_staging(s, std::max<size_t>(1, rows * 14 * sizeof(double)));
    if (st) return st;
    CK(cudaMemcpyAsync(s->staging, uniforms, rows * 14 * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    d_u = (const double*)s->staging;
  }
  epic_status st = do_inject(s, d_u);
  if (st) return st;
  return sync(s);
}

epic_status epic_inject_emitter(epic_sim* s, int k, const double* uniforms) {
  if (!s || k < 0 || k >= (int)s->emitters.size()) return fail(EPIC_ERR_INVALID, "bad emitter index");
  invalidate_acc(s);
  const double* d_u = nullptr;
  if (uniforms) {
    const size_t rows = (size_t)s->emitters[(size_t)k].numparticle;
    epic_status st = ensure_staging(s, std::max<size_t>(1, rows * 14 * sizeof(double)));
    if (st) return st;
    CK(cudaMemcpyAsync(s->staging, uniforms, rows * 14 * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    d_u = (const double*)s->staging;
  }
  epic_status st = do_inject_range(s, (size_t)k, (size_t)k + 1, d_u, k + 1 == (int)s->emitters.size());
  if (st) return st;
  return sync(s);
}

epic_status epic_ini_get(const char* path, const char* section, const char* key, char* out, int len) {
  if (!path || !section || !key || !out || len < 1) return fail(EPIC_ERR_INVALID, "bad argument");
  std::string v, err;
  int st = ini_get(path, section, key, v, err);
  if (st) return fail((epic_status)st, "%s", err.c_str());
  std::snprintf(out, (size_t)len, "%s", v.c_str());
  return EPIC_OK;
}

epic_status epic_create(const epic_config* cfg, epic_sim** out) {
  if (!cfg || !out) return fail(EPIC_ERR_INVALID, "null argument");
  *out = nullptr;
  if (cfg->nx < 3 || cfg->ny < 3) return fail(EPIC_ERR_INVALID, "grid needs at least 3x3 nodes");
  if (!(cfg->dx > 0) || !(cfg->dy > 0) || !(cfg->L > 0) || !(cfg->W > 0) || !(cfg->vel_norm > 0) ||
      !(cfg->density > 0) || !(cfg->LDe > 0))
    return fail(EPIC_ERR_INVALID, "dx, dy, L, W, vel_norm, LDe and density must be positive");
  if (cfg->shape != EPIC_CIC && cfg->shape != EPIC_NGP) return fail(EPIC_ERR_INVALID, "bad shape");
  if (cfg->bc < EPIC_PBC || cfg->bc > EPIC_REFLECTIVE) return fail(EPIC_ERR_INVALID, "bad bc");
  if (cfg->solver < EPIC_SOLVER_GS || cfg->solver > EPIC_SOLVER_HYBRID) return fail(EPIC_ERR_INVALID, "bad solver");
  if (cfg->push_order != EPIC_PUSH_CONTRACTED && cfg->push_order != EPIC_PUSH_REFERENCE)
    return fail(EPIC_ERR_INVALID, "bad push_order");
  if (cfg->poisson_bc < EPIC_POISSON_DIRICHLET || cfg->poisson_bc > EPIC_POISSON_DIRICHLET_X)
    return fail(EPIC_ERR_INVALID, "bad poisson_bc");
  if (cfg->poisson_bc != EPIC_POISSON_DIRICHLET) {
    if (cfg->nx < 5 || cfg->ny < 5) return fail(EPIC_ERR_INVALID, "poisson_bc periodic/dirichlet_x needs 5x5 nodes");
    if (!(cfg->solver == EPIC_SOLVER_PCG ||
          (cfg->solver == EPIC_SOLVER_GS && cfg->sor_mode == EPIC_SOR_LEXICOGRAPHIC)))
      return fail(EPIC_ERR_INVALID, "poisson_bc periodic/dirichlet_x is supported by the cg and (lexicographic) gs "
                                    "solvers");
  }
  int dev = 0;
  CK(cudaGetDevice(&dev));
  init_field_kernels();
  epic_sim* s = new epic_sim();
  s->cfg = *cfg;
  s->g.nx = cfg->nx;
  s->g.ny = cfg->ny;
  s->g.x0 = cfg->x0;
  s->g.y0 = cfg->y0;
  s->g.dx = cfg->dx;
  s->g.dy = cfg->dy;
  s->g.Lx = (cfg->nx - 1) * cfg->dx;
  s->g.Ly = (cfg->ny - 1) * cfg->dy;
  cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, dev);
  s->part_grid = s->num_sms * 8;
  epic_status st = EPIC_OK;
  const size_t nn = (size_t)nnodes(s);
  auto guard = [&](epic_status x) {
    if (x && !st) st = x;
  };
  guard(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) == cudaSuccess ? EPIC_OK : EPIC_ERR_CUDA);
  {
    // Keep freed stream-ordered memory in the device's pool (returning it to
    // the system would synchronise); a process-local setting.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  }
  guard(dalloc(s, &s->phi, nn));
  guard(dalloc(s, &s->rho, nn));
  guard(dalloc(s, &s->efx, nn));
  guard(dalloc(s, &s->efy, nn));
  guard(dalloc(s, &s->ef, nn));
  for (int k = 0; k < 8; k++) guard(dalloc(s, &s->work[k], nn));
  // Solver partials: up to 2 parities x 48 bytes per CTA (PCG), 16 doubles per CTA.
  guard(dalloc(s, &s->partials, 16 * (size_t)std::max(solver_max_blocks(), 320)));
  guard(dalloc(s, &s->bar, 2));
  guard(dalloc(s, &s->d_info, 1));
  guard(dalloc(s, &s->d_iter_total, 1));
  guard(dalloc(s, &s->tile_ctr, 1));
  guard(dalloc(s, &s->d_ncoll, 4));
  guard(dalloc(s, &s->d_step, 1));
  guard(dalloc(s, &s->sum_partials, 3 * (size_t)s->part_grid));
  guard(dalloc(s, &s->d_sums, 4));
  guard(dalloc(s, &s->d_flags, 1));
  guard(dalloc(s, &s->d_nold, 2));
  s->mixed = cfg->precision == EPIC_PRECISION_MIXED;
  if (s->mixed) {
    guard(dalloc(s, &s->ef32, nn));
    if (spectral_supported(s->g, cfg->solver, cfg->poisson_bc) && !st) guard(setup_spectral(s));
  } else if (cfg->shape == EPIC_CIC && cfg->push_order == EPIC_PUSH_CONTRACTED) {
    guard(dalloc(s, &s->ef_cell, 4 * (size_t)nn));
  }
  if (!st && cudaStreamSynchronize(s->stream) != cudaSuccess) st = EPIC_ERR_CUDA;
  if (st) {
    std::string e = g_err;
    epic_destroy(s);
    return fail(st, "epic_create: %s", e.c_str());
  }
  *out = s;
  return EPIC_OK;
}

void epic_destroy(epic_sim* s) {
  if (!s) return;
  if (s->ref_rng) ref_stream_destroy(static_cast<RefStream*>(s->ref_rng));
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->xfer_out) {
    cudaStreamSynchronize(s->xfer_out);
    cudaStreamSynchronize(s->xfer_in);
    cudaStreamDestroy(s->xfer_out);
    cudaStreamDestroy(s->xfer_in);
  }
  for (cudaEvent_t e : s->xfer_ev) cudaEventDestroy(e);
  if (s->h_counts) cudaFreeHost(s->h_counts);
  if (s->host_in) dfree(s, s->host_in);
  if (s->host_out) dfree(s, s->host_out);
  if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
  if (s->graph_exec_sort) cudaGraphExecDestroy(s->graph_exec_sort);
  if (s->sort_buf) dfree(s, s->sort_buf);
  for (auto& sp : s->sp) free_species(s, sp);
  void* spec[] = {s->spec.QR, s->spec.QC != s->spec.QR ? s->spec.QC : nullptr, s->spec.D, s->spec.t0, s->spec.t1,
                  s->spec.r64, s->spec.partials, s->spec.state, (void*)s->spec.fft.twR, (void*)s->spec.fft.twC,
                  s->ef32};
  for (void* p : spec) dfree(s, p);
  for (auto& pe : s->prof_pending) {
    cudaEventDestroy(pe.second.first);
    cudaEventDestroy(pe.second.second);
  }
  for (auto e : s->event_pool) cudaEventDestroy(e);
  if (s->side) {
    cudaStreamSynchronize(s->side);
    cudaStreamDestroy(s->side);
    cudaEventDestroy(s->ev_fork);
    cudaEventDestroy(s->ev_join);
  }
  dfree(s, s->mcc_ev.buf);
  dfree(s, s->mcc_ev.count);
  dfree(s, s->mcc_ev.slot);
  dfree(s, s->mcc_ev.tile_cnt);
  dfree(s, s->mcc_ev.tile_off);
  dfree(s, s->mcc_ev.cand);
  dfree(s, s->mcc_ev.cand_count);
  for (int k = 0; k < 8; k++) dfree(s, s->work[k]);
  void* ptrs[] = {s->phi, s->rho, s->efx, s->efy, s->ef, s->ef_cell, s->partials, s->bar,
                  s->d_info, s->d_iter_total, s->tile_ctr, s->d_ncoll, s->d_step, s->sum_partials, s->d_sums, s->d_flags,
                  s->tile_status, s->staging, s->d_uniforms, s->cs.tot, s->cs.ela, s->cs.exc, s->cs.ion,
                  s->cs.bin_cut, s->d_cond_rect, s->d_cond_circ, s->d_cond_nodes, s->d_cond_vals, s->d_cond_live,
                  s->d_inj, s->d_nold};
  for (void* p : ptrs)
    if (p) dfree(s, p);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

epic_status epic_add_species(epic_sim* s, const epic_species_desc* d, int* index) {
  if (!s || !d) return fail(EPIC_ERR_INVALID, "null argument");
  if (s->sp.size() >= 8) return fail(EPIC_ERR_INVALID, "at most 8 species");
  if (d->numparticle < 0 || !(d->mass > 0)) return fail(EPIC_ERR_INVALID, "bad species %s", d->name);
  epic_species_state sp;
  std::memset(&sp.soa, 0, sizeof(sp.soa));
  std::memset(&sp.mx, 0, sizeof(sp.mx));
  sp.d_n = nullptr;
  sp.den = nullptr;
  sp.acc = nullptr;
  sp.desc = *d;
  sp.desc.name[sizeof(sp.desc.name) - 1] = 0;
  sp.name = sp.desc.name;
  sp.cap = d->capacity > 0 ? d->capacity : (long long)d->numparticle + d->numparticle / 2 + 4096;
  // Fixed-point scale 2^k with k chosen so that cap * 2^k * (1 + 2^-20) < 2^63:
  // no node sum can overflow even if every particle lands on it.
  int bits = 0;
  while ((1LL << bits) < sp.cap + 1) bits++;
  int k = 62 - bits;
  if (k < 16) return fail(EPIC_ERR_INVALID, "capacity too large for the fixed-point deposit");
  sp.fx_scale = std::ldexp(1.0, k);
  sp.fx_inv_scale = std::ldexp(1.0, -k);
  epic_status st = EPIC_OK;
  auto guard = [&](epic_status x) {
    if (x && !st) st = x;
  };
  const size_t cap = (size_t)sp.cap, nn = (size_t)nnodes(s);
  if (s->mixed) {
    // 2^40 per particle in the integer CIC weights: overflow needs > 2^23
    // particles in one node's four cells.
    guard(dalloc(s, &sp.mx.cell, cap));
    guard(dalloc(s, &sp.mx.ox, cap));
    guard(dalloc(s, &sp.mx.oy, cap));
    guard(dalloc(s, &sp.mx.vx, cap));
    guard(dalloc(s, &sp.mx.vy, cap));
    guard(dalloc(s, &sp.mx.vz, cap));
  } else {
    guard(dalloc(s, &sp.soa.x, cap));
    guard(dalloc(s, &sp.soa.y, cap));
    guard(dalloc(s, &sp.soa.vx, cap));
    guard(dalloc(s, &sp.soa.vy, cap));
    guard(dalloc(s, &sp.soa.vz, cap));
  }
  guard(dalloc(s, &sp.d_n, 1));
  guard(dalloc(s, &sp.den, nn));
  guard(dalloc(s, &sp.acc, nn));
  guard(ensure_tile_status(s, sp.cap));
  if (st) {
    free_species(s, sp);
    return st;
  }
  s->sp.push_back(sp);
  if (index) *index = (int)s->sp.size() - 1;
  // A captured step no longer covers every species.
  if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
  if (s->graph_exec_sort) cudaGraphExecDestroy(s->graph_exec_sort);
  s->graph_exec = s->graph_exec_sort = nullptr;
  return EPIC_OK;
}

epic_status epic_set_particles(epic_sim* s, int i, const double* parts, int64_t n) {
  if (!valid_species(s, i) || n < 0 || (n > 0 && !parts)) return fail(EPIC_ERR_INVALID, "bad argument");
  epic_species_state& sp = s->sp[i];
  sp.acc_valid = false;
  if (n > sp.cap) return fail(EPIC_ERR_CAPACITY, "%lld particles exceed the capacity %lld of %s", (long long)n,
                              sp.cap, sp.name.c_str());
  epic_status st = ensure_staging(s, std::max<size_t>(1, (size_t)n * 5 * sizeof(double)));
  if (st) return st;
  if (n) {
    CK(cudaMemcpyAsync(s->staging, parts, (size_t)n * 5 * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    if (s->mixed)
      launch_aos_to_mixed(s->stream, s->g, (const double*)s->staging, sp.mx, n, s->d_flags, s->part_grid);
    else
      k_aos_to_soa<<<s->part_grid, 256, 0, s->stream>>>((const double*)s->staging, sp.soa, n);
    s->launches += 1;
    CKL();
  }
  long long nn = n;
  CK(cudaMemcpyAsync(sp.d_n, &nn, sizeof(long long), cudaMemcpyHostToDevice, s->stream));
  return sync(s);
}

epic_status epic_num_particles(epic_sim* s, int i, int64_t* n) {
  if (!valid_species(s, i) || !n) return fail(EPIC_ERR_INVALID, "bad argument");
  long long v = 0;
  CK(cudaMemcpyAsync(&v, s->sp[i].d_n, sizeof(long long), cudaMemcpyDeviceToHost, s->stream));
  epic_status st = sync(s);
  *n = v;
  return st;
}

epic_status epic_get_particles(epic_sim* s, int i, double* parts, int64_t capacity, int64_t* n) {
  if (!valid_species(s, i) || !n) return fail(EPIC_ERR_INVALID, "bad argument");
  int64_t cnt = 0;
  epic_status st = epic_num_particles(s, i, &cnt);
  if (st) return st;
  *n = cnt;
  if (cnt > capacity) return fail(EPIC_ERR_CAPACITY, "output buffer holds %lld of %lld particles",
                                  (long long)capacity, (long long)cnt);
  if (!cnt) return EPIC_OK;
  if ((st = ensure_staging(s, (size_t)cnt * 5 * sizeof(double)))) return st;
  if (s->mixed) launch_mixed_to_aos(s->stream, s->g, (double*)s->staging, s->sp[i].mx, s->sp[i].d_n, s->part_grid);
  else k_soa_to_aos<<<s->part_grid, 256, 0, s->stream>>>((double*)s->staging, s->sp[i].soa, s->sp[i].d_n);
  s->launches += 1;
  CKL();
  CK(cudaMemcpyAsync(parts, s->staging, (size_t)cnt * 5 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  return sync(s);
}

epic_status epic_load_particles(epic_sim* s, uint32_t seed) {
  if (!s) return fail(EPIC_ERR_INVALID, "null handle");
  if (s->ref_rng) ref_stream_destroy(static_cast<RefStream*>(s->ref_rng));
  s->ref_rng = ref_stream_create(seed);
  for (size_t i = 0; i < s->sp.size(); i++) {
    epic_status e = epic_init_species(s, (int)i);
    if (e) return e;
  }
  return EPIC_OK;
}

epic_status epic_init_species(epic_sim* s, int i) {
  if (!valid_species(s, i)) return fail(EPIC_ERR_INVALID, "bad species index");
  if (!s->ref_rng) s->ref_rng = ref_stream_create(0);
  std::vector<double> parts;
  std::string err;
  int st = load_species(s->cfg, s->sp[i].desc, parts, static_cast<RefStream*>(s->ref_rng), err, s->conductors);
  if (st) return fail((epic_status)st, "%s", err.c_str());
  return epic_set_particles(s, i, parts.data(), (int64_t)(parts.size() / 5));
}

epic_status epic_scatter_species(epic_sim* s, int i) {
  if (!valid_species(s, i)) return fail(EPIC_ERR_INVALID, "bad species index");
  epic_status st = do_deposit(s, i);
  if (st) return st;
  if ((st = do_finalize(s, FINALIZE_ONLY, i))) return st;
  return sync(s);
}

epic_status epic_compute_rho(epic_sim* s) {
  if (!s) return fail(EPIC_ERR_INVALID, "null handle");
  epic_status st = do_finalize(s, RHO_FROM_DEN, -1);
  if (st) return st;
  return sync(s);
}

epic_status epic_potential_solver(epic_sim* s, int* iterations, double* error) {
  if (!s) return fail(EPIC_ERR_INVALID, "null handle");
  epic_status st = do_solve(s);
  if (st) return st;
  if ((st = sync(s))) return st;
  SolveInfo info;
  CK(cudaMemcpyAsync(&info, s->d_info, sizeof(info), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (iterations) *iterations = info.iterations;
  if (error) *error = info.error;
  if (!info.converged)
    return fail(EPIC_WARN_NOT_CONVERGED, "solver did not reach the tolerance in %d iterations (error %g)",
                info.iterations, info.error);
  return EPIC_OK;
}

epic_status epic_calculate_efield(epic_sim* s) {
  if (!s) return fail(EPIC_ERR_INVALID, "null handle");
  epic_status st = do_efield(s);
  if (st) return st;
  return sync(s);
}

epic_status epic_push_species(epic_sim* s, int i, int sub_cycle) {
  if (!valid_species(s, i)) return fail(EPIC_ERR_INVALID, "bad species index");
  epic_status st = do_push(s, i, sub_cycle);
  if (st) return st;
  return sync(s);
}

static epic_status do_rewind(epic_sim* s, int i) {
  epic_species_state& sp = s->sp[i];
  const epic_config& c = s->cfg;
  double qm = sp.desc.charge / sp.desc.mass;
  double K = (c.density * QE * c.L) / (EPS_0 * c.W * c.vel_norm);
  double hqmK = 0.5 * qm * K;
  if (s->mixed)
    launch_rewind_mixed(s->stream, s->g, c.shape, sp.mx, sp.d_n, s->ef32, (float)(hqmK * c.DT), s->d_flags,
                        s->part_grid);
  else
    launch_rewind(s->stream, s->g, c.shape, sp.soa, sp.d_n, s->ef, hqmK, c.DT, s->d_flags, s->part_grid);
  s->launches += 1;
  CKL();
  return EPIC_OK;
}

epic_status epic_rewind_species(epic_sim* s, int i) {
  if (!valid_species(s, i)) return fail(EPIC_ERR_INVALID, "bad species index");
  epic_status st = do_rewind(s, i);
  if (st) return st;
  return sync(s);
}

epic_status epic_sort_species(epic_sim* s, int i) {
  if (!valid_species(s, i)) return fail(EPIC_ERR_INVALID, "bad species index");
  epic_status st = do_sort(s, i);
  if (st) return st;
  return sync(s);
}

static epic_status upload_tables(epic_sim* s, const double* tot, const double* ela, const double* exc,
                                 const double* ion, int64_t n) {
  // A captured step holds the old tables.
  if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
  if (s->graph_exec_sort) cudaGraphExecDestroy(s->graph_exec_sort);
  s->graph_exec = s->graph_exec_sort = nullptr;
  double** dst[4] = {&s->cs.tot, &s->cs.ela, &s->cs.exc, &s->cs.ion};
  const double* src[4] = {tot, ela, exc, ion};
  for (int k = 0; k < 4; k++) {
    if (*dst[k]) dfree(s, *dst[k]);
    *dst[k] = nullptr;
    CK(cudaMallocAsync((void**)dst[k], (size_t)n * sizeof(double), s->stream));
    CK(cudaMemcpyAsync(*dst[k], src[k], (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  }
  s->cs.n = n;
  return EPIC_OK;
}

// The speed-bin cuts of the MCC early-out for this run's vel_norm and dt.
static epic_status upload_bin_cuts(epic_sim* s, const double* tot) {
  std::vector<unsigned long long> cuts(MCC_SPEED_BINS);
  mcc_bin_cuts(s->cs, tot, s->cfg.vel_norm, s->cfg.DT / s->cfg.W, cuts.data());
  if (!s->cs.bin_cut)
    CK(cudaMallocAsync((void**)&s->cs.bin_cut, MCC_SPEED_BINS * sizeof(unsigned long long), s->stream));
  CK(cudaMemcpyAsync(s->cs.bin_cut, cuts.data(), MCC_SPEED_BINS * sizeof(unsigned long long),
                     cudaMemcpyHostToDevice, s->stream));
  return sync(s);  // the host vector goes out of scope
}

epic_status epic_set_cross_sections(epic_sim* s, const double* tot, const double* ela, const double* exc,
                                    const double* ion, int64_t n, double de) {
  if (!s || !tot || !ela || !exc || !ion || n < 2 || !(de > 0)) return fail(EPIC_ERR_INVALID, "bad argument");
  epic_status st = upload_tables(s, tot, ela, exc, ion, n);
  if (st) return st;
  s->cs.kind = 0;
  s->cs.de = de;
  // Null-collision bound: nu = tot[idx] * |v| with |v| below v(E_idx + de/2).
  double mx = 0;
  for (int64_t i = 0; i < n; i++) {
    double e = (i + 0.5) * de;
    if (i == n - 1) e = 4 * n * de;  // energies past the table reuse the last entry
    double v = sqrt(2.0 * e * EV / ME);
    mx = std::max(mx, tot[i] * v);
  }
  s->cs.nu_max = mx;
  return upload_bin_cuts(s, tot);
}

epic_status epic_set_reference_cross_sections(epic_sim* s) {
  if (!s) return fail(EPIC_ERR_INVALID, "null handle");
  std::vector<double> tot, ela, exc, ion;
  reference_tables(s->cfg, tot, ela, exc, ion);
  return epic_set_cross_sections(s, tot.data(), ela.data(), exc.data(), ion.data(), (int64_t)tot.size(), DE_CS);
}

epic_status epic_set_log_cross_sections(epic_sim* s, const double* ela, const double* exc, const double* ion,
                                        int64_t n, double e_min, double e_max) {
  if (!s || !ela || !exc || !ion || n < 2 || !(e_min > 0) || !(e_max > e_min))
    return fail(EPIC_ERR_INVALID, "bad argument");
  std::vector<double> tot(n);
  for (int64_t i = 0; i < n; i++) tot[i] = (ela[i] + exc[i] + ion[i]) * s->cfg.gas_density;
  epic_status st = upload_tables(s, tot.data(), ela, exc, ion, n);
  if (st) return st;
  s->cs.kind = 1;
  s->cs.e_min = e_min;
  s->cs.e_max = e_max;
  s->cs.log_emin = log(e_min);
  s->cs.inv_dlog = (n - 1) / (log(e_max) - log(e_min));
  double mx = 0;
  for (int64_t i = 0; i + 1 < n; i++) {
    double e1 = exp(log(e_min) + (i + 1) / s->cs.inv_dlog);
    mx = std::max(mx, std::max(tot[i], tot[i + 1]) * sqrt(2.0 * e1 * EV / ME));
  }
  mx = std::max(mx, tot[n - 1] * sqrt(2.0 * 4 * e_max * EV / ME));
  s->cs.nu_max = mx;
  return upload_bin_cuts(s, tot.data());
}

epic_status epic_handle_collisions(epic_sim* s, int e, int ion, const double* uniforms, int ustride,
                                   int64_t* collisions) {
  if (!valid_species(s, e) || !valid_species(s, ion) || e == ion) return fail(EPIC_ERR_INVALID, "bad species");
  s->sp[e].acc_valid = s->sp[ion].acc_valid = false;  // products are appended
  const double* d_u = nullptr;
  if (s->cfg.mcc_mode == EPIC_MCC_INJECTED) {
    if (!uniforms || ustride < 14) return fail(EPIC_ERR_INVALID, "injected mode needs uniforms with stride >= 14");
    int64_t ne = 0;
    epic_status st = epic_num_particles(s, e, &ne);
    if (st) return st;
    size_t len = (size_t)std::max<int64_t>(ne, 1) * ustride;
    if ((long long)len > s->uniforms_len) {
      if (s->d_uniforms) dfree(s, s->d_uniforms);
      s->d_uniforms = nullptr;
      CK(cudaMallocAsync(&s->d_uniforms, len * sizeof(double), s->stream));
      s->uniforms_len = (long long)len;
    }
    CK(cudaMemcpyAsync(s->d_uniforms, uniforms, (size_t)ne * ustride * sizeof(double), cudaMemcpyHostToDevice,
                       s->stream));
    d_u = s->d_uniforms;
  }
  epic_status st = do_mcc(s, e, ion, d_u, ustride);
  if (st) return st;
  if ((st = sync(s))) return st;
  unsigned long long nc = 0;
  CK(cudaMemcpyAsync(&nc, s->d_ncoll, sizeof(nc), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  if (collisions) *collisions = (int64_t)nc;
  return EPIC_OK;
}

epic_status epic_step(epic_sim* s, int with_collisions) {
  if (!s) return fail(EPIC_ERR_INVALID, "null handle");
  epic_status st = do_step(s, with_collisions);
  if (st) return st;
  return sync(s);
}

// One loop iteration for particles the caller holds in host memory.  Direct
// path (FP64 form, fixed-point deposit, periodic or reflective walls, no cell
// sort due, every buffer pinned): the upload kernels read the records over the
// host link and deposit on the way, the push writes the new records back as it
// goes, and the electrons (and the ions appended by ionisation) go back after
// the MCC; otherwise the same work runs through the staging buffer.
epic_status epic_step_host(epic_sim* s, int with_collisions, double* const* parts, int64_t* n,
                           const int64_t* capacity) {
  if (!s || !parts || !n || !capacity) return fail(EPIC_ERR_INVALID, "bad argument");
  invalidate_acc(s);  // the particles come from the caller and leave moved
  const int nsp = (int)s->sp.size();
  for (int k = 0; k < nsp; k++) {
    if (n[k] < 0 || n[k] > capacity[k] || (n[k] > 0 && !parts[k]))
      return fail(EPIC_ERR_INVALID, "bad particle buffer for species %d", k);
    if (n[k] > s->sp[k].cap)
      return fail(EPIC_ERR_CAPACITY, "%lld particles exceed the capacity %lld of %s", (long long)n[k], s->sp[k].cap,
                  s->sp[k].name.c_str());
  }
  const epic_config& c = s->cfg;
  bool direct = !s->mixed && c.bc != EPIC_OPEN && c.deposit_mode == EPIC_DEPOSIT_FIXED && s->conductors.empty() &&
                s->emitters.empty() &&
                !(c.sort_every > 0 && s->step_index % c.sort_every == 0);
  for (int k = 0; k < nsp && direct; k++) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, parts[k]) != cudaSuccess || at.type != cudaMemoryTypeHost) {
      cudaGetLastError();
      direct = false;
    }
  }
  epic_status st;
  if (!direct) {
    for (int k = 0; k < nsp; k++)
      if ((st = epic_set_particles(s, k, parts[k], n[k]))) return st;
    if ((st = epic_step(s, with_collisions))) return st;
    for (int k = 0; k < nsp; k++) {
      int64_t got = 0;
      if ((st = epic_get_particles(s, k, parts[k], capacity[k], &got))) return st;
      n[k] = got;
    }
    return EPIC_OK;
  }
  s->step_index++;
  for (int k = 0; k < nsp; k++) {
    epic_species_state& sp = s->sp[k];
    CK(cudaMemsetAsync(sp.acc, 0, nnodes(s) * sizeof(unsigned long long), s->stream));
    launch_upload_deposit(s->stream, s->g, c.shape, parts[k], n[k], sp.soa, sp.d_n, sp.acc, sp.fx_scale, s->d_flags,
                          s->part_grid);
    s->launches += 1;
  }
  CKL();
  if ((st = do_finalize(s, FINALIZE_AND_RHO, -1))) return st;
  if ((st = do_solve(s))) return st;
  if ((st = do_efield(s))) return st;
  const bool coll = with_collisions && nsp >= 2;
  const double K = (c.density * QE * c.L) / (EPS_0 * c.W * c.vel_norm);
  const double cc = (c.vel_norm) / (c.L * c.W);
  const bool push_e = coll && !(c.ionfixed == 1 && s->sp[0].name == "ion");
  if (push_e) {
    // The MCC changes the electrons after the push, so they go back after it;
    // their push runs on a side stream while the other species stream out.
    if (!s->side) {
      CK(cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking));
      CK(cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming));
    }
    epic_species_state& e = s->sp[0];
    CK(cudaEventRecord(s->ev_fork, s->stream));
    CK(cudaStreamWaitEvent(s->side, s->ev_fork, 0));
    launch_push(s->side, s->g, c.shape, c.bc, e.soa, e.d_n, s->ef, s->ef_cell, (e.desc.charge / e.desc.mass) * K, cc,
                c.DT, s->d_flags, s->tile_status, s->tile_ctr, s->part_grid, c.push_order == EPIC_PUSH_CONTRACTED);
    CK(cudaEventRecord(s->ev_join, s->side));
    s->launches += 1;
  }
  for (int k = coll ? 1 : 0; k < nsp; k++) {
    if (c.ionfixed == 1 && s->sp[k].name == "ion") continue;
    epic_species_state& sp = s->sp[k];
    launch_push_download(s->stream, s->g, c.shape, c.bc, sp.soa, sp.d_n, s->ef, s->ef_cell,
                         (sp.desc.charge / sp.desc.mass) * K, cc, c.DT, parts[k], s->d_flags, s->part_grid, c.push_order == EPIC_PUSH_CONTRACTED);
    s->launches += 1;
  }
  CKL();
  if (coll) {
    if (push_e) CK(cudaStreamWaitEvent(s->stream, s->ev_join, 0));
    if ((st = do_mcc(s, 0, 1, nullptr, 0))) return st;
    launch_download(s->stream, s->sp[0].soa, s->sp[0].d_n, 0, capacity[0], parts[0], s->d_flags, s->part_grid);
    launch_download(s->stream, s->sp[1].soa, s->sp[1].d_n, n[1], capacity[1], parts[1], s->d_flags, s->part_grid);
    s->launches += 2;
    CKL();
  }
  std::vector<long long> cnt(nsp);
  for (int k = 0; k < nsp; k++)
    CK(cudaMemcpyAsync(&cnt[k], s->sp[k].d_n, sizeof(long long), cudaMemcpyDeviceToHost, s->stream));
  if ((st = sync(s))) return st;
  for (int k = 0; k < nsp; k++) n[k] = cnt[k];
  return EPIC_OK;
}

// Several loop iterations for particles the caller holds in host memory,
// with every step's records going to the host and back: after each step the
// stepped records are copied device-to-host into the caller's buffers, and
// the next step's push takes its input records copied host-to-device from
// those buffers.  The copies run on two copy-engine streams, chunk by chunk
// (the host-to-device copy of a chunk follows its device-to-host copy, so the
// two directions of the link work at once), while the SMs run the next
// step's deposit, Poisson solve and E-field, which need no particle records
// (the push deposited the new positions as it moved them).
constexpr size_t RUN_HOST_CHUNK_BYTES = 32u << 20;

static epic_status run_host_streams(epic_sim* s, size_t doubles, int nevents) {
  if (!s->xfer_out) {
    CK(cudaStreamCreateWithFlags(&s->xfer_out, cudaStreamNonBlocking));
    CK(cudaStreamCreateWithFlags(&s->xfer_in, cudaStreamNonBlocking));
  }
  while ((int)s->xfer_ev.size() < nevents) {
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    s->xfer_ev.push_back(e);
  }
  if (!s->h_counts) CK(cudaMallocHost((void**)&s->h_counts, 8 * sizeof(long long)));
  if (doubles > s->host_stage_doubles) {
    if (s->host_in) dfree(s, s->host_in);
    if (s->host_out) dfree(s, s->host_out);
    s->host_in = s->host_out = nullptr;
    s->host_stage_doubles = 0;
    CK(cudaMallocAsync((void**)&s->host_in, doubles * sizeof(double), s->stream));
    CK(cudaMallocAsync((void**)&s->host_out, doubles * sizeof(double), s->stream));
    s->host_stage_doubles = doubles;
  }
  return EPIC_OK;
}

epic_status epic_run_host(epic_sim* s, int steps, int with_collisions, double* const* parts, int64_t* n,
                          const int64_t* capacity) {
  if (!s || !parts || !n || !capacity || steps < 0) return fail(EPIC_ERR_INVALID, "bad argument");
  const int nsp = (int)s->sp.size();
  for (int k = 0; k < nsp; k++) {
    if (n[k] < 0 || n[k] > capacity[k] || (n[k] > 0 && !parts[k]))
      return fail(EPIC_ERR_INVALID, "bad particle buffer for species %d", k);
    if (n[k] > s->sp[k].cap)
      return fail(EPIC_ERR_CAPACITY, "%lld particles exceed the capacity %lld of %s", (long long)n[k], s->sp[k].cap,
                  s->sp[k].name.c_str());
  }
  if (steps == 0) return EPIC_OK;
  const epic_config& c = s->cfg;
  bool direct = !s->mixed && fused_deposit(s) && c.sort_every == 0 && nsp <= 8;
  for (int k = 0; k < nsp && direct; k++) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, parts[k]) != cudaSuccess || at.type != cudaMemoryTypeHost) {
      cudaGetLastError();
      direct = false;
    }
  }
  epic_status st;
  if (!direct) {  // the same round trips, step by step
    for (int t = 0; t < steps; t++)
      if ((st = epic_step_host(s, with_collisions, parts, n, capacity))) return st;
    return EPIC_OK;
  }
  std::vector<size_t> off(nsp + 1, 0);
  for (int k = 0; k < nsp; k++) off[k + 1] = off[k] + (size_t)s->sp[k].cap * 5;
  const int max_chunks = 256;
  if ((st = run_host_streams(s, off[nsp], max_chunks + 2))) return st;
  cudaEvent_t ev_out_ready = s->xfer_ev[0], ev_in_done = s->xfer_ev[1];
  std::vector<long long> cnt(n, n + nsp);
  // Chunks of the records of every species: (species, first record, records).
  auto chunks = [&](std::vector<std::array<long long, 3>>& out) {
    out.clear();
    long long total = 0;
    for (int k = 0; k < nsp; k++) total += cnt[k];
    const long long per = std::max<long long>(
        std::max<long long>(1, (long long)(RUN_HOST_CHUNK_BYTES / 40)), (total + max_chunks - nsp - 1) / (max_chunks - nsp));
    for (int k = 0; k < nsp; k++)
      for (long long a = 0; a < cnt[k]; a += per) out.push_back({k, a, std::min(per, cnt[k] - a)});
  };
  auto soa_from_stage = [&]() -> epic_status {
    for (int k = 0; k < nsp; k++) {
      if (cnt[k] > 0)
        k_aos_to_soa<<<s->part_grid, 256, 0, s->stream>>>(s->host_in + off[k], s->sp[k].soa, cnt[k]);
      launch_set_count(s->stream, s->sp[k].d_n, cnt[k]);
      s->launches += 2;
    }
    CKL();
    return EPIC_OK;
  };
  // Inputs of the first step.
  invalidate_acc(s);
  for (int k = 0; k < nsp; k++)
    if (cnt[k] > 0)
      CK(cudaMemcpyAsync(s->host_in + off[k], parts[k], (size_t)cnt[k] * 40, cudaMemcpyHostToDevice, s->stream));
  if ((st = soa_from_stage())) return st;
  if ((st = do_step_field(s))) return st;
  std::vector<std::array<long long, 3>> ch;
  for (int t = 0; t < steps; t++) {
    if (t > 0) {  // this step's input records, back from the host
      CK(cudaStreamWaitEvent(s->stream, ev_in_done, 0));
      if ((st = soa_from_stage())) return st;
    }
    if ((st = do_step_move(s, with_collisions))) return st;
    for (int k = 0; k < nsp; k++) {
      k_soa_to_aos<<<s->part_grid, 256, 0, s->stream>>>(s->host_out + off[k], s->sp[k].soa, s->sp[k].d_n);
      CK(cudaMemcpyAsync(s->h_counts + k, s->sp[k].d_n, sizeof(long long), cudaMemcpyDeviceToHost, s->stream));
      s->launches += 1;
    }
    CKL();
    CK(cudaEventRecord(ev_out_ready, s->stream));
    if (t + 1 < steps && (st = do_step_field(s))) return st;  // the SMs go on while the records travel
    CK(cudaEventSynchronize(ev_out_ready));
    bool over = false;
    for (int k = 0; k < nsp; k++) {
      cnt[k] = s->h_counts[k];
      over |= cnt[k] > capacity[k];
    }
    if (over) {
      cudaStreamSynchronize(s->stream);
      return fail(EPIC_ERR_CAPACITY, "a species outgrew the caller's buffer");
    }
    chunks(ch);
    CK(cudaStreamWaitEvent(s->xfer_out, ev_out_ready, 0));
    for (size_t q = 0; q < ch.size(); q++) {
      const int k = (int)ch[q][0];
      const size_t a = (size_t)ch[q][1] * 5, b = (size_t)ch[q][2] * 40;
      CK(cudaMemcpyAsync(parts[k] + a, s->host_out + off[k] + a, b, cudaMemcpyDeviceToHost, s->xfer_out));
      if (t + 1 < steps) {
        CK(cudaEventRecord(s->xfer_ev[2 + q], s->xfer_out));
        CK(cudaStreamWaitEvent(s->xfer_in, s->xfer_ev[2 + q], 0));
        CK(cudaMemcpyAsync(s->host_in + off[k] + a, parts[k] + a, b, cudaMemcpyHostToDevice, s->xfer_in));
      }
    }
    if (t + 1 < steps) CK(cudaEventRecord(ev_in_done, s->xfer_in));
  }
  CK(cudaStreamSynchronize(s->xfer_out));
  for (int k = 0; k < nsp; k++) n[k] = cnt[k];
  return sync(s);
}

static epic_status do_initial_field(epic_sim* s) {
  epic_status st;
  for (int i = 0; i < (int)s->sp.size(); i++)
    if ((st = do_deposit(s, i))) return st;
  if ((st = do_finalize(s, FINALIZE_AND_RHO, -1))) return st;
  if ((st = do_solve(s))) return st;
  if ((st = do_efield(s))) return st;
  for (int i = 0; i < (int)s->sp.size(); i++)
    if ((st = do_rewind(s, i))) return st;
  return EPIC_OK;
}

epic_status epic_initial_field(epic_sim* s) {
  if (!s) return fail(EPIC_ERR_INVALID, "null handle");
  epic_status st = do_initial_field(s);
  if (st) return st;
  return sync(s);
}

epic_status epic_initial_field_async(epic_sim* s) {
  if (!s) return fail(EPIC_ERR_INVALID, "null handle");
  return do_initial_field(s);
}

// Enqueues `steps` steps on the handle's stream without waiting.
static epic_status enqueue_run(epic_sim* s, int steps, int with_collisions, int use_graph) {
  epic_status st;
  if (!use_graph) {
    for (int k = 0; k < steps; k++)
      if ((st = do_step(s, with_collisions))) return st;
    return EPIC_OK;
  }
  const bool sorting = s->cfg.sort_every > 0;
  // One step captured as a graph (all scratch allocated first: a capture
  // cannot allocate); with sorting on, a second graph for the sort steps.
  auto capture = [&](int sort, cudaGraphExec_t* exec, int64_t* nlaunch) -> epic_status {
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    const int64_t before = s->launches, step_before = s->step_index;
    s->steady_capture = fused_deposit(s);
    epic_status e = do_step(s, with_collisions, sort);
    s->steady_capture = false;
    cudaError_t ce = cudaStreamEndCapture(s->stream, &graph);
    s->step_index = step_before;
    if (e || ce != cudaSuccess) {
      cudaGetLastError();  // a failed capture leaves its error pending; do not leak it to later calls
      if (ce == cudaSuccess) cudaGraphDestroy(graph);
      s->launches = before;
      if (e) return e;
      return fail(EPIC_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
    }
    *nlaunch = s->launches - before;
    s->launches = before;
    ce = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return fail(EPIC_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
    return EPIC_OK;
  };
  // The captured step takes the accumulators as deposited (the previous step's
  // push left them so); deposit whatever another call has moved since.
  if (fused_deposit(s))
    for (int i = 0; i < (int)s->sp.size(); i++)
      if (!s->sp[i].acc_valid && (st = do_deposit(s, i))) return st;
  if (!s->graph_exec || s->graph_collisions != with_collisions || (sorting && !s->graph_exec_sort)) {
    if (s->graph_exec) cudaGraphExecDestroy(s->graph_exec);
    if (s->graph_exec_sort) cudaGraphExecDestroy(s->graph_exec_sort);
    s->graph_exec = s->graph_exec_sort = nullptr;
    if (with_collisions && s->sp.size() >= 2)
      if ((st = ensure_mcc_events(s, s->sp[0].cap))) return st;
    if (sorting && (st = ensure_sort_scratch(s))) return st;
    if ((st = capture(0, &s->graph_exec, &s->graph_launches))) return st;
    if (sorting && (st = capture(1, &s->graph_exec_sort, &s->graph_launches_sort))) return st;
    s->graph_collisions = with_collisions;
  }
  for (int k = 0; k < steps; k++) {
    const bool srt = sorting && s->step_index % s->cfg.sort_every == 0;
    s->step_index++;
    CK(cudaGraphLaunch(srt ? s->graph_exec_sort : s->graph_exec, s->stream));
    s->launches += srt ? s->graph_launches_sort : s->graph_launches;
  }
  return EPIC_OK;
}

epic_status epic_run(epic_sim* s, int steps, int with_collisions, int use_graph) {
  if (!s || steps < 0) return fail(EPIC_ERR_INVALID, "bad argument");
  epic_status st = enqueue_run(s, steps, with_collisions, use_graph);
  if (st) return st;
  return sync(s);
}

epic_status epic_run_async(epic_sim* s, int steps, int with_collisions) {
  if (!s || steps < 0) return fail(EPIC_ERR_INVALID, "bad argument");
  return enqueue_run(s, steps, with_collisions, 1);
}

epic_status epic_poll(epic_sim* s, int* done) {
  if (!s || !done) return fail(EPIC_ERR_INVALID, "bad argument");
  cudaError_t e = cudaStreamQuery(s->stream);
  if (e == cudaErrorNotReady) {
    *done = 0;
    return EPIC_OK;
  }
  *done = 1;
  if (e != cudaSuccess) return fail(EPIC_ERR_CUDA, "stream: %s", cudaGetErrorString(e));
  return take_flags(s);
}

epic_status epic_load_particles_device(epic_sim* s, uint64_t seed) {
  if (!s) return fail(EPIC_ERR_INVALID, "null handle");
  invalidate_acc(s);
  for (int i = 0; i < (int)s->sp.size(); i++) {
    epic_species_state& sp = s->sp[i];
    const long long n = sp.desc.numparticle;
    if (n > sp.cap) return fail(EPIC_ERR_CAPACITY, "%lld particles exceed the capacity %lld of %s", n, sp.cap,
                                sp.name.c_str());
    int kind = 0, narg = 0;
    std::string err;
    if (parse_load_type(sp.desc.load, &kind, &narg, err)) return fail(EPIC_ERR_INVALID, "%s", err.c_str());
    epic_status st = ensure_staging(s, std::max<size_t>(1, (size_t)n * 5 * sizeof(double)));
    if (st) return st;
    launch_load(s->stream, s->g, sp.desc, s->cfg, i, kind, narg, (double*)s->staging, seed, s->part_grid,
                (const double4*)s->d_cond_rect, s->cond_nrect, s->d_flags);
    if (n) {
      if (s->mixed)
        launch_aos_to_mixed(s->stream, s->g, (const double*)s->staging, sp.mx, n, s->d_flags, s->part_grid);
      else
        k_aos_to_soa<<<s->part_grid, 256, 0, s->stream>>>((const double*)s->staging, sp.soa, n);
    }
    launch_set_count(s->stream, sp.d_n, n);
    s->launches += n ? 3 : 1;
    CKL();
  }
  return EPIC_OK;
}

epic_status epic_digest(epic_sim* s, uint64_t out[2]) {
  if (!s || !out) return fail(EPIC_ERR_INVALID, "bad argument");
  unsigned long long* d = reinterpret_cast<unsigned long long*>(s->d_sums);  // 4 doubles of scratch
  CK(cudaMemsetAsync(d, 0, 2 * sizeof(unsigned long long), s->stream));
  launch_digest(s->stream, s->phi, 8, nullptr, nnodes(s), 1, d, s->part_grid);
  for (int i = 0; i < (int)s->sp.size(); i++) {
    epic_species_state& sp = s->sp[i];
    const unsigned long long tag = 16ull * (i + 1);
    launch_digest(s->stream, sp.d_n, 8, nullptr, 1, tag, d + 1, 1);
    if (s->mixed) {
      const void* a[6] = {sp.mx.cell, sp.mx.ox, sp.mx.oy, sp.mx.vx, sp.mx.vy, sp.mx.vz};
      for (int k = 0; k < 6; k++) launch_digest(s->stream, a[k], 4, sp.d_n, 0, tag + 1 + k, d + 1, s->part_grid);
    } else {
      const void* a[5] = {sp.soa.x, sp.soa.y, sp.soa.vx, sp.soa.vy, sp.soa.vz};
      for (int k = 0; k < 5; k++) launch_digest(s->stream, a[k], 8, sp.d_n, 0, tag + 1 + k, d + 1, s->part_grid);
    }
  }
  CKL();
  unsigned long long h[2];
  CK(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
  epic_status st = sync(s);
  if (st) return st;
  out[0] = h[0];
  out[1] = h[1];
  return EPIC_OK;
}

epic_status epic_compute_ke(epic_sim* s, int i, int norm, double out[3]) {
  if (!valid_species(s, i) || !valid_species(s, norm) || !out) return fail(EPIC_ERR_INVALID, "bad argument");
  epic_species_state& sp = s->sp[i];
  if (s->mixed)
    launch_particle_sums_mixed(s->stream, 0, sp.mx, sp.d_n, s->cfg.vel_norm, s->sum_partials, s->d_sums,
                               s->part_grid);
  else
    launch_particle_sums(s->stream, 0, sp.soa, sp.d_n, s->cfg.vel_norm, s->sum_partials, s->d_sums, s->part_grid);
  s->launches += 2;
  CKL();
  double k[3];
  CK(cudaMemcpyAsync(k, s->d_sums, 3 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  epic_status st = sync(s);
  if (st) return st;
  const epic_species_desc& n = s->sp[norm].desc;
  double Th = (n.temp * EV) * (n.spwt) * n.numparticle;
  for (int c = 0; c < 3; c++) {
    k[c] *= 0.5 * (sp.desc.spwt * sp.desc.mass);
    out[c] = k[c] / Th;
  }
  return EPIC_OK;
}

epic_status epic_compute_momentum(epic_sim* s, int i, int norm, double out[3]) {
  if (!valid_species(s, i) || !valid_species(s, norm) || !out) return fail(EPIC_ERR_INVALID, "bad argument");
  epic_species_state& sp = s->sp[i];
  if (s->mixed)
    launch_particle_sums_mixed(s->stream, 1, sp.mx, sp.d_n, s->cfg.vel_norm, s->sum_partials, s->d_sums,
                               s->part_grid);
  else
    launch_particle_sums(s->stream, 1, sp.soa, sp.d_n, s->cfg.vel_norm, s->sum_partials, s->d_sums, s->part_grid);
  s->launches += 2;
  CKL();
  double p[3];
  CK(cudaMemcpyAsync(p, s->d_sums, 3 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  epic_status st = sync(s);
  if (st) return st;
  const epic_species_desc& n = s->sp[norm].desc;
  double Thp = sqrt(n.temp * EV / ME) * n.spwt * n.numparticle * ME;
  for (int c = 0; c < 3; c++) {
    p[c] *= (sp.desc.spwt * sp.desc.mass);
    out[c] = p[c] / Thp;
  }
  return EPIC_OK;
}

epic_status epic_compute_pe(epic_sim* s, int norm, double* pe) {
  if (!valid_species(s, norm) || !pe) return fail(EPIC_ERR_INVALID, "bad argument");
  launch_grid_sums(s->stream, 0, s->g, s->efx, s->efy, s->cfg.L, s->sum_partials, s->d_sums);
  s->launches += 2;
  CKL();
  double v = 0;
  CK(cudaMemcpyAsync(&v, s->d_sums, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  epic_status st = sync(s);
  if (st) return st;
  const epic_config& c = s->cfg;
  const epic_species_desc& n = s->sp[norm].desc;
  double unnorm = (c.density * QE * c.L) / EPS_0;
  double pe_norm = 0.5 * EPS_0 * v * unnorm * unnorm;
  double Th = (n.temp * EV) * n.spwt * n.numparticle;
  *pe = pe_norm / Th;
  return EPIC_OK;
}

epic_status epic_delta_phi(epic_sim* s, double* dphi) {
  if (!s || !dphi) return fail(EPIC_ERR_INVALID, "bad argument");
  launch_grid_sums(s->stream, 1, s->g, s->phi, s->phi, 0.0, s->sum_partials, s->d_sums);
  s->launches += 2;
  CKL();
  double v[2];
  CK(cudaMemcpyAsync(v, s->d_sums, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaMemcpyAsync(v + 1, s->phi, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  epic_status st = sync(s);
  if (st) return st;
  *dphi = v[0] - v[1];
  return EPIC_OK;
}

static double* grid_ptr(epic_sim* s, int which) {
  switch (which) {
    case EPIC_GRID_PHI: return s->phi;
    case EPIC_GRID_RHO: return s->rho;
    case EPIC_GRID_EFX: return s->efx;
    case EPIC_GRID_EFY: return s->efy;
    default:
      if (which >= EPIC_GRID_DEN0 && which - EPIC_GRID_DEN0 < (int)s->sp.size()) return s->sp[which - EPIC_GRID_DEN0].den;
      return nullptr;
  }
}

epic_status epic_get_grid(epic_sim* s, int which, double* out) {
  if (!s || !out) return fail(EPIC_ERR_INVALID, "bad argument");
  double* p = grid_ptr(s, which);
  if (!p) return fail(EPIC_ERR_INVALID, "unknown grid %d", which);
  CK(cudaMemcpyAsync(out, p, nnodes(s) * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  return sync(s);
}

epic_status epic_set_grid(epic_sim* s, int which, const double* in) {
  if (!s || !in) return fail(EPIC_ERR_INVALID, "bad argument");
  double* p = grid_ptr(s, which);
  if (!p) return fail(EPIC_ERR_INVALID, "unknown grid %d", which);
  CK(cudaMemcpyAsync(p, in, nnodes(s) * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  epic_status st = sync(s);
  if (st) return st;
  if (which == EPIC_GRID_EFX || which == EPIC_GRID_EFY) {
    // keep the interleaved gather copy in step with the component grids
    std::vector<double> ex(nnodes(s)), ey(nnodes(s));
    CK(cudaMemcpyAsync(ex.data(), s->efx, nnodes(s) * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(ey.data(), s->efy, nnodes(s) * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    std::vector<double2> e2(nnodes(s));
    for (long long k = 0; k < nnodes(s); k++) e2[k] = make_double2(ex[k], ey[k]);
    CK(cudaMemcpyAsync(s->ef, e2.data(), nnodes(s) * sizeof(double2), cudaMemcpyHostToDevice, s->stream));
    if (s->ef_cell) launch_cell_coef(s->stream, s->g, s->ef, s->ef_cell);
    if (s->ef32) {
      std::vector<float2> f2(nnodes(s));
      for (long long k = 0; k < nnodes(s); k++) f2[k] = make_float2((float)ex[k], (float)ey[k]);
      CK(cudaMemcpyAsync(s->ef32, f2.data(), nnodes(s) * sizeof(float2), cudaMemcpyHostToDevice, s->stream));
    }
    CK(cudaStreamSynchronize(s->stream));  // e2, f2 are host temporaries
  }
  return EPIC_OK;
}

epic_status epic_sync(epic_sim* s) {
  if (!s) return fail(EPIC_ERR_INVALID, "null handle");
  return sync(s);
}

int64_t epic_kernel_launches(epic_sim* s) { return s ? s->launches : 0; }

void* epic_stream(epic_sim* s) { return s ? (void*)s->stream : nullptr; }

epic_status epic_set_profiling(epic_sim* s, int enable) {
  if (!s) return fail(EPIC_ERR_INVALID, "null handle");
  s->profiling = enable ? 1 : 0;
  return EPIC_OK;
}

epic_status epic_get_profile(epic_sim* s, double ms[EPIC_NUM_PHASES], int64_t counts[EPIC_NUM_PHASES],
                             int64_t* solver_iterations) {
  if (!s) return fail(EPIC_ERR_INVALID, "null handle");
  CK(cudaStreamSynchronize(s->stream));
  for (auto& pe : s->prof_pending) {
    float t = 0;
    CK(cudaEventElapsedTime(&t, pe.second.first, pe.second.second));
    s->prof_ms[pe.first] += t;
    s->prof_count[pe.first] += 1;
    s->event_pool.push_back(pe.second.first);
    s->event_pool.push_back(pe.second.second);
  }
  s->prof_pending.clear();
  unsigned long long it = 0;
  CK(cudaMemcpyAsync(&it, s->d_iter_total, sizeof(it), cudaMemcpyDeviceToHost, s->stream));
  CK(cudaStreamSynchronize(s->stream));
  CK(cudaMemsetAsync(s->d_iter_total, 0, sizeof(it), s->stream));
  for (int k = 0; k < EPIC_NUM_PHASES; k++) {
    if (ms) ms[k] = s->prof_ms[k];
    if (counts) counts[k] = s->prof_count[k];
    s->prof_ms[k] = 0;
    s->prof_count[k] = 0;
  }
  if (solver_iterations) *solver_iterations = (int64_t)it;
  return EPIC_OK;
}

}  // extern "C"
