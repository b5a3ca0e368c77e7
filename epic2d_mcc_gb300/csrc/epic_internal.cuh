// Internal declarations shared by the kernel files and the C ABI.
//
// Device data layout (HBM, one simulation):
//   particles : per species, structure of arrays x, y, vx, vy, vz (FP64),
//               capacity `cap`, live count in device memory (`d_n`) so every
//               particle kernel is a fixed-size launch that reads its bound on
//               the device (graph-capturable, no host round trip per step).
//   grids     : nx*ny FP64 arrays, node (i, j) at i*ny + j (the reference's
//               Matrix<double>(nx, ny) order): phi, rho, efx, efy, one density
//               per species, plus `ef` = interleaved (efx, efy) double2 so a
//               gather costs one 16-byte load per node.
//   deposit   : int64 fixed-point accumulators per species (deterministic) or
//               FP64 atomics straight into the density grid.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/epic2d.h"

namespace epic {

// Constants of include/domain.h:204-215 and include/collision.h:14-15,
// include/cross_sections.h:14-15 (PI is the reference's truncated value).
constexpr double EPS_0 = 8.85418782e-12;
constexpr double QE = 1.602176565e-19;
constexpr double ME = 9.10938215e-31;
constexpr double K_B = 1.380648e-23;
constexpr double PI_REF = 3.141592653;
constexpr double EV = 1.602176565e-19;
constexpr int CS_RANGES = 5000000;
constexpr double DE_CS = 0.005;
constexpr double E_EXC_TH = 11.5;
constexpr double E_ION_TH = 15.8;

// Device error flag bits (sim->d_flags[0]).
enum : int {
  FLAG_OUT_OF_GRID = 1,
  FLAG_CAPACITY = 2,
  FLAG_TIMEOUT = 4,
  FLAG_BAD_TABLE = 8,
  FLAG_LOAD_IN_CONDUCTOR = 16,  // a deterministic load placed a particle inside a conductor
};

// Bounded spin: polls of a device-side wait before it reports FLAG_TIMEOUT
// (the default).  spin_limit() is the limit the launchers pass to their
// kernels: SPIN_LIMIT unless epic_set_spin_limit chose another.
constexpr long long SPIN_LIMIT = 1ll << 24;
long long spin_limit();
__host__ __device__ inline long long spin_or_default(long long v) { return v > 0 ? v : SPIN_LIMIT; }

constexpr int PART_THREADS = 256;
constexpr int SCAN_TILE = 1024;  // particles per ordered tile (push+compact, MCC append)

struct Geom {
  int nx, ny;
  double x0, y0, dx, dy, Lx, Ly;
};

struct SoA {
  double *x, *y, *vx, *vy, *vz;
};

// Conductors on the device (the reference's Grid objects, src/grid.cpp,
// src/electrode.cpp): ReactConductorGrid rectangles {min_x, max_x, min_y,
// max_y} and the electrodes of every CircularGrid {x0, y0, r*r, -}.  A circular
// grid's electrodes exist only once gssolver has run CircularGrid::initialize,
// so circles count while *live != 0 (set by the first SOR solve's override).
struct CondSet {
  int nrect, ncirc;
  const double4* rect;
  const double4* circ;
  const int* live;
};

// Mixed-precision particle record (24 bytes): the grid node at the lower-left
// corner of the particle's cell (i*ny + j, so the deposit needs no index
// arithmetic), the FP32 offset inside the cell in units of dx/dy, in [0, 1),
// and FP32 velocities.  Position = x0 + (i + ox)*dx.
struct MixedSoA {
  int* cell;
  float *ox, *oy, *vx, *vy, *vz;
};

// Particles of one species in either layout.
struct ParticleRef {
  int mixed;
  SoA f;
  MixedSoA m;
};

// Per-launch solver outcome, written by the device.
struct SolveInfo {
  int iterations;
  int converged;
  double error;
};

struct CrossSections {
  // kind 0: linear grid E_i = de*i (E_0 = de), nearest index (the reference);
  // kind 1: logarithmic grid, linear interpolation in log E (extension).
  int kind;
  int64_t n;
  double de, log_emin, inv_dlog, e_min, e_max;
  double *tot, *ela, *exc, *ion;  // tot includes the gas density
  double nu_max;                  // bound of tot(E)*v(E) for null collisions
  // First-draw cut per speed bin (MCC_SPEED_BINS entries, see mcc_speed_bin),
  // for the direct MCC of one run's vel_norm and dt; null: the global cut.
  unsigned long long* bin_cut = nullptr;
  // Device code only: the logarithmic table staged in shared memory as
  // {tot, ela, exc, ion} per entry (mcc_stage_table), or null.
  const double4* stab = nullptr;
};
// A logarithmic table of at most this many entries is staged in shared memory
// by the collision kernels (32 bytes per entry).
constexpr int MCC_SMEM_TABLE = 1536;
inline int mcc_table_smem(const CrossSections& cs) {
  return cs.kind == 1 && cs.n <= MCC_SMEM_TABLE ? (int)cs.n * 32 : 0;
}

// Speed bins of the MCC early-out, keyed by m = max(|vx|, |vy|, |vz|) (vel_norm
// units, from the bits alone): bin 0 holds m < 2^-64, bin 1 + 4(e + 64) + q
// the m in [2^e (1 + q/4), 2^e (1 + (q+1)/4)) for e in [-64, 63], and bin
// MCC_SPEED_BINS - 1 everything from 2^64 up (infinities and NaN included),
// which always passes.  |v|^2 lies in [m^2, 3 m^2].
constexpr int MCC_SPEED_BINS = 1024;
constexpr int MCC_BIN_EMIN = -64, MCC_BIN_EMAX = 63;
// Host: the cut of every bin for the tables of cs (host copy tot of n
// entries), vel_norm and dt_phys (epic_capi.cu).
void mcc_bin_cuts(const CrossSections& cs, const double* tot, double vel_norm, double dt_phys,
                  unsigned long long* out);

// ---- kernel launchers (epic_particles.cu) ----
void launch_deposit(cudaStream_t st, const Geom& g, int shape, int fixed, const SoA& p, const long long* d_n,
                    double spwt, double* den, unsigned long long* acc, double fx_scale, int* flags, int grid);
// Host-resident particles (epic_step_host; FP64 form, fixed-point deposit,
// periodic or reflective walls): `host` is mapped pinned memory of
// {x, y, vx, vy, vz} records.
void launch_upload_deposit(cudaStream_t st, const Geom& g, int shape, const double* host, long long n, const SoA& p,
                           long long* d_n, unsigned long long* acc, double fx_scale, int* flags, int grid);
void launch_push_download(cudaStream_t st, const Geom& g, int shape, int bc, const SoA& p, const long long* d_n,
                          const double2* ef, const double2* cell, double qmK, double c, double dtsub, double* host,
                          int* flags, int grid, int contract);
void launch_download(cudaStream_t st, const SoA& p, const long long* d_n, long long from, long long cap, double* host,
                     int* flags, int grid);
// The conductors' rho override before an SOR solve (Grid::initialize inside
// gssolver, src/field.cpp:100-103): rho[nodes[k]] = vals[k], then *live = 1.
void launch_conductor_rho(cudaStream_t st, double* rho, const int* nodes, const double* vals, int n, int* live);
// The FP64 push erasing particles that end inside a conductor (order kept,
// src/species.cpp:80-97, 108-121, 150-165); needs the compaction scratch.
void launch_push_conductors(cudaStream_t st, const Geom& g, int shape, int bc, const SoA& p, long long* d_n,
                            const double2* ef, const double2* cell, double qmK, double c, double dtsub,
                            const CondSet& cs, int* flags, unsigned long long* tile_status, unsigned int* tile_ctr,
                            int grid, int contract);
// Emitter::inject into one species (slot 0: species_idx1, 1: species_idx2):
// appends num particles at the live count; the count is advanced by
// launch_emit_commit (so the two slots of one emitter read the same counts).
struct EmitDev {
  double x0, y0, x1, y1;
  double vth, vdx, vdy, vel_norm;  // vth = sqrt(2 k_B T EV_to_K / m); vdx, vdy in m/s
  int num, slot, emitter;
};
struct ParticleRef;
void launch_emit(cudaStream_t st, const ParticleRef& p, const Geom& g, const long long* d_n, long long cap,
                 const EmitDev& e, unsigned long long seed, const unsigned long long* d_inj, const double* uniforms,
                 int* flags, int grid);
void launch_emit_commit(cudaStream_t st, long long* d_n, long long num, long long cap, int* flags);
void launch_inject_tick(cudaStream_t st, unsigned long long* d_inj);
struct SelectArgs;
// The FP64 push.  ef is the node field; cell the bilinear coefficients of
// each cell (launch_cell_coef), which the contracted CIC push reads instead.
// With dep_acc (periodic or reflective walls) every pushed particle is also
// deposited at its new position into dep_acc (fixed point, fx_scale), which
// the caller has zeroed: the next step's charge deposit, bit for bit.  With
// sel as well (contracted push, electrons) it also runs the MCC's selection.
void launch_push(cudaStream_t st, const Geom& g, int shape, int bc, const SoA& p, long long* d_n,
                 const double2* ef, const double2* cell, double qmK, double c, double dtsub, int* flags,
                 unsigned long long* tile_status, unsigned int* tile_ctr, int grid, int contract,
                 unsigned long long* dep_acc = nullptr, double fx_scale = 0.0, const SelectArgs* sel = nullptr);
// The fixed-point deposit of particles [*d_from, *d_n) (the products an MCC
// call appended) into acc.
void launch_deposit_range(cudaStream_t st, const Geom& g, int shape, const SoA& p, const long long* d_from,
                          const long long* d_n, unsigned long long* acc, double fx_scale, int* flags, int grid);
// cell[4 (i ny + j) + m], m = 0..3: a0 = E00, a1 = E10 - E00, a2 = E01 - E00,
// a3 = (E11 - E10) - (E01 - E00) of cell (i, j), from the interleaved field.
void launch_cell_coef(cudaStream_t st, const Geom& g, const double2* ef, double2* cell);
void launch_rewind(cudaStream_t st, const Geom& g, int shape, const SoA& p, const long long* d_n, const double2* ef,
                   double hqmK, double dt, int* flags, int grid);
// Ionisation events of one MCC launch: products in `buf` (count, cap), the
// event index of each marked electron in `slot` (-1 otherwise; capacity of the
// electron species) and the number of events per tile of MCC_TILE electrons
// in tile_cnt, scanned into tile_off.  All of it is returned to the cleared
// state (slot -1, counts 0) by the launch itself.
constexpr int MCC_TILE = 512;
struct IonEvent;
struct McEvents {
  IonEvent* buf;
  unsigned int* count;
  unsigned int cap;
  int* slot;
  unsigned int* tile_cnt;
  unsigned int* tile_off;
  unsigned int* cand;        // electrons whose first draw passed the cut (any order)
  unsigned int* cand_count;
};
// d_step: device step counter (Philox counter word), advanced by every MCC
// launch so replayed graphs draw fresh numbers.
// skip_select: the candidates are already in ev (the electrons' push selected
// them, Philox mode, FP64 form).
void launch_mcc(cudaStream_t st, int mode, const CrossSections& cs, const ParticleRef& e, long long* d_ne,
                long long e_cap, const ParticleRef& ion, long long* d_ni, long long i_cap, double vel_norm,
                double dt_phys, double ion_mass, double ion_temp, const double* uniforms, int ustride, uint64_t seed,
                unsigned long long* d_step, const McEvents& ev, unsigned long long* d_ncoll, int* flags, int grid,
                int skip_select = 0);
// The first-draw cut of the MCC's selection: cut53 for every speed, and the
// per-speed-bin table (or null).
void mcc_select_cut(const CrossSections& cs, int mode, double dt_phys, unsigned long long* cut53,
                    const unsigned long long** bin_cut);
// The MCC's selection pass run inside the electrons' push: the candidates of
// the step's MCC (Philox mode) appended to cand.
struct SelectArgs {
  const unsigned long long* bin_cut;
  unsigned long long cut53;
  uint64_t seed;
  const unsigned long long* d_step;
  unsigned int* cand;
  unsigned int* cand_count;
};
size_t ion_event_bytes();

// ---- mixed-precision particle kernels (epic_mixed.cu) ----
void launch_aos_to_mixed(cudaStream_t st, const Geom& g, const double* aos, const MixedSoA& p, long long n,
                         int* flags, int grid);
void launch_mixed_to_aos(cudaStream_t st, const Geom& g, double* aos, const MixedSoA& p, const long long* d_n,
                         int grid);
void launch_deposit_mixed(cudaStream_t st, const Geom& g, int shape, const MixedSoA& p, const long long* d_n,
                          unsigned long long* acc, int* flags, int grid);
// CTAs of `kernel` (threads per CTA, no dynamic shared memory) resident at once
// on the current device: a grid of one full wave.
template <class K>
int resident_grid(K kernel, int threads) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, threads, 0);
  return (per > 0 ? per : 1) * (sms > 0 ? sms : 1);
}

// With dep_acc (CIC, periodic or reflective walls) every pushed particle is
// also deposited at its new position into dep_acc (integer weights), and with
// sel the electrons' MCC candidates are appended to sel->cand.  With cond,
// particles that end inside a conductor are erased (compacting push).
void launch_push_mixed(cudaStream_t st, const Geom& g, int shape, int bc, const MixedSoA& p, long long* d_n,
                       const float2* ef, float qmK_dt, float cx, float cy, int* flags,
                       unsigned long long* tile_status, unsigned int* tile_ctr, int grid,
                       unsigned long long* dep_acc = nullptr, const SelectArgs* sel = nullptr,
                       const CondSet* cond = nullptr);
void launch_deposit_mixed_range(cudaStream_t st, const Geom& g, const MixedSoA& p, const long long* d_from,
                                const long long* d_n, unsigned long long* acc, int grid);
void launch_rewind_mixed(cudaStream_t st, const Geom& g, int shape, const MixedSoA& p, const long long* d_n,
                         const float2* ef, float hqmK_dt, int* flags, int grid);
void launch_particle_sums_mixed(cudaStream_t st, int what, const MixedSoA& p, const long long* d_n,
                                double vel_norm, double* partials, double* out3, int grid);
constexpr int MIXED_OFFSET_BITS = 20;  // deposit weights: offsets quantised to 2^-20 of a cell

// ---- device loading and run digest (epic_load.cu) ----
// kind: 0 random, 1 uniform, 2 sin(n), 3 cos(n) (the reference's load types).
// rect: nrect conductor rectangles {min_x, max_x, min_y, max_y} that Init
// keeps particles out of (a random position is drawn again; a deterministic
// one inside raises FLAG_LOAD_IN_CONDUCTOR in *flags).
void launch_load(cudaStream_t st, const Geom& g, const epic_species_desc& d, const epic_config& c, int species,
                 int kind, int narg, double* aos, unsigned long long seed, int grid, const double4* rect = nullptr,
                 int nrect = 0, int* flags = nullptr);
void launch_set_count(cudaStream_t st, long long* d_n, long long n);
void launch_digest(cudaStream_t st, const void* a, int elem_bytes, const long long* d_n, long long n,
                   unsigned long long tag, unsigned long long* out, int grid);

// ---- cell sort (epic_sort.cu) ----
struct SortScratch {
  unsigned* keys[2];
  unsigned* vals[2];
  unsigned* hist;   // digit table [digit][tile], scanned in place
  unsigned* bsum;   // scan totals
  void* tmp;        // payload copy (24 or 40 bytes per particle slot)
};
size_t sort_scratch_bytes(long long cap, int payload);
SortScratch carve_sort_scratch(void* buf, long long cap);
// Sorts one species by cell (stable); returns the number of kernels launched.
int launch_sort(cudaStream_t st, const Geom& g, const ParticleRef& p, const long long* d_n, long long cap,
                const SortScratch& sc, int grid);
void launch_deposit_mixed_sorted(cudaStream_t st, const Geom& g, const MixedSoA& p, const long long* d_n,
                                 unsigned long long* acc, int grid);

// ---- spectral FP32 inner solve with FP64 refinement (epic_spectral.cu) ----
struct SolverArgs;
// Fast transforms of the mixed solve for lattices whose sides allow them
// (epic_spectral.cuh, spec_fft_unit): a line of n unknowns is transformed by
// a complex radix-2 FFT of length m, m = n for the Hartley transform
// (periodic direction, n a power of two) and m = 2 (n + 1) for the sine
// transform (DST-I by odd extension, n + 1 a power of two).
struct SpecFFT {
  int on;                  // 1: the solve's four products per stage are FFT passes
  int mR, mC, lgR, lgC;    // FFT lengths of the two directions and their log2
  int sineR, sineC;        // 1: sine transform, 0: Hartley
  float scaleR, scaleC;    // orthonormal scaling: sqrt(2 / (n + 1)) or 1 / sqrt(n)
  const float2* twR;       // e^(-2 pi i k / mR), k < mR / 2
  const float2* twC;
};
struct SpectralSolver {
  int R, C;       // lattice of unknowns: R rows of C
  int flat;       // 1: pcgsolver's lattice of the flattened vector (all nodes); 0: gssolver's interior
  int mode;       // EPIC_POISSON_* (an extension lattice: rows i = r + i0, columns j, see Lattice)
  int gs_norm;    // 1: stop on the SOR residual L2 of src/field.cpp:118-134, 0: on |b - Ax|_2
  float *QR, *QC; // R x R and C x C sine transforms, orthonormal and symmetric (shared when R = C)
  float* D;       // R x C, 1/(lambda_p + mu_q)
  float *t0, *t1; // R x C FP32 scratch
  double *r64;    // residual scratch (nx*ny)
  double* partials;
  int* state;     // [0] done flag, [1] stage, [2] converged
  SpecFFT fft;    // fft.on: FFT passes instead of the dense products (large lattices)
};
int spectral_supported(const Geom& g, int solver, int poisson_bc);
int spectral_chunks(const SpectralSolver& sp);  // residual chunks (partials needed)
void launch_spectral(cudaStream_t st, const SpectralSolver& sp, const SolverArgs& a, int stages);
void launch_particle_sums(cudaStream_t st, int what, const SoA& p, const long long* d_n, double vel_norm,
                          double* partials, double* out3, int grid);

// ---- kernel launchers (epic_field.cu) ----
// FINALIZE_ONLY: density of the active species from its accumulator;
// FINALIZE_AND_RHO: every species, then rho; RHO_FROM_DEN: rho from the
// already finalised density grids.
enum { FINALIZE_ONLY = 0, FINALIZE_AND_RHO = 1, RHO_FROM_DEN = 2 };
struct FinalizeArgs {
  Geom g;
  int nsp;
  int bc;
  int fixed;
  int stage;
  int active[8];
  double div;
  const unsigned long long* acc[8];
  double* den[8];
  double spwt[8];
  double inv_scale[8];
  double charge_over_qe[8];
  double* rho;
};
void launch_finalize(cudaStream_t st, const FinalizeArgs& a);
void launch_efield(cudaStream_t st, const Geom& g, int bc, int poisson_bc, const double* phi, double* efx,
                   double* efy, double2* ef, float2* ef32);

struct SolverArgs {
  Geom g;
  double tol;
  int max_iter;
  double omega;
  double K;          // (L*L)/(LDe*LDe)
  const double* rho;
  double* phi;
  SolveInfo* info;
  unsigned long long* iter_total;  // running sum of iterations (profiling)
  int* flags;
  // PCG workspace: 8 node vectors (b, r x2, s x2, w x2, p)
  double* work[8];
  double* partials;  // 4 * max_blocks
  unsigned int* bar; // grid barrier {count, generation}
  int warm;
  unsigned long long tol_bits;  // PCG stop test: sqrt(r.r) < tol <=> bits(r.r) < tol_bits (set by launch_pcg)
  long long spin;               // poll limit of the grid-wide waits (set by the launchers; 0 = SPIN_LIMIT)
  int poisson_bc;               // EPIC_POISSON_* (the extensions' lattices, see Lattice)
};

// The unknowns of a PCG / SOR solve as a lattice of R rows of C columns.
// EPIC_POISSON_DIRICHLET (the reference's pcgsolver): the flattened node
// vector in rows of nx (row = k / nx, col = k % nx, src/field.cpp:221-232),
// neighbours outside the lattice contribute nothing.  The extensions: rows
// are the x index i = row + i0, columns the y index j, node (row, col) at
// (row + i0) * ny + col; DIRICHLET_X has i0 = 1, R = nx - 2 (the walls are
// not unknowns) and wraps columns (C = ny - 1, node ny-1 is node 0);
// PERIODIC has i0 = 0, R = nx - 1 and wraps rows and columns.
struct Lattice {
  int R, C;
  int rs, k0;  // node of (row, col) = k0 + row * rs + col
  int wrap_r, wrap_c;
  int mode;    // EPIC_POISSON_*
};
__host__ __device__ inline Lattice make_lattice(int nx, int ny, int poisson_bc) {
  Lattice l;
  l.mode = poisson_bc;
  if (poisson_bc == EPIC_POISSON_PERIODIC) {
    l.R = nx - 1; l.C = ny - 1; l.rs = ny; l.k0 = 0; l.wrap_r = 1; l.wrap_c = 1;
  } else if (poisson_bc == EPIC_POISSON_DIRICHLET_X) {
    l.R = nx - 2; l.C = ny - 1; l.rs = ny; l.k0 = ny; l.wrap_r = 0; l.wrap_c = 1;
  } else {
    l.R = ny; l.C = nx; l.rs = nx; l.k0 = 0; l.wrap_r = 0; l.wrap_c = 0;
  }
  return l;
}
__host__ __device__ inline int lattice_node(const Lattice& l, int row, int col) { return l.k0 + row * l.rs + col; }
// Lattice position of a neighbour row / column index that may lie one step
// outside: wrapped where the lattice is periodic, else -1 (no neighbour).
__host__ __device__ inline int lattice_wrap(int v, int n, int wrap) {
  if (v >= 0 && v < n) return v;
  if (!wrap) return -1;
  return v < 0 ? v + n : v - n;
}
// The solve's duplicated nodes after an extension solve: periodic copies
// (node nx-1 from node 0, node ny-1 from node 0) and the zero x walls of
// DIRICHLET_X (epic_field.cu).
void launch_fill_poisson_nodes(cudaStream_t st, const Geom& g, int poisson_bc, double* phi);
void init_field_kernels();  // one-time kernel attributes (called by epic_create)
void set_last_error(const char* msg);  // the message epic_last_error() returns on this thread
void launch_sor_lex(cudaStream_t st, const SolverArgs& a);
// Boltzmann-electron solvers: gsfluidsolver ("gshybrid"; writes rho's edge
// values, as the reference does) and nrpcgsolver ("hybrid").
void launch_gsfluid(cudaStream_t st, const SolverArgs& a, double* rho);
void launch_nrpcg(cudaStream_t st, const SolverArgs& a);
void launch_sor_redblack(cudaStream_t st, const SolverArgs& a, int blocks);
void launch_pcg(cudaStream_t st, const SolverArgs& a, int blocks);
int solver_max_blocks();
// CTA budget of a PCG solve on `nodes` unknowns (shared by every entry point
// that runs it, so they all produce the same iterates).
int pcg_default_blocks(long long nodes, int sms);
void launch_grid_sums(cudaStream_t st, int what, const Geom& g, const double* a, const double* b, double L,
                      double* partials, double* out);

}  // namespace epic

// The opaque handle of the C ABI.
struct epic_species_state {
  epic_species_desc desc;
  std::string name;
  long long cap;
  epic::SoA soa;        // FP64 plain form
  epic::MixedSoA mx;    // mixed-precision form (cell, FP32 offsets and velocities)
  long long* d_n;
  double* den;
  unsigned long long* acc;
  double fx_scale;      // 2^k
  double fx_inv_scale;  // 2^-k
  // acc holds the fixed-point deposit of the species' current positions (set
  // by a deposit or by a push that deposits as it moves the particles;
  // cleared by anything that moves, adds or replaces particles otherwise).
  bool acc_valid = false;
};

struct epic_sim {
  epic_config cfg;
  epic::Geom g;
  cudaStream_t stream;
  cudaStream_t side = nullptr;  // epic_step_host: electrons pushed beside the other species' transfers
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // epic_run_host: copy-engine streams for each step's host round trip, their
  // events, and the records of every species staged in HBM on the way in and out.
  cudaStream_t xfer_out = nullptr, xfer_in = nullptr;
  std::vector<cudaEvent_t> xfer_ev;
  double* host_in = nullptr;
  double* host_out = nullptr;
  long long* h_counts = nullptr;  // pinned
  size_t host_stage_doubles = 0;
  int num_sms;
  int part_grid;
  std::vector<epic_species_state> sp;
  double *phi, *rho, *efx, *efy;
  double2* ef;
  double2* ef_cell;            // bilinear coefficients per cell (contracted CIC push), or null
  float2* ef32;                // FP32 (efx, efy) for the mixed-precision gather
  epic::SpectralSolver spec;   // mixed-precision Poisson solve (square grids)
  int mixed;                   // cfg.precision == EPIC_PRECISION_MIXED
  // solver workspace
  double* work[8];
  double* partials;
  unsigned int* bar;
  epic::SolveInfo* d_info;
  unsigned long long* d_iter_total;
  // particle scratch
  unsigned long long* tile_status;
  long long tile_status_len;
  unsigned int* tile_ctr;
  unsigned long long* d_ncoll;  // [0] collisions of the last MCC, [1..2] pending appends/collisions
  unsigned long long* d_step;   // MCC launches so far (Philox counter)
  epic::McEvents mcc_ev;        // ionisation event scratch (allocated on first MCC)
  long long mcc_ev_for_cap;     // electron capacity the scratch was sized for
  void* staging;                // AoS staging for uploads/downloads
  size_t staging_bytes;
  double* d_uniforms;
  long long uniforms_len;
  double* sum_partials;
  double* d_sums;
  double* h_sums;  // pinned
  int* d_flags;
  // Conductors (epic_add_conductor): host list, device geometry, rho override
  std::vector<epic_conductor> conductors;
  double4* d_cond_rect = nullptr;
  double4* d_cond_circ = nullptr;
  int* d_cond_nodes = nullptr;
  double* d_cond_vals = nullptr;
  int* d_cond_live = nullptr;
  int cond_nrect = 0, cond_ncirc = 0, cond_nnodes = 0;
  // Emitters (epic_add_emitter) and the device count of injections
  std::vector<epic_emitter> emitters;
  unsigned long long* d_inj = nullptr;
  // The reference's global mt19937 for per-species Init (epic_init_species);
  // created on first use with seed 0, reseeded by epic_load_particles.
  void* ref_rng = nullptr;
  epic::CrossSections cs;
  int64_t launches;
  cudaGraphExec_t graph_exec;       // one step
  cudaGraphExec_t graph_exec_sort;  // one step that starts with the cell sort
  int64_t graph_launches, graph_launches_sort;
  int graph_collisions;
  // cell sort
  int64_t step_index;               // steps taken (decides which steps sort)
  bool steady_capture = false;      // capturing the steady-state step (accumulators valid on entry)
  long long* d_nold = nullptr;      // electron and ion counts before the MCC (its products are deposited)
  void* sort_buf;
  long long sort_cap;               // largest capacity the buffer serves
  // per-phase profiling (events on `stream`)
  int profiling;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> prof_pending;
  std::vector<cudaEvent_t> event_pool;
  double prof_ms[EPIC_NUM_PHASES];
  int64_t prof_count[EPIC_NUM_PHASES];
  int64_t prof_iters;
  int prof_solves;
};
