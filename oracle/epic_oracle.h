/* ORACLE TEST INFRASTRUCTURE — not part of the product.
 *
 * Plain-C restatement of the ePIC2D time-step loop (deposit, charge density,
 * SOR and PCG Poisson solves, E-field, gather + leapfrog push, rewind, MCC and
 * the energy/momentum diagnostics).  Only tests/, the smoke check and the CPU
 * baseline leg of bench.py may call it, and only as the checker.
 *
 * Every function follows the reference's operation order (same association of
 * every + and *, same loop order) so that, compiled with -ffp-contract=off, it
 * reproduces the reference bit for bit; the tests pin that against the
 * reference's own objects (oracle/_ref) and against tests/golden fixtures.
 *
 * Grids are row-major doubles, element (i, j) at i*ny + j (the reference's
 * Matrix<double>(nx, ny) with i = x index).  Particles are AoS records of five
 * doubles {x, y, vx, vy, vz} (the reference's Particle, include/species.h:22-37).
 */
#ifndef EPIC_ORACLE_H
#define EPIC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Physical constants of include/domain.h:204-215 (PI is the reference's
 * truncated 3.141592653) and the MCC table constants of
 * include/collision.h:14-15, include/cross_sections.h:14-15. */
#define OR_EPS_0 8.85418782e-12
#define OR_QE 1.602176565e-19
#define OR_AMU 1.660538921e-27
#define OR_ME 9.10938215e-31
#define OR_K_B 1.380648e-23
#define OR_PI 3.141592653
#define OR_M_PI 3.14159265358979323846  /* M_PI (src/grid.cpp, src/electrode.cpp) */
#define OR_GRID_WORDS 8
#define OR_EV 1.602176565e-19
#define OR_CS_RANGES 5000000
#define OR_DE_CS 0.005
#define OR_E_EXC_TH 11.5
#define OR_E_ION_TH 15.8

enum { OR_CIC = 0, OR_NGP = 1 };
enum { OR_PBC = 0, OR_OPEN = 1, OR_REFLECTIVE = 2 };

typedef struct {
  uint32_t mt[624];
  int mti;
} or_rng;

typedef struct {
  int nx, ny;                 /* node counts (Nx+1, Ny+1) */
  double x0, y0, dx, dy, Lx, Ly;
  double DT, L, W, vel_norm, LDe, wpe, density;
  int shape, bc;
  double tolerance;
  int max_iteration;
  double gas_density;
  int elastic, excitation, ionization;
  /* Extensions with no reference counterpart (0 = the reference's behaviour):
   * poisson_bc 0 = the reference's solvers (zero on every edge), 1 = periodic
   * in x and y, 2 = phi = 0 on the x walls and periodic in y; load_3v 1 =
   * vz drawn like vx and vy (the reference loads vz = 0). */
  int poisson_bc;
  int load_3v;
} or_domain;

enum { OR_POISSON_REFERENCE = 0, OR_POISSON_PERIODIC = 1, OR_POISSON_DIRICHLET_X = 2 };

/* mt19937 + std::generate_canonical<double, 53> (two 32-bit draws per double). */
void or_rng_seed(or_rng* r, uint32_t seed);
uint32_t or_rng_u32(or_rng* r);
double or_rng_uniform(or_rng* r);

/* Init::SampleVel (src/init.cpp:104-114). */
double or_sample_vel(or_rng* r, double mass, double temp);
/* Particle loading of src/init.cpp:3-101 for load types random, uniform,
 * sin(n), cos(n) (no conductors).  Returns 0, or -1 for an unknown type. */
int or_load(const or_domain* d, or_rng* r, const char* type, int n_arg, double mass, double temp, double vsx,
            double vsy, long n, double* out);

/* Species::ScatterSpecies_serial (src/species.cpp:172-226): den is overwritten.
 * Returns the number of particles that fell outside the grid (the reference
 * throws std::out_of_range there); such particles are skipped. */
long or_scatter(const or_domain* d, const double* part, long n, double spwt, double* den);
/* Domain::ComputeRho (src/domain.cpp:194-202). */
void or_compute_rho(const or_domain* d, int nsp, const double* const* dens, const double* charges, double* rho);
/* FieldSolve::gssolver (src/field.cpp:70-139); omega = 1.4 is the reference.
 * Returns 1 if converged.  *iters = sweeps done, *err = last L2 check. */
int or_gs_solve(const or_domain* d, double omega, const double* rho, double* phi, double* err, int* iters);
/* FieldSolve::pcgsolver (src/field.cpp:212-264) with pcg() of
 * linearalgebra/solvers.h:73-100; *err = |A x - b| / n as the reference. */
int or_pcg_solve(const or_domain* d, const double* rho, double* phi, double* err, int* iters);
/* Correctly rounded sum of n doubles (any order gives the same result). */
double or_exact_sum(const double* x, long n);
/* FieldSolve::CalculateEfield (src/field.cpp:276-330). */
void or_efield(const or_domain* d, const double* phi, double* efx, double* efy);
/* Species::Push_species_serial (src/species.cpp:29-170), no conductors.
 * Returns the new particle count (open boundaries erase, order kept). */
/* Boltzmann-electron solvers: gsfluidsolver ("gshybrid", rho edited in
 * place) and nrpcgsolver ("hybrid", returns the CG iterations). */
int or_gsfluid_solve(const or_domain* d, double* rho, double* phi, double* err, int* iters);
long or_nrpcg_solve(const or_domain* d, const double* rho, double* phi, double* err);
/* Emitter::inject of one emitter (see epic_oracle.c). */
int or_inject(const or_domain* d, const double* em, double mass1, double mass2, or_rng* r, const double* pos_u,
              const double* vel_u, double* out1, long* n1, long cap1, double* out2, long* n2, long cap2);
/* Conductors (grids of OR_GRID_WORDS doubles, see epic_oracle.c). */
int or_in_conductors(const double* grids, int ng, int circles_live, double x, double y);
void or_conductor_rho(const or_domain* d, const double* grids, int ng, double* rho);
int or_load_c(const or_domain* d, or_rng* r, const char* type, int n_arg, double mass, double temp, double vsx,
              double vsy, long n, double* out, const double* grids, int ng);
long or_push_c(const or_domain* d, double mass, double charge, int sub_cycle, double* part, long n,
               const double* efx, const double* efy, const double* grids, int ng, int circles_live);
long or_push(const or_domain* d, double mass, double charge, int sub_cycle, double* part, long n,
             const double* efx, const double* efy);
/* Species::Rewind_species (src/species.cpp:229-246). */
void or_rewind(const or_domain* d, double mass, double charge, double* part, long n, const double* efx,
               const double* efy);

/* Cross sections of src/cross_section.cpp:4-39 and the 5,000,000-point linear
 * tables of src/collision.cpp:12-42 (tot already multiplied by gas density). */
double or_cs_elastic(double e, int enabled);
double or_cs_excitation(double e, int enabled);
double or_cs_ionization(double e, int enabled);
void or_cs_tables(const or_domain* d, double* tot, double* ela, double* exc, double* ion);

/* CollisionHandler::handle_collisions + collision_electron
 * (src/collision.cpp:60-207).  mode 0 draws from *rng in the reference's
 * sequential order; mode 1 gives electron p the uniforms
 * u[p*ustride + 0 ..] in the same draw order.  Ionisation products are
 * appended to the electron and ion arrays after the loop in electron order
 * (the electrons it appends are not visited in the same call, as in the
 * reference when its vector does not reallocate).  Returns collisions done;
 * *n_e, *n_i are updated; -1 if a capacity is exceeded. */
long or_mcc(const or_domain* d, const double* tot, const double* ela, const double* exc, const double* ion,
            double* e_part, long* n_e, long e_cap, double ion_mass, double ion_temp, double* i_part, long* n_i,
            long i_cap, int mode, or_rng* rng, const double* u, int ustride, int* kinds);

/* Cross-section table of the GPU implementation.  kind 0 is the reference's
 * linear grid (E_i = de*i, nearest index, src/collision.cpp:194-197); kind 1
 * is the logarithmic extension: n points from e_min to e_max, linear
 * interpolation in log E, energies clamped to [e_min, e_max].  tot includes
 * the gas density. */
typedef struct {
  int kind;
  long n;
  double de;
  double e_min, e_max, log_emin, inv_dlog;
  const double *tot, *ela, *exc, *ion;
} or_table;
void or_table_log(or_table* t, long n, double e_min, double e_max);
long or_mcc_table(const or_domain* d, const or_table* t, double* e_part, long* n_e, long e_cap, double ion_mass,
                  double ion_temp, double* i_part, long* n_i, long i_cap, int mode, or_rng* rng, const double* u,
                  int ustride, int* kinds);

/* Species::Compute_KE / Compute_Momentum (src/species.cpp:248-297) and
 * Domain::Compute_PE (src/domain.cpp:266-286). */
void or_ke(const or_domain* d, const double* part, long n, double mass, double spwt, double norm_temp,
           double norm_spwt, int norm_num, double* out3);
void or_momentum(const or_domain* d, const double* part, long n, double mass, double spwt, double norm_temp,
                 double norm_spwt, int norm_num, double* out3);
double or_pe(const or_domain* d, const double* efx, const double* efy, double norm_temp, double norm_spwt,
             int norm_num);

#ifdef __cplusplus
}
#endif
#endif
