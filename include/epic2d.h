/* epic2d.h — C ABI of the GB300 implementation of the ePIC2D time-step loop.
 *
 * One handle (epic_sim) owns one simulation resident on one GPU: particles as a
 * structure of arrays per species, and the node grids phi, rho, efx, efy and
 * one density grid per species.  Every entry point takes plain pointers and
 * sizes, never throws, and returns an epic_status; epic_last_error() gives the
 * message of the last failure on the calling thread.
 *
 * Each call replaces one method of the reference's C++ interface (the
 * reference has no FFI of its own; its seam is the method sequence of
 * src/main.cpp:359-423).  The citation beside each declaration names the
 * method it replaces.  Host arrays use the reference's layouts: grids are
 * row-major doubles with node (i, j) at i*ny + j (Matrix<double>(nx, ny),
 * linearalgebra/linalg.h:208-220) and particles are records of five doubles
 * {x, y, vx, vy, vz} (class Particle, include/species.h:22-37).
 *
 * A handle is used from one host thread at a time; all its GPU work runs in
 * order on the handle's own CUDA stream.
 */
#ifndef EPIC2D_H
#define EPIC2D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  EPIC_OK = 0,
  EPIC_ERR_INVALID = 1,       /* bad argument or configuration */
  EPIC_ERR_CUDA = 2,          /* CUDA runtime error */
  EPIC_ERR_NOMEM = 3,         /* device allocation failed */
  EPIC_ERR_CAPACITY = 4,      /* a species outgrew its particle capacity, or a grid exceeds a fixed scratch limit */
  EPIC_WARN_NOT_CONVERGED = 5,/* Poisson solve hit max_iteration (the reference prints to cerr) */
  EPIC_ERR_DOMAIN = 6,        /* a particle left the grid (the reference throws std::out_of_range) */
  EPIC_ERR_TIMEOUT = 7,       /* a device-side wait gave up */
  EPIC_ERR_BUDGET = 8,        /* admission refused: the memory budget is exhausted */
  EPIC_ERR_IO = 9             /* input file could not be read */
} epic_status;

enum { EPIC_CIC = 0, EPIC_NGP = 1 };                    /* [simulation] shapefunction */
enum { EPIC_PBC = 0, EPIC_OPEN = 1, EPIC_REFLECTIVE = 2 }; /* [simulation] bc */
/* [solver] solvertype gs | cg/iter/iterative | gshybrid | hybrid (the last two:
 * Boltzmann electrons, FieldSolve::gsfluidsolver / nrpcgsolver, src/field.cpp:7-68, 141-210) */
enum { EPIC_SOLVER_GS = 0, EPIC_SOLVER_PCG = 1, EPIC_SOLVER_GSHYBRID = 2, EPIC_SOLVER_HYBRID = 3 };
/* FP64 push arithmetic: CONTRACTED forms the CIC weights once and uses
 * multiply-adds (results within a few ulps of the reference's, well inside
 * 1e-12; under half the FP64 operations); REFERENCE keeps the operation order
 * of src/species.cpp:29-170 bit for bit.  [simulation] push_order. */
enum { EPIC_PUSH_CONTRACTED = 0, EPIC_PUSH_REFERENCE = 1 };
enum { EPIC_SOR_LEXICOGRAPHIC = 0, EPIC_SOR_REDBLACK = 1 };
enum { EPIC_DEPOSIT_FIXED = 0, EPIC_DEPOSIT_FP64 = 1 };
enum { EPIC_MCC_PHILOX = 0, EPIC_MCC_INJECTED = 1, EPIC_MCC_NULL = 2 };
enum { EPIC_GRID_PHI = 0, EPIC_GRID_RHO = 1, EPIC_GRID_EFX = 2, EPIC_GRID_EFY = 3, EPIC_GRID_DEN0 = 10 };

/* Everything Domain holds for the loop (include/domain.h:26-201), already
 * normalised as src/main.cpp:151-245 and Domain::set_normscheme
 * (src/domain.cpp:123-183) leave it, plus the GPU-side options.  Fields after
 * `gas_density`..`ionization` are options with no reference counterpart;
 * epic_config_defaults() sets each to the reference's behaviour. */
typedef struct {
  int nx, ny;                 /* node counts, Nx+1 and Ny+1 */
  double x0, y0, dx, dy;      /* origin and cell size (normalised) */
  double DT;                  /* normalised time step */
  double L, W, vel_norm;      /* length, frequency and velocity scales */
  double LDe, wpe, LDi, wpi;  /* Debye lengths and plasma frequencies */
  double density;             /* n0 [m^-3] */
  int shape;                  /* EPIC_CIC | EPIC_NGP */
  int bc;                     /* EPIC_PBC | EPIC_OPEN | EPIC_REFLECTIVE */
  int solver;                 /* EPIC_SOLVER_* */
  double tolerance;
  int max_iteration;
  int ionfixed;               /* skip the push of the species named "ion" */
  int normscheme;
  double gas_density;         /* [collision] GAS_DENSITY */
  int elastic, excitation, ionization;
  /* --- options (no reference counterpart) --- */
  double sor_omega;           /* 1.4, hard-coded at src/field.cpp:114 */
  int sor_mode;               /* EPIC_SOR_LEXICOGRAPHIC reproduces gssolver's iterates */
  int deposit_mode;           /* EPIC_DEPOSIT_FIXED: int64 fixed point, bit-reproducible */
  int mcc_mode;               /* EPIC_MCC_PHILOX: the reference's direct MCC on a Philox stream */
  uint64_t seed;              /* Philox key */
  int warm_start;             /* 0: cold-start solves as the reference */
  int solver_blocks;          /* CTAs of the grid-wide solvers; 0 = automatic */
  int precision;              /* EPIC_PRECISION_FP64 (the reference's arithmetic) | EPIC_PRECISION_MIXED */
  int sort_every;             /* sort particles by cell every k steps (0: never, the reference's order) */
  int push_order;             /* EPIC_PUSH_CONTRACTED (default) | EPIC_PUSH_REFERENCE (FP64 form) */
  int poisson_bc;             /* EPIC_POISSON_* ([solver] poisson_bc); DIRICHLET is the reference */
  int load_3v;                /* 1: Init draws vz like vx, vy ([simulation] load_3v; the reference loads vz = 0) */
  int reserved[10];
} epic_config;

/* Boundary of the Poisson problem (extension; no reference counterpart
 * except DIRICHLET).  DIRICHLET: the reference's solvers (gssolver holds
 * phi = 0 on every edge node, pcgsolver zeroes the right-hand side there).
 * PERIODIC: unknowns i in [0, nx-2], j in [0, ny-2], periodic in x and y
 * (node nx-1 is node 0, node ny-1 is node 0); the right-hand side is
 * projected onto zero mean and phi has zero mean over the unknowns.
 * DIRICHLET_X: phi = 0 on the x walls i = 0 and i = nx-1, periodic in y;
 * unknowns i in [1, nx-2], j in [0, ny-2].  The extensions keep each solver's
 * update, scaling, stopping test and residual norm, and the E-field takes
 * the periodic edge formula in periodic directions and the one-sided one at
 * the x walls.  Solvers: gs (lexicographic) and cg, both forms. */
enum { EPIC_POISSON_DIRICHLET = 0, EPIC_POISSON_PERIODIC = 1, EPIC_POISSON_DIRICHLET_X = 2 };

/* Mixed precision: particles as int32 cell + FP32 in-cell offsets + FP32
 * velocities, integer CIC weights, and a Poisson solve whose inner step is
 * FP32 (the exact sine-transform inverse of the same operator on square
 * grids) inside FP64 defect correction to the same tolerance. */
enum { EPIC_PRECISION_FP64 = 0, EPIC_PRECISION_MIXED = 1 };

/* One [species] line of input.ini (src/main.cpp:132-149) after set-up. */
typedef struct {
  char name[32];
  double mass, charge, spwt, temp;
  int numparticle;
  double vsx, vsy, fract_den;
  char load[32];              /* random | uniform | sin(n) | cos(n) */
  int64_t capacity;           /* particle slots to allocate; 0 = default */
} epic_species_desc;

typedef struct epic_sim epic_sim;

/* Message of the last failed call on this thread ("" if none). */
const char* epic_last_error(void);

/* Reference behaviour for every option field. */
void epic_config_defaults(epic_config* cfg);

/* INIParser::parse + the set-up of src/main.cpp:34-261 (normalisation, species
 * densities and weights; src/iniparser.cpp:4-113).  Also reads the optional
 * keys sor_omega, sor_mode, poisson_bc, deposit_mode, mcc_mode, seed,
 * warm_start, load_3v from [solver]/[simulation]/[collision].  *num_species is set to the number of
 * species lines; at most max_species descriptors are written. */
epic_status epic_config_from_ini(const char* path, epic_config* cfg, epic_species_desc* species, int max_species,
                                 int* num_species, int* num_ts);

/* INIParser::parse + getString (src/iniparser.cpp:4-66): copies the value of
 * [section] key into out (NUL-terminated, at most len bytes).  EPIC_ERR_INVALID
 * if the key is missing (the reference throws std::out_of_range). */
epic_status epic_ini_get(const char* path, const char* section, const char* key, char* out, int len);

/* Domain::Domain + FieldSolve::FieldSolve (src/domain.cpp:7-16, include/field.h:19). */
epic_status epic_create(const epic_config* cfg, epic_sim** out);
void epic_destroy(epic_sim* sim);

/* Species::Species (src/species.cpp:6-22).  *index receives the species index. */
epic_status epic_add_species(epic_sim* sim, const epic_species_desc* desc, int* index);

/* Init::Init for every species in index order from one mt19937 stream seeded
 * with `seed` (src/init.cpp:3-101; the reference seeds its global Rnd with 0,
 * include/domain.h:223).  Host-side start-up, as in the reference. */
epic_status epic_load_particles(epic_sim* sim, uint32_t seed);

/* Init::Init of one species (src/init.cpp:3-101), drawing from the handle's
 * copy of the reference's global generator (Rnd rnd, include/domain.h:218-231:
 * one mt19937 seeded with 0 when the handle is created and continued by every
 * call, reseeded by epic_load_particles).  Calling it for species 0, 1, ... in
 * order is epic_load_particles(sim, 0), as main runs Init per species
 * (src/main.cpp:359-362). */
epic_status epic_init_species(epic_sim* sim, int species);

/* Particle upload/download in the Particle layout (5 doubles per particle). */
epic_status epic_set_particles(epic_sim* sim, int species, const double* particles, int64_t n);
epic_status epic_get_particles(epic_sim* sim, int species, double* particles, int64_t capacity, int64_t* n);
epic_status epic_num_particles(epic_sim* sim, int species, int64_t* n);

/* Species::ScatterSpecies_serial (src/species.cpp:172-226). */
epic_status epic_scatter_species(epic_sim* sim, int species);
/* Domain::ComputeRho (src/domain.cpp:194-202). */
epic_status epic_compute_rho(epic_sim* sim);
/* FieldSolve::PotentialSolver (src/field.cpp:266-272): gssolver or pcgsolver.
 * iterations / error may be NULL; returns EPIC_WARN_NOT_CONVERGED at the cap. */
epic_status epic_potential_solver(epic_sim* sim, int* iterations, double* error);
/* FieldSolve::CalculateEfield (src/field.cpp:276-330). */
epic_status epic_calculate_efield(epic_sim* sim);
/* Species::Push_species_serial (src/species.cpp:29-170), no conductors. */
epic_status epic_push_species(epic_sim* sim, int species, int sub_cycle);
/* Species::Rewind_species (src/species.cpp:229-246). */
epic_status epic_rewind_species(epic_sim* sim, int species);
/* Cell sort (no counterpart in the reference, which never reorders
 * part_list): stable sort of the species' particles by the flat index
 * i*ny + j of the lower-left node of their cell, i = (int)((x - x0)/dx),
 * j = (int)((y - y0)/dy) (the node src/domain.cpp:207-208 deposits from).
 * Particles of one cell keep their relative order.  epic_step sorts every
 * species first on steps where step % sort_every == 0 (epic_config.sort_every,
 * 0 = never). */
epic_status epic_sort_species(epic_sim* sim, int species);

/* CollisionHandler::set_electron_cross_sections + calc_total_cross_sections
 * (src/collision.cpp:12-42): per-energy tables on the linear grid
 * E_i = de*i (E_0 = de), tot already multiplied by the gas density. */
epic_status epic_set_cross_sections(epic_sim* sim, const double* tot, const double* ela, const double* exc,
                                    const double* ion, int64_t n, double de);
/* Fills the tables with the e-/Ar fits of src/cross_section.cpp:4-39 on the
 * reference's 5,000,000-point, 0.005 eV grid (host-side start-up). */
epic_status epic_set_reference_cross_sections(epic_sim* sim);
/* Logarithmic table extension: n points from e_min to e_max [eV], sigma in
 * m^2 (not yet multiplied by the gas density), interpolated linearly in
 * log E.  Replaces the linear table. */
epic_status epic_set_log_cross_sections(epic_sim* sim, const double* ela, const double* exc, const double* ion,
                                        int64_t n, double e_min, double e_max);
/* CollisionHandler::handle_collisions (src/collision.cpp:190-207) of electron
 * species `electrons` against the neutral gas, with `ions` receiving the
 * ionisation products.  In EPIC_MCC_INJECTED mode, `uniforms` is a host array
 * of stride `ustride` per electron (the electron with index p draws
 * uniforms[p*ustride + k] in the reference's draw order); otherwise it is
 * ignored.  *collisions (may be NULL) receives the number of collisions. */
epic_status epic_handle_collisions(epic_sim* sim, int electrons, int ions, const double* uniforms, int ustride,
                                   int64_t* collisions);

/* One iteration of the loop body of src/main.cpp:405-423 (no emitters):
 * scatter all species, ComputeRho, PotentialSolver, CalculateEfield, push
 * every species (the one named "ion" is skipped if ionfixed), then
 * handle_collisions(species 0, species 1) if with_collisions. */
epic_status epic_step(epic_sim* sim, int with_collisions);
/* One loop iteration (as epic_step) for particles held by the caller in host
 * memory, as the reference holds part_list (src/main.cpp:405-423 over the
 * species' vectors): species s has n[s] records of {x, y, vx, vy, vz} at
 * parts[s] with room for capacity[s]; on return the records are the stepped
 * particles and n[s] their new count (ionisation appends electrons and ions).
 * With pinned buffers (cudaHostAlloc / cudaHostRegister) in the FP64 form,
 * with periodic or reflective walls and the fixed-point deposit, the kernels
 * read and write the buffers directly and overlap the transfers with the
 * deposit and the push; otherwise it is epic_set_particles + epic_step +
 * epic_get_particles.  Same results either way. */
epic_status epic_step_host(epic_sim* sim, int with_collisions, double* const* parts, int64_t* n,
                           const int64_t* capacity);
/* `steps` loop iterations (as epic_step_host, step after step) for particles
 * held in the caller's host buffers, which the caller leaves alone until the
 * call returns: after every step the stepped records are copied into the
 * buffers, and every step's push reads its input records copied from them.
 * With pinned buffers in the FP64 form (periodic or reflective walls, the
 * fixed-point deposit, no conductors, emitters or cell sort) the copies run
 * on copy engines, the two directions at once, while the SMs run the next
 * step's deposit, Poisson solve and E-field; otherwise each step is one
 * epic_step_host.  On return n[s] holds the counts (ionisation appends). */
epic_status epic_run_host(epic_sim* sim, int steps, int with_collisions, double* const* parts, int64_t* n,
                          const int64_t* capacity);
/* The prologue of src/main.cpp:366-382: scatter, rho, solve, E, rewind. */
epic_status epic_initial_field(epic_sim* sim);
/* Runs `steps` loop iterations; with use_graph=1 one step is captured as a
 * CUDA graph and replayed (fixed-size launches, device-side counts). */
epic_status epic_run(epic_sim* sim, int steps, int with_collisions, int use_graph);

/* Asynchronous forms for callers that keep several runs in flight (no
 * counterpart in the reference, which runs one loop in one process).  They
 * enqueue work on the handle's stream and return; epic_poll reports whether
 * the stream has drained (*done = 1) and then the status the work left, as
 * epic_sync would.  epic_run_async replays captured step graphs. */
epic_status epic_initial_field_async(epic_sim* sim);
epic_status epic_run_async(epic_sim* sim, int steps, int with_collisions);
epic_status epic_poll(epic_sim* sim, int* done);
/* Loads every species' numparticle particles on the GPU (asynchronous): the
 * placements and velocity formula of Init::Init / Init::SampleVel
 * (src/init.cpp:3-114) with uniforms from a Philox stream keyed by
 * (seed, species, particle) instead of the reference's mt19937 (use
 * epic_load_particles for the reference's own particles).  Conductor
 * rectangles keep particles out as Init's loop does (src/init.cpp:71-86): a
 * random position inside one is drawn again from the particle's stream; a
 * deterministic load type that puts one inside makes this call or the next
 * synchronising one return EPIC_ERR_INVALID. */
epic_status epic_load_particles_device(epic_sim* sim, uint64_t seed);
/* Order-independent 64-bit hashes of the run's state: out[0] of phi, out[1]
 * of every species' particle count and particle arrays (in the handle's
 * layout).  Equal digests mean bit-identical state. */
epic_status epic_digest(epic_sim* sim, uint64_t out[2]);

/* Species::Compute_KE / Compute_Momentum (src/species.cpp:248-297) and
 * Domain::Compute_PE (src/domain.cpp:266-286); norm_species is the species
 * whose temperature normalises (Output::storeKE_to_matrix, src/output.cpp:291-315). */
epic_status epic_compute_ke(epic_sim* sim, int species, int norm_species, double out[3]);
epic_status epic_compute_momentum(epic_sim* sim, int species, int norm_species, double out[3]);
epic_status epic_compute_pe(epic_sim* sim, int norm_species, double* pe);
/* max(phi) - phi(0,0) as printed by Output::diagnostics (src/output.cpp:320-336). */
epic_status epic_delta_phi(epic_sim* sim, double* delta_phi);

/* Conductors: the reference's Grid objects (include/grid.h, src/grid.cpp,
 * src/electrode.cpp), read from [Grids] (src/main.cpp:284-327).  A conductor
 * overwrites rho on its nodes with its voltage before every SOR solve
 * (Grid::initialize inside gssolver, src/field.cpp:100-103; the PCG solver
 * does not), particles that end a push inside one are erased in order
 * (src/species.cpp:80-165), and Init redraws random positions inside one
 * (src/init.cpp:71-86; a CircularGrid has electrodes only after the first SOR
 * solve, as in the reference).  Both forms (the mixed push tests the FP64
 * position rebuilt from cell and offset); load with epic_load_particles (the
 * device loader does not place particles around conductors). */
enum { EPIC_CONDUCTOR_RECT = 0, EPIC_CONDUCTOR_CIRCULAR = 1 };
typedef struct epic_conductor {
  int type;                                  /* EPIC_CONDUCTOR_* ("reactconduct", "circular") */
  int min_x, max_x, min_y, max_y;            /* RECT: ReactConductorGrid bounds */
  int x_center, y_center, electrode_number;  /* CIRCULAR: CircularGrid */
  double grid_radius, electrode_radius;
  double voltage;                            /* as the reference stores it: eV/(k_B EV_to_K) x the INI volts */
  int reserved[4];
} epic_conductor;
/* The [Grids] section in order (count = grid_count; at most max written). */
epic_status epic_conductors_from_ini(const char* path, epic_conductor* out, int max, int* count);
/* Create_Grid + grids.push_back (src/grid.cpp:88-103, src/main.cpp:312,323); before loading. */
epic_status epic_add_conductor(epic_sim* sim, const epic_conductor* c);

/* Emitters (include/emitter.h, src/emitter.cpp:5-36), read from [Emitters]
 * (src/main.cpp:330-355): at the start of every step each emitter appends
 * numparticle particles to species_idx1 (and the same number to
 * species_idx2, at the same positions, when the indices differ), positions
 * uniform on [x0, x1) x [y0, y1), velocities Init::SampleVel(temp) plus the
 * drift.  The reference draws the positions from a std::random_device-seeded
 * generator (not reproducible) and the velocities from its global stream;
 * here both come from a Philox stream keyed by (point, emitter, injection,
 * seed), or from caller uniforms (epic_inject).  Both forms. */
typedef struct epic_emitter {
  double x0, y0, x1, y1; /* injection rectangle (a segment when x0 == x1 or y0 == y1) */
  double temp;           /* eV */
  int numparticle;       /* particles (pairs) per step */
  double vdx, vdy;       /* drift in units of vel_norm */
  int species_idx1, species_idx2;
  int reserved[4];
} epic_emitter;
epic_status epic_emitters_from_ini(const char* path, epic_emitter* out, int max, int* count);
epic_status epic_add_emitter(epic_sim* sim, const epic_emitter* e);
/* Emitter::inject of every emitter, in order (what a step does first).
 * uniforms: null for the Philox stream, or for each emitter in order
 * numparticle rows of 14 doubles: the x and y uniforms, 6 velocity uniforms
 * for species_idx1 (vx then vy, three each) and 6 for species_idx2. */
epic_status epic_inject(epic_sim* sim, const double* uniforms);
/* Emitter::inject of emitter k alone (src/emitter.cpp:5-36), as the loop calls
 * it per emitter (src/main.cpp:397-403); uniforms: its numparticle rows of 14
 * or null.  The injection counter that keys the Philox streams advances after
 * the last emitter, so calling it for every emitter in order equals one
 * epic_inject. */
epic_status epic_inject_emitter(epic_sim* sim, int k, const double* uniforms);

/* Grid download/upload (which = EPIC_GRID_*, EPIC_GRID_DEN0 + s). */
epic_status epic_get_grid(epic_sim* sim, int which, double* out);
epic_status epic_set_grid(epic_sim* sim, int which, const double* in);

/* Waits for the handle's stream and reports any device-side error flag. */
epic_status epic_sync(epic_sim* sim);
/* Number of kernels this handle has launched (for launch accounting). */
int64_t epic_kernel_launches(epic_sim* sim);
/* The handle's CUDA stream (a cudaStream_t), for callers that order their own
 * work or events after the simulation's. */
void* epic_stream(epic_sim* sim);

/* Per-phase timing with CUDA events recorded on the handle's stream around
 * each phase of epic_step (no reference counterpart; the reference times the
 * whole run only, src/main.cpp:282,465-469).  Phases: 0 deposit, 1 density
 * finalisation + rho, 2 Poisson solve, 3 E-field, 4 push, 5 MCC, 6 cell sort.
 * epic_get_profile waits for the stream, then returns accumulated
 * milliseconds and step counts per phase and the solver iterations summed
 * over the profiled steps; it resets the accumulators. */
enum { EPIC_NUM_PHASES = 7 };
epic_status epic_set_profiling(epic_sim* sim, int enable);
epic_status epic_get_profile(epic_sim* sim, double ms[EPIC_NUM_PHASES], int64_t counts[EPIC_NUM_PHASES],
                             int64_t* solver_iterations);

/* Poll limit of the device-side waits (no counterpart in the reference,
 * which has no device waits): the grid barriers of the PCG and red-black SOR
 * solvers and the ordered tile look-back of the compacting pushes give up at
 * the `polls`-th unsuccessful poll and return, and the call that waited on the
 * kernel reports EPIC_ERR_TIMEOUT (the results of that kernel are void).
 * polls <= 0 restores the default (2^24 polls, far longer than any healthy
 * wait).  Process-wide; applies to launches made after the call (a step graph
 * keeps the limit it was captured with).  Meant for tests of the timeout
 * path: a limit of a few polls makes a healthy wait give up. */
epic_status epic_set_spin_limit(long long polls);

/* PCG solve with no device allocation (no counterpart in the reference: its
 * solver allocates dense matrices and vectors on every call).
 *
 * For callers that may not allocate GPU memory: frameworks whose memory pool
 * or budget owns the GPU and forbids private allocations, plugins confined to
 * the buffers their host hands them, and loops that must not meet the
 * allocator's latency or an out-of-memory failure mid-run.  rho (input)
 * and phi (output) are device arrays of nx*ny doubles in the reference's
 * layout (node (i, j) at i*ny + j); K = (L/LDe)^2.  The solve is the same as
 * epic_potential_solver with solvertype cg (same kernel and launch shape, so
 * the same phi), with all workspace in one static device array compiled into
 * the library: at most 257 x 257 nodes (larger grids return
 * EPIC_ERR_CAPACITY).  Every GPU that loads the library holds that array
 * (about 4.3 MB) until the library is unloaded.  Every call looks up the
 * array's device address on the current device (a host-side query; it stays
 * right after a device reset); the first call on a device also loads the
 * library's device code there, so make that first call before any stream
 * capture.  All calls share the array and leave their data in it; calls whose
 * GPU work overlaps race, so order them on one stream.  stream is a
 * cudaStream_t (NULL: the default stream); the call waits for the stream to
 * finish the solve, then reads the outcome back. */
epic_status epic_pcg_solve_static(const double* rho, double* phi, int nx, int ny, double dx, double K,
                                  double tolerance, int max_iteration, void* stream, int* iterations,
                                  double* error);

#ifdef __cplusplus
}
#endif
#endif
