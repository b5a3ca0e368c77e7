// epic2d.hpp — the reference's C++ interface for the time-step loop, over the
// C ABI of include/epic2d.h (header-only; link libepic2d_gb300.so).
//
// Class names, constructors, method signatures, argument meaning and error
// behaviour follow the reference, so a main written against it compiles
// here unchanged: Domain (include/domain.h:26-201), Species and Particle
// (include/species.h:22-78), Init (include/init.h:17-34), FieldSolve
// (include/field.h:14-31), CollisionHandler (include/collision.h:19-35), Grid
// with Create_Grid / GridParams / RectangularGridParams (include/grid.h:11-86),
// Emitter / EmitterParams (include/emitter.h), INIParser
// (include/iniparser.h:18-35) and the constants of namespace Const
// (include/domain.h:204-215).  The forms that take the C ABI's structs
// (Domain(const epic_config&), Species(Domain&, const epic_species_desc&),
// Push_species_serial(int), FieldSolve(Domain&), ...) are kept as overloads.
//
// All state lives on the GPU.  Domain gathers the configuration the way the
// reference's main fills it (constructor, member assignments, set_normparam,
// set_time, set_normscheme) and creates the GPU simulation when a loop call
// first needs it (Init, FieldSolve, a scatter, ...); species and conductors
// registered before that are added then, in order.  Host copies of particles
// and grids are made only on request (Species::download_part_list,
// Domain::phi() and friends).  A failing call throws std::runtime_error (the
// reference throws std::out_of_range / std::invalid_argument in the same
// places); a solver that hits max_iteration prints to std::cerr and returns
// false, as gssolver does.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/epic2d.h"

namespace epic2d {

inline void check(epic_status st) {
  if (st != EPIC_OK) throw std::runtime_error(std::string("epic2d: ") + epic_last_error());
}

// include/domain.h:204-215 (PI is the reference's truncated value).
namespace Const {
const double EPS_0 = 8.85418782e-12;
const double QE = 1.602176565e-19;
const double AMU = 1.660538921e-27;
const double ME = 9.10938215e-31;
const double K_b = 1.380648e-23;
const double PI = 3.141592653;
const double EV_to_K = QE / K_b;
const double eV = 1.602176565e-19;
}  // namespace Const

// INIParser (include/iniparser.h:18-35): sections of key = value; the lines of
// [species] are kept whole under the keys "0", "1", ...; lines starting with
// ';' or '#' are comments.  getInt/getDouble/getString throw
// std::out_of_range for a missing key, as std::map::at does there.  The
// three-argument forms read one key of a file (through the C ABI).
struct INIParser {
  using Section = std::map<std::string, std::string>;

  static void trim(std::string& s) {
    const auto a = s.find_first_not_of(" \t\r");
    const auto b = s.find_last_not_of(" \t\r");
    s = a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
  }
  static std::map<std::string, Section> parse(const std::string& filename) {
    std::ifstream f(filename);
    if (!f) throw std::runtime_error("Unable to open file: " + filename);
    std::map<std::string, Section> out;
    std::string line, cur;
    while (std::getline(f, line)) {
      if (line.empty() || line[0] == ';' || line[0] == '#') continue;
      if (line.front() == '[' && line.back() == ']') {
        cur = line.substr(1, line.size() - 2);
        out[cur];
        continue;
      }
      Section& sec = out[cur];
      if (cur == "species") {
        sec[std::to_string(sec.size())] = line;
        continue;
      }
      const auto eq = line.find('=');
      if (eq == std::string::npos) continue;
      std::string k = line.substr(0, eq), v = line.substr(eq + 1);
      trim(k);
      trim(v);
      sec[k] = v;
    }
    return out;
  }
  static std::string getString(const Section& section, const std::string& key) { return section.at(key); }
  static int getInt(const Section& section, const std::string& key) { return std::stoi(section.at(key)); }
  static double getDouble(const Section& section, const std::string& key) { return std::stod(section.at(key)); }
  static std::vector<std::string> split(const std::string& str, char delimiter) {
    std::vector<std::string> out;
    std::stringstream ss(str);
    std::string t;
    while (std::getline(ss, t, delimiter)) out.push_back(t);
    return out;
  }
  // "sin(3)" -> ("sin", 3); a plain type -> (type, 0).
  static std::pair<std::string, int> loadtypeextract(const std::string& position_init) {
    const auto lp = position_init.find('('), rp = position_init.find(')');
    if (lp != std::string::npos && rp != std::string::npos && rp > lp)
      return {position_init.substr(0, lp), std::stoi(position_init.substr(lp + 1, rp - lp - 1))};
    return {position_init, 0};
  }

  static std::string getString(const std::string& path, const std::string& section, const std::string& key) {
    char buf[512];
    check(epic_ini_get(path.c_str(), section.c_str(), key.c_str(), buf, sizeof(buf)));
    return buf;
  }
  static int getInt(const std::string& path, const std::string& section, const std::string& key) {
    return std::stoi(getString(path, section, key));
  }
  static double getDouble(const std::string& path, const std::string& section, const std::string& key) {
    return std::stod(getString(path, section, key));
  }
};

// class Particle (include/species.h:22-37).
class Particle {
 public:
  double pos[2];
  double vel[3];
  Particle(double x, double y, double vx, double vy, double vz) {
    pos[0] = x;
    pos[1] = y;
    vel[0] = vx;
    vel[1] = vy;
    vel[2] = vz;
  }
};

// Three components, indexable as the reference's vec<double> (v(i)) and as an array (v[i]).
struct vec3 : std::array<double, 3> {
  double operator()(int i) const { return (*this)[(size_t)i]; }
  double& operator()(int i) { return (*this)[(size_t)i]; }
};

class Species;
class Grid;

// The conductors of include/grid.h: GridType, GridParams (CircularGrid),
// RectangularGridParams (ReactConductorGrid), Create_Grid.  A Grid carries the
// conductor's description; the GPU simulation takes it over when the grids
// vector first reaches Init, FieldSolve or a push.
enum class GridType { Custom, Circular, Line, ReactConductor };
struct GridParams {
  int grid_centerx;
  int grid_centery;
  int num_electrodes;
  double grid_rad;
  double electrode_rad;
  double voltage;
};
struct RectangularGridParams {
  int min_x;
  int max_x;
  int min_y;
  int max_y;
  double voltage;
};
class Grid {
 public:
  explicit Grid(const epic_conductor& c) : desc(c) {}
  virtual ~Grid() = default;
  epic_conductor desc;
};

class Domain {
 public:
  // Members with the reference's names and meaning (include/domain.h:29-199).
  double x0 = 0, y0 = 0;
  double Lx = 0, Ly = 0;
  double dx = 1, dy = 1;
  int cell_no = 0;
  int nx = 0, ny = 0;
  int NUM_TS = 0, write_interval = 0, write_interval_phase = 0, sub_cycle_interval = 0;
  double LDe = 0, wpe = 0, LDi = 0, wpi = 0;
  double lenght_scale = 0, time_scale = 0;
  double W = 0, L = 0;
  double IAW_vel = 0;
  double vel_norm = 0;
  double density = 0;
  double DT = 0;
  int species_no = 0;
  double norm = 0;
  std::string SolverType = "gs";
  double tolerance = 1e-4;
  int max_iteration = 1000;
  double vel_ratio = 0;
  bool push_parallal = false, deposit_parallal = false;
  int num_threads = 1;
  double error = 0;
  std::string pload, bc = "pbc", shapefunction = "CIC", diagtype;
  int normscheme = 1, vel_normscheme = 1;
  double delta_g = 0;
  bool enable_elastic_collision = false, enable_excitation_collision = false, enable_ionization_collision = false;
  double GAS_DENSITY = 0;
  int ionfixed = 0;
  // GPU-side options with no reference counterpart (sor_omega, poisson_bc,
  // push_order, ...; epic_config_defaults gives the reference's behaviour).
  // Read when the GPU simulation is created.
  epic_config options;

  // Domain::Domain (src/domain.cpp:7-16).
  Domain(double x0_, double y0_, double dx_, double dy_, int nx_, int ny_)
      : x0(x0_), y0(y0_), dx(dx_), dy(dy_), nx(nx_), ny(ny_) {
    epic_config_defaults(&options);
    Lx = (nx - 1) * dx;
    Ly = (ny - 1) * dy;
  }
  // A complete configuration (the C ABI's); the GPU simulation is created now.
  explicit Domain(const epic_config& cfg) {
    options = cfg;
    from_config(cfg);
    check(epic_create(&options, &sim_));
  }
  ~Domain() {
    if (sim_) epic_destroy(sim_);
  }
  Domain(const Domain&) = delete;
  Domain& operator=(const Domain&) = delete;

  // Domain::set_normparam / set_time (src/domain.cpp:117-121, 185-191).
  void set_normparam(double LDe_, double wpe_, double LDi_, double wpi_) {
    LDe = LDe_;
    wpe = wpe_;
    LDi = LDi_;
    wpi = wpi_;
  }
  void set_time(double DT_, int NUM_TS_, int write_interval_, int write_interval_phase_) {
    DT = DT_;
    NUM_TS = NUM_TS_;
    write_interval = write_interval_;
    write_interval_phase = write_interval_phase_;
  }
  // Domain::set_normscheme (src/domain.cpp:123-183): L and W from the scheme;
  // vel_norm = L W (the ion-acoustic speed for vel_normscheme 3: the branches
  // for 1 and 2 are overwritten by the final if/else there).
  void set_normscheme() {
    if (normscheme == 1 || normscheme == 3) {
      L = LDe;
      W = wpe;
    } else if (normscheme == 2 || normscheme == 4) {
      L = LDi;
      W = normscheme == 2 ? wpi : wpe;
    } else if (normscheme == 5) {
      LDe = lenght_scale;
      wpe = time_scale;
      L = LDe;
      W = wpe;
      vel_norm = L * W;
      return;
    } else {
      throw std::invalid_argument("Invalid normscheme flag");
    }
    vel_norm = vel_normscheme == 3 ? IAW_vel : L * W;
  }
  // Domain::display (src/domain.cpp:18-114), the parameters and species.
  inline void display(std::vector<Species>& species);

  // Domain::ComputeRho (src/domain.cpp:194-202): rho of every species of the
  // simulation (the reference's main passes them all).
  void ComputeRho(std::vector<Species>&) { ComputeRho(); }
  void ComputeRho() { check(epic_compute_rho(handle())); }
  // Domain::Compute_PE (src/domain.cpp:266-286), normalised by `species`.
  inline double Compute_PE(Species& species);
  double Compute_PE(int norm_species) {
    double pe = 0;
    check(epic_compute_pe(handle(), norm_species, &pe));
    return pe;
  }

  std::vector<double> grid(int which) {
    std::vector<double> g((size_t)nx * ny);
    check(epic_get_grid(handle(), which, g.data()));
    return g;
  }
  std::vector<double> phi() { return grid(EPIC_GRID_PHI); }
  std::vector<double> rho() { return grid(EPIC_GRID_RHO); }
  std::vector<double> efx() { return grid(EPIC_GRID_EFX); }
  std::vector<double> efy() { return grid(EPIC_GRID_EFY); }
  // max(phi) - phi(0,0) as printed by Output::diagnostics.
  double delta_phi() {
    double d = 0;
    check(epic_delta_phi(handle(), &d));
    return d;
  }
  // Create_Grid + grids.push_back (src/grid.cpp:88-103), before any Init.
  void add_conductor(const epic_conductor& c) { check(epic_add_conductor(handle(), &c)); }
  // Takes over conductors of a grids vector not seen before (in order).
  void use_grids(const std::vector<Grid*>& grids) {
    for (const Grid* g : grids)
      if (g && std::find(grids_seen_.begin(), grids_seen_.end(), g) == grids_seen_.end()) {
        add_conductor(g->desc);
        grids_seen_.push_back(g);
      }
  }
  // The configuration the members describe, in the C ABI's form.
  epic_config config() const {
    epic_config c = options;
    c.nx = nx;
    c.ny = ny;
    c.x0 = x0;
    c.y0 = y0;
    c.dx = dx;
    c.dy = dy;
    c.DT = DT;
    c.L = L;
    c.W = W;
    c.vel_norm = vel_norm;
    c.LDe = LDe;
    c.wpe = wpe;
    c.LDi = LDi;
    c.wpi = wpi;
    c.density = density;
    c.shape = shapefunction == "NGP" ? EPIC_NGP : EPIC_CIC;
    if (shapefunction != "NGP" && shapefunction != "CIC") throw std::invalid_argument("shapefunction " + shapefunction);
    if (bc == "pbc") c.bc = EPIC_PBC;
    else if (bc == "open") c.bc = EPIC_OPEN;
    else if (bc == "reflective") c.bc = EPIC_REFLECTIVE;
    else throw std::invalid_argument("bc " + bc);
    if (SolverType == "gs") c.solver = EPIC_SOLVER_GS;
    else if (SolverType == "cg" || SolverType == "iter" || SolverType == "iterative") c.solver = EPIC_SOLVER_PCG;
    else if (SolverType == "gshybrid") c.solver = EPIC_SOLVER_GSHYBRID;
    else if (SolverType == "hybrid") c.solver = EPIC_SOLVER_HYBRID;
    else throw std::invalid_argument("solvertype " + SolverType);
    c.tolerance = tolerance;
    c.max_iteration = max_iteration;
    c.ionfixed = ionfixed;
    c.normscheme = normscheme;
    c.gas_density = GAS_DENSITY;
    c.elastic = enable_elastic_collision;
    c.excitation = enable_excitation_collision;
    c.ionization = enable_ionization_collision;
    return c;
  }
  // The GPU simulation, created on first use with the species registered so far.
  epic_sim* handle() {
    if (!sim_) {
      options = config();
      check(epic_create(&options, &sim_));
      for (const epic_species_desc& d : pending_) {
        int idx = 0;
        check(epic_add_species(sim_, &d, &idx));
      }
      pending_.clear();
    }
    return sim_;
  }
  const epic_config& config_used() const { return options; }
  // Species registration (Species's constructor); returns the species index.
  int register_species(const epic_species_desc& d) {
    if (sim_) {
      int idx = 0;
      check(epic_add_species(sim_, &d, &idx));
      return idx;
    }
    pending_.push_back(d);
    return (int)pending_.size() - 1;
  }
  // Emitter registration (Emitter's constructor); returns the emitter index.
  int register_emitter(const epic_emitter& e) {
    check(epic_add_emitter(handle(), &e));
    return emitters_++;
  }

 private:
  void from_config(const epic_config& c) {
    nx = c.nx;
    ny = c.ny;
    x0 = c.x0;
    y0 = c.y0;
    dx = c.dx;
    dy = c.dy;
    Lx = (nx - 1) * dx;
    Ly = (ny - 1) * dy;
    DT = c.DT;
    L = c.L;
    W = c.W;
    vel_norm = c.vel_norm;
    LDe = c.LDe;
    wpe = c.wpe;
    LDi = c.LDi;
    wpi = c.wpi;
    density = c.density;
    shapefunction = c.shape == EPIC_NGP ? "NGP" : "CIC";
    bc = c.bc == EPIC_OPEN ? "open" : c.bc == EPIC_REFLECTIVE ? "reflective" : "pbc";
    SolverType = c.solver == EPIC_SOLVER_PCG        ? "cg"
                 : c.solver == EPIC_SOLVER_GSHYBRID ? "gshybrid"
                 : c.solver == EPIC_SOLVER_HYBRID   ? "hybrid"
                                                    : "gs";
    tolerance = c.tolerance;
    max_iteration = c.max_iteration;
    ionfixed = c.ionfixed;
    normscheme = c.normscheme;
    GAS_DENSITY = c.gas_density;
    enable_elastic_collision = c.elastic;
    enable_excitation_collision = c.excitation;
    enable_ionization_collision = c.ionization;
  }

  epic_sim* sim_ = nullptr;
  std::vector<epic_species_desc> pending_;
  std::vector<const Grid*> grids_seen_;
  int emitters_ = 0;
};

// Create_Grid (src/grid.cpp:88-103): a CircularGrid or ReactConductorGrid
// (Custom and Line grids have no electrodes there and return a Grid without
// effect, or nullptr for Line, as the reference).
inline Grid* Create_Grid(GridType type, Domain&, const GridParams& params, const RectangularGridParams& rparam) {
  epic_conductor c{};
  switch (type) {
    case GridType::Circular:
      c.type = EPIC_CONDUCTOR_CIRCULAR;
      c.x_center = params.grid_centerx;
      c.y_center = params.grid_centery;
      c.electrode_number = params.num_electrodes;
      c.grid_radius = params.grid_rad;
      c.electrode_radius = params.electrode_rad;
      c.voltage = params.voltage;
      return new Grid(c);
    case GridType::Line:
    case GridType::ReactConductor:
      c.type = EPIC_CONDUCTOR_RECT;
      c.min_x = rparam.min_x;
      c.max_x = rparam.max_x;
      c.min_y = rparam.min_y;
      c.max_y = rparam.max_y;
      c.voltage = rparam.voltage;
      return new Grid(c);
    default:
      return nullptr;
  }
}

// One particle species (Species, src/species.cpp).
class Species {
 public:
  std::string name;
  double mass = 0, charge = 0, spwt = 0, temp = 0;
  int numparticle = 0;
  int charge_sig = 0;
  std::string initialization;
  double vsx = 0, vsy = 0, fract_den = 0;
  // Host copy of the particles, filled by download_part_list (the particles
  // live on the GPU).
  std::vector<Particle> part_list;

  // Species::Species (src/species.cpp:6-22); the species joins the domain's simulation.
  Species(std::string name_, double mass_, double charge_, double spwt_, double temp_, int numparticle_, double vsx_,
          double vsy_, double fract_den_, std::string initialization_, Domain& domain)
      : name(std::move(name_)), mass(mass_), charge(charge_), spwt(spwt_), temp(temp_), numparticle(numparticle_),
        initialization(std::move(initialization_)), vsx(vsx_), vsy(vsy_), fract_den(fract_den_), domain_(&domain) {
    epic_species_desc d{};
    std::snprintf(d.name, sizeof(d.name), "%s", name.c_str());
    d.mass = mass;
    d.charge = charge;
    d.spwt = spwt;
    d.temp = temp;
    d.numparticle = numparticle;
    d.vsx = vsx;
    d.vsy = vsy;
    d.fract_den = fract_den;
    std::snprintf(d.load, sizeof(d.load), "%s", initialization.c_str());
    index_ = domain.register_species(d);
  }
  // The C ABI's species description.
  Species(Domain& domain, const epic_species_desc& desc)
      : Species(desc.name, desc.mass, desc.charge, desc.spwt, desc.temp, desc.numparticle, desc.vsx, desc.vsy,
                desc.fract_den, desc.load, domain) {}

  // Species::ScatterSpecies_serial (src/species.cpp:172-226).
  void ScatterSpecies_serial() { check(epic_scatter_species(domain_->handle(), index_)); }
  // Species::Push_species_serial (src/species.cpp:29-170): particles that end
  // inside a conductor of `grids` are erased.
  void Push_species_serial(int sub_cycle, const std::vector<Grid*>& grids) {
    domain_->use_grids(grids);
    Push_species_serial(sub_cycle);
  }
  void Push_species_serial(int sub_cycle) { check(epic_push_species(domain_->handle(), index_, sub_cycle)); }
  // Species::Rewind_species (src/species.cpp:229-246).
  void Rewind_species() { check(epic_rewind_species(domain_->handle(), index_)); }
  // Species::Compute_KE / Compute_Momentum (src/species.cpp:248-297),
  // normalised by `species`.
  vec3 Compute_KE(const Species& species) {
    vec3 k{};
    check(epic_compute_ke(domain_->handle(), index_, species.index_, k.data()));
    return k;
  }
  vec3 Compute_Momentum(const Species& species) {
    vec3 p{};
    check(epic_compute_momentum(domain_->handle(), index_, species.index_, p.data()));
    return p;
  }
  // Species::AddParticle (src/species.cpp:24-27): appends one particle.
  void AddParticle(Particle part) {
    std::vector<double> all = particles();
    all.insert(all.end(), {part.pos[0], part.pos[1], part.vel[0], part.vel[1], part.vel[2]});
    set_particles(all);
  }
  // part_list <- the GPU's particles.
  void download_part_list() {
    const std::vector<double> a = particles();
    part_list.clear();
    part_list.reserve(a.size() / 5);
    for (size_t q = 0; q + 4 < a.size(); q += 5) part_list.emplace_back(a[q], a[q + 1], a[q + 2], a[q + 3], a[q + 4]);
  }
  // Particles as records of {x, y, vx, vy, vz} (class Particle).
  std::vector<double> particles() {
    int64_t n = size();
    std::vector<double> out((size_t)n * 5);
    if (n) check(epic_get_particles(domain_->handle(), index_, out.data(), n, &n));
    return out;
  }
  void set_particles(const std::vector<double>& parts) {
    check(epic_set_particles(domain_->handle(), index_, parts.data(), (int64_t)(parts.size() / 5)));
  }
  int64_t size() {
    int64_t n = 0;
    check(epic_num_particles(domain_->handle(), index_, &n));
    return n;
  }
  int index() const { return index_; }
  Domain& domain() { return *domain_; }

 private:
  Domain* domain_;
  int index_ = -1;
};

inline double Domain::Compute_PE(Species& species) { return Compute_PE(species.index()); }

inline void Domain::display(std::vector<Species>& species) {
  std::cout << "System Dimension: " << nx << " x " << ny << "\nNormalized Time Step: " << DT
            << "\nTotal Time Steps: " << NUM_TS << "\nPlasma Density: " << density << "\nElectron Debye Length: " << LDe
            << "\nElectron Plasma Frequency: " << wpe << "\nBoundary Condition: " << bc
            << "\nPotential Solver: " << SolverType << "\nSolver Tolerance: " << tolerance
            << "\nShape Function: " << shapefunction << "\n";
  for (Species& p : species)
    std::cout << "Species " << p.name << ": mass " << p.mass << ", charge " << p.charge << ", spwt " << p.spwt
              << ", particles " << p.numparticle << "\n";
}

// Init::Init (src/init.cpp:3-101): loads the species' particles from the
// reference's global generator (one mt19937 seeded with 0, continued from
// species to species), positions inside a conductor drawn again.
class Init {
 public:
  Init(Species& species, Domain& domain, std::vector<Grid*>& grids) {
    domain.use_grids(grids);
    check(epic_init_species(domain.handle(), species.index()));
  }
  // Init::SampleVel (src/init.cpp:104-114) is drawn inside the loader.
};

// FieldSolve (src/field.cpp): gssolver, pcgsolver, gsfluidsolver or
// nrpcgsolver by SolverType.
class FieldSolve {
 public:
  FieldSolve(Domain& d, const std::vector<Grid*>& grids) : domain_(d) { d.use_grids(grids); }
  explicit FieldSolve(Domain& d) : domain_(d) {}
  // FieldSolve::PotentialSolver (src/field.cpp:266-272).
  bool PotentialSolver() {
    int it = 0;
    double err = 0;
    epic_status st = epic_potential_solver(domain_.handle(), &it, &err);
    domain_.error = err;
    if (st == EPIC_WARN_NOT_CONVERGED) {
      std::cerr << "GS failed to converge, L2=" << err << std::endl;
      return false;
    }
    check(st);
    return true;
  }
  // The solvers by name run the configured solver (the reference's main
  // calls PotentialSolver, which dispatches on SolverType).
  bool gssolver() { return PotentialSolver(); }
  void pcgsolver() { PotentialSolver(); }
  bool gsfluidsolver() { return PotentialSolver(); }
  void nrpcgsolver() { PotentialSolver(); }
  // FieldSolve::CalculateEfield (src/field.cpp:276-330).
  void CalculateEfield() { check(epic_calculate_efield(domain_.handle())); }

 private:
  Domain& domain_;
};

// CollisionHandler (src/collision.cpp).
class CollisionHandler {
 public:
  explicit CollisionHandler(Domain& d) : domain_(d) {}
  // set_electron_cross_sections + calc_total_cross_sections (src/collision.cpp:12-42).
  void set_electron_cross_sections() { check(epic_set_reference_cross_sections(domain_.handle())); }
  void calc_total_cross_sections() {}  // formed with the tables by set_electron_cross_sections
  // handle_collisions (src/collision.cpp:190-207).
  void handle_collisions(Species& electron, Species& target_gas) { last_collisions = collide(electron, target_gas); }
  int64_t collide(Species& electron, Species& target_gas) {
    int64_t n = 0;
    check(epic_handle_collisions(domain_.handle(), electron.index(), target_gas.index(), nullptr, 0, &n));
    return n;
  }
  int64_t last_collisions = 0;

 private:
  Domain& domain_;
};

// EmitterParams / Emitter (include/emitter.h, src/emitter.cpp:5-36).
struct EmitterParams {
  double x0;
  double y0;
  double x1;
  double y1;
  double temp;
  int numparticle;
  double vdx;
  double vdy;
  int species_idx1;
  int species_idx2;
};
class Emitter {
 public:
  Emitter(const EmitterParams& params, Domain& domain) : domain_(&domain) {
    epic_emitter e{};
    e.x0 = params.x0;
    e.y0 = params.y0;
    e.x1 = params.x1;
    e.y1 = params.y1;
    e.temp = params.temp;
    e.numparticle = params.numparticle;
    e.vdx = params.vdx;
    e.vdy = params.vdy;
    e.species_idx1 = params.species_idx1;
    e.species_idx2 = params.species_idx2;
    index_ = domain.register_emitter(e);
  }
  // Emitter::inject: this emitter's particles into species_idx1 (and idx2).
  void inject(std::vector<Species>&) { check(epic_inject_emitter(domain_->handle(), index_, nullptr)); }

 private:
  Domain* domain_;
  int index_ = -1;
};

}  // namespace epic2d
