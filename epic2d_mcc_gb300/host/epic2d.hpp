// epic2d.hpp — the reference's C++ interface for the time-step loop, over the
// C ABI of include/epic2d.h (header-only; link libepic2d_gb300.so).
//
// Class and method names, argument meaning and error behaviour follow the
// reference: Domain (include/domain.h:26-201), Species (include/species.h:
// 39-78), FieldSolve (include/field.h:14-31), CollisionHandler
// (include/collision.h:19-35) and INIParser (include/iniparser.h:18-31).  A
// failing call throws std::runtime_error (the reference throws
// std::out_of_range / std::invalid_argument in the same places); a solver that
// hits max_iteration prints to std::cerr and returns false, as gssolver does.
// All state lives on the GPU; host copies are made only on request.
#pragma once

#include <array>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/epic2d.h"

namespace epic2d {

inline void check(epic_status st) {
  if (st != EPIC_OK) throw std::runtime_error(std::string("epic2d: ") + epic_last_error());
}

// INIParser::getString/getInt/getDouble over a file (src/iniparser.cpp:53-66).
struct INIParser {
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

class Species;

// The simulation domain and every grid (phi, rho, efx, efy, densities).
class Domain {
 public:
  explicit Domain(const epic_config& cfg) : cfg_(cfg) { check(epic_create(&cfg_, &sim_)); }
  ~Domain() { epic_destroy(sim_); }
  Domain(const Domain&) = delete;
  Domain& operator=(const Domain&) = delete;

  // Domain::ComputeRho (src/domain.cpp:194-202).
  void ComputeRho() { check(epic_compute_rho(sim_)); }
  // Domain::Compute_PE (src/domain.cpp:266-286).
  double Compute_PE(int norm_species) {
    double pe = 0;
    check(epic_compute_pe(sim_, norm_species, &pe));
    return pe;
  }
  std::vector<double> grid(int which) const {
    std::vector<double> g((size_t)cfg_.nx * cfg_.ny);
    check(epic_get_grid(sim_, which, g.data()));
    return g;
  }
  std::vector<double> phi() const { return grid(EPIC_GRID_PHI); }
  std::vector<double> rho() const { return grid(EPIC_GRID_RHO); }
  std::vector<double> efx() const { return grid(EPIC_GRID_EFX); }
  std::vector<double> efy() const { return grid(EPIC_GRID_EFY); }
  // max(phi) - phi(0,0) as printed by Output::diagnostics.
  double delta_phi() {
    double d = 0;
    check(epic_delta_phi(sim_, &d));
    return d;
  }
  // Create_Grid + grids.push_back (src/grid.cpp:88-103): a ReactConductorGrid
  // or CircularGrid conductor, before the particles are loaded.
  void add_conductor(const epic_conductor& c) { check(epic_add_conductor(sim_, &c)); }
  const epic_config& config() const { return cfg_; }
  epic_sim* handle() { return sim_; }
  double error = 0;  // Domain::error: last solver residual

 private:
  epic_config cfg_;
  epic_sim* sim_ = nullptr;
};

// One particle species (Species, src/species.cpp).
class Species {
 public:
  Species(Domain& domain, const epic_species_desc& desc) : domain_(domain), desc_(desc) {
    check(epic_add_species(domain.handle(), &desc_, &index_));
    name = desc_.name;
    mass = desc_.mass;
    charge = desc_.charge;
    spwt = desc_.spwt;
    temp = desc_.temp;
    numparticle = desc_.numparticle;
    fract_den = desc_.fract_den;
    vsx = desc_.vsx;
    vsy = desc_.vsy;
  }
  // Species::ScatterSpecies_serial (src/species.cpp:172-226).
  void ScatterSpecies_serial() { check(epic_scatter_species(domain_.handle(), index_)); }
  // Species::Push_species_serial (src/species.cpp:29-170); conductors are not supported.
  void Push_species_serial(int sub_cycle) { check(epic_push_species(domain_.handle(), index_, sub_cycle)); }
  // Species::Rewind_species (src/species.cpp:229-246).
  void Rewind_species() { check(epic_rewind_species(domain_.handle(), index_)); }
  // Species::Compute_KE / Compute_Momentum (src/species.cpp:248-297).
  std::array<double, 3> Compute_KE(const Species& norm) {
    std::array<double, 3> k{};
    check(epic_compute_ke(domain_.handle(), index_, norm.index_, k.data()));
    return k;
  }
  std::array<double, 3> Compute_Momentum(const Species& norm) {
    std::array<double, 3> p{};
    check(epic_compute_momentum(domain_.handle(), index_, norm.index_, p.data()));
    return p;
  }
  // part_list as records of {x, y, vx, vy, vz} (class Particle).
  std::vector<double> particles() {
    int64_t n = 0;
    check(epic_num_particles(domain_.handle(), index_, &n));
    std::vector<double> out((size_t)n * 5);
    if (n) check(epic_get_particles(domain_.handle(), index_, out.data(), n, &n));
    return out;
  }
  void set_particles(const std::vector<double>& parts) {
    check(epic_set_particles(domain_.handle(), index_, parts.data(), (int64_t)(parts.size() / 5)));
  }
  int64_t size() {
    int64_t n = 0;
    check(epic_num_particles(domain_.handle(), index_, &n));
    return n;
  }
  int index() const { return index_; }

  std::string name;
  double mass, charge, spwt, temp;
  int numparticle;
  double fract_den, vsx, vsy;

 private:
  Domain& domain_;
  epic_species_desc desc_;
  int index_ = -1;
};

// FieldSolve (src/field.cpp): gssolver or pcgsolver by solvertype.
class FieldSolve {
 public:
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
  void calc_total_cross_sections() {}  // folded into set_electron_cross_sections
  // handle_collisions (src/collision.cpp:190-207).
  int64_t handle_collisions(Species& electron, Species& target_gas) {
    int64_t n = 0;
    check(epic_handle_collisions(domain_.handle(), electron.index(), target_gas.index(), nullptr, 0, &n));
    return n;
  }

 private:
  Domain& domain_;
};

}  // namespace epic2d
