// epic2d — command-line driver of the GB300 time-step loop, the counterpart
// of the reference's src/main.cpp: reads the same input.ini, loads particles
// from the same mt19937 stream, runs the initial field and NUM_TS + 1 loop
// iterations, and prints the diagnostics line of Output::diagnostics
// (src/output.cpp:318-392) every write_diagnostics steps.  `--output DIR`
// writes the reference's result.h5 tree as NPY files under DIR/result/ on the
// reference's cadence (src/main.cpp:268-277, 426-455; epic2d_output.hpp);
// `--energy FILE` writes the time history that Output::storeKE_to_matrix keeps
// (ts*DT, KE x/y/z per species, PE) as CSV.  Plotting is not part of it.
//
//   epic2d input.ini [--steps N] [--graph] [--output DIR] [--energy energy.csv] [--quiet]
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <memory>
#include <string>
#include <vector>

#include "epic2d.hpp"
#include "epic2d_output.hpp"

using namespace epic2d;

int main(int argc, char** argv) {
  if (argc < 2) {
    std::cout << "ERROR, at least one argument expected (the input file)." << std::endl;
    return 1;
  }
  const std::string ini = argv[1];
  int steps_override = -1;
  bool graph = false, quiet = false;
  std::string energy_path, output_dir;
  for (int k = 2; k < argc; k++) {
    if (!std::strcmp(argv[k], "--steps") && k + 1 < argc) steps_override = std::atoi(argv[++k]);
    else if (!std::strcmp(argv[k], "--graph")) graph = true;
    else if (!std::strcmp(argv[k], "--quiet")) quiet = true;
    else if (!std::strcmp(argv[k], "--energy") && k + 1 < argc) energy_path = argv[++k];
    else if (!std::strcmp(argv[k], "--output") && k + 1 < argc) output_dir = argv[++k];
  }
  try {
    epic_config cfg;
    epic_species_desc descs[8];
    int nsp = 0, num_ts = 0;
    check(epic_config_from_ini(ini.c_str(), &cfg, descs, 8, &nsp, &num_ts));
    if (nsp > 8) throw std::runtime_error("at most 8 species");
    const int write_diag = INIParser::getInt(ini, "diagnostics", "write_diagnostics");
    const int write_interval = INIParser::getInt(ini, "diagnostics", "write_interval");
    const int precision = INIParser::getInt(ini, "diagnostics", "precision");
    if (steps_override >= 0) num_ts = steps_override;
    const bool collisions = cfg.elastic || cfg.excitation || cfg.ionization;

    Domain domain(cfg);
    std::vector<std::unique_ptr<Species>> species;
    for (int s = 0; s < nsp; s++) species.emplace_back(new Species(domain, descs[s]));
    // [Grids] conductors (src/main.cpp:284-327), before Init as there.
    std::vector<epic_conductor> conds(64);
    int ncond = 0;
    check(epic_conductors_from_ini(ini.c_str(), conds.data(), (int)conds.size(), &ncond));
    if (ncond > (int)conds.size()) {
      conds.resize((size_t)ncond);
      check(epic_conductors_from_ini(ini.c_str(), conds.data(), ncond, &ncond));
    }
    for (int k = 0; k < ncond; k++) domain.add_conductor(conds[(size_t)k]);
    // [Emitters] (src/main.cpp:330-355); each step injects first (src/main.cpp:397-403).
    std::vector<epic_emitter> emits(64);
    int nemit = 0;
    check(epic_emitters_from_ini(ini.c_str(), emits.data(), (int)emits.size(), &nemit));
    if (nemit > (int)emits.size()) {
      emits.resize((size_t)nemit);
      check(epic_emitters_from_ini(ini.c_str(), emits.data(), nemit, &nemit));
    }
    for (int k = 0; k < nemit; k++) check(epic_add_emitter(domain.handle(), &emits[(size_t)k]));
    FieldSolve fieldsolver(domain);
    CollisionHandler coll(domain);
    check(epic_load_particles(domain.handle(), 0));  // Init, global Rnd seeded with 0
    // Initial field and the leapfrog half step back (src/main.cpp:366-382).
    check(epic_initial_field(domain.handle()));
    coll.set_electron_cross_sections();
    coll.calc_total_cross_sections();
    // Normalising species of Output::diagnostics (src/output.cpp:323-324).
    const bool hybrid = cfg.solver == EPIC_SOLVER_HYBRID || cfg.solver == EPIC_SOLVER_GSHYBRID;
    const int norm = !hybrid && (cfg.normscheme == 2 || cfg.normscheme == 4) ? 1 : 0;
    std::ofstream energy;
    if (!energy_path.empty()) energy.open(energy_path);
    std::unique_ptr<Output> output;
    int write_phase = 0, write_flag = 0;
    if (!output_dir.empty()) {
      write_phase = INIParser::getInt(ini, "diagnostics", "write_interval_phase");
      write_flag = INIParser::getInt(ini, "diagnostics", "write_flag");
      if (write_interval <= 0 || write_phase <= 0)
        throw std::runtime_error("write_interval and write_interval_phase must be positive");
      output.reset(new Output(output_dir, domain, num_ts, write_interval, nsp));
      // Output::write_metadata / write_species_metadata (src/main.cpp:275-277).
      output->write_metadata(cfg.nx, num_ts, write_interval, write_phase,
                             INIParser::getDouble(ini, "time", "DT_coeff"), cfg.density,
                             INIParser::getInt(ini, "diagnostics", "save_fig"), cfg.normscheme,
                             INIParser::getInt(ini, "diagnostics", "sub_cycle_interval"), cfg.LDe, cfg.LDi, cfg.wpe,
                             cfg.wpi, nsp, 0);
      output->write_species_metadata(species);
    }
    auto t0 = std::chrono::steady_clock::now();
    for (int ts = 0; ts < num_ts + 1; ts++) {
      if (graph) check(epic_run(domain.handle(), 1, collisions, 1));
      else check(epic_step(domain.handle(), collisions));
      if (output) {
        // src/main.cpp:431-455
        if (ts % write_phase == 0 && ts % write_interval == 0)
          for (auto& sp : species) output->write_particle_data(ts, *sp);
        if (ts % write_interval == 0) {
          output->storeKE_to_matrix(ts, species, *species[norm]);
          if (write_flag == 1 || write_flag == 2) {
            output->write_field_data(ts);
            output->write_den_data(ts, *species[0]);
            if (nsp > 1) output->write_den_data(ts, *species[1]);
          }
        }
      }
      const bool diag = write_diag > 0 && ts % write_diag == 0;
      const bool store = !energy_path.empty() && write_interval > 0 && ts % write_interval == 0;
      if (!diag && !store) continue;
      double ke_tot = 0;
      std::vector<std::array<double, 3>> kes;
      for (auto& sp : species) {
        kes.push_back(sp->Compute_KE(*species[norm]));
        ke_tot += kes.back()[0] + kes.back()[1] + kes.back()[2];
      }
      const double pe = domain.Compute_PE(norm);
      if (store) {
        energy << ts * cfg.DT;
        for (auto& k : kes) energy << "," << k[0] << "," << k[1] << "," << k[2];
        energy << "," << pe << "\n";
      }
      if (!diag || quiet) continue;
      std::array<double, 3> mom{0, 0, 0};
      for (auto& sp : species) {
        auto p = sp->Compute_Momentum(*species[norm]);
        for (int c = 0; c < 3; c++) mom[c] += p[c];
      }
      std::cout << "TS: " << ts << "\t" << "norm: " << domain.error << " delta_phi: " << std::fixed
                << std::setprecision(2) << domain.delta_phi();
      if (cfg.bc == EPIC_OPEN)
        for (auto& sp : species) std::cout << " n_" << std::setw(4) << sp->name << ":" << sp->size();
      if (cfg.bc == EPIC_PBC)
        for (size_t s = 0; s < species.size(); s++)
          std::cout << " KE_" << std::setw(4) << species[s]->name << ": " << std::fixed << std::setprecision(precision)
                    << kes[s][0] + kes[s][1] + kes[s][2];
      std::cout << " Potential_energy: " << std::fixed << std::setprecision(precision) << pe;
      std::cout << " Kinetic_energy: " << ke_tot;
      std::cout << " Total_energy: " << ke_tot + pe;
      if (cfg.bc == EPIC_PBC)
        std::cout << " p_x: " << mom[0] << " p_y: " << mom[1] << " p_z: " << mom[2];
      std::cout << std::endl;
      std::cout.unsetf(std::ios_base::floatfield);
    }
    auto t1 = std::chrono::steady_clock::now();
    if (output) output->write_ke();
    double sec = std::chrono::duration<double>(t1 - t0).count();
    int64_t total = 0;
    for (auto& sp : species) total += sp->size();
    std::cout << "Elapsed time: " << sec << " seconds; " << (num_ts + 1) << " steps, " << total
              << " particles, " << (double)total * (num_ts + 1) / sec << " particle-steps/s" << std::endl;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return 1;
  }
  return 0;
}
