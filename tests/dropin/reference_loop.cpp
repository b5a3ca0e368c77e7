// A main in the reference's own style, compiled against epic2d.hpp: the
// set-up sequence of the reference's src/main.cpp (INIParser::parse, the
// normalisation, Domain(x0, x0, dx, dy, nx, ny) and its member assignments,
// set_normparam / set_time / set_normscheme, Species(...) per [species] line,
// Create_Grid per [Grids] entry, Emitter per [Emitters] entry) and its loop
// (Init per species, FieldSolve(domain, grids), scatter / ComputeRho /
// PotentialSolver / CalculateEfield / Rewind_species, CollisionHandler, then
// NUM_TS + 1 iterations of inject / scatter / ComputeRho / PotentialSolver /
// CalculateEfield / Push_species_serial(1, grids) / handle_collisions), with
// the reference's classes, constructors and method signatures.  Output is
// left out; at the end every species' particles and phi are written as raw
// doubles for the test to compare.
//
//   reference_loop input.ini out_prefix [steps]
#include <cmath>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "epic2d.hpp"

using namespace epic2d;

static bool string_to_bool(const std::string& s) {
  return s == "true" || s == "True" || s == "T" || s == "t" || s == "1" || s == "yes" || s == "Yes" || s == "Y" ||
         s == "y";
}

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  try {
    auto iniData = INIParser::parse(argv[1]);
    const auto& sim = iniData.at("simulation");
    const auto& dom = iniData.at("domain");
    const auto& norm = iniData.at("normalization");
    const auto& solver = iniData.at("solver");
    const auto& coll = iniData.at("collision");
    const auto& tim = iniData.at("time");
    const auto& diag = iniData.at("diagnostics");
    const int Nx = INIParser::getInt(dom, "Nx"), Ny = INIParser::getInt(dom, "Ny");
    const double x0 = INIParser::getDouble(dom, "x0");
    int NUM_TS = INIParser::getInt(tim, "NUM_TS");
    if (argc > 3) NUM_TS = std::stoi(argv[3]);
    const double DT_coeff = INIParser::getDouble(tim, "DT_coeff");
    const double den = INIParser::getDouble(sim, "density");
    const int norm_scheme = INIParser::getInt(norm, "norm_scheme");
    const double lenght_scale = INIParser::getDouble(norm, "lenght_scale");
    const std::string time_scale_s = INIParser::getString(norm, "time_scale");

    // [species] lines: name, mass, number, temperature, charge sign, fraction, vsx, vsy, load type
    std::vector<std::string> names, loads;
    std::vector<double> mass, temps, frac, vsx, vsy;
    std::vector<int> npart, sign;
    const auto& spsec = iniData.at("species");
    for (size_t k = 0; k < spsec.size(); k++) {
      auto t = INIParser::split(spsec.at(std::to_string(k)), ',');
      if (t.size() != 9) continue;
      names.push_back(t[0]);
      mass.push_back(std::stod(t[1]));
      npart.push_back(std::stoi(t[2]));
      temps.push_back(std::stod(t[3]));
      sign.push_back(std::stoi(t[4]));
      frac.push_back(std::stod(t[5]));
      vsx.push_back(std::stod(t[6]));
      vsy.push_back(std::stod(t[7]));
      loads.push_back(t[8]);
    }
    const int species_no = (int)names.size();
    double k = 0;
    for (int i = 0; i < species_no; i++) k += (-sign[i]) * frac[i];
    std::vector<double> normden(species_no, 0.0);
    normden[1] = den;
    normden[0] = den / k;
    for (int i = 2; i < species_no; i++) normden[i] = frac[i] * normden[0];
    const double LDe = std::sqrt((Const::EPS_0 * Const::K_b * temps[0] * Const::EV_to_K) / (normden[0] * Const::QE * Const::QE));
    const double wpe = std::sqrt((normden[0] * Const::QE * Const::QE) / (mass[0] * Const::EPS_0));
    const double wpi = std::sqrt((normden[1] * Const::QE * Const::QE) / (mass[1] * Const::EPS_0));
    const double LDi = std::sqrt((Const::EPS_0 * Const::K_b * temps[1] * Const::EV_to_K) / (normden[1] * Const::QE * Const::QE));
    double time_scale = time_scale_s == "omegape" ? wpe : time_scale_s == "omegapi" ? wpi : std::stod(time_scale_s);
    double dx = 0, dy = 0, DT = 0, stepSize;
    if (norm_scheme == 2 || norm_scheme == 4) {
      stepSize = LDi; dx = stepSize / LDi; dy = stepSize / LDi;
      DT = DT_coeff * (1.0 / wpi); DT = wpi * DT;
    }
    if (norm_scheme == 1 || norm_scheme == 3) {
      stepSize = LDe; dx = stepSize / LDe; dy = stepSize / LDe;
      DT = DT_coeff * (1.0 / wpe); DT = wpe * DT;
    }
    if (norm_scheme == 5) {
      stepSize = lenght_scale; dx = stepSize / lenght_scale; dy = stepSize / lenght_scale;
      DT = DT_coeff * (1.0 / time_scale); DT = time_scale * DT;
    }

    Domain domain(x0, x0, dx, dy, Nx + 1, Ny + 1);
    domain.bc = INIParser::getString(sim, "bc");
    domain.SolverType = INIParser::getString(solver, "solvertype");
    domain.tolerance = INIParser::getDouble(solver, "tolerance");
    domain.species_no = species_no;
    domain.density = den;
    domain.shapefunction = INIParser::getString(sim, "shapefunction");
    domain.max_iteration = INIParser::getInt(solver, "max_iteration");
    domain.normscheme = norm_scheme;
    domain.sub_cycle_interval = INIParser::getInt(diag, "sub_cycle_interval");
    domain.lenght_scale = lenght_scale;
    domain.time_scale = time_scale;
    domain.set_normparam(LDe, wpe, LDi, wpi);
    domain.set_time(DT, NUM_TS, INIParser::getInt(diag, "write_interval"),
                    INIParser::getInt(diag, "write_interval_phase"));
    domain.set_normscheme();
    domain.ionfixed = INIParser::getInt(sim, "ionfixed");
    domain.enable_elastic_collision = string_to_bool(INIParser::getString(coll, "elastic"));
    domain.enable_excitation_collision = string_to_bool(INIParser::getString(coll, "excitation"));
    domain.enable_ionization_collision = string_to_bool(INIParser::getString(coll, "ionization"));
    domain.GAS_DENSITY = INIParser::getDouble(coll, "GAS_DENSITY");

    std::vector<Species> species_list;
    species_list.reserve(species_no);
    for (int i = 0; i < species_no; i++) {
      const double computed_spwt = normden[i] * domain.Lx * domain.Ly * domain.L * domain.L / npart[i];
      species_list.emplace_back(names[i], mass[i], sign[i] * Const::QE, computed_spwt, temps[i], npart[i], vsx[i],
                                vsy[i], frac[i], loads[i], domain);
    }

    std::vector<Grid*> grids;
    const auto& gridsSection = iniData.at("Grids");
    const int grid_count = INIParser::getInt(gridsSection, "grid_count");
    for (int i = 0; i < grid_count; i++) {
      const std::string prefix = "grid_" + std::to_string(i) + ".";
      const std::string type = INIParser::getString(gridsSection, prefix + "type");
      GridParams gp{};
      RectangularGridParams rp{};
      const double vs = Const::eV / (Const::K_b * Const::EV_to_K);
      if (type == "circular") {
        gp.grid_centerx = INIParser::getInt(gridsSection, prefix + "x_center");
        gp.grid_centery = INIParser::getInt(gridsSection, prefix + "y_center");
        gp.num_electrodes = INIParser::getInt(gridsSection, prefix + "electrode_number");
        gp.grid_rad = INIParser::getDouble(gridsSection, prefix + "grid_radius");
        gp.electrode_rad = INIParser::getDouble(gridsSection, prefix + "electrod_radius");
        gp.voltage = vs * INIParser::getDouble(gridsSection, prefix + "electrode_voltage");
        grids.push_back(Create_Grid(GridType::Circular, domain, gp, rp));
      } else if (type == "reactconduct") {
        rp.min_x = INIParser::getInt(gridsSection, prefix + "min_x");
        rp.min_y = INIParser::getInt(gridsSection, prefix + "min_y");
        rp.max_x = INIParser::getInt(gridsSection, prefix + "max_x");
        rp.max_y = INIParser::getInt(gridsSection, prefix + "max_y");
        rp.voltage = vs * INIParser::getDouble(gridsSection, prefix + "grid_voltage");
        grids.push_back(Create_Grid(GridType::ReactConductor, domain, gp, rp));
      }
    }

    std::vector<Emitter> emitters;
    const auto& emitterSection = iniData.at("Emitters");
    const int emitter_count = INIParser::getInt(emitterSection, "count");
    for (int i = 0; i < emitter_count; i++) {
      const std::string prefix = "emitter_" + std::to_string(i) + ".";
      EmitterParams params;
      params.x0 = INIParser::getDouble(emitterSection, prefix + "x0");
      params.y0 = INIParser::getDouble(emitterSection, prefix + "y0");
      params.x1 = INIParser::getDouble(emitterSection, prefix + "x1");
      params.y1 = INIParser::getDouble(emitterSection, prefix + "y1");
      params.temp = INIParser::getDouble(emitterSection, prefix + "temp");
      params.numparticle = INIParser::getInt(emitterSection, prefix + "numparticle");
      params.vdx = INIParser::getDouble(emitterSection, prefix + "vdx");
      params.vdy = INIParser::getDouble(emitterSection, prefix + "vdy");
      params.species_idx1 = INIParser::getInt(emitterSection, prefix + "species_idx1");
      params.species_idx2 = INIParser::getInt(emitterSection, prefix + "species_idx2");
      emitters.emplace_back(params, domain);
    }

    // --- the loop of the reference's main, call for call ---
    for (Species& sp : species_list) {
      Init init(sp, domain, grids);
    }
    FieldSolve fieldsolver(domain, grids);
    for (Species& sp : species_list) sp.ScatterSpecies_serial();
    domain.ComputeRho(species_list);
    fieldsolver.PotentialSolver();
    fieldsolver.CalculateEfield();
    for (Species& sp : species_list) sp.Rewind_species();
    CollisionHandler testcoll(domain);
    testcoll.set_electron_cross_sections();
    testcoll.calc_total_cross_sections();
    const bool collide = domain.enable_elastic_collision || domain.enable_excitation_collision ||
                         domain.enable_ionization_collision;
    for (int ts = 0; ts < NUM_TS + 1; ts++) {
      for (auto& emit : emitters) emit.inject(species_list);
      for (Species& sp : species_list) sp.ScatterSpecies_serial();
      domain.ComputeRho(species_list);
      fieldsolver.PotentialSolver();
      fieldsolver.CalculateEfield();
      for (Species& sp : species_list) {
        if (sp.name == "ion" && domain.ionfixed == 1) continue;
        sp.Push_species_serial(1, grids);
      }
      if (collide) testcoll.handle_collisions(species_list[0], species_list[1]);
    }

    const std::string out = argv[2];
    for (int s = 0; s < species_no; s++) {
      const std::vector<double> p = species_list[(size_t)s].particles();
      std::ofstream f(out + "_part" + std::to_string(s) + ".bin", std::ios::binary);
      f.write(reinterpret_cast<const char*>(p.data()), (std::streamsize)(p.size() * sizeof(double)));
    }
    const std::vector<double> phi = domain.phi();
    std::ofstream f(out + "_phi.bin", std::ios::binary);
    f.write(reinterpret_cast<const char*>(phi.data()), (std::streamsize)(phi.size() * sizeof(double)));
    for (Grid* g : grids) delete g;
    std::printf("steps %d species %d\n", NUM_TS + 1, species_no);
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
    return 1;
  }
  return 0;
}
