// ORACLE TEST INFRASTRUCTURE — not part of the product.
//
// Drives the reference's own physics objects (src/domain.cpp, species.cpp,
// field.cpp, collision.cpp, cross_section.cpp, init.cpp, grid.cpp,
// electrode.cpp, iniparser.cpp, emitter.cpp — compiled from where they lie, by
// oracle/build_oracle.py) behind a small extern "C" surface so the tests can
// run the unmodified reference step by step and read back its arrays.
//
// The set-up sequence restates src/main.cpp:34-261 and :359-393 (INI parsing,
// normalisation, Domain/Species construction, particle loading, the initial
// field and the leapfrog rewind); HDF5 output, plotting and the std::cin wait
// are left out.  The loop body restates src/main.cpp:405-423.
#include "iniparser.h"
#include "field.h"
#include "init.h"
#include "domain.h"
#include "species.h"
#include "collision.h"
#include "grid.h"
#include "emitter.h"
#include "extrafun.h"

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct RefSim {
  Domain* domain = nullptr;
  std::vector<Species> species;
  std::vector<Grid*> grids;
  std::vector<Emitter> emitters;
  FieldSolve* fs = nullptr;
  CollisionHandler* coll = nullptr;
  double params[32];
  std::string error;
};

}  // namespace

extern "C" {

// Restart the reference's global mt19937 (seed 0, include/domain.h:223) so that
// every simulation built in one process sees the same stream as a fresh run.
void ref_reset_rng() { rnd = Rnd(); }

double ref_rnd() { return rnd(); }

// Build a simulation from an input.ini exactly as src/main.cpp does up to the
// first loop iteration.  load_particles=0 skips Init (particles then come from
// ref_set_particles); initial_field=0 skips the scatter/solve/rewind prologue.
void* ref_create(const char* ini_path, int load_particles, int initial_field) {
  RefSim* s = new RefSim();
  try {
    auto iniData = INIParser::parse(ini_path);
    auto species_section = iniData["species"];
    int species_no = species_section.size();
    int Nx = INIParser::getInt(iniData["domain"], "Nx");
    int Ny = INIParser::getInt(iniData["domain"], "Ny");
    int nx = Nx + 1, ny = Ny + 1;
    double x0 = INIParser::getDouble(iniData["domain"], "x0");
    std::string elastic_flag = INIParser::getString(iniData["collision"], "elastic");
    std::string excitation_flag = INIParser::getString(iniData["collision"], "excitation");
    std::string ionization_flag = INIParser::getString(iniData["collision"], "ionization");
    double GAS_DENSITY = INIParser::getDouble(iniData["collision"], "GAS_DENSITY");
    int NUM_TS = INIParser::getInt(iniData["time"], "NUM_TS");
    double DT_coeff = INIParser::getDouble(iniData["time"], "DT_coeff");
    std::string shapefunction = INIParser::getString(iniData["simulation"], "shapefunction");
    double den = INIParser::getDouble(iniData["simulation"], "density");
    std::string bc = INIParser::getString(iniData["simulation"], "bc");
    int ionfixed = INIParser::getInt(iniData["simulation"], "ionfixed");
    int write_interval = INIParser::getInt(iniData["diagnostics"], "write_interval");
    int write_interval_phase = INIParser::getInt(iniData["diagnostics"], "write_interval_phase");
    int sub_cycle_interval = INIParser::getInt(iniData["diagnostics"], "sub_cycle_interval");
    int norm_scheme = INIParser::getInt(iniData["normalization"], "norm_scheme");
    double L_scale = INIParser::getDouble(iniData["normalization"], "lenght_scale");
    std::string T_scale = INIParser::getString(iniData["normalization"], "time_scale");
    std::string SolverType = INIParser::getString(iniData["solver"], "solvertype");
    double tolerance = INIParser::getDouble(iniData["solver"], "tolerance");
    double max_iteration = INIParser::getInt(iniData["solver"], "max_iteration");

    std::vector<std::string> names, pos_init;
    std::vector<double> mass, temps, frac, vsx, vsy;
    std::vector<int> nP, sign;
    for (const auto& e : species_section) {
      auto t = INIParser::split(e.second, ',');
      if (t.size() == 9) {
        names.push_back(t[0]);
        mass.push_back(std::stod(t[1]));
        nP.push_back(std::stoi(t[2]));
        temps.push_back(std::stod(t[3]));
        sign.push_back(std::stoi(t[4]));
        frac.push_back(std::stod(t[5]));
        vsx.push_back(std::stod(t[6]));
        vsy.push_back(std::stod(t[7]));
        pos_init.push_back(t[8]);
      }
    }
    std::vector<double> normden(species_no, 0.0);
    double k = 0;
    for (int i = 0; i < species_no; i++) k += (-sign[i]) * frac[i];
    normden[1] = den;
    normden[0] = den / k;
    for (int i = 2; i < species_no; i++) normden[i] = frac[i] * normden[0];

    double LDe = sqrt((Const::EPS_0 * Const::K_b * temps[0] * Const::EV_to_K) / (normden[0] * Const::QE * Const::QE));
    double wpe = sqrt((normden[0] * Const::QE * Const::QE) / (mass[0] * Const::EPS_0));
    double wpi = sqrt((normden[1] * Const::QE * Const::QE) / (mass[1] * Const::EPS_0));
    double LDi = sqrt((Const::EPS_0 * Const::K_b * temps[1] * Const::EV_to_K) / (normden[1] * Const::QE * Const::QE));
    double CS = sqrt(temps[0] * Const::K_b * Const::EV_to_K / mass[1]);
    double time_scale;
    if (T_scale == "omegape") time_scale = wpe;
    else if (T_scale == "omegapi") time_scale = wpi;
    else time_scale = std::stod(T_scale);

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
      stepSize = L_scale; dx = stepSize / L_scale; dy = stepSize / L_scale;
      DT = DT_coeff * (1.0 / time_scale); DT = time_scale * DT;
    }
    Domain* d = new Domain(x0, x0, dx, dy, nx, ny);
    s->domain = d;
    d->bc = bc;
    d->SolverType = SolverType;
    d->tolerance = tolerance;
    d->species_no = species_no;
    d->density = den;
    d->shapefunction = shapefunction;
    d->IAW_vel = CS;
    d->max_iteration = max_iteration;
    d->normscheme = norm_scheme;
    d->sub_cycle_interval = sub_cycle_interval;
    // src/main.cpp never stores vel_norm_scheme into the Domain; any value other
    // than 3 makes Domain::set_normscheme fall through to vel_norm = L*W.
    d->vel_normscheme = 0;
    d->lenght_scale = L_scale;
    d->time_scale = time_scale;
    d->set_normparam(LDe, wpe, LDi, wpi);
    d->set_time(DT, NUM_TS, write_interval, write_interval_phase);
    d->set_normscheme();
    d->ionfixed = ionfixed;
    d->enable_elastic_collision = string_to_bool(elastic_flag);
    d->enable_excitation_collision = string_to_bool(excitation_flag);
    d->enable_ionization_collision = string_to_bool(ionization_flag);
    d->GAS_DENSITY = GAS_DENSITY;
    d->num_threads = 1;

    s->species.reserve(species_no);
    for (int i = 0; i < species_no; i++) {
      double spwt = normden[i] * d->Lx * d->Ly * d->L * d->L / nP[i];
      s->species.emplace_back(names[i], mass[i], sign[i] * Const::QE, spwt, temps[i], nP[i], vsx[i], vsy[i],
                              frac[i], pos_init[i], *d);
    }
    // Conductors as src/main.cpp:284-327 reads them (emitters are not driven here).
    {
      auto& gsec = iniData["Grids"];
      const int grid_count = INIParser::getInt(gsec, "grid_count");
      const double vscale = Const::eV / (Const::K_b * Const::EV_to_K);
      for (int g = 0; g < grid_count; g++) {
        const std::string pre = "grid_" + std::to_string(g) + ".";
        const std::string type = INIParser::getString(gsec, pre + "type");
        GridParams cp;
        RectangularGridParams rp;
        if (type == "circular") {
          cp.grid_centerx = INIParser::getInt(gsec, pre + "x_center");
          cp.grid_centery = INIParser::getInt(gsec, pre + "y_center");
          cp.num_electrodes = INIParser::getInt(gsec, pre + "electrode_number");
          cp.grid_rad = INIParser::getDouble(gsec, pre + "grid_radius");
          cp.electrode_rad = INIParser::getDouble(gsec, pre + "electrod_radius");
          cp.voltage = vscale * INIParser::getDouble(gsec, pre + "electrode_voltage");
          s->grids.push_back(Create_Grid(GridType::Circular, *d, cp, rp));
        } else if (type == "reactconduct") {
          rp.min_x = INIParser::getInt(gsec, pre + "min_x");
          rp.min_y = INIParser::getInt(gsec, pre + "min_y");
          rp.max_x = INIParser::getInt(gsec, pre + "max_x");
          rp.max_y = INIParser::getInt(gsec, pre + "max_y");
          rp.voltage = vscale * INIParser::getDouble(gsec, pre + "grid_voltage");
          s->grids.push_back(Create_Grid(GridType::ReactConductor, *d, cp, rp));
        }
      }
    }
    // Emitters as src/main.cpp:330-355 reads them.
    {
      auto& esec = iniData["Emitters"];
      const int count = INIParser::getInt(esec, "count");
      for (int e = 0; e < count; e++) {
        const std::string pre = "emitter_" + std::to_string(e) + ".";
        EmitterParams ep;
        ep.x0 = INIParser::getDouble(esec, pre + "x0");
        ep.y0 = INIParser::getDouble(esec, pre + "y0");
        ep.x1 = INIParser::getDouble(esec, pre + "x1");
        ep.y1 = INIParser::getDouble(esec, pre + "y1");
        ep.temp = INIParser::getDouble(esec, pre + "temp");
        ep.numparticle = INIParser::getInt(esec, pre + "numparticle");
        ep.vdx = INIParser::getDouble(esec, pre + "vdx");
        ep.vdy = INIParser::getDouble(esec, pre + "vdy");
        ep.species_idx1 = INIParser::getInt(esec, pre + "species_idx1");
        ep.species_idx2 = INIParser::getInt(esec, pre + "species_idx2");
        s->emitters.emplace_back(ep, *d);
      }
    }
    if (load_particles) {
      for (Species& sp : s->species) Init init(sp, *d, s->grids);
    }
    s->fs = new FieldSolve(*d, s->grids);
    if (initial_field) {
      for (Species& sp : s->species) sp.ScatterSpecies_serial();
      d->ComputeRho(s->species);
      s->fs->PotentialSolver();
      s->fs->CalculateEfield();
      for (Species& sp : s->species) sp.Rewind_species();
    }
    double* p = s->params;
    p[0] = d->nx; p[1] = d->ny; p[2] = d->x0; p[3] = d->y0; p[4] = d->dx; p[5] = d->dy;
    p[6] = d->Lx; p[7] = d->Ly; p[8] = d->DT; p[9] = d->L; p[10] = d->W; p[11] = d->vel_norm;
    p[12] = d->LDe; p[13] = d->wpe; p[14] = d->LDi; p[15] = d->wpi; p[16] = d->density;
    p[17] = species_no; p[18] = CS; p[19] = NUM_TS;
  } catch (const std::exception& e) {
    s->error = e.what();
  }
  return s;
}

const char* ref_error(void* h) { return static_cast<RefSim*>(h)->error.c_str(); }

void ref_destroy(void* h) {
  RefSim* s = static_cast<RefSim*>(h);
  delete s->coll;
  delete s->fs;
  for (Grid* g : s->grids) delete g;
  s->species.clear();
  delete s->domain;
  delete s;
}

// nx, ny, x0, y0, dx, dy, Lx, Ly, DT, L, W, vel_norm, LDe, wpe, LDi, wpi, density,
// species_no, ion acoustic speed, NUM_TS
void ref_params(void* h, double* out) { std::memcpy(out, static_cast<RefSim*>(h)->params, 20 * sizeof(double)); }

// mass, charge, spwt, temp, numparticle, vsx, vsy, fract_den
void ref_species_params(void* h, int sp, double* out) {
  Species& s = static_cast<RefSim*>(h)->species[sp];
  out[0] = s.mass; out[1] = s.charge; out[2] = s.spwt; out[3] = s.temp;
  out[4] = s.numparticle; out[5] = s.vsx; out[6] = s.vsy; out[7] = s.fract_den;
}

long ref_num_particles(void* h, int sp) { return (long)static_cast<RefSim*>(h)->species[sp].part_list.size(); }

void ref_get_particles(void* h, int sp, double* out) {
  auto& pl = static_cast<RefSim*>(h)->species[sp].part_list;
  for (size_t i = 0; i < pl.size(); i++) {
    out[5 * i + 0] = pl[i].pos[0]; out[5 * i + 1] = pl[i].pos[1];
    out[5 * i + 2] = pl[i].vel[0]; out[5 * i + 3] = pl[i].vel[1]; out[5 * i + 4] = pl[i].vel[2];
  }
}

void ref_set_particles(void* h, int sp, const double* in, long n) {
  auto& pl = static_cast<RefSim*>(h)->species[sp].part_list;
  pl.clear();
  pl.reserve(n + 1024);
  for (long i = 0; i < n; i++) pl.emplace_back(in[5 * i], in[5 * i + 1], in[5 * i + 2], in[5 * i + 3], in[5 * i + 4]);
}

// which: 0 phi, 1 rho, 2 efx, 3 efy, 10+s den of species s.  Row-major (i*ny + j).
static Matrix<double>& grid_ref(RefSim* s, int which) {
  Domain* d = s->domain;
  switch (which) {
    case 0: return d->phi;
    case 1: return d->rho;
    case 2: return d->efx;
    case 3: return d->efy;
    default: return s->species[which - 10].den;
  }
}

void ref_get_grid(void* h, int which, double* out) {
  RefSim* s = static_cast<RefSim*>(h);
  Matrix<double>& m = grid_ref(s, which);
  int nx = s->domain->nx, ny = s->domain->ny;
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) out[i * ny + j] = m(i, j);
}

void ref_set_grid(void* h, int which, const double* in) {
  RefSim* s = static_cast<RefSim*>(h);
  Matrix<double>& m = grid_ref(s, which);
  int nx = s->domain->nx, ny = s->domain->ny;
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++) m(i, j) = in[i * ny + j];
}

#define GUARD(body)                                      \
  try {                                                  \
    body;                                                \
    return 0;                                            \
  } catch (const std::exception& e) {                    \
    static_cast<RefSim*>(h)->error = e.what();           \
    return -1;                                           \
  }

// Calls that can throw (std::out_of_range from Matrix::operator()) return -1
// and leave the message in ref_error instead of unwinding through the FFI.
int ref_scatter(void* h, int sp) { GUARD(static_cast<RefSim*>(h)->species[sp].ScatterSpecies_serial()) }
void ref_compute_rho(void* h) { RefSim* s = static_cast<RefSim*>(h); s->domain->ComputeRho(s->species); }
int ref_solve(void* h) { GUARD(static_cast<RefSim*>(h)->fs->PotentialSolver()) }
double ref_solver_error(void* h) { return static_cast<RefSim*>(h)->domain->error; }
void ref_efield(void* h) { static_cast<RefSim*>(h)->fs->CalculateEfield(); }
int ref_push(void* h, int sp, int sub_cycle) {
  RefSim* s = static_cast<RefSim*>(h);
  GUARD(s->species[sp].Push_species_serial(sub_cycle, s->grids))
}
int ref_rewind(void* h, int sp) { GUARD(static_cast<RefSim*>(h)->species[sp].Rewind_species()) }

static void ensure_coll(RefSim* s) {
  if (!s->coll) {
    s->coll = new CollisionHandler(*s->domain);
    s->coll->set_electron_cross_sections();
    s->coll->calc_total_cross_sections();
  }
}

void ref_init_collisions(void* h) { ensure_coll(static_cast<RefSim*>(h)); }

static void collide_impl(void* h) {
  RefSim* s = static_cast<RefSim*>(h);
  ensure_coll(s);
  // Ionisation appends to the vector being iterated (src/collision.cpp:163-164
  // inside the range-for at :192); spare capacity keeps the iteration defined.
  s->species[0].part_list.reserve(s->species[0].part_list.size() * 2 + 1024);
  s->species[1].part_list.reserve(s->species[1].part_list.size() * 2 + 1024);
  s->coll->handle_collisions(s->species[0], s->species[1]);
}

int ref_collide(void* h) { GUARD(collide_impl(h)) }

// One iteration of the loop body of src/main.cpp:405-423 (no emitters).
static void step_impl(void* h, int with_collisions) {
  RefSim* s = static_cast<RefSim*>(h);
  for (Emitter& e : s->emitters) e.inject(s->species);  // src/main.cpp:397-403
  for (Species& sp : s->species) sp.ScatterSpecies_serial();
  s->domain->ComputeRho(s->species);
  s->fs->PotentialSolver();
  s->fs->CalculateEfield();
  for (Species& sp : s->species) {
    if (sp.name == "ion" && s->domain->ionfixed == 1) continue;
    sp.Push_species_serial(1, s->grids);
  }
  if (with_collisions) collide_impl(h);
}

int ref_step(void* h, int with_collisions) { GUARD(step_impl(h, with_collisions)) }
static void inject_impl(void* h) {
  RefSim* s = static_cast<RefSim*>(h);
  for (Emitter& e : s->emitters) e.inject(s->species);
}
int ref_inject(void* h) { GUARD(inject_impl(h)) }

void ref_ke(void* h, int sp, int norm_sp, double* out3) {
  RefSim* s = static_cast<RefSim*>(h);
  vec<double> ke = s->species[sp].Compute_KE(s->species[norm_sp]);
  out3[0] = ke(0); out3[1] = ke(1); out3[2] = ke(2);
}

void ref_momentum(void* h, int sp, int norm_sp, double* out3) {
  RefSim* s = static_cast<RefSim*>(h);
  vec<double> p = s->species[sp].Compute_Momentum(s->species[norm_sp]);
  out3[0] = p(0); out3[1] = p(1); out3[2] = p(2);
}

double ref_pe(void* h, int norm_sp) {
  RefSim* s = static_cast<RefSim*>(h);
  return s->domain->Compute_PE(s->species[norm_sp]);
}

}  // extern "C"
