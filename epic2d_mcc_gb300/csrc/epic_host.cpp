// Host-side start-up of the C ABI: input.ini parsing and normalisation, the
// particle loader, and the e-/Ar cross-section tables.  These run once per
// simulation on the host, as they do in the reference; the time-step loop is
// entirely on the GPU.
//
// Compiled with -ffp-contract=off so that aarch64 hosts round every
// multiply-add as the reference does on x86.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "epic_host.h"

namespace epic {

namespace {

using Section = std::map<std::string, std::string>;
using Ini = std::map<std::string, Section>;

void trim(std::string& s) {
  size_t a = s.find_first_not_of(" \t");
  size_t b = s.find_last_not_of(" \t");
  if (a == std::string::npos) s.clear();
  else s = s.substr(a, b - a + 1);
}

// INIParser::parse (src/iniparser.cpp:4-49): [section] headers, key = value
// lines, ';'/'#' comment lines; [species] lines are stored whole under the
// keys "0", "1", ... in file order.
bool parse_ini(const char* path, Ini& out, std::string& err) {
  std::ifstream f(path);
  if (!f.is_open()) {
    err = std::string("Error opening file: ") + path;
    return false;
  }
  std::string line, cur;
  while (std::getline(f, line)) {
    if (line.empty() || line[0] == ';' || line[0] == '#') continue;
    if (line[0] == '[' && line[line.size() - 1] == ']') {
      cur = line.substr(1, line.size() - 2);
      continue;
    }
    if (cur == "species") {
      Section& s = out[cur];
      s[std::to_string(s.size())] = line;
    } else {
      std::istringstream iss(line);
      std::string k, v;
      if (std::getline(iss, k, '=') && std::getline(iss, v)) {
        trim(k);
        trim(v);
        out[cur][k] = v;
      }
    }
  }
  return true;
}

const std::string& need(const Ini& ini, const char* sec, const char* key) {
  auto s = ini.find(sec);
  if (s == ini.end()) throw std::out_of_range(std::string("missing section [") + sec + "]");
  auto k = s->second.find(key);
  if (k == s->second.end()) throw std::out_of_range(std::string("missing key ") + key + " in [" + sec + "]");
  return k->second;
}

const std::string* opt(const Ini& ini, const char* sec, const char* key) {
  auto s = ini.find(sec);
  if (s == ini.end()) return nullptr;
  auto k = s->second.find(key);
  return k == s->second.end() ? nullptr : &k->second;
}

std::vector<std::string> split(const std::string& str, char d) {
  std::vector<std::string> t;
  std::string tok;
  std::istringstream ts(str);
  while (std::getline(ts, tok, d)) t.push_back(tok);
  return t;
}

bool to_bool(const std::string& s) {  // include/extrafun.h:6-17
  return s == "true" || s == "True" || s == "T" || s == "t" || s == "1" || s == "yes" || s == "Yes" || s == "Y" ||
         s == "y";
}

}  // namespace

int ini_get(const char* path, const char* section, const char* key, std::string& value, std::string& err) {
  Ini ini;
  if (!parse_ini(path, ini, err)) return EPIC_ERR_IO;
  auto s = ini.find(section);
  if (s == ini.end() || s->second.find(key) == s->second.end()) {
    err = std::string("missing key ") + key + " in [" + section + "]";
    return EPIC_ERR_INVALID;
  }
  value = s->second.at(key);
  return EPIC_OK;
}

// src/main.cpp:42-261 and Domain::set_normscheme (src/domain.cpp:123-183),
// same operation order.  vel_norm is always L*W: main() never stores
// vel_norm_scheme into the Domain, and set_normscheme keeps another value only
// for vel_normscheme == 3.
int config_from_ini(const char* path, epic_config* cfg, epic_species_desc* sp, int max_sp, int* nsp, int* num_ts,
                    std::string& err) {
  Ini ini;
  if (!parse_ini(path, ini, err)) return EPIC_ERR_IO;
  try {
    epic_config_defaults(cfg);
    const Section& species = ini["species"];
    int Nx = std::stoi(need(ini, "domain", "Nx"));
    int Ny = std::stoi(need(ini, "domain", "Ny"));
    double x0 = std::stod(need(ini, "domain", "x0"));
    std::string el = need(ini, "collision", "elastic"), ex = need(ini, "collision", "excitation"),
                io = need(ini, "collision", "ionization");
    double gas = std::stod(need(ini, "collision", "GAS_DENSITY"));
    int NUM_TS = std::stoi(need(ini, "time", "NUM_TS"));
    double DT_coeff = std::stod(need(ini, "time", "DT_coeff"));
    std::string shape = need(ini, "simulation", "shapefunction");
    double den = std::stod(need(ini, "simulation", "density"));
    std::string bc = need(ini, "simulation", "bc");
    int ionfixed = std::stoi(need(ini, "simulation", "ionfixed"));
    int norm_scheme = std::stoi(need(ini, "normalization", "norm_scheme"));
    double L_scale = std::stod(need(ini, "normalization", "lenght_scale"));
    std::string T_scale = need(ini, "normalization", "time_scale");
    std::string solver = need(ini, "solver", "solvertype");
    double tol = std::stod(need(ini, "solver", "tolerance"));
    int max_it = std::stoi(need(ini, "solver", "max_iteration"));

    std::vector<epic_species_desc> d;
    std::vector<int> sign;
    for (size_t i = 0; i < species.size(); i++) {
      auto it = species.find(std::to_string(i));
      if (it == species.end()) continue;
      auto t = split(it->second, ',');
      if (t.size() != 9) continue;
      epic_species_desc s;
      std::memset(&s, 0, sizeof(s));
      std::snprintf(s.name, sizeof(s.name), "%s", t[0].c_str());
      s.mass = std::stod(t[1]);
      s.numparticle = std::stoi(t[2]);
      s.temp = std::stod(t[3]);
      sign.push_back(std::stoi(t[4]));
      s.fract_den = std::stod(t[5]);
      s.vsx = std::stod(t[6]);
      s.vsy = std::stod(t[7]);
      std::snprintf(s.load, sizeof(s.load), "%s", t[8].c_str());
      d.push_back(s);
    }
    int n = (int)d.size();
    if (n < 2) throw std::invalid_argument("input needs at least two species (electrons first, ions second)");
    double k = 0;
    for (int i = 0; i < n; i++) k += (-sign[i]) * d[i].fract_den;
    std::vector<double> normden(n, 0.0);
    normden[1] = den;
    normden[0] = den / k;
    for (int i = 2; i < n; i++) normden[i] = d[i].fract_den * normden[0];
    const double EV_to_K = QE_H / K_B_H;
    double LDe = sqrt((EPS_0_H * K_B_H * d[0].temp * EV_to_K) / (normden[0] * QE_H * QE_H));
    double wpe = sqrt((normden[0] * QE_H * QE_H) / (d[0].mass * EPS_0_H));
    double wpi = sqrt((normden[1] * QE_H * QE_H) / (d[1].mass * EPS_0_H));
    double LDi = sqrt((EPS_0_H * K_B_H * d[1].temp * EV_to_K) / (normden[1] * QE_H * QE_H));
    double time_scale;
    if (T_scale == "omegape") time_scale = wpe;
    else if (T_scale == "omegapi") time_scale = wpi;
    else time_scale = std::stod(T_scale);
    double dx = 0, dy = 0, DT = 0, step;
    if (norm_scheme == 2 || norm_scheme == 4) {
      step = LDi; dx = step / LDi; dy = step / LDi;
      DT = DT_coeff * (1.0 / wpi); DT = wpi * DT;
    }
    if (norm_scheme == 1 || norm_scheme == 3) {
      step = LDe; dx = step / LDe; dy = step / LDe;
      DT = DT_coeff * (1.0 / wpe); DT = wpe * DT;
    }
    if (norm_scheme == 5) {
      step = L_scale; dx = step / L_scale; dy = step / L_scale;
      DT = DT_coeff * (1.0 / time_scale); DT = time_scale * DT;
    }
    double L, W;
    if (norm_scheme == 1 || norm_scheme == 3) { L = LDe; W = wpe; }
    else if (norm_scheme == 2 || norm_scheme == 4) { L = LDi; W = norm_scheme == 2 ? wpi : wpe; }
    else if (norm_scheme == 5) { L = L_scale; W = time_scale; LDe = L; wpe = W; }
    else throw std::invalid_argument("Invalid normscheme flag");
    cfg->nx = Nx + 1;
    cfg->ny = Ny + 1;
    cfg->x0 = x0;
    cfg->y0 = x0;  // Domain(x0, x0, ...) in src/main.cpp:226
    cfg->dx = dx;
    cfg->dy = dy;
    cfg->DT = DT;
    cfg->L = L;
    cfg->W = W;
    cfg->vel_norm = L * W;
    cfg->LDe = LDe;
    cfg->wpe = wpe;
    cfg->LDi = LDi;
    cfg->wpi = wpi;
    cfg->density = den;
    if (shape == "CIC") cfg->shape = EPIC_CIC;
    else if (shape == "NGP") cfg->shape = EPIC_NGP;
    else throw std::invalid_argument("shapefunction must be CIC or NGP");
    if (bc == "pbc") cfg->bc = EPIC_PBC;
    else if (bc == "open") cfg->bc = EPIC_OPEN;
    else if (bc == "reflective") cfg->bc = EPIC_REFLECTIVE;
    else throw std::invalid_argument("bc must be pbc, open or reflective");
    if (solver == "gs") cfg->solver = EPIC_SOLVER_GS;
    else if (solver == "cg" || solver == "iter" || solver == "iterative") cfg->solver = EPIC_SOLVER_PCG;
    else if (solver == "gshybrid") cfg->solver = EPIC_SOLVER_GSHYBRID;
    else if (solver == "hybrid") cfg->solver = EPIC_SOLVER_HYBRID;
    else
      throw std::invalid_argument("solvertype " + solver +
                                  " is not supported (gs, cg, iter, iterative, gshybrid, hybrid)");
    cfg->tolerance = tol;
    cfg->max_iteration = max_it;
    cfg->ionfixed = ionfixed;
    cfg->normscheme = norm_scheme;
    cfg->gas_density = gas;
    cfg->elastic = to_bool(el);
    cfg->excitation = to_bool(ex);
    cfg->ionization = to_bool(io);
    // Options with no reference counterpart (defaults keep reference behaviour).
    if (auto v = opt(ini, "solver", "sor_omega")) cfg->sor_omega = std::stod(*v);
    if (auto v = opt(ini, "solver", "sor_mode")) cfg->sor_mode = *v == "redblack" ? EPIC_SOR_REDBLACK : EPIC_SOR_LEXICOGRAPHIC;
    if (auto v = opt(ini, "solver", "warm_start")) cfg->warm_start = to_bool(*v);
    if (auto v = opt(ini, "solver", "poisson_bc")) {
      if (*v == "dirichlet") cfg->poisson_bc = EPIC_POISSON_DIRICHLET;
      else if (*v == "periodic") cfg->poisson_bc = EPIC_POISSON_PERIODIC;
      else if (*v == "dirichlet_x") cfg->poisson_bc = EPIC_POISSON_DIRICHLET_X;
      else throw std::invalid_argument("poisson_bc " + *v + " is not supported (dirichlet, periodic, dirichlet_x)");
    }
    if (auto v = opt(ini, "simulation", "load_3v")) cfg->load_3v = to_bool(*v);
    if (auto v = opt(ini, "simulation", "deposit_mode")) cfg->deposit_mode = *v == "fp64" ? EPIC_DEPOSIT_FP64 : EPIC_DEPOSIT_FIXED;
    if (auto v = opt(ini, "simulation", "arithmetic"))
      cfg->precision = *v == "mixed" ? EPIC_PRECISION_MIXED : EPIC_PRECISION_FP64;
    // Cell sort: off for the FP64 form (keeps the reference's particle order),
    // every 16 steps for the mixed form unless the deck says otherwise.
    if (cfg->precision == EPIC_PRECISION_MIXED) cfg->sort_every = 16;
    if (auto v = opt(ini, "simulation", "sort_every")) cfg->sort_every = std::stoi(*v);
    if (auto v = opt(ini, "simulation", "push_order")) {
      if (*v == "reference") cfg->push_order = EPIC_PUSH_REFERENCE;
      else if (*v == "contracted") cfg->push_order = EPIC_PUSH_CONTRACTED;
      else throw std::invalid_argument("push_order " + *v + " is not supported (contracted, reference)");
    }
    if (auto v = opt(ini, "collision", "mcc_mode"))
      cfg->mcc_mode = *v == "null" ? EPIC_MCC_NULL : (*v == "injected" ? EPIC_MCC_INJECTED : EPIC_MCC_PHILOX);
    if (auto v = opt(ini, "collision", "seed")) cfg->seed = std::stoull(*v);
    double Lx = (cfg->nx - 1) * dx, Ly = (cfg->ny - 1) * dy;
    for (int i = 0; i < n; i++) {
      d[i].charge = sign[i] * QE_H;
      d[i].spwt = normden[i] * Lx * Ly * L * L / d[i].numparticle;
      if (i < max_sp) sp[i] = d[i];
    }
    *nsp = n;
    if (num_ts) *num_ts = NUM_TS;
  } catch (const std::exception& e) {
    err = e.what();
    return EPIC_ERR_INVALID;
  }
  return EPIC_OK;
}

// ------------------------------------------------------------- loading ---
// Init::Init and Init::SampleVel (src/init.cpp:3-114) with the reference's
// generator: std::mt19937 feeding uniform_real_distribution<double>(0, 1)
// (include/domain.h:218-231).  The three draws of SampleVel are taken left to
// right, the order GCC gives the reference's expression.
namespace {
struct Rnd {
  std::mt19937 gen;
  std::uniform_real_distribution<double> dist{0.0, 1.0};
  explicit Rnd(uint32_t seed) : gen(seed) {}
  double operator()() { return dist(gen); }
};

double sample_vel(Rnd& rnd, double mass, double temp) {
  double v_th = sqrt(2 * K_B_H * temp * (QE_H / K_B_H) / mass);
  double u1 = rnd();
  double u2 = rnd();
  double u3 = rnd();
  return v_th * sqrt(2) * (u1 + u2 + u3 - 1.5);
}
}  // namespace

int parse_load_type(const std::string& load, int* kind, int* narg, std::string& err) {
  std::string type = load;
  *narg = 0;
  size_t lp = load.find('(');
  if (lp != std::string::npos && load.find(')', lp) != std::string::npos) {  // INIParser::loadtypeextract
    type = load.substr(0, lp);
    *narg = std::stoi(load.substr(lp + 1, load.find(')', lp) - lp - 1));
  }
  if (type == "random") *kind = 0;
  else if (type == "uniform") *kind = 1;
  else if (type == "sin") *kind = 2;
  else if (type == "cos") *kind = 3;
  else {
    err = "load type " + load + " is not supported (random, uniform, sin(n), cos(n))";
    return EPIC_ERR_INVALID;
  }
  return EPIC_OK;
}

bool in_rect_conductor(const std::vector<epic_conductor>& cond, double x, double y) {
  for (const epic_conductor& g : cond)
    if (g.type == EPIC_CONDUCTOR_RECT && x >= g.min_x && x <= g.max_x && y >= g.min_y && y <= g.max_y) return true;
  return false;
}

int conductors_from_ini(const char* path, std::vector<epic_conductor>& out, std::string& err) {
  Ini ini;
  if (!parse_ini(path, ini, err)) return EPIC_ERR_IO;
  out.clear();
  auto gs = ini.find("Grids");
  if (gs == ini.end()) return EPIC_OK;
  const Section& g = gs->second;
  try {
    auto get = [&](const std::string& k) -> const std::string& {
      auto it = g.find(k);
      if (it == g.end()) throw std::runtime_error("missing key " + k + " in [Grids]");
      return it->second;
    };
    const int count = g.count("grid_count") ? std::stoi(get("grid_count")) : 0;
    const double vscale = QE_H / (K_B_H * (QE_H / K_B_H));  // Const::eV / (K_b * EV_to_K)
    for (int i = 0; i < count; i++) {
      const std::string pre = "grid_" + std::to_string(i) + ".";
      const std::string type = get(pre + "type");
      epic_conductor c;
      std::memset(&c, 0, sizeof c);
      if (type == "circular") {
        c.type = EPIC_CONDUCTOR_CIRCULAR;
        c.x_center = std::stoi(get(pre + "x_center"));
        c.y_center = std::stoi(get(pre + "y_center"));
        c.electrode_number = std::stoi(get(pre + "electrode_number"));
        c.grid_radius = std::stod(get(pre + "grid_radius"));
        c.electrode_radius = std::stod(get(pre + "electrod_radius"));
        c.voltage = vscale * std::stod(get(pre + "electrode_voltage"));
      } else if (type == "reactconduct") {
        c.type = EPIC_CONDUCTOR_RECT;
        c.min_x = std::stoi(get(pre + "min_x"));
        c.min_y = std::stoi(get(pre + "min_y"));
        c.max_x = std::stoi(get(pre + "max_x"));
        c.max_y = std::stoi(get(pre + "max_y"));
        c.voltage = vscale * std::stod(get(pre + "grid_voltage"));
      } else {
        continue;  // src/main.cpp:303-325 ignores other types
      }
      out.push_back(c);
    }
  } catch (const std::exception& e) {
    err = e.what();
    return EPIC_ERR_INVALID;
  }
  return EPIC_OK;
}

int emitters_from_ini(const char* path, std::vector<epic_emitter>& out, std::string& err) {
  Ini ini;
  if (!parse_ini(path, ini, err)) return EPIC_ERR_IO;
  out.clear();
  auto es = ini.find("Emitters");
  if (es == ini.end()) return EPIC_OK;
  const Section& e = es->second;
  try {
    auto get = [&](const std::string& k) -> const std::string& {
      auto it = e.find(k);
      if (it == e.end()) throw std::runtime_error("missing key " + k + " in [Emitters]");
      return it->second;
    };
    const int count = e.count("count") ? std::stoi(get("count")) : 0;
    for (int i = 0; i < count; i++) {
      const std::string pre = "emitter_" + std::to_string(i) + ".";
      epic_emitter m;
      std::memset(&m, 0, sizeof m);
      m.x0 = std::stod(get(pre + "x0"));
      m.y0 = std::stod(get(pre + "y0"));
      m.x1 = std::stod(get(pre + "x1"));
      m.y1 = std::stod(get(pre + "y1"));
      m.temp = std::stod(get(pre + "temp"));
      m.numparticle = std::stoi(get(pre + "numparticle"));
      m.vdx = std::stod(get(pre + "vdx"));
      m.vdy = std::stod(get(pre + "vdy"));
      m.species_idx1 = std::stoi(get(pre + "species_idx1"));
      m.species_idx2 = std::stoi(get(pre + "species_idx2"));
      out.push_back(m);
    }
  } catch (const std::exception& ex) {
    err = ex.what();
    return EPIC_ERR_INVALID;
  }
  return EPIC_OK;
}

void conductor_geometry(const epic_config& c, const std::vector<epic_conductor>& cond, std::vector<double>& rects,
                        std::vector<double>& circles, std::vector<int>& nodes, std::vector<double>& vals) {
  rects.clear();
  circles.clear();
  std::map<int, double> over;  // node -> value; later conductors overwrite
  std::vector<int> order;
  auto set = [&](int i, int j, double v) {
    if (i < 0 || i >= c.nx || j < 0 || j >= c.ny) return;
    const int k = i * c.ny + j;
    if (!over.count(k)) order.push_back(k);
    over[k] = v;
  };
  const double PI_M = 3.14159265358979323846;  // M_PI (src/grid.cpp, src/electrode.cpp)
  for (const epic_conductor& g : cond) {
    if (g.type == EPIC_CONDUCTOR_RECT) {
      rects.insert(rects.end(), {(double)g.min_x, (double)g.max_x, (double)g.min_y, (double)g.max_y});
      // ReactConductorGrid::initialize: the border of the node rectangle
      const int min_i = (int)((g.min_x - c.x0) / c.dx), max_i = (int)((g.max_x - c.x0) / c.dx);
      const int min_j = (int)((g.min_y - c.y0) / c.dy), max_j = (int)((g.max_y - c.y0) / c.dy);
      for (int i = min_i; i <= max_i; i++)
        for (int j = min_j; j <= max_j; j++)
          if (i == min_i || i == max_i || j == min_j || j == max_j) set(i, j, g.voltage);
    } else {
      for (int k = 0; k < g.electrode_number; k++) {
        const double theta = k * (2.0 * PI_M / g.electrode_number);
        const double ex = g.x_center + g.grid_radius * cos(theta);
        const double ey = g.y_center + g.grid_radius * sin(theta);
        const double r = g.electrode_radius;
        circles.insert(circles.end(), {ex, ey, r * r, 0.0});
        // Electrode::Electrode: 100 points of the circle, rounded to nodes
        const int N = 100;
        for (int q = 0; q < N; q++) {
          const double t = 2.0 * q * PI_M / N;
          set((int)(ex + r * cos(t) + 0.5), (int)(ey + r * sin(t) + 0.5), g.voltage);
        }
      }
    }
  }
  nodes.clear();
  vals.clear();
  for (int k : order) {
    nodes.push_back(k);
    vals.push_back(over[k]);
  }
}

struct RefStream {
  Rnd rnd;
  explicit RefStream(uint32_t seed) : rnd(seed) {}
};
RefStream* ref_stream_create(uint32_t seed) { return new RefStream(seed); }
void ref_stream_destroy(RefStream* r) { delete r; }

int load_particles(const epic_config& c, const std::vector<const epic_species_desc*>& sp,
                   std::vector<std::vector<double>>& out, uint32_t seed, std::string& err,
                   const std::vector<epic_conductor>& cond) {
  RefStream rs(seed);
  out.resize(sp.size());
  for (size_t s = 0; s < sp.size(); s++)
    if (int st = load_species(c, *sp[s], out[s], &rs, err, cond)) return st;
  return EPIC_OK;
}

int load_species(const epic_config& c, const epic_species_desc& d, std::vector<double>& o, RefStream* rs,
                 std::string& err, const std::vector<epic_conductor>& cond) {
  Rnd& rnd = rs->rnd;
  const double Lx = (c.nx - 1) * c.dx, Ly = (c.ny - 1) * c.dy;
  {
    int kind = 0, narg = 0;
    if (int st = parse_load_type(d.load, &kind, &narg, err)) return st;
    const long n = d.numparticle;
    o.resize((size_t)n * 5);
    for (long p = 0; p < n; p++) {
      double x = 0, y = 0;
      for (;;) {  // src/init.cpp:71-86: positions inside a conductor are drawn again
      if (kind == 0) {
        x = c.x0 + Lx * rnd();
        y = c.y0 + Ly * rnd();
      } else if (kind == 1) {
        int nxp = (int)sqrt((double)n);
        int px = (int)(p % nxp), py = (int)(p / nxp);
        x = c.x0 + px * (Lx / (nxp - 1));
        y = c.y0 + py * (Ly / (nxp - 1));
      } else {
        x = c.x0 + p * (Lx / (n - 1));
        y = c.y0 + p * (Ly / (n - 1));
        double kx = 2 * PI_H * narg / Lx;
        double ky = 2 * PI_H * narg / Ly;
        if (kind == 2) { x += sin(kx * x); y += sin(ky * y); }
        else { x += cos(kx * x); y += cos(ky * y); }
      }
      if (!in_rect_conductor(cond, x, y)) break;
      if (kind != 0) {
        err = "load type " + std::string(d.load) + " places a particle inside a conductor (the reference loops forever)";
        return EPIC_ERR_INVALID;
      }
      }
      double vx = sample_vel(rnd, d.mass, d.temp) + d.vsx * c.vel_norm;
      double vy = sample_vel(rnd, d.mass, d.temp) + d.vsy * c.vel_norm;
      // The reference loads vz = 0 (src/init.cpp:88); load_3v draws it like
      // vx and vy (no drift), after them.
      double vz = c.load_3v ? sample_vel(rnd, d.mass, d.temp) : 0;
      vx /= c.vel_norm;
      vy /= c.vel_norm;
      vz /= c.vel_norm;
      double* q = &o[(size_t)p * 5];
      q[0] = x; q[1] = y; q[2] = vx; q[3] = vy; q[4] = vz;
    }
  }
  return EPIC_OK;
}

// ------------------------------------------------------ cross sections ---
// e-/Ar fits of src/cross_section.cpp:4-39 (energy in eV, result in m^2).
double cs_elastic(double energy, int on) {
  if (!on) return 0.0;
  return (1e-20 * fabs(6.0 / pow(1.0 + (energy / 0.1) + pow(energy / 0.6, 2.0), 3.3) -
                       1.1 * pow(energy, 1.4) / (1.0 + pow(energy / 15.0, 1.2)) /
                           sqrt(1.0 + pow(energy / 5.5, 2.5) + pow(energy / 60.0, 4.1)) +
                       0.05 / pow(1.0 + energy / 10.0, 2.0) + 0.01 * pow(energy, 3.0) / (1.0 + pow(energy / 12.0, 6.0))));
}

double cs_excitation(double energy, int on) {
  if (!on || !(energy > 11.5)) return 0.0;
  return (1e-20 * (0.034 * pow(energy - 11.5, 1.1) * (1.0 + pow(energy / 15.0, 2.8)) / (1.0 + pow(energy / 23.0, 5.5)) +
                   0.023 * (energy - 11.5) / pow(1.0 + energy / 80.0, 1.9)));
}

double cs_ionization(double energy, int on) {
  if (!on || !(energy > 15.8)) return 0.0;
  return (1e-20 * (970.0 * (energy - 15.8) / pow(70.0 + energy, 2.0) +
                   0.06 * pow(energy - 15.8, 2.0) * exp(-energy / 9)));
}

// set_electron_cross_sections + calc_total_cross_sections
// (src/collision.cpp:21-42) on the 5,000,000-point grid, spread over host threads.
void reference_tables(const epic_config& c, std::vector<double>& tot, std::vector<double>& ela,
                      std::vector<double>& exc, std::vector<double>& ion) {
  const long N = 5000000;
  tot.assign(N, 0.0);
  ela.assign(N, 0.0);
  exc.assign(N, 0.0);
  ion.assign(N, 0.0);
  unsigned nt = std::thread::hardware_concurrency();
  if (nt < 1) nt = 1;
  if (nt > 32) nt = 32;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; t++) {
    th.emplace_back([&, t]() {
      for (long i = t; i < N; i += nt) {
        double e = i == 0 ? 0.005 : 0.005 * (int)i;
        ela[i] = cs_elastic(e, c.elastic);
        exc[i] = cs_excitation(e, c.excitation);
        ion[i] = cs_ionization(e, c.ionization);
        tot[i] = (ela[i] + exc[i] + ion[i]) * c.gas_density;
      }
    });
  }
  for (auto& x : th) x.join();
}

}  // namespace epic
