// Host-side start-up helpers of the C ABI (INI, loader, cross-section tables).
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/epic2d.h"

namespace epic {

// include/domain.h:204-215 (host copies; PI is the reference's truncated value).
constexpr double EPS_0_H = 8.85418782e-12;
constexpr double QE_H = 1.602176565e-19;
constexpr double ME_H = 9.10938215e-31;
constexpr double K_B_H = 1.380648e-23;
constexpr double PI_H = 3.141592653;

int config_from_ini(const char* path, epic_config* cfg, epic_species_desc* sp, int max_sp, int* nsp, int* num_ts,
                    std::string& err);
int ini_get(const char* path, const char* section, const char* key, std::string& value, std::string& err);
int load_particles(const epic_config& c, const std::vector<const epic_species_desc*>& sp,
                   std::vector<std::vector<double>>& out, uint32_t seed, std::string& err,
                   const std::vector<epic_conductor>& cond = {});
// The reference's global generator (Rnd rnd, include/domain.h:218-231 and
// src/domain.cpp:4): one mt19937 seeded once and continued by every Init.
struct RefStream;
RefStream* ref_stream_create(uint32_t seed);
void ref_stream_destroy(RefStream* r);
// Init::Init of one species (src/init.cpp:3-101) drawing from *rs.
int load_species(const epic_config& c, const epic_species_desc& d, std::vector<double>& out, RefStream* rs,
                 std::string& err, const std::vector<epic_conductor>& cond = {});
int conductors_from_ini(const char* path, std::vector<epic_conductor>& out, std::string& err);
int emitters_from_ini(const char* path, std::vector<epic_emitter>& out, std::string& err);
// Conductor geometry for the device: rectangles {min_x, max_x, min_y, max_y},
// electrodes {x0, y0, r*r, 0} (CircularGrid::initialize, src/grid.cpp:46-57),
// and the rho override as unique (node, value) pairs, later conductors
// winning (Grid::initialize in order, src/grid.cpp:67-85, src/electrode.cpp:4-17).
void conductor_geometry(const epic_config& c, const std::vector<epic_conductor>& cond, std::vector<double>& rects,
                        std::vector<double>& circles, std::vector<int>& nodes, std::vector<double>& vals);
// Grid::IsGrid of the rectangles only (Init runs before any CircularGrid has electrodes).
bool in_rect_conductor(const std::vector<epic_conductor>& cond, double x, double y);
// INIParser::loadtypeextract (src/iniparser.cpp): "random" -> 0, "uniform" -> 1,
// "sin(n)" -> 2, "cos(n)" -> 3 with *narg = n; EPIC_ERR_INVALID otherwise.
int parse_load_type(const std::string& load, int* kind, int* narg, std::string& err);
void reference_tables(const epic_config& c, std::vector<double>& tot, std::vector<double>& ela,
                      std::vector<double>& exc, std::vector<double>& ion);
double cs_elastic(double energy, int on);
double cs_excitation(double energy, int on);
double cs_ionization(double energy, int on);

}  // namespace epic
