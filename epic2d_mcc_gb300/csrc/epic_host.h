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
                   std::vector<std::vector<double>>& out, uint32_t seed, std::string& err);
// INIParser::loadtypeextract (src/iniparser.cpp): "random" -> 0, "uniform" -> 1,
// "sin(n)" -> 2, "cos(n)" -> 3 with *narg = n; EPIC_ERR_INVALID otherwise.
int parse_load_type(const std::string& load, int* kind, int* narg, std::string& err);
void reference_tables(const epic_config& c, std::vector<double>& tot, std::vector<double>& ela,
                      std::vector<double>& exc, std::vector<double>& ion);
double cs_elastic(double energy, int on);
double cs_excitation(double energy, int on);
double cs_ionization(double energy, int on);

}  // namespace epic
