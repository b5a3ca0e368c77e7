// epic2d_output.hpp — the reference's Output (src/output.cpp:4-287) without
// HDF5, which this build does not have: the groups of result.h5 become
// directories under <outputfolder>/result/, each dataset a .npy file of the
// same name, shape and element order, and the attribute groups JSON files.
//
//   result/fielddata/pot/<ts>.npy        shape (nx, ny), buffer phi(i, j) at j*nx + i
//   result/fielddata/efieldx/<ts>.npy    (same layout)
//   result/fielddata/efieldy/<ts>.npy
//   result/fielddata/den_<name>/<ts>.npy
//   result/particle_<name>/pos<ts>.npy   shape (N, 2): x, y
//   result/particle_<name>/vel<ts>.npy   shape (N, 2): vx, vy
//   result/time_var/kinetic_energy.npy   shape (NUM_TS/write_interval + 1, 3*species + 2)
//   result/metadata.json                 Output::write_metadata's attributes
//   result/metadata_species/<name>.json  Output::write_species_metadata's attributes
//
// The reference declares the field datasets (nx, ny) while filling them in
// j*nx + i order; the same buffer and declared shape are written here so
// readers of result.h5 (its python_scripts) index the files the same way.
#pragma once

#include <cstdint>
#include <filesystem>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "epic2d.hpp"

namespace epic2d {

// NumPy .npy format version 1.0, little-endian float64, C order.
inline void write_npy(const std::filesystem::path& path, const double* data, const std::vector<size_t>& shape) {
  std::string dict = "{'descr': '<f8', 'fortran_order': False, 'shape': (";
  size_t count = 1;
  for (size_t k = 0; k < shape.size(); k++) {
    dict += std::to_string(shape[k]);
    if (shape.size() == 1 || k + 1 < shape.size()) dict += ", ";
    count *= shape[k];
  }
  dict += "), }";
  const size_t unpadded = 10 + dict.size() + 1;  // magic, version, length, dict, '\n'
  dict += std::string((64 - unpadded % 64) % 64, ' ') + "\n";
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) throw std::runtime_error("cannot write " + path.string());
  f.write("\x93NUMPY\x01\x00", 8);
  const uint16_t len = (uint16_t)dict.size();
  const char lb[2] = {(char)(len & 0xff), (char)(len >> 8)};
  f.write(lb, 2);
  f.write(dict.data(), (std::streamsize)dict.size());
  f.write(reinterpret_cast<const char*>(data), (std::streamsize)(count * sizeof(double)));
}

class Output {
 public:
  // Output::Output: clears and recreates the result tree.  The reference clears
  // the whole output folder; only its result/ subtree is cleared here.
  Output(const std::filesystem::path& outputfolder, Domain& domain, int num_ts, int write_interval, int nsp)
      : root_(outputfolder / "result"), domain_(domain), write_interval_(write_interval), nsp_(nsp) {
    if (write_interval <= 0) throw std::runtime_error("write_interval must be positive");
    std::filesystem::remove_all(root_);
    std::filesystem::create_directories(root_ / "fielddata");
    std::filesystem::create_directories(root_ / "time_var");
    std::filesystem::create_directories(root_ / "metadata_species");
    rows_ = num_ts / write_interval + 1;
    cols_ = 3 * nsp + 2;
    store_ke_.assign((size_t)rows_ * cols_, 0.0);
  }

  // Output::write_particle_data: positions and velocities (x, y components).
  void write_particle_data(int ts, Species& sp) {
    const std::filesystem::path dir = root_ / ("particle_" + sp.name);
    std::filesystem::create_directories(dir);
    const std::vector<double> p = sp.particles();
    const size_t n = p.size() / 5;
    std::vector<double> pos(2 * n), vel(2 * n);
    for (size_t k = 0; k < n; k++) {
      pos[2 * k] = p[5 * k];
      pos[2 * k + 1] = p[5 * k + 1];
      vel[2 * k] = p[5 * k + 2];
      vel[2 * k + 1] = p[5 * k + 3];
    }
    write_npy(dir / ("pos" + std::to_string(ts) + ".npy"), pos.data(), {n, 2});
    write_npy(dir / ("vel" + std::to_string(ts) + ".npy"), vel.data(), {n, 2});
  }

  // Output::write_field_data: potential and both field components.
  void write_field_data(int ts) {
    write_grid("pot", ts, domain_.grid(EPIC_GRID_PHI));
    write_grid("efieldx", ts, domain_.grid(EPIC_GRID_EFX));
    write_grid("efieldy", ts, domain_.grid(EPIC_GRID_EFY));
  }

  // Output::write_den_data: the species' density.
  void write_den_data(int ts, Species& sp) {
    write_grid("den_" + sp.name, ts, domain_.grid(EPIC_GRID_DEN0 + sp.index()));
  }

  // Output::write_metadata (the reference passes 0 for GAS_DENSITY, src/main.cpp:275-276).
  void write_metadata(int NC, int NUM_TS, int write_int, int write_int_phase, double DT, double density, int save_fig,
                      int normscheme, int subcycleint, double LDe, double LDi, double wpe, double wpi, int spno,
                      double GAS_DENSITY) {
    std::ostringstream j;
    j.precision(17);
    j << "{\"NC\": " << NC << ", \"NUM_TS\": " << NUM_TS << ", \"write_int\": " << write_int
      << ", \"write_int_phase\": " << write_int_phase << ", \"DT_coeff\": " << DT << ", \"density\": " << density
      << ", \"save_fig\": " << save_fig << ", \"norm_scheme\": " << normscheme
      << ", \"sub_cycle_interval\": " << subcycleint << ", \"LDe\": " << LDe << ", \"LDi\": " << LDi
      << ", \"wpe\": " << wpe << ", \"wpi\": " << wpi << ", \"spno\": " << spno
      << ", \"GAS_DENSITY\": " << GAS_DENSITY << "}\n";
    std::ofstream(root_ / "metadata.json") << j.str();
  }

  // Output::write_species_metadata.
  template <class List>
  void write_species_metadata(List& species_list) {
    for (auto& spp : species_list) {
      Species& sp = deref(spp);
      std::ostringstream j;
      j.precision(17);
      j << "{\"name\": \"" << sp.name << "\", \"mass\": " << sp.mass << ", \"charge\": " << sp.charge
        << ", \"spwt\": " << sp.spwt << ", \"temperature\": " << sp.temp << ", \"density\": " << sp.fract_den
        << ", \"num_particles\": " << sp.numparticle << ", \"streaming_velocity\": " << sp.vsx << "}\n";
      std::ofstream(root_ / "metadata_species" / (sp.name + ".json")) << j.str();
    }
  }

  // Output::storeKE_to_matrix: ts*DT, KE (x, y, z) per species, PE.
  template <class List>
  void storeKE_to_matrix(int ts, List& species_list, Species& norm_species) {
    const int k = ts / write_interval_;
    if (k >= rows_) return;
    double* row = &store_ke_[(size_t)k * cols_];
    row[0] = ts * domain_.config().DT;
    int j = 1;
    for (auto& spp : species_list) {
      const std::array<double, 3> ke = deref(spp).Compute_KE(norm_species);
      row[j] = ke[0];
      row[j + 1] = ke[1];
      row[j + 2] = ke[2];
      j += 3;
    }
    row[j] = domain_.Compute_PE(norm_species.index());
  }

  // Output::write_ke.
  void write_ke() {
    write_npy(root_ / "time_var" / "kinetic_energy.npy", store_ke_.data(), {(size_t)rows_, (size_t)cols_});
  }

 private:
  static Species& deref(Species& s) { return s; }
  template <class P>
  static Species& deref(P& p) { return *p; }

  void write_grid(const std::string& group, int ts, const std::vector<double>& g) {
    const epic_config& c = domain_.config();
    const size_t nx = c.nx, ny = c.ny;
    std::vector<double> out(nx * ny);
    for (size_t j = 0; j < ny; j++)
      for (size_t i = 0; i < nx; i++) out[j * nx + i] = g[i * ny + j];  // node (i, j) is at i*ny + j on the GPU
    const std::filesystem::path dir = root_ / "fielddata" / group;
    std::filesystem::create_directories(dir);
    write_npy(dir / (std::to_string(ts) + ".npy"), out.data(), {nx, ny});
  }

  std::filesystem::path root_;
  Domain& domain_;
  int write_interval_, nsp_, rows_, cols_;
  std::vector<double> store_ke_;
};

}  // namespace epic2d
