// Readers for the reference's input formats, with the reference's semantics:
//   * read_input       the `key : value` file of Phonon_Calculations/SRC/
//                      read_input.F90 (parser :90-250, defaults :368-404,
//                      sanitising :415-517);
//   * read_lammps_data LAMMPS data file, atomic / molecular / full styles
//                      (lammps_read.F90:28-243);
//   * read_q_file      nqpt lines of reduced coordinates, extra columns
//                      ignored (q_read.F90:41-131);
//   * crys_from_positions  crys = (A^-1)^T x with A^-1 from cofactors, in the
//                      reference's evaluation order (lammps_read.F90:198-200,
//                      281-309).
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace pphost {

// Raised where the reference prints an error and stops.
struct InputError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

struct InputConfig {
  std::string lammps_location = "./", lammps_name = "lammps.dat", atom_style = "A";
  int64_t atom_types = 1, natom = 1;
  std::string q_location = "./", q_name = "q_file.dat";
  int64_t nqpt = 1;
  std::string fc_location = "./", fc_name = "FC_hdf5", fc_dataset = "force_constants";
  int64_t num_qpools = 1;  // read only by -D__QPOOL builds of the reference
  bool compute_eigvecs = false;
  char comp_evec = 'N';
  bool group_velocity = false;
  char velocity_method = 'A';
  char range = 'A';
  double vl = 0.0, vu = 0.0;
  int64_t il = 1, iu = 1;
  double abstol, orfac;  // REAL*4 literal 1e-15 of read_input.F90:394-395
  int64_t mb = -1, nb = -1;
  std::string output_name = "results", output_location = "./";
  bool print_progress = true;
  std::vector<std::string> warnings;
  InputConfig();
};

InputConfig parse_input(const std::string &text, int nprocs = 1, bool check_output_exists = true);
InputConfig read_input(const std::string &path, int nprocs = 1);

struct LammpsData {
  double lat[3][3];                // rows a_i
  std::vector<double> masses;      // [ntypes]
  std::vector<int64_t> at_types;   // [natom], 1-based
  std::vector<double> real_pos;    // [natom][3]
};
LammpsData read_lammps_data(const std::string &path, int64_t natom, int64_t ntypes, const std::string &style);

std::vector<double> read_q_file(const std::string &path, int64_t nqpt);  // [nqpt][3]

// crys[I][k] for positions x[I][k]
std::vector<double> crys_from_positions(const double lat[3][3], const std::vector<double> &pos);

}  // namespace pphost
