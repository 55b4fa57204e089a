#include "inputs.hpp"

#include <sys/stat.h>

#include <algorithm>
#include <cctype>
#include <cstdio>
#include <fstream>
#include <sstream>

namespace pphost {

namespace {

bool one_of(const std::string &v, std::initializer_list<const char *> opts) {
  for (const char *o : opts)
    if (v == o) return true;
  return false;
}
const std::initializer_list<const char *> YES = {"yes", "true", "Yes", "True", "YES", "TRUE"};
const std::initializer_list<const char *> NO = {"no", "false", "No", "False", "NO", "FALSE"};

std::string trim(const std::string &s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) ++a;
  while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
  return s.substr(a, b - a);
}
std::string first_token(const std::string &s) {
  std::istringstream is(s);
  std::string t;
  is >> t;
  return t;
}
// list-directed REAL / INTEGER reads of the first item (d or D exponents)
double fortran_real(const std::string &s) {
  std::string t = first_token(s);
  for (char &c : t)
    if (c == 'd' || c == 'D') c = 'e';
  try {
    return std::stod(t);
  } catch (...) {
    throw InputError("cannot read a real number from '" + s + "'");
  }
}
int64_t fortran_int(const std::string &s) {
  try {
    return std::stoll(first_token(s));
  } catch (...) {
    throw InputError("cannot read an integer from '" + s + "'");
  }
}
bool exists(const std::string &p) {
  struct stat st;
  return stat(p.c_str(), &st) == 0;
}
std::string upper(std::string s) {
  for (char &c : s) c = (char)std::toupper((unsigned char)c);
  return s;
}

void sanitize(InputConfig &cfg, int nprocs, bool check_output_exists) {
  for (std::string *v : {&cfg.lammps_location, &cfg.q_location, &cfg.output_location, &cfg.fc_location})
    if (v->empty() || v->back() != '/') *v += "/";
  if (cfg.mb == -1) cfg.mb = std::min<int64_t>(32, cfg.natom) / nprocs + 1;
  if (cfg.nb == -1) cfg.nb = std::min<int64_t>(32, cfg.natom) / nprocs + 1;
  if (cfg.range == 'V') {
    cfg.il = 1;
    cfg.iu = cfg.natom;
  } else if (cfg.range == 'I') {
    cfg.vl = cfg.vu = 0.0;
  } else if (cfg.range == 'A') {
    cfg.il = 1;
    cfg.iu = cfg.natom;
    cfg.vl = cfg.vu = 0.0;
  }
  if (cfg.range == 'I' && cfg.il > cfg.iu) throw InputError("Invalid input for eigenvalue indices to be computed");
  if (cfg.range == 'V' && cfg.vl > cfg.vu)
    throw InputError("Invalid input for the interval in which eigenvalue is to be computed");
  if (cfg.group_velocity) cfg.comp_evec = 'V';
  // an existing output is not overwritten: <name>_v<k>.hdf5 (read_input.F90:487-513)
  if (check_output_exists && exists(cfg.output_location + cfg.output_name + ".hdf5")) {
    std::string name;
    for (int k = 1;; ++k) {
      name = cfg.output_name + "_v" + std::to_string(k);
      if (!exists(cfg.output_location + name + ".hdf5")) break;
    }
    cfg.output_name = name + ".hdf5";
  } else {
    cfg.output_name += ".hdf5";
  }
}

}  // namespace

InputConfig::InputConfig() {
  abstol = (double)1e-15f;
  orfac = (double)1e-15f;
}

InputConfig parse_input(const std::string &text, int nprocs, bool check_output_exists) {
  InputConfig cfg;
  std::istringstream in(text);
  std::string raw;
  while (std::getline(in, raw)) {
    std::string data = trim(raw);
    if (data.empty() || data[0] == '#' || data[0] == '!' || data[0] == ' ') continue;
    for (char c : {'!', '#'}) {
      const size_t p = data.find(c);
      if (p != std::string::npos) data = data.substr(0, p);
    }
    std::string key, val;
    const size_t p = data.find(':');
    if (p != std::string::npos) {
      key = trim(upper(data.substr(0, p)));
      val = trim(data.substr(p + 1));
    } else {
      val = trim(data);
    }
    if (key == "LAMMPS FILE LOCATION" || key == "LAMMPS_FILE_LOCATION") {
      cfg.lammps_location = val;
    } else if (key == "LAMMPS_FILE_NAME" || key == "LAMMPS FILE NAME") {
      cfg.lammps_name = val;
    } else if (key == "NATOM") {
      cfg.natom = fortran_int(val);
    } else if (key == "ATOM_STYLE" || key == "ATOM STYLE") {
      cfg.atom_style = val;
    } else if (key == "ATOM_TYPES" || key == "ATOM TYPES") {
      cfg.atom_types = fortran_int(val);
    } else if (key == "FORCE CONSTANT FILE LOCATION" || key == "FORCE_CONSTANT_FILE_LOCATION") {
      cfg.fc_location = val;
    } else if (key == "FORCE CONSTANT FILE NAME" || key == "FORCE_CONSTANT_FILE_NAME") {
      cfg.fc_name = val;
    } else if (key == "FORCE CONSTANT DATASET" || key == "FORCE_CONSTANT_DATASET") {
      cfg.fc_dataset = val;
    } else if (key == "Q_FILE_LOCATION" || key == "Q FILE LOCATION") {
      cfg.q_location = val;
    } else if (key == "Q_FILE_NAME" || key == "Q FILE NAME") {
      cfg.q_name = val;
    } else if (key == "NQPT") {
      cfg.nqpt = fortran_int(val);
    } else if (key == "NUM_QPOOLS" || key == "NUM QPOOLS") {
      // only read by builds with -D__QPOOL; otherwise "not recognised"
      cfg.warnings.push_back("Command " + key + " not recognised");
    } else if (key == "COMPUTE_EIGVECS" || key == "COMPUTE EIGVECS") {
      if (one_of(val, YES)) {
        cfg.comp_evec = 'V';
        cfg.compute_eigvecs = true;
      } else {
        if (!one_of(val, NO))
          cfg.warnings.push_back("Could not interpret command " + val + "; eigenvectors will not be computed.");
        cfg.comp_evec = 'N';
        cfg.compute_eigvecs = false;
      }
    } else if (key == "GROUP VELOCITY" || key == "GROUP_VELOCITY") {
      if (one_of(val, YES)) {
        cfg.group_velocity = true;
      } else {
        if (!one_of(val, NO))
          cfg.warnings.push_back("Could not interpret command " + val + "; velocity will not be computed.");
        cfg.group_velocity = false;
      }
    } else if (key == "VELOCITY METHOD" || key == "VELOCITY_METHOD") {
      if (one_of(val, {"cd", "CD", "central_difference", "CENTRAL_DIFFERENCE"})) {
        cfg.velocity_method = 'C';
      } else {
        if (!one_of(val, {"A", "a", "Analytic", "analytic"}))
          cfg.warnings.push_back("Could not interpret command " + val + "; analytic derivative used.");
        cfg.velocity_method = 'A';
      }
    } else if (key == "RANGE") {
      if (val == "A" || val == "V" || val == "I")
        cfg.range = val[0];
      else  // read_input.F90:202-206: message composed, range left unchanged
        cfg.warnings.push_back("Could not interpret command" + val);
    } else if (key == "MAX_EIGVAL" || key == "MAX EIGVAL") {
      cfg.vu = fortran_real(val);
    } else if (key == "MIN_EIGVAL" || key == "MIN EIGVAL") {
      cfg.vl = fortran_real(val);
    } else if (key == "MAX_INDEX" || key == "MAX INDEX") {
      cfg.iu = fortran_int(val);
    } else if (key == "MIN_INDEX" || key == "MIN INDEX") {
      cfg.il = fortran_int(val);
    } else if (key == "ABSTOL") {
      cfg.abstol = fortran_real(val);
    } else if (key == "ORFAC") {
      cfg.orfac = fortran_real(val);
    } else if (key == "MB") {
      cfg.mb = fortran_int(val);
    } else if (key == "NB") {
      cfg.nb = fortran_int(val);
    } else if (key == "OUTPUT FILE NAME" || key == "OUTPUT_FILE_NAME") {
      cfg.output_name = val;
    } else if (key == "OUTPUT FILE LOCATION" || key == "OUTPUT_FILE_LOCATION") {
      cfg.output_location = val;
    } else if (key == "PRINT PROGRESS" || key == "PRINT_PROGRESS") {
      if (one_of(val, YES)) {
        cfg.print_progress = true;
      } else if (one_of(val, NO)) {
        cfg.print_progress = false;
      } else {
        cfg.warnings.push_back("Could not interpret command " + val + "; progress will be printed.");
        cfg.print_progress = true;
      }
    } else {
      cfg.warnings.push_back("Command " + key + " not recognised");
    }
  }
  sanitize(cfg, nprocs, check_output_exists);
  return cfg;
}

InputConfig read_input(const std::string &path, int nprocs) {
  std::ifstream f(path);
  if (!f) throw InputError("cannot open input file " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return parse_input(ss.str(), nprocs);
}

namespace {
struct Lines {
  std::ifstream f;
  std::string path;
  std::string next() {
    std::string l;
    if (!std::getline(f, l)) throw InputError("unexpected end of " + path);
    return l;
  }
};
std::vector<double> nums(const std::string &line, size_t k) {
  std::istringstream is(line);
  std::vector<double> v;
  std::string t;
  while (v.size() < k && is >> t) v.push_back(std::stod(t));
  if (v.size() < k) throw InputError("too few numbers in line '" + line + "'");
  return v;
}
std::vector<std::string> tokens(const std::string &line) {
  std::istringstream is(line);
  std::vector<std::string> v;
  std::string t;
  while (is >> t) v.push_back(t);
  return v;
}
}  // namespace

LammpsData read_lammps_data(const std::string &path, int64_t natom, int64_t ntypes, const std::string &style) {
  Lines L{std::ifstream(path), path};
  if (!L.f) throw InputError("cannot open LAMMPS data file " + path);
  for (int i = 0; i < 5; ++i) L.next();
  const auto x = nums(L.next(), 2), y = nums(L.next(), 2), z = nums(L.next(), 2), t = nums(L.next(), 3);
  LammpsData d;
  const double lat[3][3] = {{x[1] - x[0], 0, 0}, {t[0], y[1] - y[0], 0}, {t[1], t[2], z[1] - z[0]}};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) d.lat[i][j] = lat[i][j];
  for (int i = 0; i < 3; ++i) L.next();
  d.masses.resize(ntypes);
  for (int64_t i = 0; i < ntypes; ++i) {
    const auto tk = tokens(L.next());
    if (tk.size() < 2) throw InputError("bad Masses line in " + path);
    d.masses[i] = std::stod(tk[1]);
  }
  for (int i = 0; i < 3; ++i) L.next();
  d.at_types.resize(natom);
  d.real_pos.resize(3 * natom);
  int kt, kp;
  if (style == "atomic" || style == "Atomic" || style == "ATOMIC") {
    kt = 1, kp = 2;
  } else if (style == "molecular" || style == "Molecular" || style == "MOLECULAR") {
    kt = 2, kp = 3;
  } else if (style == "full" || style == "Full" || style == "FULL") {
    kt = 2, kp = 4;
  } else {
    throw InputError("Atom style not supported. Supported styles are atomic and molecular");
  }
  for (int64_t i = 0; i < natom; ++i) {
    const auto tk = tokens(L.next());
    if ((int)tk.size() < kp + 3) throw InputError("bad Atoms line in " + path);
    d.at_types[i] = std::stoll(tk[kt]);
    for (int k = 0; k < 3; ++k) d.real_pos[3 * i + k] = std::stod(tk[kp + k]);
  }
  return d;
}

std::vector<double> read_q_file(const std::string &path, int64_t nqpt) {
  Lines L{std::ifstream(path), path};
  if (!L.f) throw InputError("cannot open q-point file " + path);
  std::vector<double> q(3 * nqpt);
  for (int64_t i = 0; i < nqpt; ++i) {
    const auto v = nums(L.next(), 3);
    for (int k = 0; k < 3; ++k) q[3 * i + k] = v[k];
  }
  return q;
}

std::vector<double> crys_from_positions(const double A[3][3], const std::vector<double> &pos) {
  auto a = [&](int i, int j) { return A[i - 1][j - 1]; };
  const double det = a(1, 1) * a(2, 2) * a(3, 3) - a(1, 1) * a(2, 3) * a(3, 2) - a(1, 2) * a(2, 1) * a(3, 3) +
                     a(1, 2) * a(2, 3) * a(3, 1) + a(1, 3) * a(2, 1) * a(3, 2) - a(1, 3) * a(2, 2) * a(3, 1);
  const double detinv = 1.0 / det;
  double B[3][3];
  B[0][0] = +detinv * (a(2, 2) * a(3, 3) - a(2, 3) * a(3, 2));
  B[1][0] = -detinv * (a(2, 1) * a(3, 3) - a(2, 3) * a(3, 1));
  B[2][0] = +detinv * (a(2, 1) * a(3, 2) - a(2, 2) * a(3, 1));
  B[0][1] = -detinv * (a(1, 2) * a(3, 3) - a(1, 3) * a(3, 2));
  B[1][1] = +detinv * (a(1, 1) * a(3, 3) - a(1, 3) * a(3, 1));
  B[2][1] = -detinv * (a(1, 1) * a(3, 2) - a(1, 2) * a(3, 1));
  B[0][2] = +detinv * (a(1, 2) * a(2, 3) - a(1, 3) * a(2, 2));
  B[1][2] = -detinv * (a(1, 1) * a(2, 3) - a(1, 3) * a(2, 1));
  B[2][2] = +detinv * (a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1));
  const size_t natom = pos.size() / 3;
  std::vector<double> c(3 * natom);
  for (size_t I = 0; I < natom; ++I)
    for (int i = 0; i < 3; ++i)  // u(i) = sum_k B(k,i) x(k), k = 1, 2, 3 in order
      c[3 * I + i] = (B[0][i] * pos[3 * I] + B[1][i] * pos[3 * I + 1]) + B[2][i] * pos[3 * I + 2];
  return c;
}

}  // namespace pphost
