// parphom_gpu.x — the parphom.x run (Phonon_Calculations/SRC/main.F90:40-70)
// on one GB300, as a native host program over the C ABI of libparphom_gpu.so.
//
// Same inputs and outputs as the reference program: the `key : value` input
// file, the LAMMPS data file, the (N,N,3,3) HDF5 force-constant dataset and
// the q-point file are read with the reference's semantics; the per-q loop
// (calculations.F90:49-53) runs on the GPU in batches (pp_solve_batch); the
// output file gets one group per q-point named '%012d' (global 1-based index)
// with `q_vec` (3,), `eigenvalues` (m,) in cm^-1, `evec` (nz, 3N) compound
// {r, i} when `compute eigvecs: yes`, and `vel` (nz, 3) in m/s when
// `group velocity: yes` (write_output.F90:98-143, 178-312, 377-484).
//
// Usage:  parphom_gpu.x <input file> [--precision mixed|fp64] [--batch B] [--quiet]
// Helper modes used by the tests (no GPU needed):
//   --parse-input <file>        print the sanitised input as JSON
//   --h5-keys <file> <group>    print the member names of a group
//   --h5-read <file> <dataset>  print the shape and the values (%.17g)
//   --h5-copy <in> <out>        rewrite the root datasets and one level of
//                               groups of <in> with this program's writer
//   --read-lammps <file> <natom> <ntypes> <style>
//                               print lat, masses, types, positions and crys
#include <unistd.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "h5min.hpp"
#include "inputs.hpp"
#include "parphom_gpu.h"

namespace {

void progress(bool on, const std::string &text) {
  if (!on) return;
  char buf[64];
  const time_t t = time(nullptr);
  strftime(buf, sizeof buf, "%d/%m/%Y %H:%M:%S", localtime(&t));
  printf("%s on %s\n", text.c_str(), buf);
  fflush(stdout);
}

std::string json_str(const std::string &s) {
  std::string o = "\"";
  for (char c : s) {
    if (c == '"' || c == '\\') o.push_back('\\');
    o.push_back(c);
  }
  return o + "\"";
}

int parse_input_mode(const char *path) {
  const pphost::InputConfig c = pphost::read_input(path);
  printf("{\"lammps_location\": %s, \"lammps_name\": %s, \"atom_style\": %s, \"atom_types\": %lld, ",
         json_str(c.lammps_location).c_str(), json_str(c.lammps_name).c_str(), json_str(c.atom_style).c_str(),
         (long long)c.atom_types);
  printf("\"natom\": %lld, \"q_location\": %s, \"q_name\": %s, \"nqpt\": %lld, \"fc_location\": %s, ",
         (long long)c.natom, json_str(c.q_location).c_str(), json_str(c.q_name).c_str(), (long long)c.nqpt,
         json_str(c.fc_location).c_str());
  printf("\"fc_name\": %s, \"fc_dataset\": %s, \"num_qpools\": %lld, \"compute_eigvecs\": %s, \"comp_evec\": \"%c\", ",
         json_str(c.fc_name).c_str(), json_str(c.fc_dataset).c_str(), (long long)c.num_qpools,
         c.compute_eigvecs ? "true" : "false", c.comp_evec);
  printf("\"group_velocity\": %s, \"velocity_method\": \"%c\", \"range_\": \"%c\", \"vl\": %.17g, \"vu\": %.17g, ",
         c.group_velocity ? "true" : "false", c.velocity_method, c.range, c.vl, c.vu);
  printf("\"il\": %lld, \"iu\": %lld, \"abstol\": %.17g, \"orfac\": %.17g, \"mb\": %lld, \"nb\": %lld, ",
         (long long)c.il, (long long)c.iu, c.abstol, c.orfac, (long long)c.mb, (long long)c.nb);
  printf("\"output_name\": %s, \"output_location\": %s, \"print_progress\": %s, \"warnings\": [",
         json_str(c.output_name).c_str(), json_str(c.output_location).c_str(), c.print_progress ? "true" : "false");
  for (size_t i = 0; i < c.warnings.size(); ++i) printf("%s%s", i ? ", " : "", json_str(c.warnings[i]).c_str());
  printf("]}\n");
  return 0;
}

int h5_keys_mode(const char *file, const char *group) {
  h5min::Reader r(file);
  for (const std::string &k : r.keys(group)) printf("%s\n", k.c_str());
  return 0;
}

int h5_read_mode(const char *file, const char *path) {
  h5min::Reader r(file);
  std::vector<uint64_t> shape;
  const std::vector<double> v = r.read_f64(path, &shape);
  printf("shape");
  for (uint64_t s : shape) printf(" %llu", (unsigned long long)s);
  printf("\n");
  for (double x : v) printf("%.17g\n", x);
  return 0;
}

int h5_copy_mode(const char *in, const char *out) {
  h5min::Reader r(in);
  h5min::Writer w(out);
  auto item = [&](const std::string &path, const std::string &name, std::vector<std::vector<double>> &keep) {
    h5min::Type t;
    std::vector<uint64_t> shape = r.shape(path, &t);
    keep.push_back(r.read_f64(path));
    return h5min::Writer::Item{name, shape, keep.back().data(), t.cls == 'c'};
  };
  for (const std::string &k : r.keys("/")) {
    std::vector<std::vector<double>> keep;
    keep.reserve(64);
    std::vector<std::string> members;
    bool is_group = true;
    try {
      members = r.keys(k);
    } catch (const h5min::Error &) {
      is_group = false;
    }
    if (is_group) {
      std::vector<h5min::Writer::Item> items;
      for (const std::string &m : members) items.push_back(item(k + "/" + m, m, keep));
      w.add_group(k, items);
    } else {
      w.add_dataset(item(k, k, keep));
    }
  }
  w.close();
  return 0;
}

int read_lammps_mode(const char *file, const char *natom, const char *ntypes, const char *style) {
  const int64_t N = std::stoll(natom);
  const pphost::LammpsData d = pphost::read_lammps_data(file, N, std::stoll(ntypes), style);
  const std::vector<double> c = pphost::crys_from_positions(d.lat, d.real_pos);
  for (int i = 0; i < 3; ++i) printf("lat %.17g %.17g %.17g\n", d.lat[i][0], d.lat[i][1], d.lat[i][2]);
  for (double m : d.masses) printf("mass %.17g\n", m);
  for (int64_t I = 0; I < N; ++I)
    printf("atom %lld %.17g %.17g %.17g %.17g %.17g %.17g\n", (long long)d.at_types[I], d.real_pos[3 * I],
           d.real_pos[3 * I + 1], d.real_pos[3 * I + 2], c[3 * I], c[3 * I + 1], c[3 * I + 2]);
  return 0;
}

void check(int rc, const char *what) {
  if (rc != PP_OK) throw std::runtime_error(std::string(what) + ": " + pp_strerror(rc) + " (code " +
                                            std::to_string(rc) + ")");
}

std::string run(const std::string &input, int precision, int64_t batch, bool quiet) {
  // relative locations in the input are relative to the run directory
  std::string dir = ".", base = input;
  const size_t sl = input.rfind('/');
  if (sl != std::string::npos) {
    dir = input.substr(0, sl);
    base = input.substr(sl + 1);
  }
  char cwd[4096];
  if (!getcwd(cwd, sizeof cwd)) throw std::runtime_error("getcwd failed");
  if (chdir(dir.c_str()) != 0) throw std::runtime_error("cannot enter " + dir);
  struct Back {
    const char *d;
    ~Back() {
      if (chdir(d) != 0) perror("chdir");
    }
  } back{cwd};

  pphost::InputConfig cfg = pphost::read_input(base);
  if (quiet) cfg.print_progress = false;
  for (auto &w : cfg.warnings) fprintf(stderr, "%s\n", w.c_str());
  const int64_t N = cfg.natom, n = 3 * N;
  const pphost::LammpsData ld =
      pphost::read_lammps_data(cfg.lammps_location + cfg.lammps_name, N, cfg.atom_types, cfg.atom_style);
  // force constants: element (3I+a, 3J+b) = dset[J, I, b, a], then
  // Phi <- 1/2 Phi^T + 1/2 Phi (force_read.F90:115-189)
  std::vector<double> phi;
  {
    h5min::Reader r(cfg.fc_location + cfg.fc_name);
    std::vector<uint64_t> shape;
    std::vector<double> dset = r.read_f64(cfg.fc_dataset, &shape);
    if (shape.size() != 4 || shape[0] != (uint64_t)N || shape[1] != (uint64_t)N || shape[2] != 3 || shape[3] != 3)
      throw pphost::InputError("force-constant dataset does not have shape (natom, natom, 3, 3)");
    std::vector<double> raw((size_t)n * n);
    for (int64_t J = 0; J < N; ++J)
      for (int64_t I = 0; I < N; ++I)
        for (int b = 0; b < 3; ++b)
          for (int a = 0; a < 3; ++a) raw[(3 * I + a) + n * (3 * J + b)] = dset[((J * N + I) * 3 + b) * 3 + a];
    dset.clear();
    dset.shrink_to_fit();
    phi.resize((size_t)n * n);
    for (int64_t c = 0; c < n; ++c)
      for (int64_t r = 0; r < n; ++r) phi[r + n * c] = 0.5 * raw[c + n * r] + 0.5 * raw[r + n * c];
  }
  progress(cfg.print_progress, "Force constants read and symmetrized");
  const std::vector<double> q = pphost::read_q_file(cfg.q_location + cfg.q_name, cfg.nqpt);
  const int64_t nq = cfg.nqpt;
  const std::vector<double> crys = pphost::crys_from_positions(ld.lat, ld.real_pos);
  // column-major copies for the C ABI
  double lat_f[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) lat_f[i + 3 * j] = ld.lat[i][j];
  std::vector<double> crys_f(3 * N), pos_f(3 * N);
  for (int64_t I = 0; I < N; ++I)
    for (int k = 0; k < 3; ++k) {
      crys_f[I + N * k] = crys[3 * I + k];
      pos_f[I + N * k] = ld.real_pos[3 * I + k];
    }
  pp_system sys{N, (int64_t)ld.masses.size(), lat_f, crys_f.data(), pos_f.data(), ld.masses.data(),
                ld.at_types.data()};
  pp_ctx *ctx = nullptr;
  check(pp_ctx_create(&sys, phi.data(), n, 0, &ctx), "pp_ctx_create");
  struct Ctx {
    pp_ctx *c;
    ~Ctx() { pp_ctx_destroy(c); }
  } ctx_guard{ctx};
  phi.clear();
  phi.shrink_to_fit();

  pp_eig_opts o{};
  o.jobz = cfg.comp_evec;
  o.range = cfg.range;
  o.vel_method = cfg.velocity_method;
  o.uplo = 'U';
  o.vel = cfg.group_velocity ? 1 : 0;
  o.precision = precision;
  o.vl = cfg.vl;
  o.vu = cfg.vu;
  o.il = cfg.il;
  o.iu = cfg.iu;
  o.abstol = cfg.abstol;
  o.orfac = cfg.orfac;
  const int64_t B = batch > 0 ? batch : std::max<int64_t>(1, std::min<int64_t>(nq, 64));
  const int64_t mz = cfg.range == 'I' ? cfg.iu - cfg.il + 1 : n;
  std::vector<double> w(B * n), z, vel;
  if (cfg.compute_eigvecs) z.resize((size_t)B * 2 * n * mz);
  if (cfg.group_velocity) vel.resize((size_t)B * 3 * n);
  std::vector<int64_t> m(B), nz(B), info(B);
  std::vector<double> qb(3 * B);

  const std::string out_path = cfg.output_location + cfg.output_name;
  h5min::Writer wr(out_path);
  for (int64_t t0 = 0; t0 < nq; t0 += B) {
    const int64_t nb = std::min(B, nq - t0);
    for (int64_t t = 0; t < nb; ++t)
      for (int k = 0; k < 3; ++k) qb[t + nb * k] = q[3 * (t0 + t) + k];
    pp_result_view rv{m.data(), nz.data(), w.data(), n, z.empty() ? nullptr : z.data(), n, 2 * n * mz,
                      vel.empty() ? nullptr : vel.data(), 3 * n, nullptr};
    check(pp_solve_batch(ctx, qb.data(), nb, nb, &o, &rv, info.data()), "pp_solve_batch");
    for (int64_t b = 0; b < nb; ++b) {
      const int64_t t = t0 + b;
      if (info[b]) fprintf(stderr, "q-point %lld: eigensolver info %lld\n", (long long)(t + 1), (long long)info[b]);
      double qv[3] = {q[3 * t], q[3 * t + 1], q[3 * t + 2]};
      std::vector<h5min::Writer::Item> items;
      items.push_back({"q_vec", {3}, qv, false});
      items.push_back({"eigenvalues", {(uint64_t)m[b]}, w.data() + b * n, false});
      if (cfg.compute_eigvecs)  // column j of z is row j of evec (nz, 3N)
        items.push_back({"evec", {(uint64_t)nz[b], (uint64_t)n}, z.data() + (size_t)b * 2 * n * mz, true});
      if (cfg.group_velocity) items.push_back({"vel", {(uint64_t)nz[b], 3}, vel.data() + b * 3 * n, false});
      char name[32];
      snprintf(name, sizeof name, "%012lld", (long long)(t + 1));
      wr.add_group(name, items);
    }
    progress(cfg.print_progress, "q-points " + std::to_string(t0 + 1) + "-" + std::to_string(t0 + nb) + " of " +
                                     std::to_string(nq) + " solved (n = " + std::to_string(n) + ")");
  }
  wr.close();
  progress(cfg.print_progress, "Results written to " + out_path);
  return dir + "/" + out_path;
}

}  // namespace

int main(int argc, char **argv) {
  try {
    if (argc >= 3 && !strcmp(argv[1], "--parse-input")) return parse_input_mode(argv[2]);
    if (argc >= 4 && !strcmp(argv[1], "--h5-keys")) return h5_keys_mode(argv[2], argv[3]);
    if (argc >= 4 && !strcmp(argv[1], "--h5-read")) return h5_read_mode(argv[2], argv[3]);
    if (argc >= 4 && !strcmp(argv[1], "--h5-copy")) return h5_copy_mode(argv[2], argv[3]);
    if (argc >= 6 && !strcmp(argv[1], "--read-lammps")) return read_lammps_mode(argv[2], argv[3], argv[4], argv[5]);
    std::string input;
    int precision = PP_PREC_MIXED;
    int64_t batch = 0;
    bool quiet = false;
    for (int i = 1; i < argc; ++i) {
      if (!strcmp(argv[i], "--precision") && i + 1 < argc) {
        const std::string p = argv[++i];
        if (p == "mixed")
          precision = PP_PREC_MIXED;
        else if (p == "fp64")
          precision = PP_PREC_FP64;
        else
          throw std::runtime_error("--precision must be mixed or fp64");
      } else if (!strcmp(argv[i], "--batch") && i + 1 < argc) {
        batch = std::stoll(argv[++i]);
      } else if (!strcmp(argv[i], "--quiet")) {
        quiet = true;
      } else if (input.empty()) {
        input = argv[i];
      } else {
        throw std::runtime_error(std::string("unexpected argument ") + argv[i]);
      }
    }
    if (input.empty()) {
      fprintf(stderr, "usage: %s <input file> [--precision mixed|fp64] [--batch B] [--quiet]\n", argv[0]);
      return 2;
    }
    printf("%s\n", run(input, precision, batch, quiet).c_str());
    return 0;
  } catch (const std::exception &e) {
    fprintf(stderr, "parphom_gpu.x: %s\n", e.what());
    return 1;
  }
}
