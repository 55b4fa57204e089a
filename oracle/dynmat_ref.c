/*
 * ORACLE — test infrastructure only.  This file is the CPU restatement of the
 * reference's dynamical-matrix element routine, used by tests/, by the
 * smoke check and by bench.py's CPU-baseline leg as the checker.  It is
 * never linked into, or called by, the GPU library.
 *
 * Restated from qtm-iisc/PARPHOM:
 *   Phonon_Calculations/SRC/dynamical_matrix.F90:200-262  create_dynamical_ij
 *   Phonon_Calculations/SRC/dynamical_matrix.F90:127-149  derivative modes
 *   Phonon_Calculations/SRC/lammps_read.F90:250-309       matinvtransp3, linsolve
 *
 * Arrays follow the Fortran driver (column-major, 1 rank => LLD = n):
 *   lat[i + 3*j]          = moire%lat(i+1, j+1), row i = lattice vector a_i
 *   crys[I + natom*k]     = moire%crys(I+1, k+1)
 *   real_pos[I + natom*k] = moire%real_pos(I+1, k+1)
 *   mass_atom[I]          = moire%mass(moire%at_types_i(I+1))
 *   fc[r + n*c]           = force_const%mat  (n = 3*natom)
 *   out[2*(r + n*c)+{0,1}] = (re, im) of D(r, c)
 *
 * The Fortran source writes several constants as default-REAL (single
 * precision) literals assigned to double-precision parameters; their values
 * are therefore the float-rounded numbers, reproduced here bit for bit:
 *   PI  = 3.141592653589793   -> (double)3.141592653589793f
 *   tol = 1e-10               -> (double)1e-10f
 *   DEL_INCREMENT = 1e-6      -> (double)1e-6f
 *   PI2 = 6.283185307179586   -> (double)6.283185307179586f
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define PI_REF ((double)3.141592653589793f)
#define TOL_REF ((double)1e-10f)
#define DEL_REF ((double)1e-6f)
#define PI2_REF ((double)6.283185307179586f)

/* lammps_read.F90:281-309 — u = B^T x with B = inverse of A (3x3). */
void oracle_linsolve(const double x[3], const double *A, double u[3]) {
#define AA(i, j) A[(i - 1) + 3 * (j - 1)]
  double detinv = 1.0 / (AA(1, 1) * AA(2, 2) * AA(3, 3) - AA(1, 1) * AA(2, 3) * AA(3, 2)
                         - AA(1, 2) * AA(2, 1) * AA(3, 3) + AA(1, 2) * AA(2, 3) * AA(3, 1)
                         + AA(1, 3) * AA(2, 1) * AA(3, 2) - AA(1, 3) * AA(2, 2) * AA(3, 1));
  double B[3][3];
  B[0][0] = +detinv * (AA(2, 2) * AA(3, 3) - AA(2, 3) * AA(3, 2));
  B[1][0] = -detinv * (AA(2, 1) * AA(3, 3) - AA(2, 3) * AA(3, 1));
  B[2][0] = +detinv * (AA(2, 1) * AA(3, 2) - AA(2, 2) * AA(3, 1));
  B[0][1] = -detinv * (AA(1, 2) * AA(3, 3) - AA(1, 3) * AA(3, 2));
  B[1][1] = +detinv * (AA(1, 1) * AA(3, 3) - AA(1, 3) * AA(3, 1));
  B[2][1] = -detinv * (AA(1, 1) * AA(3, 2) - AA(1, 2) * AA(3, 1));
  B[0][2] = +detinv * (AA(1, 2) * AA(2, 3) - AA(1, 3) * AA(2, 2));
  B[1][2] = -detinv * (AA(1, 1) * AA(2, 3) - AA(1, 3) * AA(2, 1));
  B[2][2] = +detinv * (AA(1, 1) * AA(2, 2) - AA(1, 2) * AA(2, 1));
#undef AA
  /* MATMUL(TRANSPOSE(B), x): u(i) = sum_k B(k,i) x(k) */
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int k = 0; k < 3; ++k) s += B[k][i] * x[k];
    u[i] = s;
  }
}

/* lammps_read.F90:250-274 — B = 2*pi_f * inverse-transpose of A. */
void oracle_matinvtransp3(const double *A, double *Bout) {
#define AA(i, j) A[(i - 1) + 3 * (j - 1)]
#define BB(i, j) Bout[(i - 1) + 3 * (j - 1)]
  double detinv = 1.0 / (AA(1, 1) * AA(2, 2) * AA(3, 3) - AA(1, 1) * AA(2, 3) * AA(3, 2)
                         - AA(1, 2) * AA(2, 1) * AA(3, 3) + AA(1, 2) * AA(2, 3) * AA(3, 1)
                         + AA(1, 3) * AA(2, 1) * AA(3, 2) - AA(1, 3) * AA(2, 2) * AA(3, 1));
  BB(1, 1) = +detinv * (AA(2, 2) * AA(3, 3) - AA(2, 3) * AA(3, 2)) * PI2_REF;
  BB(1, 2) = -detinv * (AA(2, 1) * AA(3, 3) - AA(2, 3) * AA(3, 1)) * PI2_REF;
  BB(1, 3) = +detinv * (AA(2, 1) * AA(3, 2) - AA(2, 2) * AA(3, 1)) * PI2_REF;
  BB(2, 1) = -detinv * (AA(1, 2) * AA(3, 3) - AA(1, 3) * AA(3, 2)) * PI2_REF;
  BB(2, 2) = +detinv * (AA(1, 1) * AA(3, 3) - AA(1, 3) * AA(3, 1)) * PI2_REF;
  BB(2, 3) = -detinv * (AA(1, 1) * AA(3, 2) - AA(1, 2) * AA(3, 1)) * PI2_REF;
  BB(3, 1) = +detinv * (AA(1, 2) * AA(2, 3) - AA(1, 3) * AA(2, 2)) * PI2_REF;
  BB(3, 2) = -detinv * (AA(1, 1) * AA(2, 3) - AA(1, 3) * AA(2, 1)) * PI2_REF;
  BB(3, 3) = +detinv * (AA(1, 1) * AA(2, 2) - AA(1, 2) * AA(2, 1)) * PI2_REF;
#undef AA
#undef BB
}

/* lammps_read.F90:198-200 — crys(I,:) = linsolve(real_pos(I,:), lat). */
void oracle_crys(int64_t natom, const double *lat, const double *real_pos, double *crys) {
  for (int64_t I = 0; I < natom; ++I) {
    double x[3] = {real_pos[I], real_pos[I + natom], real_pos[I + 2 * natom]}, u[3];
    oracle_linsolve(x, lat, u);
    for (int k = 0; k < 3; ++k) crys[I + natom * k] = u[k];
  }
}

/* dynamical_matrix.F90:200-262, for the 0-based element (r, c). */
static void dyn_ij(int64_t natom, const double *lat, const double *crys, const double *real_pos,
                   const double *mass_atom, double fcval, const double q[3], int64_t r, int64_t c,
                   int deriv_order, int derivative, double *dre, double *dim) {
  const int64_t inp_ia = r + 1, inp_ja = c + 1;
  const int64_t ia = (inp_ia + 2) / 3, ja = (inp_ja + 2) / 3; /* 1-based atoms */
  const int64_t I = ia - 1, J = ja - 1;
#define LAT(i, j) lat[(i - 1) + 3 * (j - 1)]
#define CRYS(a, k) crys[(a) + natom * ((k) - 1)]
#define POS(a, k) real_pos[(a) + natom * ((k) - 1)]
  double neigh[9];
  for (int l = 1; l <= 9; ++l) {
    int i = (l - 1) / 3 - 1;
    int j = l - 2 - 3 * (i + 1);
    double rs[3] = {CRYS(J, 1) + i, CRYS(J, 2) + j, CRYS(J, 3)};
    double rc[3];
    for (int a = 1; a <= 3; ++a) /* matmul(transpose(lat), rs) */
      rc[a - 1] = LAT(1, a) * rs[0] + LAT(2, a) * rs[1] + LAT(3, a) * rs[2];
    double dx = POS(I, 1) - rc[0], dy = POS(I, 2) - rc[1], dz = POS(I, 3) - rc[2];
    neigh[l - 1] = sqrt(dx * dx + dy * dy + dz * dz);
  }
  double minimum = neigh[0];
  for (int l = 1; l < 9; ++l)
    if (neigh[l] < minimum) minimum = neigh[l];
  double pre = 0.0, pim = 0.0;
  int mult = 0;
  for (int l = 1; l <= 9; ++l) {
    if (!(neigh[l - 1] < minimum + TOL_REF)) continue;
    int i = (l - 1) / 3 - 1;
    int j = l - 2 - 3 * (i + 1);
    double rs[3] = {CRYS(J, 1) + i - CRYS(I, 1), CRYS(J, 2) + j - CRYS(I, 2), CRYS(J, 3) - CRYS(I, 3)};
    double prephase = q[0] * rs[0] + q[1] * rs[1] + q[2] * rs[2];
    double theta = -((2.0 * PI_REF) * prephase);
    double cs = cos(theta), sn = sin(theta);
    if (deriv_order == 0) {
      pre += cs;
      pim += sn;
    } else {
      double rc[3];
      for (int a = 1; a <= 3; ++a) rc[a - 1] = LAT(1, a) * rs[0] + LAT(2, a) * rs[1] + LAT(3, a) * rs[2];
      double x = rc[derivative - 1];
      /* phase = phase - exp(...) * IM * x  with exp(...)*IM = (-sn, cs) */
      pre -= -sn * x;
      pim -= cs * x;
    }
    mult += 1;
  }
  /* dij = fc*phase/multiplicity ; dij = dij/sqrt(m_I*m_J) */
  double re = fcval * pre / (double)mult, im = fcval * pim / (double)mult;
  double s = sqrt(mass_atom[I] * mass_atom[J]);
  *dre = re / s;
  *dim = im / s;
#undef LAT
#undef CRYS
#undef POS
}

/* create_dynamical_matrix(q, derivative) for every element (all of it, both
 * triangles, as the reference's block-cyclic walk covers the full matrix).
 * vel_method: 'A' analytic, 'C' central difference (dynamical_matrix.F90:133-149). */
void oracle_dynamical_matrix(int64_t natom, const double *lat, const double *rec_lat, const double *crys,
                             const double *real_pos, const double *mass_atom, const double *fc,
                             const double q[3], int derivative, char vel_method, double *out) {
  const int64_t n = 3 * natom;
  double delta_crys[3] = {0, 0, 0}, dnorm = 1.0;
  if (derivative != 0 && vel_method != 'A') {
    double delta[3] = {0, 0, 0};
#define RL(i, j) rec_lat[(i - 1) + 3 * (j - 1)]
    double v = DEL_REF * sqrt(fabs(RL(1, 1) * RL(2, 2) - RL(1, 2) * RL(2, 1)));
    delta[derivative - 1] = v > DEL_REF ? v : DEL_REF;
#undef RL
    oracle_linsolve(delta, rec_lat, delta_crys);
    dnorm = sqrt(delta[0] * delta[0] + delta[1] * delta[1] + delta[2] * delta[2]);
  }
  for (int64_t c = 0; c < n; ++c) {
    for (int64_t r = 0; r < n; ++r) {
      double fcv = fc[r + n * c], re, im;
      if (derivative == 0) {
        dyn_ij(natom, lat, crys, real_pos, mass_atom, fcv, q, r, c, 0, 0, &re, &im);
      } else if (vel_method == 'A') {
        dyn_ij(natom, lat, crys, real_pos, mass_atom, fcv, q, r, c, 1, derivative, &re, &im);
      } else {
        double qp[3], qm[3], pr, pi, mr, mi;
        for (int k = 0; k < 3; ++k) {
          qp[k] = q[k] + delta_crys[k] / 2;
          qm[k] = q[k] - delta_crys[k] / 2;
        }
        dyn_ij(natom, lat, crys, real_pos, mass_atom, fcv, qp, r, c, 0, derivative, &pr, &pi);
        dyn_ij(natom, lat, crys, real_pos, mass_atom, fcv, qm, r, c, 0, derivative, &mr, &mi);
        re = (pr - mr) / dnorm;
        im = (pi - mi) / dnorm;
      }
      out[2 * (r + n * c)] = re;
      out[2 * (r + n * c) + 1] = im;
    }
  }
}

/* The per-pair image tie set used by dyn_ij, as a 9-bit mask (bit l-1 for
 * image l of dynamical_matrix.F90:223-237), for atoms (I, J) in the (ia, ja)
 * orientation.  Exported so tests can check the GPU geometry table. */
uint32_t oracle_image_mask(int64_t natom, const double *lat, const double *crys, const double *real_pos,
                           int64_t I, int64_t J) {
#define LAT(i, j) lat[(i - 1) + 3 * (j - 1)]
#define CRYS(a, k) crys[(a) + natom * ((k) - 1)]
#define POS(a, k) real_pos[(a) + natom * ((k) - 1)]
  double neigh[9];
  for (int l = 1; l <= 9; ++l) {
    int i = (l - 1) / 3 - 1;
    int j = l - 2 - 3 * (i + 1);
    double rs[3] = {CRYS(J, 1) + i, CRYS(J, 2) + j, CRYS(J, 3)};
    double rc[3];
    for (int a = 1; a <= 3; ++a) rc[a - 1] = LAT(1, a) * rs[0] + LAT(2, a) * rs[1] + LAT(3, a) * rs[2];
    double dx = POS(I, 1) - rc[0], dy = POS(I, 2) - rc[1], dz = POS(I, 3) - rc[2];
    neigh[l - 1] = sqrt(dx * dx + dy * dy + dz * dz);
  }
  double minimum = neigh[0];
  for (int l = 1; l < 9; ++l)
    if (neigh[l] < minimum) minimum = neigh[l];
  uint32_t mask = 0;
  for (int l = 1; l <= 9; ++l)
    if (neigh[l - 1] < minimum + TOL_REF) mask |= 1u << (l - 1);
  return mask;
#undef LAT
#undef CRYS
#undef POS
}
