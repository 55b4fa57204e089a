// Internal declarations shared by the library's translation units.
#pragma once
#include <cstdint>
#include <cstdio>
#include <vector>
#include <cuda_runtime.h>

#include "pp_common.cuh"

namespace pp {

// Counts kernel launches made by this library (pp_kernel_launches()).
void count_launch(int64_t k = 1);

// Kernel attributes (cudaFuncSetAttribute) and device properties apply to
// one device: caches of them are kept per device index, 0 .. PP_MAX_DEVICES-1.
constexpr int PP_MAX_DEVICES = 64;
// The current device's index, or -1 if it cannot be read or is out of range.
int device_index();
// Number of SMs of the current device (cached per device; 1 if unknown).
int device_sms();

// Optional per-launch CUDA-event timing of selected kernel classes
// (pp_ktimer_enable / pp_ktimer_report).
enum KClass {
  KT_ASSEMBLE = 0, KT_COLUPD, KT_REFL, KT_HEMV, KT_DOTS, KT_WCORR, KT_WFIN, KT_HER2K, KT_BISECT, KT_INVIT,
  KT_VHX, KT_BTRED, KT_APPLYV, KT_VEL, KT_XHZ, KT_N
};
extern unsigned kt_mask;
void kt_begin(int k, cudaStream_t s);
void kt_end(int k, cudaStream_t s);
#define PP_KT(k, s, launch)                         \
  do {                                              \
    const bool on__ = (pp::kt_mask >> (k)) & 1u;    \
    if (on__) pp::kt_begin((k), (s));               \
    launch;                                         \
    if (on__) pp::kt_end((k), (s));                 \
  } while (0)

// Per-batch state of the eigensolver.  Every matrix b of a batch of `B`
// Hermitian matrices has its own order nvec[b] <= nmax; all buffers use the
// leading dimensions of the largest.  Complex buffers hold 16-byte elements:
// z64 for the FP64 form, zdf for the double-float form.
struct EigWork {
  int B = 0;           // matrices in the batch
  int boff = 0;        // index of the first matrix in the whole batch (views)
  int nmax = 0;        // largest order
  int mcap = 0;        // eigenvector columns allocated per matrix
  int nb = 32;         // panel width
  int hemv_bps = 6;    // persistent blocks per SM of the Hermitian mat-vec (autotuned)
  int *nvec = nullptr; // [B] device: order of each matrix

  void *A = nullptr;   // [B][nmax*nmax]  D(q), overwritten by the reduction
  int64_t lda = 0, sA = 0;
  void *E = nullptr;   // [B][nmax*mcap]  eigenvectors
  int64_t lde = 0, sE = 0;
  void *W = nullptr;   // [B][nmax*nb]    zlatrd W panel
  void *P = nullptr;   // [B][nchunk*nmax] hemv partial sums
  int nchunk = 0;
  void *X = nullptr;   // [B][2*nb]       V^H v and W^H v
  double *nrm = nullptr;  // [B][nrb]     partial column norms
  z64 *wv = nullptr;      // [B][nrb]     partial w^H v
  int nrb = 0;            // partial-sum slots per matrix (>= row blocks of any column kernel)
  double *d = nullptr;    // [B][nmax] tridiagonal diagonal
  double *e = nullptr;    // [B][nmax] off-diagonal (real)
  z64 *tau = nullptr;     // [B][nmax] reflector scalars
  z64 *scal = nullptr;    // [B][4]    per-column scalars (scale, tau, alpha)

  // tridiagonal eigen stage
  double *w = nullptr;    // [B][nmax] eigenvalues (ascending)
  int64_t *rng = nullptr; // [B][8]  il, iu, m, flags...
  double *tinfo = nullptr;// [B][8]  gl, gu, tnorm, pivmin
  int *cls = nullptr;     // [B][nmax+1] cluster starts
  int *ncl = nullptr;     // [B]
  double *scratch = nullptr; // inverse-iteration LU factors and vector [B][5*nmax*T]
  uint8_t *piv = nullptr;    // inverse-iteration pivot flags [B][nmax*T]
  int64_t scratch_threads = 0;  // T: clusters handled per launch
  int64_t *info = nullptr;   // [B] info bits

  // back-transform
  z64 *Tf = nullptr;      // [npanels][B][32*32] compact-WY factors of all panels
  int64_t sTfp = 0;       // panel stride of Tf (the full batch's B * 1024)
  void *Wb = nullptr;     // [B][32*ldwp]     T V^H E
  void *Wp = nullptr;     // [B][ksplit][32*ldwp] split-K partials
  int ksplit = 0;
  int ldwp = 0;

  // velocities-only back-transform: boundary rows of E (see back_transform_rows)
  void *Xr = nullptr;     // [B][nmax*nbr]  Q^H P^T
  void *Eb = nullptr;     // [B][nbr*mcap]  rows of E = Q Z
  int nbr = 0;

  // tensor-core trailing update (double-float form): bf16 slices of the
  // panel rows, their exponents, and a per-matrix time-out flag
  uint8_t *tcS = nullptr; // [B][her2k_tc_bytes(nmax)]
  int64_t sTcS = 0;
  int *tcE = nullptr;     // [B][her2k_tc_exps(nmax)] (V, W) exponent pairs per row
  int64_t sTcE = 0;
  int *tcErr = nullptr;   // [B]

  size_t bytes = 0;
};

struct Geometry {
  int64_t natom = 0, n = 0;
  double lat[9];       // Fortran lat(i,j) at lat[(i-1)+3*(j-1)]
  double rec_lat[9];   // 2 pi_f (lat^-1)^T, as lammps_read.F90:228
  double delta_crys[3][3];  // CD step in reduced coordinates per direction
  double delta_norm[3];
  double *d_fc = nullptr;       // n*n Phi, upper triangle mirrored to lower
  double *d_crys = nullptr;     // natom*3
  double *d_pos = nullptr;      // natom*3
  double *d_mass = nullptr;     // natom (mass of each atom)
  uint16_t *d_mask = nullptr;   // natom*natom image tie sets, (min,max) orientation
  int64_t nbnd = 0;             // boundary blocks (I<J, non-home image, Phi != 0)
  int2 *d_bnd = nullptr;        // [nbnd] (I, J)
  uint16_t *d_bndmask = nullptr;// [nbnd]
  int64_t nbrows = 0;           // rows of atoms that appear in boundary blocks
  int *d_brows = nullptr;       // [nbrows] sorted row indices
  int *d_rowmap = nullptr;      // [n] compact index of a boundary row, -1 otherwise
};

// ---- kernels launched from pp_capi.cu -------------------------------------
cudaError_t geom_build_masks(Geometry &g, cudaStream_t s);
cudaError_t geom_symmetrize_fc(Geometry &g, int enforce_asr, cudaStream_t s);
cudaError_t geom_block_nonzero(const Geometry &g, uint8_t *d_flags, cudaStream_t s);

// D(q) for B q-points into 16-byte complex storage (z64 if dfmt==0, zdf if 1).
cudaError_t assemble_batch(const Geometry &g, const double *d_q, int B, void *A, int64_t lda, int64_t sA,
                           int dfmt, cudaStream_t s);
// dD/dq_k (derivative 1..3, method 'A' or 'C') or D (derivative 0), FP64.
cudaError_t assemble_deriv(const Geometry &g, const double *d_q, int derivative, char method, z64 *out,
                           int64_t ldo, cudaStream_t s);

// Group velocities: vel[b][3][m] (raw Re e^H dD e), E in 16-byte storage.
// With rowmap != nullptr, E holds only the boundary rows (row r of the full
// matrix at E[rowmap[r] + lde*j]).
cudaError_t velocities(const Geometry &g, const double *d_q, int B, const void *E, int64_t lde, int64_t sE,
                       int efmt, const int64_t *d_rng, int mmax, char method, double *d_vraw, double *d_part,
                       int nsplit, const int *rowmap, cudaStream_t s);

// G(r,c) += Re(M(c,r) p(r,c)), M = Z diag(wgt) Z^H for one q (FP64 Z, m columns).
cudaError_t backward_phi(const Geometry &g, const double *d_q, const z64 *Z, int64_t ldz, int m, const double *wgt,
                         double *G, int prec, cudaStream_t s);

// Eigen stages, templated on the real type (double / df) in pp_eigen.cu.
template <class R>
cudaError_t tridiagonalize(EigWork &w, cudaStream_t s);
// Trailing update of panel k0 on the tensor cores (double-float storage).
cudaError_t her2k_tc(EigWork &w, int k0, int jb, cudaStream_t s);
// X(k0+1:n, 0:ncols) -= V Y (compact-WY back-transform update) on the tensor
// cores: V the Householder vectors of panel k0, Y (jb x ncols) at Yb[a ldy + c].
cudaError_t applyV_tc(EigWork &w, int k0, int jb, zdf *X, int64_t ldx, int64_t sX, const zdf *Yb, int64_t ldy,
                      int64_t sY, int ncols, cudaStream_t s);
// Wp(a, c) = (V^H X)(a, c) on the tensor cores, split over vhx_tc_splits(w)
// row ranges into the first split-K slots of Wp.
int vhx_tc_splits(const EigWork &w);
// Eb(k, j) = sum_r conj(X(r, k)) Z(r, j) on the tensor cores (Z real, stored
// as complex with zero imaginary part), j < m of each matrix.
cudaError_t xhz_tc(EigWork &w, const zdf *X, int64_t ldx, int64_t sX, int nrows, const zdf *Z, int64_t ldz,
                   int64_t sZ, zdf *Eb, int64_t lde, int64_t sE, cudaStream_t s);
cudaError_t vhx_tc(EigWork &w, int k0, int jb, const zdf *X, int64_t ldx, int64_t sX, int ncols, zdf *Wp,
                   int64_t ldwp, int64_t sWp, cudaStream_t s);
size_t her2k_tc_bytes(int64_t nmax);
int64_t her2k_tc_exps(int64_t nmax);
cudaError_t prepare_her2k_tc();
bool tc_enabled();
// Test hook: the next tensor-core trailing update that covers batch matrix
// `matrix` makes its first wait give up after `cycles` SM clocks.
void arm_tc_stall(int64_t matrix, long long cycles);
bool tc_stall_armed();
cudaError_t prepare_bisect(size_t bytes);
// dynamic shared memory of the bisection kernel for order n (0: global-memory mode)
size_t bisect_smem(int64_t n, int mixed);
cudaError_t tridiag_eigenvalues(EigWork &w, char range, double vl, double vu, int64_t il, int64_t iu,
                                double abstol, cudaStream_t s, int mixed = 0);
template <class R>
cudaError_t tridiag_eigenvectors(EigWork &w, cudaStream_t s);
template <class R>
cudaError_t back_transform(EigWork &w, cudaStream_t s);
// Rows `rows` of E = Q Z only: X = Q^H P^T (P selects the rows), Eb = X^H Z.
template <class R>
cudaError_t back_transform_rows(EigWork &w, const int *d_rows, int nrows, cudaStream_t s);

// Per-eigenpair error estimates (residual, eigenvalue and eigenvector error
// bounds) of the eigenpairs in w (full eigenvectors in w.E), FP64; D(q) is
// assembled again into w.A.  sums: 3 * B * mcap doubles of scratch.
cudaError_t error_estimates(const Geometry &g, const double *d_q, EigWork &w, int efmt, int raw_lambda,
                            double *sums, double *resid, double *werr, double *zerr, int64_t ldw, cudaStream_t s);

// Output conversion
cudaError_t finalize_outputs(EigWork &w, int efmt, int raw_lambda, const double *d_vraw, int want_vel, int want_z,
                             double *w_out, int64_t ldw, double *z_out, int64_t ldz, int64_t zstride, double *vel_out,
                             int64_t velstride, int64_t *m_out, int64_t *nz_out, int64_t *info_out, int jobz_v,
                             cudaStream_t s);

}  // namespace pp

#define PP_CUDA_TRY(x)                  \
  do {                                  \
    cudaError_t err__ = (x);            \
    if (err__ != cudaSuccess) return err__; \
  } while (0)
