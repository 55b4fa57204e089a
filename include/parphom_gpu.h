/*
 * parphom_gpu.h — C ABI of the GB300 phonon hot path (libparphom_gpu.so).
 *
 * The library replaces, for one GPU, the body of PARPHOM's per-q loop
 * (Phonon_Calculations/SRC/calculations.F90:49-53):
 *
 *   create_dynamical_matrix(q, 0)     dynamical_matrix.F90:49-262
 *   diagonalize_dynamical_matrix()    diagonalize.F90:42-149   (pzheevx)
 *   velocity block of write_output    write_output.F90:334-466 (dD/dq, pzgemm)
 *
 * with one call per batch of q-points.  The Fortran driver keeps input
 * parsing, HDF5 I/O and MPI; it calls this header through ISO_C_BINDING
 * (the interface module is shown in INTEGRATION.md).  All integers are
 * explicit 64-bit (the reference builds with -i8, Makefile.intel:18), all
 * arrays are plain column-major buffers, and no call exits the process.
 *
 * Return codes: 0 success; -k the k-th argument is illegal (LAPACK
 * convention); positive PP_ERR_* library errors below.  Per-q eigensolver
 * status is reported separately in info[] with the pzheevx INFO bits
 * (diagonalize.F90:100-115).
 */
#ifndef PARPHOM_GPU_H
#define PARPHOM_GPU_H
#include <stdint.h>

#if defined(__GNUC__)
#define PP_API __attribute__((visibility("default")))
#else
#define PP_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pp_ctx pp_ctx;

/* Library error codes (positive). */
#define PP_OK 0
#define PP_ERR_CUDA 1001      /* a CUDA runtime call failed                    */
#define PP_ERR_NOMEM 1002     /* device allocation failed                      */
#define PP_ERR_NAN 1003       /* non-finite value in force constants or q      */
#define PP_ERR_TIMEOUT 1004   /* a bounded device wait gave up                 */
#define PP_ERR_NODEVICE 1005  /* no CUDA device / kernel image not loadable    */
#define PP_ERR_STATE 1006     /* context used after an unrecoverable error     */
#define PP_ERR_UNSUPPORTED 1007
#define PP_ERR_SIZE 1008      /* order beyond a fixed-capacity entry point    */

/* Per-q info bits, as pzheevx INFO > 0 (diagonalize.F90:100-115). */
#define PP_INFO_NOCONV 1      /* an eigenvalue failed to converge              */
#define PP_INFO_NOORTH 2      /* a cluster of eigenvectors not orthogonalised  */
#define PP_INFO_NOMEM 4       /* workspace too small for all eigenvectors      */
#define PP_INFO_NOTCOMP 8     /* an eigenvalue was not computed                */
#define PP_INFO_TIMEOUT 16    /* a bounded device wait gave up: results invalid */
#define PP_INFO_NAN 32        /* non-finite input found on the device (entry
                                 points whose input is device memory only):
                                 no eigenvalues returned                      */

/* Precision forms. */
#define PP_PREC_FP64 0        /* plain IEEE double throughout                  */
#define PP_PREC_MIXED 1       /* reduction and back-transform in double-float
                                 on the FP32 pipes, the trailing update on the
                                 tensor cores (exact bf16 slice products),
                                 FP64 inverse iteration and velocities       */

/* pp_ctx_create flags. */
#define PP_FLAG_ENFORCE_ASR 1 /* reset Phi_II = -sum_{J!=I} Phi_IJ (off by
                                 default: the reference does not)              */

/* The reference's `system` type (mod_variables.F90:83-89) as explicit
 * arguments.  Column-major like the Fortran module arrays. */
typedef struct pp_system {
  int64_t natom;
  int64_t ntypes;
  const double *lat;      /* [9]  lat(i,j) at lat[(i-1)+3*(j-1)]; row i = a_i (A)   */
  const double *crys;     /* [natom*3] crys(I,k) at crys[(I-1)+natom*(k-1)]          */
  const double *real_pos; /* [natom*3] real_pos(I,k), Cartesian (A)                  */
  const double *mass;     /* [ntypes] amu                                            */
  const int64_t *at_types;/* [natom] 1-based type of each atom                       */
} pp_system;

/* The reference's scalapack_variables + velocity switches
 * (mod_variables.F90:77-81, read_input.F90:141-218). */
typedef struct pp_eig_opts {
  char jobz;          /* 'N' eigenvalues only, 'V' eigenvectors too              */
  char range;         /* 'A' all, 'I' indices il..iu, 'V' values in (vl,vu]      */
  char vel_method;    /* 'A' analytic dD/dq, 'C' central difference             */
  char uplo;          /* must be 'U' (the reference passes 'U')                 */
  int32_t vel;        /* nonzero: group velocities (forces jobz = 'V')           */
  int32_t precision;  /* PP_PREC_FP64 or PP_PREC_MIXED                           */
  double vl, vu;      /* range 'V' bounds in the reference's units: they are
                         divided by 15.633302*33.35641 and compared with the
                         eigenvalues of D (diagonalize.F90:75,94)               */
  int64_t il, iu;     /* range 'I', 1-based                                      */
  double abstol;      /* bisection absolute tolerance (reference default 1e-15) */
  double orfac;       /* accepted for interface parity; clusters are formed by
                         the library's own relative-gap rule                    */
  int32_t raw_lambda; /* nonzero: w holds eigenvalues of D instead of cm^-1    */
  int32_t want_resid; /* nonzero: per-eigenpair error estimates in FP64 into
                         resid[], werr[], zerr[] of the result view (needs the
                         full eigenvectors: computed internally if not asked
                         for; costs an FP64 product D Z per q-point)         */
} pp_eig_opts;

/* Output buffers for nq q-points (host or device memory depending on call).
 * For q index t (0-based) and mode j:
 *   w[j + ldw*t]                      frequency in cm^-1 (or lambda)
 *   z[2*(r + ldz*j) + zstride*t]      (re, im) of eigenvector j, row r
 *   vel[d + 3*j + velstride*t]        group velocity, direction d, m/s
 * With want_resid (each may be NULL), computed in FP64 against D(q)
 * assembled in FP64, for the normalised eigenpair (lambda_j, z_j):
 *   resid[j + ldw*t]  ||D z - lambda z||_2 (units of D)
 *   werr[j + ldw*t]   estimated bound on the error of w[j] (cm^-1, or lambda
 *                     units with raw_lambda): min(resid, |lambda - rho| +
 *                     ||D z - rho z||^2 / gap), rho the Rayleigh quotient,
 *                     gap the distance to the nearest other computed
 *                     eigenvalue, carried through sign(l) sqrt|l|
 *   zerr[j + ldw*t]   estimated bound on sin(angle) between z_j and the exact
 *                     eigenvector: min(1, ||D z - rho z|| / gap) (large inside
 *                     clusters of near-degenerate modes)                    */
typedef struct pp_result_view {
  int64_t *m;         /* [nq] number of eigenvalues found (comp_num_eval)     */
  int64_t *nz;        /* [nq] number of eigenvectors (comp_num_evec)          */
  double *w;
  int64_t ldw;
  double *z;          /* may be NULL when eigenvectors are not wanted         */
  int64_t ldz;
  int64_t zstride;    /* in doubles                                           */
  double *vel;        /* may be NULL                                          */
  int64_t velstride;  /* in doubles                                           */
  double *resid;      /* may be NULL                                          */
  double *werr;       /* may be NULL                                          */
  double *zerr;       /* may be NULL                                          */
} pp_result_view;

/* Create a context on the current CUDA device: uploads Phi (after the
 * driver's symmetrisation, force_read.F90:187-189) and builds the q-
 * independent geometry tables.  Only the upper triangle of fc is referenced,
 * as pzheevx references only the upper triangle of D (diagonalize.F90:73).
 * Replaces: the state set up by read_lammps_data / read_force_constants
 * (main.F90:53-62) as seen by create_dynamical_matrix. */
PP_API int pp_ctx_create(const pp_system *sys, const double *fc, int64_t ldfc, int64_t flags, pp_ctx **out);

/* Replace the force constants of a context, keeping its geometry tables:
 * Phi is copied (host memory, or device memory with fc_on_device = 1: e.g.
 * a torch tensor of the differentiation layer, column-major with ld ldfc,
 * upper triangle referenced), symmetrised as at creation and the boundary
 * block tables rebuilt from its non-zero blocks.  Synchronous.  No
 * counterpart in the reference (one Phi per run); used when fitting force
 * constants, where Phi changes between forward passes. */
PP_API int pp_ctx_update_fc(pp_ctx *ctx, const double *fc, int64_t ldfc, int64_t flags, int32_t fc_on_device);

/* Free every device resource of the context. */
PP_API int pp_ctx_destroy(pp_ctx *ctx);

/* Solve nq q-points: q(t,k) at q[t + ldq*k] in reduced reciprocal
 * coordinates (q_file%points, q_read.F90:82-93).  Host buffers in and out;
 * the library batches internally.  info[t] receives the pzheevx-style bits.
 * Replaces: calculations.F90:50-52 (minus the HDF5 writes). */
PP_API int pp_solve_batch(pp_ctx *ctx, const double *q, int64_t ldq, int64_t nq, const pp_eig_opts *opts,
                   const pp_result_view *out, int64_t *info);

/* Same as pp_solve_batch with q, the result buffers and info in device
 * memory, enqueued on `stream` (a cudaStream_t; NULL = legacy stream). */
PP_API int pp_solve_batch_device(pp_ctx *ctx, const double *q_dev, int64_t ldq, int64_t nq, const pp_eig_opts *opts,
                          const pp_result_view *out_dev, int64_t *info_dev, void *stream);

/* Several cells (contexts of different sizes) in one launch sequence: q-point
 * t (q[t + ldq*k]) belongs to cell ctxs[cell[t]].  The q-points are grouped
 * by cell into batches of mixed orders; assembly and velocities run per cell,
 * the reduction, bisection, inverse iteration and back-transform once per
 * batch (every kernel carries each matrix's own order).  Outputs as for
 * pp_solve_batch with ldw (and ldz) at least the largest 3N; the workspace
 * belongs to ctxs[0] and is released at the end.  No counterpart in the
 * reference, which runs one cell per program. */
PP_API int pp_solve_multi(pp_ctx *const *ctxs, int64_t nctx, const int64_t *cell, const double *q, int64_t ldq,
                          int64_t nq, const pp_eig_opts *opts, const pp_result_view *out, int64_t *info);

/* Density of states by linear triangulation (Utilities/pyphutil/
 * fortran_routines/bz_integration.f90:12-133, called from
 * pyphutil.py:214-322): freq[k*ldf + b] is band b at grid point k (cm^-1),
 * func the same layout (NULL: all ones), tri[3*j + v] the vertices of
 * triangle j.  dos[i] and nd[i] receive the sums over triangles and bands of
 * the per-triangle contributions at energy[i] (unnormalised, as the Fortran
 * routine returns them).  Host buffers. */
PP_API int pp_dos_triangulation(const double *freq, int64_t ldf, int64_t nk, int64_t nbands, const double *func,
                                const int64_t *tri, int64_t ntri, const double *energy, int64_t ne, double *dos,
                                double *nd);

/* Gaussian (method 1) or Lorentzian (method 2) smearing DOS
 * (bz_integration.f90:154-199): dos[i] = sum_q weights[q] sum_b
 * g(freq[q*ldf+b], energy[i], width) / natom.  Host buffers. */
PP_API int pp_dos_smearing(int32_t method, const double *freq, int64_t ldf, int64_t nq, int64_t nbands,
                           const double *weights, double width, const double *energy, int64_t ne, int64_t natom,
                           double *dos);

/* Device-resident forms of the two DOS entry points, fed straight from the
 * outputs of pp_solve_batch_device (no host round trip, no HDF5 file):
 * freq_dev is its w output (freq_dev[q*ldf + b], ldf = its ldw), func_dev an
 * optional per-(q, band) weight with its own leading dimension ldfunc (e.g.
 * from pp_velocity_weights_device: the transport DOS), tri_dev, energy_dev,
 * weights_dev and the outputs (ne doubles each) all device memory.  Results
 * as pp_dos_triangulation / pp_dos_smearing; the bands are summed in a
 * different order (last-bit differences).  Enqueued on `stream`; nothing is
 * allocated.  Replaces the same routines as the host forms
 * (bz_integration.f90:12-199 as called from pyphutil.py:214-359). */
PP_API int pp_dos_triangulation_device(const double *freq_dev, int64_t ldf, int64_t nk, int64_t nbands,
                                       const double *func_dev, int64_t ldfunc, const int64_t *tri_dev, int64_t ntri,
                                       const double *energy_dev, int64_t ne, double *dos_dev, double *nd_dev,
                                       void *stream);
PP_API int pp_dos_smearing_device(int32_t method, const double *freq_dev, int64_t ldf, int64_t nq, int64_t nbands,
                                  const double *weights_dev, double width, const double *energy_dev, int64_t ne,
                                  int64_t natom, double *dos_dev, void *stream);

/* Weights of a velocity-weighted (transport) DOS from the velocity output
 * of pp_solve_batch_device (vel_dev[q*velstride + 3*j + d], m/s):
 * func_dev[q*ldfunc + j] = v_a v_b of mode j (a, b in 0..2: x, y, z), or
 * |v|^2 with a = b = -1.  The func argument of pyphutil's
 * density_of_states (pyphutil.py:214-260), built on the device.  Enqueued on
 * `stream`. */
PP_API int pp_velocity_weights_device(const double *vel_dev, int64_t velstride, int64_t nq, int64_t nbands, int32_t a,
                                      int32_t b, double *func_dev, int64_t ldfunc, void *stream);

/* D(q) (derivative = 0) or dD/dq_k (derivative = k in 1..3, vel_method 'A'
 * or 'C') for one q, written as the full Hermitian matrix (upper triangle
 * mirrored) to host buffer d[2*(r + ldd*c)].
 * Replaces: create_dynamical_matrix(q_indx, derivative),
 * dynamical_matrix.F90:49-191. */
PP_API int pp_dynamical_matrix(pp_ctx *ctx, const double *q, int64_t derivative, char vel_method, double *d,
                        int64_t ldd);

/* Backward pass for the force constants (no counterpart in the reference;
 * the differentiation layer of the Python package uses it).  For nq
 * q-points in device memory (q_dev[3*t + k], reduced coordinates), their
 * eigenvectors z_dev (FP64 complex, z[2*(r + ldz*j) + zstride*t], m
 * columns) and weights wgt_dev[j + ldwgt*t] = dL/dlambda_j, adds to the
 * symmetric n x n device matrix g_dev (column-major, ld n)
 *   g(r,c) += sum_t Re(M_t(c,r) p_t(r,c)),  M_t = Z_t diag(wgt_t) Z_t^H,
 * p_t being the phase/mass factor of D(q_t)(r,c) built from the upper
 * triangle; i.e. dL/dPhi for a symmetric Phi.  precision PP_PREC_FP64 or
 * PP_PREC_MIXED (double-float accumulation).  Enqueued on `stream`. */
PP_API int pp_backward_phi(pp_ctx *ctx, const double *q_dev, int64_t nq, const double *z_dev, int64_t ldz,
                           int64_t zstride, int64_t m, const double *wgt_dev, int64_t ldwgt, double *g_dev,
                           int32_t precision, void *stream);

/* Human-readable text for a return code. */
PP_API const char *pp_strerror(int code);

/* Library version: major*10000 + minor*100 + patch. */
PP_API int64_t pp_version(void);

/* Number of kernels this library launched on the calling thread's contexts
 * since load (for launch accounting in benchmarks). */
PP_API int64_t pp_kernel_launches(void);

/* Largest matrix order pp_heevx_values_noalloc accepts. */
#define PP_NOALLOC_MAX_N 1536

/* Eigenvalues of one Hermitian matrix with no device allocation at all.
 * No counterpart in the reference: it exists for callers that cannot
 * allocate device memory — drivers that hand over a fixed device pool and
 * forbid hidden allocations, stream-ordered pipelines the caller does not
 * own (where an allocation would synchronise the device), and long runs that
 * must not grow the device footprint.  The FP64 reduction and bisection use
 * one fixed scratch array of about 2.0 MB compiled into the library, which
 * every GPU that loads the library keeps until exit.
 *   a_dev   n x n complex FP64 column-major device matrix, ld lda; only the
 *           upper triangle is read (as pzheevx with uplo 'U'); overwritten.
 *           A non-finite element gives info PP_INFO_NAN and m = 0.
 *   n       1 <= n <= PP_NOALLOC_MAX_N, else PP_ERR_SIZE; lda <= 1536 too.
 *   range   'A', 'I' (il..iu, 1-based) or 'V' (eigenvalues in (vl, vu],
 *           bounds in the matrix's own units), abstol as in pzheevx.
 *   w_dev   [n] eigenvalues ascending (first *m_dev valid); m_dev, info_dev
 *           one int64 each (info: pzheevx-style bits); all device memory.
 * Enqueued on `stream`.  The first call on a device resolves the array's
 * address (cudaGetSymbolAddress) with that device current: make that first
 * call before any stream capture, and do not use the entry point across a
 * cudaDeviceReset (the address is kept for the life of the process).  All
 * calls share the one array and leave their contents in it (each call resets
 * what must start at zero); calls that overlap on the GPU (different streams
 * or threads running at once) race on it.  Do not enable pp_ktimer_enable
 * around it (the timer creates CUDA events). */
PP_API int pp_heevx_values_noalloc(double *a_dev, int64_t lda, int64_t n, char range, double vl, double vu,
                                   int64_t il, int64_t iu, double abstol, double *w_dev, int64_t *m_dev,
                                   int64_t *info_dev, void *stream);

/* Instrumentation (no counterpart in the reference): record CUDA events
 * around every launch of the named kernel classes (comma separated, e.g.
 * "hemv,vhx,applyV"; NULL or "" disables) and report, one line per class,
 * "<class> <launches> <total milliseconds>". */
PP_API int pp_ktimer_enable(const char *names);
PP_API int pp_ktimer_report(char *buf, int64_t len);

/* The launch configurations the autotuner chose in this process, one line
 * per (device, order, batch size, options): the number of streams a batch
 * is split over and the persistent blocks per SM of the Hermitian mat-vec,
 * with the batch's GPU time.  The first solve of each combination times the
 * candidates on its own first batch (PARPHOM_GPU_TUNE=0 or an explicit
 * PARPHOM_GPU_SPLIT turns this off).  No counterpart in the reference. */
PP_API int pp_autotune_report(char *buf, int64_t len);

/* Test hook for the bounded device waits (no counterpart in the reference).
 * Arms a one-shot stall: the next mixed-form tensor-core trailing update
 * whose batch contains batch matrix `matrix` (0-based index within one
 * pp_solve_batch batch) waits, before its first copy wait, on a barrier that
 * nothing completes, for at most `cycles` SM clocks (0 .. 2e9), then takes
 * the time-out path: it waits (bounded) for its own copies in flight, frees
 * its tensor memory and returns; later launches skip that matrix and its
 * info gets PP_INFO_TIMEOUT.  matrix = -1 disarms.  The call that consumes
 * the stall runs without the captured graph. */
PP_API int pp_debug_stall_tc_wait(int64_t matrix, int64_t cycles);

#ifdef __cplusplus
}
#endif
#endif /* PARPHOM_GPU_H */
