// C ABI of the phonon hot path: context lifetime, workspace sizing and the
// per-batch pipeline  D(q) -> tridiagonal -> eigenvalues -> eigenvectors ->
// back-transform -> velocities -> outputs.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <new>
#include <vector>

#include "../../include/parphom_gpu.h"
#include "pp_internal.cuh"

namespace pp {
static std::atomic<int64_t> g_launches{0};
void count_launch(int64_t k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

int device_index() {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return (dev >= 0 && dev < PP_MAX_DEVICES) ? dev : -1;
}

int device_sms() {
  static std::mutex mu;
  static int sms[PP_MAX_DEVICES] = {};
  const int dev = device_index();
  if (dev < 0) return 1;
  std::lock_guard<std::mutex> g(mu);
  if (!sms[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
      cudaGetLastError();
      v = 0;
    }
    sms[dev] = v > 0 ? v : 1;
  }
  return sms[dev];
}

unsigned kt_mask = 0;
static const char *kt_names[KT_N] = {"assemble", "colupd", "refl", "hemv", "dots", "wcorr", "wfin", "her2k",
                                     "bisect", "invit", "vhx", "btred", "applyV", "vel", "xhz"};
struct KtPending {
  int k;
  cudaEvent_t a, b;
};
static std::mutex kt_mu;
static std::vector<KtPending> kt_pending;
static std::vector<cudaEvent_t> kt_free;
static cudaEvent_t kt_open[KT_N];
static int64_t kt_count[KT_N];
static double kt_ms[KT_N];

static cudaEvent_t kt_event() {
  if (!kt_free.empty()) {
    cudaEvent_t e = kt_free.back();
    kt_free.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}
void kt_begin(int k, cudaStream_t s) {
  std::lock_guard<std::mutex> g(kt_mu);
  kt_open[k] = kt_event();
  cudaEventRecord(kt_open[k], s);
}
void kt_end(int k, cudaStream_t s) {
  std::lock_guard<std::mutex> g(kt_mu);
  cudaEvent_t e = kt_event();
  cudaEventRecord(e, s);
  kt_pending.push_back({k, kt_open[k], e});
}
static void kt_flush() {
  for (auto &p : kt_pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(p.b) == cudaSuccess && cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      kt_count[p.k] += 1;
      kt_ms[p.k] += ms;
    }
    kt_free.push_back(p.a);
    kt_free.push_back(p.b);
  }
  kt_pending.clear();
}
}  // namespace pp

using namespace pp;

struct pp_ctx {
  Geometry g;
  int device = 0;
  cudaStream_t stream = nullptr;
  int broken = 0;
  // workspace (grown on demand)
  EigWork w;
  int cap_B = 0, cap_m = 0;
  int64_t cap_n = 0, cap_nbnd = 0, cap_nbr = 0;
  int cap_prec = -1;
  void *ws = nullptr;
  size_t ws_bytes = 0;
  // velocity buffers
  double *vpart = nullptr;
  double *vraw = nullptr;
  int nsplit = 8;
  // staging for host calls
  double *d_q = nullptr;
  double *d_w = nullptr, *d_z = nullptr, *d_vel = nullptr;
  double *d_err = nullptr;  // [3][B][n] resid, werr, zerr staging
  int64_t *d_m = nullptr, *d_nz = nullptr, *d_info = nullptr;
  // extra streams for the other parts of a batch (forked from and joined to
  // the working stream with events, so that they are captured into the graph)
  static constexpr int MAX_SPLIT = 32;
  cudaStream_t aux[MAX_SPLIT - 1] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[MAX_SPLIT - 1] = {};
  // launch configuration of the current batch (autotuned or from the switches)
  int cur_split = 8, cur_bps = 6;
  // captured CUDA graph of the last batch configuration
  cudaGraphExec_t gexec = nullptr;
  char gkey[192] = {0};
  int64_t glaunches = 0;  // kernels in the captured graph
};

namespace {

constexpr double PI2_REF = (double)6.283185307179586f;  // lammps_read.F90:255
constexpr double DEL_REF = (double)1e-6f;               // dynamical_matrix.F90:60
constexpr double C_RANGE = (double)(15.633302f * 33.35641f);  // diagonalize.F90:75

int cuda_err(cudaError_t e) {
  if (e == cudaSuccess) return PP_OK;
  if (e == cudaErrorMemoryAllocation) return PP_ERR_NOMEM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver || e == cudaErrorNoKernelImageForDevice)
    return PP_ERR_NODEVICE;
  return PP_ERR_CUDA;
}

#define TRY_CUDA(x)                       \
  do {                                    \
    cudaError_t e__ = (x);                \
    if (e__ != cudaSuccess) return cuda_err(e__); \
  } while (0)

// lammps_read.F90:250-274 (B = 2 pi_f * inverse transpose), Fortran layout.
void matinvtransp3(const double *A, double *B) {
#define AA(i, j) A[(i - 1) + 3 * (j - 1)]
#define BB(i, j) B[(i - 1) + 3 * (j - 1)]
  const double detinv = 1.0 / (AA(1, 1) * AA(2, 2) * AA(3, 3) - AA(1, 1) * AA(2, 3) * AA(3, 2) -
                               AA(1, 2) * AA(2, 1) * AA(3, 3) + AA(1, 2) * AA(2, 3) * AA(3, 1) +
                               AA(1, 3) * AA(2, 1) * AA(3, 2) - AA(1, 3) * AA(2, 2) * AA(3, 1));
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

// lammps_read.F90:281-309: u = (A^-1)^T x.
void linsolve(const double *x, const double *A, double *u) {
#define AA(i, j) A[(i - 1) + 3 * (j - 1)]
  const double detinv = 1.0 / (AA(1, 1) * AA(2, 2) * AA(3, 3) - AA(1, 1) * AA(2, 3) * AA(3, 2) -
                               AA(1, 2) * AA(2, 1) * AA(3, 3) + AA(1, 2) * AA(2, 3) * AA(3, 1) +
                               AA(1, 3) * AA(2, 1) * AA(3, 2) - AA(1, 3) * AA(2, 2) * AA(3, 1));
  double Bm[3][3];
  Bm[0][0] = +detinv * (AA(2, 2) * AA(3, 3) - AA(2, 3) * AA(3, 2));
  Bm[1][0] = -detinv * (AA(2, 1) * AA(3, 3) - AA(2, 3) * AA(3, 1));
  Bm[2][0] = +detinv * (AA(2, 1) * AA(3, 2) - AA(2, 2) * AA(3, 1));
  Bm[0][1] = -detinv * (AA(1, 2) * AA(3, 3) - AA(1, 3) * AA(3, 2));
  Bm[1][1] = +detinv * (AA(1, 1) * AA(3, 3) - AA(1, 3) * AA(3, 1));
  Bm[2][1] = -detinv * (AA(1, 1) * AA(3, 2) - AA(1, 2) * AA(3, 1));
  Bm[0][2] = +detinv * (AA(1, 2) * AA(2, 3) - AA(1, 3) * AA(2, 2));
  Bm[1][2] = -detinv * (AA(1, 1) * AA(2, 3) - AA(1, 3) * AA(2, 1));
  Bm[2][2] = +detinv * (AA(1, 1) * AA(2, 2) - AA(1, 2) * AA(2, 1));
#undef AA
  for (int i = 0; i < 3; ++i) {
    double s = 0.0;
    for (int k = 0; k < 3; ++k) s += Bm[k][i] * x[k];
    u[i] = s;
  }
}

void drop_graph(pp_ctx *c) {
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  c->gexec = nullptr;
  c->gkey[0] = 0;
}

void free_ws(pp_ctx *c) {
  drop_graph(c);
  if (c->ws) cudaFree(c->ws);
  c->ws = nullptr;
  c->ws_bytes = 0;
  c->cap_B = c->cap_m = 0;
  c->cap_n = c->cap_nbnd = c->cap_nbr = 0;
  c->w = EigWork();
}

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

// Carve every batch buffer out of one allocation.
int ensure_ws_sized(pp_ctx *c, int B, int mcap, int64_t n, int64_t nbnd_max, int64_t nbr_max) {
  if (c->ws && B <= c->cap_B && mcap <= c->cap_m && n == c->cap_n && nbnd_max <= c->cap_nbnd &&
      nbr_max == c->cap_nbr)
    return PP_OK;
  free_ws(c);
  const int nb = 32;
  const int64_t lda = (n + 7) / 8 * 8;
  const int nchunk = (int)((n + 31) / 32);
  const int nrb = (int)((n + 31) / 32) + 1;  // partial sums per column kernel block
  const int64_t T = std::min<int64_t>(((int64_t)mcap + 63) / 64 * 64, 2048);
  const int nbr = (int)nbr_max;
  const int ldwp = std::max(std::max(mcap, nbr), 64);
  // split-K partials: ceil(n/512) chunks of 32 x ldwp, or the Gram product's
  // ceil(n/64) chunks of 32 x 32, whichever is larger
  const int ksplit = (int)std::max<int64_t>((n + 511) / 512, ((n + 63) / 64 * 32 + ldwp - 1) / ldwp);
  const int64_t nbnd = nbnd_max;
  std::vector<std::pair<void **, size_t>> parts;
  EigWork &w = c->w;
  w = EigWork();
  w.B = B;
  w.nmax = (int)n;
  w.mcap = mcap;
  w.nb = nb;
  w.lda = lda;
  w.sA = lda * n;
  w.lde = lda;
  w.sE = lda * mcap;
  w.nchunk = nchunk;
  w.nrb = nrb;
  w.scratch_threads = T;
  w.ldwp = ldwp;
  w.ksplit = ksplit;
  size_t off = 0;
  auto add = [&](void **p, size_t bytes) {
    parts.push_back({p, off});
    off = align_up(off + bytes);
  };
  add((void **)&w.nvec, sizeof(int) * B);
  add(&w.A, 16 * (size_t)B * w.sA);
  add(&w.E, 16 * (size_t)B * w.sE);
  add(&w.W, 16 * (size_t)B * lda * nb);
  add(&w.P, 16 * (size_t)B * nchunk * lda);
  add(&w.X, 16 * (size_t)B * 2 * nb);
  add((void **)&w.nrm, 8 * (size_t)B * nrb);
  add((void **)&w.wv, 16 * (size_t)B * nrb);
  add((void **)&w.d, 8 * (size_t)B * n);
  add((void **)&w.e, 8 * (size_t)B * n);
  add((void **)&w.tau, 16 * (size_t)B * n);
  add((void **)&w.scal, 16 * (size_t)B * 4);
  add((void **)&w.w, 8 * (size_t)B * n);
  add((void **)&w.rng, 8 * (size_t)B * 8);
  add((void **)&w.tinfo, 8 * (size_t)B * 8);
  add((void **)&w.cls, 4 * (size_t)B * (n + 1));
  add((void **)&w.ncl, 4 * (size_t)B);
  add((void **)&w.scratch, 8 * (size_t)B * 5 * n * T);
  add((void **)&w.piv, (size_t)B * n * T);
  add((void **)&w.info, 8 * (size_t)B);
  const int64_t npan = std::max<int64_t>(1, (n - 1 + nb - 1) / nb);
  w.sTfp = (int64_t)B * 1024;
  add((void **)&w.Tf, 16 * (size_t)npan * B * 1024);
  add(&w.Wb, 16 * (size_t)B * 32 * ldwp);
  add(&w.Wp, 16 * (size_t)B * ksplit * 32 * ldwp);
  w.nbr = nbr;
  add(&w.Xr, 16 * (size_t)B * lda * std::max(nbr, 1));
  add(&w.Eb, 16 * (size_t)B * std::max(nbr, 1) * mcap);
  // tensor-core trailing update of the double-float form
  w.sTcS = (int64_t)her2k_tc_bytes(n);
  w.sTcE = her2k_tc_exps(n);
  add((void **)&w.tcS, (size_t)B * w.sTcS);
  add((void **)&w.tcE, 4 * (size_t)B * w.sTcE);
  add((void **)&w.tcErr, 4 * (size_t)B);
  add((void **)&c->vpart, 8 * (size_t)B * c->nsplit * 3 * mcap + 16 * (size_t)B * nbnd * 3);
  add((void **)&c->vraw, 8 * (size_t)B * 3 * mcap);
  add((void **)&c->d_q, 8 * (size_t)B * 3);
  add((void **)&c->d_w, 8 * (size_t)B * n);
  add((void **)&c->d_err, 8 * (size_t)3 * B * n);
  add((void **)&c->d_vel, 8 * (size_t)B * 3 * mcap);
  add((void **)&c->d_m, 8 * (size_t)B);
  add((void **)&c->d_nz, 8 * (size_t)B);
  add((void **)&c->d_info, 8 * (size_t)B);
  void *base = nullptr;
  cudaError_t e = cudaMalloc(&base, off);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return PP_ERR_NOMEM;
  }
  for (auto &p : parts) *p.first = (char *)base + p.second;
  // opt the tensor-core kernel into its shared memory (outside any capture)
  TRY_CUDA(prepare_her2k_tc());
  c->ws = base;
  c->ws_bytes = off;
  w.bytes = off;
  c->cap_B = B;
  c->cap_m = mcap;
  c->cap_n = n;
  c->cap_nbnd = nbnd_max;
  c->cap_nbr = nbr_max;
  std::vector<int> nv(B, (int)n);
  TRY_CUDA(cudaMemcpy(w.nvec, nv.data(), sizeof(int) * B, cudaMemcpyHostToDevice));
  return PP_OK;
}

int ensure_ws(pp_ctx *c, int B, int mcap) { return ensure_ws_sized(c, B, mcap, c->g.n, c->g.nbnd, c->g.nbrows); }

size_t ws_bytes_estimate(int64_t n, int B, int mcap, int64_t nbnd, int64_t nbr) {
  const int64_t T = std::min<int64_t>(((int64_t)mcap + 63) / 64 * 64, 2048);
  size_t per = 16 * (size_t)n * n + 16 * (size_t)n * mcap + 8 * (size_t)5 * n * T + (size_t)n * T +
               16 * (size_t)n * 64 * 2 + 16 * (size_t)((n + 511) / 512) * 32 * std::max(mcap, 64) +
               16 * (size_t)((n + 63) / 64) * 32 * 32 + her2k_tc_bytes(n) + 8 * (size_t)(n + 128) +
               8 * 8 * 3 * (size_t)mcap + 16 * 3 * (size_t)nbnd + 16 * (size_t)nbr * (n + mcap) +
               16 * 1024 * (size_t)std::max<int64_t>(1, (n + 30) / 32);  // compact-WY factors of all panels
  return per * B;
}

int check_opts(const pp_ctx *c, const pp_eig_opts *o) {
  if (!o) return -5;
  if (o->jobz != 'N' && o->jobz != 'V') return -5;
  if (o->range != 'A' && o->range != 'I' && o->range != 'V') return -5;
  if (o->uplo != 'U' && o->uplo != 0) return -5;
  if (o->vel && o->vel_method != 'A' && o->vel_method != 'C') return -5;
  if (o->precision != PP_PREC_FP64 && o->precision != PP_PREC_MIXED) return -5;
  const int64_t n = c->g.n;
  if (o->range == 'I' && (o->il < 1 || o->iu > n || o->il > o->iu)) return -5;
  if (o->range == 'V' && !(o->vl < o->vu)) return -5;
  return PP_OK;
}

// The matrices [off, off+cnt) of a batch as a batch of their own (every
// per-matrix buffer shifted by `off` of its per-matrix stride).
EigWork view_of(const EigWork &w, int off, int cnt) {
  EigWork v = w;
  v.B = cnt;
  v.boff = w.boff + off;
  auto sh = [off](void *p, size_t stride_bytes) -> void * {
    return p ? (void *)((char *)p + stride_bytes * (size_t)off) : nullptr;
  };
  const size_t nmax = (size_t)w.nmax;
  const int64_t T = w.scratch_threads;
  v.nvec = w.nvec + off;
  v.A = sh(w.A, 16 * (size_t)w.sA);
  v.E = sh(w.E, 16 * (size_t)w.sE);
  v.W = sh(w.W, 16 * (size_t)w.lda * w.nb);
  v.P = sh(w.P, 16 * (size_t)w.nchunk * w.lda);
  v.X = sh(w.X, 16 * 2 * (size_t)w.nb);
  v.nrm = (double *)sh(w.nrm, 8 * (size_t)w.nrb);
  v.wv = (z64 *)sh(w.wv, 16 * (size_t)w.nrb);
  v.d = (double *)sh(w.d, 8 * nmax);
  v.e = (double *)sh(w.e, 8 * nmax);
  v.tau = (z64 *)sh(w.tau, 16 * nmax);
  v.scal = (z64 *)sh(w.scal, 16 * 4);
  v.w = (double *)sh(w.w, 8 * nmax);
  v.rng = (int64_t *)sh(w.rng, 8 * 8);
  v.tinfo = (double *)sh(w.tinfo, 8 * 8);
  v.cls = (int *)sh(w.cls, 4 * (nmax + 1));
  v.ncl = (int *)sh(w.ncl, 4);
  v.scratch = (double *)sh(w.scratch, 8 * 5 * nmax * (size_t)T);
  v.piv = (uint8_t *)sh(w.piv, nmax * (size_t)T);
  v.info = (int64_t *)sh(w.info, 8);
  v.Tf = (z64 *)sh(w.Tf, 16 * 1024);  // panel stride sTfp unchanged
  v.Wb = sh(w.Wb, 16 * 32 * (size_t)w.ldwp);
  v.Wp = sh(w.Wp, 16 * (size_t)w.ksplit * 32 * w.ldwp);
  v.Xr = sh(w.Xr, 16 * (size_t)w.lda * std::max(w.nbr, 1));
  v.Eb = sh(w.Eb, 16 * (size_t)std::max(w.nbr, 1) * w.mcap);
  if (w.tcS) {
    v.tcS = (uint8_t *)sh(w.tcS, (size_t)w.sTcS);
    v.tcE = (int *)sh(w.tcE, 4 * (size_t)w.sTcE);
    v.tcErr = (int *)sh(w.tcErr, 4);
  }
  return v;
}

// Eigenvectors are formed when asked for, for velocities, and for the error
// estimates (which need the full vectors).
bool needs_vectors(const pp_eig_opts *o) { return o->jobz == 'V' || o->vel || o->want_resid; }

// Velocities without eigenvector output (and without error estimates) need
// only the eigenvector rows of atoms in boundary blocks.
bool rows_only_mode(const Geometry &g, const pp_eig_opts *o, bool want_z) {
  return o->vel && !want_z && !o->want_resid && g.nbrows < g.n;
}

// Reduction, tridiagonal eigenpairs and back-transform of the matrices of w
// on stream s.
int eig_stages(pp_ctx *c, EigWork &w, const pp_eig_opts *o, bool want_z, cudaStream_t s) {
  const int prec = o->precision;
  const bool vecs = needs_vectors(o);
  if (prec == PP_PREC_MIXED)
    TRY_CUDA(tridiagonalize<df>(w, s));
  else
    TRY_CUDA(tridiagonalize<double>(w, s));
  TRY_CUDA(tridiag_eigenvalues(w, o->range, o->vl / C_RANGE, o->vu / C_RANGE, o->il, o->iu, o->abstol, s,
                               prec == PP_PREC_MIXED));
  if (vecs) {
    // Velocities without eigenvector output need only the eigenvector rows
    // of atoms in boundary blocks: back-transform those rows only.
    const bool rows_only = rows_only_mode(c->g, o, want_z);
    if (prec == PP_PREC_MIXED) {
      TRY_CUDA(tridiag_eigenvectors<df>(w, s));
      if (rows_only)
        TRY_CUDA(back_transform_rows<df>(w, c->g.d_brows, (int)c->g.nbrows, s));
      else
        TRY_CUDA(back_transform<df>(w, s));
    } else {
      TRY_CUDA(tridiag_eigenvectors<double>(w, s));
      if (rows_only)
        TRY_CUDA(back_transform_rows<double>(w, c->g.d_brows, (int)c->g.nbrows, s));
      else
        TRY_CUDA(back_transform<double>(w, s));
    }
  }
  return PP_OK;
}

// Streams a batch is split over (PARPHOM_GPU_SPLIT, 1 .. MAX_SPLIT; default 8).
int split_ways() {
  const char *e = getenv("PARPHOM_GPU_SPLIT");
  if (!e || !e[0]) return 8;
  const int k = atoi(e);
  return std::max(1, std::min(k, pp_ctx::MAX_SPLIT));
}

// Run the pipeline for B q-points already in c->d_q; results left in the
// EigWork buffers, velocities in c->vraw.  With B >= 2 the eigen stages of
// parts of the batch run on separate streams: their column recurrences are
// chains of short, latency-bound launches, and each part fills the gaps of
// the others.  (Not while per-kernel timing is on: its events assume one
// stream.)
int run_batch(pp_ctx *c, int B, const pp_eig_opts *o, int mcap, bool want_z) {
  EigWork &w = c->w;
  w.B = B;
  cudaStream_t s = c->stream;
  const int prec = o->precision;
  TRY_CUDA(assemble_batch(c->g, c->d_q, B, w.A, w.lda, w.sA, prec == PP_PREC_MIXED ? 1 : 0, s));
  (void)mcap;
  const int ways = pp::kt_mask ? 1 : std::min(B, c->cur_split);
  w.hemv_bps = c->cur_bps;
  if (ways >= 2) {
    if (!c->ev_fork) TRY_CUDA(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    for (int k = 0; k < ways - 1; ++k) {
      if (!c->aux[k]) TRY_CUDA(cudaStreamCreateWithFlags(&c->aux[k], cudaStreamNonBlocking));
      if (!c->ev_join[k]) TRY_CUDA(cudaEventCreateWithFlags(&c->ev_join[k], cudaEventDisableTiming));
    }
    TRY_CUDA(cudaEventRecord(c->ev_fork, s));
    int r = PP_OK;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < ways; ++k) {
      const int off = (int)((int64_t)B * k / ways), cnt = (int)((int64_t)B * (k + 1) / ways) - off;
      EigWork v = view_of(w, off, cnt);
      cudaStream_t sk = k == 0 ? s : c->aux[k - 1];
      if (k > 0 && e == cudaSuccess) e = cudaStreamWaitEvent(sk, c->ev_fork, 0);
      const int rk = eig_stages(c, v, o, want_z, sk);
      if (!r) r = rk;
    }
    // always join, so that a capture in progress stays well formed
    for (int k = 1; k < ways; ++k) {
      const cudaError_t ek = cudaEventRecord(c->ev_join[k - 1], c->aux[k - 1]);
      const cudaError_t ew = cudaStreamWaitEvent(s, c->ev_join[k - 1], 0);
      if (e == cudaSuccess) e = ek != cudaSuccess ? ek : ew;
    }
    if (r) return r;
    TRY_CUDA(e);
  } else {
    const int r = eig_stages(c, w, o, want_z, s);
    if (r) return r;
  }
  if (o->vel) {
    const bool rows_only = rows_only_mode(c->g, o, want_z);
    if (rows_only)
      TRY_CUDA(velocities(c->g, c->d_q, B, w.Eb, w.nbr, (int64_t)w.nbr * w.mcap, prec == PP_PREC_MIXED ? 1 : 0,
                          w.rng, w.mcap, o->vel_method, c->vraw, c->vpart, c->nsplit, c->g.d_rowmap, s));
    else
      TRY_CUDA(velocities(c->g, c->d_q, B, w.E, w.lde, w.sE, prec == PP_PREC_MIXED ? 1 : 0, w.rng, w.mcap,
                          o->vel_method, c->vraw, c->vpart, c->nsplit, nullptr, s));
  }
  return PP_OK;
}

// ---------------------------------------------------------------------------
// Autotuner.  The launch configuration of a batch -- how many streams the
// batch is split over, and how many persistent blocks per SM the Hermitian
// mat-vec runs with -- is chosen the first time a (device, order, batch size,
// options) combination is solved: each candidate's captured graph is timed
// on the GPU (CUDA events around its launch) over the call's own first
// batch, greedily (split first, then the mat-vec blocks), and the fastest is
// kept for the process.  PARPHOM_GPU_TUNE=0 or an explicit PARPHOM_GPU_SPLIT
// turns it off (split from the switch, 6 blocks per SM).
struct Tuned {
  int split, bps;
  float ms;
};
std::mutex g_tune_mu;
std::vector<std::pair<std::string, Tuned>> g_tuned;

bool autotune_enabled() {
  const char *e = getenv("PARPHOM_GPU_TUNE");
  if (e && e[0] == '0') return false;
  const char *sp = getenv("PARPHOM_GPU_SPLIT");
  return !(sp && sp[0]);
}

std::string tune_key(const pp_ctx *c, int B, const pp_eig_opts *o, bool want_z) {
  char key[160];
  snprintf(key, sizeof(key), "dev%d n=%lld B=%d prec=%d jobz=%c range=%c vel=%d z=%d resid=%d", c->device,
           (long long)c->w.nmax, B, o->precision, o->jobz, o->range, o->vel, want_z ? 1 : 0, o->want_resid ? 1 : 0);
  return key;
}

bool graphs_enabled() {
  const char *e = getenv("PARPHOM_GPU_GRAPHS");
  return !(e && e[0] == '0');
}

// run_batch through a captured CUDA graph: the launch sequence depends only on
// the batch size, the options and the workspace, so it is captured once and
// replayed (one graph launch instead of ~6 launches per matrix column).
int run_batch_graph_cfg(pp_ctx *c, int B, const pp_eig_opts *o, int mcap, bool want_z, bool launch = true);

// Time one launch configuration: capture and instantiate its graph (host
// work, not timed), then time one launch of it on the stream with events.
// Returns the milliseconds, or a negative value if the graph path is not
// available.
float time_config(pp_ctx *c, int B, const pp_eig_opts *o, int mcap, bool want_z, int split, int bps) {
  c->cur_split = split;
  c->cur_bps = bps;
  cudaStream_t s = c->stream;
  if (run_batch_graph_cfg(c, B, o, mcap, want_z, false) != PP_OK || !c->gexec) return -1.f;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    cudaGetLastError();
    if (e0) cudaEventDestroy(e0);
    return -1.f;
  }
  float ms = -1.f;
  cudaEventRecord(e0, s);
  const cudaError_t r = cudaGraphLaunch(c->gexec, s);
  pp::count_launch(c->glaunches);
  cudaEventRecord(e1, s);
  if (r == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms;
}

int run_batch_graph(pp_ctx *c, int B, const pp_eig_opts *o, int mcap, bool want_z) {
  c->cur_split = split_ways();
  c->cur_bps = 6;
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(c->stream, &cs) != cudaSuccess) {
    cudaGetLastError();
    cs = cudaStreamCaptureStatusActive;
  }
  if (autotune_enabled() && B >= 2) {
    const std::string key = tune_key(c, B, o, want_z);
    Tuned t{-1, 6, 0.f};
    {
      std::lock_guard<std::mutex> g(g_tune_mu);
      for (auto &kv : g_tuned)
        if (kv.first == key) t = kv.second;
    }
    // tune only where candidates can be timed: graphs on, no per-kernel
    // timing, no caller capture in progress
    const bool can_tune = graphs_enabled() && !pp::kt_mask && !tc_stall_armed() && cs == cudaStreamCaptureStatusNone;
    if (t.split < 0 && !can_tune) t = Tuned{split_ways(), 6, 0.f};
    if (t.split < 0) {
      // greedy: split over {4, 8, 16, 32} (at most B) with 6 mat-vec blocks per SM
      Tuned best{std::min(B, 8), 6, 1e30f};
      for (int sp : {4, 8, 16, 32}) {
        if (sp > B && sp != 4) continue;
        const int spc = std::min(sp, B);
        const float ms = time_config(c, B, o, mcap, want_z, spc, 6);
        if (ms > 0.f && ms < best.ms) best = Tuned{spc, 6, ms};
      }
      // then fewer persistent mat-vec blocks per SM (6 -> 4 -> 3 -> 2) while that helps:
      // with several streams the mat-vecs of different parts share the SMs
      for (int bps : {4, 3, 2}) {
        if (best.ms > 1e29f) break;
        const float ms = time_config(c, B, o, mcap, want_z, best.split, bps);
        if (!(ms > 0.f && ms < best.ms)) break;
        best = Tuned{best.split, bps, ms};
      }
      if (best.ms > 1e29f) best.ms = 0.f;
      t = best;
      std::lock_guard<std::mutex> g(g_tune_mu);
      g_tuned.push_back({key, t});
    }
    c->cur_split = t.split;
    c->cur_bps = t.bps;
  }
  return run_batch_graph_cfg(c, B, o, mcap, want_z);
}

// The batch through its captured graph (captured on the first use of a
// configuration); with launch = false the graph is only captured and
// instantiated (used by the autotuner, which then times the launch).
int run_batch_graph_cfg(pp_ctx *c, int B, const pp_eig_opts *o, int mcap, bool want_z, bool launch) {
  // (an armed test stall is a one-shot launch parameter: never captured)
  if (!graphs_enabled() || pp::kt_mask || tc_stall_armed()) return launch ? run_batch(c, B, o, mcap, want_z) : 1;
  char key[192];
  snprintf(key, sizeof(key), "%p|%d|%d|%c%c%c|%d|%lld|%lld|%.17g|%.17g|%.17g|%d|%d|%d|%d", c->ws, B, o->precision,
           o->jobz, o->range, o->vel_method, o->vel, (long long)o->il, (long long)o->iu, o->vl, o->vu, o->abstol,
           want_z ? 1 : 0, c->cur_split, c->cur_bps, o->want_resid ? 1 : 0);
  cudaStream_t s = c->stream;
  if (c->gexec && strcmp(key, c->gkey) == 0) {
    if (!launch) return PP_OK;
    TRY_CUDA(cudaGraphLaunch(c->gexec, s));
    pp::count_launch(c->glaunches);
    return PP_OK;
  }
  drop_graph(c);
  TRY_CUDA(prepare_bisect(bisect_smem(c->w.nmax, o->precision == PP_PREC_MIXED)));
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return launch ? run_batch(c, B, o, mcap, want_z) : 1;
  }
  const int64_t l0 = pp::g_launches.load();
  const int r = run_batch(c, B, o, mcap, want_z);
  c->glaunches = pp::g_launches.load() - l0;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &g);
  if (r != PP_OK || e != cudaSuccess || !g) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return launch ? run_batch(c, B, o, mcap, want_z) : 1;
  }
  e = cudaGraphInstantiate(&c->gexec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    c->gexec = nullptr;
    cudaGetLastError();
    return launch ? run_batch(c, B, o, mcap, want_z) : 1;
  }
  snprintf(c->gkey, sizeof(c->gkey), "%s", key);
  if (!launch) {
    pp::g_launches.fetch_sub(c->glaunches);  // captured, not launched
    return PP_OK;
  }
  TRY_CUDA(cudaGraphLaunch(c->gexec, s));
  return PP_OK;
}

int mcap_for(const pp_ctx *c, const pp_eig_opts *o) {
  const int64_t n = c->g.n;
  if (o->range == 'I') return (int)(o->iu - o->il + 1);
  return (int)n;
}

int pick_batch(pp_ctx *c, int64_t nq, int mcap) {
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  if (c->ws) fr += c->ws_bytes;
  const size_t budget = (size_t)(0.6 * (double)fr);
  int B = (int)std::min<int64_t>(nq, 64);
  while (B > 1 && ws_bytes_estimate(c->g.n, B, mcap, c->g.nbnd, c->g.nbrows) > budget) B = B / 2;
  const char *env = getenv("PARPHOM_GPU_BATCH");
  if (env) {
    int v = atoi(env);
    if (v > 0) B = std::min<int64_t>(v, nq);
  }
  return std::max(B, 1);
}

// Boundary blocks (I < J, tie set with a non-home image, Phi block
// non-zero) and the rows of their atoms, from the current Phi and tie sets;
// replaces any earlier tables.
int build_boundary_tables(pp_ctx *c) {
  Geometry &g = c->g;
  const int64_t N = g.natom, n = g.n;
  cudaStream_t s = c->stream;
  for (void *p : {(void *)g.d_bnd, (void *)g.d_bndmask, (void *)g.d_brows, (void *)g.d_rowmap})
    if (p) cudaFree(p);
  g.d_bnd = nullptr;
  g.d_bndmask = nullptr;
  g.d_brows = nullptr;
  g.d_rowmap = nullptr;
  g.nbnd = g.nbrows = 0;
  uint8_t *d_flags = nullptr;
  if (cudaMalloc(&d_flags, (size_t)N * N) != cudaSuccess) return PP_ERR_NOMEM;
  geom_block_nonzero(g, d_flags, s);
  std::vector<uint8_t> flags_h((size_t)N * N);
  std::vector<uint16_t> mask_h((size_t)N * N);
  cudaMemcpyAsync(flags_h.data(), d_flags, (size_t)N * N, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(mask_h.data(), g.d_mask, sizeof(uint16_t) * N * N, cudaMemcpyDeviceToHost, s);
  cudaError_t e = cudaStreamSynchronize(s);
  cudaFree(d_flags);
  if (e != cudaSuccess) return cuda_err(e);
  std::vector<int2> bnd;
  std::vector<uint16_t> bmask;
  for (int64_t I = 0; I < N; ++I)
    for (int64_t J = I + 1; J < N; ++J) {
      const uint16_t m = mask_h[I + N * J];
      if ((m & ~(1u << 4)) && flags_h[I + N * J]) {
        bnd.push_back(make_int2((int)I, (int)J));
        bmask.push_back(m);
      }
    }
  g.nbnd = (int64_t)bnd.size();
  // rows of the atoms that appear in boundary blocks (all the velocity
  // kernel reads of the eigenvectors)
  std::vector<int> rows, rowmap(n, -1);
  {
    std::vector<char> used(N, 0);
    for (auto &p : bnd) used[p.x] = used[p.y] = 1;
    for (int64_t I = 0; I < N; ++I)
      if (used[I])
        for (int a = 0; a < 3; ++a) {
          rowmap[3 * I + a] = (int)rows.size();
          rows.push_back((int)(3 * I + a));
        }
  }
  g.nbrows = (int64_t)rows.size();
  if (cudaMalloc(&g.d_rowmap, sizeof(int) * n) != cudaSuccess) return PP_ERR_NOMEM;
  cudaMemcpy(g.d_rowmap, rowmap.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
  if (g.nbrows) {
    if (cudaMalloc(&g.d_brows, sizeof(int) * g.nbrows) != cudaSuccess) return PP_ERR_NOMEM;
    cudaMemcpy(g.d_brows, rows.data(), sizeof(int) * g.nbrows, cudaMemcpyHostToDevice);
  }
  if (g.nbnd) {
    if (cudaMalloc(&g.d_bnd, sizeof(int2) * g.nbnd) != cudaSuccess) return PP_ERR_NOMEM;
    if (cudaMalloc(&g.d_bndmask, sizeof(uint16_t) * g.nbnd) != cudaSuccess) return PP_ERR_NOMEM;
    cudaMemcpy(g.d_bnd, bnd.data(), sizeof(int2) * g.nbnd, cudaMemcpyHostToDevice);
    cudaMemcpy(g.d_bndmask, bmask.data(), sizeof(uint16_t) * g.nbnd, cudaMemcpyHostToDevice);
  }
  const cudaError_t e2 = cudaGetLastError();
  return e2 == cudaSuccess ? PP_OK : cuda_err(e2);
}

}  // namespace

extern "C" {

int64_t pp_version(void) { return 20000; }

int64_t pp_kernel_launches(void) { return pp::g_launches.load(); }

int pp_ktimer_enable(const char *names) {
  std::lock_guard<std::mutex> g(pp::kt_mu);
  pp::kt_flush();
  unsigned mask = 0;
  if (names) {
    std::string all(names);
    size_t p = 0;
    while (p <= all.size()) {
      size_t q = all.find(',', p);
      if (q == std::string::npos) q = all.size();
      std::string tok = all.substr(p, q - p);
      for (int k = 0; k < KT_N; ++k)
        if (tok == pp::kt_names[k]) mask |= 1u << k;
      p = q + 1;
    }
  }
  for (int k = 0; k < KT_N; ++k) {
    pp::kt_count[k] = 0;
    pp::kt_ms[k] = 0.0;
  }
  pp::kt_mask = mask;
  return PP_OK;
}

int pp_autotune_report(char *buf, int64_t len) {
  if (!buf || len <= 0) return -1;
  std::lock_guard<std::mutex> g(g_tune_mu);
  std::string out;
  char line[256];
  for (auto &kv : g_tuned) {
    snprintf(line, sizeof(line), "%s -> split=%d hemv_blocks_per_sm=%d batch_ms=%.3f\n", kv.first.c_str(),
             kv.second.split, kv.second.bps, kv.second.ms);
    out += line;
  }
  strncpy(buf, out.c_str(), (size_t)len - 1);
  buf[len - 1] = 0;
  return PP_OK;
}

int pp_debug_stall_tc_wait(int64_t matrix, int64_t cycles) {
  if (matrix < -1) return -1;
  if (cycles < 0 || cycles > 2000000000LL) return -2;
  pp::arm_tc_stall(matrix, (long long)cycles);
  return PP_OK;
}

int pp_ktimer_report(char *buf, int64_t len) {
  if (!buf || len <= 0) return -1;
  std::lock_guard<std::mutex> g(pp::kt_mu);
  pp::kt_flush();
  std::string out;
  char line[128];
  for (int k = 0; k < KT_N; ++k) {
    if (!pp::kt_count[k]) continue;
    snprintf(line, sizeof(line), "%s %lld %.6f\n", pp::kt_names[k], (long long)pp::kt_count[k], pp::kt_ms[k]);
    out += line;
  }
  strncpy(buf, out.c_str(), (size_t)len - 1);
  buf[len - 1] = 0;
  return PP_OK;
}

const char *pp_strerror(int code) {
  switch (code) {
    case PP_OK: return "success";
    case PP_ERR_CUDA: return "CUDA runtime error";
    case PP_ERR_NOMEM: return "device memory allocation failed";
    case PP_ERR_NAN: return "non-finite value in the input";
    case PP_ERR_TIMEOUT: return "bounded device wait timed out";
    case PP_ERR_NODEVICE: return "no usable CUDA device for this library (sm_103a)";
    case PP_ERR_STATE: return "context is unusable after an earlier error";
    case PP_ERR_UNSUPPORTED: return "unsupported option";
    case PP_ERR_SIZE: return "matrix order exceeds the fixed scratch capacity (PP_NOALLOC_MAX_N = 1536)";
    default:
      if (code < 0) return "illegal argument (index given by -code)";
      return "unknown error";
  }
}

int pp_ctx_create(const pp_system *sys, const double *fc, int64_t ldfc, int64_t flags, pp_ctx **out) {
  if (!sys) return -1;
  if (!fc) return -2;
  if (!out) return -5;
  *out = nullptr;
  if (sys->natom < 1 || sys->ntypes < 1 || !sys->lat || !sys->crys || !sys->real_pos || !sys->mass ||
      !sys->at_types)
    return -1;
  const int64_t N = sys->natom, n = 3 * N;
  if (ldfc < n) return -3;
  if (N > 46000) return -1;  // mask table and 32-bit atom indices
  for (int64_t t = 0; t < sys->ntypes; ++t)
    if (!(sys->mass[t] > 0.0) || !std::isfinite(sys->mass[t])) return PP_ERR_NAN;
  for (int64_t I = 0; I < N; ++I)
    if (sys->at_types[I] < 1 || sys->at_types[I] > sys->ntypes) return -1;
  for (int k = 0; k < 9; ++k)
    if (!std::isfinite(sys->lat[k])) return PP_ERR_NAN;
  for (int64_t k = 0; k < 3 * N; ++k)
    if (!std::isfinite(sys->crys[k]) || !std::isfinite(sys->real_pos[k])) return PP_ERR_NAN;
  for (int64_t cc = 0; cc < n; ++cc)
    for (int64_t r = 0; r <= cc; ++r)
      if (!std::isfinite(fc[r + ldfc * cc])) return PP_ERR_NAN;

  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return PP_ERR_NODEVICE;
  }
  pp_ctx *c = new (std::nothrow) pp_ctx();
  if (!c) return PP_ERR_NOMEM;
  cudaGetDevice(&c->device);
  Geometry &g = c->g;
  g.natom = N;
  g.n = n;
  std::memcpy(g.lat, sys->lat, 9 * sizeof(double));
  matinvtransp3(g.lat, g.rec_lat);
  // CD step (dynamical_matrix.F90:134-148)
  {
    const double *rl = g.rec_lat;
    const double v = DEL_REF * std::sqrt(std::fabs(rl[0] * rl[4] - rl[3] * rl[1]));
    const double del = v > DEL_REF ? v : DEL_REF;
    for (int k = 0; k < 3; ++k) {
      double dv[3] = {0, 0, 0};
      dv[k] = del;
      linsolve(dv, g.rec_lat, g.delta_crys[k]);
      g.delta_norm[k] = std::sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
    }
  }
  std::vector<double> mass_atom(N);
  for (int64_t I = 0; I < N; ++I) mass_atom[I] = sys->mass[sys->at_types[I] - 1];

  auto fail = [&](int code) {
    pp_ctx_destroy(c);
    return code;
  };
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(PP_ERR_CUDA);
  // the streams of a split batch, created here so that none is created while
  // a stream capture (the library's or the caller's) is in progress
  if (cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess) return fail(PP_ERR_CUDA);
  for (int k = 0; k < pp_ctx::MAX_SPLIT - 1; ++k)
    if (cudaStreamCreateWithFlags(&c->aux[k], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join[k], cudaEventDisableTiming) != cudaSuccess)
      return fail(PP_ERR_CUDA);
  cudaStream_t s = c->stream;
  if (cudaMalloc(&g.d_fc, sizeof(double) * n * n) != cudaSuccess) return fail(PP_ERR_NOMEM);
  if (cudaMalloc(&g.d_crys, sizeof(double) * 3 * N) != cudaSuccess) return fail(PP_ERR_NOMEM);
  if (cudaMalloc(&g.d_pos, sizeof(double) * 3 * N) != cudaSuccess) return fail(PP_ERR_NOMEM);
  if (cudaMalloc(&g.d_mass, sizeof(double) * N) != cudaSuccess) return fail(PP_ERR_NOMEM);
  if (cudaMalloc(&g.d_mask, sizeof(uint16_t) * N * N) != cudaSuccess) return fail(PP_ERR_NOMEM);
  if (cudaMemcpy2DAsync(g.d_fc, sizeof(double) * n, fc, sizeof(double) * ldfc, sizeof(double) * n, n,
                        cudaMemcpyHostToDevice, s) != cudaSuccess)
    return fail(PP_ERR_CUDA);
  cudaMemcpyAsync(g.d_crys, sys->crys, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(g.d_pos, sys->real_pos, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(g.d_mass, mass_atom.data(), sizeof(double) * N, cudaMemcpyHostToDevice, s);
  if (geom_symmetrize_fc(g, (flags & PP_FLAG_ENFORCE_ASR) ? 1 : 0, s) != cudaSuccess) return fail(PP_ERR_CUDA);
  if (geom_build_masks(g, s) != cudaSuccess) return fail(PP_ERR_CUDA);
  {
    const int rb = build_boundary_tables(c);
    if (rb) return fail(rb);
  }
  cudaError_t e = cudaSuccess;
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(cuda_err(e));
  *out = c;
  return PP_OK;
}

int pp_ctx_update_fc(pp_ctx *c, const double *fc, int64_t ldfc, int64_t flags, int32_t fc_on_device) {
  if (!c) return -1;
  if (c->broken) return PP_ERR_STATE;
  if (!fc) return -2;
  const int64_t n = c->g.n;
  if (ldfc < n) return -3;
  if (fc_on_device != 0 && fc_on_device != 1) return -5;
  if (!fc_on_device)
    for (int64_t cc = 0; cc < n; ++cc)
      for (int64_t r = 0; r <= cc; ++r)
        if (!std::isfinite(fc[r + ldfc * cc])) return PP_ERR_NAN;
  cudaStream_t s = c->stream;
  TRY_CUDA(cudaStreamSynchronize(s));
  TRY_CUDA(cudaMemcpy2DAsync(c->g.d_fc, sizeof(double) * n, fc, sizeof(double) * ldfc, sizeof(double) * n, n,
                             fc_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s));
  TRY_CUDA(geom_symmetrize_fc(c->g, (flags & PP_FLAG_ENFORCE_ASR) ? 1 : 0, s));
  // the boundary tables follow Phi's non-zero blocks; a captured graph holds
  // the old tables' addresses and counts
  drop_graph(c);
  const int r = build_boundary_tables(c);
  if (r) {
    c->broken = 1;
    return r;
  }
  return PP_OK;
}

int pp_ctx_destroy(pp_ctx *c) {
  if (!c) return -1;
  if (c->stream) cudaStreamSynchronize(c->stream);
  free_ws(c);
  cudaFree(c->g.d_fc);
  cudaFree(c->g.d_crys);
  cudaFree(c->g.d_pos);
  cudaFree(c->g.d_mass);
  cudaFree(c->g.d_mask);
  cudaFree(c->g.d_bnd);
  cudaFree(c->g.d_bndmask);
  cudaFree(c->g.d_brows);
  cudaFree(c->g.d_rowmap);
  for (int k = 0; k < pp_ctx::MAX_SPLIT - 1; ++k) {
    if (c->aux[k]) {
      cudaStreamSynchronize(c->aux[k]);
      cudaStreamDestroy(c->aux[k]);
    }
    if (c->ev_join[k]) cudaEventDestroy(c->ev_join[k]);
  }
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return PP_OK;
}

int pp_solve_batch(pp_ctx *c, const double *q, int64_t ldq, int64_t nq, const pp_eig_opts *o,
                   const pp_result_view *out, int64_t *info) {
  if (!c) return -1;
  if (c->broken) return PP_ERR_STATE;
  if (!q && nq > 0) return -2;
  if (ldq < nq) return -3;
  if (nq < 0) return -4;
  int r = check_opts(c, o);
  if (r) return r;
  if (!out || !out->w || !out->m || !out->nz) return -6;
  if (nq == 0) return PP_OK;
  for (int64_t t = 0; t < nq; ++t)
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(q[t + ldq * k])) return PP_ERR_NAN;
  const int64_t n = c->g.n;
  const int mcap = mcap_for(c, o);
  if (out->ldw < n) return -6;
  const bool vecs = o->jobz == 'V' || o->vel;
  const bool want_z = vecs && out->z;
  if (want_z && out->ldz < n) return -6;
  const int B = pick_batch(c, nq, mcap);
  r = ensure_ws(c, B, mcap);
  if (r) return r;
  cudaStream_t s = c->stream;
  std::vector<double> qh(3 * (size_t)B);
  std::vector<int64_t> mh(B), nzh(B), infoh(B);
  for (int64_t t0 = 0; t0 < nq; t0 += B) {
    const int Bb = (int)std::min<int64_t>(B, nq - t0);
    for (int b = 0; b < Bb; ++b)
      for (int k = 0; k < 3; ++k) qh[3 * b + k] = q[(t0 + b) + ldq * k];
    TRY_CUDA(cudaMemcpyAsync(c->d_q, qh.data(), sizeof(double) * 3 * Bb, cudaMemcpyHostToDevice, s));
    r = run_batch_graph(c, Bb, o, mcap, want_z);
    if (r) {
      c->broken = 1;
      return r;
    }
    TRY_CUDA(finalize_outputs(c->w, o->precision == PP_PREC_MIXED ? 1 : 0, o->raw_lambda, c->vraw, o->vel ? 1 : 0,
                              0, c->d_w, n, nullptr, 0, 0, c->d_vel, 3 * (int64_t)c->w.mcap, c->d_m, c->d_nz, c->d_info,
                              vecs ? 1 : 0, s));
    const bool errs = o->want_resid && (out->resid || out->werr || out->zerr);
    double *e_res = c->d_err, *e_w = c->d_err + (size_t)B * n, *e_z = c->d_err + 2 * (size_t)B * n;
    if (errs)
      TRY_CUDA(error_estimates(c->g, c->d_q, c->w, o->precision == PP_PREC_MIXED ? 1 : 0, o->raw_lambda, c->vpart,
                               e_res, e_w, e_z, n, s));
    TRY_CUDA(cudaMemcpyAsync(mh.data(), c->d_m, 8 * Bb, cudaMemcpyDeviceToHost, s));
    TRY_CUDA(cudaMemcpyAsync(nzh.data(), c->d_nz, 8 * Bb, cudaMemcpyDeviceToHost, s));
    TRY_CUDA(cudaMemcpyAsync(infoh.data(), c->d_info, 8 * Bb, cudaMemcpyDeviceToHost, s));
    TRY_CUDA(cudaStreamSynchronize(s));
    for (int b = 0; b < Bb; ++b) {
      const int64_t t = t0 + b;
      out->m[t] = mh[b];
      out->nz[t] = (o->jobz == 'V' || o->vel) ? nzh[b] : 0;
      if (info) info[t] = infoh[b];
      const int64_t m = mh[b];
      if (m > 0) {
        TRY_CUDA(cudaMemcpyAsync(out->w + out->ldw * t, c->d_w + n * b, sizeof(double) * m, cudaMemcpyDeviceToHost,
                                 s));
        if (o->vel && out->vel)
          TRY_CUDA(cudaMemcpyAsync(out->vel + out->velstride * t, c->d_vel + 3 * (int64_t)c->w.mcap * b,
                                   sizeof(double) * 3 * m, cudaMemcpyDeviceToHost, s));
        if (errs) {
          const double *src[3] = {e_res, e_w, e_z};
          double *dst[3] = {out->resid, out->werr, out->zerr};
          for (int f = 0; f < 3; ++f)
            if (dst[f])
              TRY_CUDA(cudaMemcpyAsync(dst[f] + out->ldw * t, src[f] + n * b, sizeof(double) * m,
                                       cudaMemcpyDeviceToHost, s));
        }
      }
    }
    if (want_z) {
      // eigenvectors: convert to FP64 complex in the A buffer (free after the
      // back-transform and the error estimates), then copy each matrix with
      // the caller's pitch.
      double *zst = (double *)c->w.A;
      TRY_CUDA(finalize_outputs(c->w, o->precision == PP_PREC_MIXED ? 1 : 0, o->raw_lambda, c->vraw, 0, 1, nullptr,
                                0, zst, c->w.lda, 2 * c->w.sA, nullptr, 0, nullptr, nullptr, nullptr, 1, s));
      for (int b = 0; b < Bb; ++b) {
        const int64_t t = t0 + b;
        const int64_t m = mh[b];
        if (m > 0)
          TRY_CUDA(cudaMemcpy2DAsync(out->z + out->zstride * t, sizeof(double) * 2 * out->ldz,
                                     zst + 2 * c->w.sA * b, sizeof(double) * 2 * c->w.lda, sizeof(double) * 2 * n, m,
                                     cudaMemcpyDeviceToHost, s));
      }
    }
    TRY_CUDA(cudaStreamSynchronize(s));
  }
  return PP_OK;
}

int pp_solve_batch_device(pp_ctx *c, const double *q_dev, int64_t ldq, int64_t nq, const pp_eig_opts *o,
                          const pp_result_view *out, int64_t *info_dev, void *stream) {
  if (!c) return -1;
  if (c->broken) return PP_ERR_STATE;
  if (!q_dev && nq > 0) return -2;
  if (ldq < nq) return -3;
  if (nq < 0) return -4;
  int r = check_opts(c, o);
  if (r) return r;
  if (!out || !out->w || !out->m || !out->nz) return -6;
  if (nq == 0) return PP_OK;
  const int64_t n = c->g.n;
  const int mcap = mcap_for(c, o);
  if (out->ldw < n) return -6;
  const bool vecs = o->jobz == 'V' || o->vel;
  const bool want_z = vecs && out->z;
  if (want_z && out->ldz < n) return -6;
  const int B = pick_batch(c, nq, mcap);
  r = ensure_ws(c, B, mcap);
  if (r) return r;
  // A NULL stream means the legacy default stream: the work then runs on the
  // library's own stream, ordered after and before the legacy stream with
  // events (so captured graphs stay usable).
  const bool legacy = stream == nullptr;
  cudaStream_t s = legacy ? c->stream : (cudaStream_t)stream;
  if (legacy) {
    cudaEvent_t ev;
    TRY_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, cudaStreamLegacy);
    cudaStreamWaitEvent(c->stream, ev, 0);
    cudaEventDestroy(ev);
  }
  cudaStream_t saved = c->stream;
  c->stream = s;
  for (int64_t t0 = 0; t0 < nq; t0 += B) {
    const int Bb = (int)std::min<int64_t>(B, nq - t0);
    for (int k = 0; k < 3; ++k)
      TRY_CUDA(cudaMemcpy2DAsync(c->d_q + k, 3 * sizeof(double), q_dev + t0 + ldq * k, sizeof(double),
                                 sizeof(double), Bb, cudaMemcpyDeviceToDevice, s));
    r = run_batch_graph(c, Bb, o, mcap, want_z);
    if (r) {
      c->stream = saved;
      c->broken = 1;
      return r;
    }
    r = cuda_err(finalize_outputs(c->w, o->precision == PP_PREC_MIXED ? 1 : 0, o->raw_lambda, c->vraw,
                                  o->vel ? 1 : 0, want_z ? 1 : 0, out->w + out->ldw * t0, out->ldw,
                                  want_z ? out->z + out->zstride * t0 : nullptr, out->ldz, out->zstride,
                                  out->vel ? out->vel + out->velstride * t0 : nullptr, out->velstride, out->m + t0,
                                  out->nz + t0, info_dev ? info_dev + t0 : nullptr, vecs ? 1 : 0, s));
    if (!r && o->want_resid && (out->resid || out->werr || out->zerr))
      r = cuda_err(error_estimates(c->g, c->d_q, c->w, o->precision == PP_PREC_MIXED ? 1 : 0, o->raw_lambda,
                                   c->vpart, out->resid ? out->resid + out->ldw * t0 : nullptr,
                                   out->werr ? out->werr + out->ldw * t0 : nullptr,
                                   out->zerr ? out->zerr + out->ldw * t0 : nullptr, out->ldw, s));
    if (r) {
      c->stream = saved;
      return r;
    }
  }
  c->stream = saved;
  if (legacy) {
    cudaEvent_t ev;
    TRY_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, c->stream);
    cudaStreamWaitEvent(cudaStreamLegacy, ev, 0);
    cudaEventDestroy(ev);
  }
  return PP_OK;
}

int pp_backward_phi(pp_ctx *c, const double *q_dev, int64_t nq, const double *z_dev, int64_t ldz, int64_t zstride,
                    int64_t m, const double *wgt_dev, int64_t ldwgt, double *g_dev, int32_t precision, void *stream) {
  if (!c) return -1;
  if (!q_dev && nq > 0) return -2;
  if (nq < 0) return -3;
  if (!z_dev && nq > 0) return -4;
  const int64_t n = c->g.n;
  if (ldz < n) return -5;
  if (zstride < 2 * ldz * m) return -6;
  if (m < 0 || m > n) return -7;
  if (!wgt_dev && nq > 0) return -8;
  if (ldwgt < m) return -9;
  if (!g_dev) return -10;
  if (precision != PP_PREC_FP64 && precision != PP_PREC_MIXED) return -11;
  cudaStream_t s = (cudaStream_t)stream;  // NULL: the legacy default stream
  for (int64_t t = 0; t < nq; ++t) {
    cudaError_t e = backward_phi(c->g, q_dev + 3 * t, (const z64 *)(z_dev + zstride * t), ldz, (int)m,
                                 wgt_dev + ldwgt * t, g_dev, precision, s);
    if (e != cudaSuccess) return cuda_err(e);
  }
  return PP_OK;
}

int pp_dynamical_matrix(pp_ctx *c, const double *q, int64_t derivative, char vel_method, double *d, int64_t ldd) {
  if (!c) return -1;
  if (!q) return -2;
  if (derivative < 0 || derivative > 3) return -3;
  if (derivative > 0 && vel_method != 'A' && vel_method != 'C') return -4;
  if (!d) return -5;
  const int64_t n = c->g.n;
  if (ldd < n) return -6;
  cudaStream_t s = c->stream;
  double *dq = nullptr;
  z64 *dout = nullptr;
  TRY_CUDA(cudaMalloc(&dq, 3 * sizeof(double)));
  cudaError_t e = cudaMalloc(&dout, sizeof(z64) * n * n);
  if (e != cudaSuccess) {
    cudaFree(dq);
    return PP_ERR_NOMEM;
  }
  cudaMemcpyAsync(dq, q, 3 * sizeof(double), cudaMemcpyHostToDevice, s);
  e = assemble_deriv(c->g, dq, (int)derivative, vel_method, dout, n, s);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(d, sizeof(double) * 2 * ldd, dout, sizeof(z64) * n, sizeof(z64) * n, n,
                          cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(dq);
  cudaFree(dout);
  return cuda_err(e);
}


int pp_solve_multi(pp_ctx *const *ctxs, int64_t nctx, const int64_t *cell, const double *q, int64_t ldq, int64_t nq,
                   const pp_eig_opts *o, const pp_result_view *out, int64_t *info) {
  if (!ctxs || nctx < 1) return -1;
  if (!cell && nq > 0) return -3;
  if (!q && nq > 0) return -4;
  if (ldq < nq) return -5;
  if (nq < 0) return -6;
  if (!out || !out->w || !out->m || !out->nz) return -8;
  int64_t nmax = 0, nbnd = 0, nbr = 0;
  for (int64_t k = 0; k < nctx; ++k) {
    if (!ctxs[k]) return -1;
    if (ctxs[k]->broken) return PP_ERR_STATE;
    const int r = check_opts(ctxs[k], o);
    if (r) return r == -5 ? -7 : r;
    nmax = std::max(nmax, ctxs[k]->g.n);
    nbnd = std::max(nbnd, ctxs[k]->g.nbnd);
    nbr = std::max(nbr, ctxs[k]->g.nbrows);
  }
  if (nq == 0) return PP_OK;
  for (int64_t t = 0; t < nq; ++t) {
    if (cell[t] < 0 || cell[t] >= nctx) return -3;
    for (int k = 0; k < 3; ++k)
      if (!std::isfinite(q[t + ldq * k])) return PP_ERR_NAN;
  }
  if (out->ldw < nmax) return -8;
  const bool vecs = o->jobz == 'V' || o->vel;
  const bool want_z = vecs && out->z;
  if (want_z && out->ldz < nmax) return -8;
  bool rows_only = o->vel && !want_z && !o->want_resid;
  for (int64_t k = 0; k < nctx; ++k) rows_only = rows_only && ctxs[k]->g.nbrows < ctxs[k]->g.n;
  pp_ctx *h = ctxs[0];
  const int mcap = o->range == 'I' ? (int)(o->iu - o->il + 1) : (int)nmax;
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  if (h->ws) fr += h->ws_bytes;
  int B = (int)std::min<int64_t>(nq, 64);
  while (B > 1 && ws_bytes_estimate(nmax, B, mcap, nbnd, nbr) > (size_t)(0.6 * (double)fr)) B /= 2;
  if (const char *env = getenv("PARPHOM_GPU_BATCH")) {
    const int v = atoi(env);
    if (v > 0) B = (int)std::min<int64_t>(v, nq);
  }
  int r = ensure_ws_sized(h, B, mcap, nmax, nbnd, nbr);
  if (r) return r;
  EigWork &w = h->w;
  cudaStream_t s = h->stream;
  const int prec = o->precision;
  const int fmt = prec == PP_PREC_MIXED ? 1 : 0;
  // q-points grouped by cell, so that every cell's matrices are adjacent
  std::vector<int64_t> order(nq);
  for (int64_t t = 0; t < nq; ++t) order[t] = t;
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return cell[a] < cell[b]; });
  std::vector<double> qh(3 * (size_t)B);
  std::vector<int> nv(B);
  std::vector<int64_t> mh(B), nzh(B), infoh(B);
  for (int64_t t0 = 0; t0 < nq; t0 += B) {
    const int Bb = (int)std::min<int64_t>(B, nq - t0);
    struct Seg {
      pp_ctx *c;
      int off, cnt;
    };
    std::vector<Seg> segs;
    for (int b = 0; b < Bb; ++b) {
      const int64_t t = order[t0 + b];
      pp_ctx *c = ctxs[cell[t]];
      for (int k = 0; k < 3; ++k) qh[3 * b + k] = q[t + ldq * k];
      nv[b] = (int)c->g.n;
      if (segs.empty() || segs.back().c != c)
        segs.push_back({c, b, 1});
      else
        segs.back().cnt++;
    }
    TRY_CUDA(cudaMemcpyAsync(h->d_q, qh.data(), sizeof(double) * 3 * Bb, cudaMemcpyHostToDevice, s));
    TRY_CUDA(cudaMemcpyAsync(w.nvec, nv.data(), sizeof(int) * Bb, cudaMemcpyHostToDevice, s));
    w.B = Bb;
    for (auto &g : segs) {
      EigWork v = view_of(w, g.off, g.cnt);
      TRY_CUDA(assemble_batch(g.c->g, h->d_q + 3 * g.off, g.cnt, v.A, w.lda, w.sA, fmt, s));
    }
    if (prec == PP_PREC_MIXED)
      TRY_CUDA(tridiagonalize<df>(w, s));
    else
      TRY_CUDA(tridiagonalize<double>(w, s));
    TRY_CUDA(tridiag_eigenvalues(w, o->range, o->vl / C_RANGE, o->vu / C_RANGE, o->il, o->iu, o->abstol, s,
                                 prec == PP_PREC_MIXED));
    if (needs_vectors(o)) {
      if (prec == PP_PREC_MIXED)
        TRY_CUDA(tridiag_eigenvectors<df>(w, s));
      else
        TRY_CUDA(tridiag_eigenvectors<double>(w, s));
      if (!rows_only) {
        if (prec == PP_PREC_MIXED)
          TRY_CUDA(back_transform<df>(w, s));
        else
          TRY_CUDA(back_transform<double>(w, s));
      }
      for (auto &g : segs) {
        EigWork v = view_of(w, g.off, g.cnt);
        if (rows_only) {
          if (prec == PP_PREC_MIXED)
            TRY_CUDA(back_transform_rows<df>(v, g.c->g.d_brows, (int)g.c->g.nbrows, s));
          else
            TRY_CUDA(back_transform_rows<double>(v, g.c->g.d_brows, (int)g.c->g.nbrows, s));
        }
        if (o->vel) {
          double *vr = h->vraw + (size_t)g.off * 3 * w.mcap;
          if (rows_only)
            TRY_CUDA(velocities(g.c->g, h->d_q + 3 * g.off, g.cnt, v.Eb, w.nbr, (int64_t)w.nbr * w.mcap, fmt, v.rng,
                                w.mcap, o->vel_method, vr, h->vpart, h->nsplit, g.c->g.d_rowmap, s));
          else
            TRY_CUDA(velocities(g.c->g, h->d_q + 3 * g.off, g.cnt, v.E, w.lde, w.sE, fmt, v.rng, w.mcap,
                                o->vel_method, vr, h->vpart, h->nsplit, nullptr, s));
        }
      }
    }
    TRY_CUDA(finalize_outputs(w, fmt, o->raw_lambda, h->vraw, o->vel ? 1 : 0, 0, h->d_w, nmax, nullptr, 0, 0, h->d_vel,
                              3 * (int64_t)w.mcap, h->d_m, h->d_nz, h->d_info, vecs ? 1 : 0, s));
    const bool errs = o->want_resid && (out->resid || out->werr || out->zerr);
    double *e_res = h->d_err, *e_w = h->d_err + (size_t)B * nmax, *e_z = h->d_err + 2 * (size_t)B * nmax;
    if (errs)
      for (auto &g : segs) {
        EigWork v = view_of(w, g.off, g.cnt);
        const size_t o0 = (size_t)g.off * nmax;
        TRY_CUDA(error_estimates(g.c->g, h->d_q + 3 * g.off, v, fmt, o->raw_lambda, h->vpart, e_res + o0, e_w + o0,
                                 e_z + o0, nmax, s));
      }
    TRY_CUDA(cudaMemcpyAsync(mh.data(), h->d_m, 8 * Bb, cudaMemcpyDeviceToHost, s));
    TRY_CUDA(cudaMemcpyAsync(nzh.data(), h->d_nz, 8 * Bb, cudaMemcpyDeviceToHost, s));
    TRY_CUDA(cudaMemcpyAsync(infoh.data(), h->d_info, 8 * Bb, cudaMemcpyDeviceToHost, s));
    TRY_CUDA(cudaStreamSynchronize(s));
    for (int b = 0; b < Bb; ++b) {
      const int64_t t = order[t0 + b];
      out->m[t] = mh[b];
      out->nz[t] = vecs ? nzh[b] : 0;
      if (info) info[t] = infoh[b];
      if (mh[b] > 0) {
        TRY_CUDA(cudaMemcpyAsync(out->w + out->ldw * t, h->d_w + nmax * b, sizeof(double) * mh[b],
                                 cudaMemcpyDeviceToHost, s));
        if (o->vel && out->vel)
          TRY_CUDA(cudaMemcpyAsync(out->vel + out->velstride * t, h->d_vel + 3 * (int64_t)w.mcap * b,
                                   sizeof(double) * 3 * mh[b], cudaMemcpyDeviceToHost, s));
        if (errs) {
          const double *src[3] = {e_res, e_w, e_z};
          double *dst[3] = {out->resid, out->werr, out->zerr};
          for (int f = 0; f < 3; ++f)
            if (dst[f])
              TRY_CUDA(cudaMemcpyAsync(dst[f] + out->ldw * t, src[f] + nmax * b, sizeof(double) * mh[b],
                                       cudaMemcpyDeviceToHost, s));
        }
      }
    }
    if (want_z) {
      double *zst = (double *)w.A;
      TRY_CUDA(finalize_outputs(w, fmt, o->raw_lambda, h->vraw, 0, 1, nullptr, 0, zst, w.lda, 2 * w.sA, nullptr, 0,
                                nullptr, nullptr, nullptr, 1, s));
      for (int b = 0; b < Bb; ++b) {
        const int64_t t = order[t0 + b];
        if (mh[b] > 0)
          TRY_CUDA(cudaMemcpy2DAsync(out->z + out->zstride * t, sizeof(double) * 2 * out->ldz, zst + 2 * w.sA * b,
                                     sizeof(double) * 2 * w.lda, sizeof(double) * 2 * nv[b], mh[b],
                                     cudaMemcpyDeviceToHost, s));
      }
    }
    TRY_CUDA(cudaStreamSynchronize(s));
  }
  // the workspace was sized for the largest cell: release it, the next
  // single-cell call sizes its own
  free_ws(h);
  return PP_OK;
}

}  // extern "C"
