// Hermitian eigenvalues without any device allocation.
//
// Some callers cannot call cudaMalloc: drivers that hand the library a
// pre-sized device pool and forbid hidden allocations (an allocation there
// would break the pool's accounting or fail outright once the pool owns the
// memory), stream-ordered pipelines they do not own, where an allocation
// would synchronise the device, and long runs that must not grow the device
// footprint once started.  pp_heevx_values_noalloc serves them: the caller
// passes the matrix and the output buffers, and every scratch buffer of the
// FP64 reduction-and-bisection pipeline lives in the file-scope device array
// below, of fixed size (about 2.0 MB for n <= 1536), which every GPU that
// loads the library holds until the process exits.
#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/parphom_gpu.h"
#include "pp_internal.cuh"

namespace {

constexpr int64_t NOALLOC_MAX_N = PP_NOALLOC_MAX_N;
constexpr int64_t NB = 32;
constexpr int64_t LDA_MAX = (NOALLOC_MAX_N + 7) / 8 * 8;
constexpr int64_t NCHUNK_MAX = (NOALLOC_MAX_N + 31) / 32;
constexpr int64_t NRB_MAX = (NOALLOC_MAX_N + 31) / 32 + 1;

constexpr size_t al(size_t x) { return (x + 255) & ~(size_t)255; }
// byte offsets of the scratch buffers inside the array
constexpr size_t OFF_NVEC = 0;
constexpr size_t OFF_W = al(OFF_NVEC + sizeof(int));
constexpr size_t OFF_P = al(OFF_W + 16 * (size_t)LDA_MAX * NB);
constexpr size_t OFF_X = al(OFF_P + 16 * (size_t)NCHUNK_MAX * LDA_MAX);
constexpr size_t OFF_NRM = al(OFF_X + 16 * 2 * NB);
constexpr size_t OFF_WV = al(OFF_NRM + 8 * (size_t)NRB_MAX);
constexpr size_t OFF_D = al(OFF_WV + 16 * (size_t)NRB_MAX);
constexpr size_t OFF_E = al(OFF_D + 8 * (size_t)NOALLOC_MAX_N);
constexpr size_t OFF_TAU = al(OFF_E + 8 * (size_t)NOALLOC_MAX_N);
constexpr size_t OFF_SCAL = al(OFF_TAU + 16 * (size_t)NOALLOC_MAX_N);
constexpr size_t OFF_WW = al(OFF_SCAL + 16 * 4);
constexpr size_t OFF_RNG = al(OFF_WW + 8 * (size_t)NOALLOC_MAX_N);
constexpr size_t OFF_TINFO = al(OFF_RNG + 8 * 8);
constexpr size_t OFF_INFO = al(OFF_TINFO + 8 * 8);
constexpr size_t OFF_BAD = al(OFF_INFO + 8);
constexpr size_t SCRATCH_BYTES = al(OFF_BAD + 8);
// The W panel (0.79 MB) and the mat-vec partial sums (1.18 MB) dominate.
static_assert(SCRATCH_BYTES > 1900000 && SCRATCH_BYTES < 2100000, "scratch size as documented: about 2.0 MB");

}  // namespace

// The scratch array (about 2.0 MB).  Device code could name it directly;
// host code only ever uses the address cudaGetSymbolAddress returns for the
// current device, never the host-side symbol itself.
static __device__ __align__(256) unsigned char pp_noalloc_scratch[SCRATCH_BYTES];

namespace {

constexpr int MAX_DEVICES = 64;
std::mutex g_mu;
void *g_scratch[MAX_DEVICES] = {};

// Once per device, with that device current: resolve the array's address.
// The address is kept for the life of the process: after a cudaDeviceReset
// the module is loaded again and the array may move, so the entry point must
// not be used across a device reset.
int scratch_for_current_device(unsigned char **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return PP_ERR_NODEVICE;
  }
  if (dev < 0 || dev >= MAX_DEVICES) return PP_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_scratch[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, pp_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return e == cudaErrorNoKernelImageForDevice ? PP_ERR_NODEVICE : PP_ERR_CUDA;
    }
    g_scratch[dev] = p;
  }
  *out = (unsigned char *)g_scratch[dev];
  return PP_OK;
}

// Zero the per-call state that must start at zero (the array keeps what the
// previous call left in it).
__global__ void k_na_reset(int *nvec, int64_t n, int64_t *info, int *bad) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    *nvec = (int)n;
    *info = 0;
    *bad = 0;
  }
}

// Lower triangle := conjugate of the upper triangle (only 'U' is referenced,
// as pzheevx does).  A non-finite element of the upper triangle is replaced
// by zero and flagged: the call then reports PP_INFO_NAN and no eigenvalues
// (pp_solve_batch rejects such input on the host; here the matrix is only
// in device memory).
__global__ void k_na_prepare(z64 *A, int64_t lda, int64_t n, int *bad) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t c = blockIdx.y;
  if (r >= n || c >= n || r < c) return;
  z64 u = A[c + lda * r];
  if (!isfinite(u.re) || !isfinite(u.im)) {
    u = z64{0.0, 0.0};
    A[c + lda * r] = u;
    atomicExch(bad, 1);
  }
  if (r > c) A[r + lda * c] = z64{u.re, -u.im};
}

__global__ void k_na_finish(const int64_t *rng, const int64_t *info_in, const int *bad, int64_t *m_out,
                            int64_t *info_out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    *m_out = *bad ? 0 : rng[2];
    *info_out = *info_in | (*bad ? PP_INFO_NAN : 0);
  }
}

}  // namespace

extern "C" PP_API int pp_heevx_values_noalloc(double *a_dev, int64_t lda, int64_t n, char range, double vl,
                                              double vu, int64_t il, int64_t iu, double abstol, double *w_dev,
                                              int64_t *m_dev, int64_t *info_dev, void *stream) {
  if (n < 1) return -3;
  if (n > NOALLOC_MAX_N) return PP_ERR_SIZE;
  if (!a_dev) return -1;
  if (lda < n || lda > LDA_MAX) return -2;
  if (range != 'A' && range != 'I' && range != 'V') return -4;
  if (range == 'I' && (il < 1 || iu > n || il > iu)) return -7;
  if (range == 'V' && !(vl < vu)) return -5;
  if (!w_dev) return -10;
  if (!m_dev) return -11;
  if (!info_dev) return -12;
  unsigned char *base = nullptr;
  int rc = scratch_for_current_device(&base);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  pp::EigWork w;
  w.B = 1;
  w.nmax = (int)n;
  w.mcap = 0;
  w.nb = (int)NB;
  w.nvec = (int *)(base + OFF_NVEC);
  w.A = a_dev;
  w.lda = lda;
  w.sA = lda * n;
  w.W = base + OFF_W;
  w.P = base + OFF_P;
  w.nchunk = (int)((n + 31) / 32);
  w.X = base + OFF_X;
  w.nrm = (double *)(base + OFF_NRM);
  w.wv = (z64 *)(base + OFF_WV);
  w.nrb = (int)NRB_MAX;
  w.d = (double *)(base + OFF_D);
  w.e = (double *)(base + OFF_E);
  w.tau = (z64 *)(base + OFF_TAU);
  w.scal = (z64 *)(base + OFF_SCAL);
  w.w = (double *)(base + OFF_WW);
  w.rng = (int64_t *)(base + OFF_RNG);
  w.tinfo = (double *)(base + OFF_TINFO);
  w.info = (int64_t *)(base + OFF_INFO);
  int *bad = (int *)(base + OFF_BAD);
  k_na_reset<<<1, 32, 0, s>>>(w.nvec, n, w.info, bad);
  k_na_prepare<<<dim3((unsigned)((n + 127) / 128), (unsigned)n), 128, 0, s>>>((z64 *)a_dev, lda, n, bad);
  cudaError_t e = pp::tridiagonalize<double>(w, s);
  if (e == cudaSuccess) e = pp::tridiag_eigenvalues(w, range, vl, vu, il, iu, abstol, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(w_dev, w.w, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) {
    k_na_finish<<<1, 32, 0, s>>>(w.rng, w.info, bad, m_dev, info_dev);
    e = cudaGetLastError();
  }
  pp::count_launch(3);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return PP_ERR_CUDA;
  }
  return PP_OK;
}
