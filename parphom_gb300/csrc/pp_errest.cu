// Per-eigenpair error estimates of a computed spectrum, in FP64.
//
// For eigenpair j of D(q) (lambda_j from the bisection, z_j the library's
// eigenvector, in either precision form) with D assembled again in FP64:
//   r = D z - lambda z,  s1 = ||r||^2,  s2 = Re z^H r,  s3 = ||z||^2
//   t = s2 / s3 = rho - lambda  (rho the Rayleigh quotient; taken from the
//   small residual, not as z^H D z - lambda, so it carries no cancellation)
//   ||D z - rho z||^2 = s1 - t^2 s3          (D z - rho z is orthogonal to z)
//   gap = distance from lambda_j to the nearest other computed eigenvalue
// and reports
//   resid = sqrt(s1 / s3)                    residual of the normalised pair
//   dlam  = min(resid, |t| + ||D z - rho z||^2 / (s3 gap))
//           an eigenvalue of D lies within resid of lambda_j for any unit
//           z; the second term is the quadratic (Kato-Temple type) estimate
//           of the Rayleigh quotient's distance to its eigenvalue plus the
//           distance from lambda_j to the Rayleigh quotient
//   werr  = the same bound carried through w = c sign(lambda) sqrt|lambda|
//           (cm^-1; lambda units with raw_lambda)
//   zerr  = min(1, ||D z - rho z|| / (sqrt(s3) gap))
//           the Davis-Kahan bound on the sine of the angle to the exact
//           eigenvector (large inside clusters of near-degenerate modes,
//           where single eigenvectors are not determined)
// The reference reports only pzheevx's INFO (diagonalize.F90:100-115); the
// estimates are the library's own.  With range 'I' or 'V' the gap is taken
// over the computed eigenvalues only.
//
// D Z is an FP64 complex product of n^2 m multiply-adds per q-point (CUDA
// cores, 64 x 64 output tiles); its epilogue reduces the three sums per
// column over each tile's rows and adds them to per-column totals.
#include "pp_internal.cuh"

namespace pp {

namespace {

constexpr int ER_T = 64, ER_K = 16;

template <int EFMT>
__device__ __forceinline__ z64 ld_vec(const void *E, int64_t off) {
  if (EFMT == 0) return ((const z64 *)E)[off];
  const zdf v = ((const zdf *)E)[off];
  return z64{df_to(v.re), df_to(v.im)};
}

// sums[b][0..2][j] += (s1, s2, s3) over the 64 rows of this tile.
template <int EFMT>
__global__ void __launch_bounds__(256) k_resid(const z64 *Db, int64_t ldd, int64_t sD, const void *E, int64_t lde,
                                               int64_t sE, const double *ww, int64_t sd, const int *nvec,
                                               const int64_t *rng, double *sums, int64_t mstride) {
  // the two operand tiles; after the product the same bytes hold the
  // epilogue's per-column partial sums
  __shared__ __align__(16) unsigned char raw[2 * ER_K * (ER_T + 1) * sizeof(z64)];
  z64(*sDt)[ER_T + 1] = (z64(*)[ER_T + 1])raw;
  z64(*sZ)[ER_T + 1] = (z64(*)[ER_T + 1])(raw + ER_K * (ER_T + 1) * sizeof(z64));
  double(*red)[16][ER_T] = (double(*)[16][ER_T])raw;
  static_assert(3 * 16 * ER_T * sizeof(double) <= sizeof(raw), "epilogue sums fit the operand tiles");
  const int b = blockIdx.z;
  const int n = nvec[b];
  const int m = (int)rng[b * 8 + 2];
  const int r0 = blockIdx.x * ER_T, c0 = blockIdx.y * ER_T;
  if (r0 >= n || c0 >= m) return;
  const z64 *D = Db + b * sD;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  z64 acc[4][4];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = z64{0.0, 0.0};
  for (int k0 = 0; k0 < n; k0 += ER_K) {
    for (int e = threadIdx.x; e < ER_K * ER_T; e += 256) {
      const int x = e % ER_T, y = e / ER_T;
      const int k = k0 + y;
      const int r = r0 + x, c = c0 + x;
      sDt[y][x] = (k < n && r < n) ? D[r + ldd * k] : z64{0.0, 0.0};
      sZ[y][x] = (k < n && c < m) ? ld_vec<EFMT>(E, b * sE + k + lde * c) : z64{0.0, 0.0};
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < ER_K; ++k) {
      z64 d[4], z[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        d[p] = sDt[k][tx + 16 * p];
        z[p] = sZ[k][ty + 16 * p];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          acc[p][q].re = fma(d[p].re, z[q].re, acc[p][q].re);
          acc[p][q].re = fma(-d[p].im, z[q].im, acc[p][q].re);
          acc[p][q].im = fma(d[p].re, z[q].im, acc[p][q].im);
          acc[p][q].im = fma(d[p].im, z[q].re, acc[p][q].im);
        }
    }
    __syncthreads();
  }
  // epilogue: per column q of this thread, its 4 rows' contributions
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int c = c0 + ty + 16 * q;
    double s1 = 0.0, s2 = 0.0, s3 = 0.0;
    if (c < m) {
      const double lam = ww[b * sd + c];
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        const int r = r0 + tx + 16 * p;
        if (r < n) {
          const z64 z = ld_vec<EFMT>(E, b * sE + r + lde * c);
          const double xr = acc[p][q].re - lam * z.re, xi = acc[p][q].im - lam * z.im;
          s1 += xr * xr + xi * xi;
          s2 += z.re * xr + z.im * xi;
          s3 += z.re * z.re + z.im * z.im;
        }
      }
    }
    red[0][tx][ty + 16 * q] = s1;
    red[1][tx][ty + 16 * q] = s2;
    red[2][tx][ty + 16 * q] = s3;
  }
  __syncthreads();
  if (threadIdx.x < 3 * ER_T) {
    const int f = threadIdx.x / ER_T, cl = threadIdx.x % ER_T;
    const int c = c0 + cl;
    if (c < m) {
      double s = 0.0;
      for (int t = 0; t < 16; ++t) s += red[f][t][cl];
      atomicAdd(&sums[((int64_t)b * 3 + f) * mstride + c], s);
    }
  }
}

__global__ void k_errfin(const double *sums, int64_t mstride, const double *ww, int64_t sd, const int64_t *rng,
                         int raw, double c_w, double *resid, double *werr, double *zerr, int64_t ldw) {
  const int b = blockIdx.y;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t m = rng[b * 8 + 2];
  if (j >= m) return;
  const double s1 = sums[((int64_t)b * 3 + 0) * mstride + j];
  const double s2 = sums[((int64_t)b * 3 + 1) * mstride + j];
  const double s3 = fmax(sums[((int64_t)b * 3 + 2) * mstride + j], 1e-300);
  const double *w = ww + b * sd;
  const double lam = w[j];
  double gap = INFINITY;
  if (j > 0) gap = fmin(gap, lam - w[j - 1]);
  if (j + 1 < m) gap = fmin(gap, w[j + 1] - lam);
  gap = fmax(gap, 1e-300);
  const double res = sqrt(s1 / s3);
  const double t = s2 / s3;
  const double rr = fmax(s1 - t * t * s3, 0.0) / s3;  // ||D z - rho z||^2 / ||z||^2
  const double dlam = fmin(res, fabs(t) + rr / gap);
  double we = dlam;
  if (!raw) {
    // |f(a) - f(b)| for f(x) = sign(x) sqrt|x|: at most |a-b| / (sqrt|a| +
    // sqrt(|a| - |a-b|)) when |a| > |a-b|, else sqrt(2 |a-b|)
    const double al = fabs(lam);
    we = c_w * (al > dlam ? dlam / (sqrt(al) + sqrt(al - dlam)) : sqrt(2.0 * dlam));
  }
  if (resid) resid[b * ldw + j] = res;
  if (werr) werr[b * ldw + j] = we;
  if (zerr) zerr[b * ldw + j] = fmin(1.0, sqrt(rr) / gap);
}

}  // namespace

cudaError_t error_estimates(const Geometry &g, const double *d_q, EigWork &w, int efmt, int raw_lambda,
                            double *sums, double *resid, double *werr, double *zerr, int64_t ldw, cudaStream_t s) {
  // D(q) again, in FP64, into the reduction's buffer (free after the
  // back-transform)
  PP_CUDA_TRY(assemble_batch(g, d_q, w.B, w.A, w.lda, w.sA, 0, s));
  const int64_t mstride = w.mcap;
  PP_CUDA_TRY(cudaMemsetAsync(sums, 0, sizeof(double) * 3 * (size_t)w.B * mstride, s));
  dim3 grid((unsigned)((w.nmax + ER_T - 1) / ER_T), (unsigned)((w.mcap + ER_T - 1) / ER_T), (unsigned)w.B);
  if (efmt == 0)
    k_resid<0><<<grid, 256, 0, s>>>((const z64 *)w.A, w.lda, w.sA, w.E, w.lde, w.sE, w.w, w.nmax, w.nvec, w.rng,
                                    sums, mstride);
  else
    k_resid<1><<<grid, 256, 0, s>>>((const z64 *)w.A, w.lda, w.sA, w.E, w.lde, w.sE, w.w, w.nmax, w.nvec, w.rng,
                                    sums, mstride);
  const double c_w = (double)15.633302f * (double)33.35641f;  // write_output.F90:135
  dim3 gf((unsigned)((w.nmax + 127) / 128), (unsigned)w.B);
  k_errfin<<<gf, 128, 0, s>>>(sums, mstride, w.w, w.nmax, w.rng, raw_lambda, c_w, resid, werr, zerr, ldw);
  count_launch(2);
  return cudaGetLastError();
}

}  // namespace pp
