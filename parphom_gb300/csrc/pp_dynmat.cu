// Dynamical-matrix assembly, group velocities and output conversion.
//
// D(q) element (dynamical_matrix.F90:200-262): for matrix element (r, c),
// atoms I = r/3, J = c/3 (0-based); over the nine in-plane images
// t = (i, j, 0), i, j in {-1,0,1}, the distance |x_I - lat^T (c_J + t)| is
// computed from the Cartesian position of I and the reduced coordinates of
// J; the images within 1e-10 (single-precision literal) of the minimum form
// the tie set S_IJ, and
//   D(r,c) = Phi(r,c) * mean_{t in S_IJ} exp(-2 pi_f i q.(c_J + t - c_I))
//            / sqrt(m_I m_J),
// pi_f being the float-rounded pi the reference's source literal yields.
//
// The eigensolver references only the upper triangle of D (pzheevx with
// uplo 'U', diagonalize.F90:73), so the assembly writes the Hermitian matrix
// defined by the upper triangle: block (I,J) with I > J is the conjugate
// transpose of block (J,I), computed in the (J,I) orientation.  Phi is kept
// on the device with its upper triangle mirrored, so both triangles read it
// with coalesced loads.
//
// Group velocities.  Writing x_I = lat^T c_I, the analytic derivative
// (dynamical_matrix.F90:250-253) splits exactly into
//   dD/dk = -i (D X_k - X_k D) + B_k,
//   B_k(r,c) = Phi(r,c)/sqrt(m_I m_J) * mean_t (-i (lat^T t)_k) exp(...),
// with X_k = diag(x_{I,k}).  For an eigenvector e of D the commutator term
// has zero expectation, so Re e^H dD/dk e = Re e^H B_k e exactly; B_k is
// nonzero only on "boundary" blocks whose tie set holds a non-zero image.
// The central-difference option (dynamical_matrix.F90:133-149) is treated
// the same way: the home-image part of D(q +- delta/2) is a unitary
// similarity of D(q) (diag(exp(2 pi_f i delta.c/2))), whose contribution to
// the difference quotient is O(delta^2); the boundary blocks carry
//   [D(q+delta/2) - D(q-delta/2)]/|delta| restricted to the image factor.
#include <cfloat>

#include "pp_internal.cuh"

namespace pp {

constexpr double PI_REF = (double)3.141592653589793f;  // dynamical_matrix.F90:211
constexpr double TOL_REF = (double)1e-10f;             // dynamical_matrix.F90:212
// velocity and unit constants, write_output.F90:135, 443-446
constexpr double C1_REF = (double)15.633302f;
constexpr double C2_REF = (double)33.35641f;
constexpr double VEL_C2SQ = (double)(15.633302f * 15.633302f);
constexpr double PIF_REF = (double)3.141592653589793f;
constexpr int HOME_IMAGE = 4;  // l = 5 of the reference's 9-image loop: (i,j) = (0,0)

static inline int cdiv(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// Tie-set mask of the pair (ia, ja) in the reference's orientation.
__device__ __forceinline__ uint32_t tie_mask(const double *lat, const double *crys, const double *pos, int64_t N,
                                             int64_t ia, int64_t ja) {
  double nb[9];
  const double cj0 = crys[ja], cj1 = crys[ja + N], cj2 = crys[ja + 2 * N];
  const double x0 = pos[ia], x1 = pos[ia + N], x2 = pos[ia + 2 * N];
#pragma unroll
  for (int l = 0; l < 9; ++l) {
    const int i = l / 3 - 1;
    const int j = l - 1 - 3 * (i + 1);
    const double rs0 = __dadd_rn(cj0, (double)i), rs1 = __dadd_rn(cj1, (double)j), rs2 = cj2;
    double rc[3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
      rc[a] = __dadd_rn(__dadd_rn(__dmul_rn(lat[0 + 3 * a], rs0), __dmul_rn(lat[1 + 3 * a], rs1)),
                        __dmul_rn(lat[2 + 3 * a], rs2));
    const double dx = __dsub_rn(x0, rc[0]), dy = __dsub_rn(x1, rc[1]), dz = __dsub_rn(x2, rc[2]);
    nb[l] = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)));
  }
  double mn = nb[0];
#pragma unroll
  for (int l = 1; l < 9; ++l) mn = nb[l] < mn ? nb[l] : mn;
  uint32_t mask = 0;
  const double lim = __dadd_rn(mn, TOL_REF);
#pragma unroll
  for (int l = 0; l < 9; ++l)
    if (nb[l] < lim) mask |= 1u << l;
  return mask;
}

// prephase = q . (c_J + t - c_I), left-to-right as the reference evaluates it.
__device__ __forceinline__ double prephase(const double *q, const double *crys, int64_t N, int64_t ia, int64_t ja,
                                           int i, int j) {
  const double r0 = __dsub_rn(__dadd_rn(crys[ja], (double)i), crys[ia]);
  const double r1 = __dsub_rn(__dadd_rn(crys[ja + N], (double)j), crys[ia + N]);
  const double r2 = __dsub_rn(crys[ja + 2 * N], crys[ia + 2 * N]);
  return __dadd_rn(__dadd_rn(__dmul_rn(q[0], r0), __dmul_rn(q[1], r1)), __dmul_rn(q[2], r2));
}

// ---------------------------------------------------------------------------
// geometry tables
__global__ void k_masks(const double *lat9, const double *crys, const double *pos, int64_t N, uint16_t *mask) {
  __shared__ double lat[9];
  if (threadIdx.x < 9) lat[threadIdx.x] = lat9[threadIdx.x];
  __syncthreads();
  const int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t J = blockIdx.y;
  if (I >= N) return;
  const int64_t lo = I < J ? I : J, hi = I < J ? J : I;
  mask[I + N * J] = (uint16_t)tie_mask(lat, crys, pos, N, lo, hi);
}

// Phi(r,c) for r > c := Phi(c,r) (tiled transpose of the upper triangle).
__global__ void k_mirror(double *fc, int64_t n) {
  __shared__ double tile[32][33];
  const int64_t bx = blockIdx.x, by = blockIdx.y;  // tile (row block bx, col block by), lower: bx > by
  if (bx < by) return;
  const int64_t r0 = bx * 32, c0 = by * 32;
  // read the transposed tile from the upper triangle: element (c0+x, r0+y)
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t rr = c0 + threadIdx.x, cc = r0 + y;
    tile[y][threadIdx.x] = (rr < n && cc < n) ? fc[rr + n * cc] : 0.0;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int64_t rr = r0 + threadIdx.x, cc = c0 + y;
    if (rr < n && cc < n && rr > cc) fc[rr + n * cc] = tile[threadIdx.x][y];
  }
}

// Phi_II = -sum_{J != I} Phi_IJ, symmetrised.
__global__ void k_asr(double *fc, int64_t N) {
  const int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= N) return;
  const int64_t n = 3 * N;
  double s[3][3] = {};
  for (int64_t J = 0; J < N; ++J) {
    if (J == I) continue;
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) s[a][b] += fc[(3 * I + a) + n * (3 * J + b)];
  }
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) fc[(3 * I + a) + n * (3 * I + b)] = -0.5 * (s[a][b] + s[b][a]);
}

__global__ void k_block_nonzero(const double *fc, int64_t N, uint8_t *flag) {
  const int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t J = blockIdx.y;
  if (I >= N) return;
  const int64_t n = 3 * N;
  uint8_t nz = 0;
  for (int b = 0; b < 3; ++b)
    for (int a = 0; a < 3; ++a) nz |= fc[(3 * I + a) + n * (3 * J + b)] != 0.0;
  flag[I + N * J] = nz;
}

cudaError_t geom_build_masks(Geometry &g, cudaStream_t s) {
  double *dlat;
  PP_CUDA_TRY(cudaMallocAsync(&dlat, 9 * sizeof(double), s));
  PP_CUDA_TRY(cudaMemcpyAsync(dlat, g.lat, 9 * sizeof(double), cudaMemcpyHostToDevice, s));
  dim3 grid(cdiv(g.natom, 128), (unsigned)g.natom);
  k_masks<<<grid, 128, 0, s>>>(dlat, g.d_crys, g.d_pos, g.natom, g.d_mask);
  count_launch(1);
  PP_CUDA_TRY(cudaFreeAsync(dlat, s));
  return cudaGetLastError();
}

cudaError_t geom_symmetrize_fc(Geometry &g, int enforce_asr, cudaStream_t s) {
  const int nt = cdiv(g.n, 32);
  k_mirror<<<dim3(nt, nt), dim3(32, 8), 0, s>>>(g.d_fc, g.n);
  count_launch(1);
  if (enforce_asr) {
    k_asr<<<cdiv(g.natom, 128), 128, 0, s>>>(g.d_fc, g.natom);
    count_launch(1);
  }
  return cudaGetLastError();
}

cudaError_t geom_block_nonzero(const Geometry &g, uint8_t *d_flags, cudaStream_t s) {
  k_block_nonzero<<<dim3(cdiv(g.natom, 128), (unsigned)g.natom), 128, 0, s>>>(g.d_fc, g.natom, d_flags);
  count_launch(1);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// assembly of the Hermitian D(q) for a batch of q
struct GeoDev {
  const double *fc, *crys, *mass;
  const uint16_t *mask;
  int64_t N, n;
};

template <int DFMT>
__global__ void __launch_bounds__(128) k_assemble(GeoDev g, const double *qb, void *Ab, int64_t lda, int64_t sA) {
  const int64_t N = g.N, n = g.n;
  const int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t J = blockIdx.y;
  const int b = blockIdx.z;
  if (I >= N) return;
  const double q[3] = {qb[3 * b], qb[3 * b + 1], qb[3 * b + 2]};
  const int64_t lo = I < J ? I : J, hi = I < J ? J : I;
  const uint32_t mask = g.mask[I + N * J];
  double pr = 0.0, pi = 0.0;
  int mult = 0;
  for (int l = 0; l < 9; ++l) {
    if (!((mask >> l) & 1u)) continue;
    const int i = l / 3 - 1;
    const int j = l - 1 - 3 * (i + 1);
    const double p = prephase(q, g.crys, N, lo, hi, i, j);
    const double th = -(__dmul_rn(2.0 * PI_REF, p));
    double sn, cs;
    sincos(th, &sn, &cs);
    pr += cs;
    pi += sn;
    ++mult;
  }
  if (I > J) pi = -pi;  // lower block: conjugate of the upper computation
  const double inv = 1.0 / ((double)mult * sqrt(g.mass[lo] * g.mass[hi]));
  const double cr = pr * inv, ci = pi * inv;
  const double *F = g.fc;
#pragma unroll
  for (int bb = 0; bb < 3; ++bb) {
    const int64_t c = 3 * J + bb;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const int64_t r = 3 * I + a;
      const double f = F[r + n * c];
      double re = f * cr, im = f * ci;
      if (r == c) im = 0.0;
      const int64_t off = b * sA + r + lda * c;
      if (DFMT == 0) {
        ((z64 *)Ab)[off] = z64{re, im};
      } else {
        ((zdf *)Ab)[off] = zdf{df_from(re), df_from(im)};
      }
    }
  }
}

cudaError_t assemble_batch(const Geometry &g, const double *d_q, int B, void *A, int64_t lda, int64_t sA, int dfmt,
                           cudaStream_t s) {
  GeoDev gd{g.d_fc, g.d_crys, g.d_mass, g.d_mask, g.natom, g.n};
  dim3 grid(cdiv(g.natom, 128), (unsigned)g.natom, B);
  if (dfmt == 0)
    PP_KT(KT_ASSEMBLE, s, (k_assemble<0><<<grid, 128, 0, s>>>(gd, d_q, A, lda, sA)));
  else
    PP_KT(KT_ASSEMBLE, s, (k_assemble<1><<<grid, 128, 0, s>>>(gd, d_q, A, lda, sA)));
  count_launch(1);
  return cudaGetLastError();
}

// Every element in its own (row atom, column atom) orientation, as the
// reference's block-cyclic walk produces it; derivative 0..3.
struct DerivArgs {
  double lat[9];
  double dcrys[3];
  double dnorm;
};
__global__ void __launch_bounds__(128) k_assemble_deriv(GeoDev g, const double *pos, DerivArgs da, const double *q,
                                                        int derivative, char method, z64 *out, int64_t ldo) {
  const int64_t N = g.N, n = g.n;
  const int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t J = blockIdx.y;
  if (I >= N) return;
  const uint32_t mask = tie_mask(da.lat, g.crys, pos, N, I, J);
  double qs[2][3];
  int nq = 1;
  for (int k = 0; k < 3; ++k) qs[0][k] = q[k];
  if (derivative != 0 && method != 'A') {
    nq = 2;
    for (int k = 0; k < 3; ++k) {
      qs[0][k] = q[k] + da.dcrys[k] / 2;
      qs[1][k] = q[k] - da.dcrys[k] / 2;
    }
  }
  double res[2][2] = {{0, 0}, {0, 0}};
  int mult = 0;
  for (int l = 0; l < 9; ++l) {
    if (!((mask >> l) & 1u)) continue;
    const int i = l / 3 - 1;
    const int j = l - 1 - 3 * (i + 1);
    for (int s = 0; s < nq; ++s) {
      const double p = prephase(qs[s], g.crys, N, I, J, i, j);
      const double th = -(__dmul_rn(2.0 * PI_REF, p));
      double sn, cs;
      sincos(th, &sn, &cs);
      if (derivative == 0 || method != 'A') {
        res[s][0] += cs;
        res[s][1] += sn;
      } else {
        const double r0 = __dsub_rn(__dadd_rn(g.crys[J], (double)i), g.crys[I]);
        const double r1 = __dsub_rn(__dadd_rn(g.crys[J + N], (double)j), g.crys[I + N]);
        const double r2 = __dsub_rn(g.crys[J + 2 * N], g.crys[I + 2 * N]);
        const int k = derivative - 1;
        const double x = __dadd_rn(__dadd_rn(__dmul_rn(da.lat[0 + 3 * k], r0), __dmul_rn(da.lat[1 + 3 * k], r1)),
                                   __dmul_rn(da.lat[2 + 3 * k], r2));
        res[s][0] += sn * x;
        res[s][1] -= cs * x;
      }
    }
    ++mult;
  }
  const double sm = sqrt(g.mass[I] * g.mass[J]);
  for (int bb = 0; bb < 3; ++bb) {
    const int64_t c = 3 * J + bb;
    for (int a = 0; a < 3; ++a) {
      const int64_t r = 3 * I + a;
      const double f = g.fc[r + n * c];
      double re, im;
      if (nq == 1) {
        re = f * res[0][0] / (double)mult / sm;
        im = f * res[0][1] / (double)mult / sm;
      } else {
        const double pr = f * res[0][0] / (double)mult / sm, pi = f * res[0][1] / (double)mult / sm;
        const double mr = f * res[1][0] / (double)mult / sm, mi = f * res[1][1] / (double)mult / sm;
        re = (pr - mr) / da.dnorm;
        im = (pi - mi) / da.dnorm;
      }
      out[r + ldo * c] = z64{re, im};
    }
  }
}

cudaError_t assemble_deriv(const Geometry &g, const double *d_q, int derivative, char method, z64 *out, int64_t ldo,
                           cudaStream_t s) {
  GeoDev gd{g.d_fc, g.d_crys, g.d_mass, g.d_mask, g.natom, g.n};
  DerivArgs da;
  for (int k = 0; k < 9; ++k) da.lat[k] = g.lat[k];
  da.dnorm = 1.0;
  da.dcrys[0] = da.dcrys[1] = da.dcrys[2] = 0.0;
  if (derivative >= 1 && derivative <= 3) {
    for (int k = 0; k < 3; ++k) da.dcrys[k] = g.delta_crys[derivative - 1][k];
    da.dnorm = g.delta_norm[derivative - 1];
  }
  dim3 grid(cdiv(g.natom, 128), (unsigned)g.natom);
  k_assemble_deriv<<<grid, 128, 0, s>>>(gd, g.d_pos, da, d_q, derivative, method, out, ldo);
  count_launch(1);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// group velocities
struct VelArgs {
  double lat[9];
  double dcrys[3][3];
  double dnorm[3];
};

// gtab[b][blk][k] = image factor of boundary block blk for direction k.
__global__ void k_vel_gtab(const int2 *bnd, const uint16_t *bmask, int64_t nbnd, const double *crys,
                           const double *mass, int64_t N, VelArgs va, const double *qb, char method, z64 *gtab) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int b = blockIdx.y;
  if (t >= nbnd) return;
  const double q[3] = {qb[3 * b], qb[3 * b + 1], qb[3 * b + 2]};
  const int2 p = bnd[t];
  const int64_t I = p.x, J = p.y;
  const uint32_t mask = bmask[t];
  z64 g[3] = {{0, 0}, {0, 0}, {0, 0}};
  int mult = 0;
  for (int l = 0; l < 9; ++l) {
    if (!((mask >> l) & 1u)) continue;
    ++mult;
    if (l == HOME_IMAGE) continue;
    const int i = l / 3 - 1;
    const int j = l - 1 - 3 * (i + 1);
    const double pp = prephase(q, crys, N, I, J, i, j);
    const double th = -(__dmul_rn(2.0 * PI_REF, pp));
    double sn, cs;
    sincos(th, &sn, &cs);
    for (int k = 0; k < 3; ++k) {
      if (method == 'A') {
        const double T = va.lat[0 + 3 * k] * i + va.lat[1 + 3 * k] * j;  // (lat^T t)_k
        g[k].re += T * sn;   // -i T (cs + i sn) = T sn - i T cs
        g[k].im -= T * cs;
      } else {
        // (exp(-i phi) - exp(+i phi)) / |delta| = -2 i sin(phi)/|delta|, phi = pi_f delta_k . t
        const double phi = PI_REF * (va.dcrys[k][0] * i + va.dcrys[k][1] * j);
        const double f = -2.0 * sin(phi) / va.dnorm[k];
        g[k].re += -f * sn;  // (cs + i sn) * (i f) = -f sn + i f cs
        g[k].im += f * cs;
      }
    }
  }
  const double inv = 1.0 / ((double)mult * sqrt(mass[I] * mass[J]));
  for (int k = 0; k < 3; ++k) gtab[((int64_t)b * nbnd + t) * 3 + k] = z64{g[k].re * inv, g[k].im * inv};
}

template <int EFMT>
__device__ __forceinline__ z64 ld_e(const void *E, int64_t off) {
  if (EFMT == 0) return ((const z64 *)E)[off];
  const zdf v = ((const zdf *)E)[off];
  return z64{df_to(v.re), df_to(v.im)};
}

// part[b][split][k][j] = sum over this split's blocks of 2 Re(g_k h),
// h = e_I^H Phi_IJ e_J for mode j.
template <int EFMT>
__global__ void __launch_bounds__(128) k_vel(const int2 *bnd, int64_t nbnd, const double *fc, int64_t n,
                                            const z64 *gtab, const void *E, int64_t lde, int64_t sE,
                                            const int64_t *rng, int nsplit, int64_t mstride, double *part,
                                            const int *rowmap) {
  const int b = blockIdx.z;
  const int split = blockIdx.y;
  const int64_t m = rng[b * 8 + 2];
  const int64_t jm = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t per = (nbnd + nsplit - 1) / nsplit;
  const int64_t t0 = split * per, t1 = min(nbnd, t0 + per);
  double v0 = 0.0, v1 = 0.0, v2 = 0.0;
  if (jm < m) {
    const int64_t col = b * sE + lde * jm;
    int64_t lastI = -1;
    z64 eI[3];
    for (int64_t t = t0; t < t1; ++t) {
      const int2 p = bnd[t];
      if (p.x != lastI) {
        for (int a = 0; a < 3; ++a) {
          const int64_t r = 3 * (int64_t)p.x + a;
          eI[a] = ld_e<EFMT>(E, col + (rowmap ? rowmap[r] : r));
        }
        lastI = p.x;
      }
      z64 eJ[3];
      for (int a = 0; a < 3; ++a) {
        const int64_t r = 3 * (int64_t)p.y + a;
        eJ[a] = ld_e<EFMT>(E, col + (rowmap ? rowmap[r] : r));
      }
      z64 h{0.0, 0.0};
      for (int a = 0; a < 3; ++a) {
        double fr = 0.0, fi = 0.0;
        for (int bb = 0; bb < 3; ++bb) {
          const double f = fc[(3 * (int64_t)p.x + a) + n * (3 * (int64_t)p.y + bb)];
          fr += f * eJ[bb].re;
          fi += f * eJ[bb].im;
        }
        // conj(eI[a]) * (fr + i fi)
        h.re += eI[a].re * fr + eI[a].im * fi;
        h.im += eI[a].re * fi - eI[a].im * fr;
      }
      const z64 *g = gtab + ((int64_t)b * nbnd + t) * 3;
      v0 += 2.0 * (g[0].re * h.re - g[0].im * h.im);
      v1 += 2.0 * (g[1].re * h.re - g[1].im * h.im);
      v2 += 2.0 * (g[2].re * h.re - g[2].im * h.im);
    }
    double *o = part + (((int64_t)b * nsplit + split) * 3) * mstride;
    o[jm] = v0;
    o[mstride + jm] = v1;
    o[2 * mstride + jm] = v2;
  }
}

__global__ void k_vel_reduce(const double *part, int nsplit, int64_t mstride, const int64_t *rng, double *vraw) {
  const int b = blockIdx.y;
  const int64_t jm = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t m = rng[b * 8 + 2];
  if (jm >= m) return;
  for (int k = 0; k < 3; ++k) {
    double s = 0.0;
    for (int sp = 0; sp < nsplit; ++sp) s += part[(((int64_t)b * nsplit + sp) * 3 + k) * mstride + jm];
    vraw[((int64_t)b * 3 + k) * mstride + jm] = s;
  }
}

cudaError_t velocities(const Geometry &g, const double *d_q, int B, const void *E, int64_t lde, int64_t sE, int efmt,
                       const int64_t *d_rng, int mmax, char method, double *d_vraw, double *d_part, int nsplit,
                       const int *rowmap, cudaStream_t s) {
  // d_part must hold B*nsplit*3*mmax doubles plus the gtab (B*nbnd*3 z64) after it
  const int64_t mstride = mmax;
  if (g.nbnd == 0) {
    PP_CUDA_TRY(cudaMemsetAsync(d_vraw, 0, sizeof(double) * 3 * (size_t)B * mstride, s));
    return cudaSuccess;
  }
  z64 *gtab = (z64 *)(d_part + (size_t)B * nsplit * 3 * mstride);
  VelArgs va;
  for (int k = 0; k < 9; ++k) va.lat[k] = g.lat[k];
  for (int k = 0; k < 3; ++k) {
    for (int c = 0; c < 3; ++c) va.dcrys[k][c] = g.delta_crys[k][c];
    va.dnorm[k] = g.delta_norm[k];
  }
  k_vel_gtab<<<dim3(cdiv(g.nbnd, 128), B), 128, 0, s>>>(g.d_bnd, g.d_bndmask, g.nbnd, g.d_crys, g.d_mass, g.natom,
                                                         va, d_q, method, gtab);
  dim3 grid(cdiv(mmax, 128), nsplit, B);
  if (efmt == 0)
    PP_KT(KT_VEL, s, (k_vel<0><<<grid, 128, 0, s>>>(g.d_bnd, g.nbnd, g.d_fc, g.n, gtab, E, lde, sE, d_rng, nsplit, mstride, d_part, rowmap)));
  else
    PP_KT(KT_VEL, s, (k_vel<1><<<grid, 128, 0, s>>>(g.d_bnd, g.nbnd, g.d_fc, g.n, gtab, E, lde, sE, d_rng, nsplit, mstride, d_part, rowmap)));
  k_vel_reduce<<<dim3(cdiv(mmax, 128), B), 128, 0, s>>>(d_part, nsplit, mstride, d_rng, d_vraw);
  count_launch(3);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// outputs: frequencies in cm^-1 (or lambda), velocities in m/s, z as FP64
template <int EFMT>
__global__ void k_finalize(const double *ww, int64_t sd, const int64_t *rng, const int64_t *info_in, int raw,
                           const double *vraw, int64_t mstride, int want_vel, double *wout, int64_t ldw,
                           double *vout, int64_t velstride, int64_t *m_out, int64_t *nz_out, int64_t *info_out,
                           int jobz_v, const int *tcerr) {
  const int b = blockIdx.y;
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t m = rng[b * 8 + 2];
  if (j == 0) {
    if (m_out) m_out[b] = m;
    if (nz_out) nz_out[b] = jobz_v ? m : 0;
    // a time-out of a tensor-core launch after the eigenvalues (back-transform)
    if (info_out) info_out[b] = info_in[b] | ((tcerr && tcerr[b]) ? PP_INFO_TIMEOUT : 0);
  }
  if (j >= m) return;
  const double lam = ww[b * sd + j];
  // diagonalize.F90:119 then write_output.F90:135
  const double ev = sqrt(fabs(lam)) * (lam >= 0.0 ? 1.0 : -1.0);
  const double wcm = (ev * C1_REF) * C2_REF;
  if (wout) wout[b * ldw + j] = raw ? lam : wcm;
  if (want_vel && vout) {
    for (int k = 0; k < 3; ++k) {
      double x = vraw[((int64_t)b * 3 + k) * mstride + j] / fmax(2.0 * fabs(wcm), 1e-3);
      x = ((((x * C2_REF) * VEL_C2SQ) * 100.0) * 2.0) * PIF_REF;  // write_output.F90:443-446
      vout[b * velstride + 3 * j + k] = x;
    }
  }
}

template <int EFMT>
__global__ void k_copy_z(const void *E, int64_t lde, int64_t sE, const int *nvec, const int64_t *rng, double *zout,
                         int64_t ldz, int64_t zstride) {
  const int b = blockIdx.z;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t j = blockIdx.y;
  const int n = nvec[b];
  if (r >= n || j >= rng[b * 8 + 2]) return;
  const z64 v = ld_e<EFMT>(E, b * sE + r + lde * j);
  double *o = zout + b * zstride + 2 * (r + ldz * j);
  o[0] = v.re;
  o[1] = v.im;
}

cudaError_t finalize_outputs(EigWork &w, int efmt, int raw_lambda, const double *d_vraw, int want_vel, int want_z,
                             double *w_out, int64_t ldw, double *z_out, int64_t ldz, int64_t zstride, double *vel_out,
                             int64_t velstride, int64_t *m_out, int64_t *nz_out, int64_t *info_out, int jobz_v,
                             cudaStream_t s) {
  const int64_t mstride = w.mcap;
  dim3 g(cdiv(w.nmax, 128), w.B);
  if (efmt == 0)
    k_finalize<0><<<g, 128, 0, s>>>(w.w, w.nmax, w.rng, w.info, raw_lambda, d_vraw, mstride, want_vel, w_out, ldw,
                                    vel_out, velstride, m_out, nz_out, info_out, jobz_v, w.tcErr);
  else
    k_finalize<1><<<g, 128, 0, s>>>(w.w, w.nmax, w.rng, w.info, raw_lambda, d_vraw, mstride, want_vel, w_out, ldw,
                                    vel_out, velstride, m_out, nz_out, info_out, jobz_v, w.tcErr);
  count_launch(1);
  if (want_z && z_out) {
    dim3 gz(cdiv(w.nmax, 128), w.mcap, w.B);
    if (efmt == 0)
      k_copy_z<0><<<gz, 128, 0, s>>>(w.E, w.lde, w.sE, w.nvec, w.rng, z_out, ldz, zstride);
    else
      k_copy_z<1><<<gz, 128, 0, s>>>(w.E, w.lde, w.sE, w.nvec, w.rng, z_out, ldz, zstride);
    count_launch(1);
  }
  return cudaGetLastError();
}

}  // namespace pp

namespace pp {
// ---------------------------------------------------------------------------
// Backward pass for the force constants.
//
// For a loss L(w) of the frequencies, dL/dD(r,c) = M(c,r) with
// M = sum_nu c_nu e_nu e_nu^H (Hellmann-Feynman; c_nu = dL/dlambda_nu).  D is
// built from the upper triangle of Phi, D(r,c) = Phi(r,c) p(r,c) with the
// phase/mass factor p of the assembly, so for the symmetric Phi the
// reference uses, dL/dPhi(r,c) = dL/dPhi(c,r) = Re(M(c,r) p(r,c)) (half of the
// pair derivative on each of the two entries).  This kernel adds that, for
// one q, to G: one block per upper 64x64 tile (r <= c tiles), M from the
// eigenvectors Z (FP64, column-major, ldz) and the weights wgt (m) in
// arithmetic R, the phase recomputed from the tie-set table.
constexpr int BW_T = 64, BW_K = 8;
template <class R>
__global__ void __launch_bounds__(256) k_bwd_phi(GeoDev g, const double *q, const z64 *Z, int64_t ldz, int m,
                                                 const double *wgt, double *G) {
  __shared__ cx<R> sR[BW_K][BW_T], sC[BW_K][BW_T];
  if (blockIdx.x > blockIdx.y) return;  // upper tiles only (G is symmetric)
  const int64_t n = g.n, N = g.N;
  const int64_t r0 = (int64_t)blockIdx.x * BW_T, c0 = (int64_t)blockIdx.y * BW_T;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  cx<R> acc[4][4];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int s = 0; s < 4; ++s) acc[p][s] = cz<R>();
  for (int k0 = 0; k0 < m; k0 += BW_K) {
    for (int e = threadIdx.x; e < BW_K * BW_T; e += 256) {
      const int x = e % BW_T, y = e / BW_T;
      const int k = k0 + y;
      const int64_t rr = r0 + x, cc = c0 + x;
      const double wk = k < m ? wgt[k] : 0.0;
      z64 zr = (k < m && rr < n) ? Z[rr + ldz * k] : z64{0.0, 0.0};
      z64 zc = (k < m && cc < n) ? Z[cc + ldz * k] : z64{0.0, 0.0};
      sR[y][x] = cfrom64<R>(zr.re * wk, zr.im * wk);
      sC[y][x] = cfrom64<R>(zc.re, -zc.im);
    }
    __syncthreads();
#pragma unroll 2
    for (int k = 0; k < BW_K; ++k) {
      cx<R> a[4], bq[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        a[p] = sR[k][tx + 16 * p];
        bq[p] = sC[k][ty + 16 * p];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int s = 0; s < 4; ++s) cmac(acc[p][s], a[p], bq[s]);
    }
    __syncthreads();
  }
  // acc[p][s] = M(r, c) for r = r0+tx+16p, c = c0+ty+16s ; need Re(M(c,r) p(r,c)) = Re(conj(M(r,c)) p(r,c))
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int64_t r = r0 + tx + 16 * p, c = c0 + ty + 16 * s;
      if (r >= n || c >= n || r > c) continue;
      const int64_t I = r / 3, J = c / 3;
      const int64_t lo = I < J ? I : J, hi = I < J ? J : I;
      const uint32_t mask = g.mask[I + N * J];
      double pr = 0.0, pi = 0.0;
      int mult = 0;
      for (int l = 0; l < 9; ++l) {
        if (!((mask >> l) & 1u)) continue;
        const int i = l / 3 - 1;
        const int j = l - 1 - 3 * (i + 1);
        const double pp = prephase(q, g.crys, N, lo, hi, i, j);
        double sn, cs;
        sincos(-(__dmul_rn(2.0 * PI_REF, pp)), &sn, &cs);
        pr += cs;
        pi += sn;
        ++mult;
      }
      const double inv = 1.0 / ((double)mult * sqrt(g.mass[lo] * g.mass[hi]));
      pr *= inv;
      pi *= inv;  // r <= c: upper orientation, no conjugation
      const z64 Mrc = cto64(cfin(acc[p][s]));
      const double val = Mrc.re * pr + Mrc.im * pi;  // Re(conj(M) p)
      G[r + n * c] += val;
      if (r != c) G[c + n * r] += val;
    }
}

cudaError_t backward_phi(const Geometry &g, const double *d_q, const z64 *Z, int64_t ldz, int m, const double *wgt,
                         double *G, int prec, cudaStream_t s) {
  GeoDev gd{g.d_fc, g.d_crys, g.d_mass, g.d_mask, g.natom, g.n};
  const int nt = cdiv(g.n, BW_T);
  if (prec == 1)
    k_bwd_phi<df><<<dim3(nt, nt), 256, 0, s>>>(gd, d_q, Z, ldz, m, wgt, G);
  else
    k_bwd_phi<double><<<dim3(nt, nt), 256, 0, s>>>(gd, d_q, Z, ldz, m, wgt, G);
  count_launch(1);
  return cudaGetLastError();
}
}  // namespace pp
