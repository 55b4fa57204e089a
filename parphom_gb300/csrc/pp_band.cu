// Two-stage Hermitian reduction of the mixed form (double-float storage).
//
// Stage 1, dense -> band (32 sub-diagonals), panel by panel of 32 columns:
//   P = A(k1:n, k0:k1) = Q R          Householder QR of the panel
//                                     (k_panel_qr), Q = I - V T V^H
//   U = V T                           (k_band_vt)
//   X = A22 U                         A22 = A(k1:n, k1:n), tensor cores over
//                                     the full square (k_mirror_lower first)
//   Y = V^H X,  M = T^H Y             (k_band_yp, k_band_m)
//   W = X - 1/2 V M                   (k_band_w)
//   A22 -= V W^H + W V^H              tensor cores, lower triangle
// which is A22 <- Q^H A22 Q (zhetrd's blocked update with the panel QR in
// place of the zlatrd recurrence).  R becomes the band's sub-diagonal
// block; the panel's reflectors stay in A below R (unit element implicit at
// row k1 + a, made explicit once the band is copied out), so the first
// stage's back-transform runs the one-stage kernels with a row offset.
// The BLAS-2 mat-vec of the one-stage reduction (one full pass over the
// trailing matrix per column) becomes one 32-column product per panel.
//
// Stage 2, band -> real symmetric tridiagonal by bulge chasing (k_bulge):
// sweep j annihilates column j below its first sub-diagonal with a
// reflector on rows j+1 .. j+32 and chases the resulting bulge down the
// band in steps of 32 rows, one reflector per step; each step touches a
// 32 x 32 off-diagonal block and a 32 x 32 diagonal block.  One CTA per
// matrix, one sweep per warp; sweep j+1 may run step k once sweep j has
// finished step k+1 (their blocks are then disjoint), tracked by progress
// counters in shared memory with bounded waits.  The reflectors are kept in
// sweep order and applied afterwards to the boundary-row matrix (Q2^H X) or
// to the tridiagonal eigenvectors (Q2 Z) by k_q2, in diamond groups of 32
// sweeps that reuse a 63-row window of X in shared memory.
#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <mutex>

#include "pp_internal.cuh"

namespace pp {

namespace {

constexpr int BW = 32;     // bandwidth
constexpr int LDAB = 64;   // band storage: A(c + d, c) at AB[d + 64 c], d < 64 (band and bulge)
using Z = zdf;

static inline int cdiv_h(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// ---------------------------------------------------------------------------
// helpers
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ Z shfl_z(Z v, int src) {
  Z r;
  r.re.hi = __shfl_sync(0xffffffffu, v.re.hi, src);
  r.re.lo = __shfl_sync(0xffffffffu, v.re.lo, src);
  r.im.hi = __shfl_sync(0xffffffffu, v.im.hi, src);
  r.im.lo = __shfl_sync(0xffffffffu, v.im.lo, src);
  return r;
}
__device__ __forceinline__ double abs2(Z v) {
  const z64 t = cto64(v);
  return t.re * t.re + t.im * t.im;
}
// zlarfg in FP64 (the scalars of k_reflector): alpha and ||x||^2 of the rest
// give beta (real), tau and the scale 1 / (alpha - beta) of x.
struct Refl {
  z64 tau, scale;
  double beta;
};
__device__ __forceinline__ Refl make_refl(z64 alpha, double xn2) {
  Refl h;
  const double xnorm = sqrt(xn2);
  if (xnorm == 0.0 && alpha.im == 0.0) {
    h.tau = z64{0.0, 0.0};
    h.beta = alpha.re;
    h.scale = z64{1.0, 0.0};
  } else {
    const double nrm3 = sqrt(alpha.re * alpha.re + alpha.im * alpha.im + xn2);
    const double beta = -copysign(nrm3, alpha.re);
    h.tau = z64{(beta - alpha.re) / beta, -alpha.im / beta};
    const double dr = alpha.re - beta, di = alpha.im;
    const double den = dr * dr + di * di;
    h.scale = z64{dr / den, -di / den};
    h.beta = beta;
  }
  return h;
}

// ---------------------------------------------------------------------------
// Stage 1: panel QR.  One CTA per matrix; the panel stays in global memory
// (it is L2-resident); per column one pass for the norm and one for the
// dot products with the later columns and the Gram column of T.
constexpr int PQ_NT = 256;
constexpr int PQ_NV = 31;  // dot products per column step (later columns + Gram column)

__global__ void __launch_bounds__(PQ_NT) k_panel_qr(Z *Ab, int64_t lda, int64_t sA, const int *nvec, int k0, Z *Vb,
                                                    int64_t sV, z64 *tau, int64_t sd, z64 *Tf) {
  __shared__ double redd[PQ_NT / 32];
  __shared__ z64 red[PQ_NT / 32][PQ_NV];
  __shared__ z64 tot[PQ_NV];
  __shared__ z64 sT[BW][BW];
  __shared__ Refl s_h;
  const int b = blockIdx.x;
  const int n = nvec[b];
  Z *A = Ab + b * sA;
  Z *V = Vb + b * sV;
  const int k1 = k0 + BW;
  const int m = n - k1;
  const int nref = m >= 2 ? min(BW, m - 1) : 0;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int e = tid; e < BW * BW; e += PQ_NT) sT[e / BW][e % BW] = z64{0.0, 0.0};
  for (int a = 0; a < BW; ++a)
    for (int i = tid; i < max(m, 0); i += PQ_NT) V[k1 + i + lda * a] = cz<df>();
  if (tid < BW) tau[b * sd + k0 + tid] = z64{0.0, 0.0};
  __syncthreads();
  for (int j = 0; j < nref; ++j) {
    const int c = k0 + j;
    // (1) norm of the part below the diagonal
    double p = 0.0;
    for (int i = j + 1 + tid; i < m; i += PQ_NT) p += abs2(A[k1 + i + lda * c]);
    p = warp_sum_d(p);
    if (lane == 0) redd[wid] = p;
    __syncthreads();
    if (tid == 0) {
      double xn2 = 0.0;
      for (int k = 0; k < PQ_NT / 32; ++k) xn2 += redd[k];
      const Refl h = make_refl(cto64(A[k1 + j + lda * c]), xn2);
      s_h = h;
      tau[b * sd + c] = h.tau;
    }
    __syncthreads();
    const Refl h = s_h;
    // (2) v = [1, x / (alpha - beta)]: in place below the diagonal, R's
    // diagonal = beta, and explicitly in V
    const Z scz = cfrom64<df>(h.scale);
    for (int i = j + tid; i < m; i += PQ_NT) {
      Z v;
      if (i == j) {
        A[k1 + j + lda * c] = cfrom64<df>(h.beta, 0.0);
        v = cfrom64<df>(1.0, 0.0);
      } else {
        v = cmul(A[k1 + i + lda * c], scz);
        A[k1 + i + lda * c] = v;
      }
      V[k1 + i + lda * j] = v;
    }
    __syncthreads();
    // (3) dot products: s_cc = v^H P(:, cc) for the later columns cc > j, and
    // g_a = V(:, a)^H v for a < j (Gram column of T)
    Z acc[PQ_NV];
#pragma unroll
    for (int q = 0; q < PQ_NV; ++q) acc[q] = cz<df>();
    for (int i = j + tid; i < m; i += PQ_NT) {
      const Z v = V[k1 + i + lda * j];
#pragma unroll
      for (int q = 0; q < PQ_NV; ++q) {
        // q < 31 - j: column j + 1 + q of the panel; else a = q - (31 - j)
        const int cc = j + 1 + q;
        if (cc < BW) {
          cmacc(acc[q], v, A[k1 + i + lda * (k0 + cc)]);
        } else {
          const int a = cc - BW;  // 0 .. j-1
          if (a < j) cmacc(acc[q], V[k1 + i + lda * a], v);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < PQ_NV; ++q) {
      z64 t = cto64(cfin(acc[q]));
      t.re = warp_sum_d(t.re);
      t.im = warp_sum_d(t.im);
      if (lane == 0) red[wid][q] = t;
    }
    __syncthreads();
    if (tid < PQ_NV) {
      z64 t{0.0, 0.0};
      for (int k = 0; k < PQ_NT / 32; ++k) {
        t.re += red[k][tid].re;
        t.im += red[k][tid].im;
      }
      tot[tid] = t;
    }
    __syncthreads();
    // (4) P(:, cc) -= conj(tau) v s_cc for cc > j (H^H applied from the left)
    const z64 ct = zconj(h.tau);
    for (int i = j + tid; i < m; i += PQ_NT) {
      const Z v = V[k1 + i + lda * j];
      for (int cc = j + 1; cc < BW; ++cc) {
        const Z f = cfrom64<df>(zmul(ct, tot[cc - j - 1]));
        Z *x = &A[k1 + i + lda * (k0 + cc)];
        *x = csub(*x, cmul(v, f));
      }
    }
    // (5) T column j (zlarft, forward columnwise): T(a, j) = -tau_j sum_{a2 >= a} T(a, a2) g_a2
    if (tid < j) {
      z64 s{0.0, 0.0};
      for (int a2 = tid; a2 < j; ++a2) {
        const z64 g = tot[(BW - 1 - j) + a2];
        const z64 t = zmul(sT[tid][a2], g);
        s.re += t.re;
        s.im += t.im;
      }
      const z64 v = zmul(h.tau, s);
      sT[tid][j] = z64{-v.re, -v.im};
    }
    if (tid == 0) sT[j][j] = h.tau;
    __syncthreads();
  }
  for (int e = tid; e < BW * BW; e += PQ_NT) Tf[b * BW * BW + e] = sT[e / BW][e % BW];
}

// U = V T (rows >= k1), T upper triangular.
__global__ void __launch_bounds__(128) k_band_vt(const Z *Vb, Z *Ub, int64_t lda, int64_t sV, const int *nvec, int k1,
                                                 const z64 *Tf) {
  __shared__ Z sT[BW][BW];
  const int b = blockIdx.y;
  for (int e = threadIdx.x; e < BW * BW; e += 128) sT[e / BW][e % BW] = cfrom64<df>(Tf[b * BW * BW + e]);
  __syncthreads();
  const int n = nvec[b];
  const int r = k1 + blockIdx.x * 128 + threadIdx.x;
  if (r >= n) return;
  const Z *V = Vb + b * sV;
  Z *U = Ub + b * sV;
  for (int a = 0; a < BW; ++a) {
    Z acc = cz<df>();
    for (int a2 = 0; a2 <= a; ++a2) cmac(acc, V[r + lda * a2], sT[a2][a]);
    U[r + lda * a] = cfin(acc);
  }
}

// Upper triangle of A(k1:n, k1:n) := conjugate transpose of its lower
// triangle, by 32 x 32 tiles through shared memory.
__global__ void __launch_bounds__(256) k_mirror_lower(Z *Ab, int64_t lda, int64_t sA, const int *nvec, int k1) {
  __shared__ Z t[32][33];
  const int b = blockIdx.z;
  const int n = nvec[b];
  const int R = blockIdx.x, Cc = blockIdx.y;
  if (R < Cc) return;
  const int r0 = k1 + 32 * R, c0 = k1 + 32 * Cc;
  if (r0 >= n) return;
  Z *A = Ab + b * sA;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int cc = ty; cc < 32; cc += 8) {
    const int r = r0 + tx, c = c0 + cc;
    if (r < n && c < n && (R != Cc || tx > cc)) t[cc][tx] = A[r + lda * c];
  }
  __syncthreads();
  // element (r, c) of the lower tile -> A(c, r) = conj(A(r, c))
  for (int rr = ty; rr < 32; rr += 8) {
    const int c = c0 + tx, r = r0 + rr;
    if (r < n && c < n && (R != Cc || rr > tx)) A[c + lda * r] = cconj(t[tx][rr]);
  }
}

// Partial Y = V^H X over chunks of 256 rows (>= k1): Yp[b][ch][a][j].
__global__ void __launch_bounds__(256) k_band_yp(const Z *Vb, const Z *Xb, int64_t lda, int64_t sV, const int *nvec,
                                                 int k1, z64 *Yp, int nyp) {
  __shared__ Z sV_[32][BW + 1], sX[32][BW + 1];
  const int b = blockIdx.y, ch = blockIdx.x;
  const int n = nvec[b];
  const Z *V = Vb + b * sV;
  const Z *X = Xb + b * sV;
  const int a = threadIdx.x >> 3, j0 = (threadIdx.x & 7) * 4;
  Z acc[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) acc[q] = cz<df>();
  const int rb = k1 + ch * 256;
  for (int s0 = rb; s0 < min(n, rb + 256); s0 += 32) {
    for (int e = threadIdx.x; e < 32 * BW; e += 256) {
      const int rr = e & 31, cc = e >> 5, r = s0 + rr;
      sV_[rr][cc] = r < n ? V[r + lda * cc] : cz<df>();
      sX[rr][cc] = r < n ? X[r + lda * cc] : cz<df>();
    }
    __syncthreads();
    for (int rr = 0; rr < 32; ++rr) {
      const Z v = sV_[rr][a];
#pragma unroll
      for (int q = 0; q < 4; ++q) cmacc(acc[q], v, sX[rr][j0 + q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) Yp[((int64_t)b * nyp + ch) * BW * BW + a * BW + j0 + q] = cto64(cfin(acc[q]));
}

// M = T^H Y, Y = sum of the partials (FP64).
__global__ void __launch_bounds__(1024) k_band_m(const z64 *Yp, int nyp, int nch, const z64 *Tf, z64 *Mb) {
  __shared__ z64 sY[BW][BW];
  const int b = blockIdx.x;
  const int a = threadIdx.x >> 5, j = threadIdx.x & 31;
  z64 y{0.0, 0.0};
  for (int ch = 0; ch < nch; ++ch) {
    const z64 t = Yp[((int64_t)b * nyp + ch) * BW * BW + a * BW + j];
    y.re += t.re;
    y.im += t.im;
  }
  sY[a][j] = y;
  __syncthreads();
  z64 s{0.0, 0.0};
  for (int a2 = 0; a2 <= a; ++a2) {  // (T^H)(a, a2) = conj(T(a2, a)), nonzero for a2 <= a
    const z64 t = zmul(zconj(Tf[b * BW * BW + a2 * BW + a]), sY[a2][j]);
    s.re += t.re;
    s.im += t.im;
  }
  Mb[b * BW * BW + a * BW + j] = s;
}

// W = X - 1/2 V M (rows >= k1), in place in X.
__global__ void __launch_bounds__(128) k_band_w(const Z *Vb, Z *Xb, int64_t lda, int64_t sV, const int *nvec, int k1,
                                                const z64 *Mb) {
  __shared__ Z sM[BW][BW];
  const int b = blockIdx.y;
  for (int e = threadIdx.x; e < BW * BW; e += 128) {
    const z64 mv = Mb[b * BW * BW + e];
    sM[e / BW][e % BW] = cfrom64<df>(-0.5 * mv.re, -0.5 * mv.im);
  }
  __syncthreads();
  const int n = nvec[b];
  const int r = k1 + blockIdx.x * 128 + threadIdx.x;
  if (r >= n) return;
  const Z *V = Vb + b * sV;
  Z *X = Xb + b * sV;
  Z v[BW];
#pragma unroll
  for (int a = 0; a < BW; ++a) v[a] = V[r + lda * a];
  for (int j = 0; j < BW; ++j) {
    Z acc = X[r + lda * j];
#pragma unroll
    for (int a = 0; a < BW; ++a) cmac(acc, v[a], sM[a][j]);
    X[r + lda * j] = cfin(acc);
  }
}

// The band (diagonals 0..32) into AB, zero diagonals 33..63; the diagonal
// made real.  A(r, c) for r - c <= 32: the diagonal block's lower triangle,
// R (upper triangle of the sub-diagonal block below a reduced panel; V is
// stored below it), or the dense trailing block left after the last panel.
__global__ void k_band_extract(const Z *Ab, int64_t lda, int64_t sA, const int *nvec, Z *ABb, int64_t sAB) {
  const int b = blockIdx.y;
  const int n = nvec[b];
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int c = (int)(e / LDAB), d = (int)(e % LDAB);
  if (c >= n) return;
  const int r = c + d;
  Z v = cz<df>();
  if (d <= BW && r < n) {
    const int bc = c / BW, br = r / BW;
    bool keep = true;
    if (br != bc && BW * bc + BW < n - 1) keep = (r - BW * br) <= (c - BW * bc);
    if (keep) v = Ab[b * sA + r + lda * c];
    if (d == 0) v.im = df{0.f, 0.f};
  }
  ABb[b * sAB + d + (int64_t)LDAB * c] = v;
}

// Explicit unit elements of the panel reflectors (band layout): A(k0 + 32 +
// a, k0 + a) = 1 for the a < min(32, n - k0 - 33) reflectors of each panel.
__global__ void k_band_units(Z *Ab, int64_t lda, int64_t sA, const int *nvec) {
  const int b = blockIdx.y;
  const int n = nvec[b];
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  const int k0 = c / BW * BW, a = c - k0;
  if (c >= n) return;
  const int nref = max(0, min(BW, n - k0 - BW - 1));
  if (a < nref) Ab[b * sA + (k0 + BW + a) + lda * c] = cfrom64<df>(1.0, 0.0);
}

// ---------------------------------------------------------------------------
// Stage 2: bulge chasing.
//
// Reflector (j, k) of sweep j acts on rows r0 = j + 1 + 32 k .. r0 + L - 1,
// L = min(32, n - r0), for k < nsteps(j) = (n - 2 - j) / 32 + 1; they are
// stored in sweep order at index ofs(j) + k.
__host__ __device__ __forceinline__ int64_t q2_G(int64_t T) {  // sum_{t <= T} floor(t / 32)
  if (T < 0) return 0;
  const int64_t q = T / BW, rem = T % BW;
  return BW * (q * (q - 1) / 2) + q * (rem + 1);
}
__host__ __device__ __forceinline__ int64_t q2_F(int64_t T) { return T < 0 ? 0 : (T + 1) + q2_G(T); }
__host__ __device__ __forceinline__ int q2_nsteps(int n, int j) { return (n - 2 - j) / BW + 1; }
__host__ __device__ __forceinline__ int64_t q2_ofs(int n, int j) { return q2_F(n - 2) - q2_F(n - 2 - j); }

constexpr int BG_NW = 16;  // warps (concurrent sweeps) per matrix

// Band element A(r, c), r >= c, r - c < 64.
__device__ __forceinline__ Z *bel(Z *AB, int r, int c) { return AB + (r - c) + (int64_t)LDAB * c; }

// Two-sided update of the diagonal block D = A(p .. p+L-1, p .. p+L-1) by
// H = I - tau v v^H (D <- H^H D H); lane i holds v_i (zero for i >= L).
__device__ void hetwo(Z *AB, int p, int L, Z v, z64 tau, int lane) {
  const Z tz = cfrom64<df>(tau);
  Z w = cz<df>();
  {
    Z acc = cz<df>();
    for (int c = 0; c < L; ++c) {
      const Z vc = shfl_z(v, c);  // every lane takes part in the shuffle
      if (lane < L) {
        const Z d = (c <= lane) ? *bel(AB, p + lane, p + c) : cconj(*bel(AB, p + c, p + lane));
        cmac(acc, d, vc);
      }
    }
    if (lane < L) w = cmul(tz, cfin(acc));
  }
  // alpha = -1/2 tau (w^H v)
  const z64 wv = cto64(cmul(cconj(w), v));
  const double sr = warp_sum_d(lane < L ? wv.re : 0.0), si = warp_sum_d(lane < L ? wv.im : 0.0);
  const z64 al = zmul(tau, z64{sr, si});
  const Z alpha = cfrom64<df>(-0.5 * al.re, -0.5 * al.im);
  Z acc2 = w;
  cmac(acc2, alpha, v);
  w = cfin(acc2);
  __syncwarp();
  for (int c = 0; c < L; ++c) {
    const Z vc = shfl_z(v, c), wc = shfl_z(w, c);
    if (lane < L && c <= lane) {
      Z *x = bel(AB, p + lane, p + c);
      Z acc = cz<df>();
      cmac(acc, v, cconj(wc));
      cmac(acc, w, cconj(vc));
      Z nv = csub(*x, cfin(acc));
      if (c == lane) nv.im = df{0.f, 0.f};
      *x = nv;
    }
  }
  __syncwarp();
}

// Reflector from x (lane i < L holds x_i, zero above): returns v (v_0 = 1) and
// tau, x's first element replaced by beta.
__device__ __forceinline__ Z warp_refl(Z x, int L, int lane, z64 *tau_out, double *beta_out) {
  const double xn2 = warp_sum_d((lane >= 1 && lane < L) ? abs2(x) : 0.0);
  const Z a0 = shfl_z(x, 0);
  const Refl h = make_refl(cto64(a0), xn2);
  *tau_out = h.tau;
  *beta_out = h.beta;
  if (lane == 0) return cfrom64<df>(1.0, 0.0);
  if (lane >= L) return cz<df>();
  return cmul(x, cfrom64<df>(h.scale));
}

__global__ void __launch_bounds__(BG_NW * 32) k_bulge(Z *ABb, int64_t sAB, const int *nvec, Z *q2vb, z64 *q2tb,
                                                      int64_t sq, double *dd, double *ee, int64_t sd, int *errf,
                                                      long long wait_cycles) {
  __shared__ volatile long long prog[BG_NW];  // (sweep << 32) | steps done, of each warp's current sweep
  __shared__ volatile int abort_f;
  const int b = blockIdx.x;
  const int n = nvec[b];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Z *AB = ABb + b * sAB;
  Z *q2v = q2vb + b * sq * BW;
  z64 *q2t = q2tb + b * sq;
  if (lane == 0) prog[warp] = -1LL;
  if (threadIdx.x == 0) abort_f = 0;
  __syncthreads();
  const int slot = (warp + BG_NW - 1) % BG_NW;  // warp of sweep j - 1
  for (int j = warp; j <= n - 2 && !abort_f; j += BG_NW) {
    const int K = q2_nsteps(n, j);
    const int64_t ofs = q2_ofs(n, j);
    const int Kp = j > 0 ? q2_nsteps(n, j - 1) : 0;
    Z vprev = cz<df>();
    z64 tprev{0.0, 0.0};
    for (int k = 0; k < K; ++k) {
      // sweep j - 1 must have finished step k + 1 (all of it if shorter)
      if (j > 0) {
        const int need = min(k + 2, Kp);
        if (lane == 0) {
          const long long t0 = clock64();
          while (true) {
            const long long v = prog[slot];
            const long long sw = v >> 32;
            const int st = (int)(v & 0xffffffffLL);
            if (sw > j - 1 || (sw == j - 1 && st >= need)) break;
            if (abort_f) break;
            if (clock64() - t0 > wait_cycles) {
              abort_f = 1;
              atomicExch(&errf[b], 1);
              break;
            }
            __nanosleep(32);
          }
        }
        __syncwarp();
        __threadfence_block();
        if (abort_f) break;
      }
      const int r0 = j + 1 + BW * k;
      const int L = min(BW, n - r0);
      z64 tau;
      double beta;
      Z v;
      if (k == 0) {
        // column j below its diagonal
        const Z x = lane < L ? *bel(AB, r0 + lane, j) : cz<df>();
        v = warp_refl(x, L, lane, &tau, &beta);
        if (lane == 0) *bel(AB, r0, j) = cfrom64<df>(beta, 0.0);
        else if (lane < L) *bel(AB, r0 + lane, j) = cz<df>();
      } else {
        // off-diagonal block O = A(r0 .. r0+L-1, p .. p+31), p = r0 - 32
        const int p = r0 - BW;
        // (1) O <- O H_prev: lane i owns row i
        {
          Z acc = cz<df>();
          for (int c = 0; c < BW; ++c) {
            const Z vc = shfl_z(vprev, c);
            if (lane < L) cmac(acc, *bel(AB, r0 + lane, p + c), vc);
          }
          const Z y = cmul(cfrom64<df>(tprev), cfin(acc));
          for (int c = 0; c < BW; ++c) {
            const Z vc = shfl_z(vprev, c);
            if (lane < L) {
              Z *x = bel(AB, r0 + lane, p + c);
              *x = csub(*x, cmul(y, cconj(vc)));
            }
          }
        }
        __syncwarp();
        // (2) reflector from O's first column
        const Z x = lane < L ? *bel(AB, r0 + lane, p) : cz<df>();
        v = warp_refl(x, L, lane, &tau, &beta);
        if (lane == 0) *bel(AB, r0, p) = cfrom64<df>(beta, 0.0);
        else if (lane < L) *bel(AB, r0 + lane, p) = cz<df>();
        __syncwarp();
        // (3) H^H from the left on O's other columns: lane c owns column c
        const Z ct = cfrom64<df>(zconj(tau));
        Z s = cz<df>();
        for (int i = 0; i < L; ++i) {
          const Z vi = shfl_z(v, i);
          if (lane >= 1) cmacc(s, vi, *bel(AB, r0 + i, p + lane));
        }
        const Z f = cmul(ct, cfin(s));
        for (int i = 0; i < L; ++i) {
          const Z vi = shfl_z(v, i);
          if (lane >= 1) {
            Z *xx = bel(AB, r0 + i, p + lane);
            *xx = csub(*xx, cmul(vi, f));
          }
        }
        __syncwarp();
      }
      // store the reflector, then the two-sided update of the diagonal block
      q2v[(ofs + k) * BW + lane] = v;
      if (lane == 0) q2t[ofs + k] = tau;
      hetwo(AB, r0, L, v, tau, lane);
      vprev = v;
      tprev = tau;
      // release: every lane's writes of this step before the progress count
      __threadfence_block();
      __syncwarp();
      if (lane == 0) prog[warp] = ((long long)j << 32) | (long long)(k + 1);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    dd[b * sd + i] = df_to(AB[(int64_t)LDAB * i].re);
    ee[b * sd + i] = (i < n - 1) ? df_to(AB[1 + (int64_t)LDAB * i].re) : 0.0;
  }
}

// ---------------------------------------------------------------------------
// Q2 application.  CTA = 4 warps = 128 columns of X (thread = column); the
// reflectors of one diamond (sweeps gb .. gb+31, step k) act on the window
// of rows gb + 1 + 32 k .. + 62, held in shared memory.  Forward (X <- Q2^H
// X): groups ascending, steps descending, sweeps ascending inside a diamond;
// reverse (X <- Q2 X): the opposite order with H instead of H^H.
constexpr int Q2_NW = 4;
constexpr int Q2_COLS = 32 * Q2_NW;
constexpr int Q2_WR = 64;  // window rows (63 used)
constexpr size_t Q2_SMEM = (size_t)Q2_WR * Q2_COLS * sizeof(Z) + (size_t)BW * BW * sizeof(Z) + BW * sizeof(z64);

__global__ void __launch_bounds__(Q2_NW * 32) k_q2(Z *Xb, int64_t ldx, int64_t sX, int ncols, const int *nvec,
                                                   const Z *q2vb, const z64 *q2tb, int64_t sq, int reverse) {
  extern __shared__ __align__(16) unsigned char q2smem[];
  Z *win = (Z *)q2smem;                       // win[row * Q2_COLS + col]
  Z *sv = win + Q2_WR * Q2_COLS;              // sv[t * 32 + i]
  z64 *st = (z64 *)(sv + BW * BW);
  const int b = blockIdx.y;
  const int n = nvec[b];
  const int c0 = blockIdx.x * Q2_COLS;
  const int col = threadIdx.x;  // column within the CTA
  const bool colok = c0 + col < ncols;
  Z *X = Xb + b * sX + (int64_t)ldx * (c0 + col);
  const Z *q2v = q2vb + b * sq * BW;
  const z64 *q2t = q2tb + b * sq;
  const int nsw = n - 1;                       // sweeps 0 .. n-2
  const int ng = (nsw + BW - 1) / BW;
  auto load_rows = [&](int base, int w0, int w1) {  // window rows [w0, w1) <- X rows base + w
    for (int w = w0; w < w1; ++w) {
      const int r = base + w;
      win[w * Q2_COLS + col] = (colok && r < n) ? X[r] : cz<df>();
    }
  };
  auto store_rows = [&](int base, int w0, int w1) {
    for (int w = w0; w < w1; ++w) {
      const int r = base + w;
      if (colok && r < n) X[r] = win[w * Q2_COLS + col];
    }
  };
  for (int gi = 0; gi < ng; ++gi) {
    const int g = reverse ? ng - 1 - gi : gi;
    const int gb = g * BW;
    const int kmax = q2_nsteps(n, gb);  // the group's first sweep has the most steps
    for (int ki = 0; ki < kmax; ++ki) {
      const int k = reverse ? ki : kmax - 1 - ki;
      const int base = gb + 1 + BW * k;
      // window: rows base .. base + 62; the overlap with the previous
      // diamond of the group (31 rows) is moved, the rest loaded/stored
      if (ki == 0) {
        load_rows(base, 0, Q2_WR - 1);
      } else if (!reverse) {
        // moving up: the previous window started at base + 32; its rows
        // 31 .. 62 are final for this group
        store_rows(base + BW, BW - 1, Q2_WR - 1);
        for (int w = Q2_WR - 2; w >= BW; --w) win[w * Q2_COLS + col] = win[(w - BW) * Q2_COLS + col];
        load_rows(base, 0, BW);
      } else {
        // moving down: the previous window started at base - 32; its rows
        // 0 .. 31 are final
        store_rows(base - BW, 0, BW);
        for (int w = 0; w < Q2_WR - 1 - BW; ++w) win[w * Q2_COLS + col] = win[(w + BW) * Q2_COLS + col];
        load_rows(base, Q2_WR - 1 - BW, Q2_WR - 1);
      }
      // the diamond's reflectors into shared memory
      __syncthreads();
      for (int e = threadIdx.x; e < BW * BW; e += Q2_NW * 32) {
        const int t = e / BW, i = e % BW;
        const int j = gb + t;
        const bool ok = j <= n - 2 && k < q2_nsteps(n, j);
        sv[e] = ok ? q2v[(q2_ofs(n, j) + k) * BW + i] : cz<df>();
        if (i == 0) st[t] = ok ? q2t[q2_ofs(n, j) + k] : z64{0.0, 0.0};
      }
      __syncthreads();
      for (int ti = 0; ti < BW; ++ti) {
        const int t = reverse ? BW - 1 - ti : ti;
        const z64 tz = reverse ? st[t] : zconj(st[t]);
        if (tz.re == 0.0 && tz.im == 0.0) continue;
        const Z *v = sv + t * BW;
        Z s0 = cz<df>(), s1 = cz<df>();
#pragma unroll 8
        for (int i = 0; i < BW; i += 2) {
          cmacc(s0, v[i], win[(t + i) * Q2_COLS + col]);
          cmacc(s1, v[i + 1], win[(t + i + 1) * Q2_COLS + col]);
        }
        const Z f = cmul(cfrom64<df>(tz), cadd(cfin(s0), cfin(s1)));
#pragma unroll 8
        for (int i = 0; i < BW; ++i) {
          Z *x = &win[(t + i) * Q2_COLS + col];
          *x = csub(*x, cmul(v[i], f));
        }
      }
      __syncthreads();
      if (ki == kmax - 1) store_rows(base, 0, Q2_WR - 1);
    }
  }
}

}  // namespace

int64_t q2_count(int64_t n) { return n >= 2 ? q2_F(n - 2) : 0; }

cudaError_t band_reduce(EigWork &w, cudaStream_t s) {
  const int B = w.B, nmax = w.nmax;
  const int64_t lda = w.lda, sP = w.lda * BW;
  Z *A = (Z *)w.A;
  if (w.tcErr) PP_CUDA_TRY(cudaMemsetAsync(w.tcErr, 0, sizeof(int) * B, s));
  for (int k0 = 0; k0 + BW < nmax - 1; k0 += BW) {
    const int k1 = k0 + BW;
    const int m = nmax - k1;
    PP_KT(KT_BANDQR, s, (k_panel_qr<<<B, PQ_NT, 0, s>>>(A, lda, w.sA, w.nvec, k0, (Z *)w.Vb, sP, w.tau, w.nmax,
                                                         w.Tf)));
    PP_KT(KT_BANDMV, s, (k_band_vt<<<dim3(cdiv_h(m, 128), B), 128, 0, s>>>((const Z *)w.Vb, (Z *)w.Ub, lda, sP,
                                                                            w.nvec, k1, w.Tf)));
    const int nt = cdiv_h(m, 32);
    PP_KT(KT_BANDMV, s, (k_mirror_lower<<<dim3(nt, nt, B), 256, 0, s>>>(A, lda, w.sA, w.nvec, k1)));
    count_launch(3);
    PP_CUDA_TRY(band_hemm_tc(w, k1, s));
    const int nch = cdiv_h(m, 256);
    PP_KT(KT_BANDMV, s, (k_band_yp<<<dim3(nch, B), 256, 0, s>>>((const Z *)w.Vb, (const Z *)w.Xb, lda, sP, w.nvec,
                                                                 k1, w.Yp, w.nyp)));
    PP_KT(KT_BANDMV, s, (k_band_m<<<B, 1024, 0, s>>>(w.Yp, w.nyp, nch, w.Tf, w.Mb)));
    PP_KT(KT_BANDMV, s, (k_band_w<<<dim3(cdiv_h(m, 128), B), 128, 0, s>>>((const Z *)w.Vb, (Z *)w.Xb, lda, sP,
                                                                           w.nvec, k1, w.Mb)));
    count_launch(3);
    PP_CUDA_TRY(band_her2k_tc(w, k1, s));
  }
  const int64_t sAB = (int64_t)LDAB * nmax;
  k_band_extract<<<dim3(cdiv_h((int64_t)LDAB * nmax, 256), B), 256, 0, s>>>(A, lda, w.sA, w.nvec, (Z *)w.AB, sAB);
  k_band_units<<<dim3(cdiv_h(nmax, 256), B), 256, 0, s>>>(A, lda, w.sA, w.nvec);
  count_launch(2);
  w.voff = BW;
  w.band = 1;
  return cudaGetLastError();
}

cudaError_t band_to_tridiag(EigWork &w, cudaStream_t s) {
  const int64_t sAB = (int64_t)LDAB * w.nmax;
  // each wait for the preceding sweep gives up after ~0.2 s of SM clocks
  PP_KT(KT_BULGE, s, (k_bulge<<<w.B, BG_NW * 32, 0, s>>>((Z *)w.AB, sAB, w.nvec, (Z *)w.q2v, w.q2t, w.nq2, w.d, w.e,
                                                          w.nmax, w.tcErr, 400000000LL)));
  count_launch(1);
  return cudaGetLastError();
}

cudaError_t apply_q2(EigWork &w, void *X, int64_t ldx, int64_t sX, int ncols, int reverse, cudaStream_t s) {
  if (ncols <= 0 || w.nmax < 2) return cudaSuccess;
  dim3 g(cdiv_h(ncols, Q2_COLS), w.B);
  PP_KT(KT_Q2, s, (k_q2<<<g, Q2_NW * 32, Q2_SMEM, s>>>((Z *)X, ldx, sX, ncols, w.nvec, (const Z *)w.q2v, w.q2t,
                                                        w.nq2, reverse)));
  count_launch(1);
  return cudaGetLastError();
}

// The Q2 kernel's shared memory, opted into once per device.
cudaError_t prepare_band() {
  static std::mutex mu;
  static bool done[PP_MAX_DEVICES] = {};
  const int dev = device_index();
  std::lock_guard<std::mutex> g(mu);
  if (dev >= 0 && done[dev]) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(k_q2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Q2_SMEM);
  if (e == cudaSuccess && dev >= 0) done[dev] = true;
  return e;
}

}  // namespace pp
