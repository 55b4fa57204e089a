// Batched Hermitian eigensolver with pzheevx semantics (range A/I/V, abstol,
// optional eigenvectors) for the phonon hot path.
//
// Stages (each a set of batched kernels; matrix b of the batch is picked by
// blockIdx.y/z and may have its own order nvec[b]):
//  1. Householder reduction to real symmetric tridiagonal form, lower
//     formulation, blocked in panels of nb columns: the per-column work
//     (column update, reflector, Hermitian matrix-vector product and its
//     panel corrections) follows the zlatrd recurrence; after each panel the
//     trailing matrix gets the rank-2nb update A -= V W^H + W V^H.  The full
//     Hermitian square is kept so that every matrix-vector pass reads
//     coalesced columns (only its lower triangle is read after assembly).  A = Q T Q^H with Q = H(0) H(1) ... H(n-2),
//     H(i) = I - tau_i v_i v_i^H.
//  2. Eigenvalues of T by Sturm-count bisection, one thread per eigenvalue
//     index, with the dstebz tolerance rule max(abstol, pivmin,
//     2 ulp max(|lo|,|hi|)).  Always FP64.
//  3. Eigenvectors of T by inverse iteration with partial-pivoting LU of
//     T - lambda I, one thread per eigenvalue cluster, modified Gram-Schmidt
//     inside clusters (consecutive eigenvalues closer than 1e-7 ||T||), then
//     a Gram-Schmidt pass over looser clusters (closer than 1e-5 ||T||).
//     Always FP64.
//  4. Back-transform E = Q Z, panel by panel from the last, with the compact
//     WY form I - V Tf V^H (zlarft forward/columnwise).
// Stages 1 and 4 are templated on the real arithmetic R: double (plain FP64
// form) or df (double-float on the FP32 pipes, the mixed form).
#include <atomic>
#include <algorithm>
#include <mutex>
#include <cfloat>
#include <type_traits>
#include <cstdio>

#include "pp_internal.cuh"

namespace pp {

template <class R>
using C = cx<R>;

static inline int cdiv(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }
__device__ __forceinline__ int cdiv_dev(int a, int b) { return (a + b - 1) / b; }

// ---------------------------------------------------------------------------
// block reductions (double / z64)
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
template <int NT>
__device__ double block_sum(double v, double *sh) {
  v = warp_sum(v);
  int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = (threadIdx.x < NT / 32) ? sh[threadIdx.x] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  if (threadIdx.x == 0) sh[0] = r;
  __syncthreads();
  r = sh[0];
  __syncthreads();
  return r;
}
template <int NT>
__device__ z64 block_sum_z(z64 v, double *sh) {
  z64 r;
  r.re = block_sum<NT>(v.re, sh);
  r.im = block_sum<NT>(v.im, sh);
  return r;
}

// ===========================================================================
// Stage 1: reduction to tridiagonal form
// ===========================================================================
constexpr int TR_NT = 256;   // threads of the column kernels
constexpr int HV_CC = 32;    // hemv tile width = rows per partial-sum slot

// Sum of a value over groups of TPR consecutive lanes (every lane of the
// warp takes part; the group's sum ends up in each of its lanes).
template <class R, int TPR>
__device__ __forceinline__ C<R> row_reduce(C<R> y) {
#pragma unroll
  for (int o = TPR / 2; o > 0; o >>= 1) {
    C<R> other;
    float *dst = (float *)&other;
    const float *src = (const float *)&y;
#pragma unroll
    for (int f = 0; f < (int)(sizeof(C<R>) / sizeof(float)); ++f) dst[f] = __shfl_xor_sync(0xffffffffu, src[f], o);
    y = cadd(y, other);
  }
  return y;
}
constexpr int CU_TPR = 1;                // threads per row of k_colupd (one panel column left to apply)
constexpr int CU_ROWS = TR_NT / CU_TPR;  // rows per k_colupd block

// A(i:n,i) -= V(i:n,cb:jj) conj(W(i,cb:jj))^T + W(i:n,cb:jj) conj(V(i,cb:jj))^T ;
// d[i] = Re A(i,i) ; partial sums of |A(r,i)|^2 for r >= i+2.  The panel
// columns below cb = c_begin were applied already by the previous column's
// k_wcorr (which reads the same rows of V and W); here c_begin = jj - 1.
// With fin != 0 it first completes the previous panel column jj-1 (the
// zlatrd step w += alpha v, alpha = -1/2 tau (w^H v), from the partial sums
// of k_wcorr): rows >= i+1 are written back by the block that owns them;
// row i, which every block reads, is completed locally and not written (no
// later kernel reads it).
template <class R>
__global__ void __launch_bounds__(TR_NT) k_colupd(C<R> *Ab, int64_t lda, int64_t sA, C<R> *Wb, int64_t sW,
                                                  const int *nvec, int i, int k0, int jj, double *dd, int64_t sd,
                                                  double *nrm, int nrb, int fin, int nprev, z64 *scal,
                                                  const z64 *wv, int c_begin) {
  __shared__ C<R> sv[64], sw[64];
  __shared__ double red[32];
  __shared__ z64 s_alpha;
  const int b = blockIdx.y;
  const int n = nvec[b];
  if (i >= n) return;
  C<R> *A = Ab + b * sA;
  C<R> *W = Wb + b * sW;
  const int64_t ldw = lda;
  if (fin && threadIdx.x < 32) {  // warp 0 sums the previous column's partials
    z64 sacc{0.0, 0.0};
    for (int k = threadIdx.x; k < nprev; k += 32) {
      sacc.re += wv[b * nrb + k].re;
      sacc.im += wv[b * nrb + k].im;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sacc.re += __shfl_xor_sync(0xffffffffu, sacc.re, o);
      sacc.im += __shfl_xor_sync(0xffffffffu, sacc.im, o);
    }
    if (threadIdx.x == 0) {
      const z64 ts = zmul(scal[b * 4 + 1], sacc);
      s_alpha = z64{-0.5 * ts.re, -0.5 * ts.im};
    }
  }
  __syncthreads();
  const C<R> alpha = fin ? cfrom64<R>(s_alpha) : cz<R>();
  for (int c = c_begin + threadIdx.x; c < jj; c += blockDim.x) {
    sv[c] = A[i + lda * (k0 + c)];
    C<R> wc = W[i + ldw * c];
    if (fin && c == jj - 1) {
      cmac(wc, alpha, A[i + lda * (i - 1)]);
      wc = cfin(wc);
    }
    sw[c] = wc;
  }
  __syncthreads();
  // CU_TPR threads share one row, each taking the panel columns c = sub mod
  // CU_TPR, so that the loads of a row are spread over independent threads.
  const int sub = threadIdx.x % CU_TPR;
  const int r = i + blockIdx.x * CU_ROWS + threadIdx.x / CU_TPR;
  double part = 0.0;
  C<R> acc = cz<R>();
  if (r < n) {
#pragma unroll 4
    for (int c = c_begin + sub; c < jj; c += CU_TPR) {
      C<R> wrc = W[r + ldw * c];
      if (fin && c == jj - 1) {
        cmac(wrc, alpha, A[r + lda * (i - 1)]);
        wrc = cfin(wrc);
        if (r > i) W[r + ldw * c] = wrc;
      }
      cmac(acc, A[r + lda * (k0 + c)], cconj(sw[c]));
      cmac(acc, wrc, cconj(sv[c]));
    }
  }
  acc = cfin(acc);
  acc = row_reduce<R, CU_TPR>(acc);
  if (r < n && sub == 0) {
    C<R> a = A[r + lda * i];
    if (jj > 0) a = csub(a, acc);
    if (r == i) {
      a.im = RT<R>::zero();
      dd[b * sd + i] = RT<R>::to(a.re);
    }
    A[r + lda * i] = a;
    if (r == i + 1) scal[b * 4 + 2] = cto64(a);  // alpha of k_reflector
    if (r >= i + 2) {
      z64 t = cto64(a);
      part = t.re * t.re + t.im * t.im;
    }
  }
  double sn = block_sum<TR_NT>(part, red);
  if (threadIdx.x == 0) nrm[b * nrb + blockIdx.x] = sn;
}

// zlarfg on A(i+1:n, i); v := [1, x/(alpha-beta)] written back in place.
// Every block forms the same scalars (alpha = A(i+1, i) as saved by
// k_colupd, the norm from the same partial sums in the same order) and
// scales RF_ROWS rows; block 0 writes the scalars and v(i+1) = 1.
constexpr int RF_ROWS = 4 * TR_NT;
template <class R>
__global__ void __launch_bounds__(TR_NT) k_reflector(C<R> *Ab, int64_t lda, int64_t sA, const int *nvec, int i,
                                                     int nparts, const double *nrm, int nrb, double *ee, z64 *tau,
                                                     int64_t sd, z64 *scal) {
  __shared__ double red[32];
  __shared__ z64 s_scale;
  __shared__ int s_skip;
  const int b = blockIdx.y;
  const int n = nvec[b];
  if (i >= n - 1) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && i < n) {
      tau[b * sd + i] = z64{0.0, 0.0};
      ee[b * sd + i] = 0.0;
      scal[b * 4 + 0] = z64{0.0, 0.0};
      scal[b * 4 + 1] = z64{0.0, 0.0};
    }
    return;
  }
  C<R> *A = Ab + b * sA;
  double p = 0.0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) p += nrm[b * nrb + k];
  double xn2 = block_sum<TR_NT>(p, red);
  if (threadIdx.x == 0) {
    const z64 alpha = scal[b * 4 + 2];
    double xnorm = sqrt(xn2);
    z64 t, sc;
    double beta;
    int skip = 0;
    if (xnorm == 0.0 && alpha.im == 0.0) {
      t = z64{0.0, 0.0};
      beta = alpha.re;
      sc = z64{1.0, 0.0};
      skip = 1;
    } else {
      double nrm3 = sqrt(alpha.re * alpha.re + alpha.im * alpha.im + xn2);
      beta = -copysign(nrm3, alpha.re);
      t = z64{(beta - alpha.re) / beta, -alpha.im / beta};
      // 1/(alpha - beta)
      double dr = alpha.re - beta, di = alpha.im;
      double den = dr * dr + di * di;
      sc = z64{dr / den, -di / den};
    }
    if (blockIdx.x == 0) {
      ee[b * sd + i] = beta;
      tau[b * sd + i] = t;
      scal[b * 4 + 0] = sc;
      scal[b * 4 + 1] = t;
    }
    s_scale = sc;
    s_skip = skip;
  }
  __syncthreads();
  const C<R> scR = cfrom64<R>(s_scale);
  if (!s_skip) {
    const int rb = i + 2 + blockIdx.x * RF_ROWS, re = min(n, rb + RF_ROWS);
#pragma unroll
    for (int r = rb + threadIdx.x; r < re; r += TR_NT) A[r + lda * i] = cmul(A[r + lda * i], scR);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) A[(i + 1) + lda * i] = cfrom64<R>(1.0, 0.0);
}

// Lower-triangle Hermitian mat-vec y = A v on the trailing block [i+1, n),
// over the lower tile pairs (R >= C) of HL_T x HL_T: a tile is read once and
// gives both A_RC v_C (into slot C of the rows of R) and A_RC^H v_R (into
// slot R of the rows of C).  Every row receives exactly one partial per slot
// 0 .. ntiles-1, summed later by k_wcorr.  Blocks are persistent over a
// strided set of tile pairs with two shared-memory buffers: the next tile
// (and its two vector pieces) is copied by cp.async while the double-float
// arithmetic of the current one runs.
constexpr int HL_T = 32;
constexpr int HL_LD = HL_T + 1;  // padded column stride of the shared tile
constexpr int HL_NT = 128;
constexpr int HL_BPS = 6;        // resident blocks per SM
constexpr int HL_UNROLL = 4;     // inner-loop unrolling (keeps the kernel's code small)
__device__ __forceinline__ void cp_async16(void *dst, const void *src, bool valid) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(valid ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void tile_pair(int p, int &Rt, int &Ct) {
  Rt = (int)((sqrtf(8.0f * (float)p + 1.0f) - 1.0f) * 0.5f);
  while ((Rt + 1) * (Rt + 2) / 2 <= p) ++Rt;
  while (Rt * (Rt + 1) / 2 > p) --Rt;
  Ct = p - Rt * (Rt + 1) / 2;
}
template <class R>
__global__ void __launch_bounds__(HL_NT, HL_BPS) k_hemv_lower(const C<R> *Ab, int64_t lda, int64_t sA,
                                                              const int *nvec, int i, C<R> *Pb, int64_t sP,
                                                              int64_t ldp) {
  __shared__ __align__(16) C<R> tile[2][HL_T * HL_LD];  // tile[buf][c * HL_LD + r]
  __shared__ __align__(16) C<R> vR[2][HL_T], vC[2][HL_T];
  __shared__ C<R> red[2][2][HL_T];
  const int b = blockIdx.z;
  const int n = nvec[b];
  const int r0 = i + 1;
  if (r0 >= n) return;
  const int nt = (n - r0 + HL_T - 1) / HL_T;
  const int npairs = nt * (nt + 1) / 2;
  if ((int)blockIdx.x >= npairs) return;
  const C<R> *A = Ab + b * sA;
  const int tid = threadIdx.x;
  // copies of tile pair p into buffer buf (zero outside the matrix)
  auto issue = [&](int p, int buf) {
    int Rt, Ct;
    tile_pair(p, Rt, Ct);
    const int rt0 = r0 + Rt * HL_T, ct0 = r0 + Ct * HL_T;
    // element (r, c) = (tid % HL_T, tid / HL_T + CS j), j < HL_T / CS
    constexpr int CS = HL_NT / HL_T;
    const int r = tid % HL_T, cb = tid / HL_T;
    const int rr = rt0 + r;
    const C<R> *src = A + rr + lda * (ct0 + cb);
    C<R> *dst = &tile[buf][cb * HL_LD + r];
#pragma unroll
    for (int j = 0; j < HL_T / CS; ++j) {
      const bool ok = rr < n && ct0 + cb + CS * j < n;
      cp_async16(dst + CS * j * HL_LD, ok ? (const void *)(src + CS * j * lda) : (const void *)A, ok);
    }
    if (tid < HL_T) {
      const int rr = rt0 + tid;
      cp_async16(&vR[buf][tid], rr < n ? (const void *)&A[rr + lda * i] : (const void *)A, rr < n);
    } else if (tid < 2 * HL_T) {
      const int cc = ct0 + tid - HL_T;
      cp_async16(&vC[buf][tid - HL_T], cc < n ? (const void *)&A[cc + lda * i] : (const void *)A, cc < n);
    }
    cp_async_commit();
  };
  // warps 0-1: A_RC v_C (thread = row, half of the columns each);
  // warps 2-3: A_RC^H v_R (thread = column, half of the rows each)
  const int lane = tid & (HL_T - 1), wid = tid / HL_T;
  const int prod = wid >> 1, half = wid & 1;
  constexpr int SPAN = HL_T / 2;
  issue(blockIdx.x, 0);
  int buf = 0;
  for (int p = blockIdx.x; p < npairs; p += gridDim.x) {
    if (p + (int)gridDim.x < npairs)
      issue(p + gridDim.x, buf ^ 1);
    else
      cp_async_commit();  // an empty group keeps "all but the newest" meaning this tile
    cp_async_wait1();
    __syncthreads();
    int Rt, Ct;
    tile_pair(p, Rt, Ct);
    const int rt0 = r0 + Rt * HL_T, ct0 = r0 + Ct * HL_T;
    const bool diag = (Rt == Ct);
    const C<R> *tl = tile[buf];
    if (prod == 0) {
      C<R> acc = cz<R>();
      const int r = lane;
      if (!diag) {
#pragma unroll HL_UNROLL
        for (int c = half * SPAN; c < half * SPAN + SPAN; ++c) cmac(acc, tl[c * HL_LD + r], vC[buf][c]);
      } else {  // diagonal tile: the upper part is the conjugate of the mirrored element
#pragma unroll HL_UNROLL
        for (int c = half * SPAN; c < half * SPAN + SPAN; ++c) {
          const C<R> a = (r >= c) ? tl[c * HL_LD + r] : cconj(tl[r * HL_LD + c]);
          cmac(acc, a, vC[buf][c]);
        }
      }
      red[0][half][r] = cfin(acc);
    } else if (!diag) {
      C<R> acc = cz<R>();
      const int c = lane;
#pragma unroll HL_UNROLL
      for (int r = half * SPAN; r < half * SPAN + SPAN; ++r) cmacc(acc, tl[c * HL_LD + r], vR[buf][r]);
      red[1][half][c] = cfin(acc);
    }
    __syncthreads();
    if (wid == 0 && rt0 + lane < n)
      Pb[b * sP + (int64_t)Ct * ldp + rt0 + lane] = cadd(red[0][0][lane], red[0][1][lane]);
    if (wid == 2 && !diag && ct0 + lane < n)
      Pb[b * sP + (int64_t)Rt * ldp + ct0 + lane] = cadd(red[1][0][lane], red[1][1][lane]);
    __syncthreads();  // the buffer and red are free for the next iteration
    buf ^= 1;
  }
  cp_async_wait0();
}

// X[c] = V(:,c)^H v (c < jj), X[jj+c] = W(:,c)^H v, over rows [i+1, n).
template <class R>
__global__ void __launch_bounds__(TR_NT) k_dots(const C<R> *Ab, int64_t lda, int64_t sA, const C<R> *Wb, int64_t sW,
                                                const int *nvec, int i, int k0, int jj, z64 *X, int ldx) {
  __shared__ double red[32];
  const int b = blockIdx.y;
  const int n = nvec[b];
  if (i >= n - 1) return;
  const C<R> *A = Ab + b * sA;
  const C<R> *W = Wb + b * sW;
  const int c2 = blockIdx.x;
  const bool useW = c2 >= jj;
  const int c = useW ? c2 - jj : c2;
  const C<R> *Xc = useW ? (W + lda * c) : (A + lda * (k0 + c));
  C<R> acc = cz<R>();
#pragma unroll 4
  for (int r = i + 1 + threadIdx.x; r < n; r += blockDim.x) cmacc(acc, Xc[r], A[r + lda * i]);
  z64 s = block_sum_z<TR_NT>(cto64(cfin(acc)), red);
  if (threadIdx.x == 0) X[b * ldx + c2] = s;
}

// w = tau (y - W x1 - V x2) with y = sum of hemv partials; partial w^H v.
// WC_TPR threads share one row: each sums a strided subset of the partial
// slots, then a shuffle reduction; this keeps many independent loads in
// flight per row (the slots are the latency-bound part).
constexpr int WC_TPR = 8;
constexpr int WC_ROWS = TR_NT / WC_TPR;  // rows per block
template <class R>
__global__ void __launch_bounds__(TR_NT) k_wcorr(C<R> *Ab, int64_t lda, int64_t sA, C<R> *Wb, int64_t sW,
                                                 const C<R> *Pb, int64_t sP, int64_t ldp, const int *nvec, int i,
                                                 int k0, int jj, const z64 *X, int ldx, const z64 *scal, z64 *wv,
                                                 int nrb, int fuse) {
  __shared__ C<R> x1[64], x2[64], nv[64], nw[64];
  __shared__ double red[32];
  const int b = blockIdx.y;
  const int n = nvec[b];
  if (i >= n - 1) return;
  C<R> *A = Ab + b * sA;
  C<R> *W = Wb + b * sW;
  for (int c = threadIdx.x; c < jj; c += blockDim.x) {
    x1[c] = cfrom64<R>(X[b * ldx + c]);       // V^H v
    x2[c] = cfrom64<R>(X[b * ldx + jj + c]);  // W^H v
    if (fuse) {                               // row i+1 of V and W
      nv[c] = cconj(A[(i + 1) + lda * (k0 + c)]);
      nw[c] = cconj(W[(i + 1) + lda * c]);
    }
  }
  __syncthreads();
  const int sub = threadIdx.x % WC_TPR;
  const int r = i + 1 + blockIdx.x * WC_ROWS + threadIdx.x / WC_TPR;
  z64 part{0.0, 0.0};
  const int nch = cdiv_dev(n - i - 1, HV_CC);
  C<R> y = cz<R>(), nxt = cz<R>();
  if (r < n) {
    const C<R> *Pr = Pb + b * sP + r;
#pragma unroll 4
    for (int ch = sub; ch < nch; ch += WC_TPR) y = cadd(y, Pr[(int64_t)ch * ldp]);
    // this thread's share of the panel corrections, columns c = sub mod
    // WC_TPR; with fuse also the same columns' update of column i+1
    C<R> acc = cz<R>();
#pragma unroll 4
    for (int c = sub; c < jj; c += WC_TPR) {
      const C<R> wrc = W[r + lda * c], vrc = A[r + lda * (k0 + c)];
      cmac(acc, wrc, x1[c]);
      cmac(acc, vrc, x2[c]);
      if (fuse) {
        cmac(nxt, vrc, nw[c]);
        cmac(nxt, wrc, nv[c]);
      }
    }
    y = csub(y, cfin(acc));
  }
  y = row_reduce<R, WC_TPR>(y);
  if (fuse) {
    // A(r, i+1) -= V(r, 0:jj) conj(W(i+1, 0:jj))^T + W(r, 0:jj) conj(V(i+1, 0:jj))^T
    nxt = row_reduce<R, WC_TPR>(cfin(nxt));
    if (r < n && sub == 0) A[r + lda * (i + 1)] = csub(A[r + lda * (i + 1)], nxt);
  }
  if (r < n && sub == 0) {
    const C<R> t = cfrom64<R>(scal[b * 4 + 1]);
    C<R> w = cmul(t, y);
    W[r + lda * jj] = w;
    z64 w64 = cto64(w), v64 = cto64(A[r + lda * i]);
    part = z64{w64.re * v64.re + w64.im * v64.im, w64.re * v64.im - w64.im * v64.re};
  }
  z64 s = block_sum_z<TR_NT>(part, red);
  if (threadIdx.x == 0) wv[b * nrb + blockIdx.x] = s;
}

// alpha = -1/2 tau (w^H v) ; w += alpha v
template <class R>
__global__ void __launch_bounds__(TR_NT) k_wfin(const C<R> *Ab, int64_t lda, int64_t sA, C<R> *Wb, int64_t sW,
                                                const int *nvec, int i, int jj, int nparts, const z64 *scal,
                                                const z64 *wv, int nrb) {
  __shared__ z64 s_alpha;
  const int b = blockIdx.y;
  const int n = nvec[b];
  if (i >= n - 1) return;
  if (threadIdx.x == 0) {
    z64 s{0.0, 0.0};
    for (int k = 0; k < nparts; ++k) {
      s.re += wv[b * nrb + k].re;
      s.im += wv[b * nrb + k].im;
    }
    z64 t = scal[b * 4 + 1];
    z64 ts = zmul(t, s);
    s_alpha = z64{-0.5 * ts.re, -0.5 * ts.im};
  }
  __syncthreads();
  const int r = i + 1 + blockIdx.x * TR_NT + threadIdx.x;
  if (r >= n) return;
  const C<R> *A = Ab + b * sA;
  C<R> *W = Wb + b * sW;
  C<R> acc = W[r + lda * jj];
  cmac(acc, cfrom64<R>(s_alpha), A[r + lda * i]);
  W[r + lda * jj] = cfin(acc);
}

// Trailing update A(k1:n, k1:n) -= V W^H + W V^H (full square), K = jb.
constexpr int HK_T = 64, HK_K = 8;
template <class R>
__global__ void __launch_bounds__(256) k_her2k(C<R> *Ab, int64_t lda, int64_t sA, const C<R> *Wb, int64_t sW,
                                               const int *nvec, int k0, int jb) {
  __shared__ C<R> sVr[HK_K][HK_T], sWr[HK_K][HK_T], sVc[HK_K][HK_T], sWc[HK_K][HK_T];
  const int b = blockIdx.z;
  const int n = nvec[b];
  const int k1 = k0 + jb;
  if (blockIdx.x < blockIdx.y) return;  // only the lower triangle is kept
  const int r0 = k1 + blockIdx.x * HK_T, c0 = k1 + blockIdx.y * HK_T;
  if (r0 >= n || c0 >= n) return;
  C<R> *A = Ab + b * sA;
  const C<R> *W = Wb + b * sW;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  C<R> acc[4][4];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = cz<R>();
  const int jmax = min(jb, n - 1 - k0);  // reflectors that exist in this matrix
  for (int kc = 0; kc < jmax; kc += HK_K) {
    for (int e = threadIdx.x; e < HK_K * HK_T; e += 256) {
      int x = e % HK_T, y = e / HK_T;
      int k = kc + y;
      int rr = r0 + x, cc = c0 + x;
      bool ok = k < jmax;
      sVr[y][x] = (ok && rr < n) ? A[rr + lda * (k0 + k)] : cz<R>();
      sWr[y][x] = (ok && rr < n) ? W[rr + lda * k] : cz<R>();
      sVc[y][x] = (ok && cc < n) ? cconj(A[cc + lda * (k0 + k)]) : cz<R>();
      sWc[y][x] = (ok && cc < n) ? cconj(W[cc + lda * k]) : cz<R>();
    }
    __syncthreads();
#pragma unroll 2
    for (int k = 0; k < HK_K; ++k) {
      C<R> vr[4], wr[4], vc[4], wc[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        vr[p] = sVr[k][tx + 16 * p];
        wr[p] = sWr[k][tx + 16 * p];
        vc[p] = sVc[k][ty + 16 * p];
        wc[p] = sWc[k][ty + 16 * p];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          cmac(acc[p][q], vr[p], wc[q]);
          cmac(acc[p][q], wr[p], vc[q]);
        }
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int rr = r0 + tx + 16 * p, cc = c0 + ty + 16 * q;
      if (rr < n && cc < n) {
        C<R> *x = &A[rr + lda * cc];
        *x = csub(*x, cfin(acc[p][q]));
      }
    }
}

// Persistent hemv blocks: bps per SM of the current device (at most HL_BPS,
// the residency the kernel is compiled for).
static int hemv_blocks(int bps) { return device_sms() * std::max(1, std::min(bps, HL_BPS)); }

template <class R>
cudaError_t tridiagonalize(EigWork &w, cudaStream_t s) {
  C<R> *A = (C<R> *)w.A;
  C<R> *W = (C<R> *)w.W;
  C<R> *P = (C<R> *)w.P;
  const int B = w.B, nmax = w.nmax, nb = w.nb;
  const int64_t lda = w.lda, sA = w.sA, sW = (int64_t)w.lda * nb, sP = (int64_t)w.nchunk * w.lda;
  const int64_t sd = w.nmax;
  if (w.tcErr) PP_CUDA_TRY(cudaMemsetAsync(w.tcErr, 0, sizeof(int) * B, s));
  for (int k0 = 0; k0 < nmax; k0 += nb) {
    const int jb = min(nb, nmax - k0);
    int nprev = 0;  // k_wcorr blocks of the previous column, when its w is still to be completed
    for (int jj = 0; jj < jb; ++jj) {
      const int i = k0 + jj;
      const int nparts = cdiv(nmax - i, CU_ROWS);
      const int fin = (jj > 0 && nprev > 0) ? 1 : 0;
      PP_KT(KT_COLUPD, s, (k_colupd<R><<<dim3(nparts, B), TR_NT, 0, s>>>(A, lda, sA, W, sW, w.nvec, i, k0, jj, w.d, sd,
                                                                         w.nrm, w.nrb, fin, nprev, w.scal,
                                                                         (z64 *)w.wv, jj > 0 ? jj - 1 : 0)));
      nprev = 0;
      if (i >= nmax - 1) {
        count_launch(1);
        continue;
      }
      PP_KT(KT_REFL, s, (k_reflector<R><<<dim3(std::max(1, cdiv(nmax - i - 2, RF_ROWS)), B), TR_NT, 0, s>>>(
                            A, lda, sA, w.nvec, i, nparts, w.nrm, w.nrb, w.e, w.tau, sd, w.scal)));
      const int m = nmax - i - 1;
      const int nt = cdiv(m, HL_T);
      PP_KT(KT_HEMV, s, (k_hemv_lower<R><<<dim3(std::min(nt * (nt + 1) / 2, hemv_blocks(w.hemv_bps)), 1, B), HL_NT, 0, s>>>(
                            A, lda, sA, w.nvec, i, P, sP, lda)));
      if (jj > 0) PP_KT(KT_DOTS, s, (k_dots<R><<<dim3(2 * jj, B), TR_NT, 0, s>>>(A, lda, sA, W, sW, w.nvec, i, k0, jj, (z64 *)w.X, 2 * nb)));
      const int nr = cdiv(m, TR_NT);
      const int nrw = cdiv(m, WC_ROWS);
      // within a panel, k_wcorr also applies columns 0 .. jj-1 to column i+1
      PP_KT(KT_WCORR, s, (k_wcorr<R><<<dim3(nrw, B), TR_NT, 0, s>>>(A, lda, sA, W, sW, P, sP, lda, w.nvec, i, k0, jj, (z64 *)w.X, 2 * nb,
                                               w.scal, (z64 *)w.wv, w.nrb, jj + 1 < jb ? 1 : 0)));
      if (jj == jb - 1 || i == nmax - 2) {
        // last column of the panel: the trailing update reads W next
        PP_KT(KT_WFIN, s, (k_wfin<R><<<dim3(nr, B), TR_NT, 0, s>>>(A, lda, sA, W, sW, w.nvec, i, jj, nrw, w.scal, (z64 *)w.wv, w.nrb)));
        count_launch(jj > 0 ? 7 : 6);
      } else {
        nprev = nrw;  // completed by the next column's k_colupd
        count_launch(jj > 0 ? 6 : 5);
      }
    }
    const int k1 = k0 + jb;
    if (k1 < nmax) {
      if (std::is_same<R, df>::value && w.tcS && tc_enabled()) {
        PP_CUDA_TRY(her2k_tc(w, k0, jb, s));
      } else {
        const int m = nmax - k1;
        dim3 g(cdiv(m, HK_T), cdiv(m, HK_T), B);
        PP_KT(KT_HER2K, s, (k_her2k<R><<<g, 256, 0, s>>>(A, lda, sA, W, sW, w.nvec, k0, jb)));
        count_launch(1);
      }
    }
  }
  return cudaGetLastError();
}

// ===========================================================================
// Stage 2: eigenvalues of the tridiagonal matrix (FP64 bisection)
// ===========================================================================
__device__ __forceinline__ int sturm_count(const double *d, const double *e2, int n, double x, double pivmin) {
  double q = d[0] - x;
  if (fabs(q) <= pivmin) q = -pivmin;
  int c = q < 0.0;
  for (int k = 1; k < n; ++k) {
    q = d[k] - e2[k - 1] / q - x;
    if (fabs(q) <= pivmin) q = -pivmin;
    c += q < 0.0;
  }
  return c;
}

// Gerschgorin interval, pivmin and the index range of the wanted eigenvalues.
__global__ void k_tdprep(const double *dd, const double *ee, int64_t sd, const int *nvec, char range, double vl,
                         double vu, int64_t il, int64_t iu, int64_t *rng, double *tinfo, int64_t *info,
                         const int *tcerr) {
  const int b = blockIdx.x;
  if (threadIdx.x != 0) return;
  const int n = nvec[b];
  const double *d = dd + b * sd;
  const double *e = ee + b * sd;
  double gl = d[0], gu = d[0], emax2 = 0.0;
  for (int k = 0; k < n; ++k) {
    double off = (k > 0 ? fabs(e[k - 1]) : 0.0) + (k < n - 1 ? fabs(e[k]) : 0.0);
    gl = fmin(gl, d[k] - off);
    gu = fmax(gu, d[k] + off);
    if (k < n - 1) emax2 = fmax(emax2, e[k] * e[k]);
  }
  const double ulp = DBL_EPSILON;
  const double safmin = DBL_MIN;
  double tnorm = fmax(fabs(gl), fabs(gu));
  double pivmin = safmin * fmax(1.0, emax2);
  const double fudge = 2.1;
  gl = gl - fudge * tnorm * ulp * n - fudge * 2.0 * pivmin;
  gu = gu + fudge * tnorm * ulp * n + fudge * 2.0 * pivmin;
  int64_t lo = 1, hi = n;
  if (range == 'I') {
    lo = il;
    hi = iu;
  } else if (range == 'V') {
    // eigenvalues in the half-open interval (vl, vu]
    // local e^2 recomputed on the fly
    double q;
    int cl = 0, cu = 0;
    for (int pass = 0; pass < 2; ++pass) {
      double x = pass == 0 ? vl : vu;
      q = d[0] - x;
      if (fabs(q) <= pivmin) q = -pivmin;
      int c = q < 0.0;
      for (int k = 1; k < n; ++k) {
        q = d[k] - (e[k - 1] * e[k - 1]) / q - x;
        if (fabs(q) <= pivmin) q = -pivmin;
        c += q < 0.0;
      }
      if (pass == 0)
        cl = c;
      else
        cu = c;
    }
    lo = cl + 1;
    hi = cu;
  }
  int64_t m = hi - lo + 1;
  if (m < 0) m = 0;
  rng[b * 8 + 0] = lo;
  rng[b * 8 + 1] = hi;
  rng[b * 8 + 2] = m;
  tinfo[b * 8 + 0] = gl;
  tinfo[b * 8 + 1] = gu;
  tinfo[b * 8 + 2] = tnorm;
  tinfo[b * 8 + 3] = pivmin;
  info[b] = (tcerr && tcerr[b]) ? PP_INFO_TIMEOUT : 0;
}

__device__ __forceinline__ int sturm_count32(const float *d, const float *e2, int n, float x, float pivmin) {
  float q = d[0] - x;
  if (fabsf(q) <= pivmin) q = -pivmin;
  int c = q < 0.0f;
  for (int k = 1; k < n; ++k) {
    q = d[k] - __fdividef(e2[k - 1], q) - x;
    if (fabsf(q) <= pivmin) q = -pivmin;
    c += q < 0.0f;
  }
  return c;
}

// Sturm count in double-float: q_k = (d_k - x) - e2_{k-1} / q_{k-1} with
// d, e2 and x as hi + lo float pairs.  The quotient is a float estimate
// corrected once by its exact remainder (TwoProd by FMA), about 44 bits; the
// count is then exact for a tridiagonal perturbed by a few 2^-44 relative in
// each entry, the double-float analogue of the FP64 count's backward error.
__device__ __forceinline__ int sturm_count_df(const float *dh, const float *dl, const float *eh, const float *el,
                                              int n, df x, float pivmin) {
  float qh, ql;
  {
    float s, e;
    two_sum(dh[0], -x.hi, s, e);
    e = __fadd_rn(e, __fsub_rn(dl[0], x.lo));
    fast_two_sum(s, e, qh, ql);
  }
  if (fabsf(qh) <= pivmin) {
    qh = -pivmin;
    ql = 0.0f;
  }
  int c = qh < 0.0f;
  for (int k = 1; k < n; ++k) {
    // t = e2 / q
    const float a = eh[k - 1], al = el[k - 1];
    const float th = __fdividef(a, qh);
    const float p = __fmul_rn(th, qh);
    const float pe = __fmaf_rn(th, qh, -p);
    float rem = __fsub_rn(a, p);
    rem = __fsub_rn(rem, pe);
    rem = __fadd_rn(rem, al);
    rem = __fmaf_rn(-th, ql, rem);
    const float tl = __fdividef(rem, qh);
    // q = (d - x) - t as a three-term sum with one renormalisation
    float s1, e1, s2, e2;
    two_sum(dh[k], -x.hi, s1, e1);
    two_sum(s1, -th, s2, e2);
    const float lo = __fadd_rn(__fadd_rn(e1, e2), __fsub_rn(__fsub_rn(dl[k], x.lo), tl));
    fast_two_sum(s2, lo, qh, ql);
    if (fabsf(qh) <= pivmin) {
      qh = -pivmin;
      ql = 0.0f;
    }
    c += qh < 0.0f;
  }
  return c;
}

// One thread per wanted eigenvalue.  mode 0: FP64 counts from global memory;
// mode 1: the tridiagonal in shared memory, the interval first narrowed with
// FP32 Sturm counts (cheap on the FP32 pipes), then widened by a margin far
// above the FP32 backward error of the count (64 eps32 (||T|| + |x|)),
// checked with two counts (falling back to the Gerschgorin interval if the
// check fails) and finished in FP64; mode 2 (mixed form): as mode 1 but
// checked and finished with double-float counts, whose accuracy floor
// (a few 2^-44 ||T||) ends the bisection.
__global__ void __launch_bounds__(128) k_bisect(const double *dd, const double *ee, int64_t sd, const int *nvec,
                                                const int64_t *rng, const double *tinfo, double abstol, double *wout,
                                                int64_t *info, int mode) {
  extern __shared__ double sm[];
  const int b = blockIdx.y;
  const int n = nvec[b];
  const double *d = dd + b * sd;
  const double *e = ee + b * sd;
  double *sd_ = sm;
  double *se2 = sm + n;
  float *fd = (float *)(sm + 2 * n);
  float *fe2 = fd + n;
  // mode 2 layout: d.hi, d.lo, e2.hi, e2.lo
  float *gdh = (float *)sm, *gdl = gdh + n, *ge2h = gdl + n, *ge2l = ge2h + n;
  if (mode == 1) {
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      const double e2 = (k < n - 1) ? e[k] * e[k] : 0.0;
      sd_[k] = d[k];
      se2[k] = e2;
      fd[k] = (float)d[k];
      fe2[k] = (float)e2;
    }
    __syncthreads();
  } else if (mode == 2) {
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
      const double e2 = (k < n - 1) ? e[k] * e[k] : 0.0;
      const df dk = df_from(d[k]), ek = df_from(e2);
      gdh[k] = dk.hi;
      gdl[k] = dk.lo;
      ge2h[k] = ek.hi;
      ge2l[k] = ek.lo;
    }
    __syncthreads();
    fd = gdh;
    fe2 = ge2h;
  }
  const int64_t lo_idx = rng[b * 8 + 0];
  const int64_t m = rng[b * 8 + 2];
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= m) return;
  const int64_t idx = lo_idx + j;
  const double gl = tinfo[b * 8 + 0], gu = tinfo[b * 8 + 1], tnorm = tinfo[b * 8 + 2];
  const double pivmin = tinfo[b * 8 + 3];
  double lo = gl, hi = gu;
  const double ulp = DBL_EPSILON;
  const float pivdf = fmaxf(1e-30f, (float)pivmin);
  auto count64 = [&](double x) -> int {
    if (mode == 2) return sturm_count_df(gdh, gdl, ge2h, ge2l, n, df_from(x), pivdf);
    if (mode == 1) return sturm_count(sd_, se2, n, x, pivmin);
    double q = d[0] - x;
    if (fabs(q) <= pivmin) q = -pivmin;
    int c = q < 0.0;
    for (int k = 1; k < n; ++k) {
      q = d[k] - (e[k - 1] * e[k - 1]) / q - x;
      if (fabs(q) <= pivmin) q = -pivmin;
      c += q < 0.0;
    }
    return c;
  };
  if (mode != 0 && tnorm > 0.0 && tnorm < 1e30) {
    float lo32 = (float)lo, hi32 = (float)hi;
    const float piv32 = fmaxf(1e-30f, (float)pivmin);
    const float stop = 16.0f * FLT_EPSILON * (float)tnorm;
    for (int it = 0; it < 48 && hi32 - lo32 > stop; ++it) {
      const float mid = 0.5f * (lo32 + hi32);
      if (sturm_count32(fd, fe2, n, mid, piv32) >= idx)
        hi32 = mid;
      else
        lo32 = mid;
    }
    const double marg = 64.0 * FLT_EPSILON * (tnorm + fmax(fabs((double)lo32), fabs((double)hi32)));
    const double l2 = fmax(gl, (double)lo32 - marg), h2 = fmin(gu, (double)hi32 + marg);
    if (count64(l2) < idx && count64(h2) >= idx) {
      lo = l2;
      hi = h2;
    }
  }
  // accuracy floor of the double-float count (mode 2)
  const double floor_df = (mode == 2) ? 4.0 * 0x1p-44 * tnorm : 0.0;
  bool conv = false;
  for (int it = 0; it < 256; ++it) {
    double tol = fmax(fmax(fmax(abstol, pivmin), 2.0 * ulp * fmax(fabs(lo), fabs(hi))), floor_df);
    if (hi - lo <= tol) {
      conv = true;
      break;
    }
    double mid = 0.5 * (lo + hi);
    if (count64(mid) >= idx)
      hi = mid;
    else
      lo = mid;
  }
  if (!conv) atomicOr((unsigned long long *)&info[b], (unsigned long long)PP_INFO_NOCONV);
  wout[b * sd + j] = 0.5 * (lo + hi);
}

// Opt the bisection kernel into the dynamic shared memory it needs for order
// n (done once per size outside any stream capture).
size_t bisect_smem(int64_t n, int mixed) {
  const size_t b = mixed ? 4 * (size_t)n * sizeof(float) : 2 * (size_t)n * (sizeof(double) + sizeof(float));
  return b <= 200 * 1024 ? b : 0;
}

// The attribute applies to the current device only: a high-water mark is
// kept per device.
cudaError_t prepare_bisect(size_t bytes) {
  static std::mutex mu;
  static int done[PP_MAX_DEVICES] = {};
  const int need = (int)bytes;
  if (need > 200 * 1024) return cudaSuccess;
  const int dev = device_index();
  std::lock_guard<std::mutex> g(mu);
  if (dev >= 0 && need <= done[dev]) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_bisect, cudaFuncAttributeMaxDynamicSharedMemorySize, need);
  if (e == cudaSuccess && dev >= 0) done[dev] = need;
  return e;
}

cudaError_t tridiag_eigenvalues(EigWork &w, char range, double vl, double vu, int64_t il, int64_t iu, double abstol,
                                cudaStream_t s, int mixed) {
  const int64_t sd = w.nmax;
  k_tdprep<<<w.B, 32, 0, s>>>(w.d, w.e, sd, w.nvec, range, vl, vu, il, iu, w.rng, w.tinfo, w.info, w.tcErr);
  const size_t smem = bisect_smem(w.nmax, mixed);
  int mode = 0;
  if (smem) {
    mode = mixed ? 2 : 1;
    PP_CUDA_TRY(prepare_bisect(smem));
  }
  dim3 g(cdiv(w.nmax, 128), w.B);
  PP_KT(KT_BISECT, s, (k_bisect<<<g, 128, smem, s>>>(w.d, w.e, sd, w.nvec, w.rng, w.tinfo, abstol, w.w, w.info, mode)));
  count_launch(2);
  return cudaGetLastError();
}


// ===========================================================================
// Stage 3: eigenvectors of T by inverse iteration
// ===========================================================================
// Clusters of consecutive eigenvalues closer than rel * ||T||.
__global__ void k_clusters(const double *ww, int64_t sd, const int64_t *rng, const double *tinfo, int *cls,
                           int64_t scl, int *ncl, double rel) {
  const int b = blockIdx.x;
  if (threadIdx.x != 0) return;
  const int64_t m = rng[b * 8 + 2];
  const double tnorm = tinfo[b * 8 + 2];
  const double ortol = rel * tnorm;
  const double *w = ww + b * sd;
  int c = 0;
  for (int64_t j = 0; j < m; ++j) {
    if (j == 0 || w[j] - w[j - 1] > ortol) cls[b * scl + c++] = (int)j;
  }
  cls[b * scl + c] = (int)m;
  ncl[b] = c;
}

// Inverse iteration orthogonalises only inside tight clusters (where the
// iterates would otherwise converge to the same vector); eigenvectors of
// eigenvalues further apart but closer than 1e-5 ||T|| keep an overlap of
// about eps ||T|| / gap.  Modified Gram-Schmidt inside those loose clusters
// removes it, one block per cluster (block-wide dot products in FP64).
constexpr int RO_BLOCKS = 64;  // blocks per matrix of k_reorth (cluster c goes to block c mod 64)
template <class R>
__global__ void __launch_bounds__(256) k_reorth(C<R> *Eb, int64_t lde, int64_t sE, const int *nvec, const int *cls,
                                                int64_t scl, const int *ncl) {
  __shared__ double red[32];
  const int b = blockIdx.y;
  const int n = nvec[b];
  C<R> *E = Eb + b * sE;
  const int nc = ncl[b];
  for (int c = blockIdx.x; c < nc; c += gridDim.x) {  // clusters are independent
    const int j0 = cls[b * scl + c], j1 = cls[b * scl + c + 1];
    if (j1 - j0 < 2) continue;
    for (int j = j0 + 1; j < j1; ++j) {
      for (int jp = j0; jp < j; ++jp) {
        double part = 0.0;
        for (int k = threadIdx.x; k < n; k += blockDim.x) part += RT<R>::to(E[k + lde * jp].re) * RT<R>::to(E[k + lde * j].re);
        const double dot = block_sum<256>(part, red);
        for (int k = threadIdx.x; k < n; k += blockDim.x) {
          const double v = RT<R>::to(E[k + lde * j].re) - dot * RT<R>::to(E[k + lde * jp].re);
          E[k + lde * j].re = RT<R>::from(v);
        }
        __syncthreads();
      }
      double part = 0.0;
      for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const double v = RT<R>::to(E[k + lde * j].re);
        part += v * v;
      }
      const double inv = 1.0 / sqrt(block_sum<256>(part, red));
      for (int k = threadIdx.x; k < n; k += blockDim.x)
        E[k + lde * j].re = RT<R>::from(RT<R>::to(E[k + lde * j].re) * inv);
      __syncthreads();
    }
  }
}

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

// One thread per cluster of eigenvalues (clusters cbase .. cbase+T-1).
// LU of T - lam I with partial pivoting: row k of U holds (u0,u1,u2) at
// columns (k, k+1, k+2); l is the multiplier, piv marks a row interchange.
// The factors and the working vector x live in scratch interleaved by thread
// ([row][field][thread]) so that a warp's accesses coalesce; the finished
// vector is written to its column of E once.  Every pass over the rows runs
// in chunks of IV_CH rows whose loads are all issued before the chunk's
// arithmetic and stores: the recurrences are sequential in the row, and a
// load behind a store to the same scratch array would otherwise wait out one
// memory latency per row.  The arithmetic and its order are those of the
// row-by-row loops.
constexpr int IV_F = 5;   // u0, u1, u2, l, x
constexpr int IV_CH = 8;  // rows per chunk
template <class R>
__global__ void __launch_bounds__(64) k_invit(const double *__restrict__ dd, const double *__restrict__ ee, int64_t sd,
                                              const int *nvec, const double *ww, const int64_t *rng,
                                              const double *tinfo, const int *cls, int64_t scl, const int *ncl,
                                              int cbase, C<R> *Eb, int64_t lde, int64_t sE, double *scratch,
                                              uint8_t *pivb, int64_t T, int64_t sS, int64_t sPv, int64_t *info) {
  const int b = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = cbase + t;
  if (t >= T || c >= ncl[b]) return;
  const int n = nvec[b];
  const double *__restrict__ d = dd + b * sd;
  const double *__restrict__ e = ee + b * sd;
  const double *w = ww + b * sd;
  C<R> *E = Eb + b * sE;
  double *S = scratch + b * sS;
  uint8_t *PV = pivb + b * sPv;
#define SU0(k) S[((int64_t)(k)*IV_F + 0) * T + t]
#define SU1(k) S[((int64_t)(k)*IV_F + 1) * T + t]
#define SU2(k) S[((int64_t)(k)*IV_F + 2) * T + t]
#define SL(k) S[((int64_t)(k)*IV_F + 3) * T + t]
#define XS(k) S[((int64_t)(k)*IV_F + 4) * T + t]
#define PIV(k) PV[(int64_t)(k)*T + t]
  const double tnorm = tinfo[b * 8 + 2];
  const double eps = DBL_EPSILON * 0.5;
  const double pivtol = fmax(eps * tnorm, DBL_MIN);
  const int j0 = cls[b * scl + c], j1 = cls[b * scl + c + 1];
  const int iters = (j1 - j0 > 1) ? 3 : 2;
  double lam_prev = 0.0;
  int bad = 0;
  for (int j = j0; j < j1; ++j) {
    double lam = w[j];
    if (j > j0) {
      const double pert = 10.0 * eps * fmax(fabs(lam), 1e-3 * tnorm);
      if (lam <= lam_prev + pert) lam = lam_prev + pert;
    }
    lam_prev = lam;
    // ---- factor T - lam I
    double p = d[0] - lam, qv = (n > 1) ? e[0] : 0.0;
    for (int kb = 0; kb < n - 1; kb += IV_CH) {
      double ck[IV_CH], dk1[IV_CH], bk[IV_CH];
#pragma unroll
      for (int u = 0; u < IV_CH; ++u) {
        const int k = kb + u;
        ck[u] = k < n - 1 ? e[k] : 0.0;
        dk1[u] = k < n - 1 ? d[k + 1] : 0.0;
        bk[u] = k + 1 < n - 1 ? e[k + 1] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < IV_CH; ++u) {
        const int k = kb + u;
        if (k >= n - 1) break;
        const double ak1 = dk1[u] - lam;
        double u0, u1, u2, l, pn, qn, r0;
        uint8_t sw;
        // one FP64 division per row (FP64 is the scarce pipe): l from the
        // pivot's reciprocal, and U is stored with 1/u0 so that the U solves
        // multiply
        if (fabs(p) >= fabs(ck[u])) {
          r0 = (p == 0.0) ? 0.0 : 1.0 / p;
          l = ck[u] * r0;
          u0 = p;
          u1 = qv;
          u2 = 0.0;
          pn = ak1 - l * qv;
          qn = bk[u];
          sw = 0;
        } else {
          r0 = 1.0 / ck[u];
          l = p * r0;
          u0 = ck[u];
          u1 = ak1;
          u2 = bk[u];
          pn = qv - l * ak1;
          qn = -l * bk[u];
          sw = 1;
        }
        SU0(k) = (fabs(u0) < pivtol) ? 1.0 / copysign(pivtol, u0) : r0;  // 1 / guarded pivot
        SU1(k) = u1;
        SU2(k) = u2;
        SL(k) = l;
        PIV(k) = sw;
        p = pn;
        qv = qn;
      }
    }
    SU0(n - 1) = 1.0 / ((fabs(p) < pivtol) ? copysign(pivtol, p) : p);
    SU1(n - 1) = 0.0;
    SU2(n - 1) = 0.0;
    // ---- deterministic start vector in (-1, 1)
    // seeded by the eigenvalue index only: results do not depend on the batch slot
    const uint32_t seed = hash32((uint32_t)j * 2654435761u ^ 0x9e3779b9u);
    for (int k = 0; k < n; ++k) {
      const uint32_t h = hash32(seed + (uint32_t)k * 0x85ebca6bu);
      XS(k) = ((double)(h >> 8) * (1.0 / 16777216.0)) * 2.0 - 1.0;
    }
    bool ok = true;
    for (int it = 0; it < iters && ok; ++it) {
      // L solve with the recorded interchanges (x(k+1) of a chunk is read
      // before x(k) is overwritten, as in the row-by-row loop)
      double xk = XS(0);
      for (int kb = 0; kb < n - 1; kb += IV_CH) {
        double x1[IV_CH], l[IV_CH];
        uint8_t pv[IV_CH];
#pragma unroll
        for (int u = 0; u < IV_CH; ++u) {
          const int k = kb + u;
          const bool in = k < n - 1;
          x1[u] = in ? XS(k + 1) : 0.0;
          l[u] = in ? SL(k) : 0.0;
          pv[u] = in ? PIV(k) : (uint8_t)0;
        }
#pragma unroll
        for (int u = 0; u < IV_CH; ++u) {
          const int k = kb + u;
          if (k >= n - 1) break;
          if (pv[u]) {
            XS(k) = x1[u];
            xk = xk - l[u] * x1[u];
          } else {
            XS(k) = xk;
            xk = x1[u] - l[u] * xk;
          }
        }
      }
      XS(n - 1) = xk;
      // U solve
      double y1 = 0.0, y2 = 0.0, amax = 0.0;
      for (int kt = n - 1; kt >= 0; kt -= IV_CH) {
        double xv[IV_CH], a0[IV_CH], a1[IV_CH], a2[IV_CH];
#pragma unroll
        for (int u = 0; u < IV_CH; ++u) {
          const int k = kt - u;
          const bool in = k >= 0;
          xv[u] = in ? XS(k) : 0.0;
          a0[u] = in ? SU0(k) : 0.0;
          a1[u] = in ? SU1(k) : 0.0;
          a2[u] = in ? SU2(k) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < IV_CH; ++u) {
          const int k = kt - u;
          if (k < 0) break;
          const double y = (xv[u] - a1[u] * y1 - a2[u] * y2) * a0[u];
          XS(k) = y;
          amax = fmax(amax, fabs(y));
          y2 = y1;
          y1 = y;
        }
      }
      if (!(amax > 0.0) || !isfinite(amax)) {
        ok = false;
        break;
      }
      const double inv = 1.0 / amax;
      // modified Gram-Schmidt against the earlier members of the cluster
      for (int pass = 0; pass < 2 && j > j0; ++pass) {
        for (int jp = j0; jp < j; ++jp) {
          double dot = 0.0;
          for (int kb = 0; kb < n; kb += IV_CH) {
            double ev[IV_CH], xv[IV_CH];
#pragma unroll
            for (int u = 0; u < IV_CH; ++u) {
              const int k = kb + u;
              const bool in = k < n;
              ev[u] = in ? RT<R>::to(E[k + lde * jp].re) : 0.0;
              xv[u] = in ? XS(k) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < IV_CH; ++u)
              if (kb + u < n) dot += ev[u] * xv[u];
          }
          for (int kb = 0; kb < n; kb += IV_CH) {
            double ev[IV_CH], xv[IV_CH];
#pragma unroll
            for (int u = 0; u < IV_CH; ++u) {
              const int k = kb + u;
              const bool in = k < n;
              ev[u] = in ? RT<R>::to(E[k + lde * jp].re) : 0.0;
              xv[u] = in ? XS(k) : 0.0;
            }
#pragma unroll
            for (int u = 0; u < IV_CH; ++u)
              if (kb + u < n) XS(kb + u) = xv[u] - dot * ev[u];
          }
        }
      }
      double nrm2 = 0.0;
      for (int kb = 0; kb < n; kb += IV_CH) {
        double xv[IV_CH];
#pragma unroll
        for (int u = 0; u < IV_CH; ++u) xv[u] = kb + u < n ? XS(kb + u) : 0.0;
#pragma unroll
        for (int u = 0; u < IV_CH; ++u) {
          if (kb + u < n) {
            const double v = xv[u] * inv;
            nrm2 += v * v;
          }
        }
      }
      if (!(nrm2 > 1e-280)) {
        ok = false;
        break;
      }
      const double sc = inv / sqrt(nrm2);
      for (int kb = 0; kb < n; kb += IV_CH) {
        double xv[IV_CH];
#pragma unroll
        for (int u = 0; u < IV_CH; ++u) xv[u] = kb + u < n ? XS(kb + u) : 0.0;
#pragma unroll
        for (int u = 0; u < IV_CH; ++u)
          if (kb + u < n) XS(kb + u) = xv[u] * sc;
      }
    }
    if (!ok) bad = 1;
    // sign convention of dstein: the largest component is positive
    double big = -1.0;
    int kbig = 0;
    for (int kb = 0; kb < n; kb += IV_CH) {
      double xv[IV_CH];
#pragma unroll
      for (int u = 0; u < IV_CH; ++u) xv[u] = kb + u < n ? XS(kb + u) : 0.0;
#pragma unroll
      for (int u = 0; u < IV_CH; ++u) {
        const double v = fabs(xv[u]);
        if (kb + u < n && v > big) {
          big = v;
          kbig = kb + u;
        }
      }
    }
    const double sgn = XS(kbig) < 0.0 ? -1.0 : 1.0;
    for (int kb = 0; kb < n; kb += IV_CH) {
      double xv[IV_CH];
#pragma unroll
      for (int u = 0; u < IV_CH; ++u) xv[u] = kb + u < n ? XS(kb + u) : 0.0;
#pragma unroll
      for (int u = 0; u < IV_CH; ++u)
        if (kb + u < n) E[kb + u + lde * j] = cfrom64<R>(xv[u] * sgn, 0.0);
    }
  }
  if (bad) atomicOr((unsigned long long *)&info[b], (unsigned long long)PP_INFO_NOORTH);
#undef SU0
#undef SU1
#undef SU2
#undef SL
#undef XS
#undef PIV
}

template <class R>
cudaError_t tridiag_eigenvectors(EigWork &w, cudaStream_t s) {
  const int64_t sd = w.nmax;
  const int64_t scl = w.nmax + 1;
  k_clusters<<<w.B, 32, 0, s>>>(w.w, sd, w.rng, w.tinfo, w.cls, scl, w.ncl, 1e-7);
  count_launch(1);
  const int64_t T = w.scratch_threads;
  const int64_t sS = (int64_t)IV_F * w.nmax * T;
  const int64_t sPv = (int64_t)w.nmax * T;
  for (int64_t cb = 0; cb < w.mcap; cb += T) {
    dim3 g(cdiv(T, 64), w.B);
    PP_KT(KT_INVIT, s, (k_invit<R><<<g, 64, 0, s>>>(w.d, w.e, sd, w.nvec, w.w, w.rng, w.tinfo, w.cls, scl, w.ncl,
                                                    (int)cb, (C<R> *)w.E, w.lde, w.sE, w.scratch, w.piv, T, sS, sPv,
                                                    w.info)));
    count_launch(1);
  }
  k_clusters<<<w.B, 32, 0, s>>>(w.w, sd, w.rng, w.tinfo, w.cls, scl, w.ncl, 1e-5);
  PP_KT(KT_INVIT, s, (k_reorth<R><<<dim3(RO_BLOCKS, w.B), 256, 0, s>>>((C<R> *)w.E, w.lde, w.sE, w.nvec, w.cls, scl, w.ncl)));
  count_launch(2);
  return cudaGetLastError();
}

// ===========================================================================
// Stage 4: back-transform E = Q Z
// ===========================================================================
constexpr int BT_J = 64;     // columns per block
constexpr int BT_RK = 16;    // rows per k-step
constexpr int BT_RCH = 512;  // rows per split-K chunk

// Wp[ks][a][j] = sum_{r in chunk ks} conj(V(r,a)) X(r,j) for a < jb.
// V(r,a) = A(r, k0+a) for r >= k0+a+1 (zero above); j < the matrix's m, or
// ncol_fixed.
template <class R>
__global__ void __launch_bounds__(256) k_vhx(const C<R> *Ab, int64_t lda, int64_t sA, const C<R> *Xb, int64_t ldx,
                                             int64_t sX, const int *nvec, const int64_t *rng, int k0, int jb,
                                             C<R> *Wp, int64_t ldwp, int64_t sWp, int ncol_fixed, int rch) {
  __shared__ C<R> sV[BT_RK][32];
  __shared__ C<R> sXt[BT_RK][BT_J];
  const int b = blockIdx.z;
  const int n = nvec[b];
  const int ncol = ncol_fixed > 0 ? ncol_fixed : (int)rng[b * 8 + 2];
  const int j0 = blockIdx.x * BT_J;
  const int ks = blockIdx.y;
  const int rbeg = k0 + 1 + ks * rch;
  if (j0 >= ncol || rbeg >= n) return;
  const C<R> *A = Ab + b * sA;
  const C<R> *X = Xb + b * sX;
  const int64_t ldX = ldx;
  const int tj = threadIdx.x & 63, ta = threadIdx.x >> 6;
  C<R> acc[8];
#pragma unroll
  for (int p = 0; p < 8; ++p) acc[p] = cz<R>();
  const int rend = min(n, rbeg + rch);
  for (int r0 = rbeg; r0 < rend; r0 += BT_RK) {
    for (int e = threadIdx.x; e < BT_RK * 32; e += 256) {
      const int a = e & 31, rr = e >> 5;
      const int r = r0 + rr;
      sV[rr][a] = (a < jb && r < rend && r >= k0 + a + 1) ? cconj(A[r + lda * (k0 + a)]) : cz<R>();
    }
    for (int e = threadIdx.x; e < BT_RK * BT_J; e += 256) {
      const int jx = e & 63, rr = e >> 6;
      const int r = r0 + rr, j = j0 + jx;
      const bool ok = r < rend && j < ncol;
      sXt[rr][jx] = ok ? X[r + ldX * j] : cz<R>();
    }
    __syncthreads();
#pragma unroll 4
    for (int rr = 0; rr < BT_RK; ++rr) {
      const C<R> xv = sXt[rr][tj];
#pragma unroll
      for (int p = 0; p < 8; ++p) cmac(acc[p], sV[rr][ta + 4 * p], xv);
    }
    __syncthreads();
  }
  const int j = j0 + tj;
  if (j < ncol) {
#pragma unroll
    for (int p = 0; p < 8; ++p) {
      const int a = ta + 4 * p;
      if (a < jb) Wp[b * sWp + ((int64_t)ks * 32 + a) * ldwp + j] = cfin(acc[p]);
    }
  }
}

// Sum the split-K partials of V^H X and apply the panel's compact-WY factor
// (Tf at Tf + 1024 b, upper triangular): mode 1 Y = Tf (V^H X), mode 2
// Y = Tf^H (V^H X); written to Wb.
// Block of BR_NT threads = 32 columns j x 8 groups of panel rows a (a = g,
// g + 8, g + 16, g + 24): the partials are summed into shared memory, then
// every thread forms its four rows of the product with Tf.
constexpr int BR_NT = 256;
template <class R>
__global__ void __launch_bounds__(BR_NT) k_btred(const C<R> *Wp, int64_t ldwp, int64_t sWp, const int *nvec,
                                                 const int64_t *rng, int k0, int jb, int mode, const z64 *Tf,
                                                 C<R> *Wb, int64_t sWb, int ncol_fixed, int nks_fixed = 0) {
  __shared__ C<R> col[32][33];
  __shared__ z64 sT[32][33];
  const int b = blockIdx.y;
  const int n = nvec[b];
  const int ncol = ncol_fixed > 0 ? ncol_fixed : (int)rng[b * 8 + 2];
  // split-K partials to sum: one per BT_RCH rows, or nks_fixed
  const int nks = nks_fixed > 0 ? (n - k0 - 1 > 0 ? nks_fixed : 0) : (n - k0 - 1 + BT_RCH - 1) / BT_RCH;
  const int j0 = blockIdx.x * 32;
  if (j0 >= ncol || nks <= 0) return;
  for (int e = threadIdx.x; e < 32 * 32; e += BR_NT) sT[e / 32][e % 32] = Tf[b * 1024 + e];
  const int jl = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int j = j0 + jl;
  for (int a = g; a < jb; a += 8) {
    C<R> s = cz<R>();
    if (j < ncol)
      for (int ks = 0; ks < nks; ++ks) s = cadd(s, Wp[b * sWp + ((int64_t)ks * 32 + a) * ldwp + j]);
    col[a][jl] = s;
  }
  __syncthreads();
  if (j >= ncol) return;
  for (int a = g; a < jb; a += 8) {
    C<R> acc = cz<R>();
    if (mode == 1) {
      for (int a2 = a; a2 < jb; ++a2) cmac(acc, cfrom64<R>(sT[a][a2]), col[a2][jl]);
    } else {  // mode 2: Tf^H (lower triangular)
      for (int a2 = 0; a2 <= a; ++a2) cmac(acc, cfrom64<R>(zconj(sT[a2][a])), col[a2][jl]);
    }
    Wb[b * sWb + (int64_t)a * ldwp + j] = cfin(acc);
  }
}

// Compact-WY factors of every panel in one launch, one block per (panel,
// matrix): the Gram matrix G = V^H V of the panel's Householder vectors
// (products in the arithmetic R, rows staged WY_RK at a time and the sums
// renormalised after each stage, each thread four entries), then Tf by
// zlarft's forward columnwise recurrence in FP64: Tf(a,a) = tau_a,
// Tf(0:a, a) = -tau_a Tf(0:a, 0:a) G(0:a, a).  Tf of panel P for matrix b
// goes to Tf + P sTfp + 1024 b (row-major 32 x 32).  Panel widths follow the
// batch's largest order (nref = nmax - 1); reflectors past a matrix's own
// order have tau = 0 and give zero columns of Tf.
constexpr int WY_RK = 16;
template <class R>
__global__ void __launch_bounds__(256) k_wy_factors(const C<R> *Ab, int64_t lda, int64_t sA, const int *nvec,
                                                     const z64 *tau, int64_t sd, int nb, int nref, z64 *Tf,
                                                     int64_t sTfp) {
  __shared__ C<R> sV[WY_RK][33];
  __shared__ z64 G[32][33];
  __shared__ z64 sT[32][33];
  const int P = blockIdx.x, b = blockIdx.y;
  const int n = nvec[b];
  const int k0 = P * nb;
  const int jb = min(nb, nref - k0);
  const C<R> *A = Ab + b * sA;
  const int tid = threadIdx.x;
  const int ga = tid >> 3, gj = (tid & 7) * 4;  // G(ga, gj .. gj+3)
  C<R> acc[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) acc[q] = cz<R>();
  for (int r0 = k0 + 1; r0 < n; r0 += WY_RK) {
    for (int e = tid; e < WY_RK * 32; e += 256) {
      const int a = e & 31, rr = e >> 5, r = r0 + rr;
      sV[rr][a] = (a < jb && r < n && r >= k0 + a + 1) ? A[r + lda * (k0 + a)] : cz<R>();
    }
    __syncthreads();
#pragma unroll 4
    for (int rr = 0; rr < WY_RK; ++rr) {
      const C<R> va = sV[rr][ga];
#pragma unroll
      for (int q = 0; q < 4; ++q) cmacc(acc[q], va, sV[rr][gj + q]);
    }
    // renormalise after every WY_RK rows: the unnormalised low word of the
    // multiply-add is meant for short sums, the panel runs over all n rows
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[q] = cfin(acc[q]);
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) G[ga][gj + q] = cto64(cfin(acc[q]));
  for (int e = tid; e < 1024; e += 256) sT[e / 32][e % 32] = z64{0.0, 0.0};
  __syncthreads();
  if (tid < 32) {
    const int a = tid;
    for (int jj = 0; jj < jb; ++jj) {
      const int i = k0 + jj;
      const z64 tj = (i < n - 1) ? tau[b * sd + i] : z64{0.0, 0.0};
      z64 acc2{0.0, 0.0};
      for (int a2 = a; a2 < jj; ++a2) {
        const z64 g = G[a2][jj];
        const z64 tt = sT[a][a2];
        acc2.re += tt.re * g.re - tt.im * g.im;
        acc2.im += tt.re * g.im + tt.im * g.re;
      }
      __syncwarp();
      if (a < jj) {
        const z64 v = zmul(tj, acc2);
        sT[a][jj] = z64{-v.re, -v.im};
      }
      if (a == jj) sT[jj][jj] = tj;
      __syncwarp();
    }
  }
  __syncthreads();
  z64 *T = Tf + (int64_t)P * sTfp + (int64_t)b * 1024;
  for (int e = tid; e < 1024; e += 256) T[e] = sT[e / 32][e % 32];
}

// E(r, j) -= sum_a V(r, a) Y(a, j), r in [k0+1, n), j < m.
constexpr int AV_T = 64, AV_K = 16;
template <class R>
__global__ void __launch_bounds__(256) k_applyV(const C<R> *Ab, int64_t lda, int64_t sA, const C<R> *Wb,
                                                int64_t ldwp, int64_t sWb, C<R> *Eb, int64_t lde, int64_t sE,
                                                const int *nvec, const int64_t *rng, int k0, int jb, int ncol_fixed) {
  __shared__ C<R> sV[AV_K][AV_T];
  __shared__ C<R> sY[AV_K][AV_T];
  const int b = blockIdx.z;
  const int n = nvec[b];
  const int m = ncol_fixed > 0 ? ncol_fixed : (int)rng[b * 8 + 2];
  const int r0 = k0 + 1 + blockIdx.x * AV_T, c0 = blockIdx.y * AV_T;
  if (r0 >= n || c0 >= m) return;
  const C<R> *A = Ab + b * sA;
  const C<R> *Y = Wb + b * sWb;
  C<R> *E = Eb + b * sE;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  C<R> acc[4][4];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = cz<R>();
  for (int kc = 0; kc < jb; kc += AV_K) {
    for (int e = threadIdx.x; e < AV_K * AV_T; e += 256) {
      const int x = e % AV_T, y = e / AV_T;
      const int a = kc + y;
      const int r = r0 + x, c = c0 + x;
      sV[y][x] = (a < jb && r < n && r >= k0 + a + 1) ? A[r + lda * (k0 + a)] : cz<R>();
      sY[y][x] = (a < jb && c < m) ? Y[(int64_t)a * ldwp + c] : cz<R>();
    }
    __syncthreads();
#pragma unroll 4
    for (int k = 0; k < AV_K; ++k) {
      C<R> v[4], y[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        v[p] = sV[k][tx + 16 * p];
        y[p] = sY[k][ty + 16 * p];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) cmac(acc[p][q], v[p], y[q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int r = r0 + tx + 16 * p, c = c0 + ty + 16 * q;
      if (r < n && c < m) {
        C<R> *x = &E[r + lde * c];
        *x = csub(*x, cfin(acc[p][q]));
      }
    }
}

template <class R>
cudaError_t back_transform(EigWork &w, cudaStream_t s) {
  const int B = w.B, nmax = w.nmax, nb = w.nb;
  if (nmax < 2) return cudaSuccess;
  const int nref = nmax - 1;  // reflector columns 0 .. nmax-2
  const int64_t ldwp = w.ldwp;
  const int64_t sWp = (int64_t)w.ksplit * 32 * ldwp;
  const int64_t sWb = (int64_t)32 * ldwp;
  const int64_t sd = w.nmax;
  C<R> *A = (C<R> *)w.A;
  C<R> *E = (C<R> *)w.E;
  C<R> *Wp = (C<R> *)w.Wp;
  C<R> *Wb = (C<R> *)w.Wb;
  // compact-WY factors of all panels
  PP_KT(KT_BTRED, s, (k_wy_factors<R><<<dim3(cdiv(nref, nb), B), 256, 0, s>>>(A, w.lda, w.sA, w.nvec, w.tau, sd, nb,
                                                                           nref, w.Tf, w.sTfp)));
  count_launch(1);
  const int kstart = ((nref - 1) / nb) * nb;
  for (int k0 = kstart; k0 >= 0; k0 -= nb) {
    const int jb = min(nb, nref - k0);
    const int ks = cdiv(nmax - k0 - 1, BT_RCH);
    const z64 *Tf = w.Tf + (int64_t)(k0 / nb) * w.sTfp;
    // Y = Tf V^H E ; E -= V Y (on the tensor cores in the double-float form,
    // over all mcap columns)
    const bool tc = std::is_same<R, df>::value && w.tcS && tc_enabled();
    if (tc) {
      PP_CUDA_TRY(vhx_tc(w, k0, jb, (const zdf *)E, w.lde, w.sE, w.mcap, (zdf *)Wp, ldwp, sWp, s));
      PP_KT(KT_BTRED, s, (k_btred<R><<<dim3(cdiv(w.mcap, 32), B), BR_NT, 0, s>>>(Wp, ldwp, sWp, w.nvec, w.rng, k0, jb, 1, Tf, Wb, sWb, w.mcap, vhx_tc_splits(w))));
      PP_CUDA_TRY(applyV_tc(w, k0, jb, (zdf *)E, w.lde, w.sE, (const zdf *)Wb, ldwp, sWb, w.mcap, s));
      count_launch(1);
    } else {
      PP_KT(KT_VHX, s, (k_vhx<R><<<dim3(cdiv(w.mcap, BT_J), ks, B), 256, 0, s>>>(A, w.lda, w.sA, E, w.lde, w.sE, w.nvec, w.rng, k0,
                                                               jb, Wp, ldwp, sWp, 0, BT_RCH)));
      PP_KT(KT_BTRED, s, (k_btred<R><<<dim3(cdiv(w.mcap, 32), B), BR_NT, 0, s>>>(Wp, ldwp, sWp, w.nvec, w.rng, k0, jb, 1, Tf, Wb, sWb, 0)));
      PP_KT(KT_APPLYV, s, (k_applyV<R><<<dim3(cdiv(nmax - k0 - 1, AV_T), cdiv(w.mcap, AV_T), B), 256, 0, s>>>(
          A, w.lda, w.sA, Wb, ldwp, sWb, E, w.lde, w.sE, w.nvec, w.rng, k0, jb, 0)));
      count_launch(3);
    }
  }
  return cudaGetLastError();
}

// X = P^T (unit columns at the selected rows)
template <class R>
__global__ void k_rows_init(C<R> *Xb, int64_t ldx, int64_t sX, const int *rows, int nrows, const int *nvec) {
  const int b = blockIdx.z;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int k = blockIdx.y;
  if (r >= nvec[b] || k >= nrows) return;
  Xb[b * sX + r + ldx * k] = (r == rows[k]) ? cfrom64<R>(1.0, 0.0) : cz<R>();
}

// Eb(k, j) = sum_r conj(X(r,k)) Z(r,j), Z real (stored as complex with zero
// imaginary part): the selected rows of E = Q Z.
constexpr int XZ_T = 64, XZ_K = 16;
template <class R>
__global__ void __launch_bounds__(256) k_xhz(const C<R> *Xb, int64_t ldx, int64_t sX, const C<R> *Zb, int64_t ldz,
                                             int64_t sZ, C<R> *Eb, int64_t lde, int64_t sE, const int *nvec,
                                             const int64_t *rng, int nrows) {
  __shared__ C<R> sXt[XZ_K][XZ_T];
  __shared__ R sZt[XZ_K][XZ_T];
  const int b = blockIdx.z;
  const int n = nvec[b];
  const int m = (int)rng[b * 8 + 2];
  const int k0 = blockIdx.x * XZ_T, j0 = blockIdx.y * XZ_T;
  if (k0 >= nrows || j0 >= m) return;
  const C<R> *X = Xb + b * sX;
  const C<R> *Z = Zb + b * sZ;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  C<R> acc[4][4];
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[p][q] = cz<R>();
  for (int r0 = 0; r0 < n; r0 += XZ_K) {
    for (int e = threadIdx.x; e < XZ_K * XZ_T; e += 256) {
      const int x = e % XZ_T, y = e / XZ_T;
      const int r = r0 + y;
      sXt[y][x] = (r < n && k0 + x < nrows) ? cconj(X[r + ldx * (k0 + x)]) : cz<R>();
      sZt[y][x] = (r < n && j0 + x < m) ? Z[r + ldz * (j0 + x)].re : RT<R>::zero();
    }
    __syncthreads();
#pragma unroll 4
    for (int y = 0; y < XZ_K; ++y) {
      C<R> xv[4];
      R zv[4];
#pragma unroll
      for (int p = 0; p < 4; ++p) {
        xv[p] = sXt[y][tx + 16 * p];
        zv[p] = sZt[y][ty + 16 * p];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          RT<R>::mac(acc[p][q].re, xv[p].re, zv[q]);
          RT<R>::mac(acc[p][q].im, xv[p].im, zv[q]);
        }
    }
    __syncthreads();
  }
  C<R> *E = Eb + b * sE;
#pragma unroll
  for (int p = 0; p < 4; ++p)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int k = k0 + tx + 16 * p, j = j0 + ty + 16 * q;
      if (k < nrows && j < m) E[k + lde * j] = cfin(acc[p][q]);
    }
}

template <class R>
cudaError_t back_transform_rows(EigWork &w, const int *d_rows, int nrows, cudaStream_t s) {
  const int B = w.B, nmax = w.nmax, nb = w.nb;
  if (nrows <= 0) return cudaSuccess;
  const int64_t ldx = w.lda, sX = (int64_t)w.lda * w.nbr;
  C<R> *A = (C<R> *)w.A;
  C<R> *X = (C<R> *)w.Xr;
  C<R> *Wp = (C<R> *)w.Wp;
  C<R> *Wb = (C<R> *)w.Wb;
  const int64_t ldwp = w.ldwp;
  const int64_t sWp = (int64_t)w.ksplit * 32 * ldwp;
  const int64_t sWb = (int64_t)32 * ldwp;
  const int64_t sd = w.nmax;
  k_rows_init<R><<<dim3(cdiv(nmax, 256), nrows, B), 256, 0, s>>>(X, ldx, sX, d_rows, nrows, w.nvec);
  count_launch(1);
  // X <- Q^H X = Q_last^H ... Q_0^H X: panels in forward order, Tf^H
  const int nref = nmax - 1;
  PP_KT(KT_BTRED, s, (k_wy_factors<R><<<dim3(cdiv(nref, nb), B), 256, 0, s>>>(A, w.lda, w.sA, w.nvec, w.tau, sd, nb,
                                                                           nref, w.Tf, w.sTfp)));
  count_launch(1);
  for (int k0 = 0; k0 < nref; k0 += nb) {
    const int jb = min(nb, nref - k0);
    const int ks = cdiv(nmax - k0 - 1, BT_RCH);
    const z64 *Tf = w.Tf + (int64_t)(k0 / nb) * w.sTfp;
    const bool tc = std::is_same<R, df>::value && w.tcS && tc_enabled();
    if (tc) {
      PP_CUDA_TRY(vhx_tc(w, k0, jb, (const zdf *)X, ldx, sX, nrows, (zdf *)Wp, ldwp, sWp, s));
    } else {
      PP_KT(KT_VHX, s, (k_vhx<R><<<dim3(cdiv(nrows, BT_J), ks, B), 256, 0, s>>>(A, w.lda, w.sA, X, ldx, sX, w.nvec,
                                                                               w.rng, k0, jb, Wp, ldwp, sWp, nrows,
                                                                               BT_RCH)));
    }
    PP_KT(KT_BTRED, s, (k_btred<R><<<dim3(cdiv(nrows, 32), B), BR_NT, 0, s>>>(Wp, ldwp, sWp, w.nvec, w.rng, k0, jb, 2,
                                                                          Tf, Wb, sWb, nrows,
                                                                          tc ? vhx_tc_splits(w) : 0)));
    if (tc) {
      PP_CUDA_TRY(applyV_tc(w, k0, jb, (zdf *)X, ldx, sX, (const zdf *)Wb, ldwp, sWb, nrows, s));
    } else {
      PP_KT(KT_APPLYV, s, (k_applyV<R><<<dim3(cdiv(nmax - k0 - 1, AV_T), cdiv(nrows, AV_T), B), 256, 0, s>>>(
                              A, w.lda, w.sA, Wb, ldwp, sWb, X, ldx, sX, w.nvec, w.rng, k0, jb, nrows)));
    }
    count_launch(tc ? 1 : 3);  // the tensor-core helpers count their own launches
  }
  // Eb = X^H Z
  if (std::is_same<R, df>::value && w.tcS && tc_enabled()) {
    PP_CUDA_TRY(xhz_tc(w, (const zdf *)X, ldx, sX, nrows, (const zdf *)w.E, w.lde, w.sE, (zdf *)w.Eb,
                       (int64_t)w.nbr, (int64_t)w.nbr * w.mcap, s));
  } else {
    PP_KT(KT_XHZ, s, (k_xhz<R><<<dim3(cdiv(nrows, XZ_T), cdiv(w.mcap, XZ_T), B), 256, 0, s>>>(
                         X, ldx, sX, (const C<R> *)w.E, w.lde, w.sE, (C<R> *)w.Eb, (int64_t)w.nbr,
                         (int64_t)w.nbr * w.mcap, w.nvec, w.rng, nrows)));
    count_launch(1);
  }
  return cudaGetLastError();
}

// explicit instantiations
template cudaError_t tridiagonalize<double>(EigWork &, cudaStream_t);
template cudaError_t tridiagonalize<df>(EigWork &, cudaStream_t);
template cudaError_t tridiag_eigenvectors<double>(EigWork &, cudaStream_t);
template cudaError_t tridiag_eigenvectors<df>(EigWork &, cudaStream_t);
template cudaError_t back_transform<double>(EigWork &, cudaStream_t);
template cudaError_t back_transform<df>(EigWork &, cudaStream_t);
template cudaError_t back_transform_rows<double>(EigWork &, const int *, int, cudaStream_t);
template cudaError_t back_transform_rows<df>(EigWork &, const int *, int, cudaStream_t);

}  // namespace pp
