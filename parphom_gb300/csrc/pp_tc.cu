// Trailing update of the double-float reduction on the tensor cores.
//
// A(k1:n, k1:n) -= V W^H + W V^H (lower triangle) with V, W the n x jb
// panel (zlatrd, jb <= 32) in double-float, as two products X Y^H (X = V,
// Y = W, then X = W, Y = V).  Per row r each operand's 64 reals
//   [Re X(r, 0..31), Im X(r, 0..31)]
// are cut into 7 bf16 slices on a fixed-point grid set by that row's largest
// magnitude 2^E (an Ozaki-style error-free split):
//   X_r = 2^E sum_{s=0..6} 2^-8(s+1) m_s,  m_s integers, |m_0| <= 256,
//   |m_s| <= 129 for s > 0,  residual below 2^(E - 57).
// Every slice product is an integer below 2^16 and K = 64, so each sum of
// products with the same s + t (at most 2^24 in magnitude) is exact in the
// FP32 accumulation of the tensor cores.  With
//   Re(X_r Y_c^*) = ReX.ReY + ImX.ImY,   Im(X_r Y_c^*) = ImX.ReY - ReX.ImY,
// the real part pairs k-step j of the row operand with k-step j of the
// column operand and the imaginary part with k-step j ^ 2 (negated for the
// Re X half, by the instruction's negate-B bit).  The 28 slice pairs with
// s + t <= 6 go into 7 accumulators per real/imaginary part (14 x 32 TMEM
// columns); the epilogue sums them in double-float, scales by
// 2^(E_r + E_c - 16) and subtracts from A.  Separate grids for V and W keep
// both at full relative resolution; the dropped pairs and the residual bound
// the error by about 2^-55 |X_r| |Y_c| per product, the double-float level.
//
// CTA (512 threads) = 128 rows x (up to 8) column blocks of 32, both
// products in turn.  The 112 KB row operand stays in shared memory while the
// 28 KB column operands are streamed in by bulk copies, double-buffered so
// that the next block's copy overlaps this block's MMAs.  One CTA per SM
// (168 KB of shared memory, 448 tensor-memory columns).
#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <cstdlib>
#include <mutex>
#include <cuda_bf16.h>

#include "pp_internal.cuh"
#include "pp_tc.cuh"

namespace pp {

namespace {

constexpr int TC_S = 7;                          // slices
constexpr int TC_KS = 4;                         // k-steps of 16 (K = 64 reals)
constexpr int TC_TILE = 4096;                    // one (slice, k-step) tile of 128 rows
constexpr int TC_OP = TC_S * TC_KS * TC_TILE;    // one operand of a 128-row block (114688)
constexpr int TC_RBLK = 2 * TC_OP;               // V and W operands of a 128-row block
constexpr int TC_BBYTES = TC_S * TC_KS * 1024;   // one 32-row column block of one operand (28672)
constexpr int TC_CB = 8;                         // column blocks per CTA
constexpr int TC_NT = 512;                       // threads: 16 warps = 4 lane groups x 4 column quarters
constexpr int TC_CQ = 32 / (TC_NT / 128);        // columns per thread in the epilogue (8)
constexpr int TC_SMEM = TC_OP + 2 * TC_BBYTES + 2 * 256 + 64;  // + 2 x 32 exponent pairs, mbarriers, TMEM slot
constexpr int TC_NACC = 2 * TC_S;                // accumulators: (re, im) x slice-sum group
constexpr uint32_t TC_ID = tc::idesc_bf16(128, 32, 0);
constexpr uint32_t TC_IDN = tc::idesc_bf16(128, 32, 1);
static_assert(TC_NACC * 32 <= 512, "accumulators exceed tensor memory");
static_assert(TC_NT == 4 * 128, "long-K slicing maps one thread to each (row, k-step) of 128 rows");

// 2^e as a float (exact for -126 <= e <= 127)
__device__ __forceinline__ float pow2f(int e) {
  return (e >= -126 && e <= 127) ? __int_as_float((e + 127) << 23) : ldexpf(1.0f, e);
}

// Slices of one operand row held by a warp: lane a has the complex value of
// panel column a; K index a (real part) and 32 + a (imaginary part).
template <int TILE = TC_TILE>
__device__ __forceinline__ int slice_row(zdf x, uint8_t *blk, int row, int lane) {
  float amax = fmaxf(fabsf(x.re.hi), fabsf(x.im.hi));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
  int E = 0;
  if (amax > 0.f) frexpf(amax, &E);  // amax < 2^E, so |x| < 2^E
#pragma unroll
  for (int part = 0; part < 2; ++part) {
    const df v = part ? x.im : x.re;
    const int kk = lane + 32 * part;
    float th = ldexpf(v.hi, -E), tl = ldexpf(v.lo, -E);
    uint8_t *base = blk + (kk >> 4) * TILE + tc::core_off(row, kk & 15);
#pragma unroll
    for (int s = 0; s < TC_S; ++s) {
      th = __fmul_rn(th, 256.f);
      tl = __fmul_rn(tl, 256.f);
      const float mi = rintf(th);
      two_sum(__fsub_rn(th, mi), tl, th, tl);
      *(__nv_bfloat16 *)(base + s * TC_KS * TILE) = __float2bfloat16_rn(mi);
    }
  }
  return E;
}

// Source rows of one operand: element (row, a) of matrix b is
// P[b * sP + (rbase + row) * rs + a * cs] (conjugated when conj), zero for
// a >= min(jb, n_b - 1 - k0) and, with vmask, for rbase + row < k0 + a + 1
// (the zero part of a Householder panel).  Rows 0 .. nrows_b - 1 exist, with
// nrows_b = n_b - rbase (nrows_fixed == 0) or nrows_fixed.
struct TcSliceSrc {
  const zdf *P;
  int64_t sP, rs, cs;
  int rbase, nrows_fixed, vmask, conj;
};

// Slices of rows 0 .. 128 ceil(nrows_b / 128) - 1 (rows past nrows_b are
// zero): one warp per row.  Row r of matrix b goes to block r / 128 of
// S + b sS (blocks blk bytes apart), its exponent to E[b sE + r es + eo].
__global__ void __launch_bounds__(128) k_tc_slices(TcSliceSrc src, const int *nvec, int k0, int jb, uint8_t *S,
                                                   int64_t sS, int64_t blk, int *E, int64_t sE, int es, int eo) {
  const int b = blockIdx.y;
  const int n = nvec[b];
  const int nrows = src.nrows_fixed > 0 ? src.nrows_fixed : n - src.rbase;
  if (nrows <= 0) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rl = blockIdx.x * 4 + warp;
  if (rl >= (nrows + 127) / 128 * 128) return;
  const int jmax = min(jb, n - 1 - k0);
  zdf v{{0.f, 0.f}, {0.f, 0.f}};
  if (rl < nrows && lane < jmax && (!src.vmask || src.rbase + rl >= k0 + lane + 1)) {
    v = src.P[b * src.sP + (int64_t)(src.rbase + rl) * src.rs + (int64_t)lane * src.cs];
    if (src.conj) v.im = df_neg(v.im);
  }
  uint8_t *blkp = S + b * sS + (int64_t)(rl >> 7) * blk;
  const int e = slice_row(v, blkp, rl & 127, lane);
  if (lane == 0) E[b * sE + (int64_t)rl * es + eo] = e;
}

__device__ __forceinline__ df df_add_f(df a, float b) {
  float s, e;
  two_sum(a.hi, b, s, e);
  e = __fadd_rn(e, a.lo);
  df r;
  fast_two_sum(s, e, r.hi, r.lo);
  return r;
}

// sum_u acc[u] 2^-8u in double-float.  acc[u] are integers below 2^24; the
// three smallest groups are summed in float (rounding error below 2^-32 of
// the unit of acc[0]), the rest with error-free additions.
__device__ __forceinline__ df combine7(const float *acc) {
  float t = __fmul_rn(acc[6], 0x1p-48f);
  t = __fmaf_rn(acc[5], 0x1p-40f, t);
  t = __fmaf_rn(acc[4], 0x1p-32f, t);
  df s{acc[0], 0.f};
  s = df_add_f(s, __fmul_rn(acc[1], 0x1p-8f));
  s = df_add_f(s, __fmul_rn(acc[2], 0x1p-16f));
  s = df_add_f(s, __fmul_rn(acc[3], 0x1p-24f));
  s = df_add_f(s, t);
  return s;
}

// MMAs of one column block: re acc pairs row k-step j with column k-step j,
// im acc with column k-step j ^ 2, negated for j < 2 (Re X . Im Y).  Fully
// unrolled: a descriptor differs from the block's first only in its start
// address (bits 0-13, in 16-byte units), so each MMA costs one add.
__device__ __forceinline__ void tc_issue(uint32_t tm, uint32_t sa, uint32_t sb) {
  const uint64_t a0 = tc::sdesc(sa, 128, 256), b0 = tc::sdesc(sb, 128, 256);
#pragma unroll
  for (int u = 0; u < TC_S; ++u) {
#pragma unroll
    for (int s = 0; s <= u; ++s) {
      const int t = u - s;
#pragma unroll
      for (int j = 0; j < TC_KS; ++j) {
        const uint32_t acc = (s == 0 && j == 0) ? 0u : 1u;
        const uint64_t ad = a0 + (uint64_t)((s * TC_KS + j) * (TC_TILE >> 4));
        const uint64_t br = b0 + (uint64_t)((t * TC_KS + j) * (1024 >> 4));
        const uint64_t bi = b0 + (uint64_t)((t * TC_KS + (j ^ 2)) * (1024 >> 4));
        tc::mma_bf16(tm + u * 32, ad, br, TC_ID, acc);
        tc::mma_bf16(tm + (TC_S + u) * 32, ad, bi, j < 2 ? TC_IDN : TC_ID, acc);
      }
    }
  }
}

// One operand of a product C -= X Y^H: slices in 128-row blocks of TC_OP
// bytes placed blk bytes apart (matrix b at S + b sS), and the exponent of
// row r at E[b sE + r es + eo].
struct TcOperand {
  const uint8_t *S;
  int64_t sS, blk;
  const int *E;
  int64_t sE;
  int es, eo;
};
// C(rbase + r, cbase + c) -= sum_p X_p(r, :) Y_p(c, :)^H over the tiles of
// 128 rows x 32 columns of rows [0, nrows_b) and columns [0, ncols_b): all of
// them, or (tri) the lower triangle of a square trailing block.
struct TcUpdate {
  zdf *C;
  int64_t ldc, sC;
  int rbase, cbase;
  int ncols_fixed;  // columns: ncols_fixed, or n_b - cbase when 0; rows: n_b - rbase
  int tri, nprod;
  TcOperand x[2], y[2];
  // test hook (pp_debug_stall_tc_wait): matrix stall_b's first CTA waits,
  // before its first row-operand wait, on an mbarrier that nothing arrives
  // on, for stall_cycles SM clocks, and so takes the time-out path; -1: off
  int stall_b;
  long long stall_cycles;
};

__global__ void __launch_bounds__(TC_NT, 1) k_cupd_tc(TcUpdate u, const int *nvec, int *err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t *sAop = smem;                                  // row operand
  uint8_t *sBop = smem + TC_OP;                          // two column-operand buffers
  int *sEc = (int *)(smem + TC_OP + 2 * TC_BBYTES);      // two x 64 column exponents
  // mbarriers: [0] row operand landed (waited by thread 0), [1], [2] column
  // buffer 0 / 1 landed, [3] MMAs of the block done, [4] never arrived on
  // (the test hook's wait).
  // Each barrier a thread waits on completes exactly once between two of
  // its waits, so parity waits cannot skip a phase.
  uint64_t *bars = (uint64_t *)(smem + TC_OP + 2 * TC_BBYTES + 512);
  uint32_t *tslot = (uint32_t *)(bars + 5);
  const int b = blockIdx.z, R = blockIdx.y, q = blockIdx.x;
  const int n = nvec[b];
  const int nrows = n - u.rbase;
  const int ncols = u.ncols_fixed > 0 ? u.ncols_fixed : n - u.cbase;
  if (nrows <= 0 || ncols <= 0) return;
  const int nrb = (nrows + 127) / 128, ncb = (ncols + 31) / 32;
  if (R >= nrb) return;
  const int cb_beg = q * TC_CB;
  int cb_end = min(cb_beg + TC_CB, ncb);
  if (u.tri) cb_end = min(cb_end, 4 * (R + 1));
  if (cb_beg >= cb_end) return;
  // an earlier wait of this matrix gave up: its results are already invalid
  if (*(volatile int *)&err[b]) return;
  const int ncbw = cb_end - cb_beg;
  const int nblk = u.nprod * ncbw;  // (product, column block) steps

  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) tc::tmem_alloc(tslot, 512);
  if (tid == 0) {
    for (int i = 0; i < 5; ++i) tc::mbar_init(&bars[i], 1);
    tc::mbar_init_fence();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tm = *tslot;
  const bool stall = b == u.stall_b && R == 0 && q == 0;
  zdf *C = u.C + b * u.sC;
  const int r0 = u.rbase + 128 * R;  // first global row of this row block
  const int nr = min(128, nrows - 128 * R);
  // column operand of step i (product i / ncbw, column block cb)
  auto issue_cols = [&](int i) {
    const TcOperand &y = u.y[i / ncbw];
    const int cb = cb_beg + i % ncbw;
    const int buf = i & 1;
    uint64_t *bar = &bars[1 + buf];
    const uint32_t ebytes = 32u * 4u * (uint32_t)y.es;
    tc::mbar_expect_tx(bar, TC_BBYTES + ebytes);
    const uint8_t *src = y.S + b * y.sS + (int64_t)(cb >> 2) * y.blk + (cb & 3) * 1024;
    uint8_t *dst = sBop + buf * TC_BBYTES;
    for (int sj = 0; sj < TC_S * TC_KS; ++sj) tc::bulk_g2s(dst + sj * 1024, src + sj * TC_TILE, 1024, bar);
    tc::bulk_g2s(sEc + buf * 64, y.E + b * y.sE + (int64_t)32 * cb * y.es, ebytes, bar);
  };
  const int lg = warp & 3, cqt = warp >> 2;
  const int rl = 128 * R + 32 * lg + (tid & 31);  // row within the block of rows = TMEM lane
  const int r = u.rbase + rl;
  int erow[2] = {0, 0};
  for (int p = 0; p < u.nprod; ++p) erow[p] = u.x[p].E[b * u.x[p].sE + (int64_t)rl * u.x[p].es + u.x[p].eo];
  const uint32_t lane_addr = tm + ((uint32_t)(32 * lg) << 16) + TC_CQ * cqt;
  const uint32_t sa = tc::smem_u32(sAop);
  int ok = 1, failed_i = -1;
  for (int i = 0; i < nblk; ++i) {
    const int p = i / ncbw, cb = cb_beg + i % ncbw;
    const uint32_t par3 = (uint32_t)(i & 1);
    bool good = true;  // thread 0: every copy landed and every MMA was issued
    if (tid == 0) {
      if (i % ncbw == 0) {
        // row operand of product p (the previous product's MMAs are done)
        const TcOperand &x = u.x[p];
        tc::mbar_expect_tx(&bars[0], TC_OP);
        const uint8_t *src = x.S + b * x.sS + (int64_t)R * x.blk;
        for (int s = 0; s < TC_S; ++s)
          tc::bulk_g2s(sAop + s * (TC_KS * TC_TILE), src + s * (TC_KS * TC_TILE), TC_KS * TC_TILE, &bars[0]);
      }
      if (i == 0) issue_cols(0);
      if (i + 1 < nblk) issue_cols(i + 1);
      if (p == 0 && i + 1 < ncbw) {  // the next tile of C towards L2
        const int c0 = u.cbase + 32 * (cb + 1);
        for (int c = c0; c < min(c0 + 32, u.cbase + ncols); ++c)
          tc::prefetch_l2(C + r0 + u.ldc * c, (uint32_t)nr * 16u);
      }
      if (i == 0 && stall) good = tc::mbar_wait(&bars[4], 0u, u.stall_cycles);
      if (i % ncbw == 0) good = good && tc::mbar_wait(&bars[0], (uint32_t)p);
      good = good && tc::mbar_wait(&bars[1 + (i & 1)], (uint32_t)((i >> 1) & 1));
      if (good) {
        tc::fence_after();
        tc_issue(tm, sa, tc::smem_u32(sBop + (i & 1) * TC_BBYTES));
      }
      tc::mma_commit(&bars[3]);
      if (!good) atomicExch(&err[b], 1);
    }
    // this thread's entries of C, loaded while the MMAs run
    zdf cv[TC_CQ];
    const int cl0 = 32 * cb + TC_CQ * cqt;  // first column (local) of this thread
#pragma unroll
    for (int qq = 0; qq < TC_CQ; ++qq) {
      const int cl = cl0 + qq, c = u.cbase + cl;
      if (rl < nrows && cl < ncols && (!u.tri || r >= c)) cv[qq] = C[r + u.ldc * c];
    }
    bool done = tc::mbar_wait(&bars[3], par3);
    // (already complete: makes the copied column exponents visible here)
    done = done && tc::mbar_wait(&bars[1 + (i & 1)], (uint32_t)((i >> 1) & 1));
    ok = __syncthreads_and(done && ok && good);
    if (!ok) {
      failed_i = i;
      break;
    }
    tc::fence_after();
    const int er = erow[p];
    const TcOperand &y = u.y[p];
    const int *ec = sEc + (i & 1) * 64;
#pragma unroll
    for (int cc = 0; cc < TC_CQ / 4; ++cc) {
      float are[TC_S][4], aim[TC_S][4];
#pragma unroll
      for (int uu = 0; uu < TC_S; ++uu) {
        tc::tmem_ld4(lane_addr + uu * 32 + cc * 4, are[uu]);
        tc::tmem_ld4(lane_addr + (TC_S + uu) * 32 + cc * 4, aim[uu]);
      }
      tc::tmem_ld_wait();
#pragma unroll
      for (int qq = 0; qq < 4; ++qq) {
        const int q16 = 4 * cc + qq;
        const int cl = cl0 + q16, c = u.cbase + cl;
        if (rl < nrows && cl < ncols && (!u.tri || r >= c)) {
          float vr[TC_S], vi[TC_S];
#pragma unroll
          for (int uu = 0; uu < TC_S; ++uu) {
            vr[uu] = are[uu][qq];
            vi[uu] = aim[uu][qq];
          }
          const int ecol = ec[(TC_CQ * cqt + q16) * y.es + y.eo];
          const float sc = pow2f(er + ecol - 16);
          df pr = combine7(vr), pi = combine7(vi);
          pr.hi = __fmul_rn(pr.hi, sc);
          pr.lo = __fmul_rn(pr.lo, sc);
          pi.hi = __fmul_rn(pi.hi, sc);
          pi.lo = __fmul_rn(pi.lo, sc);
          zdf a = cv[q16];
          a.re = df_sub(a.re, pr);
          a.im = df_sub(a.im, pi);
          C[r + u.ldc * c] = a;
        }
      }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
  }
  if (!ok) {
    // let the copies and MMAs still in flight finish (bounded waits) before
    // the shared and tensor memory are released: the row operand of the
    // failed step's product, the failed step's MMAs and column copy, and the
    // column copy issued for the step after it
    if (tid == 0 && failed_i >= 0) {
      const int fp = failed_i / ncbw;
      tc::mbar_wait(&bars[0], (uint32_t)(fp & 1), 200000000LL);
      tc::mbar_wait(&bars[3], (uint32_t)(failed_i & 1), 200000000LL);
      tc::mbar_wait(&bars[1 + (failed_i & 1)], (uint32_t)((failed_i >> 1) & 1), 200000000LL);
      const int nx = failed_i + 1;
      if (nx < nblk) tc::mbar_wait(&bars[1 + (nx & 1)], (uint32_t)((nx >> 1) & 1), 200000000LL);
    }
    if (tid == 0) atomicExch(&err[b], 1);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
  }
  if (warp == 0) tc::tmem_dealloc(tm, 512);
}

// Long-K products on the tensor cores over column-major DF matrices read
// row-wise: element (c, r) of A at A[r + lda c] (conjugated with conj_a),
// element (j, r) of B at Bm[r + ldb j] (conjugated with conj_b, zero above a
// Householder panel's unit diagonal with vmask).  A complex A gives
// C(c, j) = sum_r A(c, r) conj(B(j, r)) (tc_issue forms the conjugate
// product); a real A (real_a) gives C(c, j) = sum_r A(c, r) B(j, r).
// Exact slice products need K <= 64 reals, so the rows r are taken in
// chunks of 32: per chunk both operands are sliced in
// shared memory on the grid of the chunk, the MMAs accumulate in tensor
// memory, and the 14 accumulators are folded into double-float registers;
// the next chunk's rows are copied (cp.async) while the MMAs run.
// CTA = 128 rows c x 32 rows j.
//   mode 0 (V^H X of the back-transform): j = the 32 panel columns, the rows
//     split over gridDim.y ranges, written to split-K slots of out
//     (out[(y 32 + j) ldo + c]);
//   mode 1 (E_b = X^H Z): A = Z (real, rows c < m_b: the eigenvector
//     index), B = X (conjugated, rows j < nrows_b: the boundary row),
//     written to out[j + ldo c].  A real A operand needs only its two real
//     k-steps sliced, so a chunk's slicing (128 x 2 + 32 x 4 k-steps) runs in
//     one pass of the CTA's threads.
struct LongK {
  const zdf *A;
  int64_t lda, sA;
  int conj_a, real_a;
  const zdf *Bm;
  int64_t ldb, sB;
  int vmask, conj_b;
  int nrows_b;         // mode 1: valid B rows
  int k0, jb;          // vmask: panel k0 of width jb
  int rbeg;            // rows [rbeg, n_b)
  int ncols_a;         // rows c < ncols_a
  const int64_t *rng;  // mode 1: rows c < rng[8 b + 2]
  zdf *out;
  int64_t ldo, sO;
  int mode;
};
constexpr int VX_LD = 33;              // staging row stride (16-byte elements)
constexpr int VX_STX = 128 * VX_LD * 16;
constexpr int VX_STV = 32 * VX_LD * 16;
constexpr int VX_SMEM = TC_OP + TC_BBYTES + VX_STX + VX_STV + 128 * 4 + 32 * 4 + 64;
__device__ __forceinline__ void cp_async16(void *dst, const void *src, bool valid) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(valid ? 16 : 0) : "memory");
}

// Slices of one k-step (16 reals) of an operand row staged in shared memory
// (strow[r], r < 32: the real parts are K = r, the imaginary parts K = 32 + r),
// on the same grid as slice_row.  The NKS threads of a row are adjacent lanes
// (lane % NKS = k-step) and share the row's exponent E (largest magnitude
// below 2^E).  Each digit is rounded onto its fixed grid without scaling:
// m = (t + 1.5 2^(23-8(s+1))) - 1.5 2^(23-8(s+1)) is t rounded to a multiple
// of 2^-8(s+1); t - m is exact, and is either 0 or at least ulp(t) > 2 |tl|,
// so Fast2Sum keeps the residual pair exact and normalised.  Every thread
// writes two 16-byte core-matrix rows per slice.
template <int TILE, int NKS>
__device__ __forceinline__ int slice_kstep(const zdf *strow, bool neg_im, uint8_t *blk, int row, int ks) {
  const int part = ks >> 1, rb = (ks & 1) * 16;
  float th[16], tl[16];
  float amax = 0.f;
#pragma unroll
  for (int t = 0; t < 16; ++t) {
    const df v = ((const df *)&strow[rb + t])[part];
    th[t] = v.hi;
    tl[t] = v.lo;
    amax = fmaxf(amax, fabsf(v.hi));
  }
  amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, 1));
  if (NKS == 4) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, 2));
  int E = 0;
  if (amax > 0.f) frexpf(amax, &E);
  // 2^-E exceeds the float range when the largest magnitude is subnormal
  // (E <= -128, e.g. the far tail of a localised eigenvector): such rows are
  // scaled in two exact power-of-two steps
  const int e1 = E < -100 ? 100 : 0;
  const float sc = (part && neg_im) ? -pow2f(-E - e1) : pow2f(-E - e1);
  if (e1) {
#pragma unroll
    for (int t = 0; t < 16; ++t) {
      th[t] = __fmul_rn(th[t], 0x1p100f);
      tl[t] = __fmul_rn(tl[t], 0x1p100f);
    }
  }
#pragma unroll
  for (int t = 0; t < 16; ++t) {
    th[t] = __fmul_rn(th[t], sc);
    tl[t] = __fmul_rn(tl[t], sc);
  }
  uint8_t *base = blk + ks * TILE + tc::core_off(row, 0);
#pragma unroll
  for (int sl = 0; sl < TC_S; ++sl) {
    const float mag = 1.5f * (float)(1 << 15) * pow2f(-8 * sl);  // 1.5 2^(23 - 8(sl+1))
    const float up = pow2f(8 * (sl + 1));
    uint32_t w[8];
#pragma unroll
    for (int t = 0; t < 16; t += 2) {
      const float m0 = __fsub_rn(__fadd_rn(th[t], mag), mag);
      const float m1 = __fsub_rn(__fadd_rn(th[t + 1], mag), mag);
      fast_two_sum(__fsub_rn(th[t], m0), tl[t], th[t], tl[t]);
      fast_two_sum(__fsub_rn(th[t + 1], m1), tl[t + 1], th[t + 1], tl[t + 1]);
      const __nv_bfloat162 h = __floats2bfloat162_rn(__fmul_rn(m0, up), __fmul_rn(m1, up));
      w[t >> 1] = *(const uint32_t *)&h;
    }
    uint8_t *dst = base + sl * TC_KS * TILE;
    *(uint4 *)dst = make_uint4(w[0], w[1], w[2], w[3]);
    *(uint4 *)(dst + 128) = make_uint4(w[4], w[5], w[6], w[7]);
  }
  return E;
}

// tc_issue for a real row operand: re acc pairs row k-step j (j < 2) with
// column k-step j, im acc the same row k-step with column k-step j + 2.
__device__ __forceinline__ void tc_issue_reala(uint32_t tm, uint32_t sa, uint32_t sb) {
  const uint64_t a0 = tc::sdesc(sa, 128, 256), b0 = tc::sdesc(sb, 128, 256);
#pragma unroll
  for (int u = 0; u < TC_S; ++u) {
#pragma unroll
    for (int s = 0; s <= u; ++s) {
      const int t = u - s;
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const uint32_t acc = (s == 0 && j == 0) ? 0u : 1u;
        const uint64_t ar = a0 + (uint64_t)((s * TC_KS + j) * (TC_TILE >> 4));
        const uint64_t br = b0 + (uint64_t)((t * TC_KS + j) * (1024 >> 4));
        const uint64_t bi = b0 + (uint64_t)((t * TC_KS + j + 2) * (1024 >> 4));
        tc::mma_bf16(tm + u * 32, ar, br, TC_ID, acc);
        tc::mma_bf16(tm + (TC_S + u) * 32, ar, bi, TC_ID, acc);
      }
    }
  }
}

__global__ void __launch_bounds__(TC_NT, 1) k_longk_tc(LongK p, const int *nvec, int *err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t *sAop = smem;                                         // A rows (c), one chunk, sliced
  uint8_t *sBop = smem + TC_OP;                                 // B rows (j), one chunk, sliced
  zdf *stX = (zdf *)(smem + TC_OP + TC_BBYTES);                 // stX[c * VX_LD + row]
  zdf *stV = (zdf *)(smem + TC_OP + TC_BBYTES + VX_STX);        // stV[j * VX_LD + row]
  int *sEc = (int *)(smem + TC_OP + TC_BBYTES + VX_STX + VX_STV);
  int *sEa = sEc + 128;
  uint64_t *bar = (uint64_t *)(sEa + 32);
  uint32_t *tslot = (uint32_t *)(bar + 1);
  const int b = blockIdx.z;
  const int n = nvec[b];
  // mode 1 walks the 32-row B tiles fastest (blockIdx.x), so that the CTAs
  // sharing one 128-row tile of Z run together and read it once from DRAM
  const int ta = p.mode == 1 ? blockIdx.y : blockIdx.x, tb = p.mode == 1 ? blockIdx.x : blockIdx.y;
  const int c0 = ta * 128;
  const int na = p.mode == 1 ? (int)p.rng[b * 8 + 2] : p.ncols_a;  // valid rows c
  if (c0 >= na) return;
  const int j0 = p.mode >= 1 ? 32 * tb : 0;
  const int nj = p.mode == 1 ? p.nrows_b : min(p.jb, n - 1 - p.k0);  // valid rows j
  if (p.mode >= 1 && j0 >= nj) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int lg = warp & 3, cqt = warp >> 2;
  const int cl = 32 * lg + lane;  // row c of this thread (TMEM lane)
  // chunks of 32 rows r: [kc_beg, kc_end)
  const int nck = n > p.rbeg ? (n - p.rbeg + 31) / 32 : 0;
  const int ns = p.mode == 0 ? gridDim.y : 1, si = p.mode == 0 ? blockIdx.y : 0;
  const int kc_beg = (int)((int64_t)nck * si / ns);
  const int kc_end = (int)((int64_t)nck * (si + 1) / ns);
  df accr[TC_CQ], acci[TC_CQ];
#pragma unroll
  for (int q = 0; q < TC_CQ; ++q) accr[q] = acci[q] = df{0.f, 0.f};
  const bool any = kc_beg < kc_end && !*(volatile int *)&err[b];
  uint32_t tm = 0;
  if (any) {
    if (warp == 0) tc::tmem_alloc(tslot, 512);
    if (tid == 0) {
      tc::mbar_init(bar, 1);
      tc::mbar_init_fence();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    tm = *tslot;
  }
  const zdf *A = p.A + b * p.sA;
  const zdf *Bm = p.Bm + b * p.sB;
  const uint32_t lane_addr = tm + ((uint32_t)(32 * lg) << 16) + TC_CQ * cqt;
  // copies of a chunk into the staging buffers: lane = row r, 8 A rows and 2
  // B rows per warp (zero outside the operands)
  auto load = [&](int kc) {
    const int r = p.rbeg + 32 * kc + lane;
#pragma unroll
    for (int jj = 0; jj < 8; ++jj) {
      const int c = 8 * warp + jj;
      const bool v = r < n && c0 + c < na;
      cp_async16(&stX[c * VX_LD + lane], v ? (const void *)&A[r + p.lda * (c0 + c)] : (const void *)A, v);
    }
#pragma unroll
    for (int jj = 0; jj < 2; ++jj) {
      const int j = 2 * warp + jj;
      bool v = r < n && j0 + j < nj;
      if (p.vmask) v = v && r >= p.k0 + j + 1;
      cp_async16(&stV[j * VX_LD + lane], v ? (const void *)&Bm[r + p.ldb * (j0 + j)] : (const void *)Bm, v);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  int ok = 1, failed_par = -1;
  if (any) load(kc_beg);
  for (int kc = kc_beg; any && kc < kc_end; ++kc) {
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    if (p.real_a) {  // A real: threads 0-255 slice its real k-steps, 256-383 slice B
      if (tid < 256) {
        const int c = tid >> 1, ks = tid & 1;
        const int e = slice_kstep<TC_TILE, 2>(&stX[c * VX_LD], false, sAop, c, ks);
        if (ks == 0) sEc[c] = e;
      } else if (tid < 384) {
        const int j = (tid - 256) >> 2, ks = tid & 3;
        const int e = slice_kstep<1024, 4>(&stV[j * VX_LD], p.conj_b != 0, sBop, j, ks);
        if (ks == 0) sEa[j] = e;
      }
    } else {
      {  // A: thread = (row c, k-step)
        const int c = tid >> 2, ks = tid & 3;
        const int e = slice_kstep<TC_TILE, 4>(&stX[c * VX_LD], p.conj_a != 0, sAop, c, ks);
        if (ks == 0) sEc[c] = e;
      }
      if (tid < 128) {
        const int j = tid >> 2, ks = tid & 3;
        const int e = slice_kstep<1024, 4>(&stV[j * VX_LD], p.conj_b != 0, sBop, j, ks);
        if (ks == 0) sEa[j] = e;
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (tid == 0) {
      if (p.real_a)
        tc_issue_reala(tm, tc::smem_u32(sAop), tc::smem_u32(sBop));
      else
        tc_issue(tm, tc::smem_u32(sAop), tc::smem_u32(sBop));
      tc::mma_commit(bar);
    }
    if (kc + 1 < kc_end) load(kc + 1);  // in flight while the MMAs run
    const bool done = tc::mbar_wait(bar, (uint32_t)((kc - kc_beg) & 1));
    ok = __syncthreads_and(done && ok);
    if (!ok) {
      failed_par = (kc - kc_beg) & 1;
      break;
    }
    tc::fence_after();
    const int ec = sEc[cl];
#pragma unroll
    for (int cc = 0; cc < TC_CQ / 4; ++cc) {
      float are[TC_S][4], aim[TC_S][4];
#pragma unroll
      for (int uu = 0; uu < TC_S; ++uu) {
        tc::tmem_ld4(lane_addr + uu * 32 + cc * 4, are[uu]);
        tc::tmem_ld4(lane_addr + (TC_S + uu) * 32 + cc * 4, aim[uu]);
      }
      tc::tmem_ld_wait();
#pragma unroll
      for (int qq = 0; qq < 4; ++qq) {
        const int q = 4 * cc + qq;
        float vr[TC_S], vi[TC_S];
#pragma unroll
        for (int uu = 0; uu < TC_S; ++uu) {
          vr[uu] = are[uu][qq];
          vi[uu] = aim[uu][qq];
        }
        const float sc = pow2f(ec + sEa[TC_CQ * cqt + q] - 16);
        df pr = combine7(vr), pi = combine7(vi);
        pr.hi = __fmul_rn(pr.hi, sc);
        pr.lo = __fmul_rn(pr.lo, sc);
        pi.hi = __fmul_rn(pi.hi, sc);
        pi.lo = __fmul_rn(pi.lo, sc);
        accr[q] = df_add(accr[q], pr);
        acci[q] = df_add(acci[q], pi);
      }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
  }
  asm volatile("cp.async.wait_group 0;" ::: "memory");  // no copy may land after exit
  if (any) {
    if (!ok) {
      // the MMAs whose wait gave up may still be running: give them (a
      // bounded) time to finish before their tensor memory is released
      if (tid == 0) {
        atomicExch(&err[b], 1);
        if (failed_par >= 0) tc::mbar_wait(bar, (uint32_t)failed_par, 200000000LL);
      }
      tc::fence_before();
      __syncthreads();
      tc::fence_after();
    }
    if (warp == 0) tc::tmem_dealloc(tm, 512);
  }
  // this thread's row c and its 8 rows j
  if (c0 + cl < na) {
    zdf *out = p.out + b * p.sO;
#pragma unroll
    for (int q = 0; q < TC_CQ; ++q) {
      const int j = TC_CQ * cqt + q;
      if (p.mode == 0)
        out[((int64_t)blockIdx.y * 32 + j) * p.ldo + c0 + cl] = zdf{accr[q], acci[q]};
      else if (j0 + j < nj)
        out[j0 + j + p.ldo * (int64_t)(c0 + cl)] = zdf{accr[q], acci[q]};
    }
  }
}

}  // namespace

// PARPHOM_GPU_TC=0 selects the CUDA-core trailing update in the double-float
// form (both are the library's own kernels; the tensor-core one is default).
bool tc_enabled() {
  static int v = -1;
  if (v < 0) {
    const char *e = getenv("PARPHOM_GPU_TC");
    v = (e && e[0] == '0') ? 0 : 1;
  }
  return v == 1;
}

size_t her2k_tc_bytes(int64_t nmax) { return (size_t)((nmax + 127) / 128) * TC_RBLK; }
int64_t her2k_tc_exps(int64_t nmax) { return 2 * ((nmax + 127) / 128) * 128; }

// Opt the tensor-core kernels into their shared memory on the current device
// (the attribute is per device; done once per device, outside any capture).
cudaError_t prepare_her2k_tc() {
  static std::mutex mu;
  static bool done[PP_MAX_DEVICES] = {};
  const int dev = device_index();
  std::lock_guard<std::mutex> g(mu);
  if (dev >= 0 && done[dev]) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_cupd_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_longk_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, VX_SMEM);
  if (e == cudaSuccess && dev >= 0) done[dev] = true;
  return e;
}

namespace {
cudaError_t launch_slices(const TcSliceSrc &src, int rows_max, EigWork &w, int k0, int jb, uint8_t *S, int64_t blk,
                          int *E, int es, int eo, cudaStream_t s) {
  const int rows = (rows_max + 127) / 128 * 128;
  if (rows <= 0) return cudaSuccess;
  PP_KT(KT_HER2K, s, (k_tc_slices<<<dim3(rows / 4, w.B), 128, 0, s>>>(src, w.nvec, k0, jb, S, w.sTcS, blk, E, w.sTcE,
                                                                      es, eo)));
  count_launch(1);
  return cudaGetLastError();
}
}  // namespace

// One-shot stall of the test hook: the global batch index of the matrix
// and the wait's limit in SM clocks (-1: not armed).
static std::mutex g_stall_mu;
static int64_t g_stall_matrix = -1;
static long long g_stall_cycles = 0;

void arm_tc_stall(int64_t matrix, long long cycles) {
  std::lock_guard<std::mutex> g(g_stall_mu);
  g_stall_matrix = matrix;
  g_stall_cycles = cycles;
}
bool tc_stall_armed() {
  std::lock_guard<std::mutex> g(g_stall_mu);
  return g_stall_matrix >= 0;
}
// The stall for a launch over batch matrices [boff, boff + B): consumed by
// the first launch that covers the armed matrix.
static int take_stall(const EigWork &w, long long *cycles) {
  std::lock_guard<std::mutex> g(g_stall_mu);
  if (g_stall_matrix < w.boff || g_stall_matrix >= (int64_t)w.boff + w.B) return -1;
  const int b = (int)(g_stall_matrix - w.boff);
  *cycles = g_stall_cycles;
  g_stall_matrix = -1;
  return b;
}

// A(k1:n, k1:n) -= V W^H + W V^H, lower triangle (panel k0 of width jb).
cudaError_t her2k_tc(EigWork &w, int k0, int jb, cudaStream_t s) {
  const int k1 = k0 + jb;
  const int mmax = w.nmax - k1;
  if (mmax <= 0) return cudaSuccess;
  const int64_t sW = (int64_t)w.lda * w.nb;
  const zdf *A = (const zdf *)w.A;
  // V rows (block part 0) and W rows (block part 1) of the trailing block
  PP_CUDA_TRY(launch_slices(TcSliceSrc{A + w.lda * k0, w.sA, 1, w.lda, k1, 0, 1, 0}, mmax, w, k0, jb, w.tcS,
                            TC_RBLK, w.tcE, 2, 0, s));
  PP_CUDA_TRY(launch_slices(TcSliceSrc{(const zdf *)w.W, sW, 1, w.lda, k1, 0, 0, 0}, mmax, w, k0, jb,
                            w.tcS + TC_OP, TC_RBLK, w.tcE, 2, 1, s));
  TcUpdate u{};
  u.C = (zdf *)w.A;
  u.ldc = w.lda;
  u.sC = w.sA;
  u.rbase = u.cbase = k1;
  u.ncols_fixed = 0;
  u.tri = 1;
  u.nprod = 2;
  const TcOperand V{w.tcS, w.sTcS, TC_RBLK, w.tcE, w.sTcE, 2, 0};
  const TcOperand Wo{w.tcS + TC_OP, w.sTcS, TC_RBLK, w.tcE, w.sTcE, 2, 1};
  u.x[0] = V;
  u.y[0] = Wo;
  u.x[1] = Wo;
  u.y[1] = V;
  u.stall_b = take_stall(w, &u.stall_cycles);
  const int nrb = (mmax + 127) / 128;
  const int nq = (4 * nrb + TC_CB - 1) / TC_CB;
  PP_KT(KT_HER2K, s, (k_cupd_tc<<<dim3(nq, nrb, w.B), TC_NT, TC_SMEM, s>>>(u, w.nvec, w.tcErr)));
  count_launch(1);
  return cudaGetLastError();
}

// X(k0+1:n, 0:ncols) -= V Y with V the Householder vectors of panel k0 (width
// jb) and Y (jb x ncols) at Yb[a ldy + c]: the update of the compact-WY
// back-transform as X Y'^H with Y'(c, a) = conj(Y(a, c)).
cudaError_t applyV_tc(EigWork &w, int k0, int jb, zdf *X, int64_t ldx, int64_t sX, const zdf *Yb, int64_t ldy,
                      int64_t sY, int ncols, cudaStream_t s) {
  const int r1 = k0 + 1;
  const int mmax = w.nmax - r1;
  if (mmax <= 0 || ncols <= 0) return cudaSuccess;
  const zdf *A = (const zdf *)w.A;
  const int64_t vbl = (int64_t)((w.nmax + 127) / 128) * TC_OP;  // the Y' slices follow the V slices
  const int64_t yexp = (w.nmax + 127) / 128 * 128;
  PP_CUDA_TRY(launch_slices(TcSliceSrc{A + w.lda * k0, w.sA, 1, w.lda, r1, 0, 1, 0}, mmax, w, k0, jb, w.tcS, TC_OP,
                            w.tcE, 1, 0, s));
  PP_CUDA_TRY(launch_slices(TcSliceSrc{Yb, sY, 1, ldy, 0, ncols, 0, 1}, ncols, w, k0, jb, w.tcS + vbl, TC_OP,
                            w.tcE + yexp, 1, 0, s));
  TcUpdate u{};
  u.C = X;
  u.ldc = ldx;
  u.sC = sX;
  u.rbase = r1;
  u.cbase = 0;
  u.ncols_fixed = ncols;
  u.tri = 0;
  u.nprod = 1;
  u.stall_b = -1;
  u.x[0] = TcOperand{w.tcS, w.sTcS, TC_OP, w.tcE, w.sTcE, 1, 0};
  u.y[0] = TcOperand{w.tcS + vbl, w.sTcS, TC_OP, w.tcE + yexp, w.sTcE, 1, 0};
  u.x[1] = u.x[0];
  u.y[1] = u.y[0];
  const int nrb = (mmax + 127) / 128;
  const int nq = ((ncols + 31) / 32 + TC_CB - 1) / TC_CB;
  PP_KT(KT_APPLYV, s, (k_cupd_tc<<<dim3(nq, nrb, w.B), TC_NT, TC_SMEM, s>>>(u, w.nvec, w.tcErr)));
  count_launch(1);
  return cudaGetLastError();
}

// Wp(a, c) = (V^H X)(a, c) over the rows r > k0 (V: panel k0 of width jb),
// c < ncols; written to the first split-K slot of Wp.
int vhx_tc_splits(const EigWork &w) { return std::max(1, std::min(4, w.ksplit)); }

cudaError_t vhx_tc(EigWork &w, int k0, int jb, const zdf *X, int64_t ldx, int64_t sX, int ncols, zdf *Wp,
                   int64_t ldwp, int64_t sWp, cudaStream_t s) {
  if (ncols <= 0) return cudaSuccess;
  LongK p{};
  p.A = X;
  p.lda = ldx;
  p.sA = sX;
  p.Bm = (const zdf *)w.A + w.lda * k0;
  p.ldb = w.lda;
  p.sB = w.sA;
  p.vmask = 1;
  p.k0 = k0;
  p.jb = jb;
  p.rbeg = k0 + 1;
  p.ncols_a = ncols;
  p.out = Wp;
  p.ldo = ldwp;
  p.sO = sWp;
  p.mode = 0;
  PP_KT(KT_VHX, s, (k_longk_tc<<<dim3((ncols + 127) / 128, vhx_tc_splits(w), w.B), TC_NT, VX_SMEM, s>>>(
                       p, w.nvec, w.tcErr)));
  count_launch(1);
  return cudaGetLastError();
}

cudaError_t xhz_tc(EigWork &w, const zdf *X, int64_t ldx, int64_t sX, int nrows, const zdf *Z, int64_t ldz,
                   int64_t sZ, zdf *Eb, int64_t lde, int64_t sE, cudaStream_t s) {
  if (nrows <= 0) return cudaSuccess;
  LongK p{};
  p.A = Z;
  p.lda = ldz;
  p.sA = sZ;
  p.real_a = 1;
  p.Bm = X;
  p.ldb = ldx;
  p.sB = sX;
  p.conj_b = 1;
  p.nrows_b = nrows;
  p.rbeg = 0;
  p.rng = w.rng;
  p.out = Eb;
  p.ldo = lde;
  p.sO = sE;
  p.mode = 1;
  PP_KT(KT_XHZ, s, (k_longk_tc<<<dim3((nrows + 31) / 32, (w.mcap + 127) / 128, w.B), TC_NT, VX_SMEM, s>>>(
                       p, w.nvec, w.tcErr)));
  count_launch(1);
  return cudaGetLastError();
}

}  // namespace pp
