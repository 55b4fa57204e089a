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
#include <cfloat>
#include <cstdint>
#include <cstdlib>
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

// 2^e as a float (exact for -126 <= e <= 127)
__device__ __forceinline__ float pow2f(int e) {
  return (e >= -126 && e <= 127) ? __int_as_float((e + 127) << 23) : ldexpf(1.0f, e);
}

// Slices of one operand row held by a warp: lane a has the complex value of
// panel column a; K index a (real part) and 32 + a (imaginary part).
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
    uint8_t *base = blk + (kk >> 4) * TC_TILE + tc::core_off(row, kk & 15);
#pragma unroll
    for (int s = 0; s < TC_S; ++s) {
      th = __fmul_rn(th, 256.f);
      tl = __fmul_rn(tl, 256.f);
      const float mi = rintf(th);
      two_sum(__fsub_rn(th, mi), tl, th, tl);
      *(__nv_bfloat16 *)(base + s * TC_KS * TC_TILE) = __float2bfloat16_rn(mi);
    }
  }
  return E;
}

// Slices of the panel rows k1 + rl, rl < 128 * ceil((n - k1)/128): one warp
// per row.  Block R of the slice array holds the V operand of rows
// 128R .. 128R+127 followed by their W operand; Ex[2 rl] and Ex[2 rl + 1]
// are the two row exponents.
__global__ void __launch_bounds__(128) k_tc_slices(const zdf *Ab, int64_t lda, int64_t sA, const zdf *Wb,
                                                   int64_t sW, const int *nvec, int k0, int jb, uint8_t *S,
                                                   int64_t sS, int *Ex, int64_t sEx) {
  const int b = blockIdx.y;
  const int n = nvec[b];
  const int k1 = k0 + jb;
  const int m = n - k1;
  if (m <= 0) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rl = blockIdx.x * 4 + warp;
  if (rl >= (m + 127) / 128 * 128) return;
  const int r = k1 + rl;
  const int jmax = min(jb, n - 1 - k0);
  zdf v{{0.f, 0.f}, {0.f, 0.f}}, w{{0.f, 0.f}, {0.f, 0.f}};
  if (r < n && lane < jmax) {
    v = Ab[b * sA + r + lda * (k0 + lane)];
    w = Wb[b * sW + r + lda * lane];
  }
  uint8_t *blk = S + b * sS + (int64_t)(rl >> 7) * TC_RBLK;
  const int ev = slice_row(v, blk, rl & 127, lane);
  const int ew = slice_row(w, blk + TC_OP, rl & 127, lane);
  if (lane == 0) {
    Ex[b * sEx + 2 * rl] = ev;
    Ex[b * sEx + 2 * rl + 1] = ew;
  }
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

__global__ void __launch_bounds__(TC_NT, 1) k_her2k_tc(zdf *Ab, int64_t lda, int64_t sA, const uint8_t *S, int64_t sS,
                                                     const int *Ex, int64_t sEx, const int *nvec, int k0, int jb,
                                                     int *err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t *sAop = smem;                                  // row operand
  uint8_t *sBop = smem + TC_OP;                          // two column-operand buffers
  int *sEc = (int *)(smem + TC_OP + 2 * TC_BBYTES);      // two x 32 (V, W) column exponent pairs
  // mbarriers: [0] row operand landed (waited by thread 0), [1], [2] column
  // buffer 0 / 1 landed, [3] MMAs of the block done.
  // Each barrier a thread waits on completes exactly once between two of
  // its waits, so parity waits cannot skip a phase.
  uint64_t *bars = (uint64_t *)(smem + TC_OP + 2 * TC_BBYTES + 512);
  uint32_t *tslot = (uint32_t *)(bars + 4);
  const int b = blockIdx.z, R = blockIdx.y, q = blockIdx.x;
  const int n = nvec[b];
  const int k1 = k0 + jb;
  const int m = n - k1;
  if (m <= 0) return;
  const int nrb = (m + 127) / 128, ncb = (m + 31) / 32;
  if (R >= nrb) return;
  const int cb_beg = q * TC_CB;
  const int cb_end = min(min(cb_beg + TC_CB, 4 * (R + 1)), ncb);
  if (cb_beg >= cb_end) return;
  // an earlier wait of this matrix gave up: its results are already invalid
  if (*(volatile int *)&err[b]) return;
  const int ncbw = cb_end - cb_beg;
  const int nblk = 2 * ncbw;  // (product, column block) steps

  const int tid = threadIdx.x, warp = tid >> 5;
  if (warp == 0) tc::tmem_alloc(tslot, 512);
  if (tid == 0) {
    for (int i = 0; i < 4; ++i) tc::mbar_init(&bars[i], 1);
    tc::mbar_init_fence();
  }
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const uint32_t tm = *tslot;
  const uint8_t *Sb = S + b * sS;
  const int *Eb = Ex + b * sEx;
  zdf *A = Ab + b * sA;
  const int r0 = k1 + 128 * R;
  const int nr = min(128, n - r0);
  // column operand of step i: product p = i / ncbw uses the W (p = 0) or V
  // (p = 1) slices of the column rows
  auto issue_cols = [&](int i) {
    const int p = i / ncbw, cb = cb_beg + i % ncbw;
    const int buf = i & 1;
    uint64_t *bar = &bars[1 + buf];
    tc::mbar_expect_tx(bar, TC_BBYTES + 256);
    const uint8_t *src = Sb + (int64_t)(cb >> 2) * TC_RBLK + (p == 0 ? TC_OP : 0) + (cb & 3) * 1024;
    uint8_t *dst = sBop + buf * TC_BBYTES;
    for (int sj = 0; sj < TC_S * TC_KS; ++sj) tc::bulk_g2s(dst + sj * 1024, src + sj * TC_TILE, 1024, bar);
    // exponents of the 32 column rows (interleaved V, W pairs: 256 bytes),
    // copied whole; the product picks its half
    tc::bulk_g2s(sEc + buf * 64, Eb + 2 * 32 * cb, 256, bar);
  };
  const int lg = warp & 3, cqt = warp >> 2;
  const int rl = 128 * R + 32 * lg + (tid & 31);  // trailing-block row = TMEM lane
  const int r = k1 + rl;
  const int Erv = Eb[2 * rl], Erw = Eb[2 * rl + 1];
  const uint32_t lane_addr = tm + ((uint32_t)(32 * lg) << 16) + TC_CQ * cqt;
  const uint32_t sa = tc::smem_u32(sAop);
  int ok = 1;
  for (int i = 0; i < nblk; ++i) {
    const int p = i / ncbw, cb = cb_beg + i % ncbw;
    const uint32_t par3 = (uint32_t)(i & 1);
    bool good = true;  // thread 0: every copy landed and every MMA was issued
    if (tid == 0) {
      if (i % ncbw == 0) {
        // row operand of product p (the previous product's MMAs are done)
        tc::mbar_expect_tx(&bars[0], TC_OP);
        const uint8_t *src = Sb + (int64_t)R * TC_RBLK + (p == 0 ? 0 : TC_OP);
        for (int s = 0; s < TC_S; ++s)
          tc::bulk_g2s(sAop + s * (TC_KS * TC_TILE), src + s * (TC_KS * TC_TILE), TC_KS * TC_TILE, &bars[0]);
      }
      if (i == 0) issue_cols(0);
      if (i + 1 < nblk) issue_cols(i + 1);
      if (p == 0 && i + 1 < ncbw) {
        const int c0 = k1 + 32 * (cb + 1);
        for (int c = c0; c < min(c0 + 32, n); ++c) tc::prefetch_l2(A + r0 + lda * c, (uint32_t)nr * 16u);
      }
      if (i % ncbw == 0) good = tc::mbar_wait(&bars[0], (uint32_t)p);
      good = good && tc::mbar_wait(&bars[1 + (i & 1)], (uint32_t)((i >> 1) & 1));
      if (good) {
        tc::fence_after();
        tc_issue(tm, sa, tc::smem_u32(sBop + (i & 1) * TC_BBYTES));
      }
      tc::mma_commit(&bars[3]);
      if (!good) atomicExch(&err[b], 1);
    }
    // this thread's 16 entries of A, loaded while the MMAs run
    zdf cv[TC_CQ];
    const int cbase = k1 + 32 * cb + TC_CQ * cqt;
#pragma unroll
    for (int qq = 0; qq < TC_CQ; ++qq) {
      const int c = cbase + qq;
      if (r < n && c < n && r >= c) cv[qq] = A[r + lda * c];
    }
    bool done = tc::mbar_wait(&bars[3], par3);
    // (already complete: makes the copied column exponents visible here)
    done = done && tc::mbar_wait(&bars[1 + (i & 1)], (uint32_t)((i >> 1) & 1));
    ok = __syncthreads_and(done && ok && good);
    if (!ok) break;
    tc::fence_after();
    const int erow = p == 0 ? Erv : Erw;
    const int *ec = sEc + (i & 1) * 64;  // (V, W) exponent pairs of the column rows
#pragma unroll
    for (int cc = 0; cc < TC_CQ / 4; ++cc) {
      float are[TC_S][4], aim[TC_S][4];
#pragma unroll
      for (int u = 0; u < TC_S; ++u) {
        tc::tmem_ld4(lane_addr + u * 32 + cc * 4, are[u]);
        tc::tmem_ld4(lane_addr + (TC_S + u) * 32 + cc * 4, aim[u]);
      }
      tc::tmem_ld_wait();
#pragma unroll
      for (int qq = 0; qq < 4; ++qq) {
        const int q16 = 4 * cc + qq;
        const int c = cbase + q16;
        if (r < n && c < n && r >= c) {
          float vr[TC_S], vi[TC_S];
#pragma unroll
          for (int u = 0; u < TC_S; ++u) {
            vr[u] = are[u][qq];
            vi[u] = aim[u][qq];
          }
          // column exponent: W half for the first product, V half for the second
          const int ecol = ec[2 * (TC_CQ * cqt + q16) + (p == 0 ? 1 : 0)];
          const float sc = pow2f(erow + ecol - 16);
          df pr = combine7(vr), pi = combine7(vi);
          pr.hi = __fmul_rn(pr.hi, sc);
          pr.lo = __fmul_rn(pr.lo, sc);
          pi.hi = __fmul_rn(pi.hi, sc);
          pi.lo = __fmul_rn(pi.lo, sc);
          zdf a = cv[q16];
          a.re = df_sub(a.re, pr);
          a.im = df_sub(a.im, pi);
          A[r + lda * c] = a;
        }
      }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
  }
  if (!ok) {
    // let the row-operand copy land before the shared memory is released
    if (tid == 0) {
      tc::mbar_wait(&bars[0], 0, 200000000LL);
      atomicExch(&err[b], 1);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
  }
  if (warp == 0) tc::tmem_dealloc(tm, 512);
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

cudaError_t prepare_her2k_tc() {
  static int done = 0;
  if (done) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_her2k_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
  if (e == cudaSuccess) done = 1;
  return e;
}

cudaError_t her2k_tc(EigWork &w, int k0, int jb, cudaStream_t s) {
  const int k1 = k0 + jb;
  const int mmax = w.nmax - k1;
  if (mmax <= 0) return cudaSuccess;
  const int nrb = (mmax + 127) / 128;
  const int rows = nrb * 128;
  PP_KT(KT_HER2K, s, (k_tc_slices<<<dim3(rows / 4, w.B), 128, 0, s>>>((const zdf *)w.A, w.lda, w.sA, (const zdf *)w.W,
                                                                      (int64_t)w.lda * w.nb, w.nvec, k0, jb, w.tcS,
                                                                      w.sTcS, w.tcE, w.sTcE)));
  const int nq = (4 * nrb + TC_CB - 1) / TC_CB;
  PP_KT(KT_HER2K, s, (k_her2k_tc<<<dim3(nq, nrb, w.B), TC_NT, TC_SMEM, s>>>((zdf *)w.A, w.lda, w.sA, w.tcS, w.sTcS,
                                                                          w.tcE, w.sTcE, w.nvec, k0, jb, w.tcErr)));
  count_launch(2);
  return cudaGetLastError();
}

}  // namespace pp
