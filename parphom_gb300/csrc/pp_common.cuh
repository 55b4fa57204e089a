// Shared device types for the phonon hot path: complex numbers over two real
// arithmetics and the two precision policies the solver is instantiated with.
//
//  * F64 — plain IEEE double (the "plain FP64" form).
//  * DF  — double-float: a value is an unevaluated sum hi + lo of two floats
//          (about 48 significand bits), computed with error-free
//          transformations on the FP32 pipes (Dekker/Knuth TwoSum, FMA-based
//          TwoProd; Joldes, Muller, Popescu, "Tight and rigorous error bounds
//          for basic building blocks of double-word arithmetic", ACM TOMS
//          2017).  GB300's FP64 rate is a small fraction of its FP32 rate, so
//          the O(n^3) parts of the mixed form run in this arithmetic.
//
// All error-free transformations use the __f*_rn intrinsics so that the
// compiler never contracts or reassociates them.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define PP_HD __host__ __device__ __forceinline__
#define PP_D __device__ __forceinline__

struct df {
  float hi, lo;
};

template <class R>
struct __align__(16) cx {
  R re, im;
};
typedef cx<double> z64;
typedef cx<df> zdf;

// ----------------------------------------------------------------------------
// double-float primitives
PP_D void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
PP_D void fast_two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  e = __fsub_rn(b, __fsub_rn(s, a));
}
PP_D df df_norm(df a) {
  df r;
  fast_two_sum(a.hi, a.lo, r.hi, r.lo);
  return r;
}
PP_D df df_add(df a, df b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  df r;
  fast_two_sum(s, e, r.hi, r.lo);
  return r;
}
PP_D df df_neg(df a) { return df{-a.hi, -a.lo}; }
PP_D df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
PP_D df df_mul(df a, df b) {
  float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  df r;
  fast_two_sum(p, e, r.hi, r.lo);
  return r;
}
// acc += a*b with the low word left unnormalised (call df_norm at the end).
PP_D void df_mac(df &acc, df a, df b) {
  float p = __fmul_rn(a.hi, b.hi);
  float pe = __fmaf_rn(a.hi, b.hi, -p);
  pe = __fmaf_rn(a.hi, b.lo, pe);
  pe = __fmaf_rn(a.lo, b.hi, pe);
  float s, e;
  two_sum(acc.hi, p, s, e);
  acc.hi = s;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(e, pe));
}
PP_HD df df_from(double x) {
  df r;
  r.hi = (float)x;
  r.lo = (float)(x - (double)r.hi);
  return r;
}
PP_HD double df_to(df a) { return (double)a.hi + (double)a.lo; }

// ----------------------------------------------------------------------------
// Real-arithmetic traits
template <class R>
struct RT;
template <>
struct RT<double> {
  PP_D static double zero() { return 0.0; }
  PP_D static double from(double x) { return x; }
  PP_D static double to(double x) { return x; }
  PP_D static double add(double a, double b) { return a + b; }
  PP_D static double sub(double a, double b) { return a - b; }
  PP_D static double mul(double a, double b) { return a * b; }
  PP_D static double neg(double a) { return -a; }
  PP_D static void mac(double &acc, double a, double b) { acc = fma(a, b, acc); }
  PP_D static double fin(double a) { return a; }
};
template <>
struct RT<df> {
  PP_D static df zero() { return df{0.f, 0.f}; }
  PP_D static df from(double x) { return df_from(x); }
  PP_D static double to(df x) { return df_to(x); }
  PP_D static df add(df a, df b) { return df_add(a, b); }
  PP_D static df sub(df a, df b) { return df_sub(a, b); }
  PP_D static df mul(df a, df b) { return df_mul(a, b); }
  PP_D static df neg(df a) { return df_neg(a); }
  PP_D static void mac(df &acc, df a, df b) { df_mac(acc, a, b); }
  PP_D static df fin(df a) { return df_norm(a); }
};

// ----------------------------------------------------------------------------
// Complex helpers over R
template <class R>
PP_D cx<R> cz() {
  return cx<R>{RT<R>::zero(), RT<R>::zero()};
}
template <class R>
PP_D cx<R> cadd(cx<R> a, cx<R> b) {
  return cx<R>{RT<R>::add(a.re, b.re), RT<R>::add(a.im, b.im)};
}
template <class R>
PP_D cx<R> csub(cx<R> a, cx<R> b) {
  return cx<R>{RT<R>::sub(a.re, b.re), RT<R>::sub(a.im, b.im)};
}
template <class R>
PP_D cx<R> cconj(cx<R> a) {
  return cx<R>{a.re, RT<R>::neg(a.im)};
}
template <class R>
PP_D cx<R> cmul(cx<R> a, cx<R> b) {
  cx<R> r = cz<R>();
  RT<R>::mac(r.re, a.re, b.re);
  RT<R>::mac(r.re, RT<R>::neg(a.im), b.im);
  RT<R>::mac(r.im, a.re, b.im);
  RT<R>::mac(r.im, a.im, b.re);
  return cx<R>{RT<R>::fin(r.re), RT<R>::fin(r.im)};
}
// acc += a*b (unnormalised accumulator)
template <class R>
PP_D void cmac(cx<R> &acc, cx<R> a, cx<R> b) {
  RT<R>::mac(acc.re, a.re, b.re);
  RT<R>::mac(acc.re, RT<R>::neg(a.im), b.im);
  RT<R>::mac(acc.im, a.re, b.im);
  RT<R>::mac(acc.im, a.im, b.re);
}
// acc += conj(a)*b
template <class R>
PP_D void cmacc(cx<R> &acc, cx<R> a, cx<R> b) {
  RT<R>::mac(acc.re, a.re, b.re);
  RT<R>::mac(acc.re, a.im, b.im);
  RT<R>::mac(acc.im, a.re, b.im);
  RT<R>::mac(acc.im, RT<R>::neg(a.im), b.re);
}
template <class R>
PP_D cx<R> cfin(cx<R> a) {
  return cx<R>{RT<R>::fin(a.re), RT<R>::fin(a.im)};
}
template <class R>
PP_D z64 cto64(cx<R> a) {
  return z64{RT<R>::to(a.re), RT<R>::to(a.im)};
}
template <class R>
PP_D cx<R> cfrom64(z64 a) {
  return cx<R>{RT<R>::from(a.re), RT<R>::from(a.im)};
}
template <class R>
PP_D cx<R> cfrom64(double re, double im) {
  return cx<R>{RT<R>::from(re), RT<R>::from(im)};
}

// FP64 complex helpers (host+device)
PP_HD z64 zmul(z64 a, z64 b) { return z64{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
PP_HD z64 zconj(z64 a) { return z64{a.re, -a.im}; }

// Error bits (match pzheevx INFO > 0 bits, diagonalize.F90:100-115)
#define PP_INFO_NOCONV 1
#define PP_INFO_NOORTH 2
#define PP_INFO_NOMEM 4
#define PP_INFO_NOTCOMP 8
#define PP_INFO_TIMEOUT 16
#define PP_INFO_NAN 32
