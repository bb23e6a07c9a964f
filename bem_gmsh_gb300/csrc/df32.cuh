// Double-float ("float-float") arithmetic for the far-field tiles.
//
// A value is the unevaluated sum h + l of two FP32 numbers with
// |l| <= ulp(h) / 2, about 48 significant bits.  GB300 issues FP32 at roughly
// sixty times its FP64 rate, so a far-field entry evaluated this way costs a
// few hundred FP32 instructions instead of ~60 FP64 ones.  The error-free
// transformations are the classical ones (Knuth's TwoSum, Dekker's
// Fast2Sum, and the FMA product error); the logarithm is table driven
// (Tang's argument reduction: log x = E log 2 + log c + log1p((m - c)/c)
// with a 129-entry table of centres c = 1 + i/128 and a series for log1p).
//
// Every product goes through mul_() so that no compiler contracts it into a
// fused multiply-add: the transformations need the rounded product.  The
// same source compiled on the host with contraction off gives bit-identical
// results, which the tests use.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD inline
#endif

namespace df {

struct f2 {
  float h, l;
};

DF_HD float mul_(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
DF_HD float add_(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
DF_HD float sub_(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
DF_HD float fma_(float a, float b, float c) { return fmaf(a, b, c); }

DF_HD uint32_t fbits(float x) {
#ifdef __CUDA_ARCH__
  return __float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}
DF_HD float ffrom(uint32_t u) {
#ifdef __CUDA_ARCH__
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}
DF_HD double dfrom(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}

DF_HD uint64_t dbits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}

// (float)(v * 2^s) on the integer pipes: the exponent field gets s added and
// the 52-bit fraction is rounded to 23 bits to nearest, ties to even.  Zeros
// give signed zeros; a result outside the normal FP32 range, or an infinite
// or NaN v, takes the FP64 multiply and conversion.
DF_HD float scale_to_f32(double v, int s) {
  const uint64_t b = dbits(v);
  const uint32_t sign = (uint32_t)(b >> 63) << 31;
  const int ex = (int)((b >> 52) & 0x7FF);
  const uint64_t m = b & 0xFFFFFFFFFFFFFull;
  if (ex == 0 && m == 0) return ffrom(sign);
  const int E = ex + s - 1023 + 127;
  if (ex == 0x7FF || E < 1 || E > 254) return (float)(v * dfrom((uint64_t)(1023 + s) << 52));
  const uint32_t top = (uint32_t)(m >> 29);
  const uint32_t rest = (uint32_t)(m & 0x1FFFFFFFu);
  uint32_t out = sign | ((uint32_t)E << 23) | top;
  if (rest > 0x10000000u || (rest == 0x10000000u && (top & 1u))) out += 1u;
  return ffrom(out);
}

// exact float of a small integer (|i| < 2^22) with one FP32 add (keeps the
// int-to-float conversion off the FP64/conversion pipe)
DF_HD float small_int_to_float(int i) { return sub_(ffrom(0x4B400000u + (uint32_t)i), 12582912.0f); }

// s + e == a + b exactly
DF_HD f2 two_sum(float a, float b) {
  const float s = add_(a, b);
  const float bb = sub_(s, a);
  const float e = add_(sub_(a, sub_(s, bb)), sub_(b, bb));
  return {s, e};
}
// requires |a| >= |b| (or a == 0)
DF_HD f2 fast_two_sum(float a, float b) {
  const float s = add_(a, b);
  return {s, sub_(b, sub_(s, a))};
}
DF_HD f2 two_prod(float a, float b) {
  const float p = mul_(a, b);
  return {p, fma_(a, b, -p)};
}

DF_HD f2 add(f2 a, f2 b) {
  const f2 s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, add_(s.l, add_(a.l, b.l)));
}
DF_HD f2 add_f(f2 a, float b) {
  const f2 s = two_sum(a.h, b);
  return fast_two_sum(s.h, add_(s.l, a.l));
}
DF_HD f2 neg(f2 a) { return {-a.h, -a.l}; }
DF_HD f2 mul(f2 a, f2 b) {
  const float p = mul_(a.h, b.h);
  float e = fma_(a.h, b.h, -p);
  e = fma_(a.h, b.l, e);
  e = fma_(a.l, b.h, e);
  return fast_two_sum(p, e);
}
DF_HD f2 mul_f(f2 a, float b) {
  const float p = mul_(a.h, b);
  float e = fma_(a.h, b, -p);
  e = fma_(a.l, b, e);
  return fast_two_sum(p, e);
}
DF_HD f2 sqr(f2 a) {
  const float p = mul_(a.h, a.h);
  float e = fma_(a.h, a.h, -p);
  e = fma_(add_(a.h, a.h), a.l, e);
  return fast_two_sum(p, e);
}
// a / b: correctly rounded reciprocal of b.h; the leading quotient is
// corrected once with its exact FMA remainder (Markstein), then the DF
// remainder of that quotient gives the low part
DF_HD f2 div(f2 a, f2 b) {
  const float r = 1.0f / b.h;
  float q1 = mul_(a.h, r);
  q1 = fma_(fma_(-q1, b.h, a.h), r, q1);
  const float p = mul_(q1, b.h);
  const float pe = fma_(q1, b.h, -p);
  const float rem = add_(sub_(sub_(a.h, p), pe), sub_(a.l, mul_(q1, b.l)));
  return fast_two_sum(q1, mul_(rem, r));
}

// exact split of a double into three floats (a + b + c == x for normal x)
DF_HD void split3(double x, float& a, float& b, float& c) {
  a = (float)x;
  const double r = x - (double)a;
  b = (float)r;
  c = (float)(r - (double)b);
}
DF_HD f2 from_double(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}

// xn - xs for coordinates given as exact three-float splits; the result is
// the DF rounding of the exact difference (relative error ~2^-48 however
// small the difference is compared with the coordinates)
DF_HD f2 diff3(float an, float bn, float cn, float as, float bs, float cs) {
  const f2 d1 = two_sum(an, -as);
  const f2 d2 = two_sum(bn, -bs);
  const f2 s = two_sum(d1.h, d2.h);
  const float rest = add_(add_(d1.l, d2.l), sub_(cn, cs));
  const f2 t = two_sum(s.h, add_(s.l, rest));
  return fast_two_sum(t.h, t.l);
}

// log table entry i (0..128): centre c = 1 + i/128, 1/c as hi + lo, log c as
// hi + lo
struct LogEntry {
  float rc_h, rc_l, lc_h, lc_l;
};
constexpr int kLogTable = 129;

// entry i in FP64 (log and reciprocal within an FP64 ulp, far below the
// 2^-48 of the split); the device builds its table with the same function
DF_HD LogEntry log_entry(int i) {
  const double c = 1.0 + i / 128.0;
  const double rc = 1.0 / c;
  const double lc = ::log(c);
  LogEntry e;
  e.rc_h = (float)rc;
  e.rc_l = (float)(rc - (double)e.rc_h);
  e.lc_h = (float)lc;
  e.lc_l = (float)(lc - (double)e.lc_h);
  return e;
}

// natural log of x = x.h + x.l (x.h positive and normal); error below
// 2^-46 max(|log x|, 1) (measured: 3.6 2^-48 at worst, from the final sums)
DF_HD f2 log(f2 x, const LogEntry* tab) {
  const uint32_t ih = fbits(x.h);
  const int E = (int)((ih >> 23) & 0xffu) - 127;
  const float m = ffrom((ih & 0x7fffffu) | 0x3f800000u);              // [1, 2)
  const float sc = ffrom((uint32_t)(127 - E) << 23);                   // 2^-E
  const int i = (int)((ih >> 15) & 0xffu);                             // top 8 fraction bits
  const int ic = (i + 1) >> 1;                                         // nearest centre
  const LogEntry T = tab[ic];
  const float c = add_(1.0f, mul_(small_int_to_float(ic), 0.0078125f));
  const float f = sub_(m, c);                                          // exact, |f| <= 2^-8
  // u = (f + x.l 2^-E) / c
  f2 u = two_prod(f, T.rc_h);
  u.l = fma_(f, T.rc_l, u.l);
  u.l = fma_(mul_(x.l, sc), T.rc_h, u.l);
  u = fast_two_sum(u.h, u.l);
  // log1p(u) = u - u^2/2 + u^3 (1/3 - u/4 + u^2/5 - u^3/6 + u^4/7)
  const f2 u2 = sqr(u);
  const float uh = u.h;
  float poly = fma_(uh, 0.142857142857142857f, -0.166666666666666667f);
  poly = fma_(uh, poly, 0.2f);
  poly = fma_(uh, poly, -0.25f);
  poly = fma_(uh, poly, 0.333333333333333333f);
  const float tail = mul_(mul_(u2.h, uh), poly);
  f2 l1 = add(u, f2{-0.5f * u2.h, -0.5f * u2.l});
  l1 = add_f(l1, tail);
  // E log 2 + log c
  const float ln2_h = 0.693147182464599609375f;          // 0x3f317218
  const float ln2_l = -1.9046542121259336e-09f;          // log 2 - ln2_h
  const float Ef = small_int_to_float(E);
  f2 el = two_prod(Ef, ln2_h);
  el.l = fma_(Ef, ln2_l, el.l);
  el = fast_two_sum(el.h, el.l);
  return add(add(el, f2{T.lc_h, T.lc_l}), l1);
}

// nearest double of h + l built with integer operations only (no FP64 or
// conversion pipe); a zero or subnormal leading part gives a signed zero
// (far-field entries are many orders above 2^-126), infinities and NaNs
// keep their class
DF_HD double to_double(f2 a) {
  const uint32_t ih = fbits(a.h);
  const uint32_t eh = (ih >> 23) & 0xffu;
  if (eh == 0u) return dfrom((uint64_t)(ih & 0x80000000u) << 32);
  if (eh == 255u)
    return dfrom(((uint64_t)(ih & 0x80000000u) << 32) | 0x7FF0000000000000ull | ((uint64_t)(ih & 0x7fffffu) << 29));
  uint64_t D = ((uint64_t)(ih & 0x80000000u) << 32) | ((uint64_t)(eh + 896u) << 52) |
               ((uint64_t)(ih & 0x7fffffu) << 29);
  const uint32_t il = fbits(a.l);
  const uint32_t el = (il >> 23) & 0xffu;
  if (el == 0u) return dfrom(D);
  const bool opp = ((ih ^ il) & 0x80000000u) != 0u;
  // l in units of the double ulp of h: Ml 2^(el - eh + 29)
  int sh = (int)el - (int)eh + 29;
  if (opp && (ih & 0x7fffffu) == 0u) sh += 1;  // result lies in the binade below
  const uint64_t Ml = (uint64_t)((il & 0x7fffffu) | 0x800000u);
  uint64_t k = 0;
  if (sh >= 0)
    k = Ml << sh;
  else if (sh > -25)
    k = (Ml + (1ull << (-sh - 1))) >> (-sh);
  D = opp ? D - k : D + k;
  return dfrom(D);
}

}  // namespace df
