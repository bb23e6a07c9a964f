// Correctly rounded elementary functions and exactly specified IEEE
// arithmetic, identical on the host and on the GPU.
//
// The reference's near-singular quadrature (the tanp3c map of
// src/Core/Integration.jl:1291-1365 with the complex pole of :1117-1160)
// amplifies rounding: for a collocation point on an element next to the one
// being integrated, the pole sits just outside [-1, 1] with a small
// imaginary part, the tangent map's constants At, Bt grow like 1/eta0, and a
// one-ulp change of one atan or tan result moves the element integral by up
// to ~5e-5 relative.  Two implementations of that map agree to the last
// bits only if every operation on the way is the same IEEE operation on the
// same operands.  So the map is evaluated here with:
//   * `ieee`, a double whose + - * / sqrt are explicit round-to-nearest
//     operations (device: __dadd_rn & co., which the compiler never fuses
//     into FMAs; host: plain operators, compiled with -ffp-contract=off), and
//   * atan, tan and cbrt correctly rounded: evaluated in double-double
//     arithmetic (about 100 significant bits; Dekker's and Knuth's exact
//     sum and product, with fma for the product's error) and rounded once.
//     A correctly rounded function has one possible result, whatever the
//     platform: the GPU, the CPU and any other correctly rounding library
//     agree bit for bit (a wrong rounding needs the exact value within
//     about 2^-100 of a rounding boundary).
//
// Methods:
//   atan: atan(x) = pi/2 - atan(1/x) for |x| > 1, then
//         atan(y) = atan(j/16) + atan((y - j/16) / (1 + y j/16)) with
//         atan(j/16) a table and the Taylor series t - t^3/3 + t^5/5 - ...
//         for |t| <= 1/32.
//   tan:  x - k pi/2 with pi/2 in three doubles (Cody and Waite), then
//         r = j/32 + s with |s| <= 1/64 and the addition theorem
//         tan(j/32 + s) = (T_j + tan s) / (1 - T_j tan s); T_j = tan(j/32)
//         is a table and tan s its Taylor series (coefficients from the
//         Bernoulli numbers); tan(x) = -1/tan(r) for odd k.
//   cbrt: one Newton step y - (y^3 - x) / (3 y^2) in double-double from the
//         platform's cbrt (whose error is at most a few ulp).
// The constants (pi/2 in three parts, atan(j/16), tan(j/32), 1/(2k+1) and
// the tan series coefficients rounded to double-double) were computed with
// 400-bit arithmetic; tests/test_crmath_cpu.py recomputes and checks them.
// GB300's FP64 pipe is a small fraction of its FP32 rate, so the operations
// are few: one reciprocal per quotient, sums without the cancellation
// handling they do not need (the Legendre recurrence, which cancels, uses
// the fully accurate sum).
#pragma once
#include <cmath>

#ifdef __CUDACC__
#define BEM_HD __host__ __device__ __forceinline__
#else
#define BEM_HD inline
#endif

namespace bem {
namespace crm {

// --------------------------------------------------------------------------
// round-to-nearest IEEE operations that are never contracted or reordered
// --------------------------------------------------------------------------
BEM_HD double add(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
BEM_HD double sub(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
BEM_HD double mul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
BEM_HD double dvd(double a, double b) {
#ifdef __CUDA_ARCH__
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}
BEM_HD double sqr(double a) {
#ifdef __CUDA_ARCH__
  return __dsqrt_rn(a);
#else
  return ::sqrt(a);
#endif
}
BEM_HD double fmaf_(double a, double b, double c) {
#ifdef __CUDA_ARCH__
  return __fma_rn(a, b, c);
#else
  return ::fma(a, b, c);
#endif
}

// A double whose arithmetic is exactly the IEEE operation written: code in
// `ieee` evaluates the same operations, in the same order, on any compiler
// and either processor.
struct ieee {
  double v;
  BEM_HD ieee() : v(0.0) {}
  BEM_HD ieee(double x) : v(x) {}
  BEM_HD explicit operator double() const { return v; }
};
BEM_HD ieee operator+(ieee a, ieee b) { return ieee(add(a.v, b.v)); }
BEM_HD ieee operator-(ieee a, ieee b) { return ieee(sub(a.v, b.v)); }
BEM_HD ieee operator*(ieee a, ieee b) { return ieee(mul(a.v, b.v)); }
BEM_HD ieee operator/(ieee a, ieee b) { return ieee(dvd(a.v, b.v)); }
BEM_HD ieee operator-(ieee a) { return ieee(-a.v); }
BEM_HD ieee& operator+=(ieee& a, ieee b) { a = a + b; return a; }
BEM_HD ieee& operator-=(ieee& a, ieee b) { a = a - b; return a; }
BEM_HD bool operator<(ieee a, ieee b) { return a.v < b.v; }
BEM_HD bool operator<=(ieee a, ieee b) { return a.v <= b.v; }
BEM_HD bool operator>(ieee a, ieee b) { return a.v > b.v; }
BEM_HD bool operator>=(ieee a, ieee b) { return a.v >= b.v; }
BEM_HD bool operator==(ieee a, ieee b) { return a.v == b.v; }
BEM_HD bool operator!=(ieee a, ieee b) { return a.v != b.v; }
BEM_HD ieee abs(ieee a) { return ieee(::fabs(a.v)); }
BEM_HD ieee sqrt(ieee a) { return ieee(sqr(a.v)); }
BEM_HD ieee max(ieee a, ieee b) { return a.v > b.v ? a : (b.v > a.v ? b : a); }
// Julia's clamp(x, lo, hi) for non-NaN x
BEM_HD ieee clamp(ieee x, ieee lo, ieee hi) { return x > hi ? hi : (x < lo ? lo : x); }
BEM_HD ieee copysign(ieee a, ieee s) { return ieee(::copysign(a.v, s.v)); }

// --------------------------------------------------------------------------
// double-double arithmetic
// --------------------------------------------------------------------------
struct dd {
  double hi, lo;
};
BEM_HD dd two_sum(double a, double b) {
  double s = add(a, b);
  double bb = sub(s, a);
  return {s, add(sub(a, sub(s, bb)), sub(b, bb))};
}
BEM_HD dd fast_two_sum(double a, double b) {  // |a| >= |b| or a == 0
  double s = add(a, b);
  return {s, sub(b, sub(s, a))};
}
BEM_HD dd two_prod(double a, double b) {
  double p = mul(a, b);
  return {p, fmaf_(a, b, -p)};
}
// Sum without cancellation: every call below adds terms of like sign or
// of very different size, where this form keeps ~2^-104 relative accuracy
// with half the operations of the fully accurate sum.
BEM_HD dd dadd(dd x, dd y) {
  dd s = two_sum(x.hi, y.hi);
  return fast_two_sum(s.hi, add(s.lo, add(x.lo, y.lo)));
}
BEM_HD dd dneg(dd x) { return {-x.hi, -x.lo}; }
BEM_HD dd dsub(dd x, dd y) { return dadd(x, dneg(y)); }
// fully accurate sum (~2^-106 relative to the result also under cancellation)
BEM_HD dd dadd_acc(dd x, dd y) {
  dd s = two_sum(x.hi, y.hi);
  dd t = two_sum(x.lo, y.lo);
  s = fast_two_sum(s.hi, add(s.lo, t.hi));
  return fast_two_sum(s.hi, add(s.lo, t.lo));
}
BEM_HD dd dsub_acc(dd x, dd y) { return dadd_acc(x, dneg(y)); }
BEM_HD dd dmul(dd x, dd y) {
  dd p = two_prod(x.hi, y.hi);
  return fast_two_sum(p.hi, add(p.lo, fmaf_(x.hi, y.lo, mul(x.lo, y.hi))));
}
BEM_HD dd dmul_d(dd x, double b) {
  dd p = two_prod(x.hi, b);
  return fast_two_sum(p.hi, fmaf_(x.lo, b, p.lo));
}
// x / y: one reciprocal, a first quotient and one correction from the exact
// remainder (x.hi - q1 y.hi is exact: q1 y.hi is within a factor 2 of x.hi)
BEM_HD dd ddiv(dd x, dd y) {
  const double inv = dvd(1.0, y.hi);
  const double q1 = mul(x.hi, inv);
  dd p = two_prod(q1, y.hi);
  double r = sub(sub(x.hi, p.hi), p.lo);
  r = add(r, x.lo);
  r = fmaf_(-q1, y.lo, r);
  return fast_two_sum(q1, mul(r, inv));
}
// the double nearest to x.hi + x.lo
BEM_HD double round_dd(dd x) { return add(x.hi, x.lo); }

// pi / 2 in three parts
#define BEM_PIO2_0 0x1.921fb54442d18p+0
#define BEM_PIO2_1 0x1.1a62633145c07p-54
#define BEM_PIO2_2 -0x1.f1976b7ed8fbcp-110

#ifdef __CUDA_ARCH__
#define BEM_CRM_TABLE static __device__ const
#else
#define BEM_CRM_TABLE static const
#endif

// --------------------------------------------------------------------------
// atan
// --------------------------------------------------------------------------
// atan(j/16), j = 0..16, as double-double
BEM_CRM_TABLE double kAtanTab[17][2] = {
    {0x0.0p+0, 0x0.0p+0},
    {0x1.ff55bb72cfdeap-5, -0x1.c934d86d23f1dp-60},
    {0x1.fd5ba9aac2f6ep-4, -0x1.cd37686760c17p-59},
    {0x1.7b97b4bce5b02p-3, 0x1.347b0b4f881cap-58},
    {0x1.f5b75f92c80ddp-3, 0x1.8ab6e3cf7afbdp-57},
    {0x1.362773707ebccp-2, -0x1.963a544b672d8p-57},
    {0x1.6f61941e4def1p-2, -0x1.c63aae6f6e918p-56},
    {0x1.a64eec3cc23fdp-2, -0x1.24dec1b50b7ffp-56},
    {0x1.dac670561bb4fp-2, 0x1.a2b7f222f65e2p-56},
    {0x1.0657e94db30d0p-1, -0x1.d5b495f6349e6p-56},
    {0x1.1e00babdefeb4p-1, -0x1.928df287a668fp-58},
    {0x1.345f01cce37bbp-1, 0x1.1021137c71102p-55},
    {0x1.4978fa3269ee1p-1, 0x1.2419a87f2a458p-56},
    {0x1.5d58987169b18p-1, 0x1.0028e4bc5e7cap-57},
    {0x1.700a7c5784634p-1, -0x1.8c34d25aadef6p-56},
    {0x1.819d0b7158a4dp-1, -0x1.bf76229d3b917p-56},
    {0x1.921fb54442d18p-1, 0x1.1a62633145c07p-55},
};
// 1/(2k+1): k = 1..5 as double-double, k = 6..11 as double
BEM_CRM_TABLE double kOddInv[5][2] = {
    {0x1.5555555555555p-2, 0x1.5555555555555p-56},
    {0x1.999999999999ap-3, -0x1.999999999999ap-57},
    {0x1.2492492492492p-3, 0x1.2492492492492p-57},
    {0x1.c71c71c71c71cp-4, 0x1.c71c71c71c71cp-58},
    {0x1.745d1745d1746p-4, -0x1.745d1745d1746p-59},
};
#define BEM_ODD13 0x1.3b13b13b13b14p-4
#define BEM_ODD15 0x1.1111111111111p-4
#define BEM_ODD17 0x1.e1e1e1e1e1e1ep-5
#define BEM_ODD19 0x1.af286bca1af28p-5
#define BEM_ODD21 0x1.8618618618618p-5
#define BEM_ODD23 0x1.642c8590b2164p-5

BEM_HD double cr_atan(double x) {
  if (!(x == x)) return x;
  double a = ::fabs(x);
  if (a < 0x1p-27) return x;  // atan(x) = x (1 - x^2/3 + ...) rounds to x
  if (a == INFINITY) return ::copysign(BEM_PIO2_0, x);
  const bool inv = a > 1.0;
  dd y = inv ? ddiv(dd{1.0, 0.0}, dd{a, 0.0}) : dd{a, 0.0};
  // atan(y) = atan(c) + atan((y - c) / (1 + y c)), c = j/16 nearest to y
  const int j = (int)::rint(mul(y.hi, 16.0));
  const double c = mul((double)j, 0.0625);
  dd num = fast_two_sum(sub(y.hi, c), y.lo);  // y.hi - c is exact (Sterbenz)
  dd den = dadd(dd{1.0, 0.0}, dmul_d(y, c));
  dd t = ddiv(num, den);  // |t| <= 1/32
  // atan t = t - t^3/3 + t^5/5 - ...: 11 terms reach 2^-110 relative
  dd z = dmul(t, t);
  double q = BEM_ODD23;
  q = fmaf_(-z.hi, q, BEM_ODD21);
  q = fmaf_(-z.hi, q, BEM_ODD19);
  q = fmaf_(-z.hi, q, BEM_ODD17);
  q = fmaf_(-z.hi, q, BEM_ODD15);
  q = fmaf_(-z.hi, q, BEM_ODD13);
  dd pq = dsub(dd{kOddInv[4][0], kOddInv[4][1]}, dmul_d(z, q));
  for (int k = 3; k >= 0; --k) pq = dsub(dd{kOddInv[k][0], kOddInv[k][1]}, dmul(z, pq));
  dd at = dsub(t, dmul(dmul(t, z), pq));
  dd r = dadd(dd{kAtanTab[j][0], kAtanTab[j][1]}, at);
  if (inv) r = dsub(dadd(dd{BEM_PIO2_0, 0.0}, dd{BEM_PIO2_1, BEM_PIO2_2}), r);
  return ::copysign(round_dd(r), x);
}

// --------------------------------------------------------------------------
// tan
// --------------------------------------------------------------------------
// tan(j/32), j = 0..25, as double-double
BEM_CRM_TABLE double kTanTab[26][2] = {
    {0x0.0p+0, 0x0.0p+0},
    {0x1.00155777aec08p-5, 0x1.5f48b25fa0262p-59},
    {0x1.005577854df01p-4, -0x1.f35b10671bea1p-58},
    {0x1.8121042019d39p-4, 0x1.e53de54163d36p-58},
    {0x1.01577af1511a5p-3, -0x1.fba60a478d2b0p-59},
    {0x1.42a13df7bb968p-3, -0x1.981948de81ac0p-57},
    {0x1.84906f1132568p-3, 0x1.20efcd2f809c3p-60},
    {0x1.c7490a1d1e12dp-3, 0x1.d2fc0e48d3694p-58},
    {0x1.05785a43c4c56p-2, -0x1.9c6bfe7769a3dp-58},
    {0x1.27d78b40b7704p-2, 0x1.f391de0df335dp-56},
    {0x1.4ad71ed51ce39p-2, -0x1.b8c42b22fff4bp-56},
    {0x1.6e8d85a6493e1p-2, -0x1.80e8ea578b238p-56},
    {0x1.9312d859bf8b0p-2, -0x1.de9ddeb7d4180p-57},
    {0x1.b8811e4d009c3p-2, -0x1.2f8192327ea6bp-58},
    {0x1.def49eaab37a1p-2, 0x1.1e48c7a265428p-56},
    {0x1.03461f08a685dp-1, -0x1.71d22a449a2eap-55},
    {0x1.17b4f5bf3474ap-1, 0x1.0c5e59201e209p-55},
    {0x1.2cd98fea0ab88p-1, 0x1.bf004c33955cbp-57},
    {0x1.42c8ba0e9537ap-1, -0x1.1817d3747956ap-56},
    {0x1.5999a9e0f5129p-1, -0x1.ebf504ca1c5d4p-56},
    {0x1.7166689d41ef0p-1, -0x1.f44ffce65ed2bp-55},
    {0x1.8a4c52ca75a77p-1, 0x1.4d66e6bea4d61p-55},
    {0x1.a46cb2be6a0b2p-1, -0x1.29a64ecb1df2ep-56},
    {0x1.bfed7cca66b49p-1, 0x1.8d237cd4d9245p-55},
    {0x1.dcfa36110eeecp-1, -0x1.f3cf665127fd2p-57},
    {0x1.fbc511df5917fp-1, 0x1.4e6ef3dde2f07p-55},
};
// Taylor coefficients of tan: 1/3, 2/15, 17/315 (double-double), then
// 62/2835, 1382/155925, 21844/6081075, 929569/638512875 (double)
#define BEM_TC1_HI 0x1.5555555555555p-2
#define BEM_TC1_LO 0x1.5555555555555p-56
#define BEM_TC2_HI 0x1.1111111111111p-3
#define BEM_TC2_LO 0x1.1111111111111p-59
#define BEM_TC3_HI 0x1.ba1ba1ba1ba1cp-5
#define BEM_TC3_LO -0x1.7917917917918p-59
#define BEM_TC4 0x1.664f4882c10fap-6
#define BEM_TC5 0x1.226e355e6c23dp-7
#define BEM_TC6 0x1.d6d3d0e157de0p-9
#define BEM_TC7 0x1.7da36452b75e3p-10

// tan(r) (odd = false) or -1/tan(r) (odd = true) of a double-double
// argument |r| <= pi/4 (+ a few ulp)
BEM_HD dd tan_reduced(dd r, bool odd) {
  const bool neg = r.hi < 0;
  if (neg) r = dneg(r);
  int j = (int)::rint(mul(r.hi, 32.0));
  if (j > 25) j = 25;
  const double c = mul((double)j, 0.03125);
  dd s = fast_two_sum(sub(r.hi, c), r.lo);  // r.hi - j/32 is exact (Sterbenz)
  dd z = dmul(s, s);
  double q = BEM_TC7;
  q = fmaf_(z.hi, q, BEM_TC6);
  q = fmaf_(z.hi, q, BEM_TC5);
  q = fmaf_(z.hi, q, BEM_TC4);
  dd p = dadd(dd{BEM_TC3_HI, BEM_TC3_LO}, dmul_d(z, q));
  p = dadd(dd{BEM_TC2_HI, BEM_TC2_LO}, dmul(z, p));
  p = dadd(dd{BEM_TC1_HI, BEM_TC1_LO}, dmul(z, p));
  dd t = dadd(s, dmul(dmul(s, z), p));  // tan s
  // tan(c + s) = (T + t) / (1 - T t); its negative reciprocal swaps them
  dd num = t, den{1.0, 0.0};
  if (j > 0) {
    dd T{kTanTab[j][0], kTanTab[j][1]};
    num = dadd(T, t);
    den = dsub(dd{1.0, 0.0}, dmul(T, t));
  }
  dd res = odd ? dneg(ddiv(den, num)) : (j > 0 ? ddiv(num, den) : num);
  return neg ? dneg(res) : res;
}

BEM_HD double cr_tan(double x) {
  if (!(x == x) || ::fabs(x) == INFINITY) return x - x;
  if (::fabs(x) < 0x1p-27) return x;  // tan(x) = x (1 + x^2/3 + ...) rounds to x
  if (::fabs(x) <= 0x1.921fb54442d18p-1) return round_dd(tan_reduced(dd{x, 0.0}, false));
  // r = x - k pi/2 with pi/2 in three parts (|k| < 2^20)
  const double k = ::rint(mul(x, 0x1.45f306dc9c883p-1));  // x * 2/pi
  dd r;
  if (::fabs(k) == 1.0) {
    r = two_sum(sub(x, mul(k, BEM_PIO2_0)), -mul(k, BEM_PIO2_1));  // x - k P0 is exact (Sterbenz)
    r = fast_two_sum(r.hi, add(r.lo, -mul(k, BEM_PIO2_2)));
  } else {
    r = dadd_acc(dd{x, 0.0}, dneg(two_prod(k, BEM_PIO2_0)));
    r = dadd_acc(r, dneg(two_prod(k, BEM_PIO2_1)));
    r = dadd_acc(r, dd{-mul(k, BEM_PIO2_2), 0.0});
  }
  const long long ki = (long long)k;
  return round_dd(tan_reduced(r, (ki & 1) != 0));
}

// --------------------------------------------------------------------------
// cbrt
// --------------------------------------------------------------------------
BEM_HD double cr_cbrt(double x) {
  if (!(x == x) || x == 0.0 || ::fabs(x) == INFINITY) return x;
  const double a = ::fabs(x);
  const double y = ::cbrt(a);
  dd y3 = dmul_d(two_prod(y, y), y);
  dd d = dsub(y3, dd{a, 0.0});
  const double corr = dvd(d.hi, mul(3.0, mul(y, y)));
  return ::copysign(round_dd(two_sum(y, -corr)), x);
}

// --------------------------------------------------------------------------
// Gauss-Legendre rule, nodes and weights correctly rounded: Newton on the
// three-term recurrence of P_n in double-double, ascending nodes.  (The
// reference calls FastGaussQuadrature's `gausslegendre`, a third-party
// package, at src/Core/Assembly_full.jl:720 and src/Core/Integration.jl:1599.)
// --------------------------------------------------------------------------
BEM_HD void legendre_eval(int n, dd z, dd& pn, dd& dpn) {
  dd p1{1.0, 0.0}, p2{0.0, 0.0};
  for (int j = 1; j <= n; ++j) {
    dd p3 = p2;
    p2 = p1;
    p1 = ddiv(dsub_acc(dmul_d(dmul(z, p2), (double)(2 * j - 1)), dmul_d(p3, (double)(j - 1))),
              dd{(double)j, 0.0});
  }
  // P_n'(z) = n (z P_n - P_{n-1}) / (z^2 - 1)
  dpn = ddiv(dmul_d(dsub_acc(dmul(z, p1), p2), (double)n), dsub_acc(dmul(z, z), dd{1.0, 0.0}));
  pn = p1;
}

inline void gauss_legendre_cr(int n, double* x, double* w) {
  const int m = (n + 1) / 2;
  for (int i = 0; i < m; ++i) {
    // largest root first: cos(pi (i + 3/4) / (n + 1/2)), refined in double
    double z0 = std::cos(3.141592653589793 * (i + 0.75) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z0 * p2 - (j - 1.0) * p3) / j;
      }
      double dp = n * (z0 * p1 - p2) / (z0 * z0 - 1.0);
      double dz = p1 / dp;
      z0 -= dz;
      if (::fabs(dz) <= 1e-15 * ::fabs(z0) + 1e-300) break;
    }
    dd z{z0, 0.0}, pn, dpn;
    if (n % 2 == 1 && i == m - 1) {
      z = dd{0.0, 0.0};  // the middle node of an odd rule
    } else {
      for (int it = 0; it < 3; ++it) {
        legendre_eval(n, z, pn, dpn);
        z = dsub_acc(z, ddiv(pn, dpn));
      }
    }
    legendre_eval(n, z, pn, dpn);
    // w = 2 / ((1 - z^2) P_n'(z)^2)
    dd wd = ddiv(dd{2.0, 0.0}, dmul(dsub_acc(dd{1.0, 0.0}, dmul(z, z)), dmul(dpn, dpn)));
    const double zr = round_dd(z), wr = round_dd(wd);
    x[n - 1 - i] = zr;
    x[i] = -zr;
    w[i] = wr;
    w[n - 1 - i] = wr;
  }
  if (n % 2 == 1) x[n / 2] = 0.0;
}

}  // namespace crm
}  // namespace bem
