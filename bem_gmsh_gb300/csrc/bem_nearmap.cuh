// The near-singular quadrature map of the reference, evaluated with exactly
// specified IEEE arithmetic (bem_crmath.cuh) so that the GPU and a CPU
// restatement of the same operations produce the same bits:
//   complex pole          src/Core/Integration.jl:1117-1160 (+ _fit_quad_complex)
//   eq. (41) collinear    src/Core/Integration.jl:1163-1217
//   p3c pole and map      src/Core/Integration.jl:1219-1288
//   tanp3c                src/Core/Integration.jl:1290-1365
// Every expression keeps the reference's order of evaluation (Julia evaluates
// a*b+c as two rounded operations, left to right; x^2 and x^3 are x*x and
// x*x*x).  Complex arithmetic restates the algorithms Julia uses for
// Complex{Float64}: the product (ac - bd, ad + bc); the quotient by Baudin
// and Smith's robust variant of Smith's method ("A robust complex division
// in Scilab", 2012), without its over/underflow rescaling, which operands of
// element-size magnitude never reach; the square root by Kahan's method
// ("Branch cuts for complex elementary functions", 1987), without its
// rescaling for the same reason.
//
// The functions are templates over the rule type: anything with members
// npg, qsi[], w[] (near-field Gauss rule) and leg_x[] (element nodes).
#pragma once
#include "bem_crmath.cuh"

namespace bem {
namespace nm {

using crm::ieee;

struct cx {
  ieee re, im;
};
BEM_HD cx operator+(cx a, cx b) { return {a.re + b.re, a.im + b.im}; }
BEM_HD cx operator-(cx a, cx b) { return {a.re - b.re, a.im - b.im}; }
BEM_HD cx operator-(cx a) { return {-a.re, -a.im}; }
BEM_HD cx operator*(cx a, cx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
BEM_HD cx operator*(ieee s, cx a) { return {s * a.re, s * a.im}; }
BEM_HD cx operator/(cx a, ieee s) { return {a.re / s, a.im / s}; }

// (a + ib) / (c + id), c >= |d| case of the robust quotient
BEM_HD void cdiv_half(ieee a, ieee b, ieee c, ieee d, ieee& p, ieee& q) {
  ieee r = d / c;
  ieee t = ieee(1.0) / (c + d * r);
  if (r != ieee(0.0)) {
    ieee br = b * r;
    p = br != ieee(0.0) ? (a + br) * t : a * t + (b * t) * r;
    ieee ar = -a * r;
    q = ar != ieee(0.0) ? (b + ar) * t : b * t + ((-a) * t) * r;
  } else {
    p = (a + d * (b / c)) * t;
    q = (b + d * ((-a) / c)) * t;
  }
}
BEM_HD cx operator/(cx x, cx y) {
  ieee p, q;
  if (abs(y.im) <= abs(y.re)) {
    cdiv_half(x.re, x.im, y.re, y.im, p, q);
  } else {
    cdiv_half(x.im, x.re, y.im, y.re, p, q);
    q = -q;
  }
  return {p, q};
}
BEM_HD cx csqrt(cx z) {
  ieee x = z.re, y = z.im;
  if (x == ieee(0.0) && y == ieee(0.0)) return {ieee(0.0), y};
  ieee rho = x * x + y * y;
  rho = abs(x) + sqrt(rho);
  rho = rho + rho;
  rho = sqrt(rho) * ieee(0.5);
  ieee xi = rho, eta = y;
  if (rho != ieee(0.0)) {
    eta = (eta / rho) / ieee(2.0);
    if (x < ieee(0.0)) {
      xi = abs(eta);
      eta = copysign(rho, y);
    }
  }
  return {xi, eta};
}
BEM_HD ieee cabs_(cx a) { return sqrt(a.re * a.re + a.im * a.im); }

// _complex_pole_1d for 2 and 3 element nodes; returns false for other
// node counts (the caller then takes the closest-point branch).
template <class RuleT>
BEM_HD bool complex_pole(const RuleT& R, const double* nx, const double* ny, int nN, double pfx, double pfy,
                         double& z0, double& e0) {
  const cx y{ieee(pfx), ieee(pfy)};
  if (nN == 2) {
    const ieee x0 = R.leg_x[0], x1 = R.leg_x[1];
    const cx Z0{ieee(nx[0]), ieee(ny[0])}, Z1{ieee(nx[1]), ieee(ny[1])};
    cx B = (Z1 - Z0) / (x1 - x0 + ieee(1e-30));
    cx C = Z0 - x0 * B;  // B * xi (complex times real)
    if (cabs_(B) < ieee(1e-30)) { z0 = 0.0; e0 = 1.0; return true; }
    cx r = (y - C) / B;
    z0 = r.re.v;
    e0 = ::fabs(r.im.v);
    return true;
  }
  if (nN != 3) return false;
  // Vandermonde [xi^2 xi 1] \ Z: the 3x3 solve by cofactors over the
  // determinant (the closed form StaticArrays uses for 3x3 systems)
  const ieee x0 = R.leg_x[0], x1 = R.leg_x[1], x2 = R.leg_x[2];
  const ieee a11 = x0 * x0, a12 = x0, a13 = 1.0;
  const ieee a21 = x1 * x1, a22 = x1, a23 = 1.0;
  const ieee a31 = x2 * x2, a32 = x2, a33 = 1.0;
  const ieee det = a11 * (a22 * a33 - a23 * a32) - a12 * (a21 * a33 - a23 * a31) + a13 * (a21 * a32 - a22 * a31);
  const cx Z0{ieee(nx[0]), ieee(ny[0])}, Z1{ieee(nx[1]), ieee(ny[1])}, Z2{ieee(nx[2]), ieee(ny[2])};
  cx A = ((a22 * a33 - a23 * a32) * Z0 + (a13 * a32 - a12 * a33) * Z1 + (a12 * a23 - a13 * a22) * Z2) / det;
  cx B = ((a23 * a31 - a21 * a33) * Z0 + (a11 * a33 - a13 * a31) * Z1 + (a13 * a21 - a11 * a23) * Z2) / det;
  cx C = ((a21 * a32 - a22 * a31) * Z0 + (a12 * a31 - a11 * a32) * Z1 + (a11 * a22 - a12 * a21) * Z2) / det;
  if (cabs_(A) < ieee(1e-14)) {
    if (cabs_(B) < ieee(1e-30)) { z0 = 0.0; e0 = 1.0; return true; }
    cx r = (y - C) / B;
    z0 = r.re.v;
    e0 = ::fabs(r.im.v);
    return true;
  }
  cx disc = csqrt(B * B - (ieee(4.0) * A) * (C - y));
  cx r1 = (-B + disc) / (ieee(2.0) * A);
  cx r2 = (-B - disc) / (ieee(2.0) * A);
  cx r = abs(r1.im) <= abs(r2.im) ? r1 : r2;
  z0 = r.re.v;
  e0 = ::fabs(r.im.v);
  return true;
}

// _eq41_collinear
BEM_HD bool eq41_collinear(ieee z0, ieee e0, bool has_den, ieee den) {
  if (abs(z0) <= ieee(1.0)) return false;
  if (abs(e0) < ieee(1e-8)) return true;
  if (has_den && abs(den) < ieee(1e-10)) return true;
  return false;
}

// _eq41_real_pole (Moebius map of a collinear real pole)
template <class RuleT>
BEM_HD int eq41_real_pole(const RuleT& R, ieee z0, double* x, double* wx) {
  const int m = R.npg;
  if (abs(z0) <= ieee(1.0)) {
    for (int i = 0; i < m; ++i) { x[i] = R.qsi[i]; wx[i] = R.w[i]; }
    return m;
  }
  ieee A = z0 * z0 - ieee(1.0), B = -z0;
  for (int i = 0; i < m; ++i) {
    ieee d = ieee(R.qsi[i]) - B;
    x[i] = (z0 - A / d).v;
    wx[i] = (ieee(R.w[i]) * (A / (d * d))).v;
  }
  return m;
}

// _tangenttrans (eq. 41)
template <class RuleT>
BEM_HD int tangenttrans(const RuleT& R, ieee z0, ieee e0, double* x, double* wx) {
  if (eq41_collinear(z0, e0, false, ieee(0.0))) return eq41_real_pole(R, z0, x, wx);
  e0 = max(e0, ieee(1e-14));
  ieee tp = crm::cr_atan(((ieee(1.0) - z0) / e0).v);
  ieee tm = crm::cr_atan(((ieee(-1.0) - z0) / e0).v);
  ieee den = tp - tm;
  if (eq41_collinear(z0, e0, true, den)) return eq41_real_pole(R, z0, x, wx);
  ieee A = ieee(2.0) * e0 / den;
  ieee B = -(tp + tm) / den;
  const ieee halfpi = ieee(3.141592653589793) / ieee(2.0) - ieee(1e-8);
  for (int i = 0; i < R.npg; ++i) {
    ieee phi = clamp(e0 * (ieee(R.qsi[i]) - B) / A, -halfpi, halfpi);
    ieee tn = crm::cr_tan(phi.v);
    x[i] = (z0 + e0 * tn).v;
    wx[i] = (ieee(R.w[i]) * ((e0 * e0 / A) * (ieee(1.0) + tn * tn))).v;
  }
  return R.npg;
}

BEM_HD ieee jsign(ieee v) { return v > ieee(0.0) ? ieee(1.0) : (v < ieee(0.0) ? ieee(-1.0) : ieee(0.0)); }

// _p3c_inv_pole: the p3c pole (zt, et) of (z0, e0), Newton on eq. (65)
BEM_HD void p3c_inv_pole(ieee z0, ieee e0, ieee& zt, ieee& et) {
  if (abs(e0) < ieee(1e-14)) {
    ieee x = z0;
    for (int it = 0; it < 25; ++it) {
      ieee g = x * x * x - ieee(3.0) * z0 * (x * x) + ieee(3.0) * x - z0;
      ieee gp = ieee(3.0) * (x * x) - ieee(6.0) * z0 * x + ieee(3.0);
      if (abs(gp) < ieee(1e-30)) break;
      x -= g / gp;
      if (abs(g) < ieee(1e-14)) break;
    }
    zt = x;
    et = 0.0;
    return;
  }
  ieee e = ieee(crm::cr_cbrt(abs(e0).v)) * jsign(e0);
  for (int it = 0; it < 20; ++it) {
    ieee g = ieee(2.0) * (e * e * e) - ieee(3.0) * e0 * (e * e) - e0;
    ieee gp = ieee(6.0) * (e * e) - ieee(6.0) * e0 * e;
    if (abs(gp) < ieee(1e-30)) break;
    e -= g / gp;
  }
  e += ieee(crm::cr_cbrt(e0.v)) * sqrt(z0 * z0 + e0 * e0);
  ieee z = z0;
  for (int it = 0; it < 30; ++it) {
    ieee den = ieee(1.0) + ieee(3.0) * (z * z) + ieee(3.0) * (e * e);
    ieee nz = (ieee(3.0) + z * z + ieee(3.0) * (e * e)) * z;
    ieee ne = ieee(2.0) * (e * e * e);
    ieee f1 = nz / den - z0, f2 = ne / den - e0;
    if (abs(f1) + abs(f2) < ieee(1e-14)) break;
    ieee denz = ieee(6.0) * z, dene = ieee(6.0) * e;
    ieee nz_z = ieee(3.0) + ieee(3.0) * (z * z) + ieee(3.0) * (e * e);
    ieee nz_e = ieee(6.0) * e * z;
    ieee ne_z = 0.0;
    ieee ne_e = ieee(6.0) * (e * e);
    ieee den2 = den * den;
    ieee j11 = (nz_z * den - nz * denz) / den2;
    ieee j12 = (nz_e * den - nz * dene) / den2;
    ieee j21 = (ne_z * den - ne * denz) / den2;
    ieee j22 = (ne_e * den - ne * dene) / den2;
    ieee det = j11 * j22 - j12 * j21;
    if (abs(det) < ieee(1e-30)) break;
    z -= (j22 * f1 - j12 * f2) / det;
    e -= (-j21 * f1 + j11 * f2) / det;
  }
  zt = z;
  et = e;
}

// _p3ctrans
template <class RuleT>
BEM_HD int p3ctrans(const RuleT& R, ieee z0, ieee e0, double* x, double* wx) {
  ieee zt, et;
  p3c_inv_pole(z0, e0, zt, et);
  ieee den = ieee(1.0) + ieee(3.0) * (zt * zt) + ieee(3.0) * (et * et);
  ieee A = ieee(3.0) / den, B = (ieee(3.0) + zt * zt) * zt / den;
  for (int i = 0; i < R.npg; ++i) {
    ieee s = R.qsi[i], ds = s - zt;
    x[i] = (A * ((ds * ds * ds) / ieee(3.0) + (et * et) * s) + B).v;
    wx[i] = (ieee(R.w[i]) * (A * ((ds * ds) + et * et))).v;
  }
  return R.npg;
}

// p3c about the tangent map's pole in the chart u = mid + h s, then the
// tangent map; appends npg nodes at x + off (_tanp3c_compose with mid = 0,
// h = 1, and _tanp3c_half)
template <class RuleT>
BEM_HD int p3c_tangent_piece(const RuleT& R, ieee spole, ieee mid, ieee h, bool chart, ieee z0, ieee e0,
                             ieee At, ieee Bt, double* x, double* wx, int off) {
  ieee zt, et;
  p3c_inv_pole(spole, ieee(1e-14), zt, et);
  ieee den = ieee(1.0) + ieee(3.0) * (zt * zt) + ieee(3.0) * (et * et);
  ieee A = ieee(3.0) / den;
  ieee B = (ieee(3.0) + zt * zt) * zt / den;
  const ieee halfpi = ieee(3.141592653589793) / ieee(2.0) - ieee(1e-8);
  for (int i = 0; i < R.npg; ++i) {
    ieee s = R.qsi[i];
    ieee ds = s - zt;
    ieee ut = A * ((ds * ds * ds) / ieee(3.0) + (et * et) * s) + B;
    ieee ws = ieee(R.w[i]) * (A * ((ds * ds) + et * et));
    if (chart) {
      ut = mid + h * ut;
      ws = ws * h;
    }
    ieee th = clamp((ut - Bt) / At, -halfpi, halfpi);
    ieee tn = crm::cr_tan(th.v);
    x[off + i] = (z0 + e0 * tn).v;
    wx[off + i] = (ws * ((e0 / At) * (ieee(1.0) + tn * tn))).v;
  }
  return R.npg;
}

// _tanp3ctrans.  Writes up to 2 npg nodes; returns the count.  A split half
// narrower than 1e-14 contributes no nodes: the reference gives it the
// full-interval tangent rule (src/Core/Integration.jl:1349), counting the
// element twice, which makes its result jump with the last bit of zeta0
// near +-1.
template <class RuleT>
BEM_HD int tanp3ctrans(const RuleT& R, double z0d, double e0d, double* x, double* wx) {
  ieee z0 = z0d, e0 = e0d;
  if (eq41_collinear(z0, e0, false, ieee(0.0))) return eq41_real_pole(R, z0, x, wx);
  e0 = max(e0, ieee(1e-14));
  ieee ap = crm::cr_atan(((ieee(1.0) - z0) / e0).v);
  ieee am = crm::cr_atan(((ieee(1.0) + z0) / e0).v);
  ieee den = ap + am;
  if (eq41_collinear(z0, e0, true, den)) return eq41_real_pole(R, z0, x, wx);
  if (abs(den) < ieee(1e-30)) return p3ctrans(R, z0, e0, x, wx);
  ieee At = ieee(2.0) / den;
  ieee Bt = -At * (ap - am) / ieee(2.0);
  ieee uL = Bt - At * ieee(3.141592653589793) / ieee(2.0);
  ieee uR = Bt + At * ieee(3.141592653589793) / ieee(2.0);
  if (abs(z0) < ieee(1.0) && ieee(-1.0) < Bt && Bt < ieee(1.0)) {
    int m = 0;
    {  // left half [-1, Bt]
      ieee lo = -1.0, hi = Bt;
      ieee mid = (hi + lo) / ieee(2.0), h = (hi - lo) / ieee(2.0);
      if (h > ieee(1e-14)) m += p3c_tangent_piece(R, (uL - mid) / h, mid, h, true, z0, e0, At, Bt, x, wx, m);
    }
    {  // right half [Bt, 1]
      ieee lo = Bt, hi = 1.0;
      ieee mid = (hi + lo) / ieee(2.0), h = (hi - lo) / ieee(2.0);
      if (h > ieee(1e-14)) m += p3c_tangent_piece(R, (uR - mid) / h, mid, h, true, z0, e0, At, Bt, x, wx, m);
    }
    return m;
  }
  ieee upole = (z0 >= ieee(1.0)) ? uL : uR;
  return p3c_tangent_piece(R, upole, ieee(0.0), ieee(1.0), false, z0, e0, At, Bt, x, wx, 0);
}

}  // namespace nm
}  // namespace bem
