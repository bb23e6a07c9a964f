// Device-side FP64 machinery for the near-singular and singular element
// integrals of the dense 2-D collocation assembly, restating the reference
// (Julia package `BEM`, paths relative to its project root):
//   shape functions       src/Core/Interpolation.jl:148-218
//   closest point         src/Core/Integration.jl:323-349, 1005-1033
//   complex pole          src/Core/Integration.jl:1117-1160
//   tanp3c map            src/Core/Integration.jl:1163-1365
//   interpolated Guiggiani src/Core/Integration.jl:1598-1845
//   kernels               src/Laplace/Fundamental.jl:19-25,
//                         src/Elasticity/Fundamental.jl:28-60
// Everything here is per-thread scalar code: one thread integrates one
// (collocation point, element) pair.  Arrays live in registers / local memory.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define BEM_MAXNN 6     // field nodes per element (degree <= 5)
#define BEM_MAXGEO 6    // CAD nodes per element
#define BEM_MAXNPG 32   // near-field Gauss rule
#define BEM_NINTERP 20  // Laurent interpolation nodes (ninterp default)
#define BEM_MAXMAP (2 * BEM_MAXNPG)

namespace bem {

constexpr double kPi = 3.141592653589793;
constexpr double kEps = 2.220446049250313e-16;

// Rule tables shared by every kernel of one assembly (passed by value).
struct Rules {
  int nn;    // field nodes per element (p+1)
  int ngeo;  // CAD nodes per element, 0 = geometry from the field nodes
  int npg;   // near-field Gauss rule size
  int pad_;
  double leg_x[BEM_MAXNN], leg_bw[BEM_MAXNN], leg_D[BEM_MAXNN * BEM_MAXNN];
  double geo_x[BEM_MAXGEO], geo_bw[BEM_MAXGEO], geo_D[BEM_MAXGEO * BEM_MAXGEO];
  double qsi[BEM_MAXNPG], w[BEM_MAXNPG];
  double gi_x[BEM_NINTERP], gi_w[BEM_NINTERP], gi_bw[BEM_NINTERP];
  double ew[BEM_MAXNN];  // element Gauss weights (elem_weight)
  // product-form weights 1 / prod_{j != i} (x_i - x_j) of the field and CAD
  // nodes (the barycentric weights above carry an arbitrary scale)
  double leg_pw[BEM_MAXNN], geo_pw[BEM_MAXGEO];
};

// Physics of one assembly.
struct Physics {
  int kind;  // 0 Laplace, 1 Kelvin
  int pad_;
  double k;        // Laplace conductivity
  double mu, nu;   // Kelvin shear modulus, effective Poisson ratio
};

// Device-resident FP64 geometry (structure of arrays).
struct GeomDev {
  int nt, n, ne, nn, ngeo, pad_;
  const double *px, *py;  // nt collocation points, boundary first
  const double *nx, *ny;  // n boundary normals
  const double *jac;      // n Jacobians at the nodes
  const double *elen;     // ne element lengths
  const double *gx, *gy;  // ne*ngeo CAD nodes
};

struct V2 {
  double x, y;
};

__device__ __forceinline__ double vnorm(double x, double y) { return sqrt(x * x + y * y); }

// interpolation_matrix row and L * Dmat (Interpolation.jl:148-178, 215-218)
__device__ __forceinline__ void shapefun(const double* nodes, const double* bw, const double* D, int n,
                                         double xx, double* L, double* dL) {
  double msum = 0.0;
  int exact = -1;
  for (int i = 0; i < n; ++i) {
    if (xx == nodes[i]) exact = i;
    L[i] = bw[i] / (xx - nodes[i]);
    msum += L[i];
  }
  if (msum == 0.0) {
    for (int i = 0; i < n; ++i) L[i] = 0.0;
  } else if (exact >= 0) {
    for (int i = 0; i < n; ++i) L[i] = 0.0;
    L[exact] = 1.0;
  } else {
    for (int i = 0; i < n; ++i) L[i] /= msum;
  }
  if (dL) {
    for (int j = 0; j < n; ++j) {
      double s = L[0] * D[j];
      for (int i = 1; i < n; ++i) s += L[i] * D[i * n + j];
      dL[j] = s;
    }
  }
}

// The same basis in product form, L_i(x) = w_i prod_{j != i} (x - x_j) with
// the product-form weights w_i = 1 / prod_{j != i} (x_i - x_j): no division
// (GB300 runs FP64 division as a long sequence on its small FP64 pipe); it
// differs from the barycentric form by rounding only (n <= 6 nodes on
// [-1, 1]).  Used per quadrature point of the element integrals.
__device__ __forceinline__ void shapefun_prod(const double* nodes, const double* bw, const double* D, int n,
                                              double xx, double* L, double* dL) {
  double d[BEM_MAXGEO > BEM_MAXNN ? BEM_MAXGEO : BEM_MAXNN];
  for (int i = 0; i < n; ++i) d[i] = xx - nodes[i];
  double pre = 1.0;
  for (int i = 0; i < n; ++i) {
    L[i] = bw[i] * pre;
    pre *= d[i];
  }
  double suf = 1.0;
  for (int i = n - 1; i >= 0; --i) {
    L[i] *= suf;
    suf *= d[i];
  }
  if (dL) {
    for (int j = 0; j < n; ++j) {
      double s = L[0] * D[j];
      for (int i = 1; i < n; ++i) s += L[i] * D[i * n + j];
      dL[j] = s;
    }
  }
}

__device__ __forceinline__ V2 comb(const double* L, const V2* p, int n) {
  V2 s{L[0] * p[0].x, L[0] * p[0].y};
  for (int k = 1; k < n; ++k) {
    s.x += L[k] * p[k].x;
    s.y += L[k] * p[k].y;
  }
  return s;
}

// --------------------------------------------------------------------------
// kernels
// --------------------------------------------------------------------------
__device__ __forceinline__ void laplace_UT(double kc, double rx, double ry, double nx, double ny,
                                           double& U, double& T) {
  double R2 = rx * rx + ry * ry;
  double inv2pi = 1.0 / (2 * kPi);
  U = -log(R2) * (0.5 * inv2pi / kc);
  T = (rx * nx + ry * ny) * (inv2pi / R2);
}

// row-major 2x2: U[2a+b], T[2a+b]
__device__ __forceinline__ void kelvin_UT(double mu, double nu, double rx, double ry, double nx,
                                          double ny, double* U, double* T) {
  double R2 = rx * rx + ry * ry;
  double R = sqrt(R2);
  double dr1 = rx / R, dr2 = ry / R;
  double drdn = dr1 * nx + dr2 * ny;
  double prod1 = 4 * kPi * (1 - nu);
  double prod2 = (3 - 4 * nu) * log(1 / R);
  double base = 2 * prod1 * mu;
  U[0] = (prod2 + dr1 * dr1) / base;
  U[1] = (dr1 * dr2) / base;
  U[2] = U[1];
  U[3] = (prod2 + dr2 * dr2) / base;
  double fat = 1 / (prod1 * R);
  double c = 1 - 2 * nu;
  T[0] = -drdn * (c + 2 * (dr1 * dr1)) * fat;
  T[3] = -drdn * (c + 2 * (dr2 * dr2)) * fat;
  T[1] = -(drdn * 2 * dr1 * dr2 - c * (dr1 * ny - dr2 * nx)) * fat;
  T[2] = -(drdn * 2 * dr1 * dr2 - c * (dr2 * nx - dr1 * ny)) * fat;
}

template <int NC>
__device__ __forceinline__ void eval_kernel(const Physics& ph, double rx, double ry, double nx,
                                            double ny, double* U, double* T) {
  if constexpr (NC == 1)
    laplace_UT(ph.k, rx, ry, nx, ny, U[0], T[0]);
  else
    kelvin_UT(ph.mu, ph.nu, rx, ry, nx, ny, U, T);
}

// Far nodal lumping of one (source, node) pair: kernel times J w.
template <int NC>
__device__ __forceinline__ void far_eval_f64(const Physics& ph, double rx, double ry, double nx,
                                             double ny, double wjk, double* U, double* T) {
  eval_kernel<NC>(ph, rx, ry, nx, ny, U, T);
  for (int c = 0; c < NC; ++c) {
    U[c] *= wjk;
    T[c] *= wjk;
  }
}

// --------------------------------------------------------------------------
// near test (Assembly_full.jl:736-754, Integration.jl:238-312), exact FP64
// --------------------------------------------------------------------------
// The near/far decision is discontinuous (integrated vs lumped value), and
// regular meshes put collocation points exactly on the cut (distance ==
// 1.5 L).  Every operation below is an explicit IEEE round-to-nearest
// multiply/add, never a fused multiply-add, so ties resolve exactly as in
// the reference's IEEE double arithmetic.
__device__ __forceinline__ double mul_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double sq2_(double x, double y) { return add_(mul_(x, x), mul_(y, y)); }

__device__ __forceinline__ double dist_chord(V2 p, V2 a, V2 b) {
  double abx = sub_(b.x, a.x), aby = sub_(b.y, a.y);
  double num = add_(mul_(sub_(p.x, a.x), abx), mul_(sub_(p.y, a.y), aby));
  double t = __ddiv_rn(num, add_(sq2_(abx, aby), kEps));
  t = fmin(fmax(t, 0.0), 1.0);
  double qx = add_(a.x, mul_(t, abx)), qy = add_(a.y, mul_(t, aby));
  return __dsqrt_rn(sq2_(sub_(p.x, qx), sub_(p.y, qy)));
}

__device__ __forceinline__ bool near_element(V2 pf, const V2* xg, int n, double L, double factor) {
  if (factor > 1e20) return true;
  double lim = mul_(factor, L);
  double lim2 = mul_(lim, lim);
  double dn2 = INFINITY;
  V2 lo = xg[0], hi = xg[0];
  for (int k = 0; k < n; ++k) {
    lo.x = fmin(lo.x, xg[k].x);
    lo.y = fmin(lo.y, xg[k].y);
    hi.x = fmax(hi.x, xg[k].x);
    hi.y = fmax(hi.y, xg[k].y);
    double d2 = sq2_(sub_(pf.x, xg[k].x), sub_(pf.y, xg[k].y));
    if (d2 < dn2) dn2 = d2;
  }
  if (dn2 < lim2) return true;
  double d2 = 0.0;
  if (pf.x < lo.x) { double t = sub_(lo.x, pf.x); d2 = add_(d2, mul_(t, t)); }
  else if (pf.x > hi.x) { double t = sub_(pf.x, hi.x); d2 = add_(d2, mul_(t, t)); }
  if (pf.y < lo.y) { double t = sub_(lo.y, pf.y); d2 = add_(d2, mul_(t, t)); }
  else if (pf.y > hi.y) { double t = sub_(pf.y, hi.y); d2 = add_(d2, mul_(t, t)); }
  if (__dsqrt_rn(d2) >= lim) return false;
  double d = INFINITY;
  if (n == 1) d = __dsqrt_rn(sq2_(sub_(pf.x, xg[0].x), sub_(pf.y, xg[0].y)));
  for (int k = 0; k + 1 < n; ++k) d = fmin(d, dist_chord(pf, xg[k], xg[k + 1]));
  return d < lim;
}

// --------------------------------------------------------------------------
// closest point (Integration.jl:323-349, 1005-1010, 1023-1033)
// --------------------------------------------------------------------------
__device__ inline double seed_1d(const Rules& R, const V2* nodes, int n, V2 pf) {
  double dx = nodes[n - 1].x - nodes[0].x, dy = nodes[n - 1].y - nodes[0].y;
  double nr = vnorm(dx, dy);
  double xi0 = (R.leg_x[n - 1] - R.leg_x[0]) * (dx * (pf.x - nodes[0].x) + dy * (pf.y - nodes[0].y)) /
                   (nr * nr + kEps) + R.leg_x[0];
  return fmin(fmax(xi0, -1.0), 1.0);
}

__device__ inline void closest_point_1d(const Rules& R, const V2* nodes, int n, V2 pf, double& xi_out,
                                 double& dist_out) {
  double xi = seed_1d(R, nodes, n, pf);
  double L[BEM_MAXNN], dL[BEM_MAXNN], d2L[BEM_MAXNN];
  for (int it = 0; it < 25; ++it) {
    shapefun(R.leg_x, R.leg_bw, R.leg_D, n, xi, L, dL);
    for (int j = 0; j < n; ++j) {
      double s = dL[0] * R.leg_D[j];
      for (int i = 1; i < n; ++i) s += dL[i] * R.leg_D[i * n + j];
      d2L[j] = s;
    }
    V2 x = comb(L, nodes, n), dx = comb(dL, nodes, n), d2x = comb(d2L, nodes, n);
    double rx = x.x - pf.x, ry = x.y - pf.y;
    double res = rx * dx.x + ry * dx.y;
    double J = (dx.x * dx.x + dx.y * dx.y) + (rx * d2x.x + ry * d2x.y);
    if (fabs(J) < 1e-30) break;
    double d = res / J;
    xi -= d;
    if (fabs(d) < 1e-14) break;
  }
  V2 xx;
  if (xi < -1 || xi > 1) {
    shapefun(R.leg_x, R.leg_bw, R.leg_D, n, -1.0, L, nullptr);
    V2 x0 = comb(L, nodes, n);
    shapefun(R.leg_x, R.leg_bw, R.leg_D, n, 1.0, L, nullptr);
    V2 x1 = comb(L, nodes, n);
    if (vnorm(x0.x - pf.x, x0.y - pf.y) <= vnorm(x1.x - pf.x, x1.y - pf.y)) { xi = -1.0; xx = x0; }
    else { xi = 1.0; xx = x1; }
  } else {
    shapefun(R.leg_x, R.leg_bw, R.leg_D, n, xi, L, nullptr);
    xx = comb(L, nodes, n);
  }
  xi_out = xi;
  dist_out = vnorm(xx.x - pf.x, xx.y - pf.y);
}

// --------------------------------------------------------------------------
// complex arithmetic for the pole
// --------------------------------------------------------------------------
struct C2 {
  double re, im;
};
__device__ __forceinline__ C2 cadd(C2 a, C2 b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ C2 csub(C2 a, C2 b) { return {a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ C2 cmul(C2 a, C2 b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__device__ __forceinline__ C2 cscale(C2 a, double s) { return {a.re * s, a.im * s}; }
__device__ __forceinline__ double cabs(C2 a) { return hypot(a.re, a.im); }
// Smith's algorithm
__device__ __forceinline__ C2 cdiv(C2 a, C2 b) {
  if (fabs(b.re) >= fabs(b.im)) {
    double r = b.im / b.re, d = b.re + b.im * r;
    return {(a.re + a.im * r) / d, (a.im - a.re * r) / d};
  }
  double r = b.re / b.im, d = b.re * r + b.im;
  return {(a.re * r + a.im) / d, (a.im * r - a.re) / d};
}
// principal square root
__device__ __forceinline__ C2 csqrt(C2 z) {
  if (z.re == 0.0 && z.im == 0.0) return {0.0, z.im};
  double r = hypot(z.re, z.im);
  if (z.re >= 0) {
    double t = sqrt(0.5 * (r + z.re));
    return {t, z.im / (2 * t)};
  }
  double t = sqrt(0.5 * (r - z.re));
  return {fabs(z.im) / (2 * t), copysign(t, z.im)};
}

// _complex_pole_1d (Integration.jl:1117-1160)
__device__ inline void complex_pole_1d(const Rules& R, const V2* nodes, int nN, V2 pf, double& z0,
                                double& e0) {
  C2 y{pf.x, pf.y};
  if (nN == 2) {
    double d = R.leg_x[1] - R.leg_x[0] + 1e-30;
    C2 B{(nodes[1].x - nodes[0].x) / d, (nodes[1].y - nodes[0].y) / d};
    C2 C = csub(C2{nodes[0].x, nodes[0].y}, cscale(B, R.leg_x[0]));
    if (cabs(B) < 1e-30) { z0 = 0.0; e0 = 1.0; return; }
    C2 r = cdiv(csub(y, C), B);
    z0 = r.re;
    e0 = fabs(r.im);
    return;
  }
  if (nN == 3) {
    const double* xs = R.leg_x;
    double a11 = xs[0] * xs[0], a12 = xs[0], a13 = 1;
    double a21 = xs[1] * xs[1], a22 = xs[1], a23 = 1;
    double a31 = xs[2] * xs[2], a32 = xs[2], a33 = 1;
    double det = a11 * (a22 * a33 - a23 * a32) - a12 * (a21 * a33 - a23 * a31) +
                 a13 * (a21 * a32 - a22 * a31);
    C2 Z0{nodes[0].x, nodes[0].y}, Z1{nodes[1].x, nodes[1].y}, Z2{nodes[2].x, nodes[2].y};
    C2 A = cscale(cadd(cadd(cscale(Z0, a22 * a33 - a23 * a32), cscale(Z1, a13 * a32 - a12 * a33)),
                       cscale(Z2, a12 * a23 - a13 * a22)), 1.0 / det);
    C2 B = cscale(cadd(cadd(cscale(Z0, a23 * a31 - a21 * a33), cscale(Z1, a11 * a33 - a13 * a31)),
                       cscale(Z2, a13 * a21 - a11 * a23)), 1.0 / det);
    C2 C = cscale(cadd(cadd(cscale(Z0, a21 * a32 - a22 * a31), cscale(Z1, a12 * a31 - a11 * a32)),
                       cscale(Z2, a11 * a22 - a12 * a21)), 1.0 / det);
    if (cabs(A) < 1e-14) {
      if (cabs(B) < 1e-30) { z0 = 0.0; e0 = 1.0; return; }
      C2 r = cdiv(csub(y, C), B);
      z0 = r.re;
      e0 = fabs(r.im);
      return;
    }
    C2 disc = csqrt(csub(cmul(B, B), cscale(cmul(A, csub(C, y)), 4.0)));
    C2 twoA = cscale(A, 2.0);
    C2 mB{-B.re, -B.im};
    C2 r1 = cdiv(cadd(mB, disc), twoA);
    C2 r2 = cdiv(csub(mB, disc), twoA);
    C2 r = fabs(r1.im) <= fabs(r2.im) ? r1 : r2;
    z0 = r.re;
    e0 = fabs(r.im);
    return;
  }
  double a, dist;
  closest_point_1d(R, nodes, nN, pf, a, dist);
  double L[BEM_MAXNN], dL[BEM_MAXNN];
  shapefun(R.leg_x, R.leg_bw, R.leg_D, nN, a, L, dL);
  V2 dx = comb(dL, nodes, nN);
  z0 = a;
  e0 = dist / fmax(vnorm(dx.x, dx.y), 1e-14);
}

// --------------------------------------------------------------------------
// tanp3c map (Integration.jl:1163-1365).  Writes up to 2*npg nodes; returns
// the count.
// --------------------------------------------------------------------------
__device__ __forceinline__ bool eq41_collinear(double z0, double e0, bool has_den, double den) {
  if (fabs(z0) <= 1) return false;
  if (fabs(e0) < 1e-8) return true;
  if (has_den && fabs(den) < 1e-10) return true;
  return false;
}

__device__ inline int eq41_real_pole(const Rules& R, double z0, double* x, double* wx) {
  int m = R.npg;
  if (fabs(z0) <= 1) {
    for (int i = 0; i < m; ++i) { x[i] = R.qsi[i]; wx[i] = R.w[i]; }
    return m;
  }
  double A = z0 * z0 - 1, B = -z0;
  for (int i = 0; i < m; ++i) {
    double d = R.qsi[i] - B;
    x[i] = z0 - A / d;
    wx[i] = R.w[i] * (A / (d * d));
  }
  return m;
}

__device__ inline int tangenttrans(const Rules& R, double z0, double e0, double* x, double* wx) {
  if (eq41_collinear(z0, e0, false, 0.0)) return eq41_real_pole(R, z0, x, wx);
  e0 = fmax(e0, 1e-14);
  double tp = atan((1 - z0) / e0), tm = atan((-1 - z0) / e0);
  double den = tp - tm;
  if (eq41_collinear(z0, e0, true, den)) return eq41_real_pole(R, z0, x, wx);
  double A = 2.0 * e0 / den, B = -(tp + tm) / den;
  double halfpi = kPi / 2 - 1e-8;
  for (int i = 0; i < R.npg; ++i) {
    double phi = fmin(fmax(e0 * (R.qsi[i] - B) / A, -halfpi), halfpi);
    double tn = tan(phi);
    x[i] = z0 + e0 * tn;
    wx[i] = R.w[i] * ((e0 * e0 / A) * (1 + tn * tn));
  }
  return R.npg;
}

__device__ __forceinline__ double jsign(double v) { return v > 0 ? 1.0 : (v < 0 ? -1.0 : 0.0); }

// _p3c_inv_pole (Integration.jl:1220-1270)
__device__ inline void p3c_inv_pole(double z0, double e0, double& zt, double& et) {
  if (fabs(e0) < 1e-14) {
    double x = z0;
    for (int it = 0; it < 25; ++it) {
      double g = x * x * x - 3 * z0 * (x * x) + 3 * x - z0;
      double gp = 3 * (x * x) - 6 * z0 * x + 3;
      if (fabs(gp) < 1e-30) break;
      x -= g / gp;
      if (fabs(g) < 1e-14) break;
    }
    zt = x;
    et = 0.0;
    return;
  }
  double e = cbrt(fabs(e0)) * jsign(e0);
  for (int it = 0; it < 20; ++it) {
    double g = 2 * (e * e * e) - 3 * e0 * (e * e) - e0;
    double gp = 6 * (e * e) - 6 * e0 * e;
    if (fabs(gp) < 1e-30) break;
    e -= g / gp;
  }
  e += cbrt(e0) * sqrt(z0 * z0 + e0 * e0);
  double z = z0;
  for (int it = 0; it < 30; ++it) {
    double den = 1 + 3 * (z * z) + 3 * (e * e);
    double nz = (3 + z * z + 3 * (e * e)) * z;
    double ne = 2 * (e * e * e);
    double f1 = nz / den - z0, f2 = ne / den - e0;
    if (fabs(f1) + fabs(f2) < 1e-14) break;
    double denz = 6 * z, dene = 6 * e;
    double nz_z = 3 + 3 * (z * z) + 3 * (e * e);
    double nz_e = 6 * e * z;
    double ne_e = 6 * (e * e);
    double den2 = den * den;
    double j11 = (nz_z * den - nz * denz) / den2;
    double j12 = (nz_e * den - nz * dene) / den2;
    double j21 = (0.0 * den - ne * denz) / den2;
    double j22 = (ne_e * den - ne * dene) / den2;
    double det = j11 * j22 - j12 * j21;
    if (fabs(det) < 1e-30) break;
    z -= (j22 * f1 - j12 * f2) / det;
    e -= (-j21 * f1 + j11 * f2) / det;
  }
  zt = z;
  et = e;
}

// p3c map of the npg rule, then the affine chart u = mid + h s and the
// tangent map; appends to x/wx at offset `off`.  (_p3ctrans,
// _tanp3c_compose, _tanp3c_half)
__device__ inline int p3c_tangent_piece(const Rules& R, double spole, double mid, double h, double z0,
                                 double e0, double At, double Bt, double* x, double* wx, int off) {
  double zt, et;
  p3c_inv_pole(spole, 1e-14, zt, et);
  double den = 1 + 3 * (zt * zt) + 3 * (et * et);
  double A = 3.0 / den;
  double B = (3 + zt * zt) * zt / den;
  double halfpi = kPi / 2 - 1e-8;
  for (int i = 0; i < R.npg; ++i) {
    double s = R.qsi[i];
    double ds = s - zt;
    double sm = A * ((ds * ds * ds) / 3 + (et * et) * s) + B;
    double ws = R.w[i] * (A * ((ds * ds) + et * et));
    double ut = mid + h * sm;
    ws = ws * h;
    double th = fmin(fmax((ut - Bt) / At, -halfpi), halfpi);
    double tn = tan(th);
    x[off + i] = z0 + e0 * tn;
    wx[off + i] = ws * ((e0 / At) * (1 + tn * tn));
  }
  return R.npg;
}

__device__ inline int p3ctrans(const Rules& R, double z0, double e0, double* x, double* wx) {
  double zt, et;
  p3c_inv_pole(z0, e0, zt, et);
  double den = 1 + 3 * (zt * zt) + 3 * (et * et);
  double A = 3.0 / den, B = (3 + zt * zt) * zt / den;
  for (int i = 0; i < R.npg; ++i) {
    double s = R.qsi[i], ds = s - zt;
    x[i] = A * ((ds * ds * ds) / 3 + (et * et) * s) + B;
    wx[i] = R.w[i] * (A * ((ds * ds) + et * et));
  }
  return R.npg;
}

// _tanp3ctrans.  A split half narrower than 1e-14 contributes no nodes (the
// reference gives it the full-interval tangent rule, counting the element
// twice; see Integration.jl:1349).
__device__ inline int tanp3ctrans(const Rules& R, double z0, double e0, double* x, double* wx) {
  if (eq41_collinear(z0, e0, false, 0.0)) return eq41_real_pole(R, z0, x, wx);
  e0 = fmax(e0, 1e-14);
  double ap = atan((1 - z0) / e0), am = atan((1 + z0) / e0);
  double den = ap + am;
  if (eq41_collinear(z0, e0, true, den)) return eq41_real_pole(R, z0, x, wx);
  if (fabs(den) < 1e-30) return p3ctrans(R, z0, e0, x, wx);
  double At = 2.0 / den;
  double Bt = -At * (ap - am) / 2.0;
  double uL = Bt - At * kPi / 2, uR = Bt + At * kPi / 2;
  if (fabs(z0) < 1 && -1 < Bt && Bt < 1) {
    int m = 0;
    // left half [-1, Bt]
    {
      double lo = -1.0, hi = Bt;
      double mid = (hi + lo) / 2, h = (hi - lo) / 2;
      if (h > 1e-14) m += p3c_tangent_piece(R, (uL - mid) / h, mid, h, z0, e0, At, Bt, x, wx, m);
    }
    {
      double lo = Bt, hi = 1.0;
      double mid = (hi + lo) / 2, h = (hi - lo) / 2;
      if (h > 1e-14) m += p3c_tangent_piece(R, (uR - mid) / h, mid, h, z0, e0, At, Bt, x, wx, m);
    }
    return m;
  }
  double upole = (z0 >= 1) ? uL : uR;
  return p3c_tangent_piece(R, upole, 0.0, 1.0, z0, e0, At, Bt, x, wx, 0);
}

// --------------------------------------------------------------------------
// element geometry at a parent point (_shape_geom, Assembly_full.jl:608-627)
// --------------------------------------------------------------------------
__device__ __forceinline__ void shape_geom(const Rules& R, const V2* nodes, const V2* geo, double xi,
                                           double* N, V2& pg, V2& dx) {
  double dN[BEM_MAXNN];
  if (R.ngeo > 0) {
    // field basis without derivatives: the geometry comes from the CAD nodes
    shapefun_prod(R.leg_x, R.leg_pw, R.leg_D, R.nn, xi, N, nullptr);
    double Ng[BEM_MAXGEO], dNg[BEM_MAXGEO];
    shapefun_prod(R.geo_x, R.geo_pw, R.geo_D, R.ngeo, xi, Ng, dNg);
    pg = V2{0.0, 0.0};
    dx = V2{0.0, 0.0};
    for (int k = 0; k < R.ngeo; ++k) {
      pg.x += Ng[k] * geo[k].x;
      pg.y += Ng[k] * geo[k].y;
      dx.x += dNg[k] * geo[k].x;
      dx.y += dNg[k] * geo[k].y;
    }
    return;
  }
  shapefun_prod(R.leg_x, R.leg_pw, R.leg_D, R.nn, xi, N, dN);
  pg = V2{0.0, 0.0};
  dx = V2{0.0, 0.0};
  for (int k = 0; k < R.nn; ++k) {
    pg.x += N[k] * nodes[k].x;
    pg.y += N[k] * nodes[k].y;
    dx.x += dN[k] * nodes[k].x;
    dx.y += dN[k] * nodes[k].y;
  }
}

__device__ __forceinline__ void load_element(const GeomDev& g, int e, V2* nodes, V2* geo) {
  for (int k = 0; k < g.nn; ++k) nodes[k] = V2{g.px[e * g.nn + k], g.py[e * g.nn + k]};
  for (int k = 0; k < g.ngeo; ++k) geo[k] = V2{g.gx[e * g.ngeo + k], g.gy[e * g.ngeo + k]};
}

// Near-singular element integral (_quad_geom + _accumulate_kernels!,
// Assembly_full.jl:649-713).  h, g: [node k][component c] with NC components.
template <int NC>
__device__ inline void integrate_near(const Rules& R, const Physics& ph, const V2* nodes, const V2* geo,
                               V2 pf, V2 nref, double* h, double* g) {
  const int nn = R.nn;
  double eta[BEM_MAXMAP], ww[BEM_MAXMAP];
  double z0, e0;
  complex_pole_1d(R, nodes, nn, pf, z0, e0);
  int m = tanp3ctrans(R, z0, e0, eta, ww);
  for (int c = 0; c < nn * NC; ++c) h[c] = g[c] = 0.0;
  double flip = 1.0;
  for (int i = 0; i < m; ++i) {
    double N[BEM_MAXNN];
    V2 pg, dx;
    shape_geom(R, nodes, geo, eta[i], N, pg, dx);
    double rx = pg.x - pf.x, ry = pg.y - pf.y;
    double J = vnorm(dx.x, dx.y);
    const double invJ = 1.0 / J;
    double tx = dx.x * invJ, ty = dx.y * invJ;
    double nxq = ty, nyq = -tx;
    if (i == 0 && (nxq * nref.x + nyq * nref.y) < 0) flip = -1.0;
    nxq *= flip;
    nyq *= flip;
    double U[4], T[4];
    eval_kernel<NC>(ph, rx, ry, nxq, nyq, U, T);
    double wi = J * ww[i];
    for (int j = 0; j < nn; ++j) {
      double Nj = N[j] * wi;
      for (int c = 0; c < NC; ++c) {
        h[j * NC + c] += T[c] * Nj;
        g[j * NC + c] += U[c] * Nj;
      }
    }
  }
}

// --------------------------------------------------------------------------
// interpolated Guiggiani (Assembly_full.jl:397-457, Integration.jl:1598-1845)
// --------------------------------------------------------------------------
__device__ __forceinline__ double hfp1(double a) { return log(fabs((1 - a) / (1 + a))); }
__device__ __forceinline__ double log_parent(double a) {
  return (1 - a) * log(fabs(1 - a)) + (1 + a) * log(fabs(1 + a)) - 2;
}

// On-element integral for source pf at parent coordinate a, orders (0, -1):
// G by the log least-squares fit, H by the CPV cascade.
template <int NC>
__device__ inline void integrate_singular(const Rules& R, const Physics& ph, const V2* nodes,
                                   const V2* geo, V2 pf, double a, V2 nref, double* h, double* g) {
  const int nn = R.nn;
  const int K = nn * NC;
  a = fmin(fmax(a, -0.9999999999999999), 0.9999999999999999);
  // _interp_rule: drop Gauss nodes within 1e-12 of a, rebuild weights
  double xi[BEM_NINTERP], wq[BEM_NINTERP], Ni[BEM_NINTERP], d[BEM_NINTERP];
  int m = 0;
  bool dropped = false;
  for (int i = 0; i < BEM_NINTERP; ++i) {
    if (fabs(R.gi_x[i] - a) <= 1e-12) { dropped = true; continue; }
    xi[m] = R.gi_x[i];
    wq[m] = R.gi_w[i];
    ++m;
  }
  {
    double msum = 0.0;
    int exact = -1;
    for (int i = 0; i < m; ++i) {
      double bw;
      if (!dropped) {
        bw = R.gi_bw[i];
      } else {
        bw = 1.0;
        for (int j = 0; j < i; ++j) bw *= xi[i] - xi[j];
        for (int j = i + 1; j < m; ++j) bw *= xi[i] - xi[j];
        bw = 1.0 / bw;
      }
      double dd = a - xi[i];
      if (dd == 0) exact = i;
      Ni[i] = bw / dd;
      msum += Ni[i];
    }
    if (exact >= 0) {
      for (int i = 0; i < m; ++i) Ni[i] = 0.0;
      Ni[exact] = 1.0;
    } else {
      double invs = 1.0 / msum;
      for (int i = 0; i < m; ++i) Ni[i] *= invs;
    }
    for (int i = 0; i < m; ++i) d[i] = xi[i] - a;
  }
  double invd[BEM_NINTERP];
  for (int i = 0; i < m; ++i) invd[i] = 1.0 / d[i];
  // samples
  double Fg[BEM_NINTERP * BEM_MAXNN * NC], Fh[BEM_NINTERP * BEM_MAXNN * NC];
  for (int i = 0; i < m; ++i) {
    double N[BEM_MAXNN];
    V2 pg, dx;
    shape_geom(R, nodes, geo, xi[i], N, pg, dx);
    double J = vnorm(dx.x, dx.y);
    double rx = pg.x - pf.x, ry = pg.y - pf.y;
    bool ok = !(J < 1e-30) && !(vnorm(rx, ry) < 1e-30);
    double U[4] = {0, 0, 0, 0}, T[4] = {0, 0, 0, 0};
    if (ok) {
      const double invJ = 1.0 / J;
      double nxq = dx.y * invJ, nyq = -(dx.x * invJ);
      if (nxq * nref.x + nyq * nref.y < 0) { nxq = -nxq; nyq = -nyq; }
      eval_kernel<NC>(ph, rx, ry, nxq, nyq, U, T);
    }
    for (int j = 0; j < nn; ++j) {
      double NjJ = ok ? N[j] * J : 0.0;
      for (int c = 0; c < NC; ++c) {
        Fg[i * K + j * NC + c] = ok ? U[c] * NjJ : 0.0;
        Fh[i * K + j * NC + c] = ok ? T[c] * NjJ : 0.0;
      }
    }
  }
  // G: log coefficient by least squares (_interp_log_coeff); log |d_i| is
  // formed once per sample (FP64 logs dominate this routine)
  double lgd[BEM_NINTERP];
  double sL = 0.0, sL2 = 0.0;
  int nused = 0;
  for (int i = 0; i < m; ++i) {
    double adi = fabs(d[i]);
    lgd[i] = log(adi);
    if (adi < 1e-14) continue;
    double lg = lgd[i];
    sL += lg;
    sL2 += lg * lg;
    ++nused;
  }
  double detA = sL2 * nused - sL * sL;
  bool fit = nused >= 2 && !(fabs(detA) < 1e-30);
  double hp1 = hfp1(a), lp = log_parent(a);
  for (int c = 0; c < K; ++c) {
    double Fm1 = Ni[0] * (Fg[c] * d[0]);
    for (int i = 1; i < m; ++i) Fm1 += Ni[i] * (Fg[i * K + c] * d[i]);
    double sW = 0.0, sWL = 0.0;
    for (int i = 0; i < m; ++i) {
      double adi = fabs(d[i]);
      if (adi < 1e-14) continue;
      double lg = lgd[i];
      double wi = Fg[i * K + c] - Fm1 * invd[i];
      sW += wi;
      sWL += wi * lg;
    }
    double F0 = fit ? (nused * sWL - sL * sW) / detA : 0.0;
    double acc = wq[0] * (Fg[c] - Fm1 * invd[0] - F0 * lgd[0]);
    for (int i = 1; i < m; ++i) acc += wq[i] * (Fg[i * K + c] - Fm1 * invd[i] - F0 * lgd[i]);
    g[c] = acc + (Fm1 * hp1 + F0 * lp);
  }
  // H: CPV cascade (_interp_cascade, order -1)
  for (int c = 0; c < K; ++c) {
    double F1 = Ni[0] * (Fh[c] * d[0]);
    for (int i = 1; i < m; ++i) F1 += Ni[i] * (Fh[i * K + c] * d[i]);
    double acc = wq[0] * (Fh[c] - F1 * invd[0]);
    for (int i = 1; i < m; ++i) acc += wq[i] * (Fh[i * K + c] - F1 * invd[i]);
    h[c] = acc + F1 * hp1;
  }
}

}  // namespace bem
