// FP64 CPU oracle for the dense 2-D BEM collocation path of the Julia package
// `BEM` (l-s-campos/BEM_gmsh).  TEST INFRASTRUCTURE ONLY: this file is the
// checker that the CUDA library is compared against.  It is loaded by tests/,
// by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, and by
// nothing else.  The product library never links or calls it.
//
// It restates, function by function, the reference's Float64 algorithm.  Every
// function cites the reference file:line it follows (paths are relative to the
// reference project root).  Summation orders follow the Julia loops so that
// the oracle agrees with the reference to a few ulps.  Build it with
// -ffp-contract=off: Julia does not fuse a*b+c into an FMA.
//
// Elementary functions on the near-singular map (atan, tan, cbrt) and the
// Gauss-Legendre rules are correctly rounded here: evaluated in IEEE quad
// precision (113-bit; __float128 with libquadmath on x86-64, long double on
// aarch64) and rounded once to double.  The reference's tanp3c map turns a
// one-ulp change of one of these values into up to ~5e-5 relative change of
// an element integral, so its result depends on the libm that evaluates it;
// a correctly rounded value is the one result every correctly rounding
// library returns (the reference's Julia libm, < 1 ulp, agrees with it for
// all but a small fraction of arguments).  Complex arithmetic on that path
// follows the algorithms of Julia's Complex{Float64} (product ac - bd,
// ad + bc; Baudin-Smith robust quotient; Kahan's square root).
//
// Layout conventions (same as the C-ABI of the CUDA library):
//   * elements are discontinuous: element e owns boundary nodes
//     e*(p+1) .. e*(p+1)+p, collocation points are boundary nodes first
//     (0..n-1) then internal points (n..nt-1);
//   * matrices are column-major (Julia layout), H is rows x rows, G is
//     rows x cols with rows = dof*nt, cols = dof*n (dof = 1 Laplace, 2 Kelvin).

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#if defined(__x86_64__) || defined(__i386__)
#include <quadmath.h>
typedef __float128 qreal;
static inline qreal q_atan(qreal x) { return atanq(x); }
static inline qreal q_tan(qreal x) { return tanq(x); }
static inline qreal q_cbrt(qreal x) { return cbrtq(x); }
static inline qreal q_cos(qreal x) { return cosq(x); }
static inline qreal q_fabs(qreal x) { return fabsq(x); }
#else
static_assert(LDBL_MANT_DIG == 113, "the oracle needs IEEE quad precision long double on this platform");
typedef long double qreal;
static inline qreal q_atan(qreal x) { return atanl(x); }
static inline qreal q_tan(qreal x) { return tanl(x); }
static inline qreal q_cbrt(qreal x) { return cbrtl(x); }
static inline qreal q_cos(qreal x) { return cosl(x); }
static inline qreal q_fabs(qreal x) { return fabsl(x); }
#endif

namespace {

constexpr double kPi = 3.141592653589793;

// correctly rounded atan, tan, cbrt (quad precision rounded once)
double cr_atan(double x) { return (double)q_atan((qreal)x); }
double cr_tan(double x) { return (double)q_tan((qreal)x); }
double cr_cbrt(double x) { return (double)q_cbrt((qreal)x); }
constexpr double kEps = 2.220446049250313e-16;  // eps(Float64)
using cplx = std::complex<double>;

// ---------------------------------------------------------------------------
// Gauss-Legendre rule.  FastGaussQuadrature 1.3.0 `gausslegendre(n)` (a
// third-party dependency, called at src/Core/Assembly_full.jl:720,
// src/Core/Input.jl:88, src/Core/Integration.jl:1599).  Restated as Newton on
// the Legendre three-term recurrence in quad precision, ascending nodes,
// nodes and weights correctly rounded.
// ---------------------------------------------------------------------------
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const int m = (n + 1) / 2;
  const qreal pi = (qreal)3.14159265358979323846264338327950288L;
  for (int i = 0; i < m; ++i) {
    qreal z = q_cos(pi * ((qreal)i + (qreal)0.75) / ((qreal)n + (qreal)0.5));
    qreal pp = 0;
    auto eval = [&](qreal zz, qreal& p1, qreal& dp) {
      qreal a = 1, b = 0;
      for (int j = 1; j <= n; ++j) {
        qreal c = b;
        b = a;
        a = ((2 * (qreal)j - 1) * zz * b - ((qreal)j - 1) * c) / (qreal)j;
      }
      p1 = a;
      dp = (qreal)n * (zz * a - b) / (zz * zz - 1);
    };
    if (n % 2 == 1 && i == m - 1) {
      z = 0;
    } else {
      for (int it = 0; it < 100; ++it) {
        qreal p1;
        eval(z, p1, pp);
        qreal dz = p1 / pp;
        z -= dz;
        if (q_fabs(dz) <= (qreal)1e-33 * q_fabs(z)) break;
      }
    }
    qreal p1;
    eval(z, p1, pp);
    double xi = (double)z;
    double wi = (double)((qreal)2 / ((1 - z * z) * pp * pp));
    x[n - 1 - i] = xi;
    x[i] = -xi;
    w[i] = wi;
    w[n - 1 - i] = wi;
  }
  if (n % 2 == 1) x[n / 2] = 0.0;
}

// ---------------------------------------------------------------------------
// Barycentric Lagrange bases.  src/Core/Interpolation.jl
// ---------------------------------------------------------------------------
struct Poly {
  int np = 0;                  // number of nodes (degree + 1)
  std::vector<double> nodes;   // parent nodes
  std::vector<double> bw;      // barycentric weights
  std::vector<double> D;       // differentiation matrix, row-major D[i*np+j]
};

// diff_matrix (Interpolation.jl:193-213)
void build_dmat(Poly& P) {
  const int n = P.np;
  P.D.assign(n * n, 0.0);
  for (int i = 0; i < n; ++i) {
    double s = 0.0;
    for (int j = 0; j < i; ++j) {
      double t = (P.bw[j] / P.bw[i]) / (P.nodes[i] - P.nodes[j]);
      P.D[i * n + j] = t;
      s += t;
    }
    for (int j = i + 1; j < n; ++j) {
      double t = (P.bw[j] / P.bw[i]) / (P.nodes[i] - P.nodes[j]);
      P.D[i * n + j] = t;
      s += t;
    }
    P.D[i * n + i] = -s;
  }
}

// Legendre(p): Gauss nodes, weights (2 isodd(i) - 1) sqrt((1-x^2) w)
// (Interpolation.jl:62-71).
Poly make_legendre(int p) {
  Poly P;
  P.np = p + 1;
  std::vector<double> x, w;
  gauss_legendre(p + 1, x, w);
  P.nodes = x;
  P.bw.resize(p + 1);
  for (int i = 0; i <= p; ++i) {
    double s = ((i + 1) % 2 == 1) ? 1.0 : -1.0;  // Julia index i+1
    P.bw[i] = s * std::sqrt((1 - x[i] * x[i]) * w[i]);
  }
  build_dmat(P);
  return P;
}

double binomial(int n, int k) {
  double r = 1;
  for (int i = 1; i <= k; ++i) r = r * (n - k + i) / i;
  return std::round(r);
}

// Equispaced(N): nodes range(-1, 1, N+1), weights (2 xor(isodd N, iseven j) - 1)
// binomial(N, j) (Interpolation.jl:88, 128).
Poly make_equispaced(int N) {
  Poly P;
  P.np = N + 1;
  P.nodes.resize(N + 1);
  P.bw.resize(N + 1);
  for (int j = 0; j <= N; ++j) {
    P.nodes[j] = (N == 0) ? 0.0 : (double)(2 * j - N) / (double)N;
    bool x = ((N % 2) == 1) != ((j % 2) == 0);
    P.bw[j] = (x ? 1.0 : -1.0) * binomial(N, j);
  }
  build_dmat(P);
  return P;
}

// weights(ArbitraryPolynomial, x) (Interpolation.jl:96-108)
std::vector<double> arbitrary_weights(const std::vector<double>& x) {
  std::vector<double> w(x.size());
  for (size_t i = 0; i < x.size(); ++i) {
    double wi = 1.0;
    for (size_t j = 0; j < i; ++j) wi *= x[i] - x[j];
    for (size_t j = i + 1; j < x.size(); ++j) wi *= x[i] - x[j];
    w[i] = 1.0 / wi;
  }
  return w;
}

// interpolation_matrix row + shapefun (Interpolation.jl:148-178, 215-218):
// L and dL = L * Dmat at one point.
void shapefun(const Poly& P, double xx, double* L, double* dL) {
  const int n = P.np;
  double msum = 0.0;
  int exact = -1;
  for (int i = 0; i < n; ++i) {
    if (xx == P.nodes[i]) exact = i;
    L[i] = P.bw[i] / (xx - P.nodes[i]);
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
      double s = L[0] * P.D[0 * n + j];
      for (int i = 1; i < n; ++i) s += L[i] * P.D[i * n + j];
      dL[j] = s;
    }
  }
}

struct V2 {
  double x, y;
};
inline double vnorm(double x, double y) { return std::sqrt(x * x + y * y); }

// ---------------------------------------------------------------------------
// Kernels.  Laplace: src/Laplace/Fundamental.jl:19-25.
// Kelvin: src/Elasticity/Fundamental.jl:28-60.
// ---------------------------------------------------------------------------
inline void laplace_UT(double k, double rx, double ry, double nx, double ny, double& U,
                       double& T) {
  double R2 = rx * rx + ry * ry;
  double inv2pi = 1.0 / (2 * kPi);
  U = -std::log(R2) * (0.5 * inv2pi / k);
  T = (rx * nx + ry * ny) * (inv2pi / R2);
}

// U and T as 2x2, row-major [a][b] -> out[2a+b]
inline void kelvin_UT(double mu, double nu, double rx, double ry, double nx, double ny,
                      double* U, double* T) {
  double R2 = rx * rx + ry * ry;
  double R = std::sqrt(R2);
  double dr1 = rx / R, dr2 = ry / R;
  double drdn = dr1 * nx + dr2 * ny;
  double prod1 = 4 * kPi * (1 - nu);
  double prod2 = (3 - 4 * nu) * std::log(1 / R);
  double base = 2 * prod1 * mu;
  U[0] = (prod2 + dr1 * dr1) / base;
  U[1] = (prod2 * 0.0 + dr1 * dr2) / base;
  U[2] = (prod2 * 0.0 + dr2 * dr1) / base;
  U[3] = (prod2 + dr2 * dr2) / base;
  double fat = 1 / (prod1 * R);
  double c = 1 - 2 * nu;
  T[0] = -drdn * (c + 2 * (dr1 * dr1)) * fat;
  T[3] = -drdn * (c + 2 * (dr2 * dr2)) * fat;
  T[1] = -(drdn * 2 * dr1 * dr2 - c * (dr1 * ny - dr2 * nx)) * fat;
  T[2] = -(drdn * 2 * dr1 * dr2 - c * (dr2 * nx - dr1 * ny)) * fat;
}

struct Problem {
  int kind = 0;  // 0 Laplace, 1 Kelvin
  double k = 1.0;
  double mu = 1.0, nu = 0.3;
  int ncomp() const { return kind == 0 ? 1 : 4; }
  // writes U[ncomp], T[ncomp]
  void eval(double rx, double ry, double nx, double ny, double* U, double* T) const {
    if (kind == 0)
      laplace_UT(k, rx, ry, nx, ny, U[0], T[0]);
    else
      kelvin_UT(mu, nu, rx, ry, nx, ny, U, T);
  }
};

// ---------------------------------------------------------------------------
// Distances (src/Core/Integration.jl:238-312) and the near test
// (src/Core/Assembly_full.jl:736-754).
// ---------------------------------------------------------------------------
double dist_chord(V2 p, V2 a, V2 b) {
  double abx = b.x - a.x, aby = b.y - a.y;
  double t = ((p.x - a.x) * abx + (p.y - a.y) * aby) / ((abx * abx + aby * aby) + kEps);
  t = std::min(std::max(t, 0.0), 1.0);
  double qx = a.x + t * abx, qy = a.y + t * aby;
  return vnorm(p.x - qx, p.y - qy);
}

double dist_element(V2 pf, const V2* xg, int n) {
  if (n == 0) return INFINITY;
  if (n == 1) return vnorm(pf.x - xg[0].x, pf.y - xg[0].y);
  if (n == 2) return dist_chord(pf, xg[0], xg[1]);
  double d = INFINITY;
  for (int k = 0; k < n - 1; ++k) d = std::min(d, dist_chord(pf, xg[k], xg[k + 1]));
  return d;
}

bool near_element(V2 pf, const V2* xg, int n, double L, double factor) {
  if (factor == INFINITY || factor > 1e20) return true;
  if (n == 0) return true;
  double lim = factor * L;
  double lim2 = lim * lim;
  double dn2 = INFINITY;
  V2 lo = xg[0], hi = xg[0];
  for (int k = 0; k < n; ++k) {
    V2 q = xg[k];
    lo.x = std::min(lo.x, q.x);
    lo.y = std::min(lo.y, q.y);
    hi.x = std::max(hi.x, q.x);
    hi.y = std::max(hi.y, q.y);
    double dx = pf.x - q.x, dy = pf.y - q.y;
    double d2 = dx * dx + dy * dy;
    if (d2 < dn2) dn2 = d2;
  }
  if (dn2 < lim2) return true;
  double d2 = 0.0;
  if (pf.x < lo.x) { double t = lo.x - pf.x; d2 += t * t; }
  else if (pf.x > hi.x) { double t = pf.x - hi.x; d2 += t * t; }
  if (pf.y < lo.y) { double t = lo.y - pf.y; d2 += t * t; }
  else if (pf.y > hi.y) { double t = pf.y - hi.y; d2 += t * t; }
  if (std::sqrt(d2) >= lim) return false;
  return dist_element(pf, xg, n) < lim;
}

// ---------------------------------------------------------------------------
// Closest point (Integration.jl:323-349, 1005-1010, 1023-1033).
// ---------------------------------------------------------------------------
double seed_1d(const Poly& P, const V2* nodes, int n, V2 pf) {
  double dx = nodes[n - 1].x - nodes[0].x, dy = nodes[n - 1].y - nodes[0].y;
  double nrm = vnorm(dx, dy);
  double xi0 = (P.nodes[n - 1] - P.nodes[0]) *
                   (dx * (pf.x - nodes[0].x) + dy * (pf.y - nodes[0].y)) / (nrm * nrm + kEps) +
               P.nodes[0];
  return std::min(std::max(xi0, -1.0), 1.0);
}

V2 interp_pt(const double* L, const V2* nodes, int n) {
  V2 s{L[0] * nodes[0].x, L[0] * nodes[0].y};
  for (int k = 1; k < n; ++k) {
    s.x += L[k] * nodes[k].x;
    s.y += L[k] * nodes[k].y;
  }
  return s;
}

void closest_point_1d(const Poly& P, const V2* nodes, int n, V2 pf, double xi0, double& xi_out,
                      V2& x_out, double& dist_out) {
  double xi = xi0;
  double L[16], dL[16], d2L[16];
  for (int it = 0; it < 25; ++it) {
    shapefun(P, xi, L, dL);
    for (int j = 0; j < n; ++j) {
      double s = dL[0] * P.D[0 * n + j];
      for (int i = 1; i < n; ++i) s += dL[i] * P.D[i * n + j];
      d2L[j] = s;
    }
    V2 x = interp_pt(L, nodes, n), dx = interp_pt(dL, nodes, n), d2x = interp_pt(d2L, nodes, n);
    double rx = x.x - pf.x, ry = x.y - pf.y;
    double res = rx * dx.x + ry * dx.y;
    double J = (dx.x * dx.x + dx.y * dx.y) + (rx * d2x.x + ry * d2x.y);
    if (std::fabs(J) < 1e-30) break;
    double d = res / J;
    xi -= d;
    if (std::fabs(d) < 1e-14) break;
  }
  V2 xx;
  if (xi < -1 || xi > 1) {
    shapefun(P, -1.0, L, nullptr);
    V2 x0 = interp_pt(L, nodes, n);
    shapefun(P, 1.0, L, nullptr);
    V2 x1 = interp_pt(L, nodes, n);
    if (vnorm(x0.x - pf.x, x0.y - pf.y) <= vnorm(x1.x - pf.x, x1.y - pf.y)) {
      xi = -1.0;
      xx = x0;
    } else {
      xi = 1.0;
      xx = x1;
    }
  } else {
    shapefun(P, xi, L, nullptr);
    xx = interp_pt(L, nodes, n);
  }
  xi_out = xi;
  x_out = xx;
  dist_out = vnorm(xx.x - pf.x, xx.y - pf.y);
}

// ---------------------------------------------------------------------------
// Near-field maps (Integration.jl:1062-1395).
// ---------------------------------------------------------------------------
using Rule = std::vector<double>;

void sinh_map(const Rule& u, double a, double b, Rule& x, Rule& J) {
  double mu = 0.5 * (std::asinh((1 + a) / b) + std::asinh((1 - a) / b));
  double eta = 0.5 * (std::asinh((1 + a) / b) - std::asinh((1 - a) / b));
  x.resize(u.size());
  J.resize(u.size());
  for (size_t i = 0; i < u.size(); ++i) {
    x[i] = a + b * std::sinh(mu * u[i] - eta);
    J[i] = b * mu * std::cosh(mu * u[i] - eta);
  }
}

double jsign(double v) { return v > 0 ? 1.0 : (v < 0 ? -1.0 : 0.0); }

void eq40_AB(double z0, double& A, double& B, double& s) {
  s = -jsign(z0);
  double lm = std::log(s * (-1 - z0));
  double lp = std::log(s * (1 - z0));
  A = 2.0 / (lp - lm);
  B = -A / 2 * (lp + lm);
}

void eq40_real_pole(const Rule& u, const Rule& w, double z0, Rule& x, Rule& wx) {
  if (std::fabs(z0) <= 1) { x = u; wx = w; return; }
  double A, B, s;
  eq40_AB(z0, A, B, s);
  if (std::fabs(A) < 1e-30) { x = u; wx = w; return; }
  x.resize(u.size());
  wx.resize(u.size());
  for (size_t i = 0; i < u.size(); ++i) {
    double e = std::exp((u[i] - B) / A);
    x[i] = z0 + s * e;
    wx[i] = w[i] * (s * e / A);
  }
}

void sinhtrans(const Rule& u, const Rule& w, double a, double b, Rule& x, Rule& wx) {
  if (std::fabs(b) < 1e-14 && std::fabs(a) > 1) { eq40_real_pole(u, w, a, x, wx); return; }
  b = std::max(b, 1e-14);
  Rule J;
  sinh_map(u, a, b, x, J);
  wx.resize(u.size());
  for (size_t i = 0; i < u.size(); ++i) wx[i] = w[i] * J[i];
}

void sinhtrans_iterated(const Rule& u, const Rule& w, double a, double b, int niter, Rule& x,
                        Rule& wx) {
  if (std::fabs(b) < 1e-14 && std::fabs(a) > 1) { eq40_real_pole(u, w, a, x, wx); return; }
  b = std::max(b, 1e-14);
  std::vector<std::pair<double, double>> maps;
  double aa = a, bb = b;
  for (int it = 0; it < niter; ++it) {
    maps.push_back({aa, bb});
    double mu = 0.5 * (std::asinh((1 + aa) / bb) + std::asinh((1 - aa) / bb));
    double eta = 0.5 * (std::asinh((1 + aa) / bb) - std::asinh((1 - aa) / bb));
    if (mu < 1e-14) break;
    aa = std::min(std::max(eta / mu, std::nextafter(-1.0, 0.0)), std::nextafter(1.0, 0.0));
    bb = std::max(kPi / (2 * mu), 1e-14);
  }
  x = u;
  Rule J(u.size(), 1.0);
  for (int m = (int)maps.size() - 1; m >= 0; --m) {
    Rule xs, dJ;
    sinh_map(x, maps[m].first, maps[m].second, xs, dJ);
    x = xs;
    for (size_t i = 0; i < J.size(); ++i) J[i] *= dJ[i];
  }
  wx.resize(u.size());
  for (size_t i = 0; i < u.size(); ++i) wx[i] = w[i] * J[i];
}

bool eq41_collinear(double z0, double e0, bool has_den = false, double den = 0.0) {
  if (std::fabs(z0) <= 1) return false;
  if (std::fabs(e0) < 1e-8) return true;
  if (has_den && std::fabs(den) < 1e-10) return true;
  return false;
}

void eq41_real_pole(const Rule& u, const Rule& w, double z0, Rule& x, Rule& wx) {
  if (std::fabs(z0) <= 1) { x = u; wx = w; return; }
  double A = z0 * z0 - 1;
  double B = -z0;
  x.resize(u.size());
  wx.resize(u.size());
  for (size_t i = 0; i < u.size(); ++i) {
    double d = u[i] - B;
    x[i] = z0 - A / d;
    wx[i] = w[i] * (A / (d * d));
  }
}

void tangenttrans(const Rule& u, const Rule& w, double z0, double e0, Rule& x, Rule& wx) {
  if (eq41_collinear(z0, e0)) { eq41_real_pole(u, w, z0, x, wx); return; }
  e0 = std::max(e0, 1e-14);
  double tp = cr_atan((1 - z0) / e0);
  double tm = cr_atan((-1 - z0) / e0);
  double den = tp - tm;
  if (eq41_collinear(z0, e0, true, den)) { eq41_real_pole(u, w, z0, x, wx); return; }
  double A = 2.0 * e0 / den;
  double B = -(tp + tm) / den;
  double halfpi = kPi / 2 - 1e-8;
  x.resize(u.size());
  wx.resize(u.size());
  for (size_t i = 0; i < u.size(); ++i) {
    double phi = std::min(std::max(e0 * (u[i] - B) / A, -halfpi), halfpi);
    double tn = cr_tan(phi);
    x[i] = z0 + e0 * tn;
    wx[i] = w[i] * ((e0 * e0 / A) * (1 + tn * tn));
  }
}

// _p3c_inv_pole (Integration.jl:1220-1270)
void p3c_inv_pole(double z0, double e0, double& zt, double& et) {
  if (std::fabs(e0) < 1e-14) {
    double x = z0;
    for (int it = 0; it < 25; ++it) {
      double g = x * x * x - 3 * z0 * (x * x) + 3 * x - z0;
      double gp = 3 * (x * x) - 6 * z0 * x + 3;
      if (std::fabs(gp) < 1e-30) break;
      x -= g / gp;
      if (std::fabs(g) < 1e-14) break;
    }
    zt = x;
    et = 0.0;
    return;
  }
  double e = cr_cbrt(std::fabs(e0)) * jsign(e0);
  for (int it = 0; it < 20; ++it) {
    double g = 2 * (e * e * e) - 3 * e0 * (e * e) - e0;
    double gp = 6 * (e * e) - 6 * e0 * e;
    if (std::fabs(gp) < 1e-30) break;
    e -= g / gp;
  }
  e += cr_cbrt(e0) * std::sqrt(z0 * z0 + e0 * e0);
  double z = z0;
  for (int it = 0; it < 30; ++it) {
    double den = 1 + 3 * (z * z) + 3 * (e * e);
    double nz = (3 + z * z + 3 * (e * e)) * z;
    double ne = 2 * (e * e * e);
    double f1 = nz / den - z0;
    double f2 = ne / den - e0;
    if (std::fabs(f1) + std::fabs(f2) < 1e-14) break;
    double denz = 6 * z, dene = 6 * e;
    double nz_z = 3 + 3 * (z * z) + 3 * (e * e);
    double nz_e = 6 * e * z;
    double ne_z = 0.0;
    double ne_e = 6 * (e * e);
    double den2 = den * den;
    double j11 = (nz_z * den - nz * denz) / den2;
    double j12 = (nz_e * den - nz * dene) / den2;
    double j21 = (ne_z * den - ne * denz) / den2;
    double j22 = (ne_e * den - ne * dene) / den2;
    double det = j11 * j22 - j12 * j21;
    if (std::fabs(det) < 1e-30) break;
    z -= (j22 * f1 - j12 * f2) / det;
    e -= (-j21 * f1 + j11 * f2) / det;
  }
  zt = z;
  et = e;
}

void p3ctrans(const Rule& u, const Rule& w, double z0, double e0, Rule& x, Rule& wx) {
  double zt, et;
  p3c_inv_pole(z0, e0, zt, et);
  double den = 1 + 3 * (zt * zt) + 3 * (et * et);
  double A = 3.0 / den;
  double B = (3 + zt * zt) * zt / den;
  x.resize(u.size());
  wx.resize(u.size());
  for (size_t i = 0; i < u.size(); ++i) {
    double s = u[i];
    double ds = s - zt;
    x[i] = A * ((ds * ds * ds) / 3 + (et * et) * s) + B;
    wx[i] = w[i] * (A * ((ds * ds) + et * et));
  }
}

void tanp3c_tail(const Rule& ut, const Rule& wt, double z0, double e0, double At, double Bt,
                 Rule& x, Rule& wx) {
  double halfpi = kPi / 2 - 1e-8;
  size_t m = ut.size();
  x.resize(m);
  wx.resize(m);
  for (size_t i = 0; i < m; ++i) {
    double th = std::min(std::max((ut[i] - Bt) / At, -halfpi), halfpi);
    double tn = cr_tan(th);
    x[i] = z0 + e0 * tn;
    wx[i] = wt[i] * ((e0 / At) * (1 + tn * tn));
  }
}

void tanp3c_compose(const Rule& u, const Rule& w, double z0, double e0, double At, double Bt,
                    double upole, Rule& x, Rule& wx) {
  Rule ut, w1;
  p3ctrans(u, w, upole, std::max(std::fabs(0.0), 1e-14), ut, w1);
  tanp3c_tail(ut, w1, z0, e0, At, Bt, x, wx);
}

// Reference deviation (documented): the reference returns the full-interval
// tangent rule when this half is narrower than 1e-14 (Integration.jl:1349),
// so the split counts the element twice and the result jumps with the last
// bit of zeta0 near +-1.  The default here gives the empty half no nodes;
// g_ref_degenerate_half = 1 reproduces the reference's rule.
int g_ref_degenerate_half = 0;

void tanp3c_half(const Rule& u, const Rule& w, double z0, double e0, double At, double Bt,
                 double lo, double hi, double upole, Rule& x, Rule& wx) {
  double mid = (hi + lo) / 2;
  double h = (hi - lo) / 2;
  if (h <= 1e-14) {
    if (g_ref_degenerate_half) { tangenttrans(u, w, z0, e0, x, wx); return; }
    x.clear();
    wx.clear();
    return;
  }
  double spole = (upole - mid) / h;
  Rule s, ws;
  p3ctrans(u, w, spole, 1e-14, s, ws);
  Rule ut(s.size()), wt(s.size());
  for (size_t i = 0; i < s.size(); ++i) {
    ut[i] = mid + h * s[i];
    wt[i] = ws[i] * h;
  }
  tanp3c_tail(ut, wt, z0, e0, At, Bt, x, wx);
}

void tanp3ctrans(const Rule& u, const Rule& w, double z0, double e0, Rule& x, Rule& wx) {
  if (eq41_collinear(z0, e0)) { eq41_real_pole(u, w, z0, x, wx); return; }
  e0 = std::max(e0, 1e-14);
  double ap = cr_atan((1 - z0) / e0);
  double am = cr_atan((1 + z0) / e0);
  double den = ap + am;
  if (eq41_collinear(z0, e0, true, den)) { eq41_real_pole(u, w, z0, x, wx); return; }
  if (std::fabs(den) < 1e-30) { p3ctrans(u, w, z0, e0, x, wx); return; }
  double At = 2.0 / den;
  double Bt = -At * (ap - am) / 2.0;
  double uL = Bt - At * kPi / 2;
  double uR = Bt + At * kPi / 2;
  if (std::fabs(z0) < 1 && -1 < Bt && Bt < 1) {
    Rule xl, wl, xr, wr;
    tanp3c_half(u, w, z0, e0, At, Bt, -1.0, Bt, uL, xl, wl);
    tanp3c_half(u, w, z0, e0, At, Bt, Bt, 1.0, uR, xr, wr);
    x = xl;
    x.insert(x.end(), xr.begin(), xr.end());
    wx = wl;
    wx.insert(wx.end(), wr.begin(), wr.end());
  } else if (z0 >= 1) {
    tanp3c_compose(u, w, z0, e0, At, Bt, uL, x, wx);
  } else {
    tanp3c_compose(u, w, z0, e0, At, Bt, uR, x, wx);
  }
}

// Complex{Float64} arithmetic as Julia evaluates it: the product
// (ac - bd, ad + bc), componentwise scaling by a real, the quotient by
// Baudin and Smith's robust Smith method ("A robust complex division in
// Scilab", 2012; its over/underflow rescaling is left out: element-size
// operands never come near those thresholds), and the square root by
// Kahan's method ("Branch cuts for complex elementary functions", 1987;
// rescaling left out for the same reason).  abs is hypot.
struct jc {
  double re, im;
};
jc jadd(jc a, jc b) { return {a.re + b.re, a.im + b.im}; }
jc jsub(jc a, jc b) { return {a.re - b.re, a.im - b.im}; }
jc jmul(jc a, jc b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
jc jscale(double s, jc a) { return {s * a.re, s * a.im}; }
jc jdivr(jc a, double s) { return {a.re / s, a.im / s}; }
double jabs(jc a) { return std::hypot(a.re, a.im); }

// one half of the robust quotient: (a + ib) / (c + id) with |d| <= |c|
double jdiv_part(double a, double b, double c, double d, double r, double t) {
  if (r != 0) {
    double br = b * r;
    return br != 0 ? (a + br) * t : a * t + (b * t) * r;
  }
  return (a + d * (b / c)) * t;
}
jc jdiv(jc x, jc y) {
  double a = x.re, b = x.im, c = y.re, d = y.im;
  if (std::fabs(d) <= std::fabs(c)) {
    double r = d / c, t = 1.0 / (c + d * r);
    return {jdiv_part(a, b, c, d, r, t), jdiv_part(b, -a, c, d, r, t)};
  }
  double r = c / d, t = 1.0 / (d + c * r);
  return {jdiv_part(b, a, d, c, r, t), -jdiv_part(a, -b, d, c, r, t)};
}
jc jsqrt(jc z) {
  double x = z.re, y = z.im;
  if (x == 0 && y == 0) return {0.0, y};
  double rho = x * x + y * y;
  rho = std::fabs(x) + std::sqrt(rho);
  rho += rho;
  rho = std::sqrt(rho) * 0.5;
  double xi = rho, eta = y;
  if (rho != 0) {
    eta = (eta / rho) / 2;
    if (x < 0) {
      xi = std::fabs(eta);
      eta = std::copysign(rho, y);
    }
  }
  return {xi, eta};
}

// _complex_pole_1d (Integration.jl:1117-1160)
void complex_pole_1d(const Poly& P, const V2* nodes, int nN, V2 pf, double& z0, double& e0) {
  jc y{pf.x, pf.y};
  if (nN == 2 || nN == 3) {
    std::vector<double> xs(P.nodes.begin(), P.nodes.end());
    if ((int)xs.size() != nN) {
      xs.resize(nN);
      for (int k = 0; k < nN; ++k) xs[k] = -1.0 + 2.0 * k / (nN - 1);
    }
    jc Z[3];
    for (int k = 0; k < nN; ++k) Z[k] = jc{nodes[k].x, nodes[k].y};
    if (nN == 2) {
      jc B = jdivr(jsub(Z[1], Z[0]), xs[1] - xs[0] + 1e-30);
      jc C = jsub(Z[0], jscale(xs[0], B));
      if (jabs(B) < 1e-30) { z0 = 0.0; e0 = 1.0; return; }
      jc r = jdiv(jsub(y, C), B);
      z0 = r.re;
      e0 = std::fabs(r.im);
      return;
    }
    // Vandermonde [xi^2 xi 1] \ Z by cofactors over the determinant
    // (_fit_quad_complex: the closed form StaticArrays uses for 3x3 solves)
    double a11 = xs[0] * xs[0], a12 = xs[0], a13 = 1;
    double a21 = xs[1] * xs[1], a22 = xs[1], a23 = 1;
    double a31 = xs[2] * xs[2], a32 = xs[2], a33 = 1;
    double det = a11 * (a22 * a33 - a23 * a32) - a12 * (a21 * a33 - a23 * a31) +
                 a13 * (a21 * a32 - a22 * a31);
    auto comb = [&](double c0, double c1, double c2) {
      return jdivr(jadd(jadd(jscale(c0, Z[0]), jscale(c1, Z[1])), jscale(c2, Z[2])), det);
    };
    jc A = comb(a22 * a33 - a23 * a32, a13 * a32 - a12 * a33, a12 * a23 - a13 * a22);
    jc B = comb(a23 * a31 - a21 * a33, a11 * a33 - a13 * a31, a13 * a21 - a11 * a23);
    jc C = comb(a21 * a32 - a22 * a31, a12 * a31 - a11 * a32, a11 * a22 - a12 * a21);
    if (jabs(A) < 1e-14) {
      if (jabs(B) < 1e-30) { z0 = 0.0; e0 = 1.0; return; }
      jc r = jdiv(jsub(y, C), B);
      z0 = r.re;
      e0 = std::fabs(r.im);
      return;
    }
    jc disc = jsqrt(jsub(jmul(B, B), jmul(jscale(4.0, A), jsub(C, y))));
    jc mB{-B.re, -B.im};
    jc twoA = jscale(2.0, A);
    jc r1 = jdiv(jadd(mB, disc), twoA);
    jc r2 = jdiv(jsub(mB, disc), twoA);
    jc r = std::fabs(r1.im) <= std::fabs(r2.im) ? r1 : r2;
    z0 = r.re;
    e0 = std::fabs(r.im);
    return;
  }
  double a, dist;
  V2 xs;
  closest_point_1d(P, nodes, nN, pf, seed_1d(P, nodes, nN, pf), a, xs, dist);
  double L[16], dL[16];
  shapefun(P, a, L, dL);
  V2 dx = interp_pt(dL, nodes, nN);
  z0 = a;
  e0 = dist / std::max(vnorm(dx.x, dx.y), 1e-14);
}

// ---------------------------------------------------------------------------
// Interpolated Guiggiani (Integration.jl:1598-1845).
// ---------------------------------------------------------------------------
struct InterpRule {
  std::vector<double> xi, w, Ni, d;
};

// _barycentric_eval (1621-1644)
std::vector<double> barycentric_eval(const std::vector<double>& xi, const std::vector<double>& bw,
                                     double a) {
  size_t n = xi.size();
  std::vector<double> Ni(n);
  double msum = 0.0;
  int exact = -1;
  for (size_t i = 0; i < n; ++i) {
    double d = a - xi[i];
    if (d == 0) exact = (int)i;
    Ni[i] = bw[i] / d;
    msum += Ni[i];
  }
  if (exact >= 0) {
    std::fill(Ni.begin(), Ni.end(), 0.0);
    Ni[exact] = 1.0;
    return Ni;
  }
  double invs = 1.0 / msum;
  for (size_t i = 0; i < n; ++i) Ni[i] *= invs;
  return Ni;
}

// _interp_rule (1653-1670); returns false if fewer than 2 nodes survive.
bool interp_rule(double a, int n, InterpRule& R) {
  std::vector<double> xi, w;
  gauss_legendre(n, xi, w);
  std::vector<double> bw = arbitrary_weights(xi);
  int ndrop = 0;
  for (int i = 0; i < n; ++i)
    if (std::fabs(xi[i] - a) <= 1e-12) ++ndrop;
  if (ndrop == 0) {
    R.xi = xi;
    R.w = w;
    R.Ni = barycentric_eval(xi, bw, a);
  } else {
    R.xi.clear();
    R.w.clear();
    for (int i = 0; i < n; ++i)
      if (std::fabs(xi[i] - a) > 1e-12) {
        R.xi.push_back(xi[i]);
        R.w.push_back(w[i]);
      }
    if (R.xi.size() < 2) return false;
    std::vector<double> bwk = arbitrary_weights(R.xi);
    R.Ni = barycentric_eval(R.xi, bwk, a);
  }
  R.d.resize(R.xi.size());
  for (size_t i = 0; i < R.xi.size(); ++i) R.d[i] = R.xi[i] - a;
  return true;
}

// Samples: F[i*K + c] for node i, component c.
// _interp_log_coeff (1797-1821) -> (0, Fm1, F0)
void interp_log_coeff(const std::vector<double>& F, int K, const InterpRule& R, double* C) {
  size_t m = R.xi.size();
  // C[0..K) = F-2 (zero), C[K..2K) = F-1, C[2K..3K) = F0
  std::vector<double> Fm1(K), sW(K, 0.0), sWL(K, 0.0);
  for (int c = 0; c < K; ++c) {
    double acc = R.Ni[0] * (F[0 * K + c] * R.d[0]);
    for (size_t i = 1; i < m; ++i) acc += R.Ni[i] * (F[i * K + c] * R.d[i]);
    Fm1[c] = acc;
  }
  double sL = 0.0, sL2 = 0.0;
  int nused = 0;
  for (size_t i = 0; i < m; ++i) {
    double adi = std::fabs(R.d[i]);
    if (adi < 1e-14) continue;
    double lg = std::log(adi);
    sL += lg;
    sL2 += lg * lg;
    for (int c = 0; c < K; ++c) {
      double wi = F[i * K + c] - Fm1[c] / R.d[i];
      sW[c] += wi;
      sWL[c] += wi * lg;
    }
    ++nused;
  }
  for (int c = 0; c < K; ++c) {
    C[c] = 0.0;
    C[K + c] = Fm1[c];
    C[2 * K + c] = 0.0;
  }
  if (nused < 2) return;
  double detA = sL2 * nused - sL * sL;
  if (std::fabs(detA) < 1e-30) return;
  for (int c = 0; c < K; ++c) C[2 * K + c] = (nused * sWL[c] - sL * sW[c]) / detA;
}

double ipow(double x, int k) {
  // Julia x^k for Float64, small non-negative k
  if (k == 0) return 1.0;
  if (k == 1) return x;
  if (k == 2) return x * x;
  if (k == 3) return x * x * x;
  double r = x * x;
  return r * r;
}

// _interp_cascade (1686-1714): returns packed 5-tuple (orders -3,-4) or
// 3-tuple (orders -1,-2), stored in C with stride K.
int interp_cascade(const std::vector<double>& F, int K, const InterpRule& R, int order, double* C) {
  size_t m = R.xi.size();
  int p = -order;
  std::vector<double> work(F);
  std::vector<double> Fk((p + 1) * K);
  for (int jj = 0; jj <= p; ++jj) {
    int k = p - jj;
    for (int c = 0; c < K; ++c) {
      double acc = R.Ni[0] * (work[0 * K + c] * ipow(R.d[0], k));
      for (size_t i = 1; i < m; ++i) acc += R.Ni[i] * (work[i * K + c] * ipow(R.d[i], k));
      Fk[jj * K + c] = acc;
    }
    if (k > 0)
      for (size_t i = 0; i < m; ++i)
        for (int c = 0; c < K; ++c) work[i * K + c] = work[i * K + c] - Fk[jj * K + c] / ipow(R.d[i], k);
  }
  // pack
  if (order == -4) {
    for (int t = 0; t < 5; ++t)
      for (int c = 0; c < K; ++c) C[t * K + c] = Fk[t * K + c];
    return 5;
  } else if (order == -3) {
    for (int c = 0; c < K; ++c) C[c] = 0.0;
    for (int t = 0; t < 4; ++t)
      for (int c = 0; c < K; ++c) C[(t + 1) * K + c] = Fk[t * K + c];
    return 5;
  } else if (order == -2) {
    for (int t = 0; t < 3; ++t)
      for (int c = 0; c < K; ++c) C[t * K + c] = Fk[t * K + c];
    return 3;
  } else {
    for (int c = 0; c < K; ++c) C[c] = 0.0;
    for (int t = 0; t < 2; ++t)
      for (int c = 0; c < K; ++c) C[(t + 1) * K + c] = Fk[t * K + c];
    return 3;
  }
}

double hfp_parent(double a, int k) {
  if (k == 1) return std::log(std::fabs((1 - a) / (1 + a)));
  if (k == 2) return -2 / (1 - a * a);
  if (k == 3) return -1 / (2 * ((1 - a) * (1 - a))) + 1 / (2 * ((1 + a) * (1 + a)));
  return -1 / (3 * ((1 - a) * (1 - a) * (1 - a))) - 1 / (3 * ((1 + a) * (1 + a) * (1 + a)));
}

double log_parent(double a) {
  return (1 - a) * std::log(std::fabs(1 - a)) + (1 + a) * std::log(std::fabs(1 + a)) - 2;
}

// _interp_reg_node (1741-1759) for one component
double interp_reg_node(double fi, double d, const double* C, int K, int c, int order) {
  if (order <= -3) {
    double F4 = C[0 * K + c], F3 = C[1 * K + c], F2 = C[2 * K + c], F1 = C[3 * K + c];
    double val = fi;
    if (order <= -4) val -= F4 / ipow(d, 4);
    val -= F3 / ipow(d, 3);
    val -= F2 / ipow(d, 2);
    val -= F1 / d;
    return val;
  }
  double F2 = C[0 * K + c], F1 = C[1 * K + c], F0 = C[2 * K + c];
  if (order == 0) return fi - F1 / d - F0 * std::log(std::fabs(d));
  if (order == -1) return fi - F1 / d;
  return fi - F2 / ipow(d, 2) - F1 / d;
}

double interp_analytic_parent(double a, const double* C, int K, int c, int order) {
  if (order <= -3) {
    double F4 = C[0 * K + c], F3 = C[1 * K + c], F2 = C[2 * K + c], F1 = C[3 * K + c];
    double ana = F1 * hfp_parent(a, 1) + F2 * hfp_parent(a, 2) + F3 * hfp_parent(a, 3);
    if (order <= -4) ana += F4 * hfp_parent(a, 4);
    return ana;
  }
  double F2 = C[0 * K + c], F1 = C[1 * K + c], F0 = C[2 * K + c];
  if (order == 0) return F1 * hfp_parent(a, 1) + F0 * log_parent(a);
  if (order == -1) return F1 * hfp_parent(a, 1);
  return F2 * hfp_parent(a, 2) + F1 * hfp_parent(a, 1);
}

// _interp_integrate (1778-1784)
void interp_integrate(const std::vector<double>& F, int K, const InterpRule& R, const double* C,
                      int order, double a, double* out) {
  size_t m = R.xi.size();
  for (int c = 0; c < K; ++c) {
    double acc = R.w[0] * interp_reg_node(F[0 * K + c], R.d[0], C, K, c, order);
    for (size_t i = 1; i < m; ++i) acc += R.w[i] * interp_reg_node(F[i * K + c], R.d[i], C, K, c, order);
    out[c] = acc + interp_analytic_parent(a, C, K, c, order);
  }
}

void interp_coeffs(const std::vector<double>& F, int K, const InterpRule& R, int order, double* C) {
  if (order == 0)
    interp_log_coeff(F, K, R, C);
  else
    interp_cascade(F, K, R, order, C);
}

// ---------------------------------------------------------------------------
// Geometry + element integration.
// ---------------------------------------------------------------------------
struct Geom {
  int nt, n, ne, p, ngeo;
  const double *px, *py, *nx, *ny, *jac, *elen, *gx, *gy, *ew;
};

struct Ctx {
  const Geom* g;
  Problem prob;
  Poly leg;        // Legendre(p)
  Poly geo_poly;   // Equispaced(ngeo-1)
  std::vector<double> qsi, w;  // npg rule
  int nearfield;   // 0 tanp3c, 1 plain, 2 euclid, 3 csinh, 4 sinhsinh, 5 tangent, 6 p3c
  int singular;    // 0 guiggiani, 1 telles
};

// _shape_geom (Assembly_full.jl:608-627)
void shape_geom(const Ctx& C, const V2* nodes, const V2* geo, double xi, double* N, V2& pg,
                V2& dx) {
  const int nn = C.leg.np;
  double dN[16];
  shapefun(C.leg, xi, N, dN);
  if (C.g->ngeo > 0) {
    const int ng = C.geo_poly.np;
    double Ng[16], dNg[16];
    shapefun(C.geo_poly, xi, Ng, dNg);
    pg = V2{0.0, 0.0};
    dx = V2{0.0, 0.0};
    for (int k = 0; k < ng; ++k) {
      pg.x += Ng[k] * geo[k].x;
      pg.y += Ng[k] * geo[k].y;
      dx.x += dNg[k] * geo[k].x;
      dx.y += dNg[k] * geo[k].y;
    }
    return;
  }
  pg = V2{0.0, 0.0};
  dx = V2{0.0, 0.0};
  for (int k = 0; k < nn; ++k) {
    pg.x += N[k] * nodes[k].x;
    pg.y += N[k] * nodes[k].y;
    dx.x += dN[k] * nodes[k].x;
    dx.y += dN[k] * nodes[k].y;
  }
}

// _sample_kernel (Assembly_full.jl:629-643) packed into the guiggiani sample
// layout F[c] for c = component*nn + j ... we use c = j*ncomp + comp.
bool sample_kernel(const Ctx& C, const V2* nodes, const V2* geo, V2 pf, double xi, V2 nref,
                   double* Fg, double* Fh) {
  const int nn = C.leg.np;
  const int nc = C.prob.ncomp();
  double N[16];
  V2 pg, dx;
  shape_geom(C, nodes, geo, xi, N, pg, dx);
  double J = vnorm(dx.x, dx.y);
  if (J < 1e-30) return false;
  double rx = pg.x - pf.x, ry = pg.y - pf.y;
  if (vnorm(rx, ry) < 1e-30) return false;
  double tx = dx.x / J, ty = dx.y / J;
  double nx = ty, ny = -tx;  // tan2normal
  if (nx * nref.x + ny * nref.y < 0) { nx = -nx; ny = -ny; }
  double U[4], T[4];
  C.prob.eval(rx, ry, nx, ny, U, T);
  for (int j = 0; j < nn; ++j) {
    double NjJ = N[j] * J;
    for (int c = 0; c < nc; ++c) {
      Fg[j * nc + c] = U[c] * NjJ;
      Fh[j * nc + c] = T[c] * NjJ;
    }
  }
  return true;
}

// _integrate_singular_guiggiani! (Assembly_full.jl:397-457) with
// _guiggiani_interp_pair (Integration.jl:1833-1845), orders (0, -1).
void integrate_singular_guiggiani(const Ctx& C, const V2* nodes, const V2* geo, V2 pf, double a,
                                  V2 nref, double* h, double* g) {
  const int nn = C.leg.np;
  const int nc = C.prob.ncomp();
  const int K = nn * nc;
  a = std::min(std::max(a, std::nextafter(-1.0, 0.0)), std::nextafter(1.0, 0.0));
  InterpRule R;
  if (!interp_rule(a, 20, R)) {
    for (int c = 0; c < K; ++c) h[c] = g[c] = NAN;
    return;
  }
  size_t m = R.xi.size();
  std::vector<double> Fg(m * K, 0.0), Fh(m * K, 0.0);
  for (size_t i = 0; i < m; ++i) {
    if (!sample_kernel(C, nodes, geo, pf, R.xi[i], nref, &Fg[i * K], &Fh[i * K])) {
      for (int c = 0; c < K; ++c) Fg[i * K + c] = Fh[i * K + c] = 0.0;
    }
  }
  std::vector<double> Cg(5 * K), Ch(5 * K);
  interp_coeffs(Fg, K, R, 0, Cg.data());
  interp_coeffs(Fh, K, R, -1, Ch.data());
  interp_integrate(Fg, K, R, Cg.data(), 0, a, g);
  interp_integrate(Fh, K, R, Ch.data(), -1, a, h);
}

// _telles_map / _integrate_singular_telles! (Assembly_full.jl:467-528)
void integrate_singular_telles(const Ctx& C, const V2* nodes, const V2* geo, V2 pf, double a,
                               V2 nref, double* h, double* g) {
  const int nn = C.leg.np;
  const int nc = C.prob.ncomp();
  const int K = nn * nc;
  for (int c = 0; c < K; ++c) h[c] = g[c] = 0.0;
  a = std::min(std::max(a, std::nextafter(-1.0, 0.0)), std::nextafter(1.0, 0.0));
  double eet = a;
  double eest = eet * eet - 1;
  double term1 = cr_cbrt(eet * eest + std::fabs(eest));
  double term2 = cr_cbrt(eet * eest - std::fabs(eest));
  double Gm = term1 + term2 + eet;
  double Q = 1 + 3 * (Gm * Gm);
  double A = 1 / Q, B = -3 * Gm / Q, Cc = 3 * (Gm * Gm) / Q, D = -B;
  std::vector<double> Fg(K), Fh(K);
  for (size_t i = 0; i < C.qsi.size(); ++i) {
    double gm = C.qsi[i];
    double eta = A * (gm * gm * gm) + B * (gm * gm) + Cc * gm + D;
    double Jt = 3 * A * (gm * gm) + 2 * B * gm + Cc;
    double N[16];
    V2 pg, dx;
    shape_geom(C, nodes, geo, eta, N, pg, dx);
    double J = vnorm(dx.x, dx.y);
    if (J < 1e-30) continue;
    double rx = pg.x - pf.x, ry = pg.y - pf.y;
    if (vnorm(rx, ry) < 1e-30) continue;
    double tx = dx.x / J, ty = dx.y / J;
    double nx = ty, ny = -tx;
    if (nx * nref.x + ny * nref.y < 0) { nx = -nx; ny = -ny; }
    double U[4], T[4];
    C.prob.eval(rx, ry, nx, ny, U, T);
    double wJ = Jt * C.w[i] * J;
    for (int j = 0; j < nn; ++j) {
      double Nj = N[j] * wJ;
      for (int c = 0; c < nc; ++c) {
        g[j * nc + c] += U[c] * Nj;
        h[j * nc + c] += T[c] * Nj;
      }
    }
  }
}

// transform (Integration.jl:68-93)
void near_rule(const Ctx& C, const V2* nodes, V2 pf, double Lel, Rule& eta, Rule& ww) {
  const int nn = C.leg.np;
  int nf = C.nearfield;
  if (nf == 1) { eta = C.qsi; ww = C.w; return; }
  if (nf == 0 || nf == 3 || nf == 4 || nf == 5 || nf == 6) {
    double z0, e0;
    complex_pole_1d(C.leg, nodes, nn, pf, z0, e0);
    if (nf == 5) { tangenttrans(C.qsi, C.w, z0, e0, eta, ww); return; }
    if (nf == 6) { p3ctrans(C.qsi, C.w, z0, e0, eta, ww); return; }
    if (nf == 0) { tanp3ctrans(C.qsi, C.w, z0, e0, eta, ww); return; }
    sinhtrans_iterated(C.qsi, C.w, z0, e0, nf == 4 ? 2 : 1, eta, ww);
    return;
  }
  double a, dist;
  V2 xs;
  closest_point_1d(C.leg, nodes, nn, pf, seed_1d(C.leg, nodes, nn, pf), a, xs, dist);
  double b = dist / std::max(Lel, kEps);
  sinhtrans(C.qsi, C.w, a, std::max(b, 1e-14), eta, ww);
}

// _quad_geom + _accumulate_kernels! (Assembly_full.jl:649-713)
void integrate_near(const Ctx& C, const V2* nodes, const V2* geo, V2 pf, double Lel, V2 nref,
                    double* h, double* g) {
  const int nn = C.leg.np;
  const int nc = C.prob.ncomp();
  Rule eta, ww;
  near_rule(C, nodes, pf, Lel, eta, ww);
  size_t m = eta.size();
  std::vector<double> Nm(m * nn), rx(m), ry(m), nxv(m), nyv(m), wJ(m);
  for (size_t i = 0; i < m; ++i) {
    V2 pg, dx;
    shape_geom(C, nodes, geo, eta[i], &Nm[i * nn], pg, dx);
    rx[i] = pg.x - pf.x;
    ry[i] = pg.y - pf.y;
    double J = vnorm(dx.x, dx.y);
    double tx = dx.x / J, ty = dx.y / J;
    nxv[i] = ty;
    nyv[i] = -tx;
    wJ[i] = J * ww[i];
  }
  if (m > 0 && (nxv[0] * nref.x + nyv[0] * nref.y) < 0)
    for (size_t i = 0; i < m; ++i) { nxv[i] = -nxv[i]; nyv[i] = -nyv[i]; }
  for (size_t i = 0; i < m; ++i) {
    double U[4], T[4];
    C.prob.eval(rx[i], ry[i], nxv[i], nyv[i], U, T);
    double wi = wJ[i];
    for (int j = 0; j < nn; ++j) {
      double Nj = Nm[i * nn + j] * wi;
      for (int c = 0; c < nc; ++c) {
        h[j * nc + c] += T[c] * Nj;
        g[j * nc + c] += U[c] * Nj;
      }
    }
  }
}

// integrate_element 2-D branch (Assembly_full.jl:262-289, 310-312).
// `source` is the collocation index or -1 (geometric dist <= 1e-12 test).
void integrate_element(const Ctx& C, int e, V2 pf, int source, double* h, double* g) {
  const Geom& G = *C.g;
  const int nn = C.leg.np;
  const int nc = C.prob.ncomp();
  V2 nodes[16], geo[16];
  for (int k = 0; k < nn; ++k) nodes[k] = V2{G.px[e * nn + k], G.py[e * nn + k]};
  for (int k = 0; k < G.ngeo; ++k) geo[k] = V2{G.gx[e * G.ngeo + k], G.gy[e * G.ngeo + k]};
  for (int c = 0; c < nn * nc; ++c) h[c] = g[c] = 0.0;
  double a, dist;
  V2 xs;
  closest_point_1d(C.leg, nodes, nn, pf, seed_1d(C.leg, nodes, nn, pf), a, xs, dist);
  bool singular = source >= 0 ? (source >= e * nn && source < (e + 1) * nn) : (dist <= 1e-12);
  V2 nref{G.nx[e * nn], G.ny[e * nn]};
  if (singular) {
    if (C.singular == 1)
      integrate_singular_telles(C, nodes, geo, pf, a, nref, h, g);
    else
      integrate_singular_guiggiani(C, nodes, geo, pf, a, nref, h, g);
    return;
  }
  integrate_near(C, nodes, geo, pf, G.elen[e], nref, h, g);
}

void setup_ctx(Ctx& C, const Geom* g, int npg) {
  C.g = g;
  C.leg = make_legendre(g->p);
  if (g->ngeo > 0) C.geo_poly = make_equispaced(g->ngeo - 1);
  gauss_legendre(npg, C.qsi, C.w);
}

// H_G_full_direct scalar (Assembly_full.jl:61-85, 354-390, 801-810) and
// vectorial (120-175, 777-787, 812-822).
void assemble(Ctx& C, double near_factor, int nthreads, double* H, double* Gm,
              const uint8_t* fixed_mask = nullptr) {
  const Geom& G = *C.g;
  const int nn = G.p + 1;
  const int dof = C.prob.kind == 0 ? 1 : 2;
  const int nc = C.prob.ncomp();
  const int64_t rows = (int64_t)dof * G.nt;
  const int64_t cols = (int64_t)dof * G.n;
  std::memset(H, 0, sizeof(double) * rows * rows);
  std::memset(Gm, 0, sizeof(double) * rows * cols);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
  for (int i = 0; i < G.nt; ++i) {
    V2 pf{G.px[i], G.py[i]};
    std::vector<double> hl(nn * nc), gl(nn * nc);
    V2 xg[16];
    for (int e = 0; e < G.ne; ++e) {
      for (int k = 0; k < nn; ++k) xg[k] = V2{G.px[e * nn + k], G.py[e * nn + k]};
      bool on = (i >= e * nn && i < (e + 1) * nn);
      bool nr = fixed_mask ? (fixed_mask[(int64_t)i * G.ne + e] != 0)
                           : near_element(pf, xg, nn, G.elen[e], near_factor);
      if (C.prob.kind == 0) nr = nr || on;
      if (nr) {
        integrate_element(C, e, pf, i, hl.data(), gl.data());
        for (int k = 0; k < nn; ++k) {
          int j = e * nn + k;
          for (int a = 0; a < dof; ++a)
            for (int b = 0; b < dof; ++b) {
              int c = k * nc + a * dof + b;
              H[(int64_t)(dof * i + a) + (int64_t)(dof * j + b) * rows] += hl[c];
              Gm[(int64_t)(dof * i + a) + (int64_t)(dof * j + b) * rows] += gl[c];
            }
        }
      } else {
        for (int k = 0; k < nn; ++k) {
          int j = e * nn + k;
          double U[4], T[4];
          C.prob.eval(G.px[j] - pf.x, G.py[j] - pf.y, G.nx[j], G.ny[j], U, T);
          double wjk = G.jac[j] * G.ew[k];
          for (int a = 0; a < dof; ++a)
            for (int b = 0; b < dof; ++b) {
              H[(int64_t)(dof * i + a) + (int64_t)(dof * j + b) * rows] += T[a * dof + b] * wjk;
              Gm[(int64_t)(dof * i + a) + (int64_t)(dof * j + b) * rows] += U[a * dof + b] * wjk;
            }
        }
      }
    }
  }
  // row-sum diagonal / rigid-body free term
  if (dof == 1) {
    for (int64_t i = 0; i < rows; ++i) {
      H[i + i * rows] = 0.0;
      double s = 0.0;
      for (int64_t j = 0; j < rows; ++j) s += H[i + j * rows];
      H[i + i * rows] = -s;
    }
  } else {
    for (int i = 0; i < G.nt; ++i) {
      for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) H[(2 * i + a) + (int64_t)(2 * i + b) * rows] = 0.0;
      for (int jd = 0; jd < 2; ++jd)
        for (int a = 0; a < 2; ++a) {
          double s = 0.0;
          for (int64_t c = jd; c < rows; c += 2) s += H[(2 * i + a) + c * rows];
          H[(2 * i + a) + (int64_t)(2 * i + jd) * rows] = -s;
        }
    }
  }
}

}  // namespace

// ===========================================================================
// C entry points (ctypes).  All pointers are host FP64 arrays.
// ===========================================================================
extern "C" {

struct OrcGeom {
  int32_t nt, n, ne, p, ngeo;
  const double *px, *py, *nx, *ny, *jac, *elen, *gx, *gy, *ew;
};

static Geom to_geom(const OrcGeom* o) {
  return Geom{o->nt, o->n, o->ne, o->p, o->ngeo, o->px, o->py, o->nx, o->ny,
              o->jac, o->elen, o->gx, o->gy, o->ew};
}

// kind 0: Laplace (prm0 = k); kind 1: Kelvin (prm0 = mu, prm1 = effective nu).
// mask: optional nt x ne near classification to use instead of the test
// (holds the near/far split fixed, e.g. to measure the integrals' rounding
// sensitivity without classification flips).
int orc_assemble(const OrcGeom* og, int kind, double prm0, double prm1, int npg,
                 double near_factor, int nearfield, int singular, int nthreads, double* H,
                 double* G, const uint8_t* mask) {
  if (!og || og->p < 1 || og->p > 8 || og->ngeo > 12 || npg < 1) return 1;
  Geom g = to_geom(og);
  Ctx C;
  setup_ctx(C, &g, npg);
  C.prob.kind = kind;
  if (kind == 0) C.prob.k = prm0;
  else { C.prob.mu = prm0; C.prob.nu = prm1; }
  C.nearfield = nearfield;
  C.singular = singular;
  assemble(C, near_factor, nthreads, H, G, mask);
  return 0;
}

// One element's local h, g for source point pf (integrate_element).
int orc_integrate_element(const OrcGeom* og, int kind, double prm0, double prm1, int npg,
                          int nearfield, int singular, int e, double pfx, double pfy, int source,
                          double* h, double* g) {
  Geom gg = to_geom(og);
  Ctx C;
  setup_ctx(C, &gg, npg);
  C.prob.kind = kind;
  if (kind == 0) C.prob.k = prm0;
  else { C.prob.mu = prm0; C.prob.nu = prm1; }
  C.nearfield = nearfield;
  C.singular = singular;
  integrate_element(C, e, V2{pfx, pfy}, source, h, g);
  return 0;
}

// Correctly rounded atan (which = 0), tan (1), cbrt (2) of x[0..n-1].
void orc_cr_fn(int which, const double* x, int n, double* out) {
  for (int i = 0; i < n; ++i)
    out[i] = which == 0 ? cr_atan(x[i]) : (which == 1 ? cr_tan(x[i]) : cr_cbrt(x[i]));
}

// The near-field rule (mapped nodes eta, weights w; up to 2 npg of them) that
// integrate_element uses for element e and source point pf, with the pole
// (z0, e0) it came from; returns the number of nodes.
int orc_near_rule(const OrcGeom* og, int npg, int nearfield, int e, double pfx, double pfy, double* eta,
                  double* w, double* z0e0) {
  Geom gg = to_geom(og);
  Ctx C;
  setup_ctx(C, &gg, npg);
  C.nearfield = nearfield;
  const int nn = C.leg.np;
  V2 nodes[16];
  for (int k = 0; k < nn; ++k) nodes[k] = V2{gg.px[e * nn + k], gg.py[e * nn + k]};
  double z0, e0;
  complex_pole_1d(C.leg, nodes, nn, V2{pfx, pfy}, z0, e0);
  z0e0[0] = z0;
  z0e0[1] = e0;
  Rule x, wx;
  near_rule(C, nodes, V2{pfx, pfy}, gg.elen[e], x, wx);
  for (size_t i = 0; i < x.size(); ++i) {
    eta[i] = x[i];
    w[i] = wx[i];
  }
  return (int)x.size();
}

// Near classification mask, nt x ne (row-major by collocation row).
int orc_near_mask(const OrcGeom* og, double near_factor, uint8_t* mask) {
  Geom g = to_geom(og);
  const int nn = g.p + 1;
  for (int i = 0; i < g.nt; ++i) {
    V2 pf{g.px[i], g.py[i]};
    for (int e = 0; e < g.ne; ++e) {
      V2 xg[16];
      for (int k = 0; k < nn; ++k) xg[k] = V2{g.px[e * nn + k], g.py[e * nn + k]};
      bool on = (i >= e * nn && i < (e + 1) * nn);
      mask[(int64_t)i * g.ne + e] = (near_element(pf, xg, nn, g.elen[e], near_factor) || on) ? 1 : 0;
    }
  }
  return 0;
}

void orc_gausslegendre(int n, double* x, double* w) {
  std::vector<double> xv, wv;
  gauss_legendre(n, xv, wv);
  std::memcpy(x, xv.data(), sizeof(double) * n);
  std::memcpy(w, wv.data(), sizeof(double) * n);
}

// kind 0 Legendre(p), 1 Equispaced(p); L, dL have p+1 entries.
void orc_shapefun(int kind, int p, double xi, double* L, double* dL) {
  Poly P = kind == 0 ? make_legendre(p) : make_equispaced(p);
  shapefun(P, xi, L, dL);
}

// poly kind 0 Legendre, 1 Equispaced; nodes xy interleaved.
void orc_closest_point_1d(int kind, int p, const double* xy, double pfx, double pfy, double* xi,
                          double* x, double* dist) {
  Poly P = kind == 0 ? make_legendre(p) : make_equispaced(p);
  std::vector<V2> nodes(p + 1);
  for (int k = 0; k <= p; ++k) nodes[k] = V2{xy[2 * k], xy[2 * k + 1]};
  V2 pf{pfx, pfy}, xs;
  closest_point_1d(P, nodes.data(), p + 1, pf, seed_1d(P, nodes.data(), p + 1, pf), *xi, xs, *dist);
  x[0] = xs.x;
  x[1] = xs.y;
}

void orc_complex_pole_1d(int kind, int p, const double* xy, double pfx, double pfy, double* z0,
                         double* e0) {
  Poly P = kind == 0 ? make_legendre(p) : make_equispaced(p);
  std::vector<V2> nodes(p + 1);
  for (int k = 0; k <= p; ++k) nodes[k] = V2{xy[2 * k], xy[2 * k + 1]};
  complex_pole_1d(P, nodes.data(), p + 1, V2{pfx, pfy}, *z0, *e0);
}

// map ids: 0 tanp3c, 2 sinh(a,b), 3 sinh iterated niter=1, 4 niter=2, 5 tangent,
// 6 p3c, 7 eq40 real pole, 8 eq41 real pole.  Output buffers hold 2n.
int orc_map(int id, const double* u, const double* w, int n, double a, double b, double* x,
            double* wx) {
  Rule uu(u, u + n), ww(w, w + n), xx, wo;
  switch (id) {
    case 0: tanp3ctrans(uu, ww, a, b, xx, wo); break;
    case 2: sinhtrans(uu, ww, a, b, xx, wo); break;
    case 3: sinhtrans_iterated(uu, ww, a, b, 1, xx, wo); break;
    case 4: sinhtrans_iterated(uu, ww, a, b, 2, xx, wo); break;
    case 5: tangenttrans(uu, ww, a, b, xx, wo); break;
    case 6: p3ctrans(uu, ww, a, b, xx, wo); break;
    case 7: eq40_real_pole(uu, ww, a, xx, wo); break;
    case 8: eq41_real_pole(uu, ww, a, xx, wo); break;
    default: return -1;
  }
  for (size_t i = 0; i < xx.size(); ++i) { x[i] = xx[i]; wx[i] = wo[i]; }
  return (int)xx.size();
}

void orc_set_reference_degenerate_half(int on) { g_ref_degenerate_half = on; }

void orc_sinh_map(const double* u, int n, double a, double b, double* x, double* J) {
  Rule uu(u, u + n), xx, jj;
  sinh_map(uu, a, b, xx, jj);
  for (int i = 0; i < n; ++i) { x[i] = xx[i]; J[i] = jj[i]; }
}

void orc_eq40_AB(double z0, double* A, double* B, double* s) { eq40_AB(z0, *A, *B, *s); }

void orc_p3c_inv_pole(double z0, double e0, double* zt, double* et) { p3c_inv_pole(z0, e0, *zt, *et); }

// Interp rule: returns number of kept nodes; buffers of length n.
int orc_interp_rule(double a, int n, double* xi, double* w, double* Ni, double* d) {
  InterpRule R;
  if (!interp_rule(a, n, R)) return -1;
  for (size_t i = 0; i < R.xi.size(); ++i) {
    xi[i] = R.xi[i]; w[i] = R.w[i]; Ni[i] = R.Ni[i]; d[i] = R.d[i];
  }
  return (int)R.xi.size();
}

typedef double (*orc_fn1)(double);

// laurent_coefficients_interp (Integration.jl:622-...): writes 3 or 5 values,
// returns the count.
int orc_laurent_coefficients_interp(orc_fn1 f, double a, int order, int n, double* out) {
  InterpRule R;
  if (!interp_rule(a, n, R)) return -1;
  std::vector<double> F(R.xi.size());
  for (size_t i = 0; i < R.xi.size(); ++i) F[i] = f(R.xi[i]);
  double C[5];
  if (order == 0) { interp_log_coeff(F, 1, R, C); for (int t = 0; t < 3; ++t) out[t] = C[t]; return 3; }
  int cnt = interp_cascade(F, 1, R, order, C);
  for (int t = 0; t < cnt; ++t) out[t] = C[t];
  return cnt;
}

// guiggiani_integral with laurent=:interp (Integration.jl:398-404, 1824-1831)
double orc_guiggiani_integral_interp(orc_fn1 f, double a, int order, int n) {
  InterpRule R;
  if (!interp_rule(a, n, R)) return NAN;
  std::vector<double> F(R.xi.size());
  for (size_t i = 0; i < R.xi.size(); ++i) F[i] = f(R.xi[i]);
  double C[5], out;
  interp_coeffs(F, 1, R, order, C);
  interp_integrate(F, 1, R, C, order, a, &out);
  return out;
}

// guiggiani_GH with laurent=:interp for a scalar pair f -> (fg, fh)
void orc_guiggiani_GH_interp(orc_fn1 fg, orc_fn1 fh, double a, int og, int oh, int n, double* Ig,
                             double* Ih) {
  InterpRule R;
  interp_rule(a, n, R);
  std::vector<double> G(R.xi.size()), Hh(R.xi.size());
  for (size_t i = 0; i < R.xi.size(); ++i) { G[i] = fg(R.xi[i]); Hh[i] = fh(R.xi[i]); }
  double Cg[5], Ch[5];
  interp_coeffs(G, 1, R, og, Cg);
  interp_coeffs(Hh, 1, R, oh, Ch);
  interp_integrate(G, 1, R, Cg, og, a, Ig);
  interp_integrate(Hh, 1, R, Ch, oh, a, Ih);
}

void orc_laplace_kernel(double k, double rx, double ry, double nx, double ny, double* U, double* T) {
  laplace_UT(k, rx, ry, nx, ny, *U, *T);
}

void orc_kelvin_kernel(double mu, double nu, double rx, double ry, double nx, double ny, double* U,
                       double* T) {
  kelvin_UT(mu, nu, rx, ry, nx, ny, U, T);
}

int orc_near_element(const double* xy, int nn, double L, double pfx, double pfy, double factor) {
  std::vector<V2> xg(nn);
  for (int k = 0; k < nn; ++k) xg[k] = V2{xy[2 * k], xy[2 * k + 1]};
  return near_element(V2{pfx, pfy}, xg.data(), nn, L, factor) ? 1 : 0;
}

// applyBC Laplace / elasticity (src/Core/Boundary_conditions.jl:54-75,
// 152-174): A = H with BC==0 columns replaced by -G[:,j];
// b = sum_{BC==0} -H[:,j] BV_j + sum_{BC!=0} G[:,j] BV_j.
// rows x rows A, cols = number of boundary DOFs.
// _dibem_FD_kernel! / _elast_dibem_FD_kernel! (src/Laplace/DIBEM_GPU.jl:194-208,
// src/Elasticity/Assembly_GPU.jl:258-280) with _dibem_phi (DIBEM_GPU.jl:116-139)
static double dibem_phi(int kind, double R, double k, double epsa) {
  const double R2 = R * R;
  switch (kind) {
    case 1: return R;
    case 2: return R2 * std::log(R + epsa);
    case 3: return R2 * R;
    case 4: return (R2 * R2) * std::log(R + epsa);
    case 5: return R2 * R2 * R;
    case 6: return (R2 * R2 * R2) * std::log(R + epsa);
    case 7: return R2 * R2 * R2 * R;
    default: return -std::log(R) / (2.0 * kPi * k);
  }
}

void orc_dibem_fd2d(int nt, const double* px, const double* py, int kind, double prm0, double prm1, int rbf,
                    double epsa, double* F, double* D) {
  const int dof = kind == 0 ? 1 : 2;
  const int64_t ldd = (int64_t)dof * nt;
  for (int64_t q = 0; q < (int64_t)nt * nt; ++q) F[q] = 0.0;
  for (int64_t q = 0; q < ldd * ldd; ++q) D[q] = 0.0;
  const double eps2 = kEps * kEps;
  for (int j = 0; j < nt; ++j)
    for (int i = 0; i < nt; ++i) {
      if (i == j) continue;
      const double rx = px[j] - px[i], ry = py[j] - py[i];
      const double R2 = rx * rx + ry * ry;
      if (!(R2 > eps2)) continue;
      const double R = std::sqrt(R2);
      if (kind == 0) {
        D[i + (int64_t)j * nt] = -std::log(R) * (1.0 / (2.0 * kPi)) / prm0;
        F[i + (int64_t)j * nt] = dibem_phi(rbf, R, prm0, epsa);
      } else {
        F[i + (int64_t)j * nt] = dibem_phi(rbf, R, 1.0, epsa);
        const double mu = prm0, nu = prm1;
        const double dr1 = rx / R, dr2 = ry / R;
        const double prod1 = 4.0 * kPi * (1.0 - nu);
        const double prod2 = (3.0 - 4.0 * nu) * (-std::log(R));
        const double base = 2.0 * prod1 * mu;
        const double u11 = (prod2 + dr1 * dr1) / base, u12 = (dr1 * dr2) / base, u22 = (prod2 + dr2 * dr2) / base;
        D[2 * i + (int64_t)(2 * j) * ldd] = u11;
        D[2 * i + 1 + (int64_t)(2 * j) * ldd] = u12;
        D[2 * i + (int64_t)(2 * j + 1) * ldd] = u12;
        D[2 * i + 1 + (int64_t)(2 * j + 1) * ldd] = u22;
      }
    }
}

// Radial integrals of the DIBEM boundary terms: phi_int of each RBF kind
// (`_dibem_phi_int2d`, src/Laplace/DIBEM_GPU.jl:141-171) and of the Laplace
// fundamental solution (`_dibem_rad_id2d`, :173-177).
static double dibem_phi_int(int kind, double R, double k, double epsa) {
  const double R2 = R * R;
  switch (kind) {
    case 1: return R2 * R / 3.0;
    case 2: { const double R4 = R2 * R2; return (4.0 * R4 * std::log(R + epsa) - R4) / 16.0; }
    case 3: return R2 * R2 * R / 5.0;
    case 4: { const double R6 = R2 * R2 * R2; return R6 * std::log(R + epsa) / 6.0 - R6 / 36.0; }
    case 5: return R2 * R2 * R2 * R / 7.0;
    case 6: { const double R8 = (R2 * R2) * (R2 * R2); return R8 * std::log(R + epsa) / 8.0 - R8 / 64.0; }
    case 7: { const double R4 = R2 * R2; return R4 * R4 * R / 9.0; }
    default: return -(2.0 * R2 * std::log(R) - R2) / (8.0 * kPi * k);
  }
}
static double dibem_rad_id(double R, double k) {
  const double R2 = R * R;
  return -(2.0 * R2 * std::log(R) - R2) / (8.0 * kPi * k);
}

// Far (lumped) boundary sums of the DIBEM domain integrals, restating
// `_dibem_IFID_kernel!` (src/Laplace/DIBEM_GPU.jl:234-270): for every
// collocation point i and boundary node j with R = |x_j - x_i| > 1e-10, and
// the element e of node j unless (i, e) is near or i lies on e (the mask of
// `_near_skip_mask`, src/Laplace/Assembly_GPU.jl:236-253):
//   IF_i += phi_int(R) w_j (r . n_j) / R^2,   ID_i += rad(R) w_j (r . n_j) / R^2
// with w_j = Jacobian_j * elem_weight_k (discontinuous elements: one element
// per node).
int orc_dibem_ifid2d(const OrcGeom* og, double k, int rbf, double epsa, double near_factor, double* IF,
                     double* ID) {
  Geom g = to_geom(og);
  const int nn = g.p + 1;
  for (int i = 0; i < g.nt; ++i) {
    const V2 pf{g.px[i], g.py[i]};
    double aF = 0.0, aD = 0.0;
    for (int e = 0; e < g.ne; ++e) {
      V2 xg[16];
      for (int q = 0; q < nn; ++q) xg[q] = V2{g.px[e * nn + q], g.py[e * nn + q]};
      const bool on = (i >= e * nn && i < (e + 1) * nn);
      if (on || near_element(pf, xg, nn, g.elen[e], near_factor)) continue;
      for (int q = 0; q < nn; ++q) {
        const int j = e * nn + q;
        const double rx = g.px[j] - pf.x, ry = g.py[j] - pf.y;
        const double R2 = rx * rx + ry * ry;
        const double R = std::sqrt(R2);
        if (!(R > 1e-10)) continue;
        const double wJn = g.jac[j] * g.ew[q] * (rx * g.nx[j] + ry * g.ny[j]) / R2;
        aF += dibem_phi_int(rbf, R, k, epsa) * wJn;
        aD += dibem_rad_id(R, k) * wJn;
      }
    }
    IF[i] = aF;
    ID[i] = aD;
  }
  return 0;
}

// Near-pair correction of the DIBEM boundary sums, restating
// `_dibem_correct_near_cpu!` (src/Laplace/DIBEM_GPU.jl:272-300) with the
// element rules of `_rim_build_elements` (src/Core/DIBEM_common.jl:112-171):
// for every element e near point i (the assembly's near test) or holding it,
// the npg-point Gauss rule on the element's field interpolant,
//   IF_i += phi_int(R) w_q J_q (r . n_q) / R^2,  ID_i += rad(R) w_q J_q (r . n_q) / R^2
// (r = y_q - x_i, points with R < 1e-14 skipped, n_q aligned with the
// element's first nodal normal).  Adds to IF, ID.
int orc_dibem_ifid_near2d(const OrcGeom* og, double k, int rbf, double epsa, double near_factor, int npg,
                          double* IF, double* ID) {
  Geom g = to_geom(og);
  const int nn = g.p + 1;
  Poly leg = make_legendre(g.p);
  std::vector<double> qsi, w;
  gauss_legendre(npg, qsi, w);
  std::vector<double> yx(g.ne * npg), yy(g.ne * npg), nxq(g.ne * npg), nyq(g.ne * npg), wJ(g.ne * npg);
  for (int e = 0; e < g.ne; ++e) {
    const V2 nref{g.nx[e * nn], g.ny[e * nn]};
    for (int q = 0; q < npg; ++q) {
      double L[16], dL[16];
      shapefun(leg, qsi[q], L, dL);
      double px = 0, py = 0, dx = 0, dy = 0;
      for (int k2 = 0; k2 < nn; ++k2) {
        px += L[k2] * g.px[e * nn + k2];
        py += L[k2] * g.py[e * nn + k2];
        dx += dL[k2] * g.px[e * nn + k2];
        dy += dL[k2] * g.py[e * nn + k2];
      }
      const double J = std::sqrt(dx * dx + dy * dy);
      double ux = nref.x, uy = nref.y;
      if (!(J < 1e-16)) { ux = dy / J; uy = -dx / J; }
      if (ux * nref.x + uy * nref.y < 0) { ux = -ux; uy = -uy; }
      const int t = e * npg + q;
      yx[t] = px; yy[t] = py; nxq[t] = ux; nyq[t] = uy;
      wJ[t] = J < 1e-16 ? 0.0 : w[q] * J;
    }
  }
  for (int i = 0; i < g.nt; ++i) {
    const V2 pf{g.px[i], g.py[i]};
    double aF = 0.0, aD = 0.0;
    for (int e = 0; e < g.ne; ++e) {
      V2 xg[16];
      for (int q = 0; q < nn; ++q) xg[q] = V2{g.px[e * nn + q], g.py[e * nn + q]};
      const bool on = (i >= e * nn && i < (e + 1) * nn);
      if (!on && !near_element(pf, xg, nn, g.elen[e], near_factor)) continue;
      for (int q = 0; q < npg; ++q) {
        const int t = e * npg + q;
        if (wJ[t] == 0) continue;
        const double rx = yx[t] - pf.x, ry = yy[t] - pf.y;
        const double R = std::sqrt(rx * rx + ry * ry);
        if (R < 1e-14) continue;
        const double wJn = wJ[t] * ((nxq[t] * rx + nyq[t] * ry) / (R * R));
        aF += dibem_phi_int(rbf, R, k, epsa) * wJn;
        aD += dibem_rad_id(R, k) * wJn;
      }
    }
    IF[i] += aF;
    ID[i] += aD;
  }
  return 0;
}

// interior_laplace (src/Laplace/Lubrication.jl:399-416): potential at m
// interior points, every element through integrate_element.
int orc_interior_laplace(const OrcGeom* og, double k, int npg, int nearfield, const double* T,
                         const double* q, int m, const double* xp, const double* yp, double* out) {
  Geom gg = to_geom(og);
  Ctx C;
  setup_ctx(C, &gg, npg);
  C.prob.kind = 0;
  C.prob.k = k;
  C.nearfield = nearfield;
  C.singular = 0;
  const int nn = gg.p + 1;
#pragma omp parallel for schedule(static)
  for (int p = 0; p < m; ++p) {
    std::vector<double> h(nn), g(nn);
    double gt = 0.0, hs = 0.0;
    for (int e = 0; e < gg.ne; ++e) {
      integrate_element(C, e, V2{xp[p], yp[p]}, -1, h.data(), g.data());
      for (int a = 0; a < nn; ++a) {
        const int j = e * nn + a;
        gt += g[a] * q[j] - h[a] * T[j];
        hs += h[a];
      }
    }
    out[p] = gt / (-hs);
  }
  return 0;
}

// recover_strain_stress! 2-D (src/Elasticity/StrainStress.jl:55-99): Kane's
// boundary strain/stress per collocation node; eps, sig n x 3 column-major.
void orc_strain_stress2d(const OrcGeom* og, double lam, double mu, const double* u, const double* t,
                         double* eps, double* sig) {
  const Geom g = to_geom(og);
  const Poly P = make_legendre(g.p);
  const int nn = g.p + 1, n = g.n;
  std::vector<double> N(nn), dN(nn);
  for (int i = 0; i < 3 * n; ++i) eps[i] = sig[i] = 0.0;
  for (int e = 0; e < g.ne; ++e) {
    for (int k = 0; k < nn; ++k) {
      shapefun(P, P.nodes[k], N.data(), dN.data());
      double dx0 = 0, dx1 = 0, du0 = 0, du1 = 0;
      for (int j = 0; j < nn; ++j) {
        const int ja = e * nn + j;
        dx0 += dN[j] * g.px[ja];
        dx1 += dN[j] * g.py[ja];
        du0 += dN[j] * u[2 * ja];
        du1 += dN[j] * u[2 * ja + 1];
      }
      const int i = e * nn + k;
      const double nlen = std::hypot(g.nx[i], g.ny[i]);
      const double n1 = g.nx[i] / nlen, n2 = g.ny[i] / nlen, t1 = -n2, t2 = n1;
      const double Jproj = t1 * dx0 + t2 * dx1;
      if (std::fabs(Jproj) < 1e-16) continue;
      const double dudt0 = du0 / Jproj, dudt1 = du1 / Jproj;
      const double ess = t1 * dudt0 + t2 * dudt1;
      const double tv0 = t[2 * i], tv1 = t[2 * i + 1];
      const double snn = n1 * tv0 + n2 * tv1, snt = t1 * tv0 + t2 * tv1;
      const double den = lam + 2 * mu;
      if (std::fabs(den) < 1e-30) continue;
      const double enn = (snn - lam * ess) / den, ent = snt / (2 * mu);
      const double sss = lam * (enn + ess) + 2 * mu * ess;
      eps[i] = enn * n1 * n1 + ess * t1 * t1 + 2 * ent * n1 * t1;
      eps[i + n] = enn * n2 * n2 + ess * t2 * t2 + 2 * ent * n2 * t2;
      eps[i + 2 * n] = 2 * (enn * n1 * n2 + ess * t1 * t2 + ent * (n1 * t2 + n2 * t1));
      sig[i] = snn * n1 * n1 + sss * t1 * t1 + 2 * snt * n1 * t1;
      sig[i + n] = snn * n2 * n2 + sss * t2 * t2 + 2 * snt * n2 * t2;
      sig[i + 2 * n] = snn * n1 * n2 + sss * t1 * t2 + snt * (n1 * t2 + n2 * t1);
    }
  }
}

void orc_apply_bc(int64_t rows, int64_t cols, const double* H, const double* G, const int32_t* BC,
                  const double* BV, double* A, double* b) {
  std::memcpy(A, H, sizeof(double) * rows * rows);
  for (int64_t j = 0; j < cols; ++j)
    if (BC[j] == 0)
      for (int64_t i = 0; i < rows; ++i) A[i + j * rows] = -G[i + j * rows];
  for (int64_t i = 0; i < rows; ++i) b[i] = 0.0;
  for (int64_t j = 0; j < cols; ++j) {
    if (BC[j] == 0) {
      for (int64_t i = 0; i < rows; ++i) b[i] -= H[i + j * rows] * BV[j];
    } else {
      for (int64_t i = 0; i < rows; ++i) b[i] += G[i + j * rows] * BV[j];
    }
  }
}

}  // extern "C"
