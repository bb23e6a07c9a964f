// Device-side FP64 machinery for the near-singular and singular element
// integrals of the dense 2-D collocation assembly, restating the reference
// (Julia package `BEM`, paths relative to its project root):
//   shape functions       src/Core/Interpolation.jl:148-218
//   closest point         src/Core/Integration.jl:323-349, 1005-1033
//   complex pole          src/Core/Integration.jl:1117-1160
//   tanp3c map            src/Core/Integration.jl:1163-1365
//   sinh-family maps      src/Core/Integration.jl:1062-1115, 1367-1395
//   interpolated Guiggiani src/Core/Integration.jl:1598-1845
//   kernels               src/Laplace/Fundamental.jl:19-25,
//                         src/Elasticity/Fundamental.jl:28-60
// Everything here is per-thread scalar code: one thread integrates one
// (collocation point, element) pair.  Arrays live in registers / local memory.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "bem_nearmap.cuh"

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
  // near-field map (`nearfield`, Integration.jl:41-93): 0 tanp3c, 1 plain
  // Gauss, 2 euclid, 3 csinh, 4 sinhsinh, 5 tangent, 6 p3c; on-element
  // rule (`singular`, Assembly_full.jl:282-283): 0 interpolated Guiggiani,
  // 1 Telles
  unsigned char nearfield, singular, pad0_, pad1_;
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
// complex pole and tanp3c map: exactly specified IEEE arithmetic and
// correctly rounded atan/tan/cbrt (bem_nearmap.cuh), so that the map's
// nodes and weights are the same bits as a CPU restatement's
// --------------------------------------------------------------------------
// _complex_pole_1d (Integration.jl:1117-1160)
__device__ inline void complex_pole_1d(const Rules& R, const V2* nodes, int nN, V2 pf, double& z0,
                                double& e0) {
  if (nN <= 3) {
    double nx[3], ny[3];
    for (int k = 0; k < nN; ++k) { nx[k] = nodes[k].x; ny[k] = nodes[k].y; }
    if (nm::complex_pole(R, nx, ny, nN, pf.x, pf.y, z0, e0)) return;
  }
  double a, dist;
  closest_point_1d(R, nodes, nN, pf, a, dist);
  double L[BEM_MAXNN], dL[BEM_MAXNN];
  shapefun(R.leg_x, R.leg_bw, R.leg_D, nN, a, L, dL);
  V2 dx = comb(dL, nodes, nN);
  z0 = a;
  e0 = dist / fmax(vnorm(dx.x, dx.y), 1e-14);
}

// _tanp3ctrans (Integration.jl:1290-1365): up to 2*npg nodes, returns the count
__device__ inline int tanp3ctrans(const Rules& R, double z0, double e0, double* x, double* wx) {
  return nm::tanp3ctrans(R, z0, e0, x, wx);
}

// --------------------------------------------------------------------------
// sinh-family maps (`:euclid`, `:csinh`, `:sinhsinh`; Integration.jl:1062-1115,
// 1367-1395).  Unlike the tangent maps these are well conditioned: a node
// moves by b cosh(mu u - eta) per unit of its argument, the width b of the
// peak that the node resolves, so one ulp of asinh, sinh or exp stays about
// one ulp of the integral; they use the platform's FP64 functions.
// --------------------------------------------------------------------------
__device__ __forceinline__ void sinh_consts(double a, double b, double& mu, double& eta) {
  const double sp = asinh((1 + a) / b), sm = asinh((1 - a) / b);
  mu = 0.5 * (sp + sm);
  eta = 0.5 * (sp - sm);
}

// eq. (40) with a collinear real pole |z0| > 1 (_eq40_real_pole, _eq40_AB):
// x = z0 + s exp((u - B) / A), s = -sign(z0), with x(+-1) = +-1
static __device__ __noinline__ int eq40_real_pole(const Rules& R, double z0, double* x, double* wx) {
  const int m = R.npg;
  double A = 0.0, B = 0.0, s = 0.0;
  if (fabs(z0) > 1) {
    s = z0 > 0 ? -1.0 : 1.0;
    const double lm = log(s * (-1 - z0)), lp = log(s * (1 - z0));
    A = 2.0 / (lp - lm);
    B = -A / 2 * (lp + lm);
  }
  if (fabs(z0) <= 1 || fabs(A) < 1e-30) {
    for (int i = 0; i < m; ++i) { x[i] = R.qsi[i]; wx[i] = R.w[i]; }
    return m;
  }
  for (int i = 0; i < m; ++i) {
    const double e = exp((R.qsi[i] - B) / A);
    x[i] = z0 + s * e;
    wx[i] = R.w[i] * (s * e / A);
  }
  return m;
}

// _sinhtrans_iterated: niter = 1 is the sinh map about (a, b) (eq. 40),
// niter = 2 the sinh-sinh map whose outer sinh sits on the inner one's
// image pole; also _sinhtrans (the `:euclid` map), which is niter = 1.
// Not inlined (nor is the `:euclid` rule below): the default tanp3c path of
// the element integrals keeps its registers.
static __device__ __noinline__ int sinhtrans(const Rules& R, double a, double b, int niter, double* x,
                                             double* wx) {
  if (fabs(b) < 1e-14 && fabs(a) > 1) return eq40_real_pole(R, a, x, wx);
  b = fmax(b, 1e-14);
  double ma[2], mb[2], mmu[2], meta[2];
  int nmap = 0;
  double aa = a, bb = b;
  for (int it = 0; it < niter && it < 2; ++it) {
    double mu, eta;
    sinh_consts(aa, bb, mu, eta);
    ma[nmap] = aa;
    mb[nmap] = bb;
    mmu[nmap] = mu;
    meta[nmap] = eta;
    ++nmap;
    if (mu < 1e-14) break;
    aa = fmin(fmax(eta / mu, nextafter(-1.0, 0.0)), nextafter(1.0, 0.0));
    bb = fmax(kPi / (2 * mu), 1e-14);
  }
  for (int i = 0; i < R.npg; ++i) {
    double xi = R.qsi[i], J = 1.0;
    for (int k = nmap - 1; k >= 0; --k) {  // the last map acts on the Gauss nodes first
      const double t = mmu[k] * xi - meta[k];
      J *= mb[k] * mmu[k] * cosh(t);
      xi = ma[k] + mb[k] * sinh(t);
    }
    x[i] = xi;
    wx[i] = R.w[i] * J;
  }
  return R.npg;
}

// `:euclid`: sinh about the Euclidean closest point, width b = d / L
static __device__ __noinline__ int euclid_rule(const Rules& R, const V2* nodes, int nn, V2 pf, double Lel,
                                               double* x, double* wx) {
  double a, dist;
  closest_point_1d(R, nodes, nn, pf, a, dist);
  return sinhtrans(R, a, fmax(dist / fmax(Lel, kEps), 1e-14), 1, x, wx);
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
                               V2 pf, double Lel, V2 nref, double* h, double* g) {
  const int nn = R.nn;
  double eta[BEM_MAXMAP], ww[BEM_MAXMAP];
  int m;
  if (R.nearfield == 1) {  // plain Gauss rule
    m = R.npg;
    for (int i = 0; i < m; ++i) { eta[i] = R.qsi[i]; ww[i] = R.w[i]; }
  } else if (R.nearfield == 2) {
    m = euclid_rule(R, nodes, nn, pf, Lel, eta, ww);
  } else {
    double z0, e0;
    complex_pole_1d(R, nodes, nn, pf, z0, e0);
    if (R.nearfield == 3 || R.nearfield == 4) m = sinhtrans(R, z0, e0, R.nearfield == 4 ? 2 : 1, eta, ww);
    else if (R.nearfield == 5) m = nm::tangenttrans(R, nm::ieee(z0), nm::ieee(e0), eta, ww);
    else if (R.nearfield == 6) m = nm::p3ctrans(R, nm::ieee(z0), nm::ieee(e0), eta, ww);
    else m = tanp3ctrans(R, z0, e0, eta, ww);
  }
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
// Telles on-element rule (_telles_map, _integrate_singular_telles!,
// Assembly_full.jl:467-528): the near-field Gauss rule through the cubic map
// whose derivative vanishes at the source's parent coordinate a.  The map's
// constants use the correctly rounded cbrt and explicit IEEE operations, so
// they are the bits of a CPU restatement.
// --------------------------------------------------------------------------
template <int NC>
__device__ inline void integrate_singular_telles(const Rules& R, const Physics& ph, const V2* nodes,
                                                 const V2* geo, V2 pf, double a, V2 nref, double* h, double* g) {
  using nm::ieee;
  const int nn = R.nn;
  for (int c = 0; c < nn * NC; ++c) h[c] = g[c] = 0.0;
  a = fmin(fmax(a, -0.9999999999999999), 0.9999999999999999);
  const ieee eet = a;
  const ieee eest = eet * eet - ieee(1.0);
  const ieee term1 = crm::cr_cbrt((eet * eest + abs(eest)).v);
  const ieee term2 = crm::cr_cbrt((eet * eest - abs(eest)).v);
  const ieee Gm = term1 + term2 + eet;
  const ieee Q = ieee(1.0) + ieee(3.0) * (Gm * Gm);
  const ieee A = ieee(1.0) / Q, B = ieee(-3.0) * Gm / Q, Cc = ieee(3.0) * (Gm * Gm) / Q, D = -B;
  for (int i = 0; i < R.npg; ++i) {
    const ieee gm = R.qsi[i];
    const double eta = (A * (gm * gm * gm) + B * (gm * gm) + Cc * gm + D).v;
    const double Jt = (ieee(3.0) * A * (gm * gm) + ieee(2.0) * B * gm + Cc).v;
    double N[BEM_MAXNN];
    V2 pg, dx;
    shape_geom(R, nodes, geo, eta, N, pg, dx);
    const double J = vnorm(dx.x, dx.y);
    if (J < 1e-30) continue;
    const double rx = pg.x - pf.x, ry = pg.y - pf.y;
    if (vnorm(rx, ry) < 1e-30) continue;
    const double invJ = 1.0 / J;
    double nxq = dx.y * invJ, nyq = -(dx.x * invJ);
    if (nxq * nref.x + nyq * nref.y < 0) { nxq = -nxq; nyq = -nyq; }
    double U[4], T[4];
    eval_kernel<NC>(ph, rx, ry, nxq, nyq, U, T);
    const double wJ = Jt * R.w[i] * J;
    for (int j = 0; j < nn; ++j) {
      const double Nj = N[j] * wJ;
      for (int c = 0; c < NC; ++c) {
        g[j * NC + c] += U[c] * Nj;
        h[j * NC + c] += T[c] * Nj;
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
