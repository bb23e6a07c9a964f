// Host build of the near-singular quadrature map the GPU kernels use
// (bem_gmsh_gb300/csrc/bem_nearmap.cuh) and of its correctly rounded
// functions (bem_crmath.cuh).  Compiled by tests/test_crmath_cpu.py with
// floating-point contraction off: `ieee` arithmetic is then the same IEEE
// operations as the device build's explicit round-to-nearest intrinsics, so
// these results are the GPU's bits.
#include "../../bem_gmsh_gb300/csrc/bem_nearmap.cuh"

namespace {
struct HostRule {
  int npg;
  double qsi[32], w[32], leg_x[8];
};
}  // namespace

extern "C" {

void h_cr_fn(int which, const double* x, int n, double* out) {
  for (int i = 0; i < n; ++i)
    out[i] = which == 0 ? bem::crm::cr_atan(x[i]) : (which == 1 ? bem::crm::cr_tan(x[i]) : bem::crm::cr_cbrt(x[i]));
}

void h_gauss(int n, double* x, double* w) { bem::crm::gauss_legendre_cr(n, x, w); }

// pi/2 in three parts, tan(j/32) (26 x 2), tan series coefficients
// (3 x 2 + 4), atan(j/16) (17 x 2), 1/(2k+1) for k = 1..5 (5 x 2) and
// k = 6..11 (6)
void h_constants(double* out) {
  int k = 0;
  out[k++] = BEM_PIO2_0;
  out[k++] = BEM_PIO2_1;
  out[k++] = BEM_PIO2_2;
  for (int j = 0; j < 26; ++j) {
    out[k++] = bem::crm::kTanTab[j][0];
    out[k++] = bem::crm::kTanTab[j][1];
  }
  const double c[] = {BEM_TC1_HI, BEM_TC1_LO, BEM_TC2_HI, BEM_TC2_LO, BEM_TC3_HI,
                      BEM_TC3_LO, BEM_TC4,    BEM_TC5,    BEM_TC6,    BEM_TC7};
  for (double v : c) out[k++] = v;
  for (int j = 0; j < 17; ++j) {
    out[k++] = bem::crm::kAtanTab[j][0];
    out[k++] = bem::crm::kAtanTab[j][1];
  }
  for (int j = 0; j < 5; ++j) {
    out[k++] = bem::crm::kOddInv[j][0];
    out[k++] = bem::crm::kOddInv[j][1];
  }
  const double o[] = {BEM_ODD13, BEM_ODD15, BEM_ODD17, BEM_ODD19, BEM_ODD21, BEM_ODD23};
  for (double v : o) out[k++] = v;
}

// tanp3c rule of an element with p+1 nodes (x, y) for source point pf:
// writes eta, w (up to 2 npg) and the pole; returns the node count, or -1
// when the element has more than 3 nodes (closest-point branch, not here).
int h_near_rule(int p, int npg, const double* nx, const double* ny, double pfx, double pfy, double* eta,
                double* w, double* z0e0) {
  HostRule R{};
  R.npg = npg;
  bem::crm::gauss_legendre_cr(npg, R.qsi, R.w);
  double lw[8];
  bem::crm::gauss_legendre_cr(p + 1, R.leg_x, lw);
  double z0, e0;
  if (!bem::nm::complex_pole(R, nx, ny, p + 1, pfx, pfy, z0, e0)) return -1;
  z0e0[0] = z0;
  z0e0[1] = e0;
  return bem::nm::tanp3ctrans(R, z0, e0, eta, w);
}

}  // extern "C"
