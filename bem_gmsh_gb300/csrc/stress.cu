// Boundary strain and stress at the collocation nodes (Kane's method),
// restating `_recover_2d!` (src/Elasticity/StrainStress.jl:55-99) of the
// reference: per node, the tangential derivative of the displacement
// interpolant on its own element and the traction t = sigma n give the local
// (n, t) strain and stress, rotated back to x, y.  Discontinuous elements:
// every node belongs to one element, no averaging.  One thread per node.
#include <cstring>

#include "bem_abi_internal.h"

namespace bem {
namespace {

__global__ void strain_stress_kernel(GeomDev g, Rules R, double lam, double mu, const double* __restrict__ u,
                                     const double* __restrict__ t, double* __restrict__ eps,
                                     double* __restrict__ sig) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const int nn = g.nn, e = i / nn, k = i % nn;
  // shapefun at the k-th parent node: N = e_k, dN = row k of the
  // differentiation matrix (Interpolation.jl:148-218)
  double dx0 = 0.0, dx1 = 0.0, du0 = 0.0, du1 = 0.0;
  for (int j = 0; j < nn; ++j) {
    const double d = R.leg_D[k * nn + j];
    const int ja = e * nn + j;
    dx0 += d * g.px[ja];
    dx1 += d * g.py[ja];
    du0 += d * u[2 * ja];
    du1 += d * u[2 * ja + 1];
  }
  for (int c = 0; c < 3; ++c) {
    eps[i + (size_t)c * g.n] = 0.0;
    sig[i + (size_t)c * g.n] = 0.0;
  }
  // local_basis2d (src/Elasticity/LocalFrame.jl:33-39)
  const double nlen = hypot(g.nx[i], g.ny[i]);
  if (!(nlen >= 2.220446049250313e-16)) return;
  const double n1 = g.nx[i] / nlen, n2 = g.ny[i] / nlen;
  const double t1 = -n2, t2 = n1;
  const double Jproj = t1 * dx0 + t2 * dx1;
  if (fabs(Jproj) < 1e-16) return;
  const double dudt0 = du0 / Jproj, dudt1 = du1 / Jproj;
  const double ess = t1 * dudt0 + t2 * dudt1;
  const double tv0 = t[2 * i], tv1 = t[2 * i + 1];
  const double snn = n1 * tv0 + n2 * tv1;
  const double snt = t1 * tv0 + t2 * tv1;
  const double den = lam + 2 * mu;
  if (fabs(den) < 1e-30) return;
  const double enn = (snn - lam * ess) / den;
  const double ent = snt / (2 * mu);
  const double sss = lam * (enn + ess) + 2 * mu * ess;
  eps[i] = enn * n1 * n1 + ess * t1 * t1 + 2 * ent * n1 * t1;
  eps[i + (size_t)g.n] = enn * n2 * n2 + ess * t2 * t2 + 2 * ent * n2 * t2;
  eps[i + 2 * (size_t)g.n] = 2 * (enn * n1 * n2 + ess * t1 * t2 + ent * (n1 * t2 + n2 * t1));
  sig[i] = snn * n1 * n1 + sss * t1 * t1 + 2 * snt * n1 * t1;
  sig[i + (size_t)g.n] = snn * n2 * n2 + sss * t2 * t2 + 2 * snt * n2 * t2;
  sig[i + 2 * (size_t)g.n] = snn * n1 * n2 + sss * t1 * t2 + snt * (n1 * t2 + n2 * t1);
}

}  // namespace
}  // namespace bem

using namespace bem;

extern "C" int bem_strain_stress2d(bem_ctx* c, const bem_geom2d* g, double lam, double mu, const double* u,
                                   const double* t, int mem, double* eps, double* sigma) {
  if (!c || !g || !u || !t || !eps || !sigma) return BEM_ERR_INVALID;
  if (mem != BEM_MEM_HOST && mem != BEM_MEM_DEVICE) return BEM_ERR_INVALID;
  if (!(mu > 0) || !(lam == lam)) return BEM_ERR_INVALID;
  int rc = bem_check_geom(g, 2, 1.5);
  if (rc) return rc;
  CallScope cs(c);
  cudaSetDevice(c->device);
  GeomDev gd;
  Rules R;
  rc = bem_stage_geom(c, g, 2, mem, gd, R);
  if (rc) return rc;
  const size_t n = (size_t)g->n;
  const double *du = u, *dt = t;
  double *de = eps, *ds = sigma;
  if (mem == BEM_MEM_HOST) {
    double* buf = (double*)c->get(bem_ctx::SLOT_OUT2, sizeof(double) * (4 * n + 6 * n));
    if (!buf) return BEM_ERR_NOMEM;
    cudaMemcpyAsync(buf, u, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(buf + 2 * n, t, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, c->stream);
    du = buf;
    dt = buf + 2 * n;
    de = buf + 4 * n;
    ds = buf + 7 * n;
  }
  strain_stress_kernel<<<(int)((n + 127) / 128), 128, 0, c->stream>>>(gd, R, lam, mu, du, dt, de, ds);
  count_launches(1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "strain_stress_kernel");
  if (mem == BEM_MEM_HOST) {
    cudaMemcpyAsync(eps, de, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(sigma, ds, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream);
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "strain_stress");
  return BEM_OK;
}
