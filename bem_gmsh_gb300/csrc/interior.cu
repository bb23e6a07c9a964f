// Laplace potential at interior points from the solved boundary data,
// restating `interior_laplace` (src/Laplace/Lubrication.jl:399-416; the
// same sum is `_interior_T`, test/laplace.jl:36-53):
//   h_j, g_j = integrate_element over every element (closest point, then the
//              on-element Guiggiani rule if the point lies on the element,
//              else the near-field quadrature, Assembly_full.jl:262-289)
//   c = -sum_j h_j,   T(p) = (g . q - h . T) / c.
// One CTA per point; its threads take elements in a fixed order and the
// FP64 partial sums are reduced in a fixed tree, so results are
// reproducible.
#include <cstring>

#include "bem_abi_internal.h"

namespace bem {
namespace {

constexpr int IT = 128;  // threads per point

__global__ void __launch_bounds__(IT) interior_laplace_kernel(GeomDev g, Rules R, Physics ph,
                                                              const double* __restrict__ T,
                                                              const double* __restrict__ q,
                                                              const double* __restrict__ xp,
                                                              const double* __restrict__ yp,
                                                              double* __restrict__ out) {
  __shared__ double s_gt[IT / 32], s_h[IT / 32];
  const int p = blockIdx.x;
  const V2 pf{xp[p], yp[p]};
  const int nn = g.nn;
  double gt = 0.0, hs = 0.0;
  for (int e = threadIdx.x; e < g.ne; e += IT) {
    V2 nodes[BEM_MAXNN], geo[BEM_MAXGEO];
    load_element(g, e, nodes, geo);
    double h[BEM_MAXNN], gg[BEM_MAXNN];
    double xa, dist;
    closest_point_1d(R, nodes, nn, pf, xa, dist);
    const V2 nref{g.nx[e * nn], g.ny[e * nn]};
    if (dist <= 1e-12)
      if (R.singular == 1)
        integrate_singular_telles<1>(R, ph, nodes, geo, pf, xa, nref, h, gg);
      else
        integrate_singular<1>(R, ph, nodes, geo, pf, xa, nref, h, gg);
    else
      integrate_near<1>(R, ph, nodes, geo, pf, g.elen[e], nref, h, gg);
    for (int a = 0; a < nn; ++a) {
      const int j = e * nn + a;
      gt += gg[a] * q[j] - h[a] * T[j];
      hs += h[a];
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    gt += __shfl_xor_sync(0xffffffffu, gt, o);
    hs += __shfl_xor_sync(0xffffffffu, hs, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s_gt[threadIdx.x >> 5] = gt;
    s_h[threadIdx.x >> 5] = hs;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < IT / 32; ++w) {
      a += s_gt[w];
      b += s_h[w];
    }
    out[p] = a / (-b);
  }
}

}  // namespace
}  // namespace bem

using namespace bem;

extern "C" int bem_interior_laplace2d(bem_ctx* c, const bem_geom2d* g, double k, int npg, const double* T,
                                      const double* q, int64_t m, const double* xp, const double* yp,
                                      int mem, double* out) {
  if (!c || !g || !T || !q || m < 0 || (m > 0 && (!xp || !yp || !out))) return BEM_ERR_INVALID;
  if (mem != BEM_MEM_HOST && mem != BEM_MEM_DEVICE) return BEM_ERR_INVALID;
  if (!(k > 0)) return BEM_ERR_INVALID;
  if (m > (int64_t)0x7fffffff) return BEM_ERR_UNSUPPORTED;
  int rc = bem_check_geom(g, npg, 1.5);
  if (rc) return rc;
  if (m == 0) return BEM_OK;
  CallScope cs(c);
  cudaSetDevice(c->device);
  GeomDev gd;
  Rules R;
  rc = bem_stage_geom(c, g, npg, mem, gd, R);
  if (rc) return rc;
  Physics ph{};
  ph.kind = 0;
  ph.k = k;
  const size_t n = (size_t)g->n, mm = (size_t)m;
  const double *dT = T, *dq = q, *dx = xp, *dy = yp;
  double* dout = out;
  if (mem == BEM_MEM_HOST) {
    double* buf = (double*)c->get(bem_ctx::SLOT_OUT3, sizeof(double) * (2 * n + 3 * mm));
    if (!buf) return BEM_ERR_NOMEM;
    cudaMemcpyAsync(buf, T, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(buf + n, q, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(buf + 2 * n, xp, sizeof(double) * mm, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(buf + 2 * n + mm, yp, sizeof(double) * mm, cudaMemcpyHostToDevice, c->stream);
    dT = buf;
    dq = buf + n;
    dx = buf + 2 * n;
    dy = buf + 2 * n + mm;
    dout = buf + 2 * n + 2 * mm;
  }
  interior_laplace_kernel<<<(unsigned)m, IT, 0, c->stream>>>(gd, R, ph, dT, dq, dx, dy, dout);
  count_launches(1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "interior_laplace_kernel");
  if (mem == BEM_MEM_HOST) cudaMemcpyAsync(out, dout, sizeof(double) * mm, cudaMemcpyDeviceToHost, c->stream);
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "interior_laplace");
  return BEM_OK;
}
