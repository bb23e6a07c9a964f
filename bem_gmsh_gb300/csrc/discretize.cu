// Boundary discretisation on the device: from each element's equispaced CAD
// nodes to its p+1 collocation nodes at the Gauss-Legendre points, with the
// Jacobian, the outward normal (tangent rotated by -90 degrees, `tan2normal`)
// and the element length |sum_k J_k w_k| -- the geometry part of `format2d`
// (src/Core/Input.jl:163-185, `_bemdata_2d` :516-535).  One thread per
// element; the Lagrange basis of the CAD nodes at the Gauss points is built
// once on the host.
#include <cmath>
#include <cstring>
#include <vector>

#include "bem_abi_internal.h"
#include "bem_crmath.cuh"

namespace bem {
namespace {

struct DiscRule {
  int nn, ngeo;
  double N[BEM_MAXNN * BEM_MAXGEO], dN[BEM_MAXNN * BEM_MAXGEO];  // [gauss k][cad m]
  double w[BEM_MAXNN];
};

__global__ void discretize_kernel(int ne, DiscRule r, const double* __restrict__ cx, const double* __restrict__ cy,
                                  double* px, double* py, double* nx, double* ny, double* jac, double* elen) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double L = 0.0;
  for (int k = 0; k < r.nn; ++k) {
    double x = 0.0, y = 0.0, dx = 0.0, dy = 0.0;
    for (int m = 0; m < r.ngeo; ++m) {
      const double gx = cx[(size_t)e * r.ngeo + m], gy = cy[(size_t)e * r.ngeo + m];
      x += r.N[k * r.ngeo + m] * gx;
      y += r.N[k * r.ngeo + m] * gy;
      dx += r.dN[k * r.ngeo + m] * gx;
      dy += r.dN[k * r.ngeo + m] * gy;
    }
    const double J = sqrt(dx * dx + dy * dy);
    const size_t j = (size_t)e * r.nn + k;
    px[j] = x;
    py[j] = y;
    nx[j] = dy / J;
    ny[j] = -dx / J;
    jac[j] = J;
    L += J * r.w[k];
  }
  elen[e] = fabs(L);
}

// Lagrange basis of the equispaced nodes -1 + 2m/(n-1) and its derivative at x
void lagrange_equi(int n, double x, double* N, double* dN) {
  std::vector<double> t(n);
  for (int m = 0; m < n; ++m) t[m] = n == 1 ? 0.0 : -1.0 + 2.0 * m / (n - 1);
  for (int m = 0; m < n; ++m) {
    double v = 1.0, d = 0.0;
    for (int q = 0; q < n; ++q) {
      if (q == m) continue;
      const double den = t[m] - t[q];
      double prod = 1.0 / den;
      for (int s = 0; s < n; ++s)
        if (s != m && s != q) prod *= (x - t[s]) / (t[m] - t[s]);
      d += prod;
      v *= (x - t[q]) / den;
    }
    N[m] = v;
    dN[m] = d;
  }
}

}  // namespace

void gauss_legendre_nodes(int n, double* x, double* w);  // bem_abi.cu

}  // namespace bem

using namespace bem;

extern "C" int bem_discretize2d(bem_ctx* c, int ne, int ngeo, int p, const double* cad_x, const double* cad_y,
                                int mem, double* px, double* py, double* nx, double* ny, double* jac,
                                double* elen, double* elem_weight) {
  if (!c || ne <= 0 || !cad_x || !cad_y || !px || !py || !nx || !ny || !jac || !elen || !elem_weight)
    return BEM_ERR_INVALID;
  if (p < 0 || p + 1 > BEM_MAXNN || ngeo < 2 || ngeo > BEM_MAXGEO) return BEM_ERR_INVALID;
  if (mem != BEM_MEM_HOST && mem != BEM_MEM_DEVICE) return BEM_ERR_INVALID;
  CallScope cs(c);
  cudaSetDevice(c->device);
  DiscRule r{};
  r.nn = p + 1;
  r.ngeo = ngeo;
  double gx[BEM_MAXNN], gw[BEM_MAXNN];
  bem::gauss_legendre_nodes(r.nn, gx, gw);
  for (int k = 0; k < r.nn; ++k) {
    lagrange_equi(ngeo, gx[k], r.N + k * ngeo, r.dN + k * ngeo);
    r.w[k] = gw[k];
    elem_weight[k] = gw[k];  // host array (p+1 values)
  }
  const size_t n = (size_t)ne * r.nn, ng = (size_t)ne * ngeo;
  const double *dcx = cad_x, *dcy = cad_y;
  double *o = nullptr;
  double *dpx = px, *dpy = py, *dnx = nx, *dny = ny, *dj = jac, *dl = elen;
  if (mem == BEM_MEM_HOST) {
    o = (double*)c->get(bem_ctx::SLOT_OUT2, sizeof(double) * (2 * ng + 5 * n + ne));
    if (!o) return BEM_ERR_NOMEM;
    cudaMemcpyAsync(o, cad_x, sizeof(double) * ng, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(o + ng, cad_y, sizeof(double) * ng, cudaMemcpyHostToDevice, c->stream);
    dcx = o;
    dcy = o + ng;
    dpx = o + 2 * ng;
    dpy = dpx + n;
    dnx = dpy + n;
    dny = dnx + n;
    dj = dny + n;
    dl = dj + n;
  }
  discretize_kernel<<<(ne + 127) / 128, 128, 0, c->stream>>>(ne, r, dcx, dcy, dpx, dpy, dnx, dny, dj, dl);
  count_launches(1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "discretize_kernel");
  if (mem == BEM_MEM_HOST) {
    cudaMemcpyAsync(px, dpx, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(py, dpy, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(nx, dnx, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(ny, dny, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(jac, dj, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(elen, dl, sizeof(double) * ne, cudaMemcpyDeviceToHost, c->stream);
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "discretize");
  return BEM_OK;
}

// ---------------------------------------------------------------------------
// outward normals (`_orient_normals_outward!`, src/Core/Input.jl:376-389)
// ---------------------------------------------------------------------------
namespace bem {
namespace {

constexpr int kOrientChunk = 256;  // cells staged per block and pass

// Even-odd ray test of point (x, y) against a polygon of 4 corners (a
// triangle repeats its last corner, whose zero-height edge never counts);
// `point_in_polygon` (src/Core/Input.jl:331-345) in explicit IEEE operations.
__device__ bool in_cell(double x, double y, const double* v) {
  using crm::ieee;
  bool inside = false;
  int j = 3;
  for (int i = 0; i < 4; ++i) {
    const ieee xi = v[2 * i], yi = v[2 * i + 1], xj = v[2 * j], yj = v[2 * j + 1];
    if ((yi.v > y) != (yj.v > y)) {
      const ieee xint = (xj - xi) * (ieee(y) - yi) / (yj - yi + ieee(1e-30)) + xi;
      if (x < xint.v) inside = !inside;
    }
    j = i;
  }
  return inside;
}

// One thread per element: the point 0.1 L behind the element's first node
// must lie in a domain cell, else the element's normals are flipped.  The
// block streams the cells through shared memory and stops once every thread
// has found its cell.
__global__ void __launch_bounds__(128) orient_kernel(int ne, int nn, const double* __restrict__ px,
                                                     const double* __restrict__ py, double* nx, double* ny,
                                                     const double* __restrict__ elen, int ncell,
                                                     const double* __restrict__ cells, int* flipped) {
  using crm::ieee;
  __shared__ double s_c[kOrientChunk * 8];
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const bool active = e < ne;
  double tx = 0.0, ty = 0.0;
  bool test = false, found = false;
  if (active) {
    const int i0 = e * nn;
    const ieee d = ieee(0.1) * ieee(elen[e]);
    if (!(d.v < 1e-16)) {
      test = true;
      tx = (ieee(px[i0]) - d * ieee(nx[i0])).v;
      ty = (ieee(py[i0]) - d * ieee(ny[i0])).v;
    }
  }
  for (int c0 = 0; c0 < ncell; c0 += kOrientChunk) {
    const int cnt = min(kOrientChunk, ncell - c0);
    __syncthreads();
    for (int t = threadIdx.x; t < cnt * 8; t += blockDim.x) s_c[t] = cells[(size_t)c0 * 8 + t];
    __syncthreads();
    if (test && !found)
      for (int k = 0; k < cnt && !found; ++k) found = in_cell(tx, ty, s_c + 8 * k);
    if (!__syncthreads_or(test && !found ? 1 : 0)) break;
  }
  if (active) {
    const bool flip = test && !found;
    flipped[e] = flip ? 1 : 0;
    if (flip)
      for (int k = 0; k < nn; ++k) {
        nx[e * nn + k] = -nx[e * nn + k];
        ny[e * nn + k] = -ny[e * nn + k];
      }
  }
}

}  // namespace
}  // namespace bem

extern "C" int bem_orient2d(bem_ctx* c, int ne, int p, const double* px, const double* py, double* nx,
                            double* ny, const double* elen, int ncell, const double* cells, int mem,
                            int32_t* flipped) {
  if (!c || ne <= 0 || p < 0 || p + 1 > BEM_MAXNN || !px || !py || !nx || !ny || !elen || !flipped)
    return BEM_ERR_INVALID;
  if (ncell < 0 || (ncell > 0 && !cells)) return BEM_ERR_INVALID;
  if (mem != BEM_MEM_HOST && mem != BEM_MEM_DEVICE) return BEM_ERR_INVALID;
  CallScope cs(c);
  cudaSetDevice(c->device);
  if (ncell == 0) {  // no 2-D mesh: the reference leaves the normals as they are
    if (mem == BEM_MEM_HOST) {
      std::memset(flipped, 0, sizeof(int32_t) * (size_t)ne);
      return BEM_OK;
    }
    cudaError_t e = cudaMemsetAsync(flipped, 0, sizeof(int32_t) * (size_t)ne, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    return e == cudaSuccess ? BEM_OK : c->cuda_fail(e, "orient");
  }
  const int nn = p + 1;
  const size_t n = (size_t)ne * nn;
  const double *dpx = px, *dpy = py, *dl = elen, *dc = cells;
  double *dnx = nx, *dny = ny;
  int32_t* df = flipped;
  if (mem == BEM_MEM_HOST) {
    const size_t doubles = 4 * n + ne + (size_t)ncell * 8;
    char* o = (char*)c->get(bem_ctx::SLOT_OUT2, sizeof(double) * doubles + sizeof(int32_t) * (size_t)ne);
    if (!o) return BEM_ERR_NOMEM;
    double* d = (double*)o;
    cudaMemcpyAsync(d, px, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(d + n, py, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(d + 2 * n, nx, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(d + 3 * n, ny, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(d + 4 * n, elen, sizeof(double) * ne, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(d + 4 * n + ne, cells, sizeof(double) * ncell * 8, cudaMemcpyHostToDevice, c->stream);
    dpx = d;
    dpy = d + n;
    dnx = d + 2 * n;
    dny = d + 3 * n;
    dl = d + 4 * n;
    dc = d + 4 * n + ne;
    df = (int32_t*)(d + doubles);
  }
  orient_kernel<<<(ne + 127) / 128, 128, 0, c->stream>>>(ne, nn, dpx, dpy, dnx, dny, dl, ncell, dc, df);
  count_launches(1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "orient_kernel");
  if (mem == BEM_MEM_HOST) {
    cudaMemcpyAsync(nx, dnx, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(ny, dny, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(flipped, df, sizeof(int32_t) * ne, cudaMemcpyDeviceToHost, c->stream);
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "orient");
  return BEM_OK;
}
