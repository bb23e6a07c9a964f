// Dense pairwise matrices of the dual-interpolation BEM (DIBEM): for every
// pair of collocation points i != j with R = |x_j - x_i|,
//   F_ij = phi(R)                      radial basis function
//   D_ij = u*(x_i, x_j)                fundamental solution
// restating `_dibem_FD_kernel!` (src/Laplace/DIBEM_GPU.jl:194-208, Laplace:
// D = -log(R)/(2 pi k)) and `_elast_dibem_FD_kernel!`
// (src/Elasticity/Assembly_GPU.jl:258-280, Kelvin: D holds the 2x2 block
// U(r) of `_kelvin2d_UT`).  phi: `_dibem_phi` (DIBEM_GPU.jl:116-139), kinds
// 1-7 the polyharmonic splines R, R^2 log(R+e), R^3, R^4 log(R+e), R^5,
// R^6 log(R+e), R^7, kind 10 the fundamental solution.  Entries with
// i == j or R^2 <= eps^2 stay zero.  Outputs column-major (Julia layout).
// Each thread writes 16 bytes (2 FP64 or 4 FP32 rows) of each of its CTA's
// 32 columns, so a warp stores contiguous 512-byte segments: the FP32 kernel
// is bound by the HBM write of F and D, the FP64 one by FP64 issue.
#include <cfloat>
#include <cmath>

#include "bem_abi_internal.h"
#include "bem_device.cuh"

namespace bem {
namespace {

template <typename T>
__device__ __forceinline__ T dibem_phi(int kind, T R, T kcond, T epsa) {
  const T R2 = R * R;
  switch (kind) {
    case 1: return R;
    case 2: return R2 * log(R + epsa);
    case 3: return R2 * R;
    case 4: return (R2 * R2) * log(R + epsa);
    case 5: return R2 * R2 * R;
    case 6: return (R2 * R2 * R2) * log(R + epsa);
    case 7: return R2 * R2 * R2 * R;
    default: return -log(R) / (T(2) * T(3.14159265358979323846) * kcond);
  }
}

// columns per CTA: the CTA's row and column coordinates are converted to T
// once (on GB300 the FP64-to-FP32 conversion runs on the slow FP64 pipe)
constexpr int JPC = 32;

// Laplace: F, D (nt x nt)
template <typename T>
__global__ void __launch_bounds__(128) dibem_laplace_kernel(int nt, const double* __restrict__ px,
                                                            const double* __restrict__ py, T kcond, int kind,
                                                            T epsa, T eps2, T* F, int64_t ldf, T* D, int64_t ldd) {
  constexpr int RPT = 16 / sizeof(T);
  __shared__ T sx[JPC], sy[JPC];
  const int j0 = blockIdx.y * JPC;
  const int nj = min(JPC, nt - j0);
  if ((int)threadIdx.x < nj) {
    sx[threadIdx.x] = (T)px[j0 + threadIdx.x];
    sy[threadIdx.x] = (T)py[j0 + threadIdx.x];
  }
  const int i0 = (blockIdx.x * blockDim.x + threadIdx.x) * RPT;
  T xi[RPT], yi[RPT];
#pragma unroll
  for (int r = 0; r < RPT; ++r) {
    const int i = min(i0 + r, nt - 1);
    xi[r] = (T)px[i];
    yi[r] = (T)py[i];
  }
  __syncthreads();
  if (i0 >= nt) return;
  // -log(R) / (2 pi k) with the constant's reciprocal formed once (per-entry
  // FP64 divisions run on GB300's small FP64 pipe)
  const T dcoef = T(1) / (T(2) * T(3.14159265358979323846) * kcond);
  const bool vec = (i0 + RPT <= nt) && ((ldf | ldd) % RPT == 0) && (((uintptr_t)F | (uintptr_t)D) % 16 == 0);
  for (int jj = 0; jj < nj; ++jj) {
    const int j = j0 + jj;
    const T xj = sx[jj], yj = sy[jj];
    T f[RPT], d[RPT];
#pragma unroll
    for (int r = 0; r < RPT; ++r) {
      const int i = i0 + r;
      f[r] = T(0);
      d[r] = T(0);
      if (i < nt && i != j) {
        const T rx = xj - xi[r], ry = yj - yi[r];
        const T R2 = rx * rx + ry * ry;
        if (R2 > eps2) {
          const T R = sqrt(R2);
          d[r] = -log(R) * dcoef;
          f[r] = dibem_phi<T>(kind, R, kcond, epsa);
        }
      }
    }
    T* Fc = F + i0 + (size_t)j * ldf;
    T* Dc = D + i0 + (size_t)j * ldd;
    if (vec) {
      if constexpr (sizeof(T) == 8) {
        *(double2*)Fc = make_double2(f[0], f[1]);
        *(double2*)Dc = make_double2(d[0], d[1]);
      } else {
        *(float4*)Fc = make_float4(f[0], f[1], f[2], f[3]);
        *(float4*)Dc = make_float4(d[0], d[1], d[2], d[3]);
      }
    } else {
#pragma unroll
      for (int r = 0; r < RPT; ++r)
        if (i0 + r < nt) {
          Fc[r] = f[r];
          Dc[r] = d[r];
        }
    }
  }
}

// Kelvin: F (nt x nt), D (2nt x 2nt, node-major 2x2 blocks u11 u12; u12 u22)
template <typename T>
__global__ void __launch_bounds__(128) dibem_kelvin_kernel(int nt, const double* __restrict__ px,
                                                           const double* __restrict__ py, T mu, T nu, int kind,
                                                           T epsa, T eps2, T* F, int64_t ldf, T* D, int64_t ldd) {
  __shared__ T sx[JPC], sy[JPC];
  const int j0 = blockIdx.y * JPC;
  const int nj = min(JPC, nt - j0);
  if ((int)threadIdx.x < nj) {
    sx[threadIdx.x] = (T)px[j0 + threadIdx.x];
    sy[threadIdx.x] = (T)py[j0 + threadIdx.x];
  }
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const T xi = (T)px[min(i, nt - 1)], yi = (T)py[min(i, nt - 1)];
  __syncthreads();
  if (i >= nt) return;
  const T pi = T(3.14159265358979323846);
  const T prod1 = T(4) * pi * (T(1) - nu);
  const T inv_base = T(1) / (T(2) * prod1 * mu);
  for (int jj = 0; jj < nj; ++jj) {
    const int j = j0 + jj;
    T f = T(0), u11 = T(0), u12 = T(0), u22 = T(0);
    if (i != j) {
      const T rx = sx[jj] - xi, ry = sy[jj] - yi;
      const T R2 = rx * rx + ry * ry;
      if (R2 > eps2) {
        const T R = sqrt(R2);
        f = dibem_phi<T>(kind, R, T(1), epsa);
        // U of the 2-D Kelvin solution (`_kelvin2d_UT`, Elasticity/Fundamental.jl)
        const T invR = T(1) / R;
        const T dr1 = rx * invR, dr2 = ry * invR;
        const T prod2 = (T(3) - T(4) * nu) * (-log(R));
        u11 = (prod2 + dr1 * dr1) * inv_base;
        u12 = (dr1 * dr2) * inv_base;
        u22 = (prod2 + dr2 * dr2) * inv_base;
      }
    }
    F[i + (size_t)j * ldf] = f;
    T* c0 = D + 2 * (size_t)i + (size_t)(2 * j) * ldd;
    T* c1 = c0 + ldd;
    c0[0] = u11;
    c0[1] = u12;
    c1[0] = u12;
    c1[1] = u22;
  }
}

// radial integral of each RBF kind (`_dibem_phi_int2d`, DIBEM_GPU.jl:141-171)
template <typename T>
__device__ __forceinline__ T dibem_phi_int(int kind, T R, T kcond, T epsa) {
  const T R2 = R * R;
  switch (kind) {
    case 1: return (R2 * R) / T(3);
    case 2: { const T R4 = R2 * R2; return (T(4) * R4 * log(R + epsa) - R4) / T(16); }
    case 3: return (R2 * R2 * R) / T(5);
    case 4: { const T R6 = R2 * R2 * R2; return R6 * log(R + epsa) / T(6) - R6 / T(36); }
    case 5: return (R2 * R2 * R2 * R) / T(7);
    case 6: { const T R8 = (R2 * R2) * (R2 * R2); return R8 * log(R + epsa) / T(8) - R8 / T(64); }
    case 7: { const T R4 = R2 * R2; return (R4 * R4 * R) / T(9); }
    default: return -(T(2) * R2 * log(R) - R2) / (T(8) * T(3.14159265358979323846) * kcond);
  }
}

// Far boundary sums IF, ID of the DIBEM domain integrals (restating
// `_dibem_IFID_kernel!`, DIBEM_GPU.jl:234-270): for every collocation point
// i and boundary node j with R > 1e-10, unless the pair (i, element of j) is
// near or i lies on that element (`_near_skip_mask`, the same exact FP64 test
// as the assembly),
//   IF_i += phi_int(R) w_j (r . n_j) / R^2,  ID_i += rad(R) w_j (r . n_j) / R^2,
// rad(R) = -(2 R^2 log R - R^2) / (8 pi k) (`_dibem_rad_id2d`, :173-177),
// w_j = Jacobian_j * elem_weight_k.  Grid: x over 128-point row blocks, y
// over 32-element chunks staged in shared memory; partial sums are added
// atomically.  A conservative FP64 box test skips the exact near test for
// pairs that are far by a margin.
constexpr int IF_EC = 32;
struct IfidRule {
  double ew[BEM_MAXNN];
};

template <typename T>
__global__ void __launch_bounds__(128) dibem_ifid_kernel(GeomDev g, IfidRule rw, int rbf, T kcond, T epsa,
                                                        double nf, T* __restrict__ IF, T* __restrict__ ID) {
  __shared__ double sx[IF_EC * BEM_MAXNN], sy[IF_EC * BEM_MAXNN];
  __shared__ T snx[IF_EC * BEM_MAXNN], sny[IF_EC * BEM_MAXNN], sw[IF_EC * BEM_MAXNN];
  __shared__ double blo[IF_EC][2], bhi[IF_EC][2], blim2[IF_EC], belen[IF_EC];
  const int nn = g.nn;
  const int e0 = blockIdx.y * IF_EC;
  const int nel = min(IF_EC, g.ne - e0);
  for (int idx = threadIdx.x; idx < nel * nn; idx += blockDim.x) {
    const int j = e0 * nn + idx;
    sx[idx] = g.px[j];
    sy[idx] = g.py[j];
    snx[idx] = (T)g.nx[j];
    sny[idx] = (T)g.ny[j];
    sw[idx] = (T)(g.jac[j] * rw.ew[idx % nn]);
  }
  for (int el = threadIdx.x; el < nel; el += blockDim.x) {
    double lx = INFINITY, ly = INFINITY, hx = -INFINITY, hy = -INFINITY;
    for (int q = 0; q < nn; ++q) {
      const int j = (e0 + el) * nn + q;
      lx = fmin(lx, g.px[j]);
      ly = fmin(ly, g.py[j]);
      hx = fmax(hx, g.px[j]);
      hy = fmax(hy, g.py[j]);
    }
    blo[el][0] = lx; blo[el][1] = ly;
    bhi[el][0] = hx; bhi[el][1] = hy;
    const double L = g.elen[e0 + el];
    belen[el] = L;
    const double lim = nf * L;
    blim2[el] = nf > 1e20 ? INFINITY : lim * lim * (1.0 + 1e-12);
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.nt) return;
  const V2 pf{g.px[i], g.py[i]};
  const T pxi = (T)pf.x, pyi = (T)pf.y;
  T aF = T(0), aD = T(0);
  const T rmin = T(1e-10);
  const T radc = T(1) / (T(8) * T(3.14159265358979323846) * kcond);
  for (int el = 0; el < nel; ++el) {
    const int e = e0 + el;
    if (i >= e * nn && i < (e + 1) * nn) continue;  // source on the element
    const double dx = fmax(fmax(blo[el][0] - pf.x, pf.x - bhi[el][0]), 0.0);
    const double dy = fmax(fmax(blo[el][1] - pf.y, pf.y - bhi[el][1]), 0.0);
    if (!(dx * dx + dy * dy > blim2[el])) {
      V2 xg[BEM_MAXNN];
      for (int q = 0; q < nn; ++q) xg[q] = V2{sx[el * nn + q], sy[el * nn + q]};
      if (near_element(pf, xg, nn, belen[el], nf)) continue;
    }
    for (int q = 0; q < nn; ++q) {
      const int s = el * nn + q;
      const T rx = (T)sx[s] - pxi, ry = (T)sy[s] - pyi;
      const T R2 = rx * rx + ry * ry;
      const T R = sqrt(R2);
      if (R > rmin) {
        const T wJn = sw[s] * (rx * snx[s] + ry * sny[s]) / R2;
        aF += dibem_phi_int<T>(rbf, R, kcond, epsa) * wJn;
        aD += -(T(2) * R2 * log(R) - R2) * radc * wJn;
      }
    }
  }
  atomicAdd(IF + i, aF);
  atomicAdd(ID + i, aD);
}

// Near-pair correction of IF and ID (`_dibem_correct_near_cpu!`,
// src/Laplace/DIBEM_GPU.jl:272-300): for every element near point i (the
// assembly's exact test) or holding it, the npg-point Gauss rule on the
// element's field interpolant (`_rim_build_elements`,
// src/Core/DIBEM_common.jl:112-171: rule points y_q, normals tan2normal of
// the tangent aligned with the element's first nodal normal, w_q J_q),
//   IF_i += phi_int(R) w_q J_q (r . n_q) / R^2,  ID_i += rad(R) w_q J_q (r . n_q) / R^2
// with r = y_q - x_i, points closer than 1e-14 skipped.  FP64.  The block's
// 16 elements and their rule points are built once in shared memory; each
// thread takes one point.
constexpr int NR_EC = 16;
__global__ void __launch_bounds__(128) dibem_near_kernel(GeomDev g, Rules R, int rbf, double kcond, double epsa,
                                                         double nf, double* __restrict__ IF,
                                                         double* __restrict__ ID) {
  __shared__ double sx[NR_EC * BEM_MAXNN], sy[NR_EC * BEM_MAXNN];
  __shared__ double qy[NR_EC * BEM_MAXNPG][5];  // y.x, y.y, n.x, n.y, w J
  __shared__ double belen[NR_EC];
  const int nn = g.nn, npg = R.npg;
  const int e0 = blockIdx.y * NR_EC;
  const int nel = min(NR_EC, g.ne - e0);
  for (int idx = threadIdx.x; idx < nel * nn; idx += blockDim.x) {
    sx[idx] = g.px[e0 * nn + idx];
    sy[idx] = g.py[e0 * nn + idx];
  }
  for (int el = threadIdx.x; el < nel; el += blockDim.x) belen[el] = g.elen[e0 + el];
  __syncthreads();
  for (int t = threadIdx.x; t < nel * npg; t += blockDim.x) {
    const int el = t / npg, q = t - el * npg;
    double L[BEM_MAXNN], dL[BEM_MAXNN];
    shapefun(R.leg_x, R.leg_bw, R.leg_D, nn, R.qsi[q], L, dL);
    double px = 0, py = 0, dx = 0, dy = 0;
    for (int k = 0; k < nn; ++k) {
      px += L[k] * sx[el * nn + k];
      py += L[k] * sy[el * nn + k];
      dx += dL[k] * sx[el * nn + k];
      dy += dL[k] * sy[el * nn + k];
    }
    const double J = sqrt(dx * dx + dy * dy);
    const int j0 = (e0 + el) * nn;
    const double rx = g.nx[j0], ry = g.ny[j0];
    double ux = rx, uy = ry;
    if (!(J < 1e-16)) { ux = dy / J; uy = -dx / J; }
    if (ux * rx + uy * ry < 0) { ux = -ux; uy = -uy; }
    qy[t][0] = px;
    qy[t][1] = py;
    qy[t][2] = ux;
    qy[t][3] = uy;
    qy[t][4] = J < 1e-16 ? 0.0 : R.w[q] * J;
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.nt) return;
  const V2 pf{g.px[i], g.py[i]};
  const double radc = 1.0 / (8.0 * kPi * kcond);
  double aF = 0.0, aD = 0.0;
  for (int el = 0; el < nel; ++el) {
    const int e = e0 + el;
    const bool on = i >= e * nn && i < (e + 1) * nn;
    if (!on) {
      V2 xg[BEM_MAXNN];
      for (int k = 0; k < nn; ++k) xg[k] = V2{sx[el * nn + k], sy[el * nn + k]};
      if (!near_element(pf, xg, nn, belen[el], nf)) continue;
    }
    for (int q = 0; q < npg; ++q) {
      const double* Y = qy[el * npg + q];
      if (Y[4] == 0.0) continue;
      const double rx = Y[0] - pf.x, ry = Y[1] - pf.y;
      const double R2 = rx * rx + ry * ry;
      const double Rr = sqrt(R2);
      if (Rr < 1e-14) continue;
      const double wJn = Y[4] * ((Y[2] * rx + Y[3] * ry) / R2);
      aF += dibem_phi_int<double>(rbf, Rr, kcond, epsa) * wJn;
      aD += -(2.0 * R2 * log(Rr) - R2) * radc * wJn;
    }
  }
  if (aF != 0.0) atomicAdd(IF + i, aF);
  if (aD != 0.0) atomicAdd(ID + i, aD);
}

}  // namespace
}  // namespace bem

using namespace bem;

extern "C" int bem_dibem_ifid2d(bem_ctx* c, const bem_geom2d* geom, double k, int rbf, double epsa,
                                double near_factor, int dtype, int mem, void* IF, void* ID) {
  if (!c || !geom || !IF || !ID) return BEM_ERR_INVALID;
  if (!((rbf >= 1 && rbf <= 7) || rbf == 10)) return BEM_ERR_INVALID;
  if (dtype != BEM_F32 && dtype != BEM_F64) return BEM_ERR_INVALID;
  if (mem != BEM_MEM_HOST && mem != BEM_MEM_DEVICE) return BEM_ERR_INVALID;
  if (!(k > 0) || !(near_factor >= 0)) return BEM_ERR_INVALID;
  int rc = bem_check_geom(geom, 2, near_factor);
  if (rc) return rc;
  CallScope cs(c);
  cudaSetDevice(c->device);
  GeomDev gd;
  Rules R;
  rc = bem_stage_geom(c, geom, 2, mem, gd, R);
  if (rc) return rc;
  IfidRule rw{};
  for (int q = 0; q < BEM_MAXNN; ++q) rw.ew[q] = R.ew[q];
  const size_t esz = dtype == BEM_F32 ? 4 : 8;
  const size_t nt = (size_t)gd.nt;
  void *dF = IF, *dD = ID;
  if (mem == BEM_MEM_HOST) {
    void* o = c->get(bem_ctx::SLOT_OUT2, 2 * esz * nt);
    if (!o) return BEM_ERR_NOMEM;
    dF = o;
    dD = (char*)o + esz * nt;
  }
  cudaMemsetAsync(dF, 0, esz * nt, c->stream);
  cudaMemsetAsync(dD, 0, esz * nt, c->stream);
  dim3 grid((unsigned)((nt + 127) / 128), (unsigned)((gd.ne + IF_EC - 1) / IF_EC));
  if (dtype == BEM_F64)
    dibem_ifid_kernel<double><<<grid, 128, 0, c->stream>>>(gd, rw, rbf, k, epsa, near_factor, (double*)dF,
                                                            (double*)dD);
  else
    dibem_ifid_kernel<float><<<grid, 128, 0, c->stream>>>(gd, rw, rbf, (float)k, (float)epsa, near_factor,
                                                           (float*)dF, (float*)dD);
  count_launches(1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "dibem_ifid_kernel");
  if (mem == BEM_MEM_HOST) {
    cudaMemcpyAsync(IF, dF, esz * nt, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(ID, dD, esz * nt, cudaMemcpyDeviceToHost, c->stream);
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "dibem_ifid");
  return BEM_OK;
}

extern "C" int bem_dibem_fd2d(bem_ctx* c, int nt, const double* px, const double* py, int kind, double prm0,
                              double prm1, int rbf, double epsa, int dtype, int mem, void* F, int64_t ldf,
                              void* D, int64_t ldd) {
  if (!c || nt <= 0 || !px || !py || !F || !D) return BEM_ERR_INVALID;
  if (kind != 0 && kind != 1) return BEM_ERR_INVALID;
  if (!((rbf >= 1 && rbf <= 7) || rbf == 10)) return BEM_ERR_INVALID;
  if (dtype != BEM_F32 && dtype != BEM_F64) return BEM_ERR_INVALID;
  if (mem != BEM_MEM_HOST && mem != BEM_MEM_DEVICE) return BEM_ERR_INVALID;
  const int dof = kind == 0 ? 1 : 2;
  if (ldf < nt || ldd < (int64_t)dof * nt) return BEM_ERR_INVALID;
  if (kind == 0 && !(prm0 > 0)) return BEM_ERR_INVALID;
  if (kind == 1 && (!(prm0 > 0) || !(prm1 < 0.5) || !(prm1 > -1.0))) return BEM_ERR_INVALID;
  CallScope cs(c);
  cudaSetDevice(c->device);
  const size_t esz = dtype == BEM_F32 ? 4 : 8;
  const size_t n = (size_t)nt;
  const double *dx = px, *dy = py;
  void *dF = F, *dD = D;
  int64_t lf = ldf, lD = ldd;
  if (mem == BEM_MEM_HOST) {
    double* g = (double*)c->get(bem_ctx::SLOT_GEOM, sizeof(double) * 2 * n);
    lf = (int64_t)((n + 3) / 4 * 4);
    lD = (int64_t)((dof * n + 3) / 4 * 4);
    void* o0 = c->get(bem_ctx::SLOT_OUT0, esz * (size_t)lf * n);
    void* o1 = c->get(bem_ctx::SLOT_OUT1, esz * (size_t)lD * dof * n);
    if (!g || !o0 || !o1) return BEM_ERR_NOMEM;
    cudaMemcpyAsync(g, px, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(g + n, py, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream);
    dx = g;
    dy = g + n;
    dF = o0;
    dD = o1;
  }
  if (kind == 0) {
    const int rpt = (int)(16 / esz);
    dim3 grid((unsigned)((n + 128 * rpt - 1) / (128 * rpt)), (unsigned)((n + JPC - 1) / JPC));
    if (dtype == BEM_F64)
      dibem_laplace_kernel<double><<<grid, 128, 0, c->stream>>>(nt, dx, dy, prm0, rbf, epsa, DBL_EPSILON * DBL_EPSILON,
                                                               (double*)dF, lf, (double*)dD, lD);
    else
      dibem_laplace_kernel<float><<<grid, 128, 0, c->stream>>>(nt, dx, dy, (float)prm0, rbf, (float)epsa,
                                                              FLT_EPSILON * FLT_EPSILON, (float*)dF, lf, (float*)dD, lD);
  } else {
    dim3 grid((unsigned)((n + 127) / 128), (unsigned)((n + JPC - 1) / JPC));
    if (dtype == BEM_F64)
      dibem_kelvin_kernel<double><<<grid, 128, 0, c->stream>>>(nt, dx, dy, prm0, prm1, rbf, epsa,
                                                              DBL_EPSILON * DBL_EPSILON, (double*)dF, lf, (double*)dD, lD);
    else
      dibem_kelvin_kernel<float><<<grid, 128, 0, c->stream>>>(nt, dx, dy, (float)prm0, (float)prm1, rbf, (float)epsa,
                                                             FLT_EPSILON * FLT_EPSILON, (float*)dF, lf, (float*)dD, lD);
  }
  count_launches(1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "dibem kernel");
  if (mem == BEM_MEM_HOST) {
    cudaMemcpy2DAsync(F, esz * ldf, dF, esz * lf, esz * n, n, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpy2DAsync(D, esz * ldd, dD, esz * lD, esz * dof * n, dof * n, cudaMemcpyDeviceToHost, c->stream);
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "dibem");
  return BEM_OK;
}

extern "C" int bem_dibem_ifid_near2d(bem_ctx* c, const bem_geom2d* geom, double k, int rbf, double epsa,
                                     double near_factor, int npg, int mem, double* IF, double* ID) {
  if (!c || !geom || !IF || !ID) return BEM_ERR_INVALID;
  if (!((rbf >= 1 && rbf <= 7) || rbf == 10)) return BEM_ERR_INVALID;
  if (mem != BEM_MEM_HOST && mem != BEM_MEM_DEVICE) return BEM_ERR_INVALID;
  if (!(k > 0) || !(near_factor >= 0)) return BEM_ERR_INVALID;
  int rc = bem_check_geom(geom, npg, near_factor);
  if (rc) return rc;
  CallScope cs(c);
  cudaSetDevice(c->device);
  GeomDev gd;
  Rules R;
  rc = bem_stage_geom(c, geom, npg, mem, gd, R);
  if (rc) return rc;
  const size_t nt = (size_t)gd.nt;
  double *dF = IF, *dD = ID;
  if (mem == BEM_MEM_HOST) {
    double* o = (double*)c->get(bem_ctx::SLOT_OUT2, 2 * sizeof(double) * nt);
    if (!o) return BEM_ERR_NOMEM;
    dF = o;
    dD = o + nt;
    cudaMemcpyAsync(dF, IF, sizeof(double) * nt, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(dD, ID, sizeof(double) * nt, cudaMemcpyHostToDevice, c->stream);
  }
  dim3 grid((unsigned)((nt + 127) / 128), (unsigned)((gd.ne + NR_EC - 1) / NR_EC));
  dibem_near_kernel<<<grid, 128, 0, c->stream>>>(gd, R, rbf, k, epsa, near_factor, dF, dD);
  count_launches(1);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "dibem_near_kernel");
  if (mem == BEM_MEM_HOST) {
    cudaMemcpyAsync(IF, dF, sizeof(double) * nt, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(ID, dD, sizeof(double) * nt, cudaMemcpyDeviceToHost, c->stream);
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "dibem_ifid_near");
  return BEM_OK;
}
