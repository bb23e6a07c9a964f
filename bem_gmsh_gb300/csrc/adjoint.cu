// Adjoint gradient of a boundary-flux misfit with respect to the boundary
// node coordinates (2-D Laplace), through assembly and solve.
//
// The reference has no adjoint of its dense path; this follows the standard
// adjoint-state method on the collocation equations F = H T - G q = 0
// (H, G from `H_G_full_direct`, src/Core/Assembly_full.jl:61-175, with the
// row-sum diagonal :384-390) and the column swap of `applyBC`
// (src/Core/Boundary_conditions.jl:20-75):
//   J = 1/2 sum_{i: BC_i = 0} (q_i - q*_i)^2,   A u = b  <=>  F(u, X) = 0,
//   A^T lambda = dJ/du,   dJ/dX = -lambda^T dF/dX  (T, q held fixed).
// With the diagonal H_ii = -sum_{j != i} H_ij folded in,
//   dJ/dX = sum_{i, j != i} a_ij dH_ij/dX + sum_{i, j} c_ij dG_ij/dX,
//   a_ij = -lambda_i (T_j - T_i),   c_ij = lambda_i q_j.
// Geometry model: elements without CAD nodes, i.e. x(xi) is the Lagrange
// interpolant of the element's p+1 collocation nodes; node normals and
// Jacobians come from that interpolant, so the node coordinates are the only
// geometric parameters.  Boundary data (BC, BV) and the target are held
// fixed.  H and G are never stored: the backward kernels recompute what they
// need.
//   far pairs      analytic derivatives of the nodal lumping (a6), chained
//                  through the node normal and Jacobian to the element nodes
//   near pairs     (same exact near test as the assembly) differences of
//                  the element integral w.r.t. the source and the element's
//                  node coordinates, step 1e-5 element lengths, central
//                  unless a branch switch of the near-field map lies inside
//                  the step (then the smooth one-sided difference)
//   on-element     central differences of the on-element integral w.r.t.
//                  the element's node coordinates (the source moves with its
//                  node)
#include <cmath>
#include <cstring>

#include "bem_abi_internal.h"
#include "bem_lu.h"

int bem_solve_mixed_dev(bem_ctx* c, int N, const double* A64, int64_t lda, const double* b, double tol,
                        int max_iter, int x3, double* x, bem_solve_stats* stats);

namespace bem {
namespace {

constexpr double kTwoPi = 6.283185307179586476925286766559;

struct AdjArgs {
  GeomDev g;
  Rules R;
  double k, near_factor;
  const double *lam, *T, *q;
  double* gX;      // 2n: dJ/dx, dJ/dy per node (node-major)
  double* gn;      // 2n: dJ/dn per node
  double* gJ;      // n : dJ/dJacobian per node
  int2* pairs;     // near pairs (i, e)
  int* count;      // [0] near pair count, [1] overflow flag
  int cap;
};

// derivative contributions of one far pair (source i, node j) -- nodal
// lumping G = -log(R^2)/(4 pi k) J w, H = (r.n)/(2 pi R^2) J w, r = x_j - x_i
__device__ __forceinline__ void far_pair_grad(const AdjArgs& a, int i, int j, double w, double& gxi,
                                              double& gyi, double* node5) {
  const GeomDev& g = a.g;
  const double rx = g.px[j] - g.px[i], ry = g.py[j] - g.py[i];
  const double R2 = rx * rx + ry * ry;
  const double nxj = g.nx[j], nyj = g.ny[j], Jj = g.jac[j];
  const double c = Jj * w;
  const double G = -log(R2) / (2 * kTwoPi * a.k) * c;
  const double rn = rx * nxj + ry * nyj;
  const double H = rn / (kTwoPi * R2) * c;
  const double aH = -a.lam[i] * (a.T[j] - a.T[i]);
  const double aG = a.lam[i] * a.q[j];
  // dG/dr = -r c / (2 pi k R2);  dH/dr = c/(2 pi) (n / R2 - 2 (r.n) r / R2^2)
  const double fG = -c / (kTwoPi * a.k * R2);
  const double fH = c / kTwoPi;
  const double grx = aG * fG * rx + aH * fH * (nxj / R2 - 2 * rn * rx / (R2 * R2));
  const double gry = aG * fG * ry + aH * fH * (nyj / R2 - 2 * rn * ry / (R2 * R2));
  gxi -= grx;
  gyi -= gry;
  node5[0] += grx;
  node5[1] += gry;
  node5[2] += aH * fH * rx / R2;  // dH/dn
  node5[3] += aH * fH * ry / R2;
  node5[4] += (aH * H + aG * G) / Jj;  // d/dJ
}

// Dense pass over (row block of 32) x (element block of 32): exact near test
// per pair; far pairs get analytic derivatives, near pairs are listed for
// the finite-difference kernel, on-element pairs are left to the singular
// kernel.  Warp w takes elements w, w+8, ... of the block; lane = row.
__global__ void __launch_bounds__(256) adj_far_kernel(AdjArgs a) {
  __shared__ double s_row[8][32][2];
  const GeomDev& g = a.g;
  const int nn = g.nn;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  const bool valid = i < g.n;
  const int ic = valid ? i : g.n - 1;
  const V2 pf{g.px[ic], g.py[ic]};
  double gxi = 0.0, gyi = 0.0;
  const int e_end = min(g.ne, (int)(blockIdx.y + 1) * 32);
  for (int e = blockIdx.y * 32 + warp; e < e_end; e += 8) {
    V2 nodes[BEM_MAXNN];
    for (int kk = 0; kk < nn; ++kk) nodes[kk] = V2{g.px[e * nn + kk], g.py[e * nn + kk]};
    const bool on = ic >= e * nn && ic < (e + 1) * nn;
    const bool near = valid && !on && near_element(pf, nodes, nn, g.elen[e], a.near_factor);
    if (near) {
      const int slot = atomicAdd(a.count, 1);
      if (slot < a.cap) a.pairs[slot] = make_int2(i, e);
      else a.count[1] = 1;
    }
    const bool far = valid && !on && !near;
    for (int kk = 0; kk < nn; ++kk) {
      double node5[5] = {0, 0, 0, 0, 0};
      if (far) far_pair_grad(a, i, e * nn + kk, a.R.ew[kk], gxi, gyi, node5);
#pragma unroll
      for (int v = 0; v < 5; ++v)
        for (int o = 16; o > 0; o >>= 1) node5[v] += __shfl_xor_sync(0xffffffffu, node5[v], o);
      if (lane == 0) {
        const int j = e * nn + kk;
        atomicAdd(a.gX + 2 * j, node5[0]);
        atomicAdd(a.gX + 2 * j + 1, node5[1]);
        atomicAdd(a.gn + 2 * j, node5[2]);
        atomicAdd(a.gn + 2 * j + 1, node5[3]);
        atomicAdd(a.gJ + j, node5[4]);
      }
    }
  }
  s_row[warp][lane][0] = gxi;
  s_row[warp][lane][1] = gyi;
  __syncthreads();
  if (warp == 0 && valid) {
    double sx = 0.0, sy = 0.0;
    for (int w = 0; w < 8; ++w) {
      sx += s_row[w][lane][0];
      sy += s_row[w][lane][1];
    }
    atomicAdd(a.gX + 2 * i, sx);
    atomicAdd(a.gX + 2 * i + 1, sy);
  }
}

// Derivative from S(-h), S(0), S(+h).  The near-field maps switch branch at
// thresholds of the pole position (the reference's tanp3c rules), so the
// discrete integral can jump by its quadrature error inside a step: when the
// one-sided slopes disagree beyond smooth curvature, the jump lies on the
// steeper side and the other side's slope is the derivative.
__device__ __forceinline__ double fd_slope(double sm, double s0, double sp, double h) {
  const double f = (sp - s0) / h, b = (s0 - sm) / h;
  const double d = fabs(f - b);
  if (d <= 1e-3 * fmax(fabs(f), fabs(b)) || d * h <= 1e-13 * fabs(s0)) return 0.5 * (f + b);
  return fabs(f) < fabs(b) ? f : b;
}

// S = sum_k a_k h_k + c_k g_k over the element's nodes for source pf
__device__ double near_value(const AdjArgs& a, int i, int e, const V2* nodes, V2 pf) {
  const GeomDev& g = a.g;
  const int nn = g.nn;
  V2 geo[BEM_MAXGEO];
  double h[BEM_MAXNN], gg[BEM_MAXNN];
  Physics ph{};
  ph.kind = 0;
  ph.k = a.k;
  const V2 nref{g.nx[e * nn], g.ny[e * nn]};
  integrate_near<1>(a.R, ph, nodes, geo, pf, g.elen[e], nref, h, gg);
  double s = 0.0;
  for (int kk = 0; kk < nn; ++kk) {
    const int j = e * nn + kk;
    s += -a.lam[i] * (a.T[j] - a.T[i]) * h[kk] + a.lam[i] * a.q[j] * gg[kk];
  }
  return s;
}

// one thread per near pair: central differences w.r.t. the source point and
// the element's node coordinates
__global__ void __launch_bounds__(64) adj_near_kernel(AdjArgs a) {
  const int cnt = min(a.count[0], a.cap);
  const GeomDev& g = a.g;
  const int nn = g.nn;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < cnt; t += gridDim.x * blockDim.x) {
    const int2 pr = a.pairs[t];
    const int i = pr.x, e = pr.y;
    V2 nodes[BEM_MAXNN];
    for (int kk = 0; kk < nn; ++kk) nodes[kk] = V2{g.px[e * nn + kk], g.py[e * nn + kk]};
    V2 pf{g.px[i], g.py[i]};
    const double h = 1e-5 * g.elen[e];
    const double s0 = near_value(a, i, e, nodes, pf);
    for (int d = 0; d < 2; ++d) {
      double* c = d == 0 ? &pf.x : &pf.y;
      const double c0 = *c;
      *c = c0 + h;
      const double sp = near_value(a, i, e, nodes, pf);
      *c = c0 - h;
      const double sm = near_value(a, i, e, nodes, pf);
      *c = c0;
      atomicAdd(a.gX + 2 * i + d, fd_slope(sm, s0, sp, h));
    }
    for (int kk = 0; kk < nn; ++kk) {
      for (int d = 0; d < 2; ++d) {
        double* c = d == 0 ? &nodes[kk].x : &nodes[kk].y;
        const double c0 = *c;
        *c = c0 + h;
        const double sp = near_value(a, i, e, nodes, pf);
        *c = c0 - h;
        const double sm = near_value(a, i, e, nodes, pf);
        *c = c0;
        atomicAdd(a.gX + 2 * (e * nn + kk) + d, fd_slope(sm, s0, sp, h));
      }
    }
  }
}

__device__ double singular_value(const AdjArgs& a, int i, int e, const V2* nodes) {
  const GeomDev& g = a.g;
  const int nn = g.nn, ai = i - e * nn;
  V2 geo[BEM_MAXGEO];
  double h[BEM_MAXNN], gg[BEM_MAXNN];
  Physics ph{};
  ph.kind = 0;
  ph.k = a.k;
  const V2 nref{g.nx[e * nn], g.ny[e * nn]};
  integrate_singular<1>(a.R, ph, nodes, geo, nodes[ai], a.R.leg_x[ai], nref, h, gg);
  double s = 0.0;
  for (int kk = 0; kk < nn; ++kk) {
    const int j = e * nn + kk;
    if (kk != ai) s += -a.lam[i] * (a.T[j] - a.T[i]) * h[kk];
    s += a.lam[i] * a.q[j] * gg[kk];
  }
  return s;
}

// one thread per boundary node: its own element, node coordinates perturbed
// (the source is one of them)
__global__ void __launch_bounds__(64) adj_singular_kernel(AdjArgs a) {
  const GeomDev& g = a.g;
  const int nn = g.nn;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const int e = i / nn;
  V2 nodes[BEM_MAXNN];
  for (int kk = 0; kk < nn; ++kk) nodes[kk] = V2{g.px[e * nn + kk], g.py[e * nn + kk]};
  const double h = 1e-5 * g.elen[e];
  const double s0 = singular_value(a, i, e, nodes);
  for (int kk = 0; kk < nn; ++kk) {
    for (int d = 0; d < 2; ++d) {
      double* c = d == 0 ? &nodes[kk].x : &nodes[kk].y;
      const double c0 = *c;
      *c = c0 + h;
      const double sp = singular_value(a, i, e, nodes);
      *c = c0 - h;
      const double sm = singular_value(a, i, e, nodes);
      *c = c0;
      atomicAdd(a.gX + 2 * (e * nn + kk) + d, fd_slope(sm, s0, sp, h));
    }
  }
}

// node normal n = (t_y, -t_x) and Jacobian J = |x'| at node j from
// x'(xi_j) = sum_m D_jm X_m: chain dJ/dn, dJ/dJac to the element's nodes
__global__ void adj_chain_kernel(AdjArgs a) {
  const GeomDev& g = a.g;
  const int nn = g.nn;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= g.ne) return;
  for (int jj = 0; jj < nn; ++jj) {
    const int j = e * nn + jj;
    double da = 0.0, db = 0.0;
    for (int m = 0; m < nn; ++m) {
      da += a.R.leg_D[jj * nn + m] * g.px[e * nn + m];
      db += a.R.leg_D[jj * nn + m] * g.py[e * nn + m];
    }
    const double J = sqrt(da * da + db * db), J3 = J * J * J;
    const double gnx = a.gn[2 * j], gny = a.gn[2 * j + 1], gj = a.gJ[j];
    // n_x = b/J, n_y = -a/J
    const double ga = gj * da / J + gnx * (-da * db / J3) + gny * (-db * db / J3);
    const double gb = gj * db / J + gnx * (da * da / J3) + gny * (da * db / J3);
    for (int m = 0; m < nn; ++m) {
      a.gX[2 * (e * nn + m)] += a.R.leg_D[jj * nn + m] * ga;
      a.gX[2 * (e * nn + m) + 1] += a.R.leg_D[jj * nn + m] * gb;
    }
  }
}

// T, q from the solution u (split_sol, src/Core/Solver.jl:88-98), the
// misfit J and its gradient w.r.t. u
__global__ void adj_split_kernel(int n, const int32_t* BC, const double* BV, const double* u, const double* qt,
                                 double* T, double* q, double* dJdu, double* Jout) {
  __shared__ double s[256];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const bool dir = BC[i] == 0;
    T[i] = dir ? BV[i] : u[i];
    q[i] = dir ? u[i] : BV[i];
    const double r = dir ? u[i] - qt[i] : 0.0;
    dJdu[i] = r;
    acc += 0.5 * r * r;
  }
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *Jout = s[0];
}

__global__ void transpose64(const double* A, int64_t lda, int N, double* At, int64_t ldt) {
  __shared__ double tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int i = bx + threadIdx.x, j = by + r;
    if (i < N && j < N) tile[r][threadIdx.x] = A[i + (size_t)j * lda];
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int i = by + threadIdx.x, j = bx + r;
    if (i < N && j < N) At[i + (size_t)j * ldt] = tile[threadIdx.x][r];
  }
}

}  // namespace
}  // namespace bem

using namespace bem;

extern "C" int bem_adjoint_laplace2d(bem_ctx* c, const bem_geom2d* g, double k, const int32_t* BC,
                                     const double* BV, const double* q_target, int npg, double near_factor,
                                     double tol, int max_iter, int mem, double* J, double* grad,
                                     bem_solve_stats* stats) {
  if (!c || !g || !BC || !BV || !q_target || !J || !grad) return BEM_ERR_INVALID;
  if (mem != BEM_MEM_HOST && mem != BEM_MEM_DEVICE) return BEM_ERR_INVALID;
  if (!(k > 0) || !(tol > 0) || max_iter < 1) return BEM_ERR_INVALID;
  int rc = bem_check_geom(g, npg, near_factor);
  if (rc) return rc;
  if (g->ngeo != 0 || g->nt != g->n) {
    c->last_error = "adjoint: elements must take their geometry from the nodes (ngeo = 0), no internal points";
    return BEM_ERR_UNSUPPORTED;
  }
  CallScope cs(c);
  cudaSetDevice(c->device);
  const int n = g->n, N = n;
  const int64_t ld = (N + 3) / 4 * 4;
  Physics ph{};
  ph.kind = 0;
  ph.k = k;
  // forward: fused assembly and mixed-precision solve
  double* A = (double*)c->get(bem_ctx::SLOT_OUT0, sizeof(double) * (size_t)ld * N);
  double* At = (double*)c->get(bem_ctx::SLOT_ADJ0, sizeof(double) * (size_t)ld * N);
  // b, u, T, q, dJdu, lambda (n each) | gX, gn (2n each), gJ | J | target, BV, BC (staged inputs)
  double* v = (double*)c->get(bem_ctx::SLOT_ADJ1, sizeof(double) * (size_t)(15 * N + 64));
  if (!A || !At || !v) return BEM_ERR_NOMEM;
  double *b = v, *u = v + N, *T = v + 2 * N, *q = v + 3 * N, *dJdu = v + 4 * N, *lam = v + 5 * N;
  double *gX = v + 7 * N, *gn = v + 9 * N, *gJ = v + 11 * N, *Jd = v + 12 * N;
  double* stg = v + 12 * (size_t)N + 8;
  double* qt = stg;
  const int32_t* dBC = BC;
  const double* dBV = BV;
  if (mem == BEM_MEM_HOST) {
    // target, BV, BC up in one copy through the pinned buffer
    const size_t words = 2 * (size_t)N + ((size_t)N + 1) / 2;
    double* h = (double*)c->pinned(words * sizeof(double));
    if (!h) return BEM_ERR_NOMEM;
    std::memcpy(h, q_target, sizeof(double) * (size_t)N);
    std::memcpy(h + N, BV, sizeof(double) * (size_t)N);
    std::memcpy(h + 2 * (size_t)N, BC, sizeof(int32_t) * (size_t)N);
    cudaMemcpyAsync(stg, h, words * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    c->pin_issued();
    dBV = stg + N;
    dBC = (const int32_t*)(stg + 2 * (size_t)N);
  } else {
    cudaMemcpyAsync(qt, q_target, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream);
  }
  const int prec = (c->opt_far_df >= 1) ? 3 : 1;
  rc = bem_assemble_system_dev(c, g, ph, BC, BV, npg, near_factor, mem, prec, A, ld, nullptr, b);
  if (rc) return rc;
  bem_solve_stats st{};
  rc = bem_solve_mixed_dev(c, N, A, ld, b, tol, max_iter, 1, u, &st);
  if (rc != BEM_OK && rc != BEM_ERR_NOT_CONVERGED) return rc;
  adj_split_kernel<<<1, 256, 0, c->stream>>>(n, dBC, dBV, u, qt, T, q, dJdu, Jd);
  // adjoint system A^T lambda = dJ/du
  transpose64<<<dim3((N + 31) / 32, (N + 31) / 32), dim3(32, 8), 0, c->stream>>>(A, ld, N, At, ld);
  count_launches(2);
  bem_solve_stats st2{};
  int rc2 = bem_solve_mixed_dev(c, N, At, ld, dJdu, tol, max_iter, 1, lam, &st2);
  if (rc2 != BEM_OK && rc2 != BEM_ERR_NOT_CONVERGED) return rc2;
  // backward: recompute, never store, the influence entries
  GeomDev gd;
  Rules R;
  rc = bem_stage_geom(c, g, npg, mem, gd, R);
  if (rc) return rc;
  const int cap = 32 * n + 1024;
  int2* pairs = (int2*)c->get(bem_ctx::SLOT_PAIRS, sizeof(int2) * (size_t)cap);
  int* cnt = (int*)c->get(bem_ctx::SLOT_COUNTERS, 64);
  if (!pairs || !cnt) return BEM_ERR_NOMEM;
  cudaMemsetAsync(cnt, 0, 2 * sizeof(int), c->stream);
  cudaMemsetAsync(gX, 0, sizeof(double) * 5 * (size_t)N, c->stream);
  AdjArgs aa{};
  aa.g = gd;
  aa.R = R;
  aa.k = k;
  aa.near_factor = near_factor;
  aa.lam = lam;
  aa.T = T;
  aa.q = q;
  aa.gX = gX;
  aa.gn = gn;
  aa.gJ = gJ;
  aa.pairs = pairs;
  aa.count = cnt;
  aa.cap = cap;
  adj_far_kernel<<<dim3((n + 31) / 32, (g->ne + 31) / 32), 256, 0, c->stream>>>(aa);
  adj_near_kernel<<<(cap + 63) / 64 < 4096 ? (cap + 63) / 64 : 4096, 64, 0, c->stream>>>(aa);
  adj_singular_kernel<<<(n + 63) / 64, 64, 0, c->stream>>>(aa);
  adj_chain_kernel<<<(g->ne + 127) / 128, 128, 0, c->stream>>>(aa);
  count_launches(4);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return c->cuda_fail(e, "adjoint kernels");
  // gradient, J and the pair counters back through the pinned buffer
  double* hout = (double*)c->pinned(sizeof(double) * (2 * (size_t)N + 2));
  if (!hout) return BEM_ERR_NOMEM;
  const int* hc = (const int*)(hout + 2 * (size_t)N + 1);
  cudaMemcpyAsync(hout + 2 * (size_t)N + 1, cnt, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  if (mem == BEM_MEM_HOST) {
    cudaMemcpyAsync(hout, gX, sizeof(double) * 2 * (size_t)N, cudaMemcpyDeviceToHost, c->stream);
    cudaMemcpyAsync(hout + 2 * (size_t)N, Jd, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  } else {
    cudaMemcpyAsync(grad, gX, sizeof(double) * 2 * (size_t)N, cudaMemcpyDeviceToDevice, c->stream);
    cudaMemcpyAsync(J, Jd, sizeof(double), cudaMemcpyDeviceToDevice, c->stream);
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "adjoint");
  if (mem == BEM_MEM_HOST) {
    std::memcpy(grad, hout, sizeof(double) * 2 * (size_t)N);
    *J = hout[2 * (size_t)N];
  }
  if (hc[1] != 0) {
    c->last_error = "adjoint: near-pair list overflow";
    return BEM_ERR_INTERNAL;
  }
  if (stats) {
    *stats = st;
    stats->iterations += st2.iterations;
  }
  return (rc == BEM_ERR_NOT_CONVERGED || rc2 == BEM_ERR_NOT_CONVERGED) ? BEM_ERR_NOT_CONVERGED : BEM_OK;
}
