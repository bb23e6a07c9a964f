// Near-singular, on-element and diagonal kernels of the dense 2-D BEM
// assembly (FP64).  See assemble_far.cu for the overall structure.
#include "bem_device.cuh"
#include "bem_kernels.h"

namespace bem {

// ---------------------------------------------------------------------------
// near kernel: listed pairs, exact FP64 test, tanp3c or FP64 lumping
// ---------------------------------------------------------------------------
// store modes: 0 FP32 (H, G); 1 FP64 (H, G); 2 FP64 (A, b); 3 FP64 + FP32 (A, b)
__device__ __forceinline__ void store_hg(const NearArgs& a, size_t row, size_t col, double hv,
                                         double gv) {
  if (a.mode == 0) {
    ((float*)a.H)[row + col * a.ld] = (float)hv;
    ((float*)a.G)[row + col * a.ldg] = (float)gv;
  } else {
    ((double*)a.H)[row + col * a.ld] = hv;
    ((double*)a.G)[row + col * a.ldg] = gv;
  }
}

__device__ __forceinline__ void store_a(const NearArgs& a, size_t row, size_t col, double av) {
  ((double*)a.H)[row + col * a.ld] = av;
  if (a.mode == 3) a.A32[row + col * a.ld] = (float)av;
}

template <int NC>
__global__ void __launch_bounds__(128) near_kernel(NearArgs a) {
  constexpr int DOF = (NC == 1) ? 1 : 2;
  const bool FUSED = a.mode >= 2;
  const int count = min(*a.pair_count, a.pair_cap);
  const GeomDev& g = a.g;
  const int nn = g.nn;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) {
    int2 pr = a.pairs[t];
    const int i = pr.x, e = pr.y;
    if (i >= e * nn && i < (e + 1) * nn) continue;  // on-element: singular_kernel
    V2 nodes[BEM_MAXNN], geo[BEM_MAXGEO];
    load_element(g, e, nodes, geo);
    V2 pf{g.px[i], g.py[i]};
    double h[BEM_MAXNN * NC], gg[BEM_MAXNN * NC];
    if (near_element(pf, nodes, nn, g.elen[e], a.near_factor)) {
      V2 nref{g.nx[e * nn], g.ny[e * nn]};
      integrate_near<NC>(a.R, a.ph, nodes, geo, pf, g.elen[e], nref, h, gg);
    } else {
      for (int k = 0; k < nn; ++k) {
        int j = e * nn + k;
        double U[4], T[4];
        far_eval_f64<NC>(a.ph, g.px[j] - pf.x, g.py[j] - pf.y, g.nx[j], g.ny[j],
                         g.jac[j] * a.R.ew[k], U, T);
        for (int c = 0; c < NC; ++c) { h[k * NC + c] = T[c]; gg[k * NC + c] = U[c]; }
      }
    }
    for (int ar = 0; ar < DOF; ++ar) {
      const size_t row = (size_t)DOF * i + ar;
      double rs[DOF], bs = 0.0;
      for (int b = 0; b < DOF; ++b) rs[b] = 0.0;
      for (int k = 0; k < nn; ++k) {
        int j = e * nn + k;
        for (int b = 0; b < DOF; ++b) {
          const size_t col = (size_t)DOF * j + b;
          double hv = h[k * NC + ar * DOF + b], gv = gg[k * NC + ar * DOF + b];
          rs[b] += hv;
          if (!FUSED) {
            store_hg(a, row, col, hv, gv);
          } else {
            int bc = a.bc[col];
            double av = (bc == 0) ? -gv : hv;
            bs += (bc == 0) ? -hv * a.bv[col] : gv * a.bv[col];
            store_a(a, row, col, av);
          }
        }
      }
      for (int b = 0; b < DOF; ++b) atomicAdd(a.rowsum + row * DOF + b, rs[b]);
      if (FUSED) atomicAdd(a.b + row, bs);
    }
  }
}

// ---------------------------------------------------------------------------
// singular kernel: collocation node i on its own element
// ---------------------------------------------------------------------------
template <int NC>
__global__ void __launch_bounds__(64) singular_kernel(NearArgs a) {
  constexpr int DOF = (NC == 1) ? 1 : 2;
  const bool FUSED = a.mode >= 2;
  const GeomDev& g = a.g;
  const int nn = g.nn;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const int e = i / nn;
  V2 nodes[BEM_MAXNN], geo[BEM_MAXGEO];
  load_element(g, e, nodes, geo);
  V2 pf{g.px[i], g.py[i]};
  double xa, dist;
  closest_point_1d(a.R, nodes, nn, pf, xa, dist);
  V2 nref{g.nx[e * nn], g.ny[e * nn]};
  double h[BEM_MAXNN * NC], gg[BEM_MAXNN * NC];
  if (a.R.singular == 1)
    integrate_singular_telles<NC>(a.R, a.ph, nodes, geo, pf, xa, nref, h, gg);
  else
    integrate_singular<NC>(a.R, a.ph, nodes, geo, pf, xa, nref, h, gg);
  for (int ar = 0; ar < DOF; ++ar) {
    const size_t row = (size_t)DOF * i + ar;
    double rs[DOF], bs = 0.0;
    for (int b = 0; b < DOF; ++b) rs[b] = 0.0;
    for (int k = 0; k < nn; ++k) {
      int j = e * nn + k;
      for (int b = 0; b < DOF; ++b) {
        const size_t col = (size_t)DOF * j + b;
        double hv = h[k * NC + ar * DOF + b], gv = gg[k * NC + ar * DOF + b];
        const bool diag_blk = (j == i);
        if (!FUSED) {
          if (!diag_blk) {
            rs[b] += hv;
            store_hg(a, row, col, hv, gv);
          } else {
            if (a.mode == 0) ((float*)a.G)[row + col * a.ldg] = (float)gv;
            else ((double*)a.G)[row + col * a.ldg] = gv;
          }
        } else {
          int bc = a.bc[col];
          if (!diag_blk) {
            rs[b] += hv;
            double av = (bc == 0) ? -gv : hv;
            bs += (bc == 0) ? -hv * a.bv[col] : gv * a.bv[col];
            store_a(a, row, col, av);
          } else {
            // the diagonal block's H comes from the row sum (finalize); its
            // G part is final here.
            a.gdiag[(size_t)DOF * DOF * i + ar * DOF + b] = gv;
            if (bc != 0) bs += gv * a.bv[col];
          }
        }
      }
    }
    for (int b = 0; b < DOF; ++b) atomicAdd(a.rowsum + row * DOF + b, rs[b]);
    if (FUSED) atomicAdd(a.b + row, bs);
  }
}

// ---------------------------------------------------------------------------
// finalize: diagonal (block) from the row sums
// ---------------------------------------------------------------------------
__device__ __forceinline__ void store_diag(const FinalArgs& a, size_t row, size_t col, double v) {
  if (a.mode == 0) ((float*)a.H)[row + col * a.ld] = (float)v;
  else ((double*)a.H)[row + col * a.ld] = v;
  if (a.mode == 3) a.A32[row + col * a.ld] = (float)v;
}

template <int NC>
__global__ void finalize_kernel(FinalArgs a) {
  constexpr int DOF = (NC == 1) ? 1 : 2;
  const bool FUSED = a.mode >= 2;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nt) return;
  if constexpr (DOF == 1) {
    double hii = -a.rowsum[i];
    if (!FUSED) {
      store_diag(a, i, i, hii);
    } else {
      double av = hii;
      if (i < a.n && a.bc[i] == 0) {
        av = -a.gdiag[i];
        a.b[i] += -hii * a.bv[i];
      }
      store_diag(a, i, i, av);
    }
  } else {
    // rigid-body row-sum (_vectorial_free_term!): block (2i+a, 2i+b) =
    // -sum of row 2i+a over columns of dof b, other blocks excluded.  The
    // row sums were accumulated per row over all columns; split by column
    // dof with the per-dof accumulators.
    for (int ar = 0; ar < 2; ++ar)
      for (int b = 0; b < 2; ++b) {
        size_t row = 2 * (size_t)i + ar, col = 2 * (size_t)i + b;
        double hv = -a.rowsum[(2 * (size_t)i + ar) * 2 + b];
        if (!FUSED) {
          store_diag(a, row, col, hv);
        } else {
          double av = hv;
          if ((size_t)i < (size_t)a.n && a.bc[col] == 0) {
            av = -a.gdiag[4 * (size_t)i + ar * 2 + b];
            a.b[row] += -hv * a.bv[col];
          }
          store_diag(a, row, col, av);
        }
      }
  }
}




void launch_near_pairs(const NearArgs& na, int nc, cudaStream_t st) {
  int nblk = (na.pair_cap + 127) / 128;
  if (nblk > 152 * 16) nblk = 152 * 16;
  if (nblk < 1) nblk = 1;
  if (nc == 1) near_kernel<1><<<nblk, 128, 0, st>>>(na);
  else near_kernel<4><<<nblk, 128, 0, st>>>(na);
}

void launch_singular(const NearArgs& na, int nc, int n, cudaStream_t st) {
  if (n <= 0) return;
  if (nc == 1) singular_kernel<1><<<(n + 63) / 64, 64, 0, st>>>(na);
  else singular_kernel<4><<<(n + 63) / 64, 64, 0, st>>>(na);
}

void launch_finalize(const FinalArgs& fi, int nc, int nt, cudaStream_t st) {
  if (nc == 1) finalize_kernel<1><<<(nt + 255) / 256, 256, 0, st>>>(fi);
  else finalize_kernel<4><<<(nt + 255) / 256, 256, 0, st>>>(fi);
}

}  // namespace bem
