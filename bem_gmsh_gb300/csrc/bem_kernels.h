// Internal interface between the CUDA kernels and the C-ABI layer.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "bem_device.cuh"

namespace bem {

// 32-byte node record for the FP32 far-field tiles (bulk-copied to smem).
struct __align__(16) NodeRec {
  float xh, xl, yh, yl;  // coordinates as FP32 hi + lo
  float nx, ny;          // outward normal
  float cG, cH;          // folded kernel constants times J w
};

// 64-byte node record of the double-float far field (Laplace): coordinates
// as exact three-float splits, normal, kernel constants and boundary value
// as hi + lo pairs (G = log(R2) cG, H = (r.n) / R2 cH).
struct __align__(16) NodeDF {
  float xa, xb, xc, ya, yb, yc;
  float nxh, nxl, nyh, nyl;
  float cGh, cGl, cHh, cHl;
  float bvh, bvl;
};

// 80-byte node record of the double-float far field (Kelvin): coordinates
// as exact three-float splits; normal, the folded kernel constants and the
// two boundary values as hi + lo pairs.  With q = r r^T / R2 and the node's
// J w folded in:  U = cUl log(R2) I + cU q,
//   T_aa = cT (r.n) / R2 (c + 2 q_aa),
//   T_ab = cT / R2 (2 (r.n) q_ab - c (r_a n_b - r_b n_a)),
// c = 1 - 2 nu (a kernel argument), the 2x2 Kelvin blocks of kelvin_UT.
struct __align__(16) NodeDFK {
  float xa, xb, xc, ya, yb, yc;
  float nxh, nxl, nyh, nyl;
  float cUh, cUl, cLh, cLl, cTh, cTl;
  float bv0h, bv0l, bv1h, bv1l;
};

// 32-byte element record: conservative bounding box + squared near limit.
struct __align__(16) ElemRec {
  float lox, loy, hix, hiy;
  float lim2, pad0, pad1, pad2;
};

struct FarArgs {
  int nt, n, ne, nn;
  int64_t ld, ldg;
  int vec_ok, pair_cap;
  Physics ph;
  const float4* rows;
  const NodeRec* nodes;
  const NodeDF* nodes_df;   // double-float variant only (Kelvin: NodeDFK records)
  float c1h, c1l;           // double-float Kelvin: c = 1 - 2 nu as hi + lo
  const float4* logtab;     // double-float log table (129 entries)
  const ElemRec* elems;
  const double *px, *py, *nx, *ny, *jac;
  double ew[BEM_MAXNN];
  void* H;      // H (or A when fused)
  void* G;      // G (unused when fused)
  float* A32;   // FP32 copy of A (mixed precision)
  const int32_t* bc;
  const double* bv;
  double* b;
  double* rowsum;   // [row * dof + column dof]
  int* pair_count;
  int2* pairs;
  int* status;
};

struct NearArgs {
  GeomDev g;
  Rules R;
  Physics ph;
  double near_factor;
  int64_t ld, ldg;
  int pair_cap;
  const int* pair_count;
  const int2* pairs;
  void* H;
  void* G;
  float* A32;
  const int32_t* bc;
  const double* bv;
  double* b;
  double* rowsum;
  double* gdiag;  // on-element G diagonal blocks (fused mode)
  int mode;       // 0 FP32 H,G; 1 FP64 H,G; 2 FP64 A,b; 3 FP64 + FP32 A,b
};

struct FinalArgs {
  int nt, n;
  int64_t ld;
  void* H;
  float* A32;
  const int32_t* bc;
  const double* bv;
  double* b;
  const double* rowsum;
  const double* gdiag;
  int mode;
};

// near pairs (listed by the far kernel), on-element rows, row-sum diagonal
void launch_near_pairs(const NearArgs& na, int nc, cudaStream_t st);
void launch_singular(const NearArgs& na, int nc, int n, cudaStream_t st);
void launch_finalize(const FinalArgs& fi, int nc, int nt, cudaStream_t st);

// One assembly request; all pointers are device pointers.
struct AsmRequest {
  GeomDev g;
  Rules R;
  Physics ph;
  double near_factor;
  int prec;    // 0 FP32, 1 FP64, 2 FP64 + FP32 copy of A, 3 FP64 output with the
               // far field in double-float (fused)
  int fused;   // 1: write A, b (applyBC fused), else H, G
  void* H;
  int64_t ld;
  void* G;
  int64_t ldg;
  float* A32;
  const int32_t* bc;
  const double* bv;
  double* b;
  // workspace
  float4* rows;
  NodeRec* nodes;
  NodeDF* nodes_df;
  float4* logtab;
  ElemRec* elems;
  double* rowsum;
  double* gdiag;
  int* counters;  // [0] pair count, [1] status
  int2* pairs;
  int pair_cap;
  unsigned long long* absmax;  // scratch: largest |coordinate|
  // optional side stream for the on-element kernel (runs beside the far and
  // near kernels; joined before the diagonal), with its fork/join events
  cudaStream_t aux = nullptr, aux2 = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_join2 = nullptr;
};

// Launch the whole assembly on `stream` (asynchronous).  Returns 0 or a
// CUDA error code.
int launch_assembly(const AsmRequest& q, cudaStream_t stream);

}  // namespace bem
