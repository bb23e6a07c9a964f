// Dense solve kernels: column equilibration, blocked LU without pivoting
// (FP32 storage, TF32 tensor-core updates), triangular solves with the
// factors, and the FP64 vector kernels of the refinement loop.
//
// The reference solves A x = b with LinearSolve.jl's dense LU
// (src/Core/LinearSolveUtils.jl:44-49, LAPACK getrf/getrs with partial
// pivoting).  Here A is first equilibrated by columns; BEM collocation
// systems equilibrated this way factor stably without row exchanges
// (growth factors of order 1-10 on the Laplace and Kelvin test systems), so
// the factorization needs no pivot search across the panel, which is the
// latency bottleneck of partial pivoting on a GPU.  The FP32 factors only
// precondition an FP64 GMRES whose residual uses the FP64 matrix, so the
// final solution has FP64 accuracy.
#include <cstdint>
#include <mutex>
#include <cuda_runtime.h>

#include "bem_lu.h"
#include "bem_prof.h"
#include "bem_tc.cuh"
#include "df32.cuh"

namespace bem {

// ---------------------------------------------------------------------------
// equilibration + FP32 copy with identity padding
// ---------------------------------------------------------------------------
// One CTA per column of the padded matrix: the column's max |a| (first
// pass, from HBM), the power-of-two column scale cs[j] = 2^s with
// max |a| 2^s in [0.5, 1), then the scaled FP32 column (second pass, the
// column's 8 N bytes are still in L2).  Padding columns and rows get the
// identity.  HBM traffic: the FP64 matrix once, the FP32 copy once.
// Everything runs on the integer pipes (GB300's FP64 pipe is a small
// fraction of its FP32 rate): the max compares |a| as bit patterns (for
// non-negative IEEE doubles the order of the patterns is the order of the
// values), and the scaled conversion adds s to the exponent field and rounds
// the 52-bit fraction to 23 bits to nearest, ties to even -- exactly
// (float)(a * 2^s).  Values whose result leaves the normal FP32 range (not
// met by a scaled column other than for zeros) take the FP64 instructions
// (df::scale_to_f32).
__global__ void __launch_bounds__(512) k_equilibrate(const double* __restrict__ A, int64_t lda, int N, int Npad,
                                                     double* __restrict__ cs, float* __restrict__ A32,
                                                     int64_t ld32) {
  const int j = blockIdx.x, t = threadIdx.x;
  float* out = A32 + (size_t)j * ld32;
  if (j >= N) {
    for (int i = t; i < Npad; i += blockDim.x) out[i] = (i == j) ? 1.f : 0.f;
    return;
  }
  const unsigned long long* col = (const unsigned long long*)(A + (size_t)j * lda);
  constexpr unsigned long long ABS = 0x7FFFFFFFFFFFFFFFull;
  // 16 independent loads in flight per thread and round
  constexpr int V = 16;
  unsigned long long mx = 0;
  for (int base = 0; base < N; base += V * 512) {
    unsigned long long v[V];
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const int i = base + q * 512 + t;
      v[q] = i < N ? col[i] : 0ull;
    }
#pragma unroll
    for (int q = 0; q < V; ++q) mx = max(mx, v[q] & ABS);
  }
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  __shared__ unsigned long long sw[16];
  __shared__ int ssh;
  if ((t & 31) == 0) sw[t >> 5] = mx;
  __syncthreads();
  if (t == 0) {
    unsigned long long r = 0;
    for (int w = 0; w < 16; ++w) r = max(r, sw[w]);
    const int ex = (int)(r >> 52);
    // zero, subnormal-only, inf or NaN columns keep scale 1
    int sh = (ex == 0 || ex == 0x7FF) ? 0 : 1022 - ex;
    if (sh < -1022) sh = -1022;
    ssh = sh;
    cs[j] = __longlong_as_double((long long)((unsigned long long)(1023 + sh) << 52));
  }
  __syncthreads();
  const int sh = ssh;
  for (int base = 0; base < Npad; base += V * 512) {
    unsigned long long v[V];
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const int i = base + q * 512 + t;
      v[q] = i < N ? col[i] : 0ull;
    }
#pragma unroll
    for (int q = 0; q < V; ++q) {
      const int i = base + q * 512 + t;
      if (i < Npad) out[i] = df::scale_to_f32(__longlong_as_double((long long)v[q]), sh);
    }
  }
}

// ---------------------------------------------------------------------------
// diagonal block: unblocked LU of a 128 x 128 block in shared memory, then
// the inverses of its unit-lower and upper triangles.
// ---------------------------------------------------------------------------
constexpr int DLD = LU_NB + 1;

// Gauss-Jordan factorization of one diagonal block, register blocked: the
// forward elimination applied to [A | I] leaves U in A and L^{-1} in the
// identity part; the backward sweep on [U | I] builds U^{-1}.  It is the
// independent check of the tiled kernel below (bem_selftest).  Warp w
// (0..15) owns rows w, w+16, ..., w+112 and lane l owns columns l, l+32,
// l+64, l+96, so every thread holds an 8 x 4 tile of [A | I] in registers.
// Step j publishes row j (one warp) and column j (one lane per warp) to
// shared memory, double-buffered by step parity, then one barrier; the
// row loads are conflict-free and the column loads are broadcasts.
// Forward elimination leaves L\U in `a` and L^{-1} in `b`; the backward sweep
// then turns a fresh identity in `b` into U^{-1}.
__global__ void __launch_bounds__(512) k_diag_factor_rb(float* __restrict__ A, int64_t ld, int k,
                                                        float* __restrict__ Dinv, int* __restrict__ info) {
  extern __shared__ float stage[];  // LU_NB * DLD
  __shared__ float prow[2][LU_NB], pcol[2][LU_NB], pb[2][LU_NB];
  __shared__ int bad;
  const int t = threadIdx.x;
  const int lane = t & 31, w = t >> 5;
  const size_t off = (size_t)k * LU_NB;
  float* Ab = A + off + off * ld;
  if (t == 0) bad = 0;
  for (int idx = t; idx < LU_NB * LU_NB; idx += blockDim.x) {
    int r = idx & (LU_NB - 1), c = idx >> 7;
    stage[c * DLD + r] = Ab[r + (size_t)c * ld];
  }
  __syncthreads();
  float a[8][4], b[8][4];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int r = w + 16 * i, c = lane + 32 * q;
      a[i][q] = stage[c * DLD + r];
      b[i][q] = (r == c) ? 1.f : 0.f;
    }
  // forward elimination on [A | I]
  for (int j = 0; j < LU_NB; ++j) {
    const int p = j & 1;
    if (w == (j & 15)) {
      const int ij = j >> 4;
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (i == ij) {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            prow[p][lane + 32 * q] = a[i][q];
            pb[p][lane + 32 * q] = b[i][q];
          }
        }
    }
    if (lane == (j & 31)) {
      const int qj = j >> 5;
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q == qj) {
#pragma unroll
          for (int i = 0; i < 8; ++i) pcol[p][w + 16 * i] = a[i][q];
        }
    }
    __syncthreads();
    const float piv = pcol[p][j];
    if (t == 0 && !(fabsf(piv) > 1e-30f && fabsf(piv) < INFINITY)) bad = 1;
    const float inv = 1.f / piv;
    // branch-free update: multipliers of inactive rows are 0, the row-j
    // values feed the U part for columns > j and the L^{-1} part otherwise
    float fa[4], fb[4], l[8];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const bool right = (lane + 32 * q) > j;
      const float rv = prow[p][lane + 32 * q], bv = pb[p][lane + 32 * q];
      fa[q] = right ? rv : 0.f;
      fb[q] = right ? 0.f : bv;
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) l[i] = (w + 16 * i > j) ? pcol[p][w + 16 * i] * inv : 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[i][q] -= l[i] * fa[q];
        b[i][q] -= l[i] * fb[q];
      }
    if (lane == (j & 31)) {  // store the multipliers as column j of L
      const int qj = j >> 5;
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q == qj) {
#pragma unroll
          for (int i = 0; i < 8; ++i)
            if (w + 16 * i > j) a[i][q] = l[i];
        }
    }
  }
  __syncthreads();
  float* Li = Dinv + (size_t)k * 2 * LU_NB * LU_NB;
  float* Ui = Li + LU_NB * LU_NB;
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) stage[(lane + 32 * q) * DLD + w + 16 * i] = a[i][q];
  __syncthreads();
  for (int idx = t; idx < LU_NB * LU_NB; idx += blockDim.x) {
    int r = idx & (LU_NB - 1), c = idx >> 7;
    Ab[r + (size_t)c * ld] = stage[c * DLD + r];
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int r = w + 16 * i, c = lane + 32 * q;
      stage[c * DLD + r] = b[i][q];
      b[i][q] = (r == c) ? 1.f : 0.f;
    }
  __syncthreads();
  for (int idx = t; idx < LU_NB * LU_NB; idx += blockDim.x) {
    int r = idx & (LU_NB - 1), c = idx >> 7;
    Li[r + c * LU_NB] = stage[c * DLD + r];
  }
  // backward sweep: U X = I from the bottom row up.  Step j publishes the
  // accumulated row j of X (before scaling) and column j of U.
  for (int j = LU_NB - 1; j >= 0; --j) {
    const int p = j & 1;
    if (w == (j & 15)) {
      const int ij = j >> 4;
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (i == ij) {
#pragma unroll
          for (int q = 0; q < 4; ++q) pb[p][lane + 32 * q] = b[i][q];
        }
    }
    if (lane == (j & 31)) {
      const int qj = j >> 5;
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q == qj) {
#pragma unroll
          for (int i = 0; i < 8; ++i) pcol[p][w + 16 * i] = a[i][q];
        }
    }
    __syncthreads();
    const float inv = 1.f / pcol[p][j];
    float xv[4], u[8];
#pragma unroll
    for (int q = 0; q < 4; ++q) xv[q] = (lane + 32 * q >= j) ? pb[p][lane + 32 * q] * inv : 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) u[i] = (w + 16 * i < j) ? pcol[p][w + 16 * i] : 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int q = 0; q < 4; ++q) b[i][q] -= u[i] * xv[q];
    if (w == (j & 15)) {  // finished row j of U^{-1}
      const int ij = j >> 4;
#pragma unroll
      for (int i = 0; i < 8; ++i)
        if (i == ij) {
#pragma unroll
          for (int q = 0; q < 4; ++q)
            if (lane + 32 * q >= j) b[i][q] = xv[q];
        }
    }
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int q = 0; q < 4; ++q) stage[(lane + 32 * q) * DLD + w + 16 * i] = b[i][q];
  __syncthreads();
  for (int idx = t; idx < LU_NB * LU_NB; idx += blockDim.x) {
    int r = idx & (LU_NB - 1), c = idx >> 7;
    Ui[r + c * LU_NB] = stage[c * DLD + r];
  }
  if (t == 0 && bad) atomicExch(info, k + 1);
}

// ---------------------------------------------------------------------------
// 128 x 128 x 128 tile GEMM on the legacy tensor-core path (mma.sync TF32),
// optionally with the 3xTF32 split (hi*hi + hi*lo + lo*hi) for FP32
// accuracy.  C = beta * C + alpha * A * B, column-major.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mma_tf32(float* c, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

constexpr int GK = 32;          // k chunk
constexpr int ALD = 128 + 4;    // As[k][m]
constexpr int BLD = GK + 4;     // Bs[n][k]

template <bool X3>
__global__ void __launch_bounds__(256) k_gemm_mma(const float* A, int64_t lda,
                                                  const float* B, int64_t ldb,
                                                  float* C, int64_t ldc, float alpha, float beta) {
  extern __shared__ __align__(16) float gsm[];
  float* As = gsm;                       // 2 stages of [GK][ALD]
  float* Bs = gsm + 2 * GK * ALD;        // 2 stages of [128][BLD]
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int wm = warp >> 2, wn = warp & 3;  // 2 x 4 warps, warp tile 64 x 32
  const int g = lane >> 2, tg = lane & 3;
  const size_t m0 = (size_t)blockIdx.x * 128, n0 = (size_t)blockIdx.y * 128;
  const float* Ab = A + m0;
  const float* Bb = B + n0 * ldb;

  auto load = [&](int stage, int kc) {
    float* as = As + stage * GK * ALD;
    float* bs = Bs + stage * 128 * BLD;
    for (int s = t; s < GK * 32; s += 256) {  // A: 32 k-columns x 32 segments of 4 m
      int kk = s >> 5, seg = s & 31;
      cp_async16(as + kk * ALD + seg * 4, Ab + (size_t)(kc + kk) * lda + seg * 4);
    }
    for (int s = t; s < 128 * 8; s += 256) {  // B: 128 n-columns x 8 segments of 4 k
      int nn = s >> 3, seg = s & 7;
      cp_async16(bs + nn * BLD + seg * 4, Bb + (size_t)nn * ldb + kc + seg * 4);
    }
    cp_async_commit();
  };

  float acc[4][4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;

  load(0, 0);
  constexpr int NCH = LU_NB / GK;
  for (int ch = 0; ch < NCH; ++ch) {
    if (ch + 1 < NCH) {
      load((ch + 1) & 1, (ch + 1) * GK);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const float* as = As + (ch & 1) * GK * ALD;
    const float* bs = Bs + (ch & 1) * 128 * BLD;
#pragma unroll
    for (int k8 = 0; k8 < GK; k8 += 8) {
      uint32_t ah[4][4], al[4][4], bh[4][2], bl[4][2];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int mr = wm * 64 + i * 16 + g;
        float v[4] = {as[(k8 + tg) * ALD + mr], as[(k8 + tg) * ALD + mr + 8],
                      as[(k8 + tg + 4) * ALD + mr], as[(k8 + tg + 4) * ALD + mr + 8]};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          ah[i][q] = tf32_rna(v[q]);
          if (X3) al[i][q] = tf32_rna(v[q] - __uint_as_float(ah[i][q]));
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int nc = wn * 32 + j * 8 + g;
        float v[2] = {bs[nc * BLD + k8 + tg], bs[nc * BLD + k8 + tg + 4]};
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          bh[j][q] = tf32_rna(v[q]);
          if (X3) bl[j][q] = tf32_rna(v[q] - __uint_as_float(bh[j][q]));
        }
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (X3) {
            mma_tf32(acc[i][j], al[i], bh[j]);
            mma_tf32(acc[i][j], ah[i], bl[j]);
          }
          mma_tf32(acc[i][j], ah[i], bh[j]);
        }
    }
    __syncthreads();
  }
  // epilogue
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const size_t r0 = m0 + wm * 64 + i * 16 + g;
      const size_t c0 = n0 + wn * 32 + j * 8 + 2 * tg;
      float* p00 = C + r0 + c0 * ldc;
      float* p01 = C + r0 + (c0 + 1) * ldc;
      float* p10 = p00 + 8;
      float* p11 = p01 + 8;
      if (beta == 0.f) {
        *p00 = alpha * acc[i][j][0];
        *p01 = alpha * acc[i][j][1];
        *p10 = alpha * acc[i][j][2];
        *p11 = alpha * acc[i][j][3];
      } else {
        *p00 = beta * *p00 + alpha * acc[i][j][0];
        *p01 = beta * *p01 + alpha * acc[i][j][1];
        *p10 = beta * *p10 + alpha * acc[i][j][2];
        *p11 = beta * *p11 + alpha * acc[i][j][3];
      }
    }
}

size_t gemm_mma_smem() { return sizeof(float) * (2 * GK * ALD + 2 * 128 * BLD); }

// C (M x N, multiples of 128) = beta C + alpha A (M x 128) B (128 x N)
void gemm_tile128(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc,
                  int M, int N, float alpha, float beta, int x3, cudaStream_t st) {
  if (M <= 0 || N <= 0) return;
  count_launches(1);
  dim3 grid(M / 128, N / 128);
  const size_t sm = gemm_mma_smem();
  if (x3)
    k_gemm_mma<true><<<grid, 256, sm, st>>>(A, lda, B, ldb, C, ldc, alpha, beta);
  else
    k_gemm_mma<false><<<grid, 256, sm, st>>>(A, lda, B, ldb, C, ldc, alpha, beta);
}

// ---------------------------------------------------------------------------
// triangular solves with the blocked factors (FP32), one block row per step
// ---------------------------------------------------------------------------
// y[kb] = Dk * r[kb], Dk = 128 x 128 inverse block; r, y FP32 (may alias)
__global__ void k_blk_apply(const float* __restrict__ D, const float* r, float* y) {
  __shared__ float rs[LU_NB];
  const int t = threadIdx.x;
  rs[t] = r[t];
  __syncthreads();
  float acc = 0.f;
#pragma unroll 8
  for (int q = 0; q < LU_NB; ++q) acc += D[t + q * LU_NB] * rs[q];
  y[t] = acc;
}

// r[rows] -= P[rows, 0:128] * y, P column-major with ld
__global__ void k_panel_gemv(const float* __restrict__ P, int64_t ld, int rows,
                             const float* __restrict__ y, float* r) {
  __shared__ float ys[LU_NB];
  if (threadIdx.x < LU_NB) ys[threadIdx.x] = y[threadIdx.x];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += gridDim.x * blockDim.x) {
    float acc = 0.f;
#pragma unroll 8
    for (int q = 0; q < LU_NB; ++q) acc += P[i + (size_t)q * ld] * ys[q];
    r[i] -= acc;
  }
}

// r[0:rows] -= P[0:rows, :] * y for an upper-triangular sweep (P = column block)
// same kernel as k_panel_gemv; kept separate for clarity of the launch sites.

// ---------------------------------------------------------------------------
// Wavefront triangular solve: P CTAs per block row, one launch per sweep.
// Block row q of the forward sweep computes y_b (b = q) = Linv_b (r_b -
// sum_{j<b} L_bj y_j); the backward sweep runs b = K-1-q downwards with U and
// Uinv_b.  The non-adjacent sum is split over the block row's P CTAs: P-1
// helpers sum the earlier blocks and publish their partial sums, the owner
// sums the latest ones, adds the partials and runs the dependent step.
// A CTA waits only for blocks solved before its own (flags set with release
// semantics after their block is written); the waits are bounded and a
// timeout is reported through `err` instead of hanging.  The launch is
// cooperative so that all CTAs are resident.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* p, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// M^L_b = Linv_b L_{b,b-1} (b >= 1) and M^U_b = Uinv_b U_{b,b+1} (b <= K-2),
// column-major in Mc[(2 b + side) 128^2]: the coupling of block b of a
// triangular sweep to the block solved just before it.  With
//   z_b = D_b (r_b - sum over the other solved blocks),  y_b = z_b - M_b y_prev
// the sweep's dependent step is one 128 x 128 product; z_b is formed while
// the previous block is still being solved.  One CTA per (block, side,
// 64 x 64 quadrant), 4 x 4 outputs per thread.
constexpr int CPL_LD = 64 + 4;
constexpr int CPL_SMEM = (int)sizeof(float) * 2 * LU_NB * CPL_LD;

__global__ void __launch_bounds__(256) k_lu_couplings(const float* __restrict__ A, int64_t ld, int K,
                                                      const float* __restrict__ Dinv, float* __restrict__ Mc) {
  extern __shared__ __align__(16) float cs_[];
  const int b = blockIdx.x, side = blockIdx.y, quad = blockIdx.z, t = threadIdx.x;
  if (side == 0 ? b == 0 : b == K - 1) return;
  const int qr = (quad & 1) * 64, qc = (quad >> 1) * 64;
  float* P = cs_;                   // D_b rows [qr, qr + 64): P[k][r]
  float* Q = cs_ + LU_NB * CPL_LD;  // coupling block columns [qc, qc + 64): Q[k][c]
  const float* Pg = Dinv + (size_t)b * 2 * LU_NB * LU_NB + (side ? LU_NB * LU_NB : 0);
  const int qb = side ? b + 1 : b - 1;
  const float* Qg = A + (size_t)b * LU_NB + (size_t)qb * LU_NB * ld;
  for (int idx = t; idx < LU_NB * 64; idx += 256) {
    const int r = idx & 63, k = idx >> 6;
    P[k * CPL_LD + r] = Pg[qr + r + (size_t)k * LU_NB];  // D_b(qr + r, k), column-major
    const int k2 = idx & (LU_NB - 1), c = idx >> 7;
    Q[k2 * CPL_LD + c] = Qg[k2 + (size_t)(qc + c) * ld];  // block(k2, qc + c), coalesced reads
  }
  __syncthreads();
  const int r0 = 4 * (t & 15), c0 = 4 * (t >> 4);
  float acc[4][4] = {};
#pragma unroll 4
  for (int k = 0; k < LU_NB; ++k) {
    const float4 a = *(const float4*)&P[k * CPL_LD + r0];
    const float4 q = *(const float4*)&Q[k * CPL_LD + c0];
    const float av[4] = {a.x, a.y, a.z, a.w}, qv[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], qv[j], acc[i][j]);
  }
  float* Mo = Mc + (size_t)(2 * b + side) * LU_NB * LU_NB;
#pragma unroll
  for (int j = 0; j < 4; ++j)
    *(float4*)&Mo[(size_t)(qc + c0 + j) * LU_NB + qr + r0] = make_float4(acc[0][j], acc[1][j], acc[2][j], acc[3][j]);
}

// Words per CTA of the partial sums (ptags): 128 (epoch, value) words, P at
// most TRSV_PMAX CTAs per block row.
template <bool UPPER>
__global__ void __launch_bounds__(256) k_trsv_wave(const float* __restrict__ A, int64_t ld, int K,
                                                   const float* __restrict__ Dinv, const float* __restrict__ Mc,
                                                   const float* r, float* y, unsigned long long* tags,
                                                   unsigned long long* ptags, int P, int epoch, int wepoch,
                                                   int wait_limit, int* err) {
  extern __shared__ float Ds[];  // the block's inverse, [col][row], LU_NB * (LU_NB + 1)
  __shared__ float ys[LU_NB];
  __shared__ float part[2][LU_NB];
  __shared__ int bad;
  const int t = threadIdx.x, row = t & (LU_NB - 1), half = t >> 7;
  const int bi = (int)blockIdx.x / P, pp = (int)blockIdx.x % P;
  const bool owner = pp == P - 1;
  const int b = UPPER ? (K - 1 - bi) : bi;
  const size_t rb = (size_t)b * LU_NB;
  const int nj = UPPER ? (K - 1 - b) : b;  // blocks solved before this one
  const int noff = nj > 1 ? nj - 1 : 0;    // ... but the adjacent one
  // this CTA's share of the non-adjacent blocks, in solve order
  const int s0 = (int)((long long)noff * pp / P), s1 = (int)((long long)noff * (pp + 1) / P);
  if (t == 0) bad = 0;
  float mreg[LU_NB / 2];
  if (owner) {
    const float* Db = Dinv + (size_t)b * 2 * LU_NB * LU_NB + (UPPER ? LU_NB * LU_NB : 0);
    for (int idx = t; idx < LU_NB * LU_NB; idx += blockDim.x) {
      int rr = idx & (LU_NB - 1), c = idx >> 7;
      Ds[c * (LU_NB + 1) + rr] = Db[rr + (size_t)c * LU_NB];
    }
    // this thread's half row of the coupling to the adjacent block
    if (nj > 0) {
      const float* Mb = Mc + (size_t)(2 * b + (UPPER ? 1 : 0)) * LU_NB * LU_NB;
#pragma unroll
      for (int q = 0; q < LU_NB / 2; ++q) mreg[q] = Mb[(size_t)(half * (LU_NB / 2) + q) * LU_NB + row];
    }
  }
  float acc = (owner && half == 0) ? r[rb + row] : 0.f;
  __syncthreads();
  // waits for the 128 (epoch, value) words at w: each of the first 128
  // threads polls its own word; false when the wait ran out
  auto fetch = [&](const unsigned long long* w0) {
    if (t < LU_NB) {
      const unsigned long long* w = w0 + t;
      unsigned long long v = ld_acquire_u64(w);
      int it = 0;
      while ((int)(v >> 32) != epoch) {
        if (++it > wait_limit) {
          bad = 1;
          break;
        }
        if (it > 8) __nanosleep(32);
        v = ld_acquire_u64(w);
      }
      ys[t] = __uint_as_float((uint32_t)v);
    }
    __syncthreads();
    return bad == 0;
  };
  // the same, starting from a word loaded earlier (no round trip when its
  // block was already published then)
  auto fetch_pre = [&](const unsigned long long* w0, unsigned long long v) {
    if (t < LU_NB) {
      if ((int)(v >> 32) != epoch) {
        const unsigned long long* w = w0 + t;
        v = ld_acquire_u64(w);
        int it = 0;
        while ((int)(v >> 32) != epoch) {
          if (++it > wait_limit) {
            bad = 1;
            break;
          }
          if (it > 8) __nanosleep(32);
          v = ld_acquire_u64(w);
        }
      }
      ys[t] = __uint_as_float((uint32_t)v);
    }
    __syncthreads();
    return bad == 0;
  };
  auto blk = [&](int s) { return UPPER ? (K - 1 - s) : s; };
  // this thread's 64 coefficients of block (b, j): row `row`, columns
  // half * 64 .. + 63 (coalesced across the warp)
  auto coef = [&](int s) { return A + (rb + row) + ((size_t)blk(s) * LU_NB + half * (LU_NB / 2)) * ld; };
  // the helpers' partial sums, loaded by the owner together with its last
  // non-adjacent block (the helpers' shares end earlier, so these words are
  // usually published by then and the owner's dependent step loses the
  // round trip it spent polling them one after another)
  unsigned long long pwv[LU_TRSV_PMAX - 1];
#pragma unroll
  for (int q = 0; q < LU_TRSV_PMAX - 1; ++q) pwv[q] = 0;
  auto pre_parts = [&]() {
    if (owner && t < LU_NB) {
#pragma unroll
      for (int q = 0; q < LU_TRSV_PMAX - 1; ++q)
        if (q + 1 < P) pwv[q] = ld_relaxed_u64(ptags + (size_t)(b * P + q) * LU_NB + t);
    }
  };
  // non-adjacent blocks, two register buffers: block s+1's coefficients
  // and its (epoch, value) words load while block s waits for its y and is
  // applied, so that a block published by then costs no round trip
  {
    float pa[LU_NB / 2], pb[LU_NB / 2];
    unsigned long long ta = 0, tb = 0;
    auto word = [&](int s) {
      if (s == s1 - 1) pre_parts();
      return t < LU_NB ? ld_relaxed_u64(tags + (size_t)blk(s) * LU_NB + t) : 0ull;
    };
    if (s0 == s1) pre_parts();
    int s = s0;
    if (s < s1) {
      const float* P0 = coef(s);
#pragma unroll
      for (int q = 0; q < LU_NB / 2; ++q) pa[q] = P0[(size_t)q * ld];
      ta = word(s);
    }
    while (s < s1) {
      if (s + 1 < s1) {
        const float* P1 = coef(s + 1);
#pragma unroll
        for (int q = 0; q < LU_NB / 2; ++q) pb[q] = P1[(size_t)q * ld];
        tb = word(s + 1);
      }
      if (!fetch_pre(tags + (size_t)blk(s) * LU_NB, ta)) {
        if (t == 0) atomicExch(err, 1);
        return;
      }
#pragma unroll
      for (int q = 0; q < LU_NB / 2; ++q) acc -= pa[q] * ys[half * (LU_NB / 2) + q];
      __syncthreads();
      if (++s >= s1) break;
      if (s + 1 < s1) {
        const float* P1 = coef(s + 1);
#pragma unroll
        for (int q = 0; q < LU_NB / 2; ++q) pa[q] = P1[(size_t)q * ld];
        ta = word(s + 1);
      }
      if (!fetch_pre(tags + (size_t)blk(s) * LU_NB, tb)) {
        if (t == 0) atomicExch(err, 1);
        return;
      }
#pragma unroll
      for (int q = 0; q < LU_NB / 2; ++q) acc -= pb[q] * ys[half * (LU_NB / 2) + q];
      __syncthreads();
      ++s;
    }
  }
  part[half][row] = acc;
  __syncthreads();
  unsigned long long* pw = ptags + (size_t)(b * P + pp) * LU_NB;
  if (!owner) {
    // a helper publishes its partial sum (0 for an empty share)
    if (t < LU_NB)
      st_relaxed_u64(pw + t, ((unsigned long long)(unsigned)wepoch << 32) | __float_as_uint(part[0][t] + part[1][t]));
    return;
  }
  float sum = (t < LU_NB) ? part[0][t] + part[1][t] : 0.f;
#pragma unroll
  for (int q = 0; q < LU_TRSV_PMAX - 1; ++q) {
    if (q + 1 >= P) break;
    if (!fetch_pre(ptags + (size_t)(b * P + q) * LU_NB, pwv[q])) {
      if (t == 0) atomicExch(err, 1);
      return;
    }
    if (t < LU_NB) sum += ys[t];
    __syncthreads();
  }
  // z_b = D_b (r_b - ...)
  if (t < LU_NB) ys[t] = sum;
  __syncthreads();
  float o0 = 0.f, o1 = 0.f;
#pragma unroll 16
  for (int q = half * (LU_NB / 2); q < (half + 1) * (LU_NB / 2); q += 2) {
    o0 += Ds[q * (LU_NB + 1) + row] * ys[q];
    o1 += Ds[(q + 1) * (LU_NB + 1) + row] * ys[q + 1];
  }
  part[half][row] = o0 + o1;
  __syncthreads();
  float yb = (t < LU_NB) ? part[0][t] + part[1][t] : 0.f;
  if (nj > 0) {
    // y_b = z_b - M_b y_adjacent
    __syncthreads();  // part and ys are reused
    if (!fetch(tags + (size_t)(UPPER ? b + 1 : b - 1) * LU_NB)) {
      if (t == 0) atomicExch(err, 1);
      return;
    }
    float m0 = 0.f, m1 = 0.f;
#pragma unroll
    for (int q = 0; q < LU_NB / 2; q += 2) {
      m0 = fmaf(mreg[q], ys[half * (LU_NB / 2) + q], m0);
      m1 = fmaf(mreg[q + 1], ys[half * (LU_NB / 2) + q + 1], m1);
    }
    part[half][row] = m0 + m1;
    __syncthreads();
    if (t < LU_NB) yb -= part[0][t] + part[1][t];
  }
  if (t < LU_NB) {
    y[rb + t] = yb;
    st_relaxed_u64(tags + rb + t, ((unsigned long long)(unsigned)wepoch << 32) | __float_as_uint(yb));
  }
}

// ---------------------------------------------------------------------------
// FP64 vector kernels of the refinement loop
// ---------------------------------------------------------------------------
// y = b - A x (FP64), one warp per 4 rows... simple row-parallel version:
// each thread owns rows; A column-major so threads read consecutive rows.
__global__ void k_residual64(const double* __restrict__ A, int64_t lda, int N,
                             const double* __restrict__ x, const double* __restrict__ b,
                             double* __restrict__ r, int col_chunk) {
  // 2-D split: blockIdx.y picks a column chunk, partial sums added atomically
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c0 = blockIdx.y * col_chunk;
  const int c1 = min(N, c0 + col_chunk);
  if (i >= N) return;
  double acc = 0.0;
  for (int c = c0; c < c1; ++c) acc = fma(A[i + (size_t)c * lda], x[c], acc);
  if (blockIdx.y == 0) acc = b[i] - acc;
  else acc = -acc;
  atomicAdd(r + i, acc);
}

__global__ void k_gemv64(const double* __restrict__ A, int64_t lda, int N,
                         const double* __restrict__ x, double* __restrict__ y, int col_chunk) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c0 = blockIdx.y * col_chunk;
  const int c1 = min(N, c0 + col_chunk);
  if (i >= N) return;
  double acc = 0.0;
  for (int c = c0; c < c1; ++c) acc = fma(A[i + (size_t)c * lda], x[c], acc);
  atomicAdd(y + i, acc);
}

// h[j] = sum_i V[i, j] w[i] for j < m  (V column-major, ld = N)
// h[j] += V[:, j] . w over this CTA's slice of the rows (h zeroed before):
// blockIdx.x = j, blockIdx.y = slice, so each vector is spread over
// gridDim.y SMs (one SM's FP64 rate is a small fraction of the GPU's)
__global__ void k_dots(const double* __restrict__ V, int64_t ldv, int N, int m,
                       const double* __restrict__ w, double* __restrict__ h) {
  const int j = blockIdx.x;
  if (j >= m) return;
  double acc = 0.0;
  for (int i = blockIdx.y * blockDim.x + threadIdx.x; i < N; i += gridDim.y * blockDim.x)
    acc = fma(V[i + (size_t)j * ldv], w[i], acc);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double s[32];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) r += s[q];
    atomicAdd(h + j, r);
  }
}

// w -= V[:, 0:m] h ; out[i] = w (FP64)
__global__ void k_sub_vh(const double* __restrict__ V, int64_t ldv, int N, int m,
                         const double* __restrict__ h, double* __restrict__ w) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    double acc = w[i];
    for (int j = 0; j < m; ++j) acc = fma(-V[i + (size_t)j * ldv], h[j], acc);
    w[i] = acc;
  }
}

// x += Z[:, 0:m] y
__global__ void k_add_zy(const double* __restrict__ Z, int64_t ldz, int N, int m,
                         const double* __restrict__ y, double* __restrict__ x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    double acc = x[i];
    for (int j = 0; j < m; ++j) acc = fma(Z[i + (size_t)j * ldz], y[j], acc);
    x[i] = acc;
  }
}

// v = w / sqrt(*n2) (zeros when *n2 is not positive): normalization by a
// norm that stays on the device
__global__ void k_scale_by_norm(const double* __restrict__ w, const double* __restrict__ n2,
                                double* __restrict__ v, int N) {
  const double q = *n2;
  const double s = q > 0.0 ? 1.0 / sqrt(q) : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) v[i] = w[i] * s;
}

__global__ void k_scale_copy(const double* __restrict__ w, double s, double* __restrict__ v, int N) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) v[i] = w[i] * s;
}

// FP64 -> FP32 padded vector
__global__ void k_to_f32(const double* __restrict__ v, int N, int Npad, float* __restrict__ o) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Npad; i += gridDim.x * blockDim.x)
    o[i] = i < N ? (float)v[i] : 0.f;
}

// z = cs .* y (FP32 -> FP64)
__global__ void k_from_f32_scale(const float* __restrict__ y, const double* __restrict__ cs, int N,
                                 double* __restrict__ z) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    z[i] = (double)y[i] * cs[i];
}

// ---------------------------------------------------------------------------
// host-side sequences
// ---------------------------------------------------------------------------
void lu_prepare(const double* A64, int64_t lda, int N, int Npad, double* cs, float* A32, int64_t ld32,
                cudaStream_t st) {
  KScope ks(st, KC_LU_PREP);
  count_launches(1);
  k_equilibrate<<<Npad, 512, 0, st>>>(A64, lda, N, Npad, cs, A32, ld32);
}

// ---------------------------------------------------------------------------
// Factorization of a 128 x 128 diagonal block (no pivoting) in shared memory
// (column-major, ld 132 so that 4 consecutive rows are one 16-byte load),
// with the inverses of its eight 16 x 16 diagonal sub-blocks of L and U, the
// inputs of the blocked triangular panel solves (k_panels).  For each
// 16-wide panel p (jb = 16 p):
//   A  warps 0-3 factor the panel: every warp holds its own copy of the 16
//      pivot rows (lane r < 16: row jb + r) and updates them identically, and
//      32 rows below them (lane: row jb + 16 + 32 w + lane), so no barrier
//      is needed between columns; the pivot rows reach the lanes two at a
//      time through a double-buffered pair of rows in shared memory (every
//      lane forms row c+1 after column c itself).  Warp 1 then
//      inverts the unit-lower 16 x 16 block (one column per lane).
//   B  block row of U: U[p, >p] = Linv_pp A[p, >p].  Column block p of L\U
//      and its lower sub-block inverse are final and are written out; warp 4
//      inverts the upper 16 x 16 block beside the next panel's factorization
//      (its columns of S no longer change).
//   C  the trailing update A22 -= L21 U12 on 4 x 4 register tiles.
// 24 block barriers in all.  In the look-ahead LU the block first gets the
// previous step's update of itself (the thin update leaves the block out):
// A_kk -= L_{k,k-1} U_{k-1,k} with that step's tensor-core operands, TMA
// loads and tcgen05 MMAs into TMEM (3xTF32) while the block loads, then one
// TMEM read per thread (the same update on mma.sync took 12 of the kernel's
// 45 us; as a separate one-tile launch it cost a launch on the chain).  73 KB
// of shared memory (201 KB with the update's four operand stages) and the
// whole register file (512 threads x 128): the kernel runs alone on an SM
// (capped at 64 registers to share an SM with a bulk-update tile it measured
// 40 % slower).  A and ld must allow 16-byte accesses (ld % 4 == 0, 16-byte
// aligned A).
// ---------------------------------------------------------------------------
constexpr int DB = LU_SB;       // panel width
constexpr int TLD = LU_NB + 4;  // shared leading dimension
// shared floats of the diagonal kernel: L\U, four warps' double-buffered
// pairs of pivot rows, the 16 x 16 scratch of the lower inverse, the two
// sub-block inverses
constexpr int DIAG_SMEM = (int)sizeof(float) * (LU_NB * TLD + 4 * 4 * DB + 16 * 20 + 4 * DB * DB);
// with the block's own update: two operand stages of the tensor-core update
// (1024-byte aligned), their barriers and the TMEM address
constexpr int DIAG_PRE_STAGES = 4;
constexpr int DIAG_B_BYTES = LU_NB * tc::BK * 4;  // a 128-column B chunk
constexpr int DIAG_STAGE_BYTES = 2 * tc::A_BYTES + 2 * DIAG_B_BYTES;
constexpr int DIAG_SMEM_PRE = DIAG_SMEM + 1024 + DIAG_PRE_STAGES * DIAG_STAGE_BYTES + 128;

// step k-1's update of diagonal block k inside k_diag_lu, A_kk -= L_{k,k-1}
// U_{k-1,k}, from that step's tensor-core operands (the maps of its TcPlan):
// Lt / Ltlo rows 0..127, U_{k-1,k} from the matrix at (k index, n index) =
// (bx0, by0), Ulo columns 0..127 (B maps with 128-column boxes).
struct DiagPre {
  int on;
  int bx0, by0;
};

// acc[i][j] += sum_{q in [qs, qe)} P(r0 + i, q) Q(q, c0 + j) for column-major
// shared blocks P (P(r, q) = Pb[q * TLD + r]) and Q (Q(q, c) = Qb[c * TLD + q]);
// qs, qe multiples of 4.
template <int CT>
__device__ __forceinline__ void tile_mm(const float* Pb, const float* Qb, int r0, int c0, int qs, int qe,
                                        float (&acc)[4][CT]) {
  for (int q = qs; q < qe; q += 4) {
    float4 p[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) p[i] = *(const float4*)&Pb[(q + i) * TLD + r0];
#pragma unroll
    for (int j = 0; j < CT; ++j) {
      const float4 qv = *(const float4*)&Qb[(c0 + j) * TLD + q];
      const float qq[4] = {qv.x, qv.y, qv.z, qv.w};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        acc[0][j] = fmaf(p[i].x, qq[i], acc[0][j]);
        acc[1][j] = fmaf(p[i].y, qq[i], acc[1][j]);
        acc[2][j] = fmaf(p[i].z, qq[i], acc[2][j]);
        acc[3][j] = fmaf(p[i].w, qq[i], acc[3][j]);
      }
    }
  }
}

template <int CT>
__device__ __forceinline__ void tile_store(float* Ob, int r0, int c0, const float (&acc)[4][CT]) {
#pragma unroll
  for (int j = 0; j < CT; ++j)
    *(float4*)&Ob[(c0 + j) * TLD + r0] = make_float4(acc[0][j], acc[1][j], acc[2][j], acc[3][j]);
}

// reciprocal: hardware approximation plus one Newton step (about 1 ulp)
__device__ __forceinline__ float rcp_nr(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return fmaf(r, fmaf(-x, r, 1.f), r);
}

__global__ void __launch_bounds__(512, 1) k_diag_lu(float* __restrict__ A, int64_t ld, int k,
                                                 float* __restrict__ SI, int* __restrict__ info,
                                                 const __grid_constant__ CUtensorMap mA,
                                                 const __grid_constant__ CUtensorMap mAlo,
                                                 const __grid_constant__ CUtensorMap mB,
                                                 const __grid_constant__ CUtensorMap mBlo, DiagPre pre) {
  extern __shared__ __align__(1024) float dsm[];
  float* S = dsm;                       // A -> L\U
  float* rowbuf = S + LU_NB * TLD;      // [warp 0-3][parity][2 rows][16]
  float* Ls = rowbuf + 4 * 4 * DB;      // 16 x 16 unit lower, column-major, ld 20
  float* LiP = Ls + 16 * 20;            // [parity][Linv_pp, Uinv_pp], column-major, ld 16
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const size_t off = (size_t)k * LU_NB;
  float* Ab = A + off + off * ld;
  float* SIk = SI + (size_t)k * LU_SI;  // [p][Linv_pp 256, Uinv_pp 256]
  // the block's own update on the tensor cores: warp 0 lane 0 loads the
  // operand chunks by TMA (four stages), warp 1 lane 0 issues the 3xTF32 MMAs
  // into TMEM while the block itself loads into S; the product is subtracted
  // from S below.  Every wait is bounded; a timeout sets info = -1.
  using namespace tc;
  uint32_t stg = 0, bars = 0, tmem = 0;
  uint32_t* s_tmem = nullptr;
  volatile int* s_pfail = nullptr;
  if (pre.on) {
    const uint32_t base_u = smem_u32(dsm);
    const uint32_t after = base_u + (uint32_t)DIAG_SMEM;
    stg = (after + 1023u) & ~1023u;
    bars = stg + DIAG_PRE_STAGES * DIAG_STAGE_BYTES;  // full[4], empty[4], done
    s_tmem = (uint32_t*)((uint8_t*)dsm + (bars - base_u) + 8 * (2 * DIAG_PRE_STAGES + 1));
    s_pfail = (volatile int*)(s_tmem + 1);
    if (t == 0) {
      *s_pfail = 0;
      for (int i = 0; i < DIAG_PRE_STAGES; ++i) {
        mbar_init(bars + 8 * i, 1);
        mbar_init(bars + 8 * (DIAG_PRE_STAGES + i), 1);
      }
      mbar_init(bars + 8 * (2 * DIAG_PRE_STAGES), 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_tmem)),
                   "r"(LU_NB)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    tmem = *s_tmem;
    constexpr int NCH = LU_NB / BK;
    const uint32_t full0 = bars, empty0 = bars + 8 * DIAG_PRE_STAGES, done = bars + 8 * 2 * DIAG_PRE_STAGES;
    if (warp == 0 && lane == 0) {
      for (int c = 0; c < NCH; ++c) {
        const int sidx = c % DIAG_PRE_STAGES;
        if (c >= DIAG_PRE_STAGES && !mbar_wait(empty0 + 8 * sidx, ((c / DIAG_PRE_STAGES) - 1) & 1)) {
          *s_pfail = 1;
          break;
        }
        const uint32_t st = stg + sidx * DIAG_STAGE_BYTES;
        mbar_expect_tx(full0 + 8 * sidx, DIAG_STAGE_BYTES);
        tma_load_2d(st, &mA, c * BK, 0, full0 + 8 * sidx);
        tma_load_2d(st + A_BYTES, &mAlo, c * BK, 0, full0 + 8 * sidx);
        tma_load_2d(st + 2 * A_BYTES, &mB, pre.bx0 + c * BK, pre.by0, full0 + 8 * sidx);
        tma_load_2d(st + 2 * A_BYTES + DIAG_B_BYTES, &mBlo, c * BK, 0, full0 + 8 * sidx);
      }
    } else if (warp == 1 && lane == 0) {
      for (int c = 0; c < NCH; ++c) {
        const int sidx = c % DIAG_PRE_STAGES;
        if (!mbar_wait(full0 + 8 * sidx, (c / DIAG_PRE_STAGES) & 1)) {
          *s_pfail = 1;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t st = stg + sidx * DIAG_STAGE_BYTES;
        const uint64_t dah = sdesc(st), dal = sdesc(st + A_BYTES);
        const uint64_t dbh = sdesc(st + 2 * A_BYTES), dbl = sdesc(st + 2 * A_BYTES + DIAG_B_BYTES);
#pragma unroll
        for (int ks = 0; ks < BK / 8; ++ks) {
          const uint64_t o = (uint64_t)((ks * 32) >> 4);
          const uint32_t acc0 = (c > 0 || ks > 0) ? 1u : 0u;
          mma_tf32(tmem, dal + o, dbh + o, acc0, IDESC_N128);
          mma_tf32(tmem, dah + o, dbl + o, 1u, IDESC_N128);
          mma_tf32(tmem, dah + o, dbh + o, 1u, IDESC_N128);
        }
        mma_commit(empty0 + 8 * sidx);
      }
      mma_commit(done);
    }
    __syncwarp();
  }
  {
    // 8 float4 per thread, all loads in flight before the first store
    float4 v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int idx = t + 512 * i, r4 = 4 * (idx & 31), c = idx >> 5;
      v[i] = __ldcg((const float4*)(Ab + r4 + (size_t)c * ld));
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int idx = t + 512 * i, r4 = 4 * (idx & 31), c = idx >> 5;
      *(float4*)&S[c * TLD + r4] = v[i];
    }
  }
  __syncthreads();
  if (pre.on) {
    // S -= the product: thread (warp w, lane l) takes row 32 (w % 4) + l
    // (its TMEM lane) and columns 32 (w / 4) .. +31
    const uint32_t done = bars + 8 * 2 * DIAG_PRE_STAGES;
    int ok = 0;
    if (lane == 0) ok = mbar_wait(done, 0) ? 1 : 0;
    ok = __shfl_sync(0xffffffffu, ok, 0);
    const int all_ok = __syncthreads_and(ok) && !*s_pfail;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (all_ok) {
      const int q = warp & 3, cb = 32 * (warp >> 2), r = 32 * q + lane;
      uint32_t v[32];
      tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)cb, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) S[(cb + j) * TLD + r] -= __uint_as_float(v[j]);
    } else if (t == 0) {
      atomicExch(info, -1);
      // the MMAs issued finish before their accumulator is freed
      mbar_wait(done, 0);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(LU_NB) : "memory");
    }
  }
  int bad = 0;
  // phase A of panel jb (warps 0-3): factor rows jb.. of columns jb..jb+15,
  // warp 1 then inverts the unit-lower 16 x 16 block into Li
  auto factor_panel = [&](int jb, float* Li) {
    float PT[DB], PB[DB];
    const int rb = jb + DB + 32 * warp + lane;
    const bool tv = lane < DB, bv = rb < LU_NB;
#pragma unroll
    for (int c = 0; c < DB; ++c) {
      PT[c] = tv ? S[(jb + c) * TLD + jb + lane] : 0.f;
      PB[c] = bv ? S[(jb + c) * TLD + rb] : 0.f;
    }
    // two columns per step: pivot rows c and c+1 go out together, and every
    // lane forms row c+1 after column c itself (the same operations lane c+1
    // performs on its own copy), so one broadcast serves two columns; the
    // results are those of the column-by-column order
    float* myrow = rowbuf + warp * 4 * DB;
#pragma unroll
    for (int c = 0; c < DB; c += 2) {
      float* rw = myrow + ((c >> 1) & 1) * 2 * DB;
      if (lane == c || lane == c + 1) {
        float* dst = rw + (lane - c) * DB;
#pragma unroll
        for (int q4 = 0; q4 < DB; q4 += 4)
          *(float4*)&dst[q4] = make_float4(PT[q4], PT[q4 + 1], PT[q4 + 2], PT[q4 + 3]);
      }
      __syncwarp();
      float r0[DB], r1[DB];
#pragma unroll
      for (int q4 = 0; q4 < DB; q4 += 4) {
        const float4 v4 = *(const float4*)&rw[q4];
        r0[q4] = v4.x; r0[q4 + 1] = v4.y; r0[q4 + 2] = v4.z; r0[q4 + 3] = v4.w;
        const float4 w4 = *(const float4*)&rw[DB + q4];
        r1[q4] = w4.x; r1[q4 + 1] = w4.y; r1[q4 + 2] = w4.z; r1[q4 + 3] = w4.w;
      }
      const float p0 = r0[c];
      if (!(fabsf(p0) > 1e-30f && fabsf(p0) < INFINITY)) bad = 1;
      const float inv0 = rcp_nr(p0);
      // pivot row c+1 after column c
      {
        const float l = r1[c] * inv0;
#pragma unroll
        for (int c2 = c + 1; c2 < DB; ++c2) r1[c2] = fmaf(-l, r0[c2], r1[c2]);
      }
      const float p1 = r1[c + 1];
      if (!(fabsf(p1) > 1e-30f && fabsf(p1) < INFINITY)) bad = 1;
      const float inv1 = rcp_nr(p1);
      if (lane > c && tv) {
        const float l = PT[c] * inv0;
        PT[c] = l;
#pragma unroll
        for (int c2 = c + 1; c2 < DB; ++c2) PT[c2] = fmaf(-l, r0[c2], PT[c2]);
      }
      if (lane > c + 1 && tv) {
        const float l = PT[c + 1] * inv1;
        PT[c + 1] = l;
#pragma unroll
        for (int c2 = c + 2; c2 < DB; ++c2) PT[c2] = fmaf(-l, r1[c2], PT[c2]);
      }
      if (bv) {
        const float l = PB[c] * inv0;
        PB[c] = l;
#pragma unroll
        for (int c2 = c + 1; c2 < DB; ++c2) PB[c2] = fmaf(-l, r0[c2], PB[c2]);
        const float m = PB[c + 1] * inv1;
        PB[c + 1] = m;
#pragma unroll
        for (int c2 = c + 2; c2 < DB; ++c2) PB[c2] = fmaf(-m, r1[c2], PB[c2]);
      }
    }
    if (bv) {
#pragma unroll
      for (int c = 0; c < DB; ++c) S[(jb + c) * TLD + rb] = PB[c];
    }
    if (warp == 0 && tv) {
#pragma unroll
      for (int c = 0; c < DB; ++c) S[(jb + c) * TLD + jb + lane] = PT[c];
    } else if (warp == 1) {
      // inverse of the unit-lower 16 x 16 block, lane c < 16 solving for
      // column c by column-oriented forward substitution
      if (tv) {
#pragma unroll
        for (int q = 0; q < DB; ++q) Ls[q * 20 + lane] = PT[q];
      }
      __syncwarp();
      float x[DB];
#pragma unroll
      for (int i = 0; i < DB; ++i) x[i] = (i == lane) ? 1.f : 0.f;
#pragma unroll
      for (int q = 0; q < DB - 1; ++q) {
#pragma unroll
        for (int i = q + 1; i < DB; ++i) x[i] = fmaf(-Ls[q * 20 + i], x[q], x[i]);
      }
      if (tv) {
#pragma unroll
        for (int i4 = 0; i4 < DB; i4 += 4)
          *(float4*)&Li[lane * DB + i4] = make_float4(x[i4], x[i4 + 1], x[i4 + 2], x[i4 + 3]);
      }
    }
  };
  // trailing update S[r, c] -= L21[r, :] U12[:, c] of panel jb for rows
  // [jb+16, 128) and the columns [c0, c1) (multiples of 4), by `nth`
  // threads numbered from `tid`
  auto trailing = [&](int jb, int c0, int c1, int tid, int nth) {
    const int nr = (LU_NB - jb - DB) / 4, ncl = (c1 - c0) / 4;
    const float* Pb = S + jb * TLD + jb + DB;  // L21(r, q)
    const float* Qb = S + c0 * TLD + jb;       // U12(q, c)
    float* Cb = S + c0 * TLD + jb + DB;
    for (int idx = tid; idx < nr * ncl; idx += nth) {
      const int r0 = 4 * (idx % nr), cc = 4 * (idx / nr);
      float acc[4][4] = {};
      tile_mm<4>(Pb, Qb, r0, cc, 0, DB, acc);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        float4 cv = *(float4*)&Cb[(cc + j) * TLD + r0];
        cv.x -= acc[0][j]; cv.y -= acc[1][j]; cv.z -= acc[2][j]; cv.w -= acc[3][j];
        *(float4*)&Cb[(cc + j) * TLD + r0] = cv;
      }
    }
  };
  // The phases are pipelined: after the block row of U of panel p, warps
  // 0-3 update only panel p+1's columns, meet at a 128-thread named barrier
  // and factor panel p+1 while warps 4-15 store panel p and apply the rest
  // of its trailing update.  The 16 x 16 inverses are double-buffered by
  // panel parity (panel p's are stored while panel p+1's are formed).
  if (warp < 4) factor_panel(0, LiP);
  __syncthreads();
  for (int p = 0; p < LU_NB / DB; ++p) {
    const int jb = p * DB;
    float* Li = LiP + (p & 1) * 2 * DB * DB;
    // ---- B: block row of U, U[p, >p] = Linv_pp A[p, >p]: four threads
    // per column (lanes 4m .. 4m+3 of one warp), rows 4 (t % 4) .. +3 each;
    // the column is read whole before any of its four threads writes ----
    {
      const int c = jb + DB + (t >> 2), i0 = 4 * (t & 3);
      const bool on = c < LU_NB;
      float o0 = 0.f, o1 = 0.f, o2 = 0.f, o3 = 0.f;
      if (on) {
        float v[DB];
#pragma unroll
        for (int q4 = 0; q4 < DB; q4 += 4) {
          const float4 a = *(const float4*)&S[c * TLD + jb + q4];
          v[q4] = a.x; v[q4 + 1] = a.y; v[q4 + 2] = a.z; v[q4 + 3] = a.w;
        }
#pragma unroll
        for (int q = 0; q < DB; ++q) {
          const float4 l = *(const float4*)&Li[q * DB + i0];
          o0 = fmaf(l.x, v[q], o0);
          o1 = fmaf(l.y, v[q], o1);
          o2 = fmaf(l.z, v[q], o2);
          o3 = fmaf(l.w, v[q], o3);
        }
      }
      __syncwarp();
      if (on) *(float4*)&S[c * TLD + jb + i0] = make_float4(o0, o1, o2, o3);
    }
    __syncthreads();
    if (warp < 4) {
      if (p + 1 < LU_NB / DB) {
        // ---- C1: the next panel's columns; then A of panel p+1 ----
        trailing(jb, jb + DB, jb + 2 * DB, t, 128);
        asm volatile("bar.sync 1, 128;" ::: "memory");
        factor_panel(jb + DB, LiP + ((p + 1) & 1) * 2 * DB * DB);
      }
    } else {
      // ---- store column block p of L\U and its lower inverse; the upper
      // inverse (warp 4, beside the next panel's factorization); C2 ----
      if (warp == 4) {
        // inverse of the upper 16 x 16 block, lane c < 16 solving for column
        // c by column-oriented back substitution; Uinv(i, c) = Ui[c * 16 + i]
        float x[DB];
#pragma unroll
        for (int i = 0; i < DB; ++i) x[i] = (i == lane) ? 1.f : 0.f;
#pragma unroll
        for (int q = DB - 1; q >= 0; --q) {
          const float* uc = S + (jb + q) * TLD + jb;
          x[q] *= rcp_nr(uc[q]);
#pragma unroll
          for (int i = 0; i < q; ++i) x[i] = fmaf(-uc[i], x[q], x[i]);
        }
        if (lane < DB) {
          float* Ug = SIk + p * 2 * DB * DB + DB * DB;
#pragma unroll
          for (int i4 = 0; i4 < DB; i4 += 4)
            *(float4*)&Ug[lane * DB + i4] = make_float4(x[i4], x[i4 + 1], x[i4 + 2], x[i4 + 3]);
        }
      } else {
        for (int idx = t - 160; idx < DB * 32; idx += 352) {
          const int cs = jb + (idx >> 5), r4 = 4 * (idx & 31);
          *(float4*)(Ab + r4 + (size_t)cs * ld) = *(const float4*)&S[cs * TLD + r4];
        }
        for (int idx = t - 160; idx < DB * DB; idx += 352) SIk[p * 2 * DB * DB + idx] = Li[idx];
      }
      if (jb + 2 * DB < LU_NB) trailing(jb, jb + 2 * DB, LU_NB, t - 128, 384);
    }
    __syncthreads();
  }
  if (warp == 0) {
    bad = __any_sync(0xffffffffu, bad);
    if (lane == 0 && bad) atomicExch(info, k + 1);
  }
}

constexpr int PW = 32;  // slice width
constexpr int PXLD = PW + 4;
// shared floats of the panel kernel: the factored block, the slice, one
// side's eight 16 x 16 sub-block inverses
constexpr int PANEL_SMEM = (int)sizeof(float) * (LU_NB * TLD + LU_NB * PXLD + LU_SI / 2 + DB * PW);

__device__ __forceinline__ void cp_async16(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}

// Panels of diagonal block k by blocked triangular solves with its factored
// block Dk (L unit lower and U upper, leading dimension ldk) and its 16 x 16
// sub-block inverses SIk (from k_diag_lu):
//   blockIdx.y == 0: columns [32 x, 32 x + 32) of B (128 rows): X = L^{-1} B.
//     For each sub-block p: X_p = Linv_pp B_p, then B_q -= L_qp X_p (q > p).
//   blockIdx.y == 1: rows [32 x, 32 x + 32) of Ap (128 columns): X = Ap U^{-1}.
//     For each sub-block p: X_p = B_p Uinv_pp, then B_q -= X_p U_pq (q > p).
// ident: the slices start as the corresponding part of the identity (not
// read), which gives the full inverses L^{-1} and U^{-1} of the block for the
// triangular sweeps.  B and Ap have leading dimension ld.  blockIdx.z
// offsets Dk, SIk and B/Ap by z times zsD, zsSI and zsX (all diagonal blocks
// in one launch).  When Lt is given, the kernel also writes the operands of
// the step's tensor-core trailing update: Lt / Ltlo = L21 and its TF32 low
// part x - tf32(x), row-major [row][k] (rows counted from the first row
// below the block), and Ulo = the low part of U12, [column][k].
__device__ __forceinline__ float tf32_low(float x) {
  return x - __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
}

__global__ void __launch_bounds__(256) k_panels(const float* __restrict__ Dk, int64_t ldk,
                                                const float* __restrict__ SIk, float* B, float* Ap, int64_t ld,
                                                int ident, int64_t zsD, int64_t zsSI, int64_t zsX,
                                                float* __restrict__ Lt, float* __restrict__ Ltlo,
                                                float* __restrict__ Ulo) {
  extern __shared__ __align__(16) float psm[];
  Dk += blockIdx.z * zsD;
  SIk += blockIdx.z * zsSI;
  B += blockIdx.z * zsX;
  Ap += blockIdx.z * zsX;
  float* Ms = psm;                   // factored block, column-major, ld TLD
  float* Xs = psm + LU_NB * TLD;     // the slice
  float* Si = Xs + LU_NB * PXLD;     // [p][16 x 16], column-major
  float* Xp = Si + LU_SI / 2;        // the current sub-block X_p (16 x 32)
  const int t = threadIdx.x;
  const int side = blockIdx.y;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const int idx = t + 256 * i, r4 = 4 * (idx & 31), kx = idx >> 5;
    cp_async16(&Ms[kx * TLD + r4], Dk + r4 + (size_t)kx * ldk);
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const int idx = t + 256 * i, p = idx >> 6, e4 = 4 * (idx & 63);
    cp_async16(&Si[p * DB * DB + e4], SIk + p * 2 * DB * DB + side * DB * DB + e4);
  }
  if (side == 0) {
    // slice [col][row], ld TLD: Xs[c * TLD + r]
    float* Bb = B + (size_t)blockIdx.x * PW * ld;
    if (ident) {
      for (int idx = t; idx < PW * LU_NB; idx += 256) {
        const int r = idx & (LU_NB - 1), c = idx >> 7;
        Xs[c * TLD + r] = (r == (int)blockIdx.x * PW + c) ? 1.f : 0.f;
      }
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int idx = t + 256 * i, k4 = 4 * (idx & 31), c = idx >> 5;
        cp_async16(&Xs[c * TLD + k4], Bb + k4 + (size_t)c * ld);
      }
    }
    cp_async_wait_all();
    __syncthreads();
    for (int p = 0; p < LU_NB / DB; ++p) {
      const int jb = p * DB;
      const float* Li = Si + p * DB * DB;  // Linv_pp(i, q) = Li[q * 16 + i]
      {
        // X_p = Linv_pp B_p into Xp[c][16]: thread -> column t / 8, rows
        // 2 (t % 8) .. +1
        const int c = t >> 3, r2 = 2 * (t & 7);
        float o0 = 0.f, o1 = 0.f;
#pragma unroll
        for (int q = 0; q < DB; ++q) {
          const float b = Xs[c * TLD + jb + q];
          o0 = fmaf(Li[q * DB + r2], b, o0);
          o1 = fmaf(Li[q * DB + r2 + 1], b, o1);
        }
        Xp[c * DB + r2] = o0;
        Xp[c * DB + r2 + 1] = o1;
      }
      __syncthreads();
      // rows jb.. of the slice take X_p (two values per thread)
      {
        const int c = t >> 3, r2 = 2 * (t & 7);
        Xs[c * TLD + jb + r2] = Xp[c * DB + r2];
        Xs[c * TLD + jb + r2 + 1] = Xp[c * DB + r2 + 1];
      }
      // B_q -= L_qp X_p: thread -> row jb + 16 + (t % 128), 16 columns
      const int i = jb + DB + (t & (LU_NB - 1));
      if (i < LU_NB) {
        float l[DB];
#pragma unroll
        for (int q = 0; q < DB; ++q) l[q] = Ms[(jb + q) * TLD + i];
        const int cb = (t >> 7) * (PW / 2);
#pragma unroll 4
        for (int cc = 0; cc < PW / 2; ++cc) {
          const int c = cb + cc;
          const float* xp = Xp + c * DB;
          float acc = Xs[c * TLD + i];
#pragma unroll
          for (int q4 = 0; q4 < DB; q4 += 4) {
            const float4 x = *(const float4*)&xp[q4];
            acc = fmaf(-l[q4], x.x, acc);
            acc = fmaf(-l[q4 + 1], x.y, acc);
            acc = fmaf(-l[q4 + 2], x.z, acc);
            acc = fmaf(-l[q4 + 3], x.w, acc);
          }
          Xs[c * TLD + i] = acc;
        }
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int idx = t + 256 * i, r4 = 4 * (idx & 31), c = idx >> 5;
      const float4 v = *(const float4*)&Xs[c * TLD + r4];
      *(float4*)&Bb[r4 + (size_t)c * ld] = v;
      if (Ulo)
        *(float4*)&Ulo[(size_t)(blockIdx.x * PW + c) * LU_NB + r4] =
            make_float4(tf32_low(v.x), tf32_low(v.y), tf32_low(v.z), tf32_low(v.w));
    }
  } else {
    // slice [col][row], ld PXLD: Xs[c * PXLD + r], 32 rows
    float* Ab = Ap + (size_t)blockIdx.x * PW;
    if (ident) {
      for (int idx = t; idx < PW * LU_NB; idx += 256) {
        const int r = idx & (PW - 1), c = idx >> 5;
        Xs[c * PXLD + r] = ((int)blockIdx.x * PW + r == c) ? 1.f : 0.f;
      }
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int idx = t + 256 * i, r4 = 4 * (idx & 7), kx = idx >> 3;
        cp_async16(&Xs[kx * PXLD + r4], Ab + r4 + (size_t)kx * ld);
      }
    }
    cp_async_wait_all();
    __syncthreads();
    const int r = t & (PW - 1), g = t >> 5;
    for (int p = 0; p < LU_NB / DB; ++p) {
      const int jb = p * DB;
      const float* Ui = Si + p * DB * DB;  // Uinv_pp(q, c) = Ui[c * 16 + q]
      {
        // X_p = B_p Uinv_pp into Xp[c][32]: thread -> row t % 32, columns
        // 2 (t / 32) .. +1
        const int c2 = 2 * g;
        float o0 = 0.f, o1 = 0.f;
#pragma unroll
        for (int q = 0; q < DB; ++q) {
          const float b = Xs[(jb + q) * PXLD + r];
          o0 = fmaf(b, Ui[c2 * DB + q], o0);
          o1 = fmaf(b, Ui[(c2 + 1) * DB + q], o1);
        }
        Xp[c2 * PW + r] = o0;
        Xp[(c2 + 1) * PW + r] = o1;
      }
      __syncthreads();
      // B_q -= X_p U_pq: thread -> row t % 32, columns jb + 16 + t / 32 + 8 m;
      // columns jb.. of the slice take X_p
      float x[DB];
#pragma unroll
      for (int q = 0; q < DB; ++q) x[q] = Xp[q * PW + r];
      Xs[(jb + 2 * g) * PXLD + r] = Xp[2 * g * PW + r];
      Xs[(jb + 2 * g + 1) * PXLD + r] = Xp[(2 * g + 1) * PW + r];
      for (int c = jb + DB + g; c < LU_NB; c += 8) {
        const float* up = Ms + c * TLD + jb;
        float acc = Xs[c * PXLD + r];
#pragma unroll
        for (int q4 = 0; q4 < DB; q4 += 4) {
          const float4 u = *(const float4*)&up[q4];
          acc = fmaf(-x[q4], u.x, acc);
          acc = fmaf(-x[q4 + 1], u.y, acc);
          acc = fmaf(-x[q4 + 2], u.z, acc);
          acc = fmaf(-x[q4 + 3], u.w, acc);
        }
        Xs[c * PXLD + r] = acc;
      }
      __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int idx = t + 256 * i, r4 = 4 * (idx & 7), c = idx >> 3;
      *(float4*)(Ab + r4 + (size_t)c * ld) = *(const float4*)&Xs[c * PXLD + r4];
    }
    if (Lt) {
      // row-major copies for the tensor-core operands: thread -> row t / 8,
      // columns 4 (t % 8) + 32 j
      const int rr = t >> 3, c4 = 4 * (t & 7);
      const size_t row = (size_t)blockIdx.x * PW + rr;
#pragma unroll
      for (int j = 0; j < LU_NB / 32; ++j) {
        const int c = 32 * j + c4;
        const float4 v = make_float4(Xs[c * PXLD + rr], Xs[(c + 1) * PXLD + rr], Xs[(c + 2) * PXLD + rr],
                                     Xs[(c + 3) * PXLD + rr]);
        *(float4*)&Lt[row * LU_NB + c] = v;
        *(float4*)&Ltlo[row * LU_NB + c] = make_float4(tf32_low(v.x), tf32_low(v.y), tf32_low(v.z), tf32_low(v.w));
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Thin look-ahead updates of one LU step in FP32 on the CUDA cores: block
// column k+1 (C: rem x 128) and block row k+1 (C: 128 x rem-128) get
// C -= L21 U12 with K = 128.  64 x 64 tiles, operands staged by cp.async,
// 4 x 4 register tiles; a 1-D grid lists the tiles.  The column part covers
// rows [ro, ro + M0) of the block column; the row part is included when
// with_row is set (the look-ahead runs the diagonal block, ro = 0 and
// M0 = 128, ahead of the rest).
// ---------------------------------------------------------------------------
constexpr int TT = 64;
constexpr int TPLD = TT + 4;      // staged L: [q][r]
constexpr int TQLD = LU_NB + 4;   // staged U: [c][q]
constexpr int THIN_SMEM = (int)sizeof(float) * (LU_NB * TPLD + TT * TQLD);

__global__ void __launch_bounds__(256) k_thin_update(float* A, int64_t ld, int kk, int rem, int ro, int M0) {
  extern __shared__ __align__(16) float tsm[];
  float* Ps = tsm;                  // Ps[q * TPLD + r] = L21(m0 + r, q)
  float* Qs = tsm + LU_NB * TPLD;   // Qs[c * TQLD + q] = U12(q, n0 + c)
  const int t = threadIdx.x;
  const int ncol = (M0 / TT) * (LU_NB / TT);
  int tile = blockIdx.x, z = 0;
  if (tile >= ncol) { tile -= ncol; z = 1; }
  const int M = z == 0 ? M0 : LU_NB;
  const int mt = M / TT;
  const int m0 = (tile % mt) * TT + (z == 0 ? ro : 0), n0 = (tile / mt) * TT;
  const int co = z == 0 ? 0 : LU_NB;
  const size_t r_abs = (size_t)kk + LU_NB + m0, c_abs = (size_t)kk + LU_NB + co + n0;
  float* C = A + r_abs + c_abs * ld;
  const float* L = A + r_abs + (size_t)kk * ld;
  const float* U = A + (size_t)kk + c_abs * ld;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int idx = t + 256 * i;
    const int q = idx >> 4, r4 = 4 * (idx & 15);
    cp_async16(&Ps[q * TPLD + r4], L + r4 + (size_t)q * ld);
    const int c = idx >> 5, q4 = 4 * (idx & 31);
    cp_async16(&Qs[c * TQLD + q4], U + q4 + (size_t)c * ld);
  }
  cp_async_wait_all();
  __syncthreads();
  const int r0 = 4 * (t & 15), c0 = 4 * (t >> 4);
  float acc[4][4] = {};
#pragma unroll 4
  for (int q = 0; q < LU_NB; q += 4) {
    float4 pv[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) pv[i] = *(const float4*)&Ps[(q + i) * TPLD + r0];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float4 qv = *(const float4*)&Qs[(c0 + j) * TQLD + q];
      const float qq[4] = {qv.x, qv.y, qv.z, qv.w};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        acc[0][j] = fmaf(pv[i].x, qq[i], acc[0][j]);
        acc[1][j] = fmaf(pv[i].y, qq[i], acc[1][j]);
        acc[2][j] = fmaf(pv[i].z, qq[i], acc[2][j]);
        acc[3][j] = fmaf(pv[i].w, qq[i], acc[3][j]);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    float4* cp = (float4*)(C + r0 + (size_t)(c0 + j) * ld);
    float4 cv = *cp;
    cv.x -= acc[0][j];
    cv.y -= acc[1][j];
    cv.z -= acc[2][j];
    cv.w -= acc[3][j];
    *cp = cv;
  }
}

// rows [ro, ro + M0) of block column k+1, plus block row k+1 if with_row
static void thin_part(float* A, int64_t ld, int k, int rem, int ro, int M0, bool with_row, cudaStream_t st) {
  const int tiles = (M0 / TT) * (LU_NB / TT) + (with_row ? (LU_NB / TT) * ((rem - LU_NB) / TT) : 0);
  if (tiles <= 0) return;
  KScope kt(st, KC_LU_THIN);
  k_thin_update<<<tiles, 256, THIN_SMEM, st>>>(A, ld, k * LU_NB, rem, ro, M0);
  count_launches(1);
}

static void lu_attrs_once();
static void lu_attrs() {
  static std::once_flag once;
  std::call_once(once, lu_attrs_once);
}
static void lu_attrs_once() {
  cudaFuncSetAttribute(k_diag_factor_rb, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(sizeof(float) * LU_NB * DLD));
  cudaFuncSetAttribute(k_diag_lu, cudaFuncAttributeMaxDynamicSharedMemorySize, DIAG_SMEM_PRE);
  cudaFuncSetAttribute(k_gemm_mma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)gemm_mma_smem());
  cudaFuncSetAttribute(k_gemm_mma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)gemm_mma_smem());
  cudaFuncSetAttribute(k_panels, cudaFuncAttributeMaxDynamicSharedMemorySize, PANEL_SMEM);
  cudaFuncSetAttribute(k_thin_update, cudaFuncAttributeMaxDynamicSharedMemorySize, THIN_SMEM);
}

// sub-block inverses of diagonal block k (after the full inverses in Dinv)
static float* sub_inverses(float* Dinv, int Npad, int k) {
  return Dinv + (size_t)(Npad / LU_NB) * 2 * LU_NB * LU_NB + (size_t)k * LU_SI;
}

// diagonal block k; with P (the plan of step k-1), the block first gets
// that step's update on the tensor cores
static void diag_block(float* A, int64_t ld, int Npad, float* Dinv, int* info, int k, cudaStream_t st,
                       const TcPlan* P = nullptr) {
  KScope kd(st, KC_LU_DIAG);
  static const CUtensorMap none{};
  DiagPre pre{0, 0, 0};
  const CUtensorMap* m[4] = {&none, &none, &none, &none};
  if (P && k > 0) {
    pre = DiagPre{1, (k - 1) * LU_NB, k * LU_NB};
    m[0] = (const CUtensorMap*)P->mA;
    m[1] = (const CUtensorMap*)P->mAlo;
    m[2] = (const CUtensorMap*)P->mB128;
    m[3] = (const CUtensorMap*)P->mBlo128;
  }
  k_diag_lu<<<1, 512, pre.on ? DIAG_SMEM_PRE : DIAG_SMEM, st>>>(A, ld, k, sub_inverses(Dinv, Npad, 0), info, *m[0],
                                                              *m[1], *m[2], *m[3], pre);
  count_launches(1);
}

// the two panels of diagonal block k: U12 = L^{-1} A12, L21 = A21 U^{-1};
// with a plan, also the step's tensor-core operands (Lt, Ltlo, Ulo)
static void panels(float* A, int64_t ld, int Npad, float* Dinv, int k, cudaStream_t st,
                   const TcPlan* P = nullptr) {
  const size_t kk = (size_t)k * LU_NB;
  const int rem = Npad - (int)kk - LU_NB;
  if (rem <= 0) return;
  float* A12 = A + kk + (kk + LU_NB) * ld;
  float* A21 = A + (kk + LU_NB) + kk * ld;
  KScope kp(st, KC_LU_PANELS);
  k_panels<<<dim3(rem / PW, 2), 256, PANEL_SMEM, st>>>(A + kk + kk * ld, ld, sub_inverses(Dinv, Npad, k), A12,
                                                       A21, ld, 0, 0, 0, 0, P ? P->Lt : nullptr,
                                                       P ? P->Ltlo : nullptr, P ? P->Ulo : nullptr);
  count_launches(1);
}

// the full inverses of the unit-lower and upper triangles of diagonal blocks
// k0 .. k0 + nk - 1 into Dinv (for the triangular sweeps), one launch
static void block_inverses(float* A, int64_t ld, int Npad, float* Dinv, int k0, int nk, cudaStream_t st) {
  const size_t kk = (size_t)k0 * LU_NB;
  float* Lo = Dinv + (size_t)k0 * 2 * LU_NB * LU_NB;
  k_panels<<<dim3(LU_NB / PW, 2, nk), 256, PANEL_SMEM, st>>>(
      A + kk + kk * ld, ld, sub_inverses(Dinv, Npad, k0), Lo, Lo + LU_NB * LU_NB, LU_NB, 1,
      (int64_t)LU_NB * (ld + 1), LU_SI, 2 * LU_NB * LU_NB, nullptr, nullptr, nullptr);
  count_launches(1);
}

// diagonal block k, its panels and its inverses on one stream
static void diag_and_panels(float* A, int64_t ld, int Npad, float* Dinv, int* info, int x3, int k,
                            cudaStream_t st) {
  (void)x3;
  diag_block(A, ld, Npad, Dinv, info, k, st);
  panels(A, ld, Npad, Dinv, k, st);
  block_inverses(A, ld, Npad, Dinv, k, 1, st);
}

int lu_factor(float* A, int64_t ld, int Npad, float* Dinv, int* info, int x3, cudaStream_t st,
              const TcPlan* tc, int* err) {
  const int K = Npad / LU_NB;
  lu_attrs();
  for (int k = 0; k < K; ++k) {
    const size_t kk = (size_t)k * LU_NB;
    const int rem = Npad - (int)kk - LU_NB;
    diag_and_panels(A, ld, Npad, Dinv, info, x3, k, st);
    if (rem <= 0) break;
    float* A12 = A + kk + (kk + LU_NB) * ld;
    float* A21 = A + (kk + LU_NB) + kk * ld;
    float* A22 = A + (kk + LU_NB) + (kk + LU_NB) * ld;
    // A22 -= L21 * U12
    if (tc && tc->ok && x3) {
      tc_split(*tc, k, st);
      int e = tc_gemm_sub(*tc, k, 0, 0, rem, rem, err, st);
      if (e) return e;
    } else {
      gemm_tile128(A21, ld, A12, ld, A22, ld, rem, rem, -1.f, 1.f, x3, st);
    }
  }
  return (int)cudaGetLastError();
}

// Lookahead-1 schedule on three streams.  `la` (the critical path) factors
// diagonal block k+1 after applying step k's update to the block itself
// (inside the diagonal kernel), then its panels; `tl` meanwhile applies the rest of step k's thin update (block
// column k+1 below the diagonal block and block row k+1 right of it, FP32);
// `st` runs the bulk of step k's trailing update (its tensor-core operands
// come from the panel kernel), and at the end forms the full inverses
// of all diagonal blocks in one launch.  evP[k]: panels of step k ready;
// evT[k]: bulk update of step k done; evR[k]: thin update of step k done.
// tc[2]: plans with separate lo/transposed buffers for even and odd steps.
int lu_factor_lookahead(float* A, int64_t ld, int Npad, float* Dinv, int* info, cudaStream_t st,
                        cudaStream_t la, cudaEvent_t fork, cudaEvent_t* evP, cudaEvent_t* evT,
                        cudaStream_t tl, cudaEvent_t* evR, const TcPlan* tc, int* err, int* ctr) {
  const int K = Npad / LU_NB;
  lu_attrs();
  KScope total(st, KC_LU_TOTAL);
  cudaEventRecord(fork, st);
  cudaStreamWaitEvent(la, fork, 0);
  diag_block(A, ld, Npad, Dinv, info, 0, la);
  panels(A, ld, Npad, Dinv, 0, la, &tc[0]);
  cudaEventRecord(evP[0], la);
  for (int k = 0; k + 1 < K; ++k) {
    const int rem = Npad - (k + 1) * LU_NB;
    const TcPlan& P = tc[k & 1];
    if (k >= 1) cudaStreamWaitEvent(la, evT[k - 1], 0);
    // thin update of step k without the diagonal block: needs panels k
    // (evP[k]) and the bulk update of step k-1
    cudaStreamWaitEvent(tl, evP[k], 0);
    if (k >= 1) cudaStreamWaitEvent(tl, evT[k - 1], 0);
    thin_part(A, ld, k, rem, LU_NB, rem - LU_NB, true, tl);
    cudaEventRecord(evR[k], tl);
    {
      KScope crit(la, KC_LU_CRIT);
      diag_block(A, ld, Npad, Dinv, info, k + 1, la, &P);
      cudaStreamWaitEvent(la, evR[k], 0);
      panels(A, ld, Npad, Dinv, k + 1, la, &tc[(k + 1) & 1]);
    }
    cudaEventRecord(evP[k + 1], la);
    cudaStreamWaitEvent(st, evP[k], 0);
    if (rem > LU_NB) {
      KScope trail(st, KC_LU_TRAIL);
      // operands Lt, Ltlo, Ulo of step k were written by its panels
      int e = tc_gemm_sub(P, k, LU_NB, LU_NB, rem - LU_NB, rem - LU_NB, err, st, ctr);
      if (e) return e;
    }
    cudaEventRecord(evT[k], st);
  }
  cudaStreamWaitEvent(st, evP[K - 1], 0);
  // all block inverses in one launch once the factorization is done
  block_inverses(A, ld, Npad, Dinv, 0, K, st);
  return (int)cudaGetLastError();
}

// y = (L U)^{-1} r in place on a padded FP32 vector
static void lu_solve_vec_steps(const float* A, int64_t ld, int Npad, const float* Dinv, float* r, float* tmp,
                  cudaStream_t st) {
  const int K = Npad / LU_NB;
  // forward: L y = r (unit lower)
  for (int k = 0; k < K; ++k) {
    const size_t kk = (size_t)k * LU_NB;
    const float* Li = Dinv + (size_t)k * 2 * LU_NB * LU_NB;
    k_blk_apply<<<1, LU_NB, 0, st>>>(Li, r + kk, tmp);
    cudaMemcpyAsync(r + kk, tmp, sizeof(float) * LU_NB, cudaMemcpyDeviceToDevice, st);
    const int rows = Npad - (int)kk - LU_NB;
    if (rows > 0)
      k_panel_gemv<<<(rows + 255) / 256, 256, 0, st>>>(A + kk + LU_NB + kk * ld, ld, rows, r + kk,
                                                       r + kk + LU_NB);
  }
  // backward: U x = y
  for (int k = K - 1; k >= 0; --k) {
    const size_t kk = (size_t)k * LU_NB;
    const float* Ui = Dinv + (size_t)k * 2 * LU_NB * LU_NB + LU_NB * LU_NB;
    k_blk_apply<<<1, LU_NB, 0, st>>>(Ui, r + kk, tmp);
    cudaMemcpyAsync(r + kk, tmp, sizeof(float) * LU_NB, cudaMemcpyDeviceToDevice, st);
    if (kk > 0)
      k_panel_gemv<<<((int)kk + 255) / 256, 256, 0, st>>>(A + kk * ld, ld, (int)kk, r + kk, r);
  }
}

// y = (L U)^{-1} r on a padded FP32 vector.  r is overwritten with the
// forward result; the solution lands in `out`.  flags: 2K ints of scratch.
void lu_couplings(const float* A, int64_t ld, int Npad, const float* Dinv, float* Mc, cudaStream_t st) {
  static std::once_flag once;
  std::call_once(once, [] {
    cudaFuncSetAttribute(k_lu_couplings, cudaFuncAttributeMaxDynamicSharedMemorySize, CPL_SMEM);
  });
  const int K = Npad / LU_NB;
  if (K < 2) return;
  KScope ks(st, KC_TRSV);
  count_launches(1);
  k_lu_couplings<<<dim3(K, 2, 4), 256, CPL_SMEM, st>>>(A, ld, K, Dinv, Mc);
}

int lu_solve_vec(const float* A, int64_t ld, int Npad, const float* Dinv, const float* Mc, float* r, float* tmp,
                 float* out, unsigned long long* tags, int epoch, int* err, cudaStream_t st, int wait_limit,
                 int wepoch_shift, int pmax) {
  const int wepoch = epoch + wepoch_shift;
  const int K = Npad / LU_NB;
  static int max_coresident = 0;
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int dsm = (int)(sizeof(float) * LU_NB * (LU_NB + 1));
    cudaFuncSetAttribute(k_trsv_wave<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, dsm);
    cudaFuncSetAttribute(k_trsv_wave<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, dsm);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_trsv_wave<false>, 256, dsm);
    max_coresident = nsm * per;
  });
  const size_t dsm = sizeof(float) * LU_NB * (LU_NB + 1);
  if (K > max_coresident) {  // too many block rows to keep resident: step-wise launches
    lu_solve_vec_steps(A, ld, Npad, Dinv, r, tmp, st);
    cudaMemcpyAsync(out, r, sizeof(float) * Npad, cudaMemcpyDeviceToDevice, st);
    return 0;
  }
  // CTAs per block row: as many as stay resident, at most pmax
  const int pcap = pmax < 1 ? 1 : (pmax > LU_TRSV_PMAX ? LU_TRSV_PMAX : pmax);
  int P = max_coresident / K;
  P = P < 1 ? 1 : (P > pcap ? pcap : P);
  KScope ks(st, KC_TRSV);
  count_launches(2);
  unsigned long long* t0 = tags;
  unsigned long long* t1 = tags + Npad;
  unsigned long long* p0 = tags + 2 * (size_t)Npad;
  unsigned long long* p1 = p0 + (size_t)LU_TRSV_PMAX * Npad;
  const dim3 grid(K * P);
  {
    void* args[] = {(void*)&A, (void*)&ld, (void*)&K, (void*)&Dinv, (void*)&Mc, (void*)&r, (void*)&tmp,
                    (void*)&t0, (void*)&p0, (void*)&P, (void*)&epoch, (void*)&wepoch, (void*)&wait_limit,
                    (void*)&err};
    // forward: r -> tmp (separate output so that no CTA reads a block another rewrote)
    cudaError_t e = cudaLaunchCooperativeKernel((void*)k_trsv_wave<false>, grid, dim3(256), args, dsm, st);
    if (e != cudaSuccess) return (int)e;
  }
  {
    void* args[] = {(void*)&A, (void*)&ld, (void*)&K, (void*)&Dinv, (void*)&Mc, (void*)&tmp, (void*)&out,
                    (void*)&t1, (void*)&p1, (void*)&P, (void*)&epoch, (void*)&wepoch, (void*)&wait_limit,
                    (void*)&err};
    cudaError_t e = cudaLaunchCooperativeKernel((void*)k_trsv_wave<true>, grid, dim3(256), args, dsm, st);
    if (e != cudaSuccess) return (int)e;
  }
  return 0;
}

void residual64(const double* A, int64_t lda, int N, const double* x, const double* b, double* r,
                cudaStream_t st) {
  KScope ks(st, KC_GEMV);
  count_launches(1);
  cudaMemsetAsync(r, 0, sizeof(double) * N, st);
  const int chunk = 512;
  dim3 grid((N + 127) / 128, (N + chunk - 1) / chunk);
  k_residual64<<<grid, 128, 0, st>>>(A, lda, N, x, b, r, chunk);
}

void gemv64(const double* A, int64_t lda, int N, const double* x, double* y, cudaStream_t st) {
  KScope ks(st, KC_GEMV);
  count_launches(1);
  cudaMemsetAsync(y, 0, sizeof(double) * N, st);
  const int chunk = 512;
  dim3 grid((N + 127) / 128, (N + chunk - 1) / chunk);
  k_gemv64<<<grid, 128, 0, st>>>(A, lda, N, x, y, chunk);
}

void dots64(const double* V, int64_t ldv, int N, int m, const double* w, double* h, cudaStream_t st) {
  count_launches(1);
  cudaMemsetAsync(h, 0, sizeof(double) * m, st);
  const int slices = (N + 2047) / 2048 < 16 ? (N + 2047) / 2048 : 16;
  k_dots<<<dim3(m, slices > 0 ? slices : 1), 256, 0, st>>>(V, ldv, N, m, w, h);
}
void sub_vh64(const double* V, int64_t ldv, int N, int m, const double* h, double* w, cudaStream_t st) {
  count_launches(1);
  k_sub_vh<<<(N + 255) / 256, 256, 0, st>>>(V, ldv, N, m, h, w);
}
void add_zy64(const double* Z, int64_t ldz, int N, int m, const double* y, double* x, cudaStream_t st) {
  count_launches(1);
  k_add_zy<<<(N + 255) / 256, 256, 0, st>>>(Z, ldz, N, m, y, x);
}
void scale_by_norm64(const double* w, const double* n2, double* v, int N, cudaStream_t st) {
  count_launches(1);
  k_scale_by_norm<<<(N + 255) / 256, 256, 0, st>>>(w, n2, v, N);
}
void scale_copy64(const double* w, double s, double* v, int N, cudaStream_t st) {
  count_launches(1);
  k_scale_copy<<<(N + 255) / 256, 256, 0, st>>>(w, s, v, N);
}
void to_f32(const double* v, int N, int Npad, float* o, cudaStream_t st) {
  count_launches(1);
  k_to_f32<<<(Npad + 255) / 256, 256, 0, st>>>(v, N, Npad, o);
}
void from_f32_scale(const float* y, const double* cs, int N, double* z, cudaStream_t st) {
  count_launches(1);
  k_from_f32_scale<<<(N + 255) / 256, 256, 0, st>>>(y, cs, N, z);
}

}  // namespace bem

namespace bem {
// Self-check: factor the diagonal block at (0, 0) of A1 with the blocked
// kernel and of A2 (a copy) with the register-blocked Gauss-Jordan kernel;
// D1, D2 receive the two pairs of triangular inverses.
void diag_selftest(float* A1, float* A2, int64_t ld, float* D1, float* D2, float* SI, int* info,
                   cudaStream_t st) {
  lu_attrs();
  {
    static const CUtensorMap none{};
    k_diag_lu<<<1, 512, DIAG_SMEM, st>>>(A1, ld, 0, SI, info, none, none, none, none, DiagPre{0, 0, 0});
  }
  k_panels<<<dim3(LU_NB / PW, 2), 256, PANEL_SMEM, st>>>(A1, ld, SI, D1, D1 + LU_NB * LU_NB, LU_NB, 1, 0, 0, 0,
                                                        nullptr, nullptr, nullptr);
  k_diag_factor_rb<<<1, 512, sizeof(float) * LU_NB * DLD, st>>>(A2, ld, 0, D2, info);
  count_launches(3);
}
}  // namespace bem
