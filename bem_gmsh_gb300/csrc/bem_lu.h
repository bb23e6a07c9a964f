// Internal interface of the dense solve kernels (lu.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define LU_NB 128  // LU block size (rows/columns of a diagonal block)
#define LU_SB 16   // sub-block of the diagonal factorization and of the panel solves
// floats per diagonal block of the 16 x 16 sub-block inverses (L^{-1}, U^{-1})
#define LU_SI (2 * (LU_NB / LU_SB) * LU_SB * LU_SB)

namespace bem {

// cs[j] = 2^s_j with max_i |A[i, j]| 2^s_j in [0.5, 1); A32 = A * diag(cs)
// rounded to FP32, identity padding up to Npad (a multiple of LU_NB).
void lu_prepare(const double* A64, int64_t lda, int N, int Npad, double* cs, float* A32,
                int64_t ld32, cudaStream_t st);
// In-place blocked LU without pivoting of the Npad x Npad FP32 matrix.
// Dinv (lu_dinv_floats(K) floats) receives, per diagonal block, the inverses
// of its unit-lower and upper triangles (2 x LU_NB^2 floats per block), and
// after all blocks the 16 x 16 sub-block inverses (LU_SI floats per block).
// info: first block with a vanishing pivot (1-based), untouched otherwise.
// x3: 3xTF32 updates.
inline size_t lu_dinv_floats(int K) { return (size_t)K * (2 * LU_NB * LU_NB + LU_SI); }
struct TcPlan;
int lu_factor(float* A, int64_t ld, int Npad, float* Dinv, int* info, int x3, cudaStream_t st,
              const TcPlan* tc = nullptr, int* err = nullptr);
// M_b couplings of the triangular sweeps (Mc: K * 2 * 128^2 floats), after
// the factorization
void lu_couplings(const float* A, int64_t ld, int Npad, const float* Dinv, float* Mc, cudaStream_t st);
// (epoch, value) words of the triangular sweeps: y of both sweeps (2 Npad)
// and the helpers' partial sums (at most LU_TRSV_PMAX CTAs per block row)
constexpr int LU_TRSV_PMAX = 4;
inline size_t lu_tag_words(int Npad) { return (size_t)(2 + 2 * LU_TRSV_PMAX) * (size_t)Npad; }
// out <- U^{-1} L^{-1} r on padded FP32 vectors.  tmp: Npad floats (the
// forward result); tags: lu_tag_words(Npad) words of (epoch, value) scratch,
// zeroed before the first call; epoch: > 0 and different in every call on
// the same tags; err: timeout flag, set when a wait polled wait_limit times
// in vain.  wepoch_shift (failure injection, normally 0): results are
// published under epoch + wepoch_shift, so that a nonzero shift makes every
// dependent wait run out.  pmax: at most this many CTAs per block row (the
// count also stays within what the GPU keeps resident).  r may be clobbered.
// Returns 0 or a CUDA error.
int lu_solve_vec(const float* A, int64_t ld, int Npad, const float* Dinv, const float* Mc, float* r, float* tmp,
                 float* out, unsigned long long* tags, int epoch, int* err, cudaStream_t st,
                 int wait_limit = 1 << 20, int wepoch_shift = 0, int pmax = LU_TRSV_PMAX);

void residual64(const double* A, int64_t lda, int N, const double* x, const double* b, double* r,
                cudaStream_t st);
void gemv64(const double* A, int64_t lda, int N, const double* x, double* y, cudaStream_t st);
void dots64(const double* V, int64_t ldv, int N, int m, const double* w, double* h, cudaStream_t st);
void sub_vh64(const double* V, int64_t ldv, int N, int m, const double* h, double* w, cudaStream_t st);
void add_zy64(const double* Z, int64_t ldz, int N, int m, const double* y, double* x, cudaStream_t st);
void scale_copy64(const double* w, double s, double* v, int N, cudaStream_t st);
// v = w / sqrt(*n2), n2 on the device
void scale_by_norm64(const double* w, const double* n2, double* v, int N, cudaStream_t st);
void to_f32(const double* v, int N, int Npad, float* o, cudaStream_t st);
void from_f32_scale(const float* y, const double* cs, int N, double* z, cudaStream_t st);

// C (M x N) = beta C + alpha A (M x 128) B (128 x N); M, N multiples of 128.
void gemm_tile128(const float* A, int64_t lda, const float* B, int64_t ldb, float* C, int64_t ldc,
                  int M, int N, float alpha, float beta, int x3, cudaStream_t st);

void diag_selftest(float* A1, float* A2, int64_t ld, float* D1, float* D2, float* SI, int* info,
                   cudaStream_t st);

// tcgen05 trailing update (gemm_tc.cu).  The plan holds the TMA maps of the
// transposed L panel, its lo part, the matrix (U panel) and the U lo part.
struct TcPlan {
  float* A = nullptr;
  int64_t ld = 0;
  int Npad = 0;
  float* Lt = nullptr;    // Npad x 128, K-major
  float* Ltlo = nullptr;  // Npad x 128
  float* Ulo = nullptr;   // 128 x Npad (K-major per column)
  alignas(64) unsigned char mA[128];
  alignas(64) unsigned char mAlo[128];
  alignas(64) unsigned char mB[128];
  alignas(64) unsigned char mBlo[128];
  alignas(64) unsigned char mC[128];  // the matrix as C (persistent kernel)
  alignas(64) unsigned char mB128[128];    // B and B lo with 128-column boxes
  alignas(64) unsigned char mBlo128[128];  // (the diagonal block's own update)
  bool ok = false;
  int variant = 1;  // 1: one CTA per tile; 2: persistent, warp-specialized
  int grid = 0;     // persistent kernel: CTAs (SMs) it may use
};
// variant 2 runs the persistent kernel on all SMs but `reserve`
bool tc_plan(TcPlan& p, float* A, int64_t ld, int Npad, float* Lt, float* Ltlo, float* Ulo, int variant = 1,
             int reserve = 0);
// Lt, Ltlo, Ulo of step k (from the factored panels)
void tc_split(const TcPlan& p, int k, cudaStream_t st);
// part of step k's trailing update: rows [ro, ro+M), columns [co, co+N) of
// the trailing matrix  A22 -= L21 U12.  ctr: two zeroed device ints that the
// persistent kernel's CTAs claim tiles from (and rearm when done), or null
// for a static tile order; launches sharing ctr must not overlap.
int tc_gemm_sub(const TcPlan& p, int k, int ro, int co, int M, int N, int* err, cudaStream_t st,
                int* ctr = nullptr);
// ctr: two zeroed device ints for the bulk updates' tile counter (or null)
int lu_factor_lookahead(float* A, int64_t ld, int Npad, float* Dinv, int* info, cudaStream_t st,
                        cudaStream_t la, cudaEvent_t fork, cudaEvent_t* evP, cudaEvent_t* evT,
                        cudaStream_t tl, cudaEvent_t* evR, const TcPlan* tc, int* err, int* ctr = nullptr);

}  // namespace bem
