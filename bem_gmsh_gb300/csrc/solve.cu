// Solve layer of the C ABI: FP64 GMRES iterative refinement around the FP32
// tensor-core LU (mixed mode), and the FP64 baseline (cuSOLVER getrf/getrs,
// loaded at run time, used only as the FP64 comparison).
//
// Replaces `solve(dad)` = `applyBC` + `bem_linsolve` (src/Core/Solver.jl:24-64,
// 114-131; src/Core/LinearSolveUtils.jl:44-49) for dense systems.
#include <dlfcn.h>
#include <mutex>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/bem_gb300.h"
#include "bem_abi_internal.h"
#include "bem_lu.h"

namespace {

// ---------------------------------------------------------------------------
// cuSOLVER (FP64 comparison path), resolved with dlopen so that the library
// has no link-time dependency on it.
// ---------------------------------------------------------------------------
struct Cusolver {
  using Create = int (*)(void**);
  using Destroy = int (*)(void*);
  using SetStream = int (*)(void*, cudaStream_t);
  using BufSize = int (*)(void*, int, int, double*, int, int*);
  using Getrf = int (*)(void*, int, int, double*, int, double*, int*, int*);
  using Getrs = int (*)(void*, int, int, int, const double*, int, const int*, double*, int, int*);
  void* so = nullptr;
  bool loaded = false;
  Create create = nullptr;
  Destroy destroy = nullptr;
  SetStream set_stream = nullptr;
  BufSize bufsize = nullptr;
  Getrf getrf = nullptr;
  Getrs getrs = nullptr;
  bool ok() const { return loaded; }
};

// cuSOLVER entry points, resolved once per process (thread-safe); each
// context creates its own handle (handles are not shared across threads)
Cusolver* cusolver() {
  static Cusolver cs;
  static std::once_flag once;
  std::call_once(once, [] {
    const char* names[] = {"libcusolver.so.12", "libcusolver.so.13", "libcusolver.so",
                           "/usr/local/cuda/lib64/libcusolver.so.12", "/usr/local/cuda/lib64/libcusolver.so"};
    for (const char* n : names) {
      cs.so = dlopen(n, RTLD_NOW | RTLD_LOCAL);
      if (cs.so) break;
    }
    if (!cs.so) return;
    cs.create = (Cusolver::Create)dlsym(cs.so, "cusolverDnCreate");
    cs.destroy = (Cusolver::Destroy)dlsym(cs.so, "cusolverDnDestroy");
    cs.set_stream = (Cusolver::SetStream)dlsym(cs.so, "cusolverDnSetStream");
    cs.bufsize = (Cusolver::BufSize)dlsym(cs.so, "cusolverDnDgetrf_bufferSize");
    cs.getrf = (Cusolver::Getrf)dlsym(cs.so, "cusolverDnDgetrf");
    cs.getrs = (Cusolver::Getrs)dlsym(cs.so, "cusolverDnDgetrs");
    cs.loaded = cs.create && cs.destroy && cs.set_stream && cs.bufsize && cs.getrf && cs.getrs;
  });
  return cs.ok() ? &cs : nullptr;
}

struct Timer {
  cudaEvent_t a = nullptr, b = nullptr;
  bool own = true;
  Timer() {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
  }
  // borrows the context's timing events 2i, 2i+1 (no create/destroy per call)
  Timer(bem_ctx* c, int i) {
    a = c->timing_event(2 * i);
    b = c->timing_event(2 * i + 1);
    own = !a || !b;
    if (own) {
      cudaEventCreate(&a);
      cudaEventCreate(&b);
    }
  }
  ~Timer() {
    if (!own) return;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
  void start(cudaStream_t s) { cudaEventRecord(a, s); }
  void stop(cudaStream_t s) { cudaEventRecord(b, s); }
  double ms() {
    float v = 0.f;
    cudaEventSynchronize(b);
    cudaEventElapsedTime(&v, a, b);
    return v;
  }
};

// <v, w> on the device, read back through the pinned word `hpin`
double dev_dot(bem_ctx* c, const double* v, const double* w, int N, double* hbuf, double* hpin) {
  bem::dots64(v, N, N, 1, w, hbuf, c->stream);
  cudaMemcpyAsync(hpin, hbuf, sizeof(double), cudaMemcpyDeviceToHost, c->stream);
  cudaStreamSynchronize(c->stream);
  return *hpin;
}

// Pinned host words of one solve: the Gram-Schmidt coefficients (64), the
// least-squares solution (32), a dot product, the LU status words.
struct SolvePin {
  double* hh;
  double* y;
  double* dot;
  int* info;  // 4 ints
};
bool solve_pin(bem_ctx* c, SolvePin& p) {
  char* b = c->pinned(1024);
  if (!b) return false;
  double* d = (double*)b;
  p.hh = d;
  p.y = d + 64;
  p.dot = d + 96;
  p.info = (int*)(d + 100);
  return true;
}

}  // namespace

void bem_release_solver(bem_ctx* c) {
  Cusolver* cs = cusolver();
  if (cs && c->cusolver_handle) cs->destroy(c->cusolver_handle);
  c->cusolver_handle = nullptr;
}

// ---------------------------------------------------------------------------
// mixed precision: FP32 LU (3xTF32 updates) preconditioning FP64 FGMRES
// ---------------------------------------------------------------------------
// A64, b, x: device FP64 (x is output).  A64 is not modified.
int bem_solve_mixed_dev(bem_ctx* c, int N, const double* A64, int64_t lda, const double* b,
                        double tol, int max_iter, int x3, double* x, bem_solve_stats* stats) {
  const int Npad = (N + LU_NB - 1) / LU_NB * LU_NB;
  const int K = Npad / LU_NB;
  const int m = 30;  // restart length
  cudaStream_t st = c->stream;
  c->mixed_fail = bem_ctx::MIXED_OK;
  float* A32 = (float*)c->get(bem_ctx::SLOT_LU0, sizeof(float) * (size_t)Npad * Npad);
  double* cs = (double*)c->get(bem_ctx::SLOT_LU1, sizeof(double) * (size_t)N);
  float* Dinv = (float*)c->get(bem_ctx::SLOT_LU2, sizeof(float) * bem::lu_dinv_floats(K));
  double* V = (double*)c->get(bem_ctx::SLOT_LU3, sizeof(double) * (size_t)N * (m + 1));
  double* Z = (double*)c->get(bem_ctx::SLOT_LU4, sizeof(double) * (size_t)N * m);
  double* w = (double*)c->get(bem_ctx::SLOT_LU5, sizeof(double) * ((size_t)N + 64));
  float* rf = (float*)c->get(bem_ctx::SLOT_LU6, sizeof(float) * (3 * (size_t)Npad + 64) +
                                                   sizeof(unsigned long long) * bem::lu_tag_words(Npad));
  int* info = (int*)c->get(bem_ctx::SLOT_LU7, 256);
  float* Mc = (float*)c->get(bem_ctx::SLOT_LU8, sizeof(float) * (size_t)K * 2 * LU_NB * LU_NB);
  if (!A32 || !cs || !Dinv || !V || !Z || !w || !rf || !info || !Mc) return BEM_ERR_NOMEM;
  double* hbuf = w + N;  // 64 doubles of scratch
  float* tmpf = rf + Npad;
  float* outf = rf + 2 * (size_t)Npad;
  // (epoch, value) words of the triangular sweeps; zeroed once per solve,
  // every preconditioner application uses the next epoch
  unsigned long long* tags = (unsigned long long*)(rf + 3 * (size_t)Npad + 64);
  cudaMemsetAsync(tags, 0, sizeof(unsigned long long) * bem::lu_tag_words(Npad), c->stream);
  int epoch = 0;
  int* werr = info + 1;
  SolvePin pin;
  if (!solve_pin(c, pin)) return BEM_ERR_NOMEM;
  Timer tf(c, 1), tr(c, 2);
  bem::TcPlan tcp[2];
  const bool use_tc = c->opt_tcgen05 && x3 && c->lookahead_ready(K);
  if (use_tc) {
    for (int h = 0; h < 2; ++h) {
      float* Lt = (float*)c->get(bem_ctx::SLOT_TC0 + 3 * h, sizeof(float) * (size_t)Npad * LU_NB);
      float* Ltlo = (float*)c->get(bem_ctx::SLOT_TC1 + 3 * h, sizeof(float) * (size_t)Npad * LU_NB);
      float* Ulo = (float*)c->get(bem_ctx::SLOT_TC2 + 3 * h, sizeof(float) * (size_t)Npad * LU_NB);
      if (!Lt || !Ltlo || !Ulo) return BEM_ERR_NOMEM;
      bem::tc_plan(tcp[h], A32, Npad, Npad, Lt, Ltlo, Ulo, c->opt_tcgen05, c->opt_tc_reserve);
    }
  }
  const bool lookahead = use_tc && tcp[0].ok && tcp[1].ok;
  // the whole factorization as one launch sequence (equilibration, LU, block
  // inverses, sweep couplings)
  // info[16], info[17]: tile counter of the persistent bulk updates
  auto factor = [&]() -> int {
    cudaMemsetAsync(info, 0, 2 * sizeof(int), st);
    cudaMemsetAsync(info + 16, 0, 2 * sizeof(int), st);
    bem::lu_prepare(A64, lda, N, Npad, cs, A32, Npad, st);
    int r;
    if (lookahead)
      r = bem::lu_factor_lookahead(A32, Npad, Npad, Dinv, info, st, c->la_stream, c->fork_event,
                                   c->events.data(), c->events.data() + K, c->thin_stream,
                                   c->events.data() + 2 * K, tcp, werr, info + 16);
    else
      r = bem::lu_factor(A32, Npad, Npad, Dinv, info, x3, st, nullptr, werr);
    if (r) return r;
    bem::lu_couplings(A32, Npad, Npad, Dinv, Mc, st);
    return 0;
  };
  // A CUDA graph of that sequence (three streams, ~8 launches per LU step)
  // replaces its launches from the second call with the same buffers on:
  // the replay removes the host launch gaps between dependent kernels of
  // the critical chain.  Its kernel arguments (tensor maps included) are
  // fixed at capture, hence the key.
  const std::vector<const void*> key = {A64, (const void*)(intptr_t)lda, (const void*)(intptr_t)N, A32, cs, Dinv,
                                        Mc, info, tcp[0].Lt, tcp[0].Ltlo, tcp[0].Ulo, tcp[1].Lt, tcp[1].Ltlo,
                                        tcp[1].Ulo, st, (const void*)(intptr_t)lookahead,
                                        (const void*)(intptr_t)tcp[0].variant, (const void*)(intptr_t)tcp[0].grid};
  const bool graphs = c->opt_graphs && lookahead && !c->prof.on;
  if (graphs && c->lu_graph_key != key) {
    if (c->lu_graph) cudaGraphExecDestroy(c->lu_graph);
    c->lu_graph = nullptr;
    c->lu_graph_key = key;
    c->lu_graph_calls = 0;
  }
  ++c->lu_graph_calls;
  int rc = 0;
  if (graphs && !c->lu_graph && c->lu_graph_calls >= 2) {
    const long long l0 = bem::tl_launches;
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (ce == cudaSuccess) {
      rc = factor();
      ce = cudaStreamEndCapture(st, &g);
    }
    if (ce == cudaSuccess && rc == 0 && g) ce = cudaGraphInstantiate(&c->lu_graph, g, 0);
    if (g) cudaGraphDestroy(g);
    if (ce != cudaSuccess || rc != 0) {
      // capture is an optimisation: fall back to direct launches
      c->lu_graph = nullptr;
      c->opt_graphs = 0;
      cudaGetLastError();
      rc = 0;
    }
    c->lu_graph_launches = bem::tl_launches - l0;
    bem::g_launches.fetch_sub(c->lu_graph_launches);  // counted when replayed
    bem::tl_launches = l0;
  }
  tf.start(st);
  if (graphs && c->lu_graph) {
    cudaError_t ce = cudaGraphLaunch(c->lu_graph, st);
    if (ce != cudaSuccess) return c->cuda_fail(ce, "factorization graph");
    bem::count_launches(c->lu_graph_launches);
  } else {
    rc = factor();
  }
  if (rc) return c->cuda_fail((cudaError_t)rc, "lu_factor");
  tf.stop(st);
  int* hinfo2 = pin.info;
  cudaMemcpyAsync(hinfo2, info, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return c->cuda_fail(e, "factor");
  if (stats) stats->t_factor_ms = tf.ms();
  const int hinfo = hinfo2[0];
  if (hinfo2[1]) {
    c->last_error = "tensor-core GEMM wait timed out in the LU";
    return BEM_ERR_INTERNAL;
  }
  if (hinfo != 0) {
    c->last_error = "vanishing pivot in block " + std::to_string(hinfo - 1) + " of the LU";
    c->mixed_fail = bem_ctx::MIXED_PIVOT;
    if (stats) stats->status = BEM_ERR_NOT_CONVERGED;
    return BEM_ERR_NOT_CONVERGED;
  }
  int prc = 0;
  auto precond = [&](const double* v, double* z) {
    bem::to_f32(v, N, Npad, rf, st);
    int e2 = bem::lu_solve_vec(A32, Npad, Npad, Dinv, Mc, rf, tmpf, outf, tags, ++epoch, werr, st,
                               c->opt_wait_limit, (c->opt_inject & 2) ? 1 : 0, c->opt_sweep_ctas);
    if (e2) prc = e2;
    bem::from_f32_scale(outf, cs, N, z, st);
  };
  tr.start(st);
  cudaMemsetAsync(x, 0, sizeof(double) * N, st);
  const double bnorm = std::sqrt(dev_dot(c, b, b, N, hbuf, pin.dot));
  if (!(bnorm > 0)) {
    tr.stop(st);
    if (stats) { stats->iterations = 0; stats->rel_residual = 0; stats->status = BEM_OK; stats->t_refine_ms = tr.ms(); }
    return BEM_OK;
  }
  int iters = 0;
  double relres = 1.0;
  std::vector<double> H((m + 1) * m), cg(m), sg(m), gvec(m + 1), y(m);
  bool converged = false;
  double prev_beta = INFINITY;
  bool x_zero = true;  // x was just zeroed: the first residual is b itself
  while (iters < max_iter && !converged) {
    // r = b - A x (FP64)
    if (x_zero)
      cudaMemcpyAsync(w, b, sizeof(double) * N, cudaMemcpyDeviceToDevice, st);
    else
      bem::residual64(A64, lda, N, x, b, w, st);
    x_zero = false;
    double beta = std::sqrt(dev_dot(c, w, w, N, hbuf, pin.dot));
    relres = beta / bnorm;
    if (relres <= tol) { converged = true; break; }
    if (beta > 0.5 * prev_beta) {
      // a restart cycle that no longer halves the true residual.  Below 1e-10
      // this is the FP64 rounding floor of the matrix (about eps |A| |x| / |b|;
      // a tol below it cannot be reached): x is then backward stable, as
      // accurate as FP64 allows -- what the reference's LU returns -- and
      // counts as converged (stats report the residual reached).
      if (relres < 1e-10) { converged = true; break; }
      // far above that floor the same stall means the unpivoted FP32 factors
      // are no preconditioner for this matrix (pivot growth)
      c->mixed_fail = bem_ctx::MIXED_STAGNATION;
      break;
    }
    prev_beta = beta;
    bem::scale_copy64(w, 1.0 / beta, V, N, st);
    std::fill(gvec.begin(), gvec.end(), 0.0);
    gvec[0] = beta;
    int j = 0;
    for (; j < m && iters < max_iter; ++j) {
      ++iters;
      double* zj = Z + (size_t)j * N;
      precond(V + (size_t)j * N, zj);
      bem::gemv64(A64, lda, N, zj, w, st);
      // classical Gram-Schmidt, two passes, and the normalization, all on
      // the device (pass p's coefficients in hbuf[32 p ..], the squared
      // norm in hbuf[62]); one copy brings them to the host
      for (int pass = 0; pass < 2; ++pass) {
        bem::dots64(V, N, N, j + 1, w, hbuf + 32 * pass, st);
        bem::sub_vh64(V, N, N, j + 1, hbuf + 32 * pass, w, st);
      }
      bem::dots64(w, N, N, 1, w, hbuf + 62, st);
      bem::scale_by_norm64(w, hbuf + 62, V + (size_t)(j + 1) * N, N, st);
      const double* hh = pin.hh;
      cudaMemcpyAsync(pin.hh, hbuf, sizeof(double) * 64, cudaMemcpyDeviceToHost, st);
      cudaStreamSynchronize(st);
      std::vector<double> h(j + 2, 0.0);
      for (int q = 0; q <= j; ++q) h[q] = hh[q] + hh[32 + q];
      const double hn = hh[62] > 0.0 ? std::sqrt(hh[62]) : 0.0;
      h[j + 1] = hn;
      // Givens
      for (int q = 0; q < j; ++q) {
        double t = cg[q] * h[q] + sg[q] * h[q + 1];
        h[q + 1] = -sg[q] * h[q] + cg[q] * h[q + 1];
        h[q] = t;
      }
      double den = std::hypot(h[j], h[j + 1]);
      cg[j] = den > 0 ? h[j] / den : 1.0;
      sg[j] = den > 0 ? h[j + 1] / den : 0.0;
      h[j] = den;
      h[j + 1] = 0.0;
      gvec[j + 1] = -sg[j] * gvec[j];
      gvec[j] = cg[j] * gvec[j];
      for (int q = 0; q <= j; ++q) H[q + (size_t)j * (m + 1)] = h[q];
      if (std::fabs(gvec[j + 1]) / bnorm <= 0.1 * tol || hn == 0.0) { ++j; break; }
    }
    // y = R^{-1} g, x += Z y
    for (int q = j - 1; q >= 0; --q) {
      double s = gvec[q];
      for (int p = q + 1; p < j; ++p) s -= H[q + (size_t)p * (m + 1)] * y[p];
      y[q] = s / H[q + (size_t)q * (m + 1)];
    }
    std::memcpy(pin.y, y.data(), sizeof(double) * j);
    cudaMemcpyAsync(hbuf, pin.y, sizeof(double) * j, cudaMemcpyHostToDevice, st);
    bem::add_zy64(Z, N, N, j, hbuf, x, st);
  }
  if (!converged) {
    bem::residual64(A64, lda, N, x, b, w, st);
    relres = std::sqrt(dev_dot(c, w, w, N, hbuf, pin.dot)) / bnorm;
    converged = relres <= tol;
  }
  tr.stop(st);
  cudaMemcpyAsync(pin.info + 2, werr, sizeof(int), cudaMemcpyDeviceToHost, st);
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return c->cuda_fail(e, "refinement");
  if (prc) return c->cuda_fail((cudaError_t)prc, "triangular solve launch");
  const int herr = pin.info[2];
  if (herr) {
    c->last_error = "triangular-solve wait timed out";
    return BEM_ERR_INTERNAL;
  }
  if (stats) {
    stats->iterations = iters;
    stats->rel_residual = relres;
    stats->status = converged ? BEM_OK : BEM_ERR_NOT_CONVERGED;
    stats->t_refine_ms = tr.ms();
  }
  if (!converged) {
    if (c->mixed_fail == bem_ctx::MIXED_STAGNATION) {
      c->last_error = "GMRES refinement stagnated (the unpivoted LU is no preconditioner for this matrix)";
    } else {
      c->mixed_fail = bem_ctx::MIXED_CAP;
      c->last_error = "GMRES refinement reached its iteration cap";
    }
    return BEM_ERR_NOT_CONVERGED;
  }
  return BEM_OK;
}

// FP64 baseline: LU with partial pivoting (cuSOLVER), A64 overwritten.
int bem_solve_fp64_dev(bem_ctx* c, int N, double* A64, int64_t lda, const double* b, double* x,
                       bem_solve_stats* stats) {
  Cusolver* cs = cusolver();
  if (cs && !c->cusolver_handle) {
    void* h = nullptr;
    if (cs->create(&h) == 0) c->cusolver_handle = h;
  }
  if (!cs || !c->cusolver_handle) {
    c->last_error = "cuSOLVER could not be loaded for the FP64 comparison path";
    return BEM_ERR_UNSUPPORTED;
  }
  cudaStream_t st = c->stream;
  cs->set_stream(c->cusolver_handle, st);
  int lwork = 0;
  if (cs->bufsize(c->cusolver_handle, N, N, A64, (int)lda, &lwork) != 0) return BEM_ERR_CUDA;
  double* work = (double*)c->get(bem_ctx::SLOT_LU3, sizeof(double) * ((size_t)lwork + 16));
  int* ipiv = (int*)c->get(bem_ctx::SLOT_LU4, sizeof(int) * ((size_t)N + 16));
  int* info = (int*)c->get(bem_ctx::SLOT_LU7, 256);
  if (!work || !ipiv || !info) return BEM_ERR_NOMEM;
  SolvePin pin;
  if (!solve_pin(c, pin)) return BEM_ERR_NOMEM;
  Timer tf(c, 1), tr(c, 2);
  tf.start(st);
  if (cs->getrf(c->cusolver_handle, N, N, A64, (int)lda, work, ipiv, info) != 0) return BEM_ERR_CUDA;
  tf.stop(st);
  tr.start(st);
  cudaMemcpyAsync(x, b, sizeof(double) * N, cudaMemcpyDeviceToDevice, st);
  if (cs->getrs(c->cusolver_handle, 0, N, 1, A64, (int)lda, ipiv, x, N, info + 1) != 0) return BEM_ERR_CUDA;
  tr.stop(st);
  const int* hi = pin.info;
  cudaMemcpyAsync(pin.info, info, 2 * sizeof(int), cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return c->cuda_fail(e, "cuSOLVER getrf/getrs");
  if (stats) {
    stats->iterations = 0;
    stats->rel_residual = NAN;
    stats->status = (hi[0] == 0 && hi[1] == 0) ? BEM_OK : BEM_ERR_NOT_CONVERGED;
    stats->t_factor_ms = tf.ms();
    stats->t_refine_ms = tr.ms();
  }
  if (hi[0] != 0) {
    c->last_error = "singular matrix (getrf info " + std::to_string(hi[0]) + ")";
    return BEM_ERR_NOT_CONVERGED;
  }
  return BEM_OK;
}

// The mixed solve with its pivoting safety net (BEM_OPT_PIVOT_FALLBACK).
// The reference factors with partial pivoting (LAPACK getrf behind
// `bem_linsolve`, src/Core/LinearSolveUtils.jl:44-49); the FP32 LU here does
// not pivot, which BEM collocation systems (column-equilibrated) never need
// but an arbitrary matrix can.  When that LU meets a vanishing pivot, or the
// refinement stagnates far above the FP64 rounding floor, the system is
// solved again by LU with partial pivoting in FP64.  A64 is factored in
// place when `a_scratch` (the caller's copy), otherwise a copy is.
int bem_solve_mixed_safe(bem_ctx* c, int N, double* A64, int64_t lda, bool a_scratch, const double* b,
                         double tol, int max_iter, double* x, bem_solve_stats* stats) {
  int rc = bem_solve_mixed_dev(c, N, A64, lda, b, tol, max_iter, 1, x, stats);
  if (rc != BEM_ERR_NOT_CONVERGED || !c->opt_pivot_fallback) return rc;
  if (c->mixed_fail != bem_ctx::MIXED_PIVOT && c->mixed_fail != bem_ctx::MIXED_STAGNATION) return rc;
  double* Af = A64;
  int64_t ldf = lda;
  if (!a_scratch) {
    Af = (double*)c->get(bem_ctx::SLOT_OUT2, sizeof(double) * (size_t)N * N);
    if (!Af) return BEM_ERR_NOMEM;
    cudaMemcpy2DAsync(Af, sizeof(double) * N, A64, sizeof(double) * lda, sizeof(double) * N, N,
                      cudaMemcpyDeviceToDevice, c->stream);
    ldf = N;
  }
  bem_solve_stats st2{};
  int rc2 = bem_solve_fp64_dev(c, N, Af, ldf, b, x, &st2);
  if (stats) {
    stats->pivoted = 1;
    stats->status = st2.status;
    stats->rel_residual = NAN;
    stats->t_factor_ms += st2.t_factor_ms;
    stats->t_refine_ms += st2.t_refine_ms;
  }
  return rc2;
}

extern "C" int bem_solve_system(bem_ctx* c, int64_t n, const double* A, int64_t lda, const double* b,
                                int mode, double tol, int max_iter, int mem, double* x,
                                bem_solve_stats* stats) {
  if (!c || !A || !b || !x || n <= 0 || lda < n || n >= (1 << 30)) return BEM_ERR_INVALID;
  if (mode != BEM_SOLVE_FP64 && mode != BEM_SOLVE_MIXED) return BEM_ERR_INVALID;
  if (mem != BEM_MEM_HOST && mem != BEM_MEM_DEVICE) return BEM_ERR_INVALID;
  if (!(tol > 0) || max_iter < 1) return BEM_ERR_INVALID;
  CallScope cscope(c);
  cudaSetDevice(c->device);
  const int N = (int)n;
  if (stats) std::memset(stats, 0, sizeof(*stats));
  const double* dA = A;
  const double* db = b;
  double* dx = x;
  double* Acopy = nullptr;
  if (mem == BEM_MEM_HOST || mode == BEM_SOLVE_FP64) {
    // FP64 overwrites its matrix; host inputs need device copies anyway
    Acopy = (double*)c->get(bem_ctx::SLOT_OUT2, sizeof(double) * (size_t)N * N);
    if (!Acopy) return BEM_ERR_NOMEM;
    cudaMemcpy2DAsync(Acopy, sizeof(double) * N, A, sizeof(double) * lda, sizeof(double) * N, N,
                      mem == BEM_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                      c->stream);
    dA = Acopy;
  }
  const int64_t ldd = Acopy ? N : lda;
  if (mem == BEM_MEM_HOST) {
    double* tmp = (double*)c->get(bem_ctx::SLOT_OUT3, sizeof(double) * 2 * (size_t)N);
    if (!tmp) return BEM_ERR_NOMEM;
    cudaMemcpyAsync(tmp, b, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream);
    db = tmp;
    dx = tmp + N;
  }
  int rc = mode == BEM_SOLVE_MIXED
               ? bem_solve_mixed_safe(c, N, (double*)dA, ldd, Acopy != nullptr, db, tol, max_iter, dx, stats)
               : bem_solve_fp64_dev(c, N, (double*)dA, ldd, db, dx, stats);
  if (rc != BEM_OK && rc != BEM_ERR_NOT_CONVERGED) return rc;
  if (mem == BEM_MEM_HOST) {
    cudaMemcpyAsync(x, dx, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "copy x to host");
  }
  return rc;
}

extern "C" int bem_solve2d(bem_ctx* c, const bem_geom2d* g, int kind, double prm0, double prm1,
                           const int32_t* BC, const double* BV, int npg, double near_factor,
                           int mode, double tol, int max_iter, int mem, double* x,
                           bem_solve_stats* stats) {
  if (!c || !g || !BC || !BV || !x) return BEM_ERR_INVALID;
  if (kind != 0 && kind != 1) return BEM_ERR_INVALID;
  if (mode != BEM_SOLVE_FP64 && mode != BEM_SOLVE_MIXED) return BEM_ERR_INVALID;
  if (mem != BEM_MEM_HOST && mem != BEM_MEM_DEVICE) return BEM_ERR_INVALID;
  if (!(tol > 0) || max_iter < 1) return BEM_ERR_INVALID;
  CallScope cscope(c);
  bem::Physics ph{};
  ph.kind = kind;
  if (kind == 0) {
    if (!(prm0 > 0)) return BEM_ERR_INVALID;
    ph.k = prm0;
  } else {
    if (!(prm0 > 0) || !(prm1 < 0.5) || !(prm1 > -1.0)) return BEM_ERR_INVALID;
    ph.mu = prm0;
    ph.nu = prm1;
  }
  int rc = bem_check_geom(g, npg, near_factor);
  if (rc) return rc;
  cudaSetDevice(c->device);
  if (stats) std::memset(stats, 0, sizeof(*stats));
  const int dof = kind == 0 ? 1 : 2;
  const int N = dof * g->nt;
  const int64_t ld = (N + 3) / 4 * 4;
  double* A = (double*)c->get(bem_ctx::SLOT_OUT0, sizeof(double) * (size_t)ld * N);
  double* bx = (double*)c->get(bem_ctx::SLOT_OUT1, sizeof(double) * 2 * (size_t)N);
  if (!A || !bx) return BEM_ERR_NOMEM;
  double* b = bx;
  double* dx = mem == BEM_MEM_DEVICE ? x : bx + N;
  Timer ta(c, 0);
  ta.start(c->stream);
  // the FP64 comparison path keeps FP64 arithmetic throughout
  const int prec = (mode == BEM_SOLVE_MIXED && c->opt_far_df >= 1) ? 3 : 1;
  rc = bem_assemble_system_dev(c, g, ph, BC, BV, npg, near_factor, mem, prec, A, ld, nullptr, b);
  ta.stop(c->stream);
  if (rc) return rc;
  double t_asm = ta.ms();
  rc = mode == BEM_SOLVE_MIXED ? bem_solve_mixed_safe(c, N, A, ld, true, b, tol, max_iter, dx, stats)
                               : bem_solve_fp64_dev(c, N, A, ld, b, dx, stats);
  if (stats) stats->t_assemble_ms = t_asm;
  if (rc != BEM_OK && rc != BEM_ERR_NOT_CONVERGED) return rc;
  if (mem == BEM_MEM_HOST) {
    double* hx = (double*)c->pinned(sizeof(double) * (size_t)N);
    if (!hx) return BEM_ERR_NOMEM;
    cudaMemcpyAsync(hx, dx, sizeof(double) * N, cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "copy x to host");
    std::memcpy(x, hx, sizeof(double) * N);
  }
  return rc;
}

// ---------------------------------------------------------------------------
// options and self-test
// ---------------------------------------------------------------------------
extern "C" int bem_ctx_set_option(bem_ctx* c, int option, int value) {
  if (!c) return BEM_ERR_INVALID;
  if (option == BEM_OPT_TCGEN05) {
    if (value < 0 || value > 2) return BEM_ERR_INVALID;
    c->opt_tcgen05 = value;
    return BEM_OK;
  }
  if (option == BEM_OPT_TC_RESERVE) {
    if (value < 0 || value > 64) return BEM_ERR_INVALID;
    c->opt_tc_reserve = value;
    return BEM_OK;
  }
  if (option == BEM_OPT_KERNEL_TIMING) {
    c->prof.on = value != 0;
    return BEM_OK;
  }
  if (option == BEM_OPT_FAR_DF) {
    if (value < 0 || value > 2) return BEM_ERR_INVALID;
    c->opt_far_df = value;
    return BEM_OK;
  }
  if (option == BEM_OPT_GRAPHS) {
    c->opt_graphs = value ? 1 : 0;
    return BEM_OK;
  }
  if (option == BEM_OPT_PIVOT_FALLBACK) {
    c->opt_pivot_fallback = value ? 1 : 0;
    return BEM_OK;
  }
  if (option == BEM_OPT_WAIT_LIMIT) {
    if (value < 1) return BEM_ERR_INVALID;
    c->opt_wait_limit = value;
    return BEM_OK;
  }
  if (option == BEM_OPT_NEARFIELD) {
    if (value < 0 || value > 6) return BEM_ERR_INVALID;
    c->opt_nearfield = value;
    return BEM_OK;
  }
  if (option == BEM_OPT_SWEEP_CTAS) {
    if (value < 1 || value > bem::LU_TRSV_PMAX) return BEM_ERR_INVALID;
    c->opt_sweep_ctas = value;
    return BEM_OK;
  }
  if (option == BEM_OPT_SINGULAR) {
    if (value != 0 && value != 1) return BEM_ERR_INVALID;
    c->opt_singular = value;
    return BEM_OK;
  }
  if (option == BEM_OPT_INJECT) {
    if (value < 0 || value > 3) return BEM_ERR_INVALID;
    c->opt_inject = value;
    return BEM_OK;
  }
  return BEM_ERR_INVALID;
}

namespace {
__global__ void k_fill_test(float* A, int n, int64_t ld, uint32_t seed) {
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < (int64_t)n * n;
       idx += (int64_t)gridDim.x * blockDim.x) {
    int i = (int)(idx % n), j = (int)(idx / n);
    uint32_t h = (uint32_t)idx * 2654435761u ^ seed;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    float v = ((h & 0xFFFFFF) / 16777216.0f - 0.5f) / sqrtf((float)n);
    if (i == j) v += 2.0f;
    A[i + (size_t)j * ld] = v;
  }
}
__global__ void k_maxdiff(const float* A, const float* B, int64_t cnt, float* out) {
  float m = 0.f, a = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x) {
    m = fmaxf(m, fabsf(A[i] - B[i]));
    a = fmaxf(a, fabsf(B[i]));
  }
  for (int o = 16; o > 0; o >>= 1) {
    m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    a = fmaxf(a, __shfl_xor_sync(0xffffffffu, a, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax((int*)out, __float_as_int(m));
    atomicMax((int*)out + 1, __float_as_int(a));
  }
}
}  // namespace

// which = 1: LU of an n x n test matrix with the tcgen05 trailing updates and
// with the legacy mma.sync ones; out[0] = max |difference of the factors|,
// out[1] = max |factor|, out[2] / out[3] = factor times (ms) tcgen05 / legacy.
extern "C" int bem_selftest(bem_ctx* c, int which, int n, double* out) {
  if (!c || !out || which < 1 || which > 4 || n < LU_NB || n % LU_NB != 0 || n > 16384)
    return BEM_ERR_INVALID;
  if ((which == 3 || which == 4) && n < 2 * LU_NB) return BEM_ERR_INVALID;
  cudaSetDevice(c->device);
  cudaStream_t st = c->stream;
  if (which == 3) {
    // the bulk trailing update of LU step 0 alone: C (n-128)^2 -= L21 U12,
    // repeated; nothing else runs on the device meanwhile
    float* A1 = (float*)c->get(bem_ctx::SLOT_TEST0, sizeof(float) * (size_t)n * n);
    float* Lt = (float*)c->get(bem_ctx::SLOT_TC0, sizeof(float) * (size_t)n * LU_NB);
    float* Ltlo = (float*)c->get(bem_ctx::SLOT_TC1, sizeof(float) * (size_t)n * LU_NB);
    float* Ulo = (float*)c->get(bem_ctx::SLOT_TC2, sizeof(float) * (size_t)n * LU_NB);
    int* info = (int*)c->get(bem_ctx::SLOT_LU7, 256);
    if (!A1 || !Lt || !Ltlo || !Ulo || !info) return BEM_ERR_NOMEM;
    bem::TcPlan tcp;
    if (!bem::tc_plan(tcp, A1, n, n, Lt, Ltlo, Ulo, c->opt_tcgen05, c->opt_tc_reserve)) {
      c->last_error = "tensor map encoding failed";
      return BEM_ERR_UNSUPPORTED;
    }
    k_fill_test<<<1024, 256, 0, st>>>(A1, n, n, 4242u);
    cudaMemsetAsync(info, 0, 16, st);
    cudaMemsetAsync(info + 16, 0, 8, st);
    bem::tc_split(tcp, 0, st);
    const int rem = n - LU_NB, reps = 20;
    for (int i = 0; i < 3; ++i) bem::tc_gemm_sub(tcp, 0, 0, 0, rem, rem, info + 1, st, info + 16);
    Timer t;
    t.start(st);
    for (int i = 0; i < reps; ++i) bem::tc_gemm_sub(tcp, 0, 0, 0, rem, rem, info + 1, st, info + 16);
    t.stop(st);
    int herr = 0;
    cudaMemcpyAsync(&herr, info + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return c->cuda_fail(e, "selftest gemm");
    if (herr) {
      c->last_error = "bulk update reported a barrier timeout";
      return BEM_ERR_CUDA;
    }
    const double ms = t.ms() / reps;
    out[0] = ms;
    out[1] = 8.0 * (double)rem * rem / (ms * 1e-3) / 1e9;
    out[2] = 3.0 * 2.0 * (double)rem * rem * LU_NB / (ms * 1e-3) / 1e12;
    out[3] = 0.0;
    return BEM_OK;
  }
  if (which == 4) {
    // the two bulk-update kernels on the same operands: step 0's update of
    // the whole trailing matrix and, on a second copy, of its part past the
    // first block row and column (the look-ahead's shape); out[0] / out[1] =
    // max |difference| / max |entry| of the two results, out[2] / out[3] =
    // the same for the second shape
    if (c->opt_tcgen05 != 2) return BEM_ERR_INVALID;
    float* A1 = (float*)c->get(bem_ctx::SLOT_TEST0, sizeof(float) * (size_t)n * n);
    float* A2 = (float*)c->get(bem_ctx::SLOT_TEST1, sizeof(float) * (size_t)n * n);
    float* Lt = (float*)c->get(bem_ctx::SLOT_TC0, sizeof(float) * (size_t)n * LU_NB);
    float* Ltlo = (float*)c->get(bem_ctx::SLOT_TC1, sizeof(float) * (size_t)n * LU_NB);
    float* Ulo = (float*)c->get(bem_ctx::SLOT_TC2, sizeof(float) * (size_t)n * LU_NB);
    int* info = (int*)c->get(bem_ctx::SLOT_LU7, 256);
    if (!A1 || !A2 || !Lt || !Ltlo || !Ulo || !info) return BEM_ERR_NOMEM;
    bem::TcPlan p1, p2;
    if (!bem::tc_plan(p1, A1, n, n, Lt, Ltlo, Ulo, 1, 0) ||
        !bem::tc_plan(p2, A2, n, n, Lt, Ltlo, Ulo, 2, c->opt_tc_reserve) || p2.variant != 2) {
      c->last_error = "tensor map encoding failed";
      return BEM_ERR_UNSUPPORTED;
    }
    const int rem = n - LU_NB;
    float* d = (float*)(info + 8);
    float h[4];
    cudaMemsetAsync(info, 0, 16, st);
    cudaMemsetAsync(info + 16, 0, 8, st);
    cudaMemsetAsync(d, 0, 16, st);
    for (int shape = 0; shape < 2; ++shape) {
      const int o = shape ? LU_NB : 0;
      if (rem - o <= 0) break;
      k_fill_test<<<1024, 256, 0, st>>>(A1, n, n, 999u + shape);
      cudaMemcpyAsync(A2, A1, sizeof(float) * (size_t)n * n, cudaMemcpyDeviceToDevice, st);
      bem::tc_split(p1, 0, st);
      bem::tc_gemm_sub(p1, 0, o, o, rem - o, rem - o, info + 1, st);
      bem::tc_gemm_sub(p2, 0, o, o, rem - o, rem - o, info + 1, st, info + 16);
      k_maxdiff<<<512, 256, 0, st>>>(A1, A2, (int64_t)n * n, d + 2 * shape);
    }
    int herr = 0;
    cudaMemcpyAsync(h, d, 16, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&herr, info + 1, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return c->cuda_fail(e, "selftest bulk kernels");
    if (herr) {
      c->last_error = "bulk update reported a barrier timeout";
      return BEM_ERR_CUDA;
    }
    for (int i = 0; i < 4; ++i) out[i] = h[i];
    return BEM_OK;
  }
  if (which == 2) {
    float* A1 = (float*)c->get(bem_ctx::SLOT_TEST0, sizeof(float) * (size_t)n * n);
    float* A2 = (float*)c->get(bem_ctx::SLOT_TEST1, sizeof(float) * (size_t)n * n);
    float* D = (float*)c->get(bem_ctx::SLOT_LU2, sizeof(float) * (4 * LU_NB * LU_NB + LU_SI));
    int* info = (int*)c->get(bem_ctx::SLOT_LU7, 256);
    if (!A1 || !A2 || !D || !info) return BEM_ERR_NOMEM;
    k_fill_test<<<1024, 256, 0, st>>>(A1, n, n, 777u);
    cudaMemcpyAsync(A2, A1, sizeof(float) * (size_t)n * n, cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(info, 0, 16, st);
    bem::diag_selftest(A1, A2, n, D, D + 2 * LU_NB * LU_NB, D + 4 * LU_NB * LU_NB, info, st);
    float* d = (float*)(info + 8);
    float h[6];
    cudaMemsetAsync(d, 0, 24, st);
    k_maxdiff<<<512, 256, 0, st>>>(A1, A2, (int64_t)n * LU_NB, d);  // first block column
    k_maxdiff<<<512, 256, 0, st>>>(D, D + 2 * LU_NB * LU_NB, 2 * LU_NB * LU_NB, d + 2);
    cudaMemcpyAsync(h, d, 16, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return c->cuda_fail(e, "selftest diag");
    out[0] = h[0]; out[1] = h[1]; out[2] = h[2]; out[3] = h[3];
    return BEM_OK;
  }
  const int K = n / LU_NB;
  float* A1 = (float*)c->get(bem_ctx::SLOT_TEST0, sizeof(float) * (size_t)n * n);
  float* A2 = (float*)c->get(bem_ctx::SLOT_TEST1, sizeof(float) * (size_t)n * n);
  float* Dinv = (float*)c->get(bem_ctx::SLOT_LU2, sizeof(float) * bem::lu_dinv_floats(K));
  int* info = (int*)c->get(bem_ctx::SLOT_LU7, 256);
  float* Lt = (float*)c->get(bem_ctx::SLOT_TC0, sizeof(float) * (size_t)n * LU_NB);
  float* Ltlo = (float*)c->get(bem_ctx::SLOT_TC1, sizeof(float) * (size_t)n * LU_NB);
  float* Ulo = (float*)c->get(bem_ctx::SLOT_TC2, sizeof(float) * (size_t)n * LU_NB);
  if (!A1 || !A2 || !Dinv || !info || !Lt || !Ltlo || !Ulo) return BEM_ERR_NOMEM;
  k_fill_test<<<1024, 256, 0, st>>>(A1, n, n, 12345u);
  cudaMemcpyAsync(A2, A1, sizeof(float) * (size_t)n * n, cudaMemcpyDeviceToDevice, st);
  cudaMemsetAsync(info, 0, 16, st);
  bem::TcPlan tcp[2];
  float* Lt2 = (float*)c->get(bem_ctx::SLOT_TC3, sizeof(float) * (size_t)n * LU_NB);
  float* Ltlo2 = (float*)c->get(bem_ctx::SLOT_TC4, sizeof(float) * (size_t)n * LU_NB);
  float* Ulo2 = (float*)c->get(bem_ctx::SLOT_TC5, sizeof(float) * (size_t)n * LU_NB);
  if (!Lt2 || !Ltlo2 || !Ulo2 || !c->lookahead_ready(K)) return BEM_ERR_NOMEM;
  if (!bem::tc_plan(tcp[0], A1, n, n, Lt, Ltlo, Ulo, c->opt_tcgen05, c->opt_tc_reserve) ||
      !bem::tc_plan(tcp[1], A1, n, n, Lt2, Ltlo2, Ulo2, c->opt_tcgen05, c->opt_tc_reserve)) {
    c->last_error = "tensor map encoding failed";
    return BEM_ERR_UNSUPPORTED;
  }
  Timer t1, t2;
  cudaMemsetAsync(info + 16, 0, 8, st);
  t1.start(st);
  int rc = bem::lu_factor_lookahead(A1, n, n, Dinv, info, st, c->la_stream, c->fork_event,
                                    c->events.data(), c->events.data() + K,
                                  c->thin_stream, c->events.data() + 2 * K, tcp, info + 1, info + 16);
  t1.stop(st);
  if (rc) return c->cuda_fail((cudaError_t)rc, "selftest tcgen05 LU");
  t2.start(st);
  rc = bem::lu_factor(A2, n, n, Dinv, info, 1, st, nullptr, nullptr);
  t2.stop(st);
  if (rc) return c->cuda_fail((cudaError_t)rc, "selftest legacy LU");
  float* d = (float*)(info + 8);
  cudaMemsetAsync(d, 0, 8, st);
  k_maxdiff<<<512, 256, 0, st>>>(A1, A2, (int64_t)n * n, d);
  float h[2];
  int hi[2];
  cudaMemcpyAsync(h, d, 8, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(hi, info, 8, cudaMemcpyDeviceToHost, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return c->cuda_fail(e, "selftest");
  out[0] = h[0];
  out[1] = h[1];
  out[2] = t1.ms();
  out[3] = t2.ms();
  if (hi[1]) {
    c->last_error = "tensor-core GEMM wait timed out";
    return BEM_ERR_INTERNAL;
  }
  return BEM_OK;
}
