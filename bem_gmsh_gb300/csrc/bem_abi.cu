// C-ABI layer: context, workspace, argument checks, host<->device staging.
// The entry points are declared (with the reference interfaces they replace)
// in include/bem_gb300.h.
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bem_gb300.h"
#include "bem_abi_internal.h"
#include "bem_crmath.cuh"
#include "bem_kernels.h"

namespace bem {
std::atomic<long long> g_launches{0};
thread_local long long tl_launches = 0;
thread_local KProf* tl_prof = nullptr;
}  // namespace bem

using bem::AsmRequest;
using bem::GeomDev;
using bem::Physics;
using bem::Rules;

// ---------------------------------------------------------------------------
// host-side rule tables
// ---------------------------------------------------------------------------
namespace {

// Gauss-Legendre nodes (ascending) and weights, correctly rounded (Newton in
// double-double arithmetic, bem_crmath.cuh): the tanp3c map amplifies a
// one-ulp change of a node, so every implementation of the assembly must use
// the same bits, and correct rounding is the one platform-independent choice.
void gauss_legendre(int n, double* x, double* w) { bem::crm::gauss_legendre_cr(n, x, w); }

// differentiation matrix of a barycentric basis (Interpolation.jl:193-213)
void diff_matrix(const double* x, const double* bw, int n, double* D) {
  for (int i = 0; i < n; ++i) {
    double s = 0.0;
    for (int j = 0; j < n; ++j) {
      if (j == i) continue;
      double t = (bw[j] / bw[i]) / (x[i] - x[j]);
      D[i * n + j] = t;
      s += t;
    }
    D[i * n + i] = -s;
  }
}

void build_rules(const bem_geom2d* g, int npg, const double* ew_host, Rules& R) {
  std::memset(&R, 0, sizeof(R));
  const int nn = g->p + 1;
  R.nn = nn;
  R.ngeo = g->ngeo;
  R.npg = npg;
  // Legendre(p): Gauss nodes, weights (2 isodd(i) - 1) sqrt((1 - x^2) w)
  double x[64], w[64];
  gauss_legendre(nn, x, w);
  for (int i = 0; i < nn; ++i) {
    R.leg_x[i] = x[i];
    R.leg_bw[i] = ((i % 2) == 0 ? 1.0 : -1.0) * std::sqrt((1 - x[i] * x[i]) * w[i]);
  }
  diff_matrix(R.leg_x, R.leg_bw, nn, R.leg_D);
  // Equispaced(ngeo-1): nodes (2j-N)/N, weights (-1)^(j+N) binomial(N, j)
  if (g->ngeo > 0) {
    const int N = g->ngeo - 1;
    double binom = 1.0;
    for (int j = 0; j <= N; ++j) {
      if (j > 0) binom = std::round(binom * (N - j + 1) / j);
      R.geo_x[j] = N == 0 ? 0.0 : (double)(2 * j - N) / (double)N;
      bool pos = ((N % 2) == 1) != ((j % 2) == 0);
      R.geo_bw[j] = (pos ? 1.0 : -1.0) * binom;
    }
    diff_matrix(R.geo_x, R.geo_bw, g->ngeo, R.geo_D);
  }
  gauss_legendre(npg, R.qsi, R.w);
  gauss_legendre(BEM_NINTERP, R.gi_x, R.gi_w);
  for (int i = 0; i < BEM_NINTERP; ++i) {
    double b = 1.0;
    for (int j = 0; j < BEM_NINTERP; ++j)
      if (j != i) b *= R.gi_x[i] - R.gi_x[j];
    R.gi_bw[i] = 1.0 / b;
  }
  for (int k = 0; k < nn; ++k) R.ew[k] = ew_host[k];
  auto product_weights = [](const double* xs, int n, double* pw) {
    for (int i = 0; i < n; ++i) {
      long double b = 1.0L;
      for (int j = 0; j < n; ++j)
        if (j != i) b *= (long double)xs[i] - (long double)xs[j];
      pw[i] = (double)(1.0L / b);
    }
  };
  product_weights(R.leg_x, nn, R.leg_pw);
  if (g->ngeo > 0) product_weights(R.geo_x, g->ngeo, R.geo_pw);
}

}  // namespace

namespace bem {
void gauss_legendre_nodes(int n, double* x, double* w) { gauss_legendre(n, x, w); }
}  // namespace bem

void bem_build_rules(const bem_geom2d* g, int npg, const double* ew_host, Rules& R) {
  build_rules(g, npg, ew_host, R);
}

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
void* bem_ctx::get(int slot, size_t bytes) {
  if (opt_inject & 1) return nullptr;  // injected allocation failure (BEM_OPT_INJECT bit 0)
  Buf& b = slots[slot];
  if (bytes == 0) bytes = 16;
  if (b.bytes >= bytes) return b.p;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  size_t want = bytes + bytes / 8;
  if (cudaMalloc(&b.p, want) != cudaSuccess) {
    cudaGetLastError();
    b.p = nullptr;
    return nullptr;
  }
  b.bytes = want;
  return b.p;
}

void bem_ctx::pin_issued() {
  if (!pin_ev && cudaEventCreateWithFlags(&pin_ev, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    pin_ev = nullptr;
  }
  if (pin_ev) {
    cudaEventRecord(pin_ev, stream);
    pin_pending = true;
  } else {
    cudaStreamSynchronize(stream);
  }
}

char* bem_ctx::pinned(size_t bytes) {
  if (pin_pending) {
    cudaEventSynchronize(pin_ev);
    pin_pending = false;
  }
  if (bytes == 0) bytes = 64;
  if (pin_bytes >= bytes) return pin;
  if (pin) {
    cudaStreamSynchronize(stream);
    cudaFreeHost(pin);
  }
  pin = nullptr;
  pin_bytes = 0;
  size_t want = (bytes + bytes / 8 + 4095) / 4096 * 4096;
  if (cudaHostAlloc((void**)&pin, want, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    pin = nullptr;
    return nullptr;
  }
  pin_bytes = want;
  return pin;
}

cudaEvent_t bem_ctx::timing_event(int i) {
  if (!tev[i] && cudaEventCreate(&tev[i]) != cudaSuccess) {
    cudaGetLastError();
    tev[i] = nullptr;
  }
  return tev[i];
}

bool bem_ctx::lookahead_ready(int k) {
  if (!la_stream) {
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (cudaStreamCreateWithPriority(&la_stream, cudaStreamNonBlocking, hi) != cudaSuccess) {
      la_stream = nullptr;
      return false;
    }
    if (cudaEventCreateWithFlags(&fork_event, cudaEventDisableTiming) != cudaSuccess) return false;
  }
  if (!thin_stream) {
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (cudaStreamCreateWithPriority(&thin_stream, cudaStreamNonBlocking, hi) != cudaSuccess) {
      thin_stream = nullptr;
      return false;
    }
  }
  while ((int)events.size() < 3 * k) {
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return false;
    events.push_back(e);
  }
  return true;
}

int bem_ctx::cuda_fail(cudaError_t e, const char* where) {
  last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? BEM_ERR_NOMEM : BEM_ERR_CUDA;
}

extern "C" int bem_ctx_create(int device, bem_ctx** out) {
  if (!out) return BEM_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return BEM_ERR_INVALID;
  }
  bem_ctx* c = new bem_ctx();
  c->device = device;
  // failure injection for tests (BEM_OPT_INJECT), from the environment
  if (const char* inj = std::getenv("BEM_INJECT")) c->opt_inject = std::atoi(inj);
  cudaSetDevice(device);
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return BEM_ERR_CUDA;
  }
  c->stream = c->own_stream;
  *out = c;
  return BEM_OK;
}

extern "C" int bem_ctx_destroy(bem_ctx* c) {
  if (!c) return BEM_ERR_INVALID;
  for (bem_ctx* w : c->workers) bem_ctx_destroy(w);
  c->workers.clear();
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  bem_release_solver(c);
  for (auto& b : c->slots)
    if (b.p) cudaFree(b.p);
  if (c->pin) cudaFreeHost(c->pin);
  if (c->pin_ev) cudaEventDestroy(c->pin_ev);
  for (auto e : c->tev)
    if (e) cudaEventDestroy(e);
  c->prof.release();
  for (auto e : c->events) cudaEventDestroy(e);
  if (c->asm_fork) cudaEventDestroy(c->asm_fork);
  if (c->asm_join) cudaEventDestroy(c->asm_join);
  if (c->asm_join2) cudaEventDestroy(c->asm_join2);
  if (c->asm_stream) cudaStreamDestroy(c->asm_stream);
  if (c->asm_stream2) cudaStreamDestroy(c->asm_stream2);
  if (c->lu_graph) cudaGraphExecDestroy(c->lu_graph);
  if (c->fork_event) cudaEventDestroy(c->fork_event);
  if (c->la_stream) cudaStreamDestroy(c->la_stream);
  if (c->thin_stream) cudaStreamDestroy(c->thin_stream);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
  return BEM_OK;
}

extern "C" int bem_ctx_set_stream(bem_ctx* c, void* s) {
  if (!c) return BEM_ERR_INVALID;
  c->stream = s ? (cudaStream_t)s : c->own_stream;
  return BEM_OK;
}

extern "C" const char* bem_last_error(bem_ctx* c) { return c ? c->last_error.c_str() : ""; }

extern "C" const char* bem_status_string(int s) {
  switch (s) {
    case BEM_OK: return "ok";
    case BEM_ERR_INVALID: return "invalid argument";
    case BEM_ERR_CUDA: return "CUDA error";
    case BEM_ERR_NOMEM: return "device out of memory";
    case BEM_ERR_NOT_CONVERGED: return "refinement did not converge";
    case BEM_ERR_INTERNAL: return "device wait timed out";
    case BEM_ERR_UNSUPPORTED: return "unsupported size or degree";
    default: return "unknown status";
  }
}

// ---------------------------------------------------------------------------
// geometry staging
// ---------------------------------------------------------------------------
int bem_check_geom(const bem_geom2d* g, int npg, double near_factor) {
  if (!g) return BEM_ERR_INVALID;
  if (g->p < 1 || g->p + 1 > BEM_MAXNN) return BEM_ERR_UNSUPPORTED;
  if (g->ngeo < 0 || g->ngeo == 1 || g->ngeo > BEM_MAXGEO) return BEM_ERR_UNSUPPORTED;
  if (g->ne <= 0 || g->n != g->ne * (g->p + 1) || g->nt < g->n) return BEM_ERR_INVALID;
  if (npg < 1 || npg > BEM_MAXNPG) return BEM_ERR_UNSUPPORTED;
  if (!(near_factor > 0)) return BEM_ERR_INVALID;
  if (!g->px || !g->py || !g->nx || !g->ny || !g->jac || !g->elen || !g->elem_weight)
    return BEM_ERR_INVALID;
  if (g->ngeo > 0 && (!g->geo_x || !g->geo_y)) return BEM_ERR_INVALID;
  // pair indices and column offsets are 32-bit
  if ((int64_t)g->nt * 2 >= (int64_t)1 << 30) return BEM_ERR_UNSUPPORTED;
  return BEM_OK;
}

int bem_stage_geom(bem_ctx* c, const bem_geom2d* g, int npg, int mem, GeomDev& gd, Rules& R, int64_t nb,
                   const int32_t* BC, const double* BV, const int32_t** dBC, const double** dBV) {
  const int nn = g->p + 1;
  double ew[BEM_MAXNN];
  if (mem == BEM_MEM_HOST) {
    std::memcpy(ew, g->elem_weight, sizeof(double) * nn);
  } else {
    // the element weights set up the host-side rule tables
    double* h = (double*)c->pinned(sizeof(double) * BEM_MAXNN);
    if (!h) return BEM_ERR_NOMEM;
    cudaMemcpyAsync(h, g->elem_weight, sizeof(double) * nn, cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "elem_weight");
    std::memcpy(ew, h, sizeof(double) * nn);
  }
  build_rules(g, npg, ew, R);
  R.nearfield = (unsigned char)c->opt_nearfield;
  R.singular = (unsigned char)c->opt_singular;
  gd.nt = g->nt;
  gd.n = g->n;
  gd.ne = g->ne;
  gd.nn = nn;
  gd.ngeo = g->ngeo;
  if (mem == BEM_MEM_DEVICE) {
    gd.px = g->px; gd.py = g->py; gd.nx = g->nx; gd.ny = g->ny;
    gd.jac = g->jac; gd.elen = g->elen; gd.gx = g->geo_x; gd.gy = g->geo_y;
    if (dBC) *dBC = BC;
    if (dBV) *dBV = BV;
    return BEM_OK;
  }
  // one device block [geometry | BV | BC], filled from the same layout in
  // the pinned buffer by one copy
  const bool bcs = nb > 0 && BC && BV && dBC && dBV;
  const size_t ng = (size_t)g->ne * g->ngeo;
  const size_t tot = 2 * (size_t)g->nt + 3 * (size_t)g->n + (size_t)g->ne + 2 * ng;
  const size_t nbv = bcs ? (size_t)nb : 0;
  const size_t nbc = bcs ? ((size_t)nb + 1) / 2 : 0;  // int32 codes, in doubles
  const size_t words = tot + nbv + nbc;
  double* d = (double*)c->get(bem_ctx::SLOT_GEOM, words * sizeof(double));
  double* h = (double*)c->pinned(words * sizeof(double));
  if (!d || !h) return BEM_ERR_NOMEM;
  size_t o = 0;
  auto put = [&](const double* src, size_t cnt) -> const double* {
    if (cnt) std::memcpy(h + o, src, cnt * sizeof(double));
    const double* dst = d + o;
    o += cnt;
    return dst;
  };
  gd.px = put(g->px, g->nt);
  gd.py = put(g->py, g->nt);
  gd.nx = put(g->nx, g->n);
  gd.ny = put(g->ny, g->n);
  gd.jac = put(g->jac, g->n);
  gd.elen = put(g->elen, g->ne);
  gd.gx = ng ? put(g->geo_x, ng) : nullptr;
  gd.gy = ng ? put(g->geo_y, ng) : nullptr;
  if (bcs) {
    *dBV = put(BV, nbv);
    std::memcpy(h + o, BC, sizeof(int32_t) * (size_t)nb);
    *dBC = (const int32_t*)(d + o);
    o += nbc;
  }
  cudaMemcpyAsync(d, h, o * sizeof(double), cudaMemcpyHostToDevice, c->stream);
  c->pin_issued();
  return BEM_OK;
}

// Runs one assembly (device pointers already set in q), retrying once with
// a larger pair list if the first estimate overflowed.
int bem_run_assembly(bem_ctx* c, AsmRequest& q) {
  const int nt = q.g.nt;
  const int dof = q.ph.kind == 0 ? 1 : 2;
  q.rows = (float4*)c->get(bem_ctx::SLOT_ROWS, sizeof(float4) * (size_t)nt);
  q.nodes = (bem::NodeRec*)c->get(bem_ctx::SLOT_NODES, sizeof(bem::NodeRec) * (size_t)q.g.n);
  q.elems = (bem::ElemRec*)c->get(bem_ctx::SLOT_ELEMS, sizeof(bem::ElemRec) * (size_t)q.g.ne);
  q.rowsum = (double*)c->get(bem_ctx::SLOT_ROWSUM, sizeof(double) * (size_t)nt * dof * dof);
  q.gdiag = (double*)c->get(bem_ctx::SLOT_GDIAG, sizeof(double) * (size_t)q.g.n * dof * dof);
  q.counters = (int*)c->get(bem_ctx::SLOT_COUNTERS, 64);
  q.absmax = (unsigned long long*)((char*)q.counters + 32);
  if (!q.rows || !q.nodes || !q.elems || !q.rowsum || !q.gdiag || !q.counters) return BEM_ERR_NOMEM;
  if (!c->asm_stream) {
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (cudaStreamCreateWithPriority(&c->asm_stream, cudaStreamNonBlocking, hi) != cudaSuccess ||
        cudaStreamCreateWithPriority(&c->asm_stream2, cudaStreamNonBlocking, hi) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->asm_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->asm_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->asm_join2, cudaEventDisableTiming) != cudaSuccess)
      return c->cuda_fail(cudaGetLastError(), "assembly side streams");
  }
  q.aux = c->asm_stream;
  q.aux2 = c->asm_stream2;
  q.ev_fork = c->asm_fork;
  q.ev_join = c->asm_join;
  q.ev_join2 = c->asm_join2;
  if (q.prec == 3) {
    const size_t rec = q.ph.kind == 0 ? sizeof(bem::NodeDF) : sizeof(bem::NodeDFK);
    q.nodes_df = (bem::NodeDF*)c->get(bem_ctx::SLOT_NODES_DF, rec * (size_t)q.g.n);
    q.logtab = (float4*)c->get(bem_ctx::SLOT_LOGTAB, sizeof(float4) * 136);
    if (!q.nodes_df || !q.logtab) return BEM_ERR_NOMEM;
  }
  int cap = c->pair_cap_hint > 0 ? c->pair_cap_hint : nt * 16 + 4096;
  for (int attempt = 0; attempt < 3; ++attempt) {
    q.pairs = (int2*)c->get(bem_ctx::SLOT_PAIRS, sizeof(int2) * (size_t)cap);
    if (!q.pairs) return BEM_ERR_NOMEM;
    q.pair_cap = cap;
    int rc = bem::launch_assembly(q, c->stream);
    if (rc != 0) return c->cuda_fail((cudaError_t)rc, "launch_assembly");
    // pair count and far-kernel status through the pinned buffer
    int* hc = (int*)c->pinned(64);
    if (!hc) return BEM_ERR_NOMEM;
    cudaMemcpyAsync(hc, q.counters, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "assembly");
    if (hc[1] != 0) {
      c->last_error = "bulk-copy wait timed out in the far-field kernel";
      return BEM_ERR_INTERNAL;
    }
    if (hc[0] <= cap) {
      c->pair_cap_hint = std::max(c->pair_cap_hint, hc[0] + hc[0] / 4 + 1024);
      return BEM_OK;
    }
    cap = hc[0] + hc[0] / 4 + 1024;
  }
  return BEM_ERR_INTERNAL;
}

// ---------------------------------------------------------------------------
// H, G assembly
// ---------------------------------------------------------------------------
static int assemble_hg(bem_ctx* c, const bem_geom2d* g, const Physics& ph, int npg, double nf,
                       int dtype, int mem, void* H, int64_t ldh, void* G, int64_t ldg) {
  if (!c) return BEM_ERR_INVALID;
  CallScope cs(c);
  int rc = bem_check_geom(g, npg, nf);
  if (rc) return rc;
  if (dtype != BEM_F32 && dtype != BEM_F64) return BEM_ERR_INVALID;
  if (mem != BEM_MEM_HOST && mem != BEM_MEM_DEVICE) return BEM_ERR_INVALID;
  const int dof = ph.kind == 0 ? 1 : 2;
  const int64_t rows = (int64_t)dof * g->nt, hcols = rows, gcols = (int64_t)dof * g->n;
  if (!H || !G || ldh < rows || ldg < rows) return BEM_ERR_INVALID;
  cudaSetDevice(c->device);
  AsmRequest q{};
  rc = bem_stage_geom(c, g, npg, mem, q.g, q.R);
  if (rc) return rc;
  q.ph = ph;
  q.near_factor = nf;
  q.prec = dtype == BEM_F32 ? 0 : 1;
  q.fused = 0;
  const size_t esz = dtype == BEM_F32 ? 4 : 8;
  if (mem == BEM_MEM_DEVICE) {
    q.H = H; q.ld = ldh; q.G = G; q.ldg = ldg;
  } else {
    const int64_t ldp = (rows + 3) / 4 * 4;
    q.H = c->get(bem_ctx::SLOT_OUT0, esz * (size_t)ldp * hcols);
    q.G = c->get(bem_ctx::SLOT_OUT1, esz * (size_t)ldp * gcols);
    if (!q.H || !q.G) return BEM_ERR_NOMEM;
    q.ld = q.ldg = ldp;
  }
  rc = bem_run_assembly(c, q);
  if (rc) return rc;
  if (mem == BEM_MEM_HOST) {
    cudaMemcpy2DAsync(H, esz * ldh, q.H, esz * q.ld, esz * rows, hcols, cudaMemcpyDeviceToHost,
                      c->stream);
    cudaMemcpy2DAsync(G, esz * ldg, q.G, esz * q.ldg, esz * rows, gcols, cudaMemcpyDeviceToHost,
                      c->stream);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return c->cuda_fail(e, "copy H, G to host");
  }
  return BEM_OK;
}

extern "C" int bem_assemble_laplace2d(bem_ctx* c, const bem_geom2d* g, double k, int npg,
                                      double nf, int dtype, int mem, void* H, int64_t ldh, void* G,
                                      int64_t ldg) {
  if (!(k > 0) || !std::isfinite(k)) return BEM_ERR_INVALID;
  Physics ph{};
  ph.kind = 0;
  ph.k = k;
  return assemble_hg(c, g, ph, npg, nf, dtype, mem, H, ldh, G, ldg);
}

extern "C" int bem_assemble_kelvin2d(bem_ctx* c, const bem_geom2d* g, double mu, double nu,
                                     int npg, double nf, int dtype, int mem, void* H, int64_t ldh,
                                     void* G, int64_t ldg) {
  if (!(mu > 0) || !(nu < 0.5) || !(nu > -1.0)) return BEM_ERR_INVALID;
  Physics ph{};
  ph.kind = 1;
  ph.mu = mu;
  ph.nu = nu;
  return assemble_hg(c, g, ph, npg, nf, dtype, mem, H, ldh, G, ldg);
}

// ---------------------------------------------------------------------------
// fused system assembly
// ---------------------------------------------------------------------------
int bem_assemble_system_dev(bem_ctx* c, const bem_geom2d* g, const Physics& ph, const int32_t* BC,
                            const double* BV, int npg, double nf, int mem, int prec, double* A,
                            int64_t lda, float* A32, double* b) {
  int rc = bem_check_geom(g, npg, nf);
  if (rc) return rc;
  const int dof = ph.kind == 0 ? 1 : 2;
  const int64_t nb = (int64_t)dof * g->n;
  cudaSetDevice(c->device);
  AsmRequest q{};
  rc = bem_stage_geom(c, g, npg, mem, q.g, q.R, nb, BC, BV, &q.bc, &q.bv);
  if (rc) return rc;
  q.ph = ph;
  q.near_factor = nf;
  q.prec = prec;
  q.fused = 1;
  q.H = A;
  q.ld = lda;
  q.G = nullptr;
  q.ldg = lda;
  q.A32 = A32;
  q.b = b;
  return bem_run_assembly(c, q);
}

extern "C" int bem_assemble_system2d(bem_ctx* c, const bem_geom2d* g, int kind, double prm0,
                                     double prm1, const int32_t* BC, const double* BV, int npg,
                                     double nf, int mem, double* A, int64_t lda, double* b) {
  if (!c || !g || !BC || !BV || !A || !b) return BEM_ERR_INVALID;
  if (kind != 0 && kind != 1) return BEM_ERR_INVALID;
  if (mem != BEM_MEM_HOST && mem != BEM_MEM_DEVICE) return BEM_ERR_INVALID;
  CallScope cs(c);
  Physics ph{};
  ph.kind = kind;
  if (kind == 0) {
    if (!(prm0 > 0)) return BEM_ERR_INVALID;
    ph.k = prm0;
  } else {
    if (!(prm0 > 0) || !(prm1 < 0.5) || !(prm1 > -1.0)) return BEM_ERR_INVALID;
    ph.mu = prm0;
    ph.nu = prm1;
  }
  const int dof = kind == 0 ? 1 : 2;
  const int64_t rows = (int64_t)dof * g->nt;
  if (lda < rows) return BEM_ERR_INVALID;
  const int prec = c->opt_far_df >= 2 ? 3 : 1;
  if (mem == BEM_MEM_DEVICE)
    return bem_assemble_system_dev(c, g, ph, BC, BV, npg, nf, mem, prec, A, lda, nullptr, b);
  const int64_t ldp = (rows + 3) / 4 * 4;
  double* dA = (double*)c->get(bem_ctx::SLOT_OUT0, sizeof(double) * (size_t)ldp * rows);
  double* db = (double*)c->get(bem_ctx::SLOT_OUT1, sizeof(double) * (size_t)rows);
  if (!dA || !db) return BEM_ERR_NOMEM;
  int rc = bem_assemble_system_dev(c, g, ph, BC, BV, npg, nf, mem, prec, dA, ldp, nullptr, db);
  if (rc) return rc;
  cudaMemcpy2DAsync(A, 8 * lda, dA, 8 * ldp, 8 * rows, rows, cudaMemcpyDeviceToHost, c->stream);
  cudaMemcpyAsync(b, db, 8 * rows, cudaMemcpyDeviceToHost, c->stream);
  cudaError_t e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return c->cuda_fail(e, "copy A, b to host");
  return BEM_OK;
}

extern "C" int bem_kernel_times(bem_ctx* c, double* ms, int64_t* counts, int n) {
  if (!c || n < 0) return BEM_ERR_INVALID;
  c->prof.collect();
  for (int i = 0; i < n; ++i) {
    if (ms) ms[i] = i < bem::KC_COUNT ? c->prof.ms[i] : 0.0;
    if (counts) counts[i] = i < bem::KC_COUNT ? c->prof.n[i] : 0;
  }
  for (int i = 0; i < bem::KC_COUNT; ++i) {
    c->prof.ms[i] = 0.0;
    c->prof.n[i] = 0;
  }
  return BEM_OK;
}

extern "C" int bem_kernel_trace(bem_ctx* c, int cap, int* cls, double* t0, double* t1) {
  if (!c || cap < 0) return -BEM_ERR_INVALID;
  c->prof.collect();
  const int n = (int)c->prof.trace.size() < cap ? (int)c->prof.trace.size() : cap;
  for (int i = 0; i < n; ++i) {
    if (cls) cls[i] = c->prof.trace[i].cls;
    if (t0) t0[i] = c->prof.trace[i].t0;
    if (t1) t1[i] = c->prof.trace[i].t1;
  }
  c->prof.trace.clear();
  return n;
}

extern "C" int64_t bem_launch_count(void) { return (int64_t)bem::g_launches.load(); }
