// Batched solves (and adjoint shape gradients) of many independent domains
// with uneven sizes on one GPU.
//
// The reference solves one mesh per call; a batch here is a set of domains
// described by an array of bem_geom2d plus offset arrays into concatenated
// BC/BV/x vectors.  A pool of host worker threads, each driving its own
// sub-context (own stream, own device workspace sized for its largest
// domain), takes domains largest-first from a shared counter and runs the
// full assembly + solve pipeline of bem_solve2d on it.  The blocked LU of one
// domain is latency-bound on its diagonal chain, so running several domains
// at once fills the SMs that one domain leaves idle.  Results are identical
// to single-domain calls (same kernels, same order of operations per domain).
#include <algorithm>
#include <atomic>
#include <numeric>
#include <thread>
#include <vector>

#include "bem_abi_internal.h"

namespace {

constexpr int kMaxWorkers = 32;

int ensure_workers(bem_ctx* c, int w) {
  while ((int)c->workers.size() < w) {
    bem_ctx* s = nullptr;
    int rc = bem_ctx_create(c->device, &s);
    if (rc != BEM_OK) return rc;
    c->workers.push_back(s);
  }
  for (bem_ctx* s : c->workers) {
    // concurrent pipelines share the SMs: the one-CTA-per-tile bulk update
    // (two per SM) interleaves with the other workers' kernels, where the
    // persistent kernel holds whole SMs (2 % more batch throughput measured)
    s->opt_tcgen05 = c->opt_tcgen05 == 2 ? 1 : c->opt_tcgen05;
    s->opt_tc_reserve = c->opt_tc_reserve;
    s->opt_far_df = c->opt_far_df;
    s->opt_pivot_fallback = c->opt_pivot_fallback;
    s->opt_wait_limit = c->opt_wait_limit;
    s->opt_inject = c->opt_inject;
    s->opt_nearfield = c->opt_nearfield;
    s->opt_singular = c->opt_singular;
    // concurrent pipelines share the SMs: one CTA per block row in the sweeps
    s->opt_sweep_ctas = 1;
  }
  return BEM_OK;
}

// Runs fn(worker context, domain) for every domain on w worker threads,
// largest domains (by key) first.  Returns the first hard error (keeping the
// message of the domain that raised it), else BEM_ERR_NOT_CONVERGED if a
// domain stopped short of its tolerance, else BEM_OK.
template <class Fn>
int run_pool(bem_ctx* c, int ndom, int w, const std::vector<int64_t>& key, Fn fn) {
  std::vector<int> order(ndom);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key[a] > key[b]; });
  std::atomic<int> next{0};
  std::atomic<int> first_err{BEM_OK};
  std::vector<std::string> errs(w);
  auto run = [&](int wi) {
    bem_ctx* s = c->workers[wi];
    cudaSetDevice(s->device);
    for (;;) {
      const int i = next.fetch_add(1);
      if (i >= ndom) break;
      const int d = order[i];
      const int r = fn(s, d);
      if (r != BEM_OK && r != BEM_ERR_NOT_CONVERGED) {
        // a hard error replaces "not converged" but not an earlier hard error
        int cur = first_err.load();
        while ((cur == BEM_OK || cur == BEM_ERR_NOT_CONVERGED) && !first_err.compare_exchange_weak(cur, r)) {
        }
        if (cur == BEM_OK || cur == BEM_ERR_NOT_CONVERGED)
          errs[wi] = "domain " + std::to_string(d) + ": " + s->last_error;
      } else if (r == BEM_ERR_NOT_CONVERGED) {
        int expected = BEM_OK;
        first_err.compare_exchange_strong(expected, r);
      }
    }
  };
  std::vector<std::thread> th;
  th.reserve(w);
  for (int i = 0; i < w; ++i) th.emplace_back(run, i);
  for (auto& t : th) t.join();
  const int e = first_err.load();
  if (e != BEM_OK) {
    for (auto& m : errs)
      if (!m.empty()) c->last_error = m;
  }
  return e;
}

// Workers for a batch of ndom domains; the caller's stream orders the batch
// (workers start after the work already queued there).
int start_pool(bem_ctx* c, int ndom, int nworkers, int* w) {
  *w = std::min(nworkers > 0 ? nworkers : 8, ndom);
  cudaSetDevice(c->device);
  int rc = ensure_workers(c, *w);
  if (rc != BEM_OK) return rc;
  cudaStreamSynchronize(c->stream);
  return BEM_OK;
}

}  // namespace

extern "C" int bem_solve2d_batch(bem_ctx* c, int ndom, const bem_geom2d* geoms, int kind, double prm0,
                                 double prm1, const int32_t* BC, const double* BV, const int64_t* bc_off,
                                 int npg, double near_factor, int mode, double tol, int max_iter, int mem,
                                 double* x, const int64_t* x_off, int nworkers, bem_solve_stats* stats) {
  if (!c || ndom < 0 || (ndom > 0 && (!geoms || !BC || !BV || !bc_off || !x || !x_off)))
    return BEM_ERR_INVALID;
  if (nworkers < 0 || nworkers > kMaxWorkers) return BEM_ERR_INVALID;
  if (ndom == 0) return BEM_OK;
  std::vector<int64_t> key(ndom);
  for (int d = 0; d < ndom; ++d) {
    if (bc_off[d] < 0 || x_off[d] < 0) return BEM_ERR_INVALID;
    if (geoms[d].nt <= 0 || geoms[d].n <= 0) return BEM_ERR_INVALID;
    key[d] = geoms[d].nt;
  }
  int w = 0;
  int rc = start_pool(c, ndom, nworkers, &w);
  if (rc != BEM_OK) return rc;
  // largest domains first (longest critical paths start early)
  return run_pool(c, ndom, w, key, [&](bem_ctx* s, int d) {
    bem_solve_stats st{};
    const int r = bem_solve2d(s, &geoms[d], kind, prm0, prm1, BC + bc_off[d], BV + bc_off[d], npg, near_factor,
                              mode, tol, max_iter, mem, x + x_off[d], stats ? &st : nullptr);
    if (stats) stats[d] = st;
    return r;
  });
}

extern "C" int bem_adjoint_laplace2d_batch(bem_ctx* c, int ndom, const bem_geom2d* geoms, double k,
                                           const int32_t* BC, const double* BV, const double* q_target,
                                           const int64_t* off, int npg, double near_factor, double tol,
                                           int max_iter, double* J, double* grad, int nworkers,
                                           bem_solve_stats* stats) {
  if (!c || ndom < 0 || (ndom > 0 && (!geoms || !BC || !BV || !q_target || !off || !J || !grad)))
    return BEM_ERR_INVALID;
  if (nworkers < 0 || nworkers > kMaxWorkers) return BEM_ERR_INVALID;
  if (ndom == 0) return BEM_OK;
  std::vector<int64_t> key(ndom);
  for (int d = 0; d < ndom; ++d) {
    if (off[d] < 0 || geoms[d].n <= 0) return BEM_ERR_INVALID;
    key[d] = geoms[d].n;
  }
  int w = 0;
  int rc = start_pool(c, ndom, nworkers, &w);
  if (rc != BEM_OK) return rc;
  return run_pool(c, ndom, w, key, [&](bem_ctx* s, int d) {
    bem_solve_stats st{};
    const int64_t o = off[d];
    const int r = bem_adjoint_laplace2d(s, &geoms[d], k, BC + o, BV + o, q_target + o, npg, near_factor, tol,
                                        max_iter, BEM_MEM_HOST, J + d, grad + 2 * o, stats ? &st : nullptr);
    if (stats) stats[d] = st;
    return r;
  });
}
