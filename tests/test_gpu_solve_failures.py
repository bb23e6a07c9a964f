"""The `bem_linsolve` seam on matrices the unpivoted mixed LU cannot factor,
and the failure paths of the solve, all through the C ABI.

The reference solves with LAPACK getrf/getrs (partial pivoting) through
LinearSolve (src/Core/LinearSolveUtils.jl:44-49).  The mixed solve factors
without pivoting; when that breaks down (vanishing pivot) or its refinement
stagnates, it solves again with partial pivoting in FP64
(BEM_OPT_PIVOT_FALLBACK), so a permuted identity, a zero leading pivot and a
non-diagonally-dominant random matrix come out within 1e-12 of LAPACK.

Failures are made on the host, never by faulting the GPU: an iteration cap
of 1, the fallback switched off, every workspace allocation refused
(BEM_OPT_INJECT bit 0), and triangular sweeps whose results are published
under an epoch their readers do not wait for (bit 1), so that their bounded
waits run out after BEM_OPT_WAIT_LIMIT polls; the context must stay usable
after each."""
import numpy as np
import pytest

from bem_gmsh_gb300 import _lib
from bem_gmsh_gb300.api import solve_system

pytestmark = pytest.mark.gpu

NOT_CONVERGED, NOMEM, INTERNAL = 4, 3, 5


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


def lapack(A, b):
    import scipy.linalg as sla
    return sla.lu_solve(sla.lu_factor(A), b)


def _cases():
    rng = np.random.default_rng(4)
    out = {}
    n = 300
    P = np.eye(n)[rng.permutation(n)]
    out["permuted_identity"] = np.asfortranarray(P)
    A = rng.standard_normal((n, n)) / np.sqrt(n) + 2.0 * np.eye(n)
    A[0, 0] = 0.0
    out["zero_leading_pivot"] = np.asfortranarray(A)
    out["random_gaussian"] = np.asfortranarray(rng.standard_normal((500, 500)))
    B = rng.standard_normal((n, n))
    B[:128, :128] = np.triu(B[:128, :128], 1)  # singular leading block
    out["singular_leading_block"] = np.asfortranarray(B + 1e-3 * np.eye(n)[::-1])
    return out


@pytest.mark.parametrize("name", sorted(_cases()))
def test_mixed_solve_matches_lapack_without_pivot_structure(name):
    A = _cases()[name]
    b = np.random.default_rng(9).standard_normal(A.shape[0])
    x, st = solve_system(A, b, mode="mixed")
    xr = lapack(A, b)
    print(name, "pivoted" if st["pivoted"] else "unpivoted", rel(x, xr))
    assert rel(x, xr) < 1e-12, (name, rel(x, xr), st)
    if name in ("permuted_identity", "zero_leading_pivot"):
        assert st["pivoted"], st


def test_fallback_off_reports_not_converged():
    ctx = _lib.Context()
    try:
        ctx.set_option(_lib.BEM_OPT_PIVOT_FALLBACK, 0)
        A = _cases()["zero_leading_pivot"]
        with pytest.raises(_lib.BemError) as e:
            solve_system(A, np.ones(A.shape[0]), mode="mixed", ctx=ctx)
        assert e.value.status == NOT_CONVERGED
    finally:
        ctx.close()


def test_iteration_cap_reports_not_converged():
    rng = np.random.default_rng(1)
    n = 400
    A = np.asfortranarray(rng.standard_normal((n, n)) / np.sqrt(n) + 2 * np.eye(n))
    b = rng.standard_normal(n)
    ctx = _lib.Context()
    try:
        with pytest.raises(_lib.BemError) as e:
            solve_system(A, b, mode="mixed", tol=1e-15, max_iter=1, ctx=ctx)
        assert e.value.status == NOT_CONVERGED
        x, st = solve_system(A, b, mode="mixed", ctx=ctx)  # the same context, default cap
        assert rel(x, lapack(A, b)) < 1e-12 and not st["pivoted"]
    finally:
        ctx.close()


def test_injected_allocation_failure_reports_nomem():
    rng = np.random.default_rng(2)
    n = 200
    A = np.asfortranarray(rng.standard_normal((n, n)) / np.sqrt(n) + 2 * np.eye(n))
    b = rng.standard_normal(n)
    ctx = _lib.Context()
    try:
        ctx.set_option(_lib.BEM_OPT_INJECT, 1)
        with pytest.raises(_lib.BemError) as e:
            solve_system(A, b, mode="mixed", ctx=ctx)
        assert e.value.status == NOMEM
        ctx.set_option(_lib.BEM_OPT_INJECT, 0)
        x, st = solve_system(A, b, mode="mixed", ctx=ctx)
        assert rel(x, lapack(A, b)) < 1e-12
    finally:
        ctx.close()


def test_sweep_wait_runs_out_and_context_recovers():
    """Triangular sweeps whose waits are never satisfied: each wait gives up
    after BEM_OPT_WAIT_LIMIT polls, the call returns BEM_ERR_INTERNAL, and the
    next solve on the same context is correct."""
    rng = np.random.default_rng(3)
    n = 700  # six 128-row blocks: blocks 1..5 wait on their predecessors
    A = np.asfortranarray(rng.standard_normal((n, n)) / np.sqrt(n) + 2 * np.eye(n))
    b = rng.standard_normal(n)
    ctx = _lib.Context()
    try:
        ctx.set_option(_lib.BEM_OPT_WAIT_LIMIT, 2000)
        ctx.set_option(_lib.BEM_OPT_INJECT, 2)
        with pytest.raises(_lib.BemError) as e:
            solve_system(A, b, mode="mixed", max_iter=3, ctx=ctx)
        assert e.value.status == INTERNAL
        ctx.set_option(_lib.BEM_OPT_INJECT, 0)
        ctx.set_option(_lib.BEM_OPT_WAIT_LIMIT, 1 << 20)
        x, st = solve_system(A, b, mode="mixed", ctx=ctx)
        assert rel(x, lapack(A, b)) < 1e-12
    finally:
        ctx.close()
