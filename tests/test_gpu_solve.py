"""GPU solve parity: mixed precision (FP32 tensor-core LU + FP64 GMRES) and
the FP64 comparison path, against FP64 LAPACK solves of the oracle systems.
Bar: refined solution within 1e-10 relative of the FP64 solution of the same
system; rel_error against the analytic field no worse than the oracle's."""
import numpy as np
import pytest

from bem_gmsh_gb300 import (quadrado, star_domain, quadrado_elasticity, Elasticity,
                            ana_laplace_linear, attach_analytical, ana_elasticity_patch,
                            apply_analytical_bc, rel_error, rel_error_flux)
from bem_gmsh_gb300.api import solve, solve_system, assemble_system

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n", [7, 128, 300, 1000])
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_solve_system_dense(n, mode):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n)) / np.sqrt(n) + 2.0 * np.eye(n)
    A *= rng.uniform(0.1, 10.0, size=n)[None, :]  # uneven column scales
    A = np.asfortranarray(A)
    b = rng.standard_normal(n)
    x, st = solve_system(A, b, mode=mode)
    xr = np.linalg.solve(A, b)
    assert rel(x, xr) < 1e-12, (rel(x, xr), st)
    if mode == "mixed":  # an FP32-accurate LU preconditioner needs only a few iterations
        assert st["iterations"] <= 8, st


def test_solve_system_device_pointers():
    import torch
    rng = np.random.default_rng(3)
    n = 513
    A = np.asfortranarray(rng.standard_normal((n, n)) / np.sqrt(n) + 3 * np.eye(n))
    b = rng.standard_normal(n)
    At = torch.from_numpy(np.ascontiguousarray(A.T)).cuda().t()  # column-major view
    bt = torch.from_numpy(b).cuda()
    x, st = solve_system(At, bt)
    assert rel(x.cpu().numpy(), np.linalg.solve(A, b)) < 1e-12


# C1: the reference's unit square (19 linear elements per side, left T = 0,
# right q = -1); C1': 20 elements per side with T prescribed on left (0) and
# right (1), q = 0 on top and bottom
C1_CASES = {"C1": dict(ndiv=20), "C1prime": dict(ndiv=21, bcs={"right": (0, 1.0)})}


@pytest.mark.parametrize("case", sorted(C1_CASES))
@pytest.mark.parametrize("mode", ["mixed", "fp64"])
def test_quadrado_pipeline(orc, mode, case):
    dad = quadrado(pontointerno=True, **C1_CASES[case])
    attach_analytical(dad, ana_laplace_linear())
    ref = quadrado(pontointerno=True, **C1_CASES[case])
    attach_analytical(ref, ana_laplace_linear())
    orc.assemble(ref, npg=20)
    orc.solve(ref)
    solve(dad, npg=20, mode=mode)
    assert rel(dad.cache["x"], ref.cache["x"]) < 1e-10
    assert rel_error(dad) <= rel_error(ref) * (1 + 1e-6) + 1e-12
    assert rel_error(dad) < 0.05


@pytest.mark.parametrize("ne", [300, 1100])
def test_star_pipeline_mixed(orc, ne):
    dad = star_domain(ne, p=2, seed=11)
    A, b = assemble_system(dad, npg=16)
    x_fp64 = np.linalg.solve(A, b)
    T, st = solve(dad, npg=16, mode="mixed", return_stats=True)
    # solver parity on the same system
    assert rel(dad.cache["x"], x_fp64) < 1e-10, st
    # end-to-end against the oracle's assembly + LAPACK solve
    ref = star_domain(ne, p=2, seed=11)
    orc.assemble(ref, npg=16)
    orc.solve(ref)
    assert rel(dad.cache["x"], ref.cache["x"]) < 1e-10
    from bem_gmsh_gb300.geometry import analytical
    scale = np.linalg.norm(ref.cache["x"]) / np.linalg.norm(analytical(ref))
    assert abs(rel_error(dad) - rel_error(ref)) <= 1e-10 * scale + 1e-12
    assert st["rel_residual"] <= 1e-14
    assert st["iterations"] <= 8, st


def test_kelvin_patch_pipeline(orc):
    dad = quadrado_elasticity(ndiv=9, props=Elasticity(1.0, 0.3, 1.0))
    ana = ana_elasticity_patch(E=1.0, nu=0.3, exx=0.01)
    apply_analytical_bc(dad, ana, neumann_nodes=np.arange(0, dad.n // 2))
    ref = quadrado_elasticity(ndiv=9, props=Elasticity(1.0, 0.3, 1.0))
    apply_analytical_bc(ref, ana, neumann_nodes=np.arange(0, ref.n // 2))
    orc.assemble(ref, npg=12)
    orc.solve(ref)
    solve(dad, npg=12, mode="mixed")
    assert rel(dad.cache["x"], ref.cache["x"]) < 1e-10
    assert rel_error_flux(dad) < 0.15 and rel_error(dad) < 0.15


def test_solve_bad_args():
    from bem_gmsh_gb300._lib import BemError
    dad = quadrado(ndiv=5)
    with pytest.raises(KeyError):
        solve(dad, mode="fp16")
    A = np.asfortranarray(np.eye(4))
    with pytest.raises(BemError):
        solve_system(A, np.ones(4), tol=-1.0)


def test_lu_building_blocks():
    """The tensor-core trailing updates and the blocked diagonal factorization
    agree with the independent implementations to FP32 rounding."""
    from bem_gmsh_gb300 import _lib
    c = _lib.default_context()
    d = c.selftest_diag(256)
    assert d[0] / d[1] < 1e-5 and d[2] / d[3] < 1e-5, d
    r = c.selftest_lu(1024)
    assert r[0] / r[1] < 1e-5, r


@pytest.mark.parametrize("n", [384, 512, 2048, 4096])
def test_persistent_bulk_update_matches_per_tile_kernel(n):
    """The persistent warp-specialized tcgen05 update (TMEM double buffer,
    C through TMA, several tiles per CTA at n = 4096) against the one-CTA-per-
    tile kernel on the same operands, for the whole trailing matrix and for
    the look-ahead's shape (past the first block row and column, a half tile
    at the last column at n = 384 and 512): the same MMA sequence and the same
    epilogue formula, so the results agree to FP32 rounding of the epilogue
    (bit-identical in practice)."""
    from bem_gmsh_gb300 import _lib
    ctx = _lib.Context()
    try:
        ctx.set_option(_lib.BEM_OPT_TCGEN05, 2)
        for reserve in (0, 8):
            ctx.set_option(_lib.BEM_OPT_TC_RESERVE, reserve)
            r = ctx.selftest_bulk_compare(n)
            assert r[0] <= 1e-6 * r[1] and r[2] <= 1e-6 * r[3], r
    finally:
        ctx.close()


@pytest.mark.parametrize("variant", [1, 2])
def test_lu_with_each_bulk_kernel(variant):
    """The look-ahead LU with either tcgen05 bulk-update kernel agrees with the
    legacy mma.sync factorization to FP32 rounding."""
    from bem_gmsh_gb300 import _lib
    ctx = _lib.Context()
    try:
        ctx.set_option(_lib.BEM_OPT_TCGEN05, variant)
        r = ctx.selftest_lu(2048)
        assert r[0] / r[1] < 1e-5, r
    finally:
        ctx.close()


def test_factorization_graph_replay_matches_direct_launches():
    """The mixed solve captures its factorization in a CUDA graph on the
    second call with unchanged buffers and replays it afterwards; replayed
    solves agree with direct launches (BEM_OPT_GRAPHS = 0)."""
    from bem_gmsh_gb300 import _lib
    ctx = _lib.Context()
    try:
        dad = star_domain(700, p=2, seed=4)
        ctx.set_option(_lib.BEM_OPT_GRAPHS, 0)
        solve(dad, npg=16, mode="mixed", ctx=ctx)
        x_direct = dad.cache["x"].copy()
        ctx.set_option(_lib.BEM_OPT_GRAPHS, 1)
        xs = []
        for _ in range(4):  # direct, capture + replay, replay, replay
            _, st = solve(dad, npg=16, mode="mixed", ctx=ctx, return_stats=True)
            xs.append(dad.cache["x"].copy())
            assert st["rel_residual"] <= 1e-14, st
        for x in xs:
            assert rel(x, x_direct) < 1e-12
    finally:
        ctx.close()


def test_large_system_uses_stepwise_sweeps():
    """N = 20100 (157 block rows, more than the co-resident CTAs of the
    wavefront sweep): the preconditioner falls back to step-wise sweeps and
    the mixed solve still matches the FP64 path."""
    dad = star_domain(6700, p=2, seed=2)
    assert dad.nt == 20100
    _, st = solve(dad, npg=16, mode="mixed", return_stats=True)
    x_mixed = dad.cache["x"].copy()
    ref = star_domain(6700, p=2, seed=2)
    solve(ref, npg=16, mode="fp64")
    assert rel(x_mixed, ref.cache["x"]) < 1e-10, st
    assert st["rel_residual"] <= 1e-14, st


def test_full_size_solve_matches_oracle(orc):
    """The headline solve (2731 quadratic elements, N = 8193), mixed
    precision, against the oracle's FP64 assembly + LAPACK LU: the solutions
    within 1e-10, and the error against the analytic field the same to the
    digits it has (|difference| <= 1e-10 of the solution's scale)."""
    import os
    from bem_gmsh_gb300.geometry import analytical
    dad = star_domain(2731, p=2, seed=0)
    T, st = solve(dad, npg=16, mode="mixed", return_stats=True)
    ref = star_domain(2731, p=2, seed=0)
    orc.assemble(ref, npg=16, threads=os.cpu_count() or 1)
    orc.solve(ref)
    e = rel(dad.cache["x"], ref.cache["x"])
    ra, rb = rel_error(dad), rel_error(ref)
    scale = np.linalg.norm(ref.cache["x"]) / np.linalg.norm(analytical(ref))
    print(f"N = 8193: solution vs oracle {e:.2e}; rel_error GPU {ra:.12e}, oracle {rb:.12e}")
    assert e < 1e-10, e
    assert abs(ra - rb) <= 1e-10 * scale, (ra, rb)


def test_lu_options_give_the_same_solution():
    """The bulk-update variant, the SM reserve and the sweep CTAs per block row
    change the schedule, not the answer: every setting reaches the FP64
    residual floor with the same iterations, and out-of-range values are
    rejected."""
    from bem_gmsh_gb300 import _lib
    ctx = _lib.Context()
    try:
        dad = star_domain(700, p=2, seed=5)
        solve(dad, npg=16, mode="mixed", ctx=ctx)
        x0 = dad.cache["x"].copy()
        for opt, val in [(_lib.BEM_OPT_TC_RESERVE, 0), (_lib.BEM_OPT_TC_RESERVE, 24),
                         (_lib.BEM_OPT_SWEEP_CTAS, 1), (_lib.BEM_OPT_SWEEP_CTAS, 2),
                         (_lib.BEM_OPT_TCGEN05, 1), (_lib.BEM_OPT_TCGEN05, 0)]:
            ctx.set_option(opt, val)
            _, st = solve(dad, npg=16, mode="mixed", ctx=ctx, return_stats=True)
            assert st["rel_residual"] <= 1e-14, (opt, val, st)
            assert rel(dad.cache["x"], x0) < 1e-12, (opt, val)
        for opt, val in [(_lib.BEM_OPT_TC_RESERVE, -1), (_lib.BEM_OPT_TC_RESERVE, 65),
                         (_lib.BEM_OPT_SWEEP_CTAS, 0), (_lib.BEM_OPT_SWEEP_CTAS, 5), (_lib.BEM_OPT_TCGEN05, 3),
                         (_lib.BEM_OPT_NEARFIELD, 7), (_lib.BEM_OPT_NEARFIELD, -1)]:
            with pytest.raises(_lib.BemError):
                ctx.set_option(opt, val)
    finally:
        ctx.close()


def test_kernel_timeline():
    """With kernel timing on, every timed launch of a mixed solve appears in
    the timeline with its class and a non-negative duration, and the LU's
    classes lie inside its total."""
    from bem_gmsh_gb300 import _lib
    ctx = _lib.Context()
    try:
        dad = star_domain(700, p=2, seed=6)
        solve(dad, npg=16, mode="mixed", ctx=ctx)
        ctx.set_option(_lib.BEM_OPT_KERNEL_TIMING, 1)
        ctx.kernel_times()
        ctx.kernel_trace()
        solve(dad, npg=16, mode="mixed", ctx=ctx)
        tr = ctx.kernel_trace()
        ctx.set_option(_lib.BEM_OPT_KERNEL_TIMING, 0)
        assert tr and all(b >= a for _, a, b in tr)
        names = {c for c, _, _ in tr}
        assert {"lu_total", "lu_diag", "lu_panels", "lu_trail", "trsv", "gemv", "far"} <= names, names
        tot = [(a, b) for c, a, b in tr if c == "lu_total"]
        assert len(tot) == 1
        t0, t1 = tot[0]
        for c, a, b in tr:
            if c in ("lu_diag", "lu_panels", "lu_trail", "lu_thin"):
                assert t0 - 1e-3 <= a and b <= t1 + 1e-3, (c, a, b, t0, t1)
        assert ctx.kernel_trace() == []
    finally:
        ctx.close()
