"""Adjoint shape gradient (bem_adjoint_laplace2d) against central finite
differences (h = 1e-6) of the FP64 oracle pipeline: assemble + applyBC +
LAPACK LU on the node-interpolant geometry, boundary data and target fixed
(config C5)."""
import numpy as np
import pytest

from bem_gmsh_gb300 import Laplace, from_nodes, star_adjoint_case
from bem_gmsh_gb300.api import adjoint_laplace, solve

pytestmark = pytest.mark.gpu


def oracle_J(orc, X, p, BC, BV, qt, npg):
    dad = from_nodes("fd", X, p, Laplace(1.0), BC, BV)
    H, G = orc.assemble(dad, npg=npg, store=False)
    A, b = orc.apply_bc(dad, H, G)
    u = orc.lu_solve(A, b)
    d = BC == 0
    return 0.5 * float(np.sum((u[d] - qt[d]) ** 2))


def target_q(orc, target):
    H, G = orc.assemble(target, npg=16, store=False)
    A, b = orc.apply_bc(target, H, G)
    u = orc.lu_solve(A, b)
    return np.where(target.BC == 0, u, 0.0)


def fd_grad(orc, dad, qt, coords, h=1e-6, npg=16):
    p = dad.p
    X0 = np.asarray(dad.collocation).reshape(dad.ne, p + 1, 2)
    g = np.zeros(len(coords))
    for t, (j, d) in enumerate(coords):
        Xp = X0.copy()
        Xm = X0.copy()
        Xp.reshape(-1, 2)[j, d] += h
        Xm.reshape(-1, 2)[j, d] -= h
        g[t] = (oracle_J(orc, Xp, p, dad.BC, dad.BV, qt, npg) - oracle_J(orc, Xm, p, dad.BC, dad.BV, qt, npg)) / (2 * h)
    return g


def test_adjoint_gradient_small_all_coordinates(orc):
    dad, target = star_adjoint_case(14, p=2, seed=3)
    qt = target_q(orc, target)
    J, grad = adjoint_laplace(dad, qt, npg=16)
    J_ref = oracle_J(orc, np.asarray(dad.collocation).reshape(dad.ne, 3, 2), 2, dad.BC, dad.BV, qt, 16)
    assert abs(J - J_ref) <= 1e-8 * J_ref
    coords = [(j, d) for j in range(dad.n) for d in range(2)]
    g_fd = fd_grad(orc, dad, qt, coords)
    g = grad.reshape(-1)
    err = np.linalg.norm(g - g_fd) / np.linalg.norm(g_fd)
    assert err < 1e-5, err
    assert np.max(np.abs(g - g_fd)) < 1e-4 * np.max(np.abs(g_fd))


def test_adjoint_gradient_c5_domain_sampled(orc):
    """One C5 domain (341 quadratic elements, 1023 nodes): sampled
    coordinates, among them the largest gradient components."""
    dad, target = star_adjoint_case(341, p=2, seed=5)
    qt = target_q(orc, target)
    J, grad = adjoint_laplace(dad, qt, npg=16)
    g = grad.reshape(-1)
    rng = np.random.default_rng(0)
    # 1049 and 752: near pairs whose near-field map switches branch within
    # 1e-5 element lengths of this shape (a plain central difference there
    # picked up the jump)
    idx = [1049, 752] + list(np.argsort(-np.abs(g))[:4]) + list(rng.choice(2 * dad.n, 6, replace=False))
    coords = [(int(i) // 2, int(i) % 2) for i in idx]
    g_fd = fd_grad(orc, dad, qt, coords)
    scale = np.max(np.abs(g))
    assert np.max(np.abs(g[idx] - g_fd)) < 1e-5 * scale, (g[idx], g_fd)


def test_adjoint_batch_matches_single_calls():
    from bem_gmsh_gb300.api import adjoint_laplace_batch
    cases = [star_adjoint_case(n_el, p=2, seed=s) for s, n_el in enumerate((40, 75, 21, 60, 33))]
    qts = []
    for _, tg in cases:
        solve(tg, npg=16, mode="mixed")
        qts.append(np.where(tg.BC == 0, tg.cache["x"], 0.0))
    pairs = [(d, q) for (d, _), q in zip(cases, qts)]
    out, st = adjoint_laplace_batch(pairs, npg=16, nworkers=3, return_stats=True)
    assert len(out) == len(pairs) and all(s["status"] == 0 for s in st)
    for (d, q), (J, g) in zip(pairs, out):
        J1, g1 = adjoint_laplace(d, q, npg=16)
        assert g.shape == (d.n, 2)
        # same kernels per domain; row sums use FP64 atomics, so agree to rounding
        assert abs(J - J1) <= 1e-10 * max(abs(J1), 1e-300)
        assert np.linalg.norm(g - g1) <= 1e-9 * np.linalg.norm(g1)


def test_rrule_call_sequence(orc):
    """The call sequence of the Julia ChainRulesCore rrule,
    through its Python mirror: the primal equals the rrule's value, the
    pullback scales the gradient by the incoming cotangent, and a tangent V
    contracted with the pullback's output -- what reverse-mode AD does for
    theta -> J(X0 + theta V) -- matches central differences (h = 1e-6) of
    the FP64 oracle."""
    from bem_gmsh_gb300.api import shape_misfit, shape_misfit_rrule
    dad, target = star_adjoint_case(20, p=2, seed=7)
    qt = target_q(orc, target)
    X0 = np.asarray(dad.collocation).copy()
    J, pb = shape_misfit_rrule(X0, 2, dad.BC, dad.BV, qt)
    # the same value as the primal (to rounding: the row sums are FP64 atomics)
    assert abs(J - shape_misfit(X0, 2, dad.BC, dad.BV, qt)) <= 1e-12 * J
    g1 = pb(1.0)
    assert g1.shape == X0.shape
    assert np.array_equal(pb(2.5), 2.5 * g1)
    # a smooth tangent: radial bulge cos(3 theta)
    th = np.arctan2(X0[:, 1], X0[:, 0])
    V = (np.cos(3 * th))[:, None] * X0 / np.linalg.norm(X0, axis=1)[:, None]
    dJ = float(np.sum(g1 * V))
    h = 1e-6
    Jp = oracle_J(orc, (X0 + h * V).reshape(dad.ne, 3, 2), 2, dad.BC, dad.BV, qt, 16)
    Jm = oracle_J(orc, (X0 - h * V).reshape(dad.ne, 3, 2), 2, dad.BC, dad.BV, qt, 16)
    fd = (Jp - Jm) / (2 * h)
    assert abs(dJ - fd) <= 1e-5 * abs(fd), (dJ, fd)
