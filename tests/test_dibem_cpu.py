"""Pairwise DIBEM matrices in the oracle (`_dibem_FD_kernel!`,
src/Laplace/DIBEM_GPU.jl:194-208; `_elast_dibem_FD_kernel!`,
src/Elasticity/Assembly_GPU.jl:258-280): closed-form entries and symmetry."""
import math

import numpy as np
import pytest


@pytest.mark.parametrize("rbf,phi", [
    (1, lambda R: R), (2, lambda R: R * R * math.log(R + 1e-16)), (3, lambda R: R ** 3),
    (4, lambda R: R ** 4 * math.log(R + 1e-16)), (5, lambda R: R ** 5),
    (6, lambda R: R ** 6 * math.log(R + 1e-16)), (7, lambda R: R ** 7),
    (10, lambda R: -math.log(R) / (2 * math.pi * 2.0)),
])
def test_laplace_entries(orc, rbf, phi):
    pts = np.array([[0.0, 0.0], [2.0, 0.0], [0.5, 1.5]])
    F, D = orc.dibem_fd(pts, kind=0, prm0=2.0, rbf=rbf)
    R = 2.0
    assert F[0, 1] == pytest.approx(phi(R), rel=1e-15)
    assert D[0, 1] == pytest.approx(-math.log(R) / (2 * math.pi) / 2.0, rel=1e-15)
    assert np.all(np.diag(F) == 0) and np.all(np.diag(D) == 0)
    np.testing.assert_allclose(F, F.T, rtol=1e-15)
    np.testing.assert_allclose(D, D.T, rtol=1e-15)


def test_kelvin_blocks(orc):
    mu, nu = 80.0, 0.3
    pts = np.array([[0.0, 0.0], [0.6, 0.8], [-1.0, 0.5], [0.2, -0.7]])
    F, D = orc.dibem_fd(pts, kind=1, prm0=mu, prm1=nu, rbf=3)
    assert D.shape == (8, 8) and F.shape == (4, 4)
    # block (0, 1): r = (0.6, 0.8), R = 1
    base = 2 * 4 * math.pi * (1 - nu) * mu
    assert D[0, 2] == pytest.approx(0.36 / base, rel=1e-14)
    assert D[0, 3] == pytest.approx(0.48 / base, rel=1e-14)
    assert D[1, 3] == pytest.approx(0.64 / base, rel=1e-14)
    np.testing.assert_allclose(D, D.T, rtol=1e-14, atol=0)


def _circle(ne, centre=True):
    from bem_gmsh_gb300.geometry import from_cad
    from bem_gmsh_gb300 import Laplace
    th = 2 * np.pi * (np.arange(ne)[:, None] + np.arange(3)[None, :] / 2) / ne
    cad = np.stack([np.cos(th), np.sin(th)], -1)
    return from_cad("circle", cad, 2, Laplace(1.0), np.ones((ne, 1), np.int32), np.zeros((ne, 1)),
                    internal=[[0.0, 0.0]] if centre else None)


@pytest.mark.parametrize("rbf,exact", [(1, 2 * math.pi / 3), (3, 2 * math.pi / 5), (5, 2 * math.pi / 7)])
def test_ifid_radial_integration_identity(orc, rbf, exact):
    """IF and ID are boundary forms of domain integrals (radial integration):
    at the centre of the unit disc IF -> int phi(R) = 2 pi / (m + 2) for
    phi = R^m, and ID -> int u* = 1 / (4 k)."""
    IF, ID = orc.dibem_ifid(_circle(256), rbf=rbf)
    assert IF[-1] == pytest.approx(exact, rel=1e-8)
    assert ID[-1] == pytest.approx(0.25, rel=1e-12)


def test_ifid_skips_near_and_own_elements(orc):
    """Brute-force restatement with the oracle's own near mask."""
    dad = _circle(24)
    IF, ID = orc.dibem_ifid(dad, rbf=3, near_factor=1.5)
    mask = orc.near_mask(dad, near_factor=1.5)
    pts = np.asarray(dad.collocation)
    nrm = np.asarray(dad.normal)
    w = np.asarray(dad.jacobian) * np.tile(np.asarray(dad.elem_weight), dad.n // 3)
    IFb = np.zeros(dad.nt)
    for i in range(dad.nt):
        for j in range(dad.n):
            e = j // 3
            if mask[i, e] or (3 * e <= i < 3 * e + 3):
                continue
            r = pts[j] - pts[i]
            R = np.hypot(*r)
            if R > 1e-10:
                IFb[i] += R ** 5 / 5 * w[j] * (r @ nrm[j]) / R ** 2
    np.testing.assert_allclose(IF, IFb, rtol=1e-12, atol=1e-15)
    assert mask.sum() > 0 and np.isfinite(ID).all()
