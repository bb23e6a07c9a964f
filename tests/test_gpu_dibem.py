"""Pairwise DIBEM matrices on the GPU (bem_dibem_fd2d) against the oracle."""
import numpy as np
import pytest

from bem_gmsh_gb300 import star_domain, quadrado, Elasticity
from bem_gmsh_gb300.geometry import plate_with_hole
from bem_gmsh_gb300.api import dibem_fd

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rbf", ["PHS1", "PHS2", "PHS3", "PHS6", "fundamental"])
def test_laplace_fd_matches_oracle(orc, rbf):
    from bem_gmsh_gb300.api import RBF_KINDS
    dad = quadrado(ndiv=9, pontointerno=True)
    F, D = dibem_fd(dad, rbf=rbf)
    Fr, Dr = orc.dibem_fd(dad.collocation, kind=0, prm0=1.0, rbf=RBF_KINDS[rbf])
    assert np.max(np.abs(F - Fr)) <= 1e-14 * np.max(np.abs(Fr))
    assert np.max(np.abs(D - Dr)) <= 1e-14 * np.max(np.abs(Dr))
    F32, D32 = dibem_fd(dad, rbf=rbf, dtype=np.float32)
    assert np.max(np.abs(F32 - Fr)) <= 1e-5 * np.max(np.abs(Fr))
    assert np.max(np.abs(D32 - Dr)) <= 1e-5 * np.max(np.abs(Dr))


def test_kelvin_fd_matches_oracle(orc):
    dad = plate_with_hole(n_outer_el=40, n_hole_el=12, p=2, sigma=1.0, props=Elasticity(1.0, 0.3, 1.0))
    F, D = dibem_fd(dad, rbf="PHS3")
    Fr, Dr = orc.dibem_fd(dad.collocation, kind=1, prm0=dad.properties.mu, prm1=dad.properties.nu_eff, rbf=3)
    assert np.max(np.abs(F - Fr)) <= 1e-14 * np.max(np.abs(Fr))
    assert np.max(np.abs(D - Dr)) <= 1e-14 * np.max(np.abs(Dr))


def test_large_star_fp32():
    dad = star_domain(1000, p=2, seed=1)
    F, D = dibem_fd(dad, rbf="PHS3", dtype=np.float32)
    assert F.shape == (3000, 3000) and np.isfinite(F).all() and np.isfinite(D).all()
    np.testing.assert_allclose(F, F.T, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("rbf", ["PHS1", "PHS3", "PHS6", "fundamental"])
def test_ifid_matches_oracle(orc, rbf):
    from bem_gmsh_gb300.api import RBF_KINDS, dibem_ifid
    dad = star_domain(400, p=2, seed=3, pontointerno=True)
    IF, ID = dibem_ifid(dad, rbf=rbf)
    IFr, IDr = orc.dibem_ifid(dad, rbf=RBF_KINDS[rbf])
    assert np.max(np.abs(IF - IFr)) <= 1e-12 * np.max(np.abs(IFr))
    assert np.max(np.abs(ID - IDr)) <= 1e-12 * np.max(np.abs(IDr))
    IF32, ID32 = dibem_ifid(dad, rbf=rbf, dtype=np.float32)
    assert np.max(np.abs(IF32 - IFr)) <= 1e-4 * np.max(np.abs(IFr))
    assert np.max(np.abs(ID32 - IDr)) <= 1e-4 * np.max(np.abs(IDr))


def test_ifid_radial_integration_identity_on_device():
    """At the centre of the unit disc IF -> 2 pi / 5 (PHS3) and ID -> 1 / 4."""
    from bem_gmsh_gb300.api import dibem_ifid
    from bem_gmsh_gb300.geometry import from_cad
    from bem_gmsh_gb300 import Laplace
    ne = 512
    th = 2 * np.pi * (np.arange(ne)[:, None] + np.arange(3)[None, :] / 2) / ne
    cad = np.stack([np.cos(th), np.sin(th)], -1)
    dad = from_cad("circle", cad, 2, Laplace(1.0), np.ones((ne, 1), np.int32), np.zeros((ne, 1)),
                   internal=[[0.0, 0.0]])
    IF, ID = dibem_ifid(dad, rbf="PHS3")
    assert IF[-1] == pytest.approx(2 * np.pi / 5, rel=1e-9)
    assert ID[-1] == pytest.approx(0.25, rel=1e-12)


@pytest.mark.parametrize("rbf", ["PHS3", "PHS1"])
def test_ifid_near_correction_matches_oracle(orc, rbf):
    """Far sums plus the near-pair Gauss-rule correction (bem_dibem_ifid_near2d,
    replacing `_dibem_correct_near_cpu!`) against the oracle's restatement, on
    a curved quadratic boundary with internal points close to it."""
    from bem_gmsh_gb300.api import RBF_KINDS, dibem_ifid
    from bem_gmsh_gb300 import star_domain
    from bem_gmsh_gb300.geometry import from_cad
    d0 = star_domain(90, p=2, seed=4)
    inner = d0.collocation[::7] - 0.02 * d0.normal[::7]
    cad = d0.geo
    dad = from_cad("star", cad, 2, d0.properties, np.ones((90, 1), np.int32), np.zeros((90, 1)), internal=inner)
    IF, ID = dibem_ifid(dad, rbf=rbf, near=True)
    IFr, IDr = orc.dibem_ifid(dad, rbf=RBF_KINDS[rbf])
    IFr, IDr = orc.dibem_ifid_near(dad, IFr, IDr, rbf=RBF_KINDS[rbf])
    assert np.max(np.abs(IF - IFr)) <= 1e-12 * np.max(np.abs(IFr))
    assert np.max(np.abs(ID - IDr)) <= 1e-12 * np.max(np.abs(IDr))


def test_ifid_near_correction_radial_integration_identity():
    """Unit disc, points 0.005 to 0.1 inside the circle: with the correction,
    IF (PHS3) and ID are the domain integrals of R^3 and of the fundamental
    solution, int over the disc of |y - x|^3 dy and (1 - |x|^2) / 4, far more
    closely than the lumped far sums alone."""
    from bem_gmsh_gb300.api import dibem_ifid
    from bem_gmsh_gb300.geometry import from_cad
    from bem_gmsh_gb300 import Laplace
    ne = 128
    th = 2 * np.pi * (np.arange(ne)[:, None] + np.arange(3)[None, :] / 2) / ne
    cad = np.stack([np.cos(th), np.sin(th)], -1)
    rad = 1.0 - np.array([0.005, 0.01, 0.02, 0.05, 0.1])
    ang = np.array([0.1, 1.3, 2.2, 3.9, 5.1])
    pts = np.stack([rad * np.cos(ang), rad * np.sin(ang)], -1)
    dad = from_cad("circle", cad, 2, Laplace(1.0), np.ones((ne, 1), np.int32), np.zeros((ne, 1)), internal=pts)
    IF0, ID0 = dibem_ifid(dad, rbf="PHS3")
    IF, ID = dibem_ifid(dad, rbf="PHS3", near=True)
    t = np.linspace(0, 2 * np.pi, 20001)[:-1]
    u = np.stack([np.cos(t), np.sin(t)], -1)
    exact_F, exact_D = [], []
    for x0 in pts:
        a = u @ x0
        rho = -a + np.sqrt(a * a + 1 - x0 @ x0)
        exact_F.append(np.mean(rho ** 5 / 5) * 2 * np.pi)
        exact_D.append((1 - x0 @ x0) / 4)
    eF = np.abs(IF[-5:] - exact_F) / np.abs(exact_F)
    eD = np.abs(ID[-5:] - exact_D) / np.abs(exact_D)
    eF0 = np.abs(IF0[-5:] - exact_F) / np.abs(exact_F)
    eD0 = np.abs(ID0[-5:] - exact_D) / np.abs(exact_D)
    print("IF rel err near/far-only:", eF, eF0, "ID:", eD, eD0)
    assert np.all(eF < 1e-6) and np.all(eD < 1e-6)
    assert eD.max() < 0.1 * eD0.max()
