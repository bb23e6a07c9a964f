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
