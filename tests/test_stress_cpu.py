"""Boundary strain/stress recovery (Kane) in the oracle, pinned by the
reference's own patch test (test/elasticity.jl:193-208, 2-D part)."""
import numpy as np

from bem_gmsh_gb300 import Elasticity, quadrado_elasticity
from bem_gmsh_gb300.geometry import ana_elasticity_patch, apply_analytical_bc
from bem_gmsh_gb300.api import kirsch_static


def test_kane_patch_2d_oracle(orc):
    props = Elasticity(1.0, 0.3, 1.0)
    dad = quadrado_elasticity(ndiv=8, props=props)
    apply_analytical_bc(dad, ana_elasticity_patch(E=1.0, nu=0.3, exx=0.01))
    orc.assemble(dad, npg=12)
    orc.solve(dad)
    eps, sig = orc.strain_stress(dad)
    assert np.mean(np.abs(eps[:, 0] - 0.01)) < 0.05
    sxx = (props.lam + 2 * props.mu) * 0.01
    assert np.mean(np.abs(sig[:, 0] - sxx)) / abs(sxx) < 0.08


def test_kane_recovers_uniform_state_exactly(orc):
    """With the exact patch field given as (u, t), Kane's recovery returns
    the uniform strain and stress at every node (tangential derivative of a
    linear field, Hooke's law in the local frame)."""
    props = Elasticity(2.0, 0.25, 1.0)
    dad = quadrado_elasticity(ndiv=6, ordem=2, props=props)
    exx, eyy, gxy = 0.01, -0.004, 0.006
    X = np.asarray(dad.collocation[: dad.n])
    Nrm = np.asarray(dad.normal)
    u = np.empty(2 * dad.n)
    u[0::2] = exx * X[:, 0] + 0.5 * gxy * X[:, 1]
    u[1::2] = 0.5 * gxy * X[:, 0] + eyy * X[:, 1]
    lam, mu = props.lam, props.mu
    sxx, syy, sxy = lam * (exx + eyy) + 2 * mu * exx, lam * (exx + eyy) + 2 * mu * eyy, mu * gxy
    t = np.empty(2 * dad.n)
    t[0::2] = sxx * Nrm[:, 0] + sxy * Nrm[:, 1]
    t[1::2] = sxy * Nrm[:, 0] + syy * Nrm[:, 1]
    eps, sig = orc.strain_stress(dad, u, t)
    np.testing.assert_allclose(eps, np.tile([exx, eyy, gxy], (dad.n, 1)), atol=1e-12)
    np.testing.assert_allclose(sig, np.tile([sxx, syy, sxy], (dad.n, 1)), atol=1e-12 * abs(sxx))


def test_kirsch_formula():
    srr, stt, srt = kirsch_static(1.0, np.pi / 2, a=1.0, sigma_inf=2.0)
    assert abs(stt - 6.0) < 1e-14 and abs(srr) < 1e-14 and abs(srt) < 1e-14
    _, stt0, _ = kirsch_static(1.0, 0.0, a=1.0, sigma_inf=2.0)
    assert abs(stt0 + 2.0) < 1e-14
    srr, stt, srt = kirsch_static(1e6, 0.3, a=1.0, sigma_inf=1.0)  # far field: sigma_xx only
    assert abs(srr - np.cos(0.3) ** 2) < 1e-9 and abs(stt - np.sin(0.3) ** 2) < 1e-9


def test_large_plate_kirsch_oracle(orc):
    """The oracle's Kelvin solve + Kane recovery on a hole r = 0.3 in a
    40 x 40 plate reproduces the infinite-plate Kirsch hoop stress."""
    from bem_gmsh_gb300.geometry import plate_with_hole
    from bem_gmsh_gb300.api import hoop_stress
    dad = plate_with_hole(n_outer_el=256, n_hole_el=86, p=2, half=20.0, radius=0.3, sigma=1.0)
    orc.assemble(dad, npg=16)
    orc.solve(dad)
    eps, sig = orc.strain_stress(dad)
    hole = np.arange(dad.n - 3 * 86, dad.n)
    X = np.asarray(dad.collocation[hole])
    th = np.arctan2(X[:, 1], X[:, 0])
    _, kir, _ = kirsch_static(0.3, th, a=0.3, sigma_inf=1.0)
    assert np.max(np.abs(hoop_stress(dad, sigma=sig)[hole] - kir)) < 0.01
