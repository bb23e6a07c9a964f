"""Interior points: grid generation (src/Core/InternalPoints.jl) and the
oracle's interior potential, pinned by the reference's near-field approach
test (test/laplace.jl:55-86, T at (0.5, d) for d -> 0)."""
import numpy as np

from bem_gmsh_gb300 import quadrado, star_domain, internal_grid, point_in_domain
from bem_gmsh_gb300.geometry import ana_laplace_linear, attach_analytical


def test_point_in_domain_and_grid():
    dad = quadrado(ndiv=11, pontointerno=False)
    inside = point_in_domain(dad, [[0.5, 0.5], [1.5, 0.5], [-0.1, 0.2], [0.999, 0.001]])
    assert list(inside) == [True, False, False, True]
    pts = internal_grid(dad, 9, 9, d_min=0.0)
    # gera layout: i / (n + 1) on the unit square, all inside
    assert pts.shape == (81, 2)
    np.testing.assert_allclose(np.unique(pts[:, 0]), np.arange(1, 10) / 10, atol=1e-15)
    # clearance drops the ring nearest the boundary
    L = float(np.max(dad.elem_length))
    pts2 = internal_grid(dad, 9, 9, d_min=1.01 * 0.1 / L)
    assert pts2.shape == (49, 2)
    star = star_domain(300, p=2, seed=4)
    sp = internal_grid(star, 15, 15)
    assert len(sp) > 60 and np.all(point_in_domain(star, sp))


def test_interior_potential_approach_oracle(orc):
    """test/laplace.jl:55-86, tanp3c map: |T(0.5, d) - 0.5| < 5e-3 for
    d = 1e-1 .. 1e-6 on quadrado(ndiv=20), T = x."""
    dad = quadrado(ndiv=20, pontointerno=False)
    attach_analytical(dad, ana_laplace_linear((1.0, 0.0)))  # builder BCs are those of T = x
    orc.assemble(dad, npg=16)
    orc.solve(dad)
    ds = [1e-1, 1e-2, 1e-3, 1e-4, 1e-5, 1e-6]
    T = orc.interior_laplace(dad, [[0.5, d] for d in ds], npg=16)
    assert np.max(np.abs(T - 0.5)) < 5e-3, T
