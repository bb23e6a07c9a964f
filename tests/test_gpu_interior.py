"""Interior potential on the GPU (bem_interior_laplace2d) against the oracle,
the reference's near-field approach test, and a curved domain against the
analytic field."""
import numpy as np
import pytest

from bem_gmsh_gb300 import quadrado, star_domain, internal_grid
from bem_gmsh_gb300.geometry import ana_laplace_linear, ana_laplace_expcos, attach_analytical
from bem_gmsh_gb300.api import solve, interior_laplace

pytestmark = pytest.mark.gpu


def test_interior_matches_oracle(orc):
    dad = star_domain(200, p=2, seed=9)
    orc.assemble(dad, npg=16)
    orc.solve(dad)
    T, q = dad.cache["T"], dad.cache["q"]
    pts = internal_grid(dad, 12, 12)
    pts = np.concatenate([pts, [[0.0, 0.0]]])
    ref = orc.interior_laplace(dad, pts, npg=16, T=T, q=q)
    got = interior_laplace(dad, pts, npg=16, T=T, q=q)
    # per point within 1e-11 of the largest value: the near-field map is the
    # oracle's to the bit (correctly rounded atan / tan, same IEEE operations),
    # what remains is the rounding of the kernel sums
    scale = np.max(np.abs(ref))
    err = np.abs(got - ref) / scale
    print(f"interior: max {err.max():.2e} of the largest value")
    assert np.all(err <= 1e-11), err.max()
    # almost every point agrees to rounding
    assert np.mean(err <= 1e-13) > 0.9


@pytest.mark.parametrize("nearfield", ["euclid", "csinh", "sinhsinh", "plain"])
def test_interior_with_other_near_maps_matches_oracle(orc, nearfield):
    """The near-field map chosen by the problem's `nearfield` also drives the
    interior integrals (src/Laplace/Lubrication.jl:399-416 through
    `transform`): the GPU and the oracle with the same map, points down to
    1e-3 from the boundary."""
    dad = star_domain(200, p=2, seed=9)
    orc.assemble(dad, npg=16)
    orc.solve(dad)
    T, q = dad.cache["T"], dad.cache["q"]
    pts = np.concatenate([internal_grid(dad, 8, 8), [[0.0, 0.0]], 0.999 * dad.collocation[::37]])
    ref = orc.interior_laplace(dad, pts, npg=16, nearfield=nearfield, T=T, q=q)
    got = interior_laplace(dad, pts, npg=16, T=T, q=q, nearfield=nearfield)
    err = np.abs(got - ref) / np.max(np.abs(ref))
    print(f"interior {nearfield}: max {err.max():.2e} of the largest value")
    assert np.all(err <= 1e-11), err.max()


def test_interior_approach_gpu():
    """test/laplace.jl:55-86 (tanp3c): |T(0.5, d) - 0.5| < 5e-3, d -> 1e-6."""
    dad = quadrado(ndiv=20, pontointerno=False)
    attach_analytical(dad, ana_laplace_linear((1.0, 0.0)))
    solve(dad, npg=16, mode="fp64")
    ds = [1e-1, 1e-2, 1e-3, 1e-4, 1e-5, 1e-6]
    T = interior_laplace(dad, [[0.5, d] for d in ds], npg=16)
    assert np.max(np.abs(T - 0.5)) < 5e-3, T


def test_interior_star_analytic():
    """Curved quadratic boundary, T = e^x cos y: interior values from the
    mixed-precision solve follow the analytic field."""
    dad = star_domain(900, p=2, seed=2)
    ana = ana_laplace_expcos()
    solve(dad, npg=16, mode="mixed")
    pts = internal_grid(dad, 20, 20, d_min=0.5)
    T = interior_laplace(dad, pts, npg=16)
    exact = np.exp(pts[:, 0]) * np.cos(pts[:, 1])
    assert np.max(np.abs(T - exact)) < 5e-4 * np.max(np.abs(exact))
