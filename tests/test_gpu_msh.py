"""`format2d` from a Gmsh mesh file with the device steps: the geometry loop
(bem_discretize2d) and the outward orientation (bem_orient2d, replacing
`_orient_normals_outward!`, src/Core/Input.jl:376-389), against the oracle,
and a solve from the file against the same square built by `quadrado`."""
import os
import tempfile

import numpy as np
import pytest

from msh_files import square_mesh, write_v41

pytestmark = pytest.mark.gpu


def _path(ndiv, p, reverse=()):
    nodes, curves, cells = square_mesh(ndiv, p=p, reverse=reverse)
    path = os.path.join(tempfile.mkdtemp(prefix="msh_"), "square.msh")
    write_v41(path, nodes, curves, cells, p)
    return path


@pytest.mark.parametrize("p", [1, 2, 3])
def test_device_orientation_matches_oracle(orc, p):
    from bem_gmsh_gb300 import Laplace, format2d
    from bem_gmsh_gb300.msh import read_msh
    from bem_gmsh_gb300.geometry import discretize_curves
    path = _path(9, p, reverse=("right", "top"))
    dad = format2d(path, Laplace(1.0), pontointerno=False)
    m = read_msh(path)
    nodes, normal, J, L, w = discretize_curves(m.lines, p)
    ref, flipped = orc.orient_normals(nodes.reshape(-1, 2), normal.reshape(-1, 2), L, p, m.cells)
    assert flipped.sum() == 2 * 8  # the two clockwise sides
    assert np.max(np.abs(dad.normal - ref)) < 1e-13  # device vs host discretisation rounding
    assert np.max(np.abs(dad.collocation - nodes.reshape(-1, 2))) < 1e-15


def test_orientation_flags_and_many_cells():
    """More cells than one shared-memory chunk (a 40 x 40 grid): every element
    finds its cell, and the clockwise curve is the one flipped."""
    from bem_gmsh_gb300 import Laplace
    from bem_gmsh_gb300.msh import read_msh
    from bem_gmsh_gb300.geometry import from_cad
    from bem_gmsh_gb300.api import discretize, orient_normals
    m = read_msh(_path(41, 2, reverse=("left",)))
    ne = m.lines.shape[0]
    dad = from_cad("sq", m.lines, 2, Laplace(1.0), np.ones((ne, 1)), np.zeros((ne, 1)), discretize=discretize)
    flipped = orient_normals(dad, m.cells)
    assert np.array_equal(flipped, m.line_entity == 4)
    c = dad.collocation - 0.5
    assert np.all(np.sum(dad.normal * c, axis=1) > 0)


def test_solve_from_mesh_file_matches_quadrado():
    """T = x on the unit square (the reference's `quadrado` case) read from a
    mesh file with quadratic elements and internal points at the cell
    centroids: the same boundary solution as the `quadrado` builder."""
    from bem_gmsh_gb300 import Laplace, format2d, quadrado, ana_laplace_linear, attach_analytical, rel_error
    from bem_gmsh_gb300.api import solve
    dad = format2d(_path(12, 2), Laplace(1.0), pontointerno=True)
    ref = quadrado(ndiv=12, ordem=2, pontointerno=True)
    assert (dad.n, dad.nt) == (ref.n, ref.nt)
    for d in (dad, ref):
        attach_analytical(d, ana_laplace_linear())
        solve(d, npg=16, mode="mixed")
    xb, xr = dad.cache["x"][:dad.n], ref.cache["x"][:ref.n]
    assert np.linalg.norm(xb - xr) / np.linalg.norm(xr) < 1e-10
    assert rel_error(dad) < 0.05 and abs(rel_error(dad) - rel_error(ref)) < 1e-8
