"""Gmsh mesh files for `format2d` (src/Core/Input.jl:136-197), on the host:
the reader (formats 4.1 and 2.2), the boundary conditions from physical names
(`parse_pairs`, :564-582) and the outward orientation of the normals by the
oracle's restatement of `_orient_normals_outward!` (:376-389)."""
import os
import tempfile

import numpy as np
import pytest

from msh_files import square_mesh, write_v41, write_v22


def _write(kind, ndiv=6, p=2, reverse=()):
    nodes, curves, cells = square_mesh(ndiv, p=p, reverse=reverse)
    d = tempfile.mkdtemp(prefix="msh_")
    path = os.path.join(d, f"square_{kind}.msh")
    (write_v41 if kind == "41" else write_v22)(path, nodes, curves, cells, p)
    return path


def test_parse_pairs():
    from bem_gmsh_gb300.msh import parse_pairs
    assert parse_pairs("1;-1") == ([1], [-1.0])
    assert parse_pairs("0;0;1;2.5") == ([0, 1], [0.0, 2.5])
    assert parse_pairs("wall") == ([1], [0.0])
    with pytest.raises(ValueError):
        parse_pairs("1;x")


@pytest.mark.parametrize("p", [1, 2, 3])
def test_reader_formats_agree(p):
    from bem_gmsh_gb300.msh import read_msh
    a = read_msh(_write("41", p=p))
    b = read_msh(_write("22", p=p))
    assert a.order == b.order == p
    assert np.array_equal(a.lines, b.lines) and np.array_equal(a.line_entity, b.line_entity)
    assert a.names == b.names == {1: "1;0", 2: "1;-1", 3: "1;0", 4: "0;0"}
    assert len(a.cells) == len(b.cells) == 25
    # equispaced node order along each element
    d = np.diff(a.lines, axis=1)
    assert np.allclose(d, d[:, :1], atol=1e-15)


def test_orientation_of_reversed_curves_on_the_host(orc):
    """Curves written clockwise get inward normals from the tangents; the
    orientation flips exactly those elements, and every normal then points
    out of the unit square."""
    from bem_gmsh_gb300.msh import read_msh
    from bem_gmsh_gb300.geometry import discretize_curves
    m = read_msh(_write("41", ndiv=7, p=2, reverse=("top", "left")))
    nodes, normal, J, L, w = discretize_curves(m.lines, 2)
    nodes, normal = nodes.reshape(-1, 2), normal.reshape(-1, 2)
    out, flipped = orc.orient_normals(nodes, normal, L, 2, m.cells)
    ents = m.line_entity
    assert np.array_equal(flipped, np.isin(ents, [3, 4]))
    c = nodes - 0.5
    # outward: along the side's normal direction away from the centre
    assert np.all(np.sum(out * c, axis=1) > 0)
    out2, fl2 = orc.orient_normals(nodes, normal, L, 2, [])
    assert not fl2.any() and np.array_equal(out2, normal)  # no 2-D mesh: unchanged
