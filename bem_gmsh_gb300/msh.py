"""Gmsh mesh files (ASCII formats 4.1 and 2.2) for the 2-D boundary path.

The reference reads a Gmsh model through the Gmsh API in `format2d`
(src/Core/Input.jl:136-197): the 1-D line elements of the boundary, their
physical-group names as boundary conditions (`_entity_bc`, :274-281,
`parse_pairs`, :564-582) and the 2-D cells that orient the normals and give
the internal points (`_gmsh_domain_cells`, :391-412).  Gmsh itself is not a
dependency here; this module reads the same information from the file.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# 1-D Gmsh element types: order and the node order that makes the nodes
# equispaced along the element (Gmsh lists both end nodes first)
# (`_gmsh_line_layout`, src/Core/Input.jl:253-267)
LINE_TYPES = {1: 1, 8: 2, 26: 3, 27: 4, 28: 5}
# 2-D types: number of corner nodes among the element's nodes
# (`_cell_corners`, src/Core/Input.jl:302-317)
CELL_CORNERS = {2: 3, 9: 3, 20: 3, 21: 3, 22: 3, 23: 3, 3: 4, 10: 4, 16: 4, 36: 4}
# nodes per element of the Gmsh element types a 2-D mesh file holds (points,
# lines, triangles, quadrangles; from the Gmsh file format documentation)
NODES_PER_TYPE = {15: 1, 1: 2, 8: 3, 26: 4, 27: 5, 28: 6, 2: 3, 9: 6, 20: 9, 21: 10, 22: 12, 23: 15,
                  3: 4, 16: 8, 10: 9, 36: 16}


@dataclass
class MshMesh:
    """What `format2d` needs from a mesh file."""
    lines: np.ndarray            # (ne, p + 1, 2) line element nodes, equispaced order
    line_type: int               # Gmsh type of the line elements
    line_entity: np.ndarray      # (ne,) curve (entity) tag of each line element
    cells: list = field(default_factory=list)   # corner arrays (3 or 4, 2) of the 2-D elements
    names: dict = field(default_factory=dict)   # curve tag -> physical name of its first group

    @property
    def order(self) -> int:
        return LINE_TYPES[self.line_type]


def line_reorder(order: int):
    """Gmsh node order of a line element -> equispaced order: end 0, the
    interior nodes, end 1."""
    n = order + 1
    return [0] + list(range(2, n)) + [1] if n >= 3 else [0, 1]


def parse_pairs(s: str):
    """Boundary condition pairs of a physical name, "type;value;type;value..."
    (`parse_pairs`, src/Core/Input.jl:564-582): a bare label means (1, 0)."""
    parts = [p.strip() for p in s.split(";") if p.strip()]
    try:
        int(parts[0])
        ok = len(parts) >= 2
    except (ValueError, IndexError):
        ok = False
    if not ok:
        return [1], [0.0]
    npair = len(parts) // 2
    ints, floats = [], []
    for k in range(npair):
        try:
            ints.append(int(parts[2 * k]))
            floats.append(float(parts[2 * k + 1]))
        except ValueError:
            raise ValueError(f"Bad BC pair in '{s}'") from None
    return ints, floats


def _tokens(text):
    return text.split()


def read_msh(path: str) -> MshMesh:
    """Read a Gmsh ASCII mesh (format 4.1 or 2.2)."""
    with open(path, "r", encoding="utf-8") as f:
        txt = f.read()
    sections = {}
    pos = 0
    while True:
        a = txt.find("$", pos)
        if a < 0:
            break
        b = txt.find("\n", a)
        name = txt[a + 1:b].strip()
        end = txt.find("$End" + name, b)
        if end < 0:
            raise ValueError(f"{path}: section ${name} is not closed")
        sections[name] = txt[b + 1:end]
        pos = end + len(name) + 4
    if "MeshFormat" not in sections:
        raise ValueError(f"{path}: no $MeshFormat")
    fmt = _tokens(sections["MeshFormat"])
    version, ftype = fmt[0], int(fmt[1])
    if ftype != 0:
        raise ValueError(f"{path}: binary mesh files are not supported (ASCII only)")
    phys = {}
    if "PhysicalNames" in sections:
        lines = sections["PhysicalNames"].strip().splitlines()
        for ln in lines[1:]:
            d, t, nm = ln.split(None, 2)
            phys[(int(d), int(t))] = nm.strip().strip('"')
    if version.startswith("4"):
        return _read_v4(sections, phys, path)
    if version.startswith("2"):
        return _read_v2(sections, phys, path)
    raise ValueError(f"{path}: unsupported mesh format version {version}")


def _finish(line_rows, line_type, cells, names, path):
    if not line_rows:
        raise ValueError(f"{path}: no 1-D line elements")
    order = LINE_TYPES[line_type]
    ro = line_reorder(order)
    pts = np.array([[xy for xy in r[1]] for r in line_rows], dtype=np.float64)[:, ro, :]
    ent = np.array([r[0] for r in line_rows], dtype=np.int64)
    return MshMesh(lines=pts, line_type=line_type, line_entity=ent, cells=cells, names=names)


def _read_v4(sec, phys, path):
    # entities: physical tags of the curves (dim 1)
    names = {}
    if "Entities" in sec:
        t = _tokens(sec["Entities"])
        i = 0
        npt, ncu, nsu, nvo = (int(x) for x in t[i:i + 4])
        i += 4
        for _ in range(npt):
            # tag x y z numPhysicalTags physicalTag...
            nphys = int(t[i + 4])
            i += 5 + nphys
        for _ in range(ncu):
            tag = int(t[i])
            nphys = int(t[i + 7])
            ptags = [int(x) for x in t[i + 8:i + 8 + nphys]]
            i += 8 + nphys
            nb = int(t[i])
            i += 1 + nb
            if ptags:
                names[tag] = phys.get((1, abs(ptags[0])), "")
        # surfaces and volumes are not needed
    # nodes
    t = _tokens(sec["Nodes"])
    nblk = int(t[0])
    i = 4
    coords = {}
    for _ in range(nblk):
        parametric = int(t[i + 2])
        nn = int(t[i + 3])
        i += 4
        tags = [int(x) for x in t[i:i + nn]]
        i += nn
        stride = 3
        if parametric:
            raise ValueError(f"{path}: parametric node coordinates are not supported")
        for k in range(nn):
            coords[tags[k]] = (float(t[i + stride * k]), float(t[i + stride * k + 1]))
        i += stride * nn
    # elements
    t = _tokens(sec["Elements"])
    nblk = int(t[0])
    i = 4
    line_rows, cells, ltype = [], [], None
    for _ in range(nblk):
        edim, etag, etype, ne = (int(x) for x in t[i:i + 4])
        i += 4
        npe = NODES_PER_TYPE.get(etype)
        if npe is None:
            raise ValueError(f"{path}: unsupported Gmsh element type {etype}")
        for k in range(ne):
            nodes = [int(x) for x in t[i + 1:i + 1 + npe]]
            i += 1 + npe
            if edim == 1 and etype in LINE_TYPES:
                if ltype is None:
                    ltype = etype
                if etype != ltype:
                    raise ValueError(f"{path}: mixed 1-D element orders")
                line_rows.append((etag, [coords[n] for n in nodes]))
            elif edim == 2 and etype in CELL_CORNERS:
                cells.append(np.array([coords[n] for n in nodes[:CELL_CORNERS[etype]]]))
    return _finish(line_rows, ltype, cells, names, path)


def _read_v2(sec, phys, path):
    t = _tokens(sec["Nodes"])
    nn = int(t[0])
    coords = {}
    for k in range(nn):
        coords[int(t[1 + 4 * k])] = (float(t[2 + 4 * k]), float(t[3 + 4 * k]))
    t = _tokens(sec["Elements"])
    ne = int(t[0])
    i = 1
    line_rows, cells, ltype = [], [], None
    names = {}
    for _ in range(ne):
        etype, ntags = int(t[i + 1]), int(t[i + 2])
        tags = [int(x) for x in t[i + 3:i + 3 + ntags]]
        npe = NODES_PER_TYPE.get(etype)
        if npe is None:
            raise ValueError(f"{path}: unsupported Gmsh element type {etype}")
        nodes = [int(x) for x in t[i + 3 + ntags:i + 3 + ntags + npe]]
        i += 3 + ntags + npe
        ptag = tags[0] if ntags >= 1 else 0
        etag = tags[1] if ntags >= 2 else ptag
        if etype in LINE_TYPES:
            if ltype is None:
                ltype = etype
            if etype != ltype:
                raise ValueError(f"{path}: mixed 1-D element orders")
            line_rows.append((etag, [coords[n] for n in nodes]))
            if ptag and etag not in names:
                names[etag] = phys.get((1, ptag), "")
        elif etype in CELL_CORNERS:
            cells.append(np.array([coords[n] for n in nodes[:CELL_CORNERS[etype]]]))
    return _finish(line_rows, ltype, cells, names, path)
