"""Gmsh ASCII mesh files (formats 4.1 and 2.2) of simple 2-D domains, written
for the tests of the mesh reader (the reference builds these with Gmsh,
e.g. `quadrado`, data/Laplace/Laplace_dad.jl:238-280)."""
import numpy as np


def square_mesh(ndiv, p=1, reverse=(), names=None):
    """Unit square: ndiv points per side (ndiv - 1 line elements of order p per
    side, curves bottom, right, top, left), (ndiv - 1)^2 quadrangle cells.
    Curves listed in `reverse` are written clockwise (their elements run
    backwards).  Returns (nodes {tag: (x, y)}, curves [(tag, name, [element
    node-tag lists in Gmsh order])], cells [node-tag lists])."""
    names = names or {"bottom": "1;0", "right": "1;-1", "top": "1;0", "left": "0;0"}
    m = ndiv - 1
    nodes = {}
    tag = [0]

    def node(x, y):
        tag[0] += 1
        nodes[tag[0]] = (float(x), float(y))
        return tag[0]

    grid = {}
    for j in range(ndiv):
        for i in range(ndiv):
            grid[i, j] = node(i / m, j / m)
    corners = [(0.0, 0.0), (1.0, 0.0), (1.0, 1.0), (0.0, 1.0)]
    sides = ["bottom", "right", "top", "left"]
    gidx = [lambda k: (k, 0), lambda k: (m, k), lambda k: (m - k, m), lambda k: (0, m - k)]
    curves = []
    for s, nm in enumerate(sides):
        a, b = np.array(corners[s]), np.array(corners[(s + 1) % 4])
        els = []
        for k in range(m):
            e0, e1 = gidx[s](k), gidx[s](k + 1)
            t0, t1 = grid[e0], grid[e1]
            inner = []
            for q in range(1, p):
                xy = a + (b - a) * (k + q / p) / m
                inner.append(node(*xy))
            els.append([t0, t1] + inner)
        if nm in reverse:
            els = [[e[1], e[0]] + e[2:][::-1] for e in els[::-1]]
        curves.append((s + 1, names[nm], els))
    cells = [[grid[i, j], grid[i + 1, j], grid[i + 1, j + 1], grid[i, j + 1]] for j in range(m) for i in range(m)]
    return nodes, curves, cells


LINE_TYPE = {1: 1, 2: 8, 3: 26}


def write_v41(path, nodes, curves, cells, p):
    lt = LINE_TYPE[p]
    with open(path, "w") as f:
        f.write("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n")
        f.write(f"$PhysicalNames\n{len(curves)}\n")
        for tag, nm, _ in curves:
            f.write(f'1 {tag} "{nm}"\n')
        f.write("$EndPhysicalNames\n")
        f.write(f"$Entities\n0 {len(curves)} 1 0\n")
        for tag, _, _ in curves:
            f.write(f"{tag} 0 0 0 1 1 0 1 {tag} 0\n")
        f.write("1 0 0 0 1 1 0 0 0\n$EndEntities\n")
        tags = sorted(nodes)
        f.write(f"$Nodes\n1 {len(tags)} 1 {max(tags)}\n2 1 0 {len(tags)}\n")
        for t in tags:
            f.write(f"{t}\n")
        for t in tags:
            f.write(f"{nodes[t][0]!r} {nodes[t][1]!r} 0\n")
        f.write("$EndNodes\n")
        nel = sum(len(e) for _, _, e in curves) + len(cells)
        f.write(f"$Elements\n{len(curves) + 1} {nel} 1 {nel}\n")
        eid = 0
        for tag, _, els in curves:
            f.write(f"1 {tag} {lt} {len(els)}\n")
            for e in els:
                eid += 1
                f.write(f"{eid} " + " ".join(map(str, e)) + "\n")
        f.write(f"2 1 3 {len(cells)}\n")
        for c in cells:
            eid += 1
            f.write(f"{eid} " + " ".join(map(str, c)) + "\n")
        f.write("$EndElements\n")


def write_v22(path, nodes, curves, cells, p):
    lt = LINE_TYPE[p]
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n")
        f.write(f"$PhysicalNames\n{len(curves)}\n")
        for tag, nm, _ in curves:
            f.write(f'1 {tag} "{nm}"\n')
        f.write("$EndPhysicalNames\n")
        tags = sorted(nodes)
        f.write(f"$Nodes\n{len(tags)}\n")
        for t in tags:
            f.write(f"{t} {nodes[t][0]!r} {nodes[t][1]!r} 0\n")
        f.write("$EndNodes\n")
        nel = sum(len(e) for _, _, e in curves) + len(cells)
        f.write(f"$Elements\n{nel}\n")
        eid = 0
        for tag, _, els in curves:
            for e in els:
                eid += 1
                f.write(f"{eid} {lt} 2 {tag} {tag} " + " ".join(map(str, e)) + "\n")
        for c in cells:
            eid += 1
            f.write(f"{eid} 3 2 100 1 " + " ".join(map(str, c)) + "\n")
        f.write("$EndElements\n")
