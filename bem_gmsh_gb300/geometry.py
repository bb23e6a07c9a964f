"""Problem container and Gmsh-free boundary builders.

Mirrors the reference's `BEMdata` (src/Core/Structures.jl:504-519) and the
geometry `format2d` produces (src/Core/Input.jl:136-197): discontinuous
Gauss-Legendre collocation, each element owning `p+1` private nodes placed at
the Gauss points of its CAD curve, Jacobian and outward normal at each node
(`tan2normal`, src/Core/Input.jl:584), element length `|sum J w|`, the CAD
nodes kept for near/singular geometry (`Element.geo`).  The builders follow
the Gmsh-free construction pattern of `bemdata_from_loops`
(src/Topology/Topology.jl:288-333).

Builders:
  * `quadrado`            -- unit square of data/Laplace/Laplace_dad.jl:238-280
                             (`ndiv` transfinite points per side, BCs for T=x)
  * `quadrado_elasticity` -- data/Laplace/Laplace_dad.jl:289-323
  * `star_domain`         -- seeded star-shaped curve r(t)=1+sum a_k cos(k t+phi_k)
  * `plate_with_hole`     -- square plate with a central circular hole
All host-side numpy: this is input preparation, not the hot path.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np


# ---------------------------------------------------------------------------
# physics
# ---------------------------------------------------------------------------
@dataclass
class Laplace:
    """Steady heat conduction, conductivity k; flux q = -k dT/dn
    (src/Core/Structures.jl:101-103)."""
    k: float = 1.0
    ndof: int = 1


@dataclass
class Elasticity:
    """2-D isotropic elasticity (src/Core/Structures.jl:149-199).  Plane strain
    by default; plane stress maps to the effective Poisson ratio nu/(1+nu)
    (`effective_nu`, Structures.jl:260-263)."""
    E: float = 1.0
    nu: float = 0.3
    rho: float = 1.0
    plane_strain: bool = True
    ndof: int = 2

    @property
    def mu(self) -> float:
        return self.E / (2 * (1 + self.nu))

    @property
    def nu_eff(self) -> float:
        return self.nu if self.plane_strain else self.nu / (1 + self.nu)

    @property
    def lam(self) -> float:
        ne = self.nu_eff
        den = (1 + ne) * (1 - 2 * ne)
        return math.inf if abs(den) < np.finfo(float).eps else self.E * ne / den


# ---------------------------------------------------------------------------
# 1-D Lagrange bases
# ---------------------------------------------------------------------------
def gauss_legendre(n: int):
    """Gauss-Legendre nodes (ascending) and weights on [-1, 1]."""
    x, w = np.polynomial.legendre.leggauss(n)
    return np.asarray(x, dtype=np.float64), np.asarray(w, dtype=np.float64)


def lagrange_basis(nodes: np.ndarray, xi: np.ndarray):
    """Values and derivatives of the Lagrange basis on `nodes` at points `xi`.
    Returns (N, dN) with shape (len(xi), len(nodes))."""
    nodes = np.asarray(nodes, dtype=np.float64)
    xi = np.atleast_1d(np.asarray(xi, dtype=np.float64))
    m = len(nodes)
    N = np.ones((len(xi), m))
    dN = np.zeros((len(xi), m))
    for j in range(m):
        for k in range(m):
            if k == j:
                continue
            N[:, j] *= (xi - nodes[k]) / (nodes[j] - nodes[k])
        for l in range(m):
            if l == j:
                continue
            t = np.ones_like(xi) / (nodes[j] - nodes[l])
            for k in range(m):
                if k == j or k == l:
                    continue
                t = t * (xi - nodes[k]) / (nodes[j] - nodes[k])
            dN[:, j] += t
    return N, dN


def equispaced_nodes(p: int) -> np.ndarray:
    return np.array([(2 * j - p) / p for j in range(p + 1)], dtype=np.float64)


# ---------------------------------------------------------------------------
# container
# ---------------------------------------------------------------------------
@dataclass
class BEMdata:
    """Host-side problem container (reference `BEMdata`).

    Element `e` owns boundary nodes `e*(p+1) .. e*(p+1)+p`; collocation points
    are the `n` boundary nodes followed by `ni` internal points.
    """
    name: str
    p: int
    ngeo: int
    collocation: np.ndarray          # (nt, 2)
    normal: np.ndarray               # (n, 2)
    jacobian: np.ndarray             # (n,)
    elem_length: np.ndarray          # (ne,)
    geo: np.ndarray                  # (ne, ngeo, 2)
    elem_weight: np.ndarray          # (p+1,)
    properties: object
    BC: np.ndarray                   # (ndof*n,) int32, 0 = primary prescribed
    BV: np.ndarray                   # (ndof*n,)
    region: np.ndarray = None        # (ne,) int tag of the boundary piece
    cache: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return self.normal.shape[0]

    @property
    def nt(self) -> int:
        return self.collocation.shape[0]

    @property
    def ni(self) -> int:
        return self.nt - self.n

    @property
    def ne(self) -> int:
        return self.elem_length.shape[0]

    @property
    def ndof(self) -> int:
        return self.properties.ndof

    @property
    def Nodes(self) -> np.ndarray:
        return self.collocation[: self.n]

    @property
    def internalNodes(self) -> np.ndarray:
        return self.collocation[self.n:]

    def __getattr__(self, name):
        cache = self.__dict__.get("cache")
        if cache is not None and name in cache:
            return cache[name]
        raise AttributeError(f"BEMdata has no property or cache field `{name}`")

    def set_cache(self, **kw):
        self.cache.update(kw)
        return self

    def has_cache(self, key) -> bool:
        return key in self.cache

    def set_internal_nodes(self, pts):
        pts = np.asarray(pts, dtype=np.float64).reshape(-1, 2)
        self.collocation = np.vstack([self.Nodes, pts])
        self.cache.clear()
        return self

    def contiguous(self):
        for k in ("collocation", "normal", "jacobian", "elem_length", "geo", "elem_weight", "BV"):
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.float64))
        self.BC = np.ascontiguousarray(self.BC, dtype=np.int32)
        return self


def discretize_curves(cad: np.ndarray, p: int):
    """Collocation nodes, Jacobians, normals and lengths for elements given by
    their equispaced CAD nodes `cad` (ne, p+1, 2) (src/Core/Input.jl:163-185)."""
    qsi, wi = gauss_legendre(p + 1)
    Ng, dNg = lagrange_basis(equispaced_nodes(cad.shape[1] - 1), qsi)
    nodes = np.einsum("qk,ekd->eqd", Ng, cad)
    dx = np.einsum("qk,ekd->eqd", dNg, cad)
    J = np.sqrt(dx[..., 0] ** 2 + dx[..., 1] ** 2)
    t = dx / J[..., None]
    normal = np.stack([t[..., 1], -t[..., 0]], axis=-1)
    L = np.abs(J @ wi)
    return nodes, normal, J, L, wi


def from_cad(name, cad, p, properties, bc_type, bc_value, internal=None, region=None,
             keep_geo=True, discretize=None) -> BEMdata:
    """Build a BEMdata from CAD nodes `cad` (ne, ngeo, 2) and per-element BC data
    `bc_type` (ne, ndof), `bc_value` (ne, ndof) or per-node arrays (n, ndof).
    `discretize(cad, p)` makes the nodes, normals, Jacobians, lengths and
    weights (default: `discretize_curves` on the host)."""
    cad = np.asarray(cad, dtype=np.float64)
    ne = cad.shape[0]
    nodes, normal, J, L, wi = (discretize or discretize_curves)(cad, p)
    n = ne * (p + 1)
    ndof = properties.ndof
    bt = np.asarray(bc_type).reshape(-1, ndof)
    bv = np.asarray(bc_value, dtype=np.float64).reshape(-1, ndof)
    if bt.shape[0] == ne:
        bt = np.repeat(bt, p + 1, axis=0)
        bv = np.repeat(bv, p + 1, axis=0)
    assert bt.shape[0] == n
    coll = nodes.reshape(n, 2)
    if internal is not None and len(internal):
        coll = np.vstack([coll, np.asarray(internal, dtype=np.float64).reshape(-1, 2)])
    dad = BEMdata(
        name=name, p=p, ngeo=cad.shape[1] if keep_geo else 0, collocation=coll,
        normal=normal.reshape(n, 2), jacobian=J.reshape(n), elem_length=L,
        geo=cad if keep_geo else np.zeros((ne, 0, 2)), elem_weight=wi,
        properties=properties, BC=bt.reshape(-1).astype(np.int32),
        BV=bv.reshape(-1), region=np.asarray(region if region is not None else np.zeros(ne), np.int64))
    return dad.contiguous()


def format2d(path: str, properties, tipo: Optional[int] = None, pontointerno: bool = True,
             discretize=None, orient=None) -> BEMdata:
    """`format2d(file, properties; tipo, pontointerno)` (src/Core/Input.jl:108-197)
    from a Gmsh ASCII mesh file: the boundary's line elements (their nodes as
    equispaced CAD nodes of degree p = the mesh order; p + 1 Gauss-Legendre
    collocation nodes each), boundary conditions from each curve's physical
    name ("type;value" pairs, `parse_pairs`), normals oriented outward with
    the 2-D cells (`_orient_normals_outward!`) and, with pontointerno, the
    cells' centroids as internal points.  The discretisation and the
    orientation run on the device (`api.discretize`, `api.orient_normals`);
    `discretize(cad, p)` and `orient(dad, cells)` replace them."""
    from .msh import read_msh, parse_pairs
    from . import api
    m = read_msh(path)
    p = m.order
    if tipo is not None and int(tipo) != p:
        raise ValueError(f"format2d: the mesh has order {p}; changing it (tipo={tipo}) needs Gmsh")
    ndof = properties.ndof
    ne = m.lines.shape[0]
    bt = np.ones((ne, ndof), np.int32)
    bv = np.zeros((ne, ndof))
    for e in range(ne):
        nm = m.names.get(int(m.line_entity[e]))
        if nm is None:
            continue
        ints, floats = parse_pairs(nm)
        k = min(len(ints), ndof)
        bt[e, :k] = ints[:k]
        bv[e, :k] = floats[:k]
    cells = [c for c in m.cells if abs(polygon_area(c)) >= 1e-18]
    internal = np.array([c.mean(axis=0) for c in cells]) if (pontointerno and cells) else None
    dad = from_cad(os.path.basename(path), m.lines, p, properties, bt, bv, internal=None,
                   region=m.line_entity, discretize=discretize or api.discretize)
    (orient or api.orient_normals)(dad, cells)
    if internal is not None:
        dad.collocation = np.ascontiguousarray(np.vstack([dad.collocation, internal]))
    dad.cache["cells"] = cells
    return dad.contiguous()


def polygon_area(verts) -> float:
    """Signed area of a closed polygon, counter-clockwise positive
    (`polygon_area`, src/Core/Input.jl:287-298)."""
    v = np.asarray(verts, dtype=np.float64)
    x, y = v[:, 0], v[:, 1]
    return 0.5 * float(np.sum(x * np.roll(y, -1) - np.roll(x, -1) * y))


def from_nodes(name, X, p, properties, bc_type, bc_value) -> BEMdata:
    """BEMdata whose elements take their geometry from their own p+1
    collocation nodes `X` (ne, p+1, 2) at the Gauss-Legendre points (no CAD
    nodes): normals and Jacobians at the nodes come from the nodes' Lagrange
    interpolant (`tan2normal`, src/Core/Input.jl:584), so the node
    coordinates are the only geometric parameters (as the adjoint needs)."""
    X = np.asarray(X, dtype=np.float64)
    ne = X.shape[0]
    qsi, wi = gauss_legendre(p + 1)
    _, D = lagrange_basis(qsi, qsi)
    dx = np.einsum("qk,ekd->eqd", D, X)
    J = np.sqrt(dx[..., 0] ** 2 + dx[..., 1] ** 2)
    t = dx / J[..., None]
    normal = np.stack([t[..., 1], -t[..., 0]], axis=-1)
    L = np.abs(J @ wi)
    n = ne * (p + 1)
    ndof = properties.ndof
    bt = np.asarray(bc_type).reshape(-1, ndof)
    bv = np.asarray(bc_value, dtype=np.float64).reshape(-1, ndof)
    if bt.shape[0] == ne:
        bt = np.repeat(bt, p + 1, axis=0)
        bv = np.repeat(bv, p + 1, axis=0)
    dad = BEMdata(
        name=name, p=p, ngeo=0, collocation=X.reshape(n, 2), normal=normal.reshape(n, 2),
        jacobian=J.reshape(n), elem_length=L, geo=np.zeros((ne, 0, 2)), elem_weight=wi,
        properties=properties, BC=bt.reshape(-1).astype(np.int32), BV=bv.reshape(-1),
        region=np.zeros(ne, np.int64))
    return dad.contiguous()


def c4_node_counts(count: int = 512, lo: int = 64, hi: int = 4096, seed: int = 0) -> np.ndarray:
    """Node counts of the batched uneven workload (config C4): log-uniform in
    [lo, hi], rounded to multiples of 3 (quadratic elements)."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(lo), np.log(hi), count))
    return np.maximum(3 * np.round(n / 3).astype(int), 3 * (lo // 3))


def c4_domains(sizes, seed0: int = 100, amp: float = 0.1):
    """Star domains of the batched workload: domain i has sizes[i] nodes and
    seed seed0 + i (a_k ~ U(0, amp))."""
    return [star_domain(int(n) // 3, p=2, seed=seed0 + i, amp=amp) for i, n in enumerate(sizes)]


def star_adjoint_case(ne: int, p: int = 2, seed: int = 0, amp: float = 0.1, target_amp: float = 0.02):
    """Shape-gradient case (config C5): star boundary with nodes at the
    Gauss-Legendre points of each element's angular span, node-interpolant
    geometry (`from_nodes`), T = e^x cos y with Dirichlet data on theta in
    [0, pi) and Neumann data on [pi, 2 pi).  The target shape scales the node
    radii by a smooth seeded factor 1 + target_amp z(theta), z a unit-variance
    random trigonometric sum of degree <= 3.  Returns (dad, target_dad): the
    target shares the boundary data arrays, so solving it gives q* on the
    Dirichlet nodes."""
    props = Laplace(1.0)
    r, _ = star_radius(seed, amp)
    qsi, _ = gauss_legendre(p + 1)
    th = 2 * np.pi * (np.arange(ne)[:, None] + (qsi[None, :] + 1) / 2) / ne
    rad = r(th)
    X = np.stack([rad * np.cos(th), rad * np.sin(th)], axis=-1)
    start = 2 * np.pi * np.arange(ne) / ne
    dirichlet = np.repeat(start < np.pi, p + 1)
    base = from_nodes(f"adj{seed}", X, p, props, np.ones((ne, 1), np.int32), np.zeros((ne, 1)))
    Xn = base.collocation
    Tv = np.exp(Xn[:, 0]) * np.cos(Xn[:, 1])
    gx, gy = Tv, -np.exp(Xn[:, 0]) * np.sin(Xn[:, 1])
    qv = -(gx * base.normal[:, 0] + gy * base.normal[:, 1])
    BC = np.where(dirichlet, 0, 1).astype(np.int32)
    BV = np.where(dirichlet, Tv, qv)
    dad = from_nodes(f"adj{seed}", X, p, props, BC, BV)
    rng = np.random.default_rng(10_000 + seed)
    z = rng.standard_normal(7)
    zt = (z[0] + sum(z[2 * k - 1] * np.cos(k * th) + z[2 * k] * np.sin(k * th) for k in (1, 2, 3))) / np.sqrt(7.0)
    Xt = X * (1 + target_amp * zt)[..., None]
    target = from_nodes(f"adj{seed}_target", Xt, p, props, BC, BV)
    return dad, target


def _segment_cad(a, b, nel, p):
    """CAD nodes of `nel` straight elements from a to b, p+1 equispaced each."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    t = np.arange(nel + 1) / nel
    corners = a[None, :] * (1 - t[:, None]) + b[None, :] * t[:, None]
    cad = np.empty((nel, p + 1, 2))
    for e in range(nel):
        for k in range(p + 1):
            s = k / p
            cad[e, k] = (1 - s) * corners[e] + s * corners[e + 1]
    return cad


# ---------------------------------------------------------------------------
# builders
# ---------------------------------------------------------------------------
def quadrado(ndiv: int = 10, Lx: float = 1.0, Ly: float = 1.0, ordem: int = 1,
             pontointerno: bool = True, k: float = 1.0, bcs: Optional[dict] = None) -> BEMdata:
    """Square [0,Lx]x[0,Ly] as `quadrado` + `format2d` build it
    (data/Laplace/Laplace_dad.jl:238-280): `ndiv` transfinite points per side,
    so `ndiv-1` elements per side, curves bottom/right/top/left in that order,
    internal points at the centroids of the (ndiv-1)^2 quad cells.
    Default BCs (for T = x, q = -k dT/dn): bottom/top q=0, right q=-1, left T=0.
    `bcs` maps side name -> (type, value) to override."""
    sides = {"bottom": (1, 0.0), "right": (1, -1.0), "top": (1, 0.0), "left": (0, 0.0)}
    if bcs:
        sides.update(bcs)
    m = ndiv - 1
    P = [(0.0, 0.0), (Lx, 0.0), (Lx, Ly), (0.0, Ly)]
    segs = [("bottom", P[0], P[1]), ("right", P[1], P[2]), ("top", P[2], P[3]), ("left", P[3], P[0])]
    cads, bt, bv, reg = [], [], [], []
    for r, (nm, a, b) in enumerate(segs):
        c = _segment_cad(a, b, m, ordem)
        cads.append(c)
        bt += [[sides[nm][0]]] * m
        bv += [[sides[nm][1]]] * m
        reg += [r + 1] * m
    internal = None
    if pontointerno:
        xs = np.arange(ndiv) / (ndiv - 1) * Lx
        ys = np.arange(ndiv) / (ndiv - 1) * Ly
        cx = 0.25 * (xs[:-1] + xs[1:] + xs[1:] + xs[:-1])
        cy = 0.25 * (ys[:-1] + ys[:-1] + ys[1:] + ys[1:])
        gx, gy = np.meshgrid(cx, cy, indexing="ij")
        internal = np.stack([gx.ravel(), gy.ravel()], axis=1)
    return from_cad("quadrado", np.concatenate(cads), ordem, Laplace(k), np.array(bt),
                    np.array(bv), internal=internal, region=reg)


def quadrado_elasticity(ndiv: int = 10, Lx: float = 1.0, Ly: float = 1.0, ordem: int = 1,
                        props: Optional[Elasticity] = None, pontointerno: bool = False) -> BEMdata:
    """Square for elasticity patch tests (data/Laplace/Laplace_dad.jl:289-323):
    left edge clamped (`0;0;0;0`), other edges traction-free (`1;0;1;0`)."""
    props = props or Elasticity()
    m = ndiv - 1
    P = [(0.0, 0.0), (Lx, 0.0), (Lx, Ly), (0.0, Ly)]
    segs = [("bottom", P[0], P[1]), ("right", P[1], P[2]), ("top", P[2], P[3]), ("left", P[3], P[0])]
    cads, bt, bv, reg = [], [], [], []
    for r, (nm, a, b) in enumerate(segs):
        cads.append(_segment_cad(a, b, m, ordem))
        if nm == "left":
            bt += [[0, 0]] * m
        else:
            bt += [[1, 1]] * m
        bv += [[0.0, 0.0]] * m
        reg += [r + 1] * m
    internal = None
    if pontointerno:
        xs = (np.arange(m) + 0.5) / m * Lx
        ys = (np.arange(m) + 0.5) / m * Ly
        gx, gy = np.meshgrid(xs, ys, indexing="ij")
        internal = np.stack([gx.ravel(), gy.ravel()], axis=1)
    return from_cad("quadrado_elast", np.concatenate(cads), ordem, props, np.array(bt),
                    np.array(bv), internal=internal, region=reg)


def star_radius(seed: int, amp: float = 0.08):
    """Seeded r(t) = 1 + sum_{k=2..6} a_k cos(k t + phi_k), a_k ~ U(0, amp),
    phi_k ~ U(0, 2 pi).  Returns (r, dr/dt) callables and the coefficients."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.0, amp, size=5)
    ph = rng.uniform(0.0, 2 * np.pi, size=5)
    ks = np.arange(2, 7)

    def r(t):
        t = np.asarray(t, np.float64)
        return 1.0 + np.sum(a[:, None] * np.cos(ks[:, None] * t.ravel()[None, :] + ph[:, None]),
                            axis=0).reshape(t.shape)

    return r, (a, ph)


def star_domain(ne: int, p: int = 2, seed: int = 0, amp: float = 0.08,
                field: str = "expcos", props=None, pontointerno: bool = False) -> BEMdata:
    """Star-shaped domain with `ne` elements of degree `p` (n = ne*(p+1) nodes),
    element corners equally spaced in angle, p+1 CAD nodes per element on the
    exact curve.  Mixed data for T = e^x cos y: Dirichlet where the element's
    start angle is in [0, pi), Neumann (q = -k dT/dn) on [pi, 2 pi)."""
    props = props or Laplace(1.0)
    r, _ = star_radius(seed, amp)
    th = 2 * np.pi * (np.arange(ne)[:, None] + np.arange(p + 1)[None, :] / p) / ne
    rad = r(th)
    cad = np.stack([rad * np.cos(th), rad * np.sin(th)], axis=-1)
    nd = props.ndof
    dad = from_cad(f"star{seed}", cad, p, props, np.ones((ne, nd), np.int32), np.zeros((ne, nd)),
                   region=np.zeros(ne))
    if pontointerno:
        rr = 0.5 * r(np.linspace(0, 2 * np.pi, 16, endpoint=False))
        tt = np.linspace(0, 2 * np.pi, 16, endpoint=False)
        dad.set_internal_nodes(np.stack([rr * np.cos(tt), rr * np.sin(tt)], axis=1))
    if nd != 1:
        return dad  # traction-free; callers set their own data
    ana = ana_laplace_expcos(props.k)
    dirichlet_elem = th[:, 0] < np.pi
    dmask = np.repeat(dirichlet_elem, p + 1)
    set_mixed_bc(dad, ana, dmask)
    dad.set_cache(analytical=ana)
    return dad


def plate_with_hole(n_outer_el: int = 1024, n_hole_el: int = 342, p: int = 2, half: float = 1.0,
                    radius: float = 0.3, sigma: float = 1e8, props: Optional[Elasticity] = None,
                    pin: bool = True) -> BEMdata:
    """Square plate [-half, half]^2 with a central hole, uniform traction
    sigma_xx = sigma on x = +-half, traction-free top/bottom and hole.  Outer
    boundary counter-clockwise, hole clockwise (normals point out of the solid).
    With `pin`, three displacement DOFs are prescribed to zero to remove rigid
    motion: u_x and u_y at the bottom-edge node nearest x=0, u_x at the
    top-edge node nearest x=0."""
    props = props or Elasticity(E=210e9, nu=0.3, plane_strain=True)
    per = n_outer_el // 4
    P = [(-half, -half), (half, -half), (half, half), (-half, half)]
    names = ["bottom", "right", "top", "left"]
    cads, bt, bv, reg = [], [], [], []
    for s in range(4):
        cads.append(_segment_cad(P[s], P[(s + 1) % 4], per, p))
        tx = sigma if names[s] == "right" else (-sigma if names[s] == "left" else 0.0)
        bt += [[1, 1]] * per
        bv += [[tx, 0.0]] * per
        reg += [s + 1] * per
    # hole, clockwise
    th = -2 * np.pi * (np.arange(n_hole_el)[:, None] + np.arange(p + 1)[None, :] / p) / n_hole_el
    hole = np.stack([radius * np.cos(th), radius * np.sin(th)], axis=-1)
    cads.append(hole)
    bt += [[1, 1]] * n_hole_el
    bv += [[0.0, 0.0]] * n_hole_el
    reg += [5] * n_hole_el
    dad = from_cad("plate_hole", np.concatenate(cads), p, props, np.array(bt), np.array(bv),
                   region=reg)
    if pin:
        nodes = dad.Nodes
        nn = p + 1
        bottom = np.arange(0, per * nn)
        top = np.arange(2 * per * nn, 3 * per * nn)
        ib = bottom[np.argmin(np.abs(nodes[bottom, 0]))]
        it = top[np.argmin(np.abs(nodes[top, 0]))]
        for dof in (2 * ib, 2 * ib + 1, 2 * it):
            dad.BC[dof] = 0
            dad.BV[dof] = 0.0
    return dad


# ---------------------------------------------------------------------------
# interior point grids (src/Core/InternalPoints.jl)
# ---------------------------------------------------------------------------
def _boundary_chords(dad: "BEMdata"):
    """Element chords of the CAD nodes (or first/last field node)
    (`_boundary_segments`, InternalPoints.jl:216-231)."""
    if dad.ngeo >= 2:
        g = np.asarray(dad.geo)
        a, b = g[:, :-1].reshape(-1, 2), g[:, 1:].reshape(-1, 2)
    else:
        X = np.asarray(dad.collocation[: dad.n]).reshape(dad.ne, dad.p + 1, 2)
        a, b = X[:, 0], X[:, -1]
    return a, b


def point_in_domain(dad: "BEMdata", pts) -> np.ndarray:
    """Even-odd ray test against the boundary chords (`point_in_domain`,
    `_inside_segments`, InternalPoints.jl:198-245)."""
    P = np.atleast_2d(np.asarray(pts, np.float64))
    a, b = _boundary_chords(dad)
    px, py = P[:, 0:1], P[:, 1:2]
    yi, yj = a[None, :, 1], b[None, :, 1]
    cross = (yi > py) != (yj > py)
    xint = (b[None, :, 0] - a[None, :, 0]) * (py - yi) / (yj - yi + 1e-30) + a[None, :, 0]
    hits = np.sum(cross & (px < xint), axis=1)
    return hits % 2 == 1


def _dist_to_boundary(dad: "BEMdata", pts) -> np.ndarray:
    """Distance to the piecewise-linear interpolant through each element's
    CAD nodes (`_dist_to_boundary`, `_dist_element`, InternalPoints.jl:330-340,
    Integration.jl:238-312)."""
    P = np.atleast_2d(np.asarray(pts, np.float64))
    a, b = _boundary_chords(dad)
    ab = b - a
    ap = P[:, None, :] - a[None, :, :]
    t = np.clip(np.sum(ap * ab[None], -1) / (np.sum(ab * ab, -1)[None] + np.finfo(float).eps), 0, 1)
    d = ap - t[..., None] * ab[None]
    return np.sqrt(np.min(np.sum(d * d, -1), axis=1))


def internal_grid(dad: "BEMdata", nx: int, ny: int, d_min: float = 0.01, layout: str = "gera") -> np.ndarray:
    """Cartesian interior points in the boundary's bounding box, kept when
    inside and at least d_min * (longest element) from the boundary
    (`internal_grid`, InternalPoints.jl:23-42; layouts `_axis_nodes`, :62-73)."""
    if nx < 1 or ny < 1:
        raise ValueError("nx, ny must be >= 1")
    X = np.asarray(dad.collocation[: dad.n])
    if dad.ngeo:
        X = np.concatenate([X, np.asarray(dad.geo).reshape(-1, 2)])
    lo, hi = X.min(0), X.max(0)

    def axis(n, lo_, hi_):
        i = np.arange(1, n + 1)
        if layout == "gera":
            return lo_ + (hi_ - lo_) * i / (n + 1)
        if layout == "cell":
            return lo_ + (hi_ - lo_) * (i - 0.5) / n
        if layout == "cheb":
            return lo_ + (hi_ - lo_) * (1 - np.cos(np.pi * (i - 0.5) / n)) / 2
        raise ValueError(f"layout must be gera, cell or cheb (got {layout})")

    xs, ys = axis(nx, lo[0], hi[0]), axis(ny, lo[1], hi[1])
    P = np.stack(np.meshgrid(xs, ys, indexing="xy"), -1).reshape(-1, 2)  # x fastest, as `for y, x`
    keep = point_in_domain(dad, P)
    clear = d_min * float(np.max(dad.elem_length))
    if clear > 0:
        keep &= _dist_to_boundary(dad, P) >= clear
    return P[keep]


# ---------------------------------------------------------------------------
# analytic fields (src/Core/Analytical.jl)
# ---------------------------------------------------------------------------
@dataclass
class AnalyticalSolution:
    name: str
    u: Callable
    q: Optional[Callable] = None


def ana_laplace_linear(direction=(1.0, 0.0), k: float = 1.0) -> AnalyticalSolution:
    """T = d.x, q = -k d.n (src/Core/Analytical.jl:171-182)."""
    d = np.asarray(direction, np.float64)
    return AnalyticalSolution("laplace_linear", lambda x: np.asarray(x) @ d,
                              lambda x, n: -k * (np.asarray(n) @ d))


def ana_laplace_expcos(k: float = 1.0) -> AnalyticalSolution:
    """T = e^x cos y (harmonic), q = -k grad T . n."""
    def u(x):
        x = np.asarray(x)
        return np.exp(x[..., 0]) * np.cos(x[..., 1])

    def q(x, n):
        x = np.asarray(x)
        n = np.asarray(n)
        gx = np.exp(x[..., 0]) * np.cos(x[..., 1])
        gy = -np.exp(x[..., 0]) * np.sin(x[..., 1])
        return -k * (gx * n[..., 0] + gy * n[..., 1])

    return AnalyticalSolution("laplace_expcos", u, q)


def ana_elasticity_patch(E=1.0, nu=0.3, exx=0.01, eyy=0.0, exy=0.0) -> AnalyticalSolution:
    """Uniform plane-strain patch u = eps . x, t = sigma . n
    (src/Core/Analytical.jl:546-586, dim=2)."""
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    sxx = lam * (exx + eyy) + 2 * mu * exx
    syy = lam * (exx + eyy) + 2 * mu * eyy
    sxy = 2 * mu * exy

    def u(x):
        x = np.asarray(x)
        return np.stack([exx * x[..., 0] + exy * x[..., 1], exy * x[..., 0] + eyy * x[..., 1]], axis=-1)

    def q(x, n):
        n = np.asarray(n)
        return np.stack([sxx * n[..., 0] + sxy * n[..., 1], sxy * n[..., 0] + syy * n[..., 1]], axis=-1)

    return AnalyticalSolution("elasticity_patch", u, q)


def attach_analytical(dad: BEMdata, ana: AnalyticalSolution) -> BEMdata:
    dad.set_cache(analytical=ana)
    return dad


def apply_analytical_bc(dad: BEMdata, ana: AnalyticalSolution, neumann_nodes=None) -> BEMdata:
    """Dirichlet from `ana.u` everywhere except `neumann_nodes`
    (src/Core/Analytical.jl:84-156)."""
    dmask = np.ones(dad.n, bool)
    if neumann_nodes is not None:
        dmask[np.asarray(neumann_nodes, int)] = False
    set_mixed_bc(dad, ana, dmask)
    attach_analytical(dad, ana)
    return dad


def set_mixed_bc(dad: BEMdata, ana: AnalyticalSolution, dirichlet_mask: np.ndarray):
    nd = dad.ndof
    uval = np.asarray(ana.u(dad.Nodes)).reshape(dad.n, nd)
    qval = np.asarray(ana.q(dad.Nodes, dad.normal)).reshape(dad.n, nd) if ana.q else np.zeros((dad.n, nd))
    bc = np.where(dirichlet_mask[:, None], 0, 1).repeat(nd, axis=1)
    bv = np.where(dirichlet_mask[:, None], uval, qval)
    dad.BC = np.ascontiguousarray(bc.reshape(-1), dtype=np.int32)
    dad.BV = np.ascontiguousarray(bv.reshape(-1), dtype=np.float64)
    return dad


def analytical(dad: BEMdata) -> np.ndarray:
    """Analytic primary field at every collocation point (Analytical.jl:45-66)."""
    ana = dad.cache["analytical"]
    return np.asarray(ana.u(dad.collocation), dtype=np.float64).reshape(-1)


def analytical_flux(dad: BEMdata) -> np.ndarray:
    ana = dad.cache["analytical"]
    return np.asarray(ana.q(dad.Nodes, dad.normal), dtype=np.float64).reshape(-1)


def rel_error(dad: BEMdata) -> float:
    """Relative L2 error of dad.T (or dad.u) against the attached analytic
    field (src/Core/Analytical.jl:617-630)."""
    Tana = analytical(dad)
    Tnum = dad.cache["T"] if "T" in dad.cache else dad.cache["u"]
    n = min(len(Tnum), len(Tana))
    num = np.linalg.norm(Tnum[:n] - Tana[:n])
    den = np.linalg.norm(Tana[:n])
    return float(num / den) if den > 0 else float(num)


def rel_error_flux(dad: BEMdata) -> float:
    """Relative L2 error of dad.q / dad.traction (Analytical.jl:667-679)."""
    qana = analytical_flux(dad)
    qnum = dad.cache["q"] if "q" in dad.cache else dad.cache["traction"]
    n = min(len(qnum), len(qana))
    num = np.linalg.norm(qnum[:n] - qana[:n])
    den = np.linalg.norm(qana[:n])
    return float(num / den) if den > 0 else float(num)
