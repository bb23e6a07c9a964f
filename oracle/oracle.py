"""Python face of the FP64 CPU oracle.  TEST INFRASTRUCTURE ONLY.

Loaded by tests/, by `__graft_entry__.smoke()` and by bench.py's CPU-baseline
leg (and its `--impl reference` arm) -- as the checker, never by the product
package.  Wraps oracle/_build/liborc.so (a C++ restatement of the reference's
Float64 dense path, see bem_oracle.cpp) and adds the dense solve the
reference runs through LinearSolve.jl -> OpenBLAS LU
(src/Core/LinearSolveUtils.jl:44-49), here SciPy's LAPACK getrf/getrs.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liborc.so")

NEARFIELD = {"tanp3c": 0, "plain": 1, "euclid": 2, "csinh": 3, "sinhsinh": 4, "tangent": 5, "p3c": 6}


class OrcGeom(ctypes.Structure):
    _fields_ = [("nt", ctypes.c_int32), ("n", ctypes.c_int32), ("ne", ctypes.c_int32),
                ("p", ctypes.c_int32), ("ngeo", ctypes.c_int32)] + [
        (nm, ctypes.POINTER(ctypes.c_double))
        for nm in ("px", "py", "nx", "ny", "jac", "elen", "gx", "gy", "ew")]


_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        build()  # make: rebuilds only when the source is newer than the library
        _lib = ctypes.CDLL(LIB_PATH)
        d = ctypes.c_double
        P = ctypes.POINTER(d)
        i = ctypes.c_int
        _lib.orc_assemble.argtypes = [ctypes.POINTER(OrcGeom), i, d, d, i, d, i, i, i, P, P,
                                      ctypes.c_void_p]
        _lib.orc_assemble.restype = i
        _lib.orc_integrate_element.argtypes = [ctypes.POINTER(OrcGeom), i, d, d, i, i, i, i, d, d, i, P, P]
        _lib.orc_near_mask.argtypes = [ctypes.POINTER(OrcGeom), d, ctypes.POINTER(ctypes.c_uint8)]
        _lib.orc_gausslegendre.argtypes = [i, P, P]
        _lib.orc_shapefun.argtypes = [i, i, d, P, P]
        _lib.orc_closest_point_1d.argtypes = [i, i, P, d, d, P, P, P]
        _lib.orc_complex_pole_1d.argtypes = [i, i, P, d, d, P, P]
        _lib.orc_map.argtypes = [i, P, P, i, d, d, P, P]
        _lib.orc_map.restype = i
        _lib.orc_sinh_map.argtypes = [P, i, d, d, P, P]
        _lib.orc_eq40_AB.argtypes = [d, P, P, P]
        _lib.orc_p3c_inv_pole.argtypes = [d, d, P, P]
        _lib.orc_interp_rule.argtypes = [d, i, P, P, P, P]
        _lib.orc_interp_rule.restype = i
        FN = ctypes.CFUNCTYPE(d, d)
        _lib.FN = FN
        _lib.orc_laurent_coefficients_interp.argtypes = [FN, d, i, i, P]
        _lib.orc_laurent_coefficients_interp.restype = i
        _lib.orc_guiggiani_integral_interp.argtypes = [FN, d, i, i]
        _lib.orc_guiggiani_integral_interp.restype = d
        _lib.orc_guiggiani_GH_interp.argtypes = [FN, FN, d, i, i, i, P, P]
        _lib.orc_laplace_kernel.argtypes = [d, d, d, d, d, P, P]
        _lib.orc_kelvin_kernel.argtypes = [d, d, d, d, d, d, P, P]
        _lib.orc_near_element.argtypes = [P, i, d, d, d, d]
        _lib.orc_near_element.restype = i
        _lib.orc_apply_bc.argtypes = [ctypes.c_int64, ctypes.c_int64, P, P,
                                      ctypes.POINTER(ctypes.c_int32), P, P, P]
        _lib.orc_strain_stress2d.argtypes = [ctypes.POINTER(OrcGeom), d, d, P, P, P, P]
        _lib.orc_interior_laplace.argtypes = [ctypes.POINTER(OrcGeom), d, i, i, P, P, i, P, P, P]
        _lib.orc_interior_laplace.restype = i
        _lib.orc_dibem_fd2d.argtypes = [i, P, P, i, d, d, i, d, P, P]
        _lib.orc_dibem_ifid2d.argtypes = [ctypes.POINTER(OrcGeom), d, i, d, d, P, P]
        _lib.orc_dibem_ifid2d.restype = i
        _lib.orc_cr_fn.argtypes = [i, P, i, P]
        _lib.orc_dibem_ifid_near2d.argtypes = [ctypes.POINTER(OrcGeom), d, i, d, d, i, P, P]
        _lib.orc_dibem_ifid_near2d.restype = i
        _lib.orc_near_rule.argtypes = [ctypes.POINTER(OrcGeom), i, i, i, d, d, P, P, P]
        _lib.orc_near_rule.restype = i
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_geom(dad):
    """Pack a BEMdata into the oracle's struct; returns (struct, keepalive)."""
    keep = dict(
        px=np.ascontiguousarray(dad.collocation[:, 0]), py=np.ascontiguousarray(dad.collocation[:, 1]),
        nx=np.ascontiguousarray(dad.normal[:, 0]), ny=np.ascontiguousarray(dad.normal[:, 1]),
        jac=np.ascontiguousarray(dad.jacobian), elen=np.ascontiguousarray(dad.elem_length),
        gx=np.ascontiguousarray(dad.geo[..., 0].reshape(-1)) if dad.ngeo else np.zeros(1),
        gy=np.ascontiguousarray(dad.geo[..., 1].reshape(-1)) if dad.ngeo else np.zeros(1),
        ew=np.ascontiguousarray(dad.elem_weight))
    g = OrcGeom(dad.nt, dad.n, dad.ne, dad.p, dad.ngeo, *[_p(keep[k]) for k in
                ("px", "py", "nx", "ny", "jac", "elen", "gx", "gy", "ew")])
    return g, keep


def _props(dad):
    pr = dad.properties
    if pr.ndof == 1:
        return 0, float(pr.k), 0.0
    return 1, float(pr.mu), float(pr.nu_eff)


def assemble(dad, npg=20, near_factor=1.5, nearfield="tanp3c", singular="guiggiani", threads=0,
             store=True, mask=None):
    """Dense FP64 H, G (H_G_full_direct, src/Core/Assembly_full.jl:61-175).
    `mask` (nt x ne uint8) fixes the near/far split instead of testing it."""
    L = lib()
    g, keep = make_geom(dad)
    kind, a, b = _props(dad)
    rows = dad.ndof * dad.nt
    cols = dad.ndof * dad.n
    H = np.zeros((rows, rows), order="F")
    G = np.zeros((rows, cols), order="F")
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
    rc = L.orc_assemble(ctypes.byref(g), kind, a, b, npg, float(near_factor), NEARFIELD[nearfield],
                        1 if singular == "telles" else 0, threads, _p(H), _p(G),
                        None if m is None else m.ctypes.data)
    if rc != 0:
        raise ValueError(f"oracle assemble failed ({rc})")
    if store:
        dad.set_cache(H=H, G=G)
    return H, G


def integrate_element(dad, e, pf, source=-1, npg=20, nearfield="tanp3c", singular="guiggiani"):
    L = lib()
    g, keep = make_geom(dad)
    kind, a, b = _props(dad)
    nc = 1 if kind == 0 else 4
    h = np.zeros((dad.p + 1) * nc)
    gg = np.zeros((dad.p + 1) * nc)
    L.orc_integrate_element(ctypes.byref(g), kind, a, b, npg, NEARFIELD[nearfield],
                            1 if singular == "telles" else 0, e, float(pf[0]), float(pf[1]),
                            int(source), _p(h), _p(gg))
    return h, gg


def cr_fn(name, x):
    """Correctly rounded atan / tan / cbrt of the doubles x (quad precision
    rounded once)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    lib().orc_cr_fn({"atan": 0, "tan": 1, "cbrt": 2}[name], _p(x), x.size, _p(out))
    return out


def near_rule(dad, e, pf, npg=16, nearfield="tanp3c"):
    """Mapped nodes and weights of the near-field rule for element e and source
    point pf, and the complex pole (z0, e0) they came from."""
    g, keep = make_geom(dad)
    eta = np.zeros(2 * npg + 2)
    w = np.zeros(2 * npg + 2)
    ze = np.zeros(2)
    m = lib().orc_near_rule(ctypes.byref(g), npg, NEARFIELD[nearfield], int(e), float(pf[0]), float(pf[1]),
                            _p(eta), _p(w), _p(ze))
    return eta[:m], w[:m], ze


def near_mask(dad, near_factor=1.5):
    L = lib()
    g, keep = make_geom(dad)
    m = np.zeros((dad.nt, dad.ne), np.uint8)
    L.orc_near_mask(ctypes.byref(g), float(near_factor), m.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)))
    return m


def apply_bc(dad, H=None, G=None):
    """Column swap into A x = b (src/Core/Boundary_conditions.jl:54-75, 152-174)."""
    H = dad.cache["H"] if H is None else H
    G = dad.cache["G"] if G is None else G
    rows, cols = G.shape
    A = np.zeros((rows, rows), order="F")
    b = np.zeros(rows)
    BC = np.ascontiguousarray(dad.BC, dtype=np.int32)
    BV = np.ascontiguousarray(dad.BV, dtype=np.float64)
    lib().orc_apply_bc(rows, cols, _p(np.asfortranarray(H)), _p(np.asfortranarray(G)),
                       BC.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), _p(BV), _p(A), _p(b))
    return A, b


def lu_solve(A, b):
    """Dense LU with partial pivoting (LAPACK getrf/getrs through SciPy)."""
    import scipy.linalg as sla
    lu, piv = sla.lu_factor(A, overwrite_a=False, check_finite=False)
    return sla.lu_solve((lu, piv), b, check_finite=False)


def split_sol(dad, x):
    """Scatter x into (T, q) or (u, traction) (src/Core/Solver.jl:88-98, 133-146)."""
    BC, BV = dad.BC, dad.BV
    if dad.ndof == 1:
        T = np.array(x[: dad.nt], dtype=np.float64)
        q = np.zeros(dad.n)
        d = BC == 0
        q[d] = T[: dad.n][d]
        T[: dad.n][d] = BV[d]
        q[~d] = BV[~d]
        dad.set_cache(T=T, q=q, x=np.asarray(x))
        return T
    nb = 2 * dad.n
    u = np.where(BC == 0, BV, x[:nb])
    t = np.where(BC == 0, x[:nb], BV)
    dad.set_cache(u=u, traction=t, T=u, x=np.asarray(x))
    return u


def dibem_fd(pts, kind=0, prm0=1.0, prm1=0.0, rbf=3, epsa=1e-16):
    """Pairwise DIBEM F, D (`_dibem_FD_kernel!`, src/Laplace/DIBEM_GPU.jl:194-208;
    Kelvin `_elast_dibem_FD_kernel!`, src/Elasticity/Assembly_GPU.jl:258-280)."""
    pts = np.asarray(pts, np.float64).reshape(-1, 2)
    nt = len(pts)
    dof = 1 if kind == 0 else 2
    px, py = np.ascontiguousarray(pts[:, 0]), np.ascontiguousarray(pts[:, 1])
    F = np.zeros((nt, nt), order="F")
    D = np.zeros((dof * nt, dof * nt), order="F")
    lib().orc_dibem_fd2d(nt, _p(px), _p(py), kind, float(prm0), float(prm1), int(rbf), float(epsa), _p(F), _p(D))
    return F, D


def dibem_ifid(dad, rbf=3, epsa=1e-16, near_factor=1.5):
    """Far boundary sums IF, ID of the DIBEM domain integrals
    (`_dibem_IFID_kernel!`, src/Laplace/DIBEM_GPU.jl:234-270)."""
    L = lib()
    g, keep = make_geom(dad)
    IF = np.zeros(dad.nt)
    ID = np.zeros(dad.nt)
    L.orc_dibem_ifid2d(ctypes.byref(g), float(dad.properties.k), int(rbf), float(epsa), float(near_factor),
                       _p(IF), _p(ID))
    return IF, ID


def discretize(cad, p):
    """Collocation nodes, normals, Jacobians, element lengths and weights of
    elements given by equispaced CAD nodes `cad` (ne, ngeo, 2): the geometry
    loop of `format2d` (src/Core/Input.jl:163-185): nodes = Ngeo*X,
    dx = dNgeo*X, J = |dx|, normal = tan2normal(dx/J) = (t_y, -t_x),
    L = |J . w| with Gauss-Legendre (qsi, w) of p+1 points
    (`discontinuous_nodes_weights`).  Basis from monomial coefficients, Gauss
    points from numpy's leggauss."""
    cad = np.asarray(cad, np.float64)
    ngeo = cad.shape[1]
    qsi, w = np.polynomial.legendre.leggauss(p + 1)
    t = np.linspace(-1.0, 1.0, ngeo)
    N = np.empty((p + 1, ngeo))
    dN = np.empty((p + 1, ngeo))
    for m in range(ngeo):
        c = np.poly(np.delete(t, m))
        c = c / np.polyval(c, t[m])
        N[:, m] = np.polyval(c, qsi)
        dN[:, m] = np.polyval(np.polyder(c), qsi)
    nodes = np.einsum("qm,emd->eqd", N, cad)
    dx = np.einsum("qm,emd->eqd", dN, cad)
    J = np.hypot(dx[..., 0], dx[..., 1])
    normal = np.stack([dx[..., 1] / J, -dx[..., 0] / J], axis=-1)
    L = np.abs(J @ w)
    return nodes, normal, J, L, w


def dibem_ifid_near(dad, IF, ID, rbf=3, epsa=1e-16, near_factor=1.5, npg=16):
    """Adds the near-pair Gauss-rule correction to IF, ID
    (`_dibem_correct_near_cpu!`, src/Laplace/DIBEM_GPU.jl:272-300); returns them."""
    g, keep = make_geom(dad)
    IF = np.array(IF, dtype=np.float64)
    ID = np.array(ID, dtype=np.float64)
    lib().orc_dibem_ifid_near2d(ctypes.byref(g), float(dad.properties.k), int(rbf), float(epsa),
                                float(near_factor), int(npg), _p(IF), _p(ID))
    return IF, ID


def interior_laplace(dad, pts, npg=16, nearfield="tanp3c", T=None, q=None):
    """Potential at interior points (`interior_laplace`, src/Laplace/Lubrication.jl:399-416)."""
    pts = np.ascontiguousarray(np.asarray(pts, dtype=np.float64).reshape(-1, 2))
    T = np.ascontiguousarray((dad.cache["T"] if T is None else T)[: dad.n], dtype=np.float64)
    q = np.ascontiguousarray(dad.cache["q"] if q is None else q, dtype=np.float64)
    xp, yp = np.ascontiguousarray(pts[:, 0]), np.ascontiguousarray(pts[:, 1])
    out = np.zeros(len(pts))
    g, keep = make_geom(dad)
    lib().orc_interior_laplace(ctypes.byref(g), float(dad.properties.k), int(npg), NEARFIELD[nearfield],
                               _p(T), _p(q), len(pts), _p(xp), _p(yp), _p(out))
    return out


def strain_stress(dad, u=None, t=None):
    """Kane boundary strain/stress, n x 3 each (`recover_strain_stress!`,
    src/Elasticity/StrainStress.jl:35-99)."""
    u = np.ascontiguousarray(dad.cache["u"] if u is None else u, dtype=np.float64)
    t = np.ascontiguousarray(dad.cache["traction"] if t is None else t, dtype=np.float64)
    g, keep = make_geom(dad)
    eps = np.zeros((dad.n, 3), order="F")
    sig = np.zeros((dad.n, 3), order="F")
    pr = dad.properties
    lib().orc_strain_stress2d(ctypes.byref(g), float(pr.lam), float(pr.mu), _p(u), _p(t), _p(eps), _p(sig))
    return eps, sig


def solve(dad):
    """applyBC + LU solve + split (src/Core/Solver.jl:24-64, 114-131)."""
    A, b = apply_bc(dad)
    x = lu_solve(A, b)
    dad.set_cache(A=A, b=b)
    return split_sol(dad, x)


def timed_pipeline(dad, npg=16, threads=0):
    """assemble + applyBC + LU + split, wall-clock seconds per stage."""
    t0 = time.perf_counter()
    assemble(dad, npg=npg, threads=threads)
    t1 = time.perf_counter()
    A, b = apply_bc(dad)
    t2 = time.perf_counter()
    x = lu_solve(A, b)
    t3 = time.perf_counter()
    split_sol(dad, x)
    return dict(assemble=t1 - t0, apply_bc=t2 - t1, lu=t3 - t2, total=t3 - t0, x=x)


def point_in_polygon(p, verts):
    """Even-odd ray test, boundary outside (`point_in_polygon`,
    src/Core/Input.jl:331-345)."""
    inside = False
    nv = len(verts)
    j = nv - 1
    for i in range(nv):
        yi, yj = verts[i][1], verts[j][1]
        if (yi > p[1]) != (yj > p[1]):
            xint = (verts[j][0] - verts[i][0]) * (p[1] - yi) / (yj - yi + 1e-30) + verts[i][0]
            if p[0] < xint:
                inside = not inside
        j = i
    return inside


def orient_normals(nodes, normal, elen, p, cells):
    """`_orient_normals_outward!` (src/Core/Input.jl:376-389): the normals of
    element e flip unless the point 0.1 L behind its first node lies in a
    cell.  nodes, normal: (n, 2); returns (oriented normals, flipped mask)."""
    normal = np.array(normal, dtype=np.float64)
    nn = p + 1
    ne = len(elen)
    flipped = np.zeros(ne, bool)
    if not len(cells):
        return normal, flipped
    for e in range(ne):
        i0 = e * nn
        d = 0.1 * float(elen[e])
        if d < 1e-16:
            continue
        pt = (nodes[i0][0] - d * normal[i0][0], nodes[i0][1] - d * normal[i0][1])
        if any(point_in_polygon(pt, c) for c in cells):
            continue
        normal[i0:i0 + nn] = -normal[i0:i0 + nn]
        flipped[e] = True
    return normal, flipped
