"""GPU parity of the assembly against the FP64 oracle, through the C ABI.

Tolerances: FP64 path ||dM||/||M|| < 1e-10 (reference test/laplace.jl:414)
and every entry within 1e-10 of the matrix's largest entry; FP32 path
< 1e-6 (test/laplace.jl:454-455).

The reference's near-singular tanp3c map amplifies rounding (a one-ulp
change of an atan value or of the pole moves a neighbouring-element integral
by up to ~5e-5 relative; tests/test_crmath_cpu.py measures it).  The GPU's
map and the oracle's are the same IEEE operations with correctly rounded
atan / tan / cbrt and Gauss rules, and tests/test_crmath_cpu.py checks their
nodes and weights bit for bit; so the FP64 bar needs no allowance for that
sensitivity.  Regular meshes put points exactly on the near cut (distance =
1.5 L): the GPU's near test is IEEE round-to-nearest without contraction and
resolves those ties as the reference does."""
import numpy as np
import pytest

from bem_gmsh_gb300 import (quadrado, quadrado_elasticity, star_domain, Elasticity, Laplace,
                            ana_laplace_linear, attach_analytical, from_cad)
from bem_gmsh_gb300.api import H_G_gpu, assemble_system

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
TOL32 = 1e-6


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def perturbed(dad, seed=0):
    """Copy of `dad` with every coordinate moved by one ulp (random sign)."""
    import copy
    d = copy.deepcopy(dad)
    rng = np.random.default_rng(seed)
    sgn = np.where(rng.random(d.collocation.shape) < 0.5, -np.inf, np.inf)
    d.collocation = np.nextafter(d.collocation, sgn)
    if d.ngeo:
        sg = np.where(rng.random(d.geo.shape) < 0.5, -np.inf, np.inf)
        d.geo = np.nextafter(d.geo, sg)
    return d.contiguous()


def check64(M, Mr, what=""):
    """FP64 bar: relative Frobenius error and every entry within 1e-10."""
    M = np.asarray(M, np.float64)
    e = rel(M, Mr)
    d = float(np.max(np.abs(M - Mr))) / float(np.max(np.abs(Mr)))
    assert e < TOL64 and d < TOL64, (what, e, d)
    return e, d


CASES = [
    ("quadrado8", lambda: quadrado(ndiv=8, pontointerno=True), 12),
    ("quadrado10_noint", lambda: quadrado(ndiv=10, pontointerno=False), 12),
    ("quadrado20", lambda: quadrado(ndiv=20, pontointerno=True), 20),
    ("quadrado_p2", lambda: quadrado(ndiv=7, ordem=2, pontointerno=True), 16),
    ("quadrado_p3", lambda: quadrado(ndiv=6, ordem=3, pontointerno=False), 16),
    ("star_p2", lambda: star_domain(120, p=2, seed=1), 16),
    ("star_p2_int", lambda: star_domain(90, p=2, seed=2, pontointerno=True), 16),
    ("star_p1", lambda: star_domain(150, p=1, seed=3), 8),
]


@pytest.mark.parametrize("name,mk,npg", CASES, ids=[c[0] for c in CASES])
def test_laplace_hg_parity(orc, name, mk, npg):
    dad = mk()
    Hr, Gr = orc.assemble(dad, npg=npg, store=False)
    H, G = H_G_gpu(dad, T=np.float64, npg=npg, store=False)
    check64(H, Hr, "H")
    check64(G, Gr, "G")
    H32, G32 = H_G_gpu(dad, T=np.float32, npg=npg, store=False)
    assert rel(H32, Hr) < TOL32 and rel(G32, Gr) < TOL32, (rel(H32, Hr), rel(G32, Gr))
    assert np.all(np.isfinite(H)) and np.all(np.isfinite(G32))


def test_geometry_from_nodes(orc):
    """ngeo = 0: element geometry from the collocation nodes (no CAD nodes)."""
    dad = star_domain(80, p=2, seed=4)
    dad.ngeo = 0
    dad.geo = np.zeros((dad.ne, 0, 2))
    Hr, Gr = orc.assemble(dad, npg=16, store=False)
    H, G = H_G_gpu(dad, T=np.float64, npg=16, store=False)
    check64(H, Hr, "H")
    check64(G, Gr, "G")


def test_all_near(orc):
    """near_factor = inf: every pair integrated (no far lumping)."""
    dad = quadrado(ndiv=6, pontointerno=True)
    Hr, Gr = orc.assemble(dad, npg=12, near_factor=np.inf, store=False)
    H, G = H_G_gpu(dad, T=np.float64, npg=12, near_factor=np.inf, store=False)
    check64(H, Hr, "H")
    check64(G, Gr, "G")


@pytest.mark.parametrize("ndiv", [5, 9])
def test_kelvin_hg_parity(orc, ndiv):
    dad = quadrado_elasticity(ndiv=ndiv, props=Elasticity(1.0, 0.3, 1.0), pontointerno=True)
    Hr, Gr = orc.assemble(dad, npg=12, store=False)
    H, G = H_G_gpu(dad, T=np.float64, npg=12, store=False)
    check64(H, Hr, "H")
    check64(G, Gr, "G")
    H32, G32 = H_G_gpu(dad, T=np.float32, npg=12, store=False)
    assert rel(H32, Hr) < TOL32 and rel(G32, Gr) < TOL32, (rel(H32, Hr), rel(G32, Gr))


def test_kelvin_curved_plane_stress(orc):
    pr = Elasticity(E=210e9, nu=0.3, plane_strain=False)
    dad = star_domain(60, p=2, seed=5, props=pr)
    dad.BC = np.ones(2 * dad.n, np.int32)
    dad.BV = np.zeros(2 * dad.n)
    Hr, Gr = orc.assemble(dad, npg=16, store=False)
    H, G = H_G_gpu(dad, T=np.float64, npg=16, store=False)
    check64(H, Hr, "H")
    check64(G, Gr, "G")


@pytest.mark.parametrize("kind", ["laplace", "kelvin"])
def test_fused_system_matches_applybc(orc, kind):
    if kind == "laplace":
        dad = star_domain(100, p=2, seed=6, pontointerno=True)
    else:
        dad = quadrado_elasticity(ndiv=7, props=Elasticity(1.0, 0.3, 1.0))
        dad.BC[::3] = 0
        dad.BV = np.linspace(-1, 1, dad.BV.size)
    Hr, Gr = orc.assemble(dad, npg=16, store=False)
    Ar, br = orc.apply_bc(dad, Hr, Gr)
    A, b = assemble_system(dad, npg=16)
    check64(A, Ar, "A")
    assert rel(b, br) < TOL64, rel(b, br)


def _kelvin_plate():
    from bem_gmsh_gb300.geometry import plate_with_hole
    return plate_with_hole(n_outer_el=128, n_hole_el=42, p=2, sigma=1e8)


def _kelvin_square():
    dad = quadrado_elasticity(ndiv=13, ordem=2, props=Elasticity(1.0, 0.3, 1.0), pontointerno=True)
    dad.BC[::3] = 0
    dad.BV = np.linspace(-1, 1, dad.BV.size)
    return dad


@pytest.mark.parametrize("name,mk", [
    ("star", lambda: star_domain(400, p=2, seed=3, pontointerno=True)),
    ("quadrado_p2", lambda: quadrado(ndiv=12, ordem=2, pontointerno=True)),
    ("quadrado_p1", lambda: quadrado(ndiv=30, pontointerno=False)),
    ("kelvin_plate", _kelvin_plate),
    ("kelvin_square_p2", _kelvin_square),
])
def test_double_float_far_field_matches_fp64(name, mk):
    """BEM_OPT_FAR_DF = 2: the fused Laplace and Kelvin systems with their far
    field in double-float (FP32 pairs) equal the FP64-arithmetic systems to
    ~1e-14 of the largest entry, and entrywise to 2^-43 relative above a
    floor: 1e-16 of the largest entry for Laplace, 1e-14 for Kelvin, whose
    off-diagonal traction entries c (r_x n_y - r_y n_x) / R^2 cancel to
    near zero for nearly collinear pairs."""
    from bem_gmsh_gb300 import _lib
    dad = mk()
    ctx = _lib.Context()
    try:
        ctx.set_option(_lib.BEM_OPT_FAR_DF, 0)
        A64, b64 = assemble_system(dad, npg=16, ctx=ctx)
        ctx.set_option(_lib.BEM_OPT_FAR_DF, 2)
        Adf, bdf = assemble_system(dad, npg=16, ctx=ctx)
    finally:
        ctx.close()
    scale = np.abs(A64).max()
    d = np.abs(Adf - A64)
    assert d.max() <= 1e-13 * scale, d.max() / scale
    # entrywise: within 2^-43 relative (double-float ops are ~2^-48 each)
    # plus an absolute floor far below the matrix scale
    floor = (1e-14 if name.startswith("kelvin") else 1e-16) * scale
    assert np.all(d <= 2.0 ** -43 * np.abs(A64) + floor), float(np.max(d / (np.abs(A64) + 1e-300)))
    assert np.abs(bdf - b64).max() <= 1e-13 * np.abs(b64).max()


def test_device_pointers_and_ld(orc):
    """BEM_MEM_DEVICE with a padded leading dimension."""
    import torch
    dad = star_domain(70, p=2, seed=7, pontointerno=True)
    Hr, Gr = orc.assemble(dad, npg=16, store=False)
    ld = dad.nt + 5
    Hs = torch.zeros((dad.nt, ld), dtype=torch.float64, device="cuda")  # row-major storage of H^T
    Gs = torch.zeros((dad.n, ld), dtype=torch.float64, device="cuda")
    H = Hs.t()[: dad.nt]  # column-major view with ld
    G = Gs.t()[: dad.nt]
    H_G_gpu(dad, T=np.float64, npg=16, out=(H, G), store=False)
    check64(H.cpu().numpy(), Hr, "H")
    check64(G.cpu().numpy(), Gr, "G")


def test_repeated_calls_reuse_workspace(orc):
    a = quadrado(ndiv=12, pontointerno=True)
    b = star_domain(200, p=2, seed=8)
    for dad in (a, b, a):
        Hr, Gr = orc.assemble(dad, npg=16, store=False)
        H, G = H_G_gpu(dad, T=np.float64, npg=16, store=False)
        check64(H, Hr, "H")
        check64(G, Gr, "G")


def test_invalid_arguments_raise():
    from bem_gmsh_gb300._lib import BemError
    dad = quadrado(ndiv=5)
    with pytest.raises(ValueError):
        H_G_gpu(dad, device="cpu")
    with pytest.raises(ValueError):
        H_G_gpu(dad, T=np.float16)
    dad.properties = Laplace(k=-1.0)
    with pytest.raises(BemError):
        H_G_gpu(dad)


def test_full_size_parity_every_entry(orc):
    """The full-size solve's matrices (2731 quadratic elements, N = 8193):
    every entry of the FP64 H and G within 1e-10 of the largest entry, near
    and on-element entries included (no rounding-sensitivity allowance)."""
    import os
    dad = star_domain(2731, p=2, seed=0)
    H, G = H_G_gpu(dad, T=np.float64, npg=16, near="gpu", store=False)
    Ho, Go = orc.assemble(dad, npg=16, threads=os.cpu_count() or 1, store=False)
    eh, dh = check64(H, Ho, "H")
    eg, dg = check64(G, Go, "G")
    # the near entries (neighbouring elements) on their own, relative to themselves
    m = orc.near_mask(dad)
    rows, els = np.nonzero(m)
    cols = (3 * els[:, None] + np.arange(3)[None, :]).ravel()
    rr = np.repeat(rows, 3)
    off = rr != cols
    gn = np.abs(G[rr, cols] - Go[rr, cols]) / np.abs(Go[rr, cols])
    hn = np.abs(H[rr[off], cols[off]] - Ho[rr[off], cols[off]]) / np.abs(Ho[rr[off], cols[off]])
    print(f"H: rel {eh:.2e} max entry {dh:.2e}; G: rel {eg:.2e} max entry {dg:.2e}; "
          f"near entries max rel: G {gn.max():.2e}, H {hn.max():.2e}")
    assert gn.max() < 1e-10


@pytest.mark.parametrize("nearfield", ["plain", "euclid", "csinh", "sinhsinh", "tangent", "p3c"])
def test_nearfield_maps_match_oracle(orc, nearfield):
    """The reference's `nearfield` knob (src/Core/Integration.jl:41-93): the
    plain Gauss rule, the sinh maps (about the closest point, on the complex
    pole, iterated sinh-sinh; the straight edges' collinear poles take the
    eq. (40) exponential branch) and the tangent and complete-cubic maps,
    Laplace on curved quadratic and straight cubic elements (whose pole
    comes from the closest point) and Kelvin, against the oracle with the
    same map (FP64, every entry)."""
    for dad in (star_domain(150, p=2, seed=12, pontointerno=True),
                quadrado(ndiv=6, ordem=3, pontointerno=True),
                quadrado_elasticity(ndiv=9, ordem=2, props=Elasticity(1.0, 0.3, 1.0), pontointerno=True)):
        Hr, Gr = orc.assemble(dad, npg=16, nearfield=nearfield, store=False)
        H, G = H_G_gpu(dad, T=np.float64, npg=16, nearfield=nearfield, store=False)
        check64(H, Hr, f"H {nearfield}")
        check64(G, Gr, f"G {nearfield}")


def test_telles_on_element_rule_matches_oracle(orc):
    """`singular=:telles` (src/Core/Assembly_full.jl:282-283, 467-528), which the
    reference's Kelvin H_G_gpu accepts (src/Elasticity/Assembly_GPU.jl:23):
    Kelvin and Laplace on curved quadratic elements against the oracle's
    Telles rule, and close to the interpolated Guiggiani result."""
    pr = Elasticity(E=210e9, nu=0.3, plane_strain=True)
    for dad in (star_domain(80, p=2, seed=5, props=pr), star_domain(120, p=2, seed=6, pontointerno=True)):
        Hr, Gr = orc.assemble(dad, npg=16, singular="telles", store=False)
        H, G = H_G_gpu(dad, T=np.float64, npg=16, singular="telles", store=False)
        check64(H, Hr, "H telles")
        check64(G, Gr, "G telles")
        Hg, Gg = H_G_gpu(dad, T=np.float64, npg=16, store=False)
        assert rel(G, Gg) < 5e-2  # two quadratures of the same log-singular integrals
