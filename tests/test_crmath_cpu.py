"""Bit-level agreement of the near-singular quadrature map between the GPU
code and the oracle, checked on the host.

The reference's tanp3c map turns a one-ulp change of a pole coordinate, a
Gauss node or an atan / tan value into up to ~5e-5 relative change of an
element integral (test_near_map_rounding_sensitivity below measures it), so
the GPU and the oracle agree to 1e-10 only if they compute the map's nodes
and weights to the last bit.  Both evaluate atan, tan, cbrt and the
Gauss-Legendre rules correctly rounded -- the GPU code by double-double
arithmetic (bem_crmath.cuh), the oracle by quad precision -- and the map in
the same IEEE operations.  The harness builds the GPU code for the host with
contraction off, which gives the device's bits."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
P = ctypes.POINTER(ctypes.c_double)


def _p(a):
    return a.ctypes.data_as(P)


@pytest.fixture(scope="module")
def h():
    d = tempfile.mkdtemp(prefix="nearmap_")
    so = os.path.join(d, "libnearmap.so")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-shared", "-fPIC",
                           os.path.join(HERE, "native", "nearmap_harness.cpp"), "-o", so])
    L = ctypes.CDLL(so)
    L.h_cr_fn.argtypes = [ctypes.c_int, P, ctypes.c_int, P]
    L.h_gauss.argtypes = [ctypes.c_int, P, P]
    L.h_constants.argtypes = [P]
    L.h_near_rule.argtypes = [ctypes.c_int, ctypes.c_int, P, P, ctypes.c_double, ctypes.c_double, P, P, P]
    L.h_near_rule.restype = ctypes.c_int
    return L


def _hfn(h, which, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    h.h_cr_fn({"atan": 0, "tan": 1, "cbrt": 2}[which], _p(x), x.size, _p(out))
    return out


def _samples():
    rng = np.random.default_rng(7)
    halfpi = np.pi / 2 - 1e-8
    return {
        "atan": np.concatenate([rng.uniform(-4, 4, 40000), np.exp(rng.uniform(-40, 40, 40000)) *
                                rng.choice([-1, 1], 40000), rng.uniform(1e7, 1e9, 20000) *
                                rng.choice([-1, 1], 20000)]),
        "tan": np.concatenate([rng.uniform(-halfpi, halfpi, 60000),
                               halfpi - np.exp(rng.uniform(np.log(1e-16), np.log(1e-2), 20000)),
                               -halfpi + np.exp(rng.uniform(np.log(1e-16), np.log(1e-2), 20000))]),
        "cbrt": np.concatenate([np.exp(rng.uniform(-80, 80, 50000)), [1e-14, 8.0, 27.0, 1e-300]]),
    }


def test_correctly_rounded_functions_agree_bitwise(h, orc):
    """GPU code (double-double) and oracle (quad) give the same doubles."""
    for name, x in _samples().items():
        a = _hfn(h, name, x)
        b = orc.cr_fn(name, x)
        bad = np.nonzero(a != b)[0]
        assert bad.size == 0, (name, x[bad[:5]], a[bad[:5]], b[bad[:5]])


def test_correctly_rounded_against_arbitrary_precision(h):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 300
    rng = np.random.default_rng(11)
    for name, fn in (("atan", mpmath.atan), ("tan", mpmath.tan), ("cbrt", mpmath.cbrt)):
        x = rng.permutation(_samples()[name])[:1500]
        got = _hfn(h, name, x)
        want = np.array([float(fn(mpmath.mpf(float(v)))) for v in x])
        bad = np.nonzero(got != want)[0]
        assert bad.size == 0, (name, x[bad[:5]])


def test_constants_of_the_correctly_rounded_functions(h):
    mpmath = pytest.importorskip("mpmath")
    from fractions import Fraction
    mpmath.mp.prec = 400
    c = np.zeros(3 + 52 + 10 + 34 + 10 + 6)
    h.h_constants(_p(c))

    def parts(v, n):
        out = []
        for _ in range(n):
            out.append(float(v))
            v = v - mpmath.mpf(out[-1])
        return out

    assert list(c[:3]) == parts(mpmath.pi / 2, 3)
    for j in range(26):
        assert list(c[3 + 2 * j:5 + 2 * j]) == parts(mpmath.tan(mpmath.mpf(j) / 32), 2), j
    coef = [Fraction(1, 3), Fraction(2, 15), Fraction(17, 315), Fraction(62, 2835), Fraction(1382, 155925),
            Fraction(21844, 6081075), Fraction(929569, 638512875)]
    # the Taylor coefficients of tan from the Bernoulli numbers
    sympy = pytest.importorskip("sympy")
    for k, fr in enumerate(coef, start=1):
        n = 2 * k + 2
        a = (-1) ** k * 2 ** n * (2 ** n - 1) * sympy.bernoulli(n) / sympy.factorial(n)
        assert sympy.Rational(fr.numerator, fr.denominator) == a
    t = c[55:]
    for k in range(3):
        assert list(t[2 * k:2 * k + 2]) == parts(mpmath.mpf(coef[k].numerator) / coef[k].denominator, 2)
    for k in range(3, 7):
        assert t[3 + k] == float(mpmath.mpf(coef[k].numerator) / coef[k].denominator)
    a = c[65:]
    for j in range(17):
        assert list(a[2 * j:2 * j + 2]) == parts(mpmath.atan(mpmath.mpf(j) / 16), 2), j
    o = a[34:]
    for k in range(1, 6):
        assert list(o[2 * (k - 1):2 * k]) == parts(mpmath.mpf(1) / (2 * k + 1), 2), k
    for k in range(6, 12):
        assert o[10 + k - 6] == float(mpmath.mpf(1) / (2 * k + 1)), k


def test_gauss_legendre_rules_agree_bitwise(h, orc):
    L = orc.lib()
    for n in list(range(1, 33)) + [20]:
        xa, wa, xb, wb = (np.zeros(n) for _ in range(4))
        h.h_gauss(n, _p(xa), _p(wa))
        L.orc_gausslegendre(n, _p(xb), _p(wb))
        assert np.array_equal(xa, xb) and np.array_equal(wa, wb), n
        xl, wl = np.polynomial.legendre.leggauss(n)
        assert np.max(np.abs(xa - xl)) <= 4e-16 and np.max(np.abs(wa - wl)) <= 1e-13 * np.max(wl)


def test_gauss_legendre_rules_correctly_rounded(h):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.prec = 250
    for n in (2, 3, 5, 16, 20, 32):
        x, w = np.zeros(n), np.zeros(n)
        h.h_gauss(n, _p(x), _p(w))
        for i in range((n + 1) // 2, n):
            z = mpmath.findroot(lambda t: mpmath.legendre(n, t), mpmath.mpf(float(x[i])))
            dp = mpmath.diff(lambda t: mpmath.legendre(n, t), z)
            assert x[i] == float(z) and x[n - 1 - i] == -float(z), (n, i)
            assert w[i] == float(2 / ((1 - z * z) * dp * dp)), (n, i)


def _pairs(dad, orc):
    m = orc.near_mask(dad)
    rows, els = np.nonzero(m)
    own = (rows < dad.n) & ((rows // (dad.p + 1)) == els)
    return rows[~own], els[~own]


@pytest.mark.parametrize("case", ["star2731", "star_interior", "square_p1"])
def test_near_map_agrees_bitwise_with_oracle(h, orc, case):
    """Nodes, weights and pole of every near (point, element) pair: the GPU
    map (run on the host) and the oracle's map are the same doubles.  The
    first case is the full-size solve (2731 quadratic elements, N = 8193)."""
    from bem_gmsh_gb300 import star_domain, quadrado
    if case == "star2731":
        dad = star_domain(2731, p=2, seed=0)
    elif case == "star_interior":
        dad = star_domain(120, p=2, seed=4)
    else:
        dad = quadrado(ndiv=21, pontointerno=True)
    nn = dad.p + 1
    px, py = dad.collocation[:, 0], dad.collocation[:, 1]
    if case == "star_interior":
        # points just inside the boundary, facing the middle of each element
        # at 0.05 .. 0.6 element lengths: the pole lies inside the element
        rng = np.random.default_rng(2)
        els = np.repeat(np.arange(dad.ne), 3)
        mid = dad.collocation[els * nn + 1]
        d = rng.uniform(0.05, 0.6, els.size) * dad.elem_length[els]
        pts = mid - d[:, None] * dad.normal[els * nn + 1]
    else:
        rows, els = _pairs(dad, orc)
        pts = dad.collocation[rows]
    assert len(els) > 100
    L = orc.lib()
    g, keep = orc.make_geom(dad)
    npg = 16
    ea, wa, za, eb, wb, zb = (np.zeros(2 * npg + 2) for _ in range(6))
    nx, ny = np.zeros(nn), np.zeros(nn)
    branches = set()
    for r, (e, pf) in enumerate(zip(els, pts)):
        nx[:] = px[e * nn:(e + 1) * nn]
        ny[:] = py[e * nn:(e + 1) * nn]
        ma = h.h_near_rule(dad.p, npg, _p(nx), _p(ny), float(pf[0]), float(pf[1]), _p(ea), _p(wa), _p(za))
        mb = L.orc_near_rule(ctypes.byref(g), npg, 0, int(e), float(pf[0]), float(pf[1]), _p(eb), _p(wb),
                             _p(zb))
        assert ma == mb, (r, e, ma, mb)
        assert np.array_equal(za[:2], zb[:2]), (r, e, za[:2], zb[:2])
        assert np.array_equal(ea[:ma], eb[:mb]) and np.array_equal(wa[:ma], wb[:mb]), (r, e)
        branches.add(ma)
    if case == "star_interior":
        assert 2 * npg in branches  # the split branch (pole inside the element) was exercised


def test_near_map_rounding_sensitivity(orc):
    """Why the bits matter: a one-ulp change of the pole's imaginary part
    moves the near integrals of most neighbouring-element pairs of the
    full-size mesh by more than 1e-10 relative (up to ~1e-5)."""
    from bem_gmsh_gb300 import star_domain
    dad = star_domain(2731, p=2, seed=0)
    rows, els = _pairs(dad, orc)
    rng = np.random.default_rng(0)
    pick = rng.choice(len(rows), 400, replace=False)
    nn = 3
    changed, worst = 0, 0.0
    for k in pick:
        r, e = rows[k], els[k]
        pf = dad.collocation[r].copy()
        h0, g0 = orc.integrate_element(dad, e, pf, source=int(r), npg=16)
        # the same pair with the point moved by one ulp along the element's normal direction
        pf2 = pf + np.spacing(np.abs(pf)) * np.sign(dad.normal[e * nn])
        h1, g1 = orc.integrate_element(dad, e, pf2, source=int(r), npg=16)
        d = np.max(np.abs(g1 - g0) / np.maximum(np.abs(g0), 1e-300))
        changed += d > 1e-10
        worst = max(worst, d)
    print(f"pairs moved by > 1e-10: {changed} / {len(pick)}, largest relative change {worst:.2e}")
    assert changed > len(pick) // 4 and worst > 1e-8
