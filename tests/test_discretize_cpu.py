"""Boundary discretisation (format2d geometry loop, src/Core/Input.jl:163-185):
the oracle against closed-form answers and against the host mirror."""
import numpy as np
import pytest

from bem_gmsh_gb300.geometry import discretize_curves


def _curved_cad(rng, ne, ngeo):
    base = rng.uniform(-1, 1, (ne, 1, 2))
    s = np.linspace(0, 1, ngeo)[None, :, None]
    d = rng.uniform(0.2, 1.0, (ne, 1, 2))
    bow = 0.15 * rng.standard_normal((ne, 1, 2)) * (s * (1 - s))
    return base + s * d + bow


@pytest.mark.parametrize("p,ngeo", [(0, 2), (1, 2), (2, 3), (3, 4), (4, 5), (5, 6), (2, 2), (1, 4)])
def test_oracle_matches_host_mirror(orc, p, ngeo):
    cad = _curved_cad(np.random.default_rng(10 * p + ngeo), 50, ngeo)
    ref = orc.discretize(cad, p)
    got = discretize_curves(cad, p)
    for a, b in zip(got, ref):
        assert np.max(np.abs(a - b)) <= 1e-13 * max(1.0, np.max(np.abs(b)))


@pytest.mark.parametrize("p", [0, 1, 2, 5])
def test_straight_segment_known_answer(orc, p):
    # element from (0, 0) to (2, 0): J = 1, nodes at 1 + qsi, normal (0, -1), L = 2
    ngeo = max(p + 1, 2)
    cad = np.zeros((1, ngeo, 2))
    cad[0, :, 0] = np.linspace(0.0, 2.0, ngeo)
    nodes, normal, J, L, w = orc.discretize(cad, p)
    qsi, _ = np.polynomial.legendre.leggauss(p + 1)
    np.testing.assert_allclose(nodes[0, :, 0], 1.0 + qsi, atol=1e-14)
    np.testing.assert_allclose(nodes[0, :, 1], 0.0, atol=1e-15)
    np.testing.assert_allclose(J, 1.0, rtol=1e-13)
    np.testing.assert_allclose(normal[0], np.tile([0.0, -1.0], (p + 1, 1)), atol=1e-14)
    assert abs(L[0] - 2.0) < 1e-13


def test_circle_perimeter_converges(orc):
    # counter-clockwise unit circle by quadratic elements: outward normals and
    # sum L -> 2 pi at fourth order in the element size
    errs = []
    for ne in (16, 32, 64):
        th = 2 * np.pi * (np.arange(ne)[:, None] + np.arange(3)[None, :] / 2) / ne
        cad = np.stack([np.cos(th), np.sin(th)], axis=-1)
        nodes, normal, J, L, w = orc.discretize(cad, 2)
        radial = nodes / np.linalg.norm(nodes, axis=-1, keepdims=True)
        assert np.min(np.sum(normal * radial, axis=-1)) > 0.99
        errs.append(abs(L.sum() - 2 * np.pi))
    assert errs[-1] < 1e-5
    assert errs[0] / errs[1] > 12 and errs[1] / errs[2] > 12
