"""On-device boundary discretisation (bem_discretize2d) against the oracle,
and assembly from device-discretised geometry against the host-built one."""
import numpy as np
import pytest

from bem_gmsh_gb300 import Laplace
from bem_gmsh_gb300 import _lib
from bem_gmsh_gb300.api import discretize, H_G_gpu
from bem_gmsh_gb300.geometry import from_cad, star_radius

pytestmark = pytest.mark.gpu


def _curved_cad(rng, ne, ngeo):
    base = rng.uniform(-1, 1, (ne, 1, 2))
    s = np.linspace(0, 1, ngeo)[None, :, None]
    d = rng.uniform(0.2, 1.0, (ne, 1, 2))
    bow = 0.15 * rng.standard_normal((ne, 1, 2)) * (s * (1 - s))
    return base + s * d + bow


@pytest.mark.parametrize("p,ngeo", [(0, 2), (1, 2), (2, 3), (3, 4), (4, 5), (5, 6), (2, 6)])
def test_discretize_matches_oracle(orc, p, ngeo):
    cad = _curved_cad(np.random.default_rng(p * 7 + ngeo), 333, ngeo)
    got = discretize(cad, p)
    ref = orc.discretize(cad, p)
    for a, b in zip(got, ref):
        assert a.shape == b.shape
        assert np.max(np.abs(a - b)) <= 1e-13 * max(1.0, np.max(np.abs(b)))


def test_discretize_rejects_bad_arguments():
    ctx = _lib.default_context()
    cad = np.zeros((4, 3, 2))
    for ne, ngeo, p in [(0, 3, 2), (4, 1, 2), (4, 7, 2), (4, 3, 6), (4, 3, -1)]:
        out = [np.empty(64) for _ in range(7)]
        rc = ctx.L.bem_discretize2d(ctx.h, ne, ngeo, p, cad.ctypes.data, cad.ctypes.data, _lib.BEM_MEM_HOST,
                                    *[o.ctypes.data for o in out])
        assert rc == 1  # BEM_ERR_INVALID


def test_assembly_from_device_geometry():
    ne, p = 400, 2
    r, _ = star_radius(3, 0.08)
    th = 2 * np.pi * (np.arange(ne)[:, None] + np.arange(p + 1)[None, :] / p) / ne
    rad = r(th)
    cad = np.stack([rad * np.cos(th), rad * np.sin(th)], axis=-1)
    bt, bv = np.ones((ne, 1), np.int32), np.zeros((ne, 1))
    host = from_cad("h", cad, p, Laplace(1.0), bt, bv)
    dev = from_cad("d", cad, p, Laplace(1.0), bt, bv, discretize=discretize)
    assert np.max(np.abs(dev.collocation - host.collocation)) < 1e-14
    H0, G0 = H_G_gpu(host, T=np.float64, npg=16, near="gpu")
    H1, G1 = H_G_gpu(dev, T=np.float64, npg=16, near="gpu")
    assert np.max(np.abs(H1 - H0)) <= 1e-11 * np.max(np.abs(H0))
    assert np.max(np.abs(G1 - G0)) <= 1e-11 * np.max(np.abs(G0))
