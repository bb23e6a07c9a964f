"""The allocation-free assembly entry point, for callers that cannot allocate
device memory while they run (their device memory belongs to another
allocator's pool, or they may only allocate at start-up).

bem_assemble_laplace2d_noalloc keeps its scratch in a fixed device array of
the library instead of calling cudaMalloc.  Its H and G must match the
allocating entry point bem_assemble_laplace2d (within the assembly tests'
tolerances: 1e-10 for FP64, 1e-6 for FP32) on two calls in a row, since the
second call reuses the array the first one left behind.  This file is named
to be collected last, and it also passes on its own in a fresh process."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {np.float64: 1e-10, np.float32: 1e-6}


def _rel(a, b):
    a = a.double().cpu().numpy()
    b = b.double().cpu().numpy()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_noalloc_matches_allocating_entry_point(T):
    import torch
    from bem_gmsh_gb300 import _lib, star_domain
    from bem_gmsh_gb300.api import H_G_gpu, geom_struct

    L = _lib.load()
    dad = star_domain(300, p=2, seed=3, pontointerno=True)
    nt, n = dad.nt, dad.n
    tdt = torch.float64 if T == np.float64 else torch.float32
    ld = nt + 4

    def fresh():
        Hs = torch.full((nt, ld), float("nan"), dtype=tdt, device="cuda")
        Gs = torch.full((n, ld), float("nan"), dtype=tdt, device="cuda")
        return Hs.t()[:nt], Gs.t()[:nt]

    Href, Gref = fresh()
    H_G_gpu(dad, T=T, npg=16, out=(Href, Gref), store=False)  # existing entry point
    g, keep = geom_struct(dad, device=True)
    dt = _lib.BEM_F64 if T == np.float64 else _lib.BEM_F32
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        H, G = fresh()
        rc = L.bem_assemble_laplace2d_noalloc(g, 1.0, 16, 1.5, dt, H.data_ptr(), ld, G.data_ptr(), ld,
                                              stream)
        assert rc == 0, (call, rc)
        torch.cuda.synchronize()
        assert torch.isfinite(H).all() and torch.isfinite(G).all()
        assert _rel(H, Href) < TOL[T] and _rel(G, Gref) < TOL[T], (call, _rel(H, Href), _rel(G, Gref))


def test_noalloc_rejects_sizes_beyond_its_array():
    import torch
    from bem_gmsh_gb300 import _lib, quadrado
    from bem_gmsh_gb300.api import geom_struct

    L = _lib.load()
    dad = quadrado(ndiv=4200, pontointerno=False)  # 4 * 4199 elements > BEM_NOALLOC_MAX_NE
    g, keep = geom_struct(dad, device=True)
    H = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = L.bem_assemble_laplace2d_noalloc(g, 1.0, 16, 1.5, _lib.BEM_F64, H.data_ptr(), dad.nt, H.data_ptr(),
                                          dad.nt, None)
    assert rc == 6  # BEM_ERR_UNSUPPORTED, before any device work
