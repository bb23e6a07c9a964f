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
BEM_ERR_UNSUPPORTED = 6


def _rel(a, b):
    a = a.double().cpu().numpy()
    b = b.double().cpu().numpy()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _fresh(nt, n, ld, tdt):
    import torch
    Hs = torch.full((nt, ld), float("nan"), dtype=tdt, device="cuda")
    Gs = torch.full((n, ld), float("nan"), dtype=tdt, device="cuda")
    return Hs.t()[:nt], Gs.t()[:nt]


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

    Href, Gref = _fresh(nt, n, ld, tdt)
    H_G_gpu(dad, T=T, npg=16, out=(Href, Gref), store=False)  # existing entry point
    g, keep = geom_struct(dad, device=True)
    dt = _lib.BEM_F64 if T == np.float64 else _lib.BEM_F32
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        H, G = _fresh(nt, n, ld, tdt)
        rc = L.bem_assemble_laplace2d_noalloc(g, 1.0, 16, 1.5, dt, H.data_ptr(), ld, G.data_ptr(), ld,
                                              stream)
        assert rc == 0, (call, rc)
        torch.cuda.synchronize()
        assert torch.isfinite(H).all() and torch.isfinite(G).all()
        assert _rel(H, Href) < TOL[T] and _rel(G, Gref) < TOL[T], (call, _rel(H, Href), _rel(G, Gref))


def test_noalloc_reads_weights_after_the_callers_stream_work():
    """The element weights are written by a kernel on a non-blocking stream
    right before the call on that stream (behind a long matrix product): the
    call must see the new weights, not the zeros the buffer held before."""
    import torch
    from bem_gmsh_gb300 import _lib, star_domain
    from bem_gmsh_gb300.api import H_G_gpu, geom_struct

    L = _lib.load()
    dad = star_domain(300, p=2, seed=5)
    nt, n, ld = dad.nt, dad.n, dad.nt
    Href, Gref = _fresh(nt, n, ld, torch.float64)
    H_G_gpu(dad, T=np.float64, npg=16, out=(Href, Gref), store=False)
    g, keep = geom_struct(dad, device=True)
    ew_true = keep["ew"].clone()
    keep["ew"].zero_()
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    big = torch.randn(4096, 4096, device="cuda")
    for _ in range(2):
        H, G = _fresh(nt, n, ld, torch.float64)
        keep["ew"].zero_()
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            for _ in range(8):
                big = big @ big.t() / 4096.0  # keeps the stream busy before the write
            keep["ew"].copy_(ew_true)
        rc = L.bem_assemble_laplace2d_noalloc(g, 1.0, 16, 1.5, _lib.BEM_F64, H.data_ptr(), ld, G.data_ptr(),
                                              ld, s.cuda_stream)
        assert rc == 0, rc
        s.synchronize()
        assert _rel(H, Href) < 1e-10 and _rel(G, Gref) < 1e-10, (_rel(H, Href), _rel(G, Gref))


def test_noalloc_rejects_sizes_beyond_its_array():
    """nt beyond BEM_NOALLOC_MAX_NT is refused before any device work.  The
    element limit cannot be exceeded on its own: every element holds at least
    two nodes, so ne <= n / 2 <= nt / 2, and the nt check covers it; this case
    exceeds only the nt limit (few elements, many internal points)."""
    import torch
    from bem_gmsh_gb300 import _lib, quadrado
    from bem_gmsh_gb300.api import geom_struct

    L = _lib.load()
    dad = quadrado(ndiv=128, pontointerno=True)  # 508 elements, 1016 + 16129 points
    assert dad.nt > _lib.BEM_NOALLOC_MAX_NT and dad.ne <= _lib.BEM_NOALLOC_MAX_NE
    g, keep = geom_struct(dad, device=True)
    H = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = L.bem_assemble_laplace2d_noalloc(g, 1.0, 16, 1.5, _lib.BEM_F64, H.data_ptr(), dad.nt, H.data_ptr(),
                                          dad.nt, None)
    assert rc == BEM_ERR_UNSUPPORTED


def test_noalloc_reports_near_pair_overflow():
    """A near factor that makes every (point, element) pair near lists more
    pairs than the fixed array holds: the call returns BEM_ERR_UNSUPPORTED
    (H and G are then undefined), and the next call is unaffected."""
    import torch
    from bem_gmsh_gb300 import _lib, star_domain
    from bem_gmsh_gb300.api import H_G_gpu, geom_struct

    L = _lib.load()
    dad = star_domain(400, p=2, seed=2)  # 1200 x 400 pairs > 24 * BEM_NOALLOC_MAX_NT
    assert dad.nt * dad.ne > 24 * _lib.BEM_NOALLOC_MAX_NT
    g, keep = geom_struct(dad, device=True)
    nt, n, ld = dad.nt, dad.n, dad.nt
    H, G = _fresh(nt, n, ld, torch.float64)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.bem_assemble_laplace2d_noalloc(g, 1.0, 16, 1e6, _lib.BEM_F64, H.data_ptr(), ld, G.data_ptr(), ld,
                                          stream)
    assert rc == BEM_ERR_UNSUPPORTED
    Href, Gref = _fresh(nt, n, ld, torch.float64)
    H_G_gpu(dad, T=np.float64, npg=16, out=(Href, Gref), store=False)
    rc = L.bem_assemble_laplace2d_noalloc(g, 1.0, 16, 1.5, _lib.BEM_F64, H.data_ptr(), ld, G.data_ptr(), ld,
                                          stream)
    assert rc == 0
    torch.cuda.synchronize()
    assert _rel(H, Href) < 1e-10 and _rel(G, Gref) < 1e-10
