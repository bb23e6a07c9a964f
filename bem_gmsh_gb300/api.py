"""Host-side mirror of the reference's user API for the dense path.

    dad = quadrado(ndiv=20)                    # format2d equivalent
    assemble(dad, 20, method="gpu")            # assemble!(dad, npg; method=:gpu)
    solve(dad)                                 # solve(dad) -> dad.T, dad.q
    rel_error(dad)

Reference: `assemble!` (src/Core/Assembly_full.jl:107-118), `H_G_gpu`
(src/Laplace/Assembly_GPU.jl:120-150, src/Elasticity/Assembly_GPU.jl:15-51),
`solve` (src/Core/Solver.jl:24-64, 114-131).  Every call goes through the C
ABI of libbem_gb300.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from .geometry import BEMdata, Laplace, Elasticity, from_nodes

_KEEP = "_bem_keepalive"


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def geom_struct(dad: BEMdata, device: bool = False):
    """Pack a BEMdata into the C struct `bem_geom2d`.

    device=False: host numpy arrays (BEM_MEM_HOST).  device=True: the arrays
    are copied once to CUDA tensors (BEM_MEM_DEVICE).  Returns (struct, keep)
    where `keep` holds the arrays alive."""
    arrs = dict(
        px=np.ascontiguousarray(dad.collocation[:, 0], dtype=np.float64),
        py=np.ascontiguousarray(dad.collocation[:, 1], dtype=np.float64),
        nx=np.ascontiguousarray(dad.normal[:, 0], dtype=np.float64),
        ny=np.ascontiguousarray(dad.normal[:, 1], dtype=np.float64),
        jac=np.ascontiguousarray(dad.jacobian, dtype=np.float64),
        elen=np.ascontiguousarray(dad.elem_length, dtype=np.float64),
        gx=np.ascontiguousarray(dad.geo[..., 0].reshape(-1), dtype=np.float64),
        gy=np.ascontiguousarray(dad.geo[..., 1].reshape(-1), dtype=np.float64),
        ew=np.ascontiguousarray(dad.elem_weight, dtype=np.float64))
    if device:
        import torch
        arrs = {k: torch.from_numpy(v).cuda() for k, v in arrs.items()}
        ptr = {k: (v.data_ptr() if v.numel() else None) for k, v in arrs.items()}
    else:
        ptr = {k: (v.ctypes.data if v.size else None) for k, v in arrs.items()}
    g = _lib.BemGeom2D(dad.nt, dad.n, dad.ne, dad.p, dad.ngeo, 0, ptr["px"], ptr["py"], ptr["nx"],
                       ptr["ny"], ptr["jac"], ptr["elen"], ptr["gx"], ptr["gy"], ptr["ew"])
    return g, arrs


def _ptr(x):
    if _is_torch(x):
        return x.data_ptr()
    return x.ctypes.data


def _ld(x) -> int:
    """Leading dimension of a column-major 2-D array / tensor."""
    if _is_torch(x):
        s = x.stride()
        assert s[0] == 1, "expected column-major (Fortran-ordered) storage"
        return s[1] if x.shape[1] > 1 else x.shape[0]
    assert x.flags.f_contiguous, "expected a Fortran-ordered array"
    return x.shape[0]


class _rules:
    """The reference's per-problem quadrature knobs (`nearfield`,
    src/Core/Integration.jl:41-93; `singular`, src/Core/Assembly_full.jl:
    282-283) as context options for the duration of one call."""

    def __init__(self, ctx, nearfield: str, singular: str):
        if nearfield not in _lib.NEARFIELD:
            raise ValueError(f"nearfield must be one of {sorted(_lib.NEARFIELD)}; got {nearfield!r}")
        if singular not in ("guiggiani", "telles"):
            raise ValueError(f"singular must be 'guiggiani' or 'telles'; got {singular!r}")
        self.ctx, self.nf, self.sg = ctx, _lib.NEARFIELD[nearfield], int(singular == "telles")

    def __enter__(self):
        self.ctx.set_option(_lib.BEM_OPT_NEARFIELD, self.nf)
        self.ctx.set_option(_lib.BEM_OPT_SINGULAR, self.sg)

    def __exit__(self, *exc):
        self.ctx.set_option(_lib.BEM_OPT_NEARFIELD, 0)
        self.ctx.set_option(_lib.BEM_OPT_SINGULAR, 0)
        return False


def H_G_gpu(dad: BEMdata, T=np.float32, npg: int = 20, near: str = "cpu", near_factor: float = 1.5,
            device: str = "cuda", out=None, ctx: _lib.Context | None = None, store: bool = True,
            nearfield: str = "tanp3c", singular: str = "guiggiani"):
    """Dense H, G on the GPU (reference `H_G_gpu`).

    T: np.float32 (far field in FP32, near/singular FP64) or np.float64.
    near: "cpu" in the reference means near/singular entries by
    `integrate_element`; here they are computed on the GPU in FP64, so "cpu"
    and "gpu" are both accepted and give the full near correction.
    nearfield ("tanp3c", "plain", "euclid", "csinh", "sinhsinh", "tangent",
    "p3c") and singular
    ("guiggiani", "telles") select the near-singular map and the on-element
    rule, as the reference's cached `nearfield` and `singular` do.
    device must be "cuda" (no CPU fallback).  `out=(H, G)` may pass
    preallocated column-major numpy arrays or CUDA tensors."""
    if device != "cuda":
        raise ValueError("device must be 'cuda'; this build has no CPU path")
    if near not in ("cpu", "gpu"):
        raise ValueError(f"near must be 'cpu' or 'gpu'; got {near!r}")
    T = np.dtype(T)
    if T not in (np.float32, np.float64):
        raise ValueError(f"H_G_gpu T must be float32 or float64; got {T}")
    ctx = ctx or _lib.default_context()
    pr = dad.properties
    dof = pr.ndof
    rows, gcols = dof * dad.nt, dof * dad.n
    dev = False
    if out is None:
        H = np.zeros((rows, rows), dtype=T, order="F")
        G = np.zeros((rows, gcols), dtype=T, order="F")
    else:
        H, G = out
        dev = _is_torch(H)
    g, keep = geom_struct(dad, device=dev)
    mem = _lib.BEM_MEM_DEVICE if dev else _lib.BEM_MEM_HOST
    dt = _lib.BEM_F32 if T == np.float32 else _lib.BEM_F64
    if not isinstance(pr, (Laplace, Elasticity)):
        raise ValueError(f"H_G_gpu supports Laplace and Elasticity; got {type(pr).__name__}")
    with _rules(ctx, nearfield, singular):
        if isinstance(pr, Laplace):
            rc = ctx.L.bem_assemble_laplace2d(ctx.h, g, float(pr.k), int(npg), float(near_factor), dt, mem,
                                              _ptr(H), _ld(H), _ptr(G), _ld(G))
        else:
            rc = ctx.L.bem_assemble_kelvin2d(ctx.h, g, float(pr.mu), float(pr.nu_eff), int(npg),
                                             float(near_factor), dt, mem, _ptr(H), _ld(H), _ptr(G), _ld(G))
    ctx.check(rc, "H_G_gpu")
    if store:
        dad.set_cache(H=H, G=G)
    return H, G


def assemble(dad: BEMdata, npg: int = 20, method: str = "gpu", **kw):
    """`assemble!(dad, npg; method)` for the GPU method."""
    if method != "gpu":
        raise ValueError("this package provides method='gpu' only")
    return H_G_gpu(dad, npg=npg, **kw)


def assemble_system(dad: BEMdata, npg: int = 20, near_factor: float = 1.5, out=None,
                    ctx: _lib.Context | None = None):
    """Assembly with `applyBC`'s column swap fused: FP64 A, b."""
    ctx = ctx or _lib.default_context()
    pr = dad.properties
    dof = pr.ndof
    rows = dof * dad.nt
    if out is None:
        A = np.zeros((rows, rows), order="F")
        b = np.zeros(rows)
        dev = False
        BC = np.ascontiguousarray(dad.BC, dtype=np.int32)
        BV = np.ascontiguousarray(dad.BV, dtype=np.float64)
    else:
        A, b = out
        dev = _is_torch(A)
        if dev:
            import torch
            BC = torch.as_tensor(np.asarray(dad.BC, np.int32)).cuda()
            BV = torch.as_tensor(np.asarray(dad.BV, np.float64)).cuda()
        else:
            BC = np.ascontiguousarray(dad.BC, dtype=np.int32)
            BV = np.ascontiguousarray(dad.BV, dtype=np.float64)
    g, keep = geom_struct(dad, device=dev)
    kind = 0 if isinstance(pr, Laplace) else 1
    p0 = float(pr.k) if kind == 0 else float(pr.mu)
    p1 = 0.0 if kind == 0 else float(pr.nu_eff)
    rc = ctx.L.bem_assemble_system2d(ctx.h, g, kind, p0, p1, _ptr(BC), _ptr(BV), int(npg),
                                     float(near_factor),
                                     _lib.BEM_MEM_DEVICE if dev else _lib.BEM_MEM_HOST, _ptr(A), _ld(A),
                                     _ptr(b))
    ctx.check(rc, "assemble_system")
    return A, b


def split_sol(dad: BEMdata, x: np.ndarray):
    """Scatter the solution of A x = b into the fields (`split_sol!`,
    src/Core/Solver.jl:88-98 for Laplace, 133-146 for elasticity)."""
    x = np.asarray(x, dtype=np.float64)
    BC, BV = np.asarray(dad.BC), np.asarray(dad.BV)
    if dad.ndof == 1:
        T = x[: dad.nt].copy()
        q = np.where(BC == 0, T[: dad.n], BV)
        T[: dad.n] = np.where(BC == 0, BV, T[: dad.n])
        dad.set_cache(T=T, q=q, x=x)
        return T
    nb = 2 * dad.n
    u = np.where(BC == 0, BV, x[:nb])
    t = np.where(BC == 0, x[:nb], BV)
    dad.set_cache(u=u, traction=t, T=u, x=x)
    return u


_MODES = {"mixed": _lib.BEM_SOLVE_MIXED, "fp64": _lib.BEM_SOLVE_FP64}


def solve(dad: BEMdata, npg: int = 20, mode: str = "mixed", tol: float = 1e-14, max_iter: int = 200,
          near_factor: float = 1.5, ctx: _lib.Context | None = None, return_stats: bool = False):
    """`assemble!` + `solve(dad)` on the GPU: fused assembly of A x = b,
    then the mixed-precision solve (FP32 tensor-core LU + FP64 GMRES) or the
    FP64 comparison solve; fills dad.T/dad.q (or dad.u/dad.traction)."""
    ctx = ctx or _lib.default_context()
    pr = dad.properties
    kind = 0 if isinstance(pr, Laplace) else 1
    p0 = float(pr.k) if kind == 0 else float(pr.mu)
    p1 = 0.0 if kind == 0 else float(pr.nu_eff)
    g, keep = geom_struct(dad)
    BC = np.ascontiguousarray(dad.BC, dtype=np.int32)
    BV = np.ascontiguousarray(dad.BV, dtype=np.float64)
    x = np.zeros(pr.ndof * dad.nt)
    st = _lib.BemSolveStats()
    rc = ctx.L.bem_solve2d(ctx.h, g, kind, p0, p1, BC.ctypes.data, BV.ctypes.data, int(npg),
                           float(near_factor), _MODES[mode], float(tol), int(max_iter),
                           _lib.BEM_MEM_HOST, x.ctypes.data, st)
    ctx.check(rc, "solve")
    split_sol(dad, x)
    stats = dict(iterations=st.iterations, rel_residual=st.rel_residual, pivoted=bool(st.pivoted),
                 t_assemble_ms=st.t_assemble_ms,
                 t_factor_ms=st.t_factor_ms, t_refine_ms=st.t_refine_ms)
    dad.set_cache(solve_stats=stats)
    return (dad.T, stats) if return_stats else dad.T


def solve_system(A, b, mode: str = "mixed", tol: float = 1e-14, max_iter: int = 200,
                 ctx: _lib.Context | None = None):
    """Dense A x = b (the `bem_linsolve` seam).  A: column-major numpy array
    or CUDA tensor (FP64); returns (x, stats)."""
    ctx = ctx or _lib.default_context()
    dev = _is_torch(A)
    n = A.shape[0]
    if dev:
        import torch
        x = torch.zeros(n, dtype=torch.float64, device=A.device)
    else:
        A = np.asfortranarray(A, dtype=np.float64)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(n)
    st = _lib.BemSolveStats()
    rc = ctx.L.bem_solve_system(ctx.h, n, _ptr(A), _ld(A), _ptr(b), _MODES[mode], float(tol),
                                int(max_iter), _lib.BEM_MEM_DEVICE if dev else _lib.BEM_MEM_HOST,
                                _ptr(x), st)
    ctx.check(rc, "solve_system")
    return x, dict(iterations=st.iterations, rel_residual=st.rel_residual,
                   t_factor_ms=st.t_factor_ms, t_refine_ms=st.t_refine_ms, pivoted=bool(st.pivoted))


def recover_strain_stress(dad: BEMdata, u=None, t=None, ctx: _lib.Context | None = None):
    """Boundary strain and stress at the collocation nodes of a solved Kelvin
    problem (`recover_strain_stress!`, src/Elasticity/StrainStress.jl:35-99):
    (eps, sigma), n x 3 Voigt each; stored in dad.cache as strain, stress.
    u, t default to the cached solution (`dad.u`, `dad.traction`)."""
    pr = dad.properties
    if not isinstance(pr, Elasticity):
        raise ValueError("recover_strain_stress needs an elasticity problem")
    if u is None or t is None:
        if "u" not in dad.cache or "traction" not in dad.cache:
            raise ValueError("no displacement/traction: call solve first")
    u = np.ascontiguousarray(dad.cache["u"] if u is None else u, dtype=np.float64)
    t = np.ascontiguousarray(dad.cache["traction"] if t is None else t, dtype=np.float64)
    ctx = ctx or _lib.default_context()
    g, keep = geom_struct(dad, device=False)
    eps = np.zeros((dad.n, 3), order="F")
    sig = np.zeros((dad.n, 3), order="F")
    rc = ctx.L.bem_strain_stress2d(ctx.h, g, float(pr.lam), float(pr.mu), _ptr(u), _ptr(t),
                                   _lib.BEM_MEM_HOST, _ptr(eps), _ptr(sig))
    ctx.check(rc, "strain_stress")
    dad.set_cache(strain=eps, stress=sig)
    return eps, sig


def hoop_stress(dad: BEMdata, center=(0.0, 0.0), sigma=None):
    """sigma_theta_theta at the boundary nodes about `center` (polar rotation
    of the recovered stress)."""
    sig = dad.cache["stress"] if sigma is None else sigma
    X = np.asarray(dad.collocation[: dad.n]) - np.asarray(center)
    th = np.arctan2(X[:, 1], X[:, 0])
    s, c = np.sin(th), np.cos(th)
    return sig[:, 0] * s * s + sig[:, 1] * c * c - 2 * sig[:, 2] * s * c


def kirsch_static(r, theta, a=1.0, sigma_inf=1.0):
    """Static Kirsch stresses (sigma_rr, sigma_tt, sigma_rt) around a hole of
    radius a under remote sigma_xx (data/elastico/iso/analytical_elastodynamics.jl:532-540)."""
    r2 = (a / np.asarray(r)) ** 2
    r4 = r2 * r2
    srr = sigma_inf / 2 * (1 - r2) + sigma_inf / 2 * (1 - 4 * r2 + 3 * r4) * np.cos(2 * theta)
    stt = sigma_inf / 2 * (1 + r2) - sigma_inf / 2 * (1 + 3 * r4) * np.cos(2 * theta)
    srt = -sigma_inf / 2 * (1 + 2 * r2 - 3 * r4) * np.sin(2 * theta)
    return srr, stt, srt


def interior_laplace(dad: BEMdata, pts, npg: int = 16, T=None, q=None, ctx: _lib.Context | None = None,
                     nearfield: str = "tanp3c", singular: str = "guiggiani"):
    """Laplace potential at interior points from the solved boundary data
    (`interior_laplace`, src/Laplace/Lubrication.jl:399-416): every element
    integrated with the near-field quadrature, T(p) = (g.q - h.T) / c.
    nearfield and singular select the near-singular map (the problem's
    cached `nearfield`) and the rule for points on an element, as in
    `H_G_gpu`."""
    if not isinstance(dad.properties, Laplace):
        raise ValueError("interior_laplace needs a Laplace problem")
    if T is None or q is None:
        if "T" not in dad.cache or "q" not in dad.cache:
            raise ValueError("no boundary solution: call solve first")
    pts = np.ascontiguousarray(np.asarray(pts, dtype=np.float64).reshape(-1, 2))
    T = np.ascontiguousarray((dad.cache["T"] if T is None else T)[: dad.n], dtype=np.float64)
    q = np.ascontiguousarray(dad.cache["q"] if q is None else q, dtype=np.float64)
    xp, yp = np.ascontiguousarray(pts[:, 0]), np.ascontiguousarray(pts[:, 1])
    out = np.zeros(len(pts))
    ctx = ctx or _lib.default_context()
    g, keep = geom_struct(dad, device=False)
    with _rules(ctx, nearfield, singular):
        rc = ctx.L.bem_interior_laplace2d(ctx.h, g, float(dad.properties.k), int(npg), _ptr(T), _ptr(q),
                                          len(pts), _ptr(xp), _ptr(yp), _lib.BEM_MEM_HOST, _ptr(out))
    ctx.check(rc, "interior_laplace")
    return out


# worker counts chosen by tune_batch, per batch shape
_BATCH_TUNED: dict = {}
BATCH_WORKERS_DEFAULT = 16


def _batch_key(dads, npg: int, mode: str):
    """Shape class of a batch: mode, rule, and the number of domains and
    sum of N^2 each to within a factor of two."""
    nt = np.fromiter((d.nt * d.ndof for d in dads), dtype=np.float64, count=len(dads))
    return (mode, int(npg), len(dads).bit_length(), int(np.sum(nt * nt)).bit_length())


def batch_workers(dads, npg: int = 20, mode: str = "mixed") -> int:
    """Worker count `solve_batch(..., nworkers=0)` uses for this batch: the
    tuned one for its shape class, else BATCH_WORKERS_DEFAULT."""
    return _BATCH_TUNED.get(_batch_key(list(dads), npg, mode), BATCH_WORKERS_DEFAULT)


def tune_batch(dads, npg: int = 20, mode: str = "mixed", candidates=(4, 8, 16, 24, 32),
               ctx: _lib.Context | None = None, repeats: int = 1, **kw):
    """Autotuner of the batched solve's concurrency (the number of worker
    streams that overlap the domains' pipelines).

    Runs one warm-up pass at the largest candidate (it sizes every worker's
    device workspace and page-locked staging), then times `solve_batch` over
    `dads` `repeats` times per candidate and keeps the fastest (minimum over
    repeats) for batches of this shape class (`_batch_key`); later
    `solve_batch(..., nworkers=0)` calls use it.  The solutions do not depend
    on the worker count.  Returns (best, {count: seconds})."""
    import time
    dads = list(dads)
    cands = sorted({int(c) for c in candidates if 1 <= int(c) <= 32})
    if not dads or not cands:
        raise ValueError("tune_batch: needs domains and worker counts in 1..32")
    solve_batch(dads, npg=npg, mode=mode, nworkers=cands[-1], ctx=ctx, **kw)
    times = {}
    for w in cands:
        best = float("inf")
        for _ in range(max(1, int(repeats))):
            t0 = time.perf_counter()
            solve_batch(dads, npg=npg, mode=mode, nworkers=w, ctx=ctx, **kw)
            best = min(best, time.perf_counter() - t0)
        times[w] = best
    pick = min(times, key=lambda w: (times[w], w))
    _BATCH_TUNED[_batch_key(dads, npg, mode)] = pick
    return pick, times


def solve_batch(dads, npg: int = 20, mode: str = "mixed", tol: float = 1e-14, max_iter: int = 200,
                near_factor: float = 1.5, nworkers: int = 0, ctx: _lib.Context | None = None,
                return_stats: bool = False):
    """`solve(dad)` for many independent domains in one call
    (bem_solve2d_batch): every domain is assembled and solved on the GPU;
    worker threads with their own streams overlap the domains (`nworkers`;
    0: the count `tune_batch` chose for this batch shape, else
    BATCH_WORKERS_DEFAULT).  All domains share the physics of the first one.
    Returns the list of solution vectors (and the per-domain stats)."""
    dads = list(dads)
    if not dads:
        return ([], []) if return_stats else []
    if nworkers == 0:
        nworkers = batch_workers(dads, npg, mode)
    ctx = ctx or _lib.default_context()
    pr = dads[0].properties
    kind = 0 if isinstance(pr, Laplace) else 1
    for d in dads:
        if type(d.properties) is not type(pr) or d.properties != pr:
            raise ValueError("solve_batch: all domains need the same physics")
    dof = pr.ndof
    geoms = (_lib.BemGeom2D * len(dads))()
    keep = []
    for i, d in enumerate(dads):
        g, k = geom_struct(d, device=False)
        geoms[i] = g
        keep.append(k)
    bc_len = [dof * d.n for d in dads]
    x_len = [dof * d.nt for d in dads]
    bc_off = np.concatenate([[0], np.cumsum(bc_len)[:-1]]).astype(np.int64)
    x_off = np.concatenate([[0], np.cumsum(x_len)[:-1]]).astype(np.int64)
    BC = np.ascontiguousarray(np.concatenate([np.asarray(d.BC, np.int32) for d in dads]))
    BV = np.ascontiguousarray(np.concatenate([np.asarray(d.BV, np.float64) for d in dads]))
    x = np.zeros(int(sum(x_len)))
    stats = (_lib.BemSolveStats * len(dads))()
    p0 = float(pr.k) if kind == 0 else float(pr.mu)
    p1 = 0.0 if kind == 0 else float(pr.nu_eff)
    rc = ctx.L.bem_solve2d_batch(ctx.h, len(dads), geoms, kind, p0, p1, _ptr(BC), _ptr(BV),
                                 bc_off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), int(npg),
                                 float(near_factor), _MODES[mode], float(tol), int(max_iter),
                                 _lib.BEM_MEM_HOST, _ptr(x),
                                 x_off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), int(nworkers), stats)
    if rc not in (_lib.BEM_OK, 4):
        ctx.check(rc, "solve_batch")
    xs = [x[o:o + n].copy() for o, n in zip(x_off, x_len)]
    for d, xi in zip(dads, xs):
        split_sol(d, xi)
    if return_stats:
        st = [dict(status=s.status, iterations=s.iterations, rel_residual=s.rel_residual,
                   t_assemble_ms=s.t_assemble_ms, t_factor_ms=s.t_factor_ms, t_refine_ms=s.t_refine_ms)
              for s in stats]
        return xs, st
    return xs


def adjoint_laplace(dad: BEMdata, q_target, npg: int = 16, near_factor: float = 1.5, tol: float = 1e-14,
                    max_iter: int = 200, ctx: _lib.Context | None = None, return_stats: bool = False):
    """J = 1/2 sum_{BC=0} (q - q_target)^2 and its gradient dJ/d(node x, y),
    (n, 2), by the adjoint method through assembly and the mixed-precision
    solve (bem_adjoint_laplace2d).  `dad` must take its element geometry from
    its nodes (`from_nodes`)."""
    if not isinstance(dad.properties, Laplace):
        raise ValueError("adjoint_laplace needs a Laplace problem")
    if dad.ngeo != 0 or dad.nt != dad.n:
        raise ValueError("adjoint_laplace needs node-interpolant elements (from_nodes) and no internal points")
    ctx = ctx or _lib.default_context()
    g, keep = geom_struct(dad, device=False)
    BC = np.ascontiguousarray(dad.BC, dtype=np.int32)
    BV = np.ascontiguousarray(dad.BV, dtype=np.float64)
    qt = np.ascontiguousarray(q_target, dtype=np.float64)
    if qt.shape != (dad.n,):
        raise ValueError("q_target must have one value per boundary node")
    J = ctypes.c_double()
    grad = np.zeros(2 * dad.n)
    st = _lib.BemSolveStats()
    rc = ctx.L.bem_adjoint_laplace2d(ctx.h, g, float(dad.properties.k), _ptr(BC), _ptr(BV), _ptr(qt), int(npg),
                                     float(near_factor), float(tol), int(max_iter), _lib.BEM_MEM_HOST,
                                     ctypes.byref(J), _ptr(grad), ctypes.byref(st))
    if rc not in (_lib.BEM_OK, 4):
        ctx.check(rc, "adjoint_laplace")
    out = (J.value, grad.reshape(dad.n, 2))
    if return_stats:
        return out + (dict(status=st.status, iterations=st.iterations, t_assemble_ms=st.t_assemble_ms,
                           t_factor_ms=st.t_factor_ms, t_refine_ms=st.t_refine_ms),)
    return out


def shape_misfit(X, p: int, BC, BV, q_target, npg: int = 16, ctx: _lib.Context | None = None) -> float:
    """J(X) = 1/2 sum_{BC=0} (q_i - q_target_i)^2 for boundary nodes X (n, 2)
    of elements that interpolate their own p+1 nodes (element e owns rows
    e(p+1) .. e(p+1)+p), BC, BV and q_target fixed.  The primal of the
    ChainRulesCore `rrule` that INTEGRATION.md gives for Julia."""
    return shape_misfit_rrule(X, p, BC, BV, q_target, npg=npg, ctx=ctx)[0]


def shape_misfit_rrule(X, p: int, BC, BV, q_target, npg: int = 16, ctx: _lib.Context | None = None):
    """(J, pullback) with pullback(dJ) = dJ * dJ/dX, (n, 2): the call sequence
    of the Julia `rrule` -- one bem_adjoint_laplace2d call (forward solve,
    adjoint solve, backward kernels) for the value and the gradient, and a
    pullback that only scales the stored gradient by the incoming cotangent."""
    X = np.asarray(X, dtype=np.float64)
    n = X.shape[0]
    if X.shape != (n, 2) or n % (p + 1):
        raise ValueError("X must be (n, 2) with n a multiple of p + 1")
    dad = from_nodes("shape", X.reshape(n // (p + 1), p + 1, 2), p, Laplace(1.0), BC, BV)
    J, grad = adjoint_laplace(dad, q_target, npg=npg, ctx=ctx)

    def pullback(dJ):
        return float(dJ) * grad

    return J, pullback


def adjoint_laplace_batch(cases, npg: int = 16, near_factor: float = 1.5, tol: float = 1e-14,
                          max_iter: int = 200, nworkers: int = 16, ctx: _lib.Context | None = None,
                          return_stats: bool = False):
    """`adjoint_laplace` for many independent domains in one call
    (bem_adjoint_laplace2d_batch): `cases` is a sequence of (dad, q_target)
    pairs sharing the conductivity of the first; worker threads with their
    own streams overlap the domains.  Returns the list of (J, grad) (and the
    per-domain stats)."""
    cases = list(cases)
    if not cases:
        return ([], []) if return_stats else []
    dads = [d for d, _ in cases]
    k = dads[0].properties
    for d in dads:
        if not isinstance(d.properties, Laplace) or d.properties != k:
            raise ValueError("adjoint_laplace_batch needs Laplace problems with the same conductivity")
        if d.ngeo != 0 or d.nt != d.n:
            raise ValueError("adjoint_laplace_batch needs node-interpolant elements (from_nodes) and no "
                             "internal points")
    qts = [np.asarray(q, dtype=np.float64).reshape(-1) for _, q in cases]
    for d, q in zip(dads, qts):
        if q.shape != (d.n,):
            raise ValueError("q_target must have one value per boundary node")
    ctx = ctx or _lib.default_context()
    geoms = (_lib.BemGeom2D * len(dads))()
    keep = []
    for i, d in enumerate(dads):
        g, kp = geom_struct(d, device=False)
        geoms[i] = g
        keep.append(kp)
    lens = np.array([d.n for d in dads], np.int64)
    off = np.zeros(len(dads), np.int64)
    np.cumsum(lens[:-1], out=off[1:])
    BC = np.ascontiguousarray(np.concatenate([np.asarray(d.BC, np.int32) for d in dads]))
    BV = np.ascontiguousarray(np.concatenate([np.asarray(d.BV, np.float64) for d in dads]))
    QT = np.ascontiguousarray(np.concatenate(qts))
    J = np.zeros(len(dads))
    grad = np.zeros(2 * int(lens.sum()))
    stats = (_lib.BemSolveStats * len(dads))()
    rc = ctx.L.bem_adjoint_laplace2d_batch(ctx.h, len(dads), geoms, float(k.k), _ptr(BC), _ptr(BV), _ptr(QT),
                                           off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), int(npg),
                                           float(near_factor), float(tol), int(max_iter), _ptr(J), _ptr(grad),
                                           int(nworkers), stats)
    if rc not in (_lib.BEM_OK, 4):
        ctx.check(rc, "adjoint_laplace_batch")
    out = [(float(J[i]), grad[2 * o:2 * (o + n)].reshape(n, 2).copy()) for i, (o, n) in enumerate(zip(off, lens))]
    if return_stats:
        st = [dict(status=s.status, iterations=s.iterations, t_assemble_ms=s.t_assemble_ms,
                   t_factor_ms=s.t_factor_ms, t_refine_ms=s.t_refine_ms) for s in stats]
        return out, st
    return out


RBF_KINDS = {"PHS1": 1, "PHS2": 2, "PHS3": 3, "PHS4": 4, "PHS5": 5, "PHS6": 6, "PHS7": 7, "fundamental": 10}


def dibem_ifid(dad: BEMdata, rbf: str = "PHS3", dtype=np.float64, epsa: float = 1e-16, near_factor: float = 1.5,
               ctx: _lib.Context | None = None, near: bool = False, npg: int = 16):
    """Boundary sums IF, ID of the DIBEM domain integrals at every collocation
    point: the far sums (`_dibem_IFID_ka`, src/Laplace/DIBEM_GPU.jl:209-270),
    which skip near and on-element pairs, and with `near` also their npg-point
    Gauss-rule correction (`_dibem_correct_near_cpu!`, :272-300, FP64), which
    together are the reference's IF, ID."""
    ctx = ctx or _lib.default_context()
    if not isinstance(dad.properties, Laplace):
        raise ValueError("dibem_ifid supports Laplace meshes")
    g, keep = geom_struct(dad)
    IF = np.zeros(dad.nt, dtype=dtype)
    ID = np.zeros(dad.nt, dtype=dtype)
    dt = _lib.BEM_F64 if np.dtype(dtype) == np.float64 else _lib.BEM_F32
    rc = ctx.L.bem_dibem_ifid2d(ctx.h, g, float(dad.properties.k), RBF_KINDS[rbf], float(epsa), float(near_factor),
                                dt, _lib.BEM_MEM_HOST, _ptr(IF), _ptr(ID))
    ctx.check(rc, "dibem_ifid")
    if near:
        IF = np.ascontiguousarray(IF, dtype=np.float64)
        ID = np.ascontiguousarray(ID, dtype=np.float64)
        rc = ctx.L.bem_dibem_ifid_near2d(ctx.h, g, float(dad.properties.k), RBF_KINDS[rbf], float(epsa),
                                         float(near_factor), int(npg), _lib.BEM_MEM_HOST, _ptr(IF), _ptr(ID))
        ctx.check(rc, "dibem_ifid_near")
    return IF, ID


def discretize(cad, p: int, ctx: _lib.Context | None = None):
    """Collocation nodes (ne, p+1, 2), outward normals, Jacobians (ne, p+1),
    element lengths (ne,) and Gauss weights (p+1,) of elements given by their
    equispaced CAD nodes `cad` (ne, ngeo, 2), computed on the device: the
    geometry loop of `format2d` (src/Core/Input.jl:163-185).  Same outputs as
    `geometry.discretize_curves`; pass it as `from_cad(..., discretize=...)`."""
    ctx = ctx or _lib.default_context()
    cad = np.asarray(cad, dtype=np.float64)
    ne, ngeo = cad.shape[0], cad.shape[1]
    cx, cy = np.ascontiguousarray(cad[..., 0]), np.ascontiguousarray(cad[..., 1])
    n = ne * (p + 1)
    px, py, nx, ny, J = (np.empty(n) for _ in range(5))
    L = np.empty(ne)
    wi = np.empty(p + 1)
    rc = ctx.L.bem_discretize2d(ctx.h, ne, ngeo, p, _ptr(cx), _ptr(cy), _lib.BEM_MEM_HOST, _ptr(px), _ptr(py),
                                _ptr(nx), _ptr(ny), _ptr(J), _ptr(L), _ptr(wi))
    ctx.check(rc, "discretize")
    nodes = np.stack([px, py], axis=-1).reshape(ne, p + 1, 2)
    normal = np.stack([nx, ny], axis=-1).reshape(ne, p + 1, 2)
    return nodes, normal, J.reshape(ne, p + 1), L, wi


def cells_array(cells) -> np.ndarray:
    """Corner arrays of triangles and quadrangles as (ncell, 4, 2), a triangle
    repeating its last corner (the layout of bem_orient2d)."""
    out = np.empty((len(cells), 4, 2))
    for i, c in enumerate(cells):
        c = np.asarray(c, dtype=np.float64)
        out[i, :len(c)] = c
        out[i, len(c):] = c[-1]
    return out


def orient_normals(dad: BEMdata, cells, ctx: _lib.Context | None = None) -> np.ndarray:
    """Flip, in place, the normals of every element whose point 0.1 L behind
    its first node lies in none of the domain `cells` (`_orient_normals_outward!`,
    src/Core/Input.jl:376-389), on the device; returns the flipped mask (ne,)."""
    ctx = ctx or _lib.default_context()
    n, p = dad.n, dad.p
    px = np.ascontiguousarray(dad.collocation[:n, 0])
    py = np.ascontiguousarray(dad.collocation[:n, 1])
    nx = np.ascontiguousarray(dad.normal[:, 0])
    ny = np.ascontiguousarray(dad.normal[:, 1])
    elen = np.ascontiguousarray(dad.elem_length, dtype=np.float64)
    cz = np.ascontiguousarray(cells_array(cells)) if len(cells) else np.zeros((1, 4, 2))
    flipped = np.zeros(dad.ne, np.int32)
    rc = ctx.L.bem_orient2d(ctx.h, dad.ne, p, _ptr(px), _ptr(py), _ptr(nx), _ptr(ny), _ptr(elen), len(cells),
                            _ptr(cz), _lib.BEM_MEM_HOST, _ptr(flipped))
    ctx.check(rc, "orient_normals")
    dad.normal = np.ascontiguousarray(np.stack([nx, ny], axis=-1))
    return flipped.astype(bool)


def dibem_fd(dad: BEMdata, rbf: str = "PHS3", dtype=np.float64, epsa: float = 1e-16,
             ctx: _lib.Context | None = None):
    """Dense pairwise DIBEM matrices over all collocation points
    (`_dibem_FD_ka`, src/Laplace/DIBEM_GPU.jl:179-208; Kelvin
    src/Elasticity/Assembly_GPU.jl:258-280): F_ij = phi(R), D_ij = u*(x_i, x_j)."""
    ctx = ctx or _lib.default_context()
    pr = dad.properties
    kind = 0 if isinstance(pr, Laplace) else 1
    p0 = float(pr.k) if kind == 0 else float(pr.mu)
    p1 = 0.0 if kind == 0 else float(pr.nu_eff)
    pts = np.asarray(dad.collocation, np.float64)
    px, py = np.ascontiguousarray(pts[:, 0]), np.ascontiguousarray(pts[:, 1])
    nt = len(pts)
    dof = 1 if kind == 0 else 2
    F = np.zeros((nt, nt), dtype=dtype, order="F")
    D = np.zeros((dof * nt, dof * nt), dtype=dtype, order="F")
    dt = _lib.BEM_F64 if dtype == np.float64 else _lib.BEM_F32
    rc = ctx.L.bem_dibem_fd2d(ctx.h, nt, _ptr(px), _ptr(py), kind, p0, p1, RBF_KINDS[rbf], float(epsa), dt,
                              _lib.BEM_MEM_HOST, _ptr(F), nt, _ptr(D), dof * nt)
    ctx.check(rc, "dibem_fd")
    return F, D
