"""ctypes binding of libbem_gb300.so (the C ABI declared in include/bem_gb300.h).

There is no CPU fallback: if the library is missing or no CUDA device is
present the calls raise.
"""
from __future__ import annotations

import ctypes
import os

from . import _build

BEM_OK = 0
BEM_F32, BEM_F64 = 32, 64
BEM_MEM_HOST, BEM_MEM_DEVICE = 0, 1
BEM_SOLVE_FP64, BEM_SOLVE_MIXED = 0, 1
BEM_OPT_TCGEN05 = 1
BEM_OPT_KERNEL_TIMING = 2
BEM_OPT_FAR_DF = 3
BEM_OPT_GRAPHS = 4
BEM_OPT_PIVOT_FALLBACK = 5
BEM_OPT_WAIT_LIMIT = 6
BEM_OPT_INJECT = 7
BEM_OPT_NEARFIELD = 8
BEM_OPT_SINGULAR = 9
BEM_OPT_TC_RESERVE = 10
BEM_OPT_SWEEP_CTAS = 11
NEARFIELD = {"tanp3c": 0, "plain": 1, "euclid": 2, "csinh": 3, "sinhsinh": 4, "tangent": 5, "p3c": 6}
BEM_NOALLOC_MAX_NT, BEM_NOALLOC_MAX_NE = 16384, 8192
KERNEL_CLASSES = ["far", "near", "lu_prep", "lu_crit", "lu_trail", "trsv", "gemv", "lu_total", "lu_diag",
                  "lu_panels", "lu_thin"]

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "device out of memory",
          4: "refinement did not converge", 5: "device wait timed out", 6: "unsupported"}

D = ctypes.c_double
PD = ctypes.POINTER(ctypes.c_double)
I32 = ctypes.c_int32
I64 = ctypes.c_int64
VP = ctypes.c_void_p


class BemGeom2D(ctypes.Structure):
    _fields_ = [("nt", I32), ("n", I32), ("ne", I32), ("p", I32), ("ngeo", I32), ("reserved", I32),
                ("px", VP), ("py", VP), ("nx", VP), ("ny", VP), ("jac", VP), ("elen", VP),
                ("geo_x", VP), ("geo_y", VP), ("elem_weight", VP)]


class BemSolveStats(ctypes.Structure):
    _fields_ = [("status", I32), ("iterations", I32), ("rel_residual", D), ("t_assemble_ms", D),
                ("t_factor_ms", D), ("t_refine_ms", D), ("pivoted", I32), ("reserved", I32)]


class BemError(RuntimeError):
    """A C-ABI call failed; `status` is its BEM_ERR_* code."""

    def __init__(self, msg: str, status: int = 0):
        super().__init__(msg)
        self.status = status


_lib = None


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the shared library (building it first only if asked)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_build.LIB):
        if not build_if_missing:
            raise BemError(f"{_build.LIB} is missing: run __graft_entry__.build() first")
        _build.build()
    L = ctypes.CDLL(_build.LIB)
    ctx_p = ctypes.c_void_p
    sig = {
        "bem_ctx_create": ([ctypes.c_int, ctypes.POINTER(ctx_p)], ctypes.c_int),
        "bem_ctx_destroy": ([ctx_p], ctypes.c_int),
        "bem_ctx_set_stream": ([ctx_p, VP], ctypes.c_int),
        "bem_last_error": ([ctx_p], ctypes.c_char_p),
        "bem_status_string": ([ctypes.c_int], ctypes.c_char_p),
        "bem_assemble_laplace2d": ([ctx_p, ctypes.POINTER(BemGeom2D), D, ctypes.c_int, D, ctypes.c_int,
                                    ctypes.c_int, VP, I64, VP, I64], ctypes.c_int),
        "bem_assemble_kelvin2d": ([ctx_p, ctypes.POINTER(BemGeom2D), D, D, ctypes.c_int, D, ctypes.c_int,
                                   ctypes.c_int, VP, I64, VP, I64], ctypes.c_int),
        "bem_assemble_system2d": ([ctx_p, ctypes.POINTER(BemGeom2D), ctypes.c_int, D, D, VP, VP,
                                   ctypes.c_int, D, ctypes.c_int, VP, I64, VP], ctypes.c_int),
    }
    optional = {
        "bem_solve2d": ([ctx_p, ctypes.POINTER(BemGeom2D), ctypes.c_int, D, D, VP, VP, ctypes.c_int, D,
                         ctypes.c_int, D, ctypes.c_int, ctypes.c_int, VP, ctypes.POINTER(BemSolveStats)],
                        ctypes.c_int),
        "bem_solve_system": ([ctx_p, I64, VP, I64, VP, ctypes.c_int, D, ctypes.c_int, ctypes.c_int, VP,
                              ctypes.POINTER(BemSolveStats)], ctypes.c_int),
        "bem_ctx_set_option": ([ctx_p, ctypes.c_int, ctypes.c_int], ctypes.c_int),
        "bem_selftest": ([ctx_p, ctypes.c_int, ctypes.c_int, PD], ctypes.c_int),
        "bem_kernel_trace": ([ctx_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int), PD, PD], ctypes.c_int),
        "bem_kernel_times": ([ctx_p, PD, ctypes.POINTER(I64), ctypes.c_int], ctypes.c_int),
        "bem_launch_count": ([], I64),
        "bem_dibem_ifid2d": ([ctx_p, ctypes.POINTER(BemGeom2D), D, ctypes.c_int, D, D, ctypes.c_int, ctypes.c_int,
                              VP, VP], ctypes.c_int),
        "bem_discretize2d": ([ctx_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, VP, VP, ctypes.c_int, VP, VP,
                              VP, VP, VP, VP, VP], ctypes.c_int),
        "bem_dibem_ifid_near2d": ([ctx_p, ctypes.POINTER(BemGeom2D), D, ctypes.c_int, D, D, ctypes.c_int,
                                   ctypes.c_int, VP, VP], ctypes.c_int),
        "bem_orient2d": ([ctx_p, ctypes.c_int, ctypes.c_int, VP, VP, VP, VP, VP, ctypes.c_int, VP, ctypes.c_int,
                          VP], ctypes.c_int),
        "bem_dibem_fd2d": ([ctx_p, ctypes.c_int, VP, VP, ctypes.c_int, D, D, ctypes.c_int, D, ctypes.c_int,
                            ctypes.c_int, VP, I64, VP, I64], ctypes.c_int),
        "bem_adjoint_laplace2d": ([ctx_p, ctypes.POINTER(BemGeom2D), D, VP, VP, VP, ctypes.c_int, D, D,
                                   ctypes.c_int, ctypes.c_int, PD, VP, ctypes.POINTER(BemSolveStats)],
                                  ctypes.c_int),
        "bem_adjoint_laplace2d_batch": ([ctx_p, ctypes.c_int, ctypes.POINTER(BemGeom2D), D, VP, VP, VP,
                                         ctypes.POINTER(I64), ctypes.c_int, D, D, ctypes.c_int, VP, VP,
                                         ctypes.c_int, ctypes.POINTER(BemSolveStats)], ctypes.c_int),
        "bem_solve2d_batch": ([ctx_p, ctypes.c_int, ctypes.POINTER(BemGeom2D), ctypes.c_int, D, D, VP, VP,
                               ctypes.POINTER(I64), ctypes.c_int, D, ctypes.c_int, D, ctypes.c_int,
                               ctypes.c_int, VP, ctypes.POINTER(I64), ctypes.c_int,
                               ctypes.POINTER(BemSolveStats)], ctypes.c_int),
        "bem_interior_laplace2d": ([ctx_p, ctypes.POINTER(BemGeom2D), D, ctypes.c_int, VP, VP, I64, VP, VP,
                                    ctypes.c_int, VP], ctypes.c_int),
        "bem_strain_stress2d": ([ctx_p, ctypes.POINTER(BemGeom2D), D, D, VP, VP, ctypes.c_int, VP, VP],
                                ctypes.c_int),
        "bem_assemble_laplace2d_noalloc": ([ctypes.POINTER(BemGeom2D), D, ctypes.c_int, D, ctypes.c_int, VP, I64,
                                            VP, I64, VP], ctypes.c_int),
    }
    for name, (args, res) in {**sig, **optional}.items():
        if not hasattr(L, name):
            if name in sig:
                raise BemError(f"{_build.LIB} does not export {name}")
            continue
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


class Context:
    """One device, one stream, cached device workspace (bem_ctx)."""

    def __init__(self, device: int = 0):
        self.L = load()
        self.h = ctypes.c_void_p()
        rc = self.L.bem_ctx_create(device, ctypes.byref(self.h))
        if rc != BEM_OK:
            raise BemError(f"bem_ctx_create({device}) failed: {STATUS.get(rc, rc)}")

    def check(self, rc: int, what: str):
        if rc != BEM_OK:
            msg = self.L.bem_last_error(self.h).decode()
            raise BemError(f"{what}: {STATUS.get(rc, rc)} {msg}".strip(), rc)

    def set_option(self, option: int, value: int):
        self.check(self.L.bem_ctx_set_option(self.h, option, value), "set_option")

    def selftest_lu(self, n: int):
        """Factor an n x n test matrix with tcgen05 and legacy updates:
        (max |diff|, max |factor|, ms tcgen05, ms legacy)."""
        out = (ctypes.c_double * 4)()
        self.check(self.L.bem_selftest(self.h, 1, n, out), "selftest")
        return tuple(out)

    def kernel_times(self):
        """{class: (ms, groups)} since the last call (needs BEM_OPT_KERNEL_TIMING)."""
        n = len(KERNEL_CLASSES)
        ms = (ctypes.c_double * n)()
        cnt = (I64 * n)()
        self.check(self.L.bem_kernel_times(self.h, ms, cnt, n), "kernel_times")
        return {k: (ms[i], cnt[i]) for i, k in enumerate(KERNEL_CLASSES)}

    def kernel_trace(self, cap: int = 65536):
        """[(class, start ms, end ms)] of the timed kernel classes since the
        last call (needs BEM_OPT_KERNEL_TIMING)."""
        cls = (ctypes.c_int * cap)()
        t0 = (ctypes.c_double * cap)()
        t1 = (ctypes.c_double * cap)()
        n = self.L.bem_kernel_trace(self.h, cap, cls, t0, t1)
        if n < 0:
            self.check(-n, "kernel_trace")
        return [(KERNEL_CLASSES[cls[i]] if cls[i] < len(KERNEL_CLASSES) else cls[i], t0[i], t1[i])
                for i in range(n)]

    def launch_count(self) -> int:
        return int(self.L.bem_launch_count())

    def selftest_gemm(self, n: int):
        """Bulk trailing update of one LU step on an n x n matrix, timed alone:
        (ms per launch, algorithmic GB/s, TF32 TFLOP/s)."""
        out = (ctypes.c_double * 4)()
        self.check(self.L.bem_selftest(self.h, 3, n, out), "selftest")
        return out[0], out[1], out[2]

    def selftest_bulk_compare(self, n: int):
        """Persistent vs per-tile bulk update on the same operands (needs
        BEM_OPT_TCGEN05 = 2): (max |diff|, max |entry|) for the whole trailing
        matrix, then for its part past the first block row and column."""
        out = (ctypes.c_double * 4)()
        self.check(self.L.bem_selftest(self.h, 4, n, out), "selftest")
        return tuple(out)

    def selftest_diag(self, n: int = 128):
        """Blocked vs Gauss-Jordan factorization of one 128 x 128 block:
        (max |diff L\\U|, max |L\\U|, max |diff inverses|, max |inverse|)."""
        out = (ctypes.c_double * 4)()
        self.check(self.L.bem_selftest(self.h, 2, n, out), "selftest")
        return tuple(out)

    def set_stream(self, stream_ptr: int):
        self.check(self.L.bem_ctx_set_stream(self.h, ctypes.c_void_p(stream_ptr)), "set_stream")

    def close(self):
        if self.h:
            self.L.bem_ctx_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = {}


def default_context(device: int = 0) -> Context:
    c = _default_ctx.get(device)
    if c is None:
        c = _default_ctx[device] = Context(device)
    return c
