"""CPU-side checks of the C ABI: the library loads and exports every entry
point declared in include/*.h; argument checks need no GPU."""
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        for m in re.finditer(r"\b(bem_[a-z0-9_]+)\s*\(", txt):
            names.add(m.group(1))
    return names


def test_library_exports_declared_symbols():
    from bem_gmsh_gb300 import _lib, _build
    if not os.path.exists(_build.LIB):
        _build.build()
    L = _lib.load()
    syms = declared_symbols()
    assert "bem_assemble_laplace2d" in syms
    missing = [s for s in sorted(syms) if not hasattr(L, s)]
    assert not missing, missing


def test_status_strings_and_bad_device():
    import ctypes
    from bem_gmsh_gb300 import _lib
    L = _lib.load()
    assert L.bem_status_string(0) == b"ok"
    h = ctypes.c_void_p()
    # no GPU in this container (or an out-of-range id on a GPU machine): invalid
    assert L.bem_ctx_create(1 << 20, ctypes.byref(h)) == 1


def test_geometry_builders():
    import numpy as np
    from bem_gmsh_gb300 import quadrado, star_domain, plate_with_hole
    d = quadrado(ndiv=20)
    assert (d.n, d.nt, d.ne) == (152, 513, 76)
    assert np.allclose(np.linalg.norm(d.normal, axis=1), 1)
    s = star_domain(2731, p=2, seed=0)
    assert s.n == 8193 and s.ngeo == 3
    # outward normals: n . x > 0 on a star-shaped curve around the origin
    assert np.all(np.sum(s.normal * s.Nodes, axis=1) > 0)
    pl = plate_with_hole()
    assert pl.n == (1024 + 342) * 3 and pl.ndof == 2
    assert int((pl.BC == 0).sum()) == 3


def declared_arity():
    """{name: number of parameters} of every function declared in include/*.h."""
    out = {}
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        txt = re.sub(r"//[^\n]*", "", txt)
        for m in re.finditer(r"\b(bem_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;", txt, flags=re.S):
            params = m.group(2).strip()
            out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_python_bindings_match_declared_arity():
    # every ctypes binding passes exactly the parameters the header declares
    from bem_gmsh_gb300 import _lib, _build
    if not os.path.exists(_build.LIB):
        _build.build()
    L = _lib.load()
    arity = declared_arity()
    assert arity.get("bem_adjoint_laplace2d_batch") == 16
    checked = 0
    for name, n in sorted(arity.items()):
        f = getattr(L, name)
        if f.argtypes is None:
            continue
        assert len(f.argtypes) == n, (name, len(f.argtypes), n)
        checked += 1
    assert checked >= 20


def test_python_constants_match_header_defines():
    from bem_gmsh_gb300 import _lib
    txt = open(os.path.join(ROOT, "include", "bem_gb300.h")).read()
    defines = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(BEM_[A-Z0-9_]+)\s+(\d+)\b", txt)}
    for name in ("BEM_NOALLOC_MAX_NT", "BEM_NOALLOC_MAX_NE"):
        assert getattr(_lib, name) == defines[name], name
    # every option, status and kind constant the binding defines has the header's value
    named = [n for n in defines if hasattr(_lib, n)]
    assert sum(n.startswith("BEM_OPT_") for n in named) >= 11, named
    for name in named:
        assert getattr(_lib, name) == defines[name], name


def test_nearfield_codes_match_the_oracle():
    """The near-field map names of the binding carry the codes the oracle
    uses for the same maps (the GPU parity tests pass one name to both)."""
    from bem_gmsh_gb300 import _lib
    from oracle import oracle as orc
    assert _lib.NEARFIELD == orc.NEARFIELD


def test_quadrature_knobs_rejected_on_the_host():
    """Names outside the built maps and rules (the anisotropic `:zsinh`, a
    misspelt rule) raise before any device call, as the reference's
    `transform` / `H_G_gpu` reject them."""
    from bem_gmsh_gb300.api import _rules
    with pytest.raises(ValueError):
        _rules(None, "zsinh", "guiggiani")
    with pytest.raises(ValueError):
        _rules(None, "tanp3c", "gauss")
    r = _rules(None, "sinhsinh", "telles")
    assert (r.nf, r.sg) == (4, 1)
