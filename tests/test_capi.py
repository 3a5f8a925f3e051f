"""The C-ABI library loads and exports every symbol include/jump_mpm.h
declares; argument errors are reported without touching the GPU."""
import ctypes as C
import os
import re

import pytest

from jump_gb300 import _capi

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "jump_mpm.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(mpm_[a-z_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def L():
    if not os.path.exists(_capi.LIB_PATH):
        from jump_gb300 import build
        build.build()
    return _capi.lib()


def test_every_declared_symbol_is_exported(L):
    syms = header_symbols()
    assert "mpm_create" in syms and "mpm_step" in syms
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) == set(_capi.SIGNATURES), "ctypes signatures must cover exactly the header"


def test_abi_version(L):
    assert L.mpm_abi_version() == _capi.ABI_VERSION == 10


def test_argument_errors_without_gpu(L):
    h = C.c_void_p()
    g = _capi.GridDesc()
    p = _capi.Params()
    assert L.mpm_create(None, None, 0, None, C.byref(h)) == _capi.MPM_ERR_ARG
    assert b"null" in L.mpm_last_error()
    g.dim = 4
    p.dt = 1e-3
    assert L.mpm_create(C.byref(g), None, 0, C.byref(p), C.byref(h)) == _capi.MPM_ERR_ARG
    g.dim = 2
    g.nodes[0], g.nodes[1] = 1, 5
    g.xmax[0], g.xmax[1] = 1.0, 1.0
    assert L.mpm_create(C.byref(g), None, 0, C.byref(p), C.byref(h)) == _capi.MPM_ERR_ARG
    g.nodes[0] = 5
    p.dt = 0.0
    assert L.mpm_create(C.byref(g), None, 0, C.byref(p), C.byref(h)) == _capi.MPM_ERR_ARG
    assert L.mpm_step(None, 1, None) == _capi.MPM_ERR_ARG
    assert L.mpm_destroy(None) == _capi.MPM_OK


def test_double_word_precision_refusals_without_gpu(L):
    """MPM_PREC_DW takes 3D USL (any basis) with one velocity field and linear
    elastic, J2 or rigid bodies; anything else is refused before any device work."""
    from jump_gb300 import scenarios
    from jump_gb300.engine import Descriptors

    h = C.c_void_p()
    grid, solids, alg, data = scenarios.two_disks(nodes=11)
    d = Descriptors(grid, solids, tolerance=alg.tolerance, dt=data["dt"], precision="dw")
    assert L.mpm_create(C.byref(d.grid), d.bodies, len(solids), C.byref(d.params), C.byref(h)) == \
        _capi.MPM_ERR_UNSUPPORTED  # 2D
    assert b"MPM_PREC_DW" in L.mpm_last_error()
    grid, solids, alg, data = scenarios.taylor_bar(h=2e-3)
    for kw in ({"algorithm": "musl"}, {"contact": True}):
        d = Descriptors(grid, solids, tolerance=alg.tolerance, dt=data["dt"], precision="dw", **kw)
        assert L.mpm_create(C.byref(d.grid), d.bodies, len(solids), C.byref(d.params), C.byref(h)) == \
            _capi.MPM_ERR_UNSUPPORTED, kw
    from jump_gb300.material import NeoHookeanMaterial
    m = solids[0].mat
    solids[0].mat = NeoHookeanMaterial(m.E, m.nu, m.density, solids[0].parCount)
    d = Descriptors(grid, solids, tolerance=alg.tolerance, dt=data["dt"], precision="dw")
    assert L.mpm_create(C.byref(d.grid), d.bodies, len(solids), C.byref(d.params), C.byref(h)) == \
        _capi.MPM_ERR_UNSUPPORTED  # neo-Hookean
    assert not h.value
    assert L.mpm_batch_create(None, 0, _capi.MPM_PREC_DW, C.byref(h)) == _capi.MPM_ERR_ARG
    assert L.mpm_probe_dw(99, 1, None, None, None, None) == _capi.MPM_ERR_ARG


def test_python_constants_match_the_header():
    """Every integer #define of include/jump_mpm.h that _capi also names has the
    header's value (strategies, tuner candidates, materials, error codes)."""
    import os
    import re
    hdr = os.path.join(os.path.dirname(__file__), "..", "include", "jump_mpm.h")
    defs = dict(re.findall(r"^#define\s+(MPM_\w+)\s+\(?(-?\d+)\)?(?:\s*/\*.*)?\s*$", open(hdr).read(), re.M))
    shared = [k for k in defs if hasattr(_capi, k)]
    assert {"MPM_P2G_TILE", "MPM_P2G_TILE_WARP", "MPM_TUNE_CANDIDATES", "MPM_OK"} <= set(shared)
    for k in shared:
        assert getattr(_capi, k) == int(defs[k]), k
