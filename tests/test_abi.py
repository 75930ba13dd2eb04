"""C-ABI checks that need no GPU: the library builds for sm_103a, loads,
exports every entry point declared in include/*.h, reports field shapes as
the reference allocates them, and refuses to run without a CUDA device (no
CPU fallback)."""
import ctypes as C
import glob
import os
import re

import pytest

from suli_gb300 import _abi
from suli_gb300 import build as sbuild

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        names |= set(re.findall(r"^\s*(?:int|void)\s+(suli_\w+)\s*\(", txt, flags=re.M))
    return names


@pytest.fixture(scope="module")
def lib():
    sbuild.build()
    from suli_gb300 import solver
    return solver.load_library()


def test_exports_every_declared_symbol(lib):
    declared = _declared()
    assert len(declared) >= 25
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    from suli_gb300 import solver
    assert set(solver.EXPORTS) == declared


def test_field_shapes_match_reference_allocations(lib):
    p = _abi.default_params(nx=10, ny=7, nz=5, dx=0.1, dy=0.1, dz=0.1, dt=1e-3)
    for name, fid in _abi.FIELD_ID.items():
        lo = (C.c_int * 3)()
        hi = (C.c_int * 3)()
        assert lib.suli_field_shape(C.byref(p), fid, lo, hi) == 0
        elo, ehi = _abi.field_bounds(p, name)
        assert tuple(lo) == elo and tuple(hi) == ehi, name


def test_default_params_agree(lib):
    a = _abi.SuliParams()
    lib.suli_default_params(C.byref(a))
    b = _abi.default_params()
    for name, _ in _abi.SuliParams._fields_:
        x, y = getattr(a, name), getattr(b, name)
        if hasattr(x, "__len__"):        # fixed-size arrays (the Stokes V coefficients)
            x, y = list(x), list(y)
        assert x == y, name


def test_no_cpu_fallback_without_device(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from suli_gb300 import solver
    from suli_gb300 import cases
    with pytest.raises(solver.SuliError) as ei:
        solver.SuliGPU(cases.dam_break(8, 8, 8).params)
    assert ei.value.code == _abi.SULI_NO_DEVICE


def test_bad_config_is_rejected_before_device(lib):
    from suli_gb300 import solver
    p = _abi.default_params(nx=8, ny=8, nz=8, dx=0.1, dy=0.1, dz=0.1, dt=1e-3, der=1)
    h = C.c_void_p()
    rc = lib.suli_create(C.byref(p), C.byref(h))
    assert rc == _abi.SULI_BAD_CONFIG
    assert "der" in solver.last_error()
