"""suli_conmassa_noalloc: the divergence check for callers that cannot let a
library allocate device memory (their device buffers belong to their own
allocator or budget).  It must give what suli_conmassa gives for an FP64
handle and what the oracle's CONMASSA gives (4_plot.f90:386-394), call after
call, while working only in the caller's buffers and its built-in scratch:
the device's free memory does not move across its calls.

Collected last on purpose (file name), so a failure here never hides the
result of another test."""
import ctypes as C

import numpy as np
import pytest

import pyoracle
from suli_gb300 import cases

pytestmark = pytest.mark.gpu


def _fields(p, rng):
    from suli_gb300._abi import field_shape
    return {n: np.asfortranarray(rng.standard_normal(field_shape(p, n))) for n in ("U", "V", "W")}


def test_noalloc_divergence_matches_conmassa_and_oracle(gpu_lib):
    import torch
    case = cases.dam_break(40, 24, 20)
    p = case.params
    L = gpu_lib.load_library()
    rng = np.random.default_rng(11)
    g = gpu_lib.SuliGPU(p)
    o = pyoracle.Oracle(p)
    for call in range(2):                      # two calls in a row share the scratch
        f = _fields(p, rng)
        # the caller's own device buffers (reference layout, column-major)
        dev = {n: torch.from_numpy(np.ascontiguousarray(a.T)).cuda() for n, a in f.items()}
        div = torch.zeros((p.nz, p.ny, p.nx), dtype=torch.float64, device="cuda")
        mx = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = L.suli_conmassa_noalloc(dev["U"].data_ptr(), dev["V"].data_ptr(), dev["W"].data_ptr(),
                                     p.nx, p.ny, p.nz, p.dx, p.dy, p.dz, div.data_ptr(), mx.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        d_new = div.cpu().numpy().T
        # the existing entry point on the same field
        for n, a in f.items():
            g.upload(n, a)
        m_ref = g.conmassa()
        d_ref = g.download("DIV")
        assert np.allclose(d_new, d_ref, rtol=1e-12, atol=1e-12 * np.abs(d_ref).max())
        assert abs(mx.item() - m_ref) <= 1e-12 * m_ref
        # and the oracle's CONMASSA: the same formula in the same order
        for n, a in f.items():
            o.set_field(n, a)
        m_o = o.conmassa()
        assert np.array_equal(d_new, o.field("DIV"))
        assert mx.item() == m_o
    g.close()


def test_noalloc_allocates_nothing(gpu_lib):
    import torch
    case = cases.dam_break(64, 32, 32)
    p = case.params
    L = gpu_lib.load_library()
    f = _fields(p, np.random.default_rng(2))
    dev = {n: torch.from_numpy(np.ascontiguousarray(a.T)).cuda() for n, a in f.items()}
    div = torch.zeros((p.nz, p.ny, p.nx), dtype=torch.float64, device="cuda")
    mx = torch.zeros((1,), dtype=torch.float64, device="cuda")
    args = (dev["U"].data_ptr(), dev["V"].data_ptr(), dev["W"].data_ptr(), p.nx, p.ny, p.nz, p.dx, p.dy, p.dz,
            div.data_ptr(), mx.data_ptr(), None)
    assert L.suli_conmassa_noalloc(*args) == 0     # warm-up: module loaded, scratch address looked up
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        assert L.suli_conmassa_noalloc(*args) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert mx.item() > 0


def test_noalloc_rejects_too_many_planes(gpu_lib):
    L = gpu_lib.load_library()
    one = C.c_void_p(8)                        # never dereferenced: rejected before launch
    rc = L.suli_conmassa_noalloc(one, one, one, 4, 4, 4097, 1.0, 1.0, 1.0, one, one, None)
    assert rc == 5                             # SULI_BAD_ARG
