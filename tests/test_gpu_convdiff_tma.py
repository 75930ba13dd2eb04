"""The TMA-staged convdiff (operands staged in shared memory by tensor-map
loads, k_convdiff_tma.cu) against the gather kernel (operands read from
global memory, SULI_CONVDIFF=0) from the same state: the same per-face
arithmetic (conv_faces.cuh), so the tendencies agree to round-off, in both
forms, for an uneven batch and for the configurations whose stencils take
the other paths -- periodic x (the end units read the wrap from global
memory), surface tension, the k equation, the sponge.  Then one whole step
(the fused convdiff + complementos) from the same state."""
import numpy as np
import pytest

from helpers import STATE_FIELDS, model_fields, rel_l2
from suli_gb300 import cases
from suli_gb300._abi import PREC_FP64, PREC_MIXED

pytestmark = pytest.mark.gpu


def _batch(kind, prec):
    if kind == "uneven":
        dims, hcol, amp = cases.ensemble_dims(4, seed=3, lo=20, hi=70)
        return [cases.ensemble_case(i, dims, hcol, amp, precision=prec) for i in range(4)]
    if kind == "periodic_ibm":
        return [cases.open_channel(70, 12, 20, dt=2e-3, radius=0.25, cg_tol=1e-10, periodic=True, precision=prec)]
    if kind == "capillary":
        return [cases.capillary_column(40, 6, 0.25, precision=prec)]
    if kind == "k_les":
        return [cases.k_channel(40, 10, 20, m_turb=2, precision=prec)]
    return [cases.sponge_tank(48, 6, 20, esp_type=1, precision=prec)]


def _handle(gpu_lib, cs):
    g = gpu_lib.SuliGPU([c.params for c in cs])
    g.start([c.fields for c in cs])
    return g


def _same_state(src, dst):
    for q, p in enumerate(src.params):
        for n in STATE_FIELDS + model_fields(p):
            dst.upload(n, src.download(n, case=q), case=q)
        for s in ("VOL_INI", "VOL_INS"):
            dst.set_scalar(s, src.scalar(s, case=q), case=q)
    for s in ("T", "IT", "RNG"):
        dst.set_scalar(s, src.scalar(s))


@pytest.mark.parametrize("prec", [PREC_FP64, PREC_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["uneven", "periodic_ibm", "capillary", "k_les", "sponge"])
def test_tma_convdiff_matches_gather(gpu_lib, monkeypatch, kind, prec):
    cs = _batch(kind, prec)
    ga = _handle(gpu_lib, cs)
    ga.step(2)
    monkeypatch.setenv("SULI_CONVDIFF", "0")
    gb = _handle(gpu_lib, _batch(kind, prec))
    monkeypatch.delenv("SULI_CONVDIFF", raising=False)
    _same_state(ga, gb)
    for g in (ga, gb):
        g.set_stage(2)
        g.convdiff()
    tol = 1e-13 if prec == PREC_FP64 else 2e-6
    for q in range(len(cs)):
        # the three components as one vector (Fv is zero in a y-uniform flow)
        a = np.concatenate([ga.download(n, case=q).ravel() for n in ("FU", "FV", "FW")])
        b = np.concatenate([gb.download(n, case=q).ravel() for n in ("FU", "FV", "FW")])
        assert np.abs(b).max() > 0
        assert rel_l2(a, b) <= tol, (kind, q, rel_l2(a, b))
    # one whole step (the fused convdiff + complementos) from the same state
    _same_state(ga, gb)
    for g in (ga, gb):
        g.step(1)
    tol = 1e-9 if prec == PREC_FP64 else 1e-5
    for q in range(len(cs)):
        va = np.concatenate([ga.download(n, case=q).ravel() for n in ("U", "V", "W")])
        vb = np.concatenate([gb.download(n, case=q).ravel() for n in ("U", "V", "W")])
        assert rel_l2(va, vb) <= tol, (kind, q, rel_l2(va, vb))
    ga.close()
    gb.close()
