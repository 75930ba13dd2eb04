"""The mixed form (FP32 storage and stencils, FP32 CG with FP64 reliable
updates, FP64 sums) against the FP64 oracle, and the batched form (uneven
cases in one launch) against single-case runs."""
import numpy as np
import pytest

from helpers import oracle_for, rel_l2
from suli_gb300 import cases
from suli_gb300._abi import PREC_MIXED

pytestmark = pytest.mark.gpu


def _vel(get):
    return np.concatenate([get(n).ravel() for n in ("U", "V", "W")])


@pytest.mark.parametrize("nsteps", [5])
def test_mixed_dam_break_against_oracle(gpu_lib, nsteps):
    case = cases.dam_break(32, 16, 16, cg_tol=1e-12)
    o = oracle_for(case)
    o.step(nsteps)
    cm = cases.dam_break(32, 16, 16, precision=PREC_MIXED, cg_tol=1e-12)
    g = gpu_lib.SuliGPU(cm.params)
    g.start(cm.fields)
    g.step(nsteps)
    ev = rel_l2(_vel(g.download), _vel(o.field))
    els = rel_l2(g.download("LS"), o.field("LS"))
    pg = g.download("PRD1")[1:-1, 1:-1, 1:-1]
    po = o.field("PRD1")[1:-1, 1:-1, 1:-1]
    ep = rel_l2(pg - pg.mean(), po - po.mean())
    g.close()
    print("mixed vs oracle after %d steps: velocity %.2e ls %.2e p %.2e" % (nsteps, ev, els, ep))
    assert ev <= 1e-5 and els <= 1e-6 and ep <= 1e-5


def test_mixed_cg_converges_on_fp64_residual(gpu_lib):
    cm = cases.dam_break(32, 16, 16, precision=PREC_MIXED, cg_tol=1e-10)
    g = gpu_lib.SuliGPU(cm.params)
    g.start(cm.fields)
    g.step(2)
    d = g.diag()
    assert all(n > 0 for n in d.cg_iters)
    assert all(n >= 1 for n in d.cg_outer)
    assert d.maxdiv < 1e-6
    g.close()


def test_batch_equals_single_cases(gpu_lib):
    dims, hcol, amp = cases.ensemble_dims(3, seed=7, lo=12, hi=20)
    cs = [cases.ensemble_case(i, dims, hcol, amp) for i in range(3)]
    gb = gpu_lib.SuliGPU([c.params for c in cs])
    gb.start([c.fields for c in cs])
    for _ in range(2):
        gb.step(1)
    for i, c in enumerate(cs):
        gs = gpu_lib.SuliGPU(c.params)
        gs.start(c.fields)
        gs.step(2)
        for name in ("U", "V", "W", "LS", "PRD1"):
            a = gb.download(name, case=i)
            b = gs.download(name)
            assert np.array_equal(a, b) or rel_l2(a, b) < 1e-12, (i, name, rel_l2(a, b))
        gs.close()
    gb.close()
