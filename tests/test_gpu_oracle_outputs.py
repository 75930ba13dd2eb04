"""Two outputs of the hot path checked against the oracle on identical
inputs: the divergence field and max|div| of CONMASSA (4_plot.f90:386-394)
on a random staggered velocity field, and the masked RMS errors of the
manufactured solution (13_mms.f90:391-451) at 16^3 and 32^3."""
import numpy as np
import pytest

import pyoracle
from helpers import copy_state, oracle_for, rel_l2
from suli_gb300 import cases
from suli_gb300._abi import PREC_FP64, PREC_MIXED, field_shape

pytestmark = pytest.mark.gpu


def _random_velocity(p, seed):
    rng = np.random.default_rng(seed)
    return {n: np.asfortranarray(rng.standard_normal(field_shape(p, n))) for n in ("U", "V", "W")}


@pytest.mark.parametrize("dims", [(40, 24, 20), (17, 9, 33)])
def test_conmassa_divergence_against_oracle(gpu_lib, dims):
    case = cases.dam_break(*dims)
    p = case.params
    f = _random_velocity(p, 3)
    o = pyoracle.Oracle(p)
    for n, a in f.items():
        o.set_field(n, a)
    m_o = o.conmassa()
    div_o = o.field("DIV").copy()
    # FP64 form: the same formula in the same order, so the same bits
    g = gpu_lib.SuliGPU(p)
    for n, a in f.items():
        g.upload(n, a)
    m_g = g.conmassa()
    assert np.array_equal(g.download("DIV"), div_o)
    assert m_g == m_o
    g.close()
    # mixed form: FP64 divergence of the FP64 masters times the reciprocal
    # spacings, stored in FP32
    pm = p.copy()
    pm.precision = PREC_MIXED
    gm = gpu_lib.SuliGPU(pm)
    for n, a in f.items():
        gm.upload(n, a)
    m_m = gm.conmassa()
    assert rel_l2(gm.download("DIV"), div_o) <= 1e-7
    assert abs(m_m - m_o) <= 1e-13 * m_o
    gm.close()


@pytest.mark.parametrize("n", [16, 32])
@pytest.mark.parametrize("precision", [PREC_FP64, PREC_MIXED])
def test_mms_error_against_oracle(gpu_lib, n, precision):
    case = cases.mms_case(n)
    o = oracle_for(case, warm_steps=3)
    e_o = o.mms_error()
    c2 = cases.mms_case(n, precision=precision)
    g = gpu_lib.SuliGPU(c2.params)
    g.start(c2.fields)
    copy_state(o, g)
    e_g = g.mms_error()
    g.close()
    assert all(x > 0 for x in e_o[:3]), e_o
    tol = 1e-12 if precision == PREC_FP64 else 1e-6
    for a, b in zip(e_g, e_o):
        assert abs(a - b) <= tol * abs(b) + 1e-300, (e_g, e_o)
