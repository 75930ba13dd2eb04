"""The manufactured solution of 13_mms.f90 (steady, a = 0) on the GPU in both
forms: the error against the analytic fields falls under refinement, and the
mixed form's error is the FP64 form's (its own rounding is orders of
magnitude below the discretisation error)."""
import math

import pytest

from suli_gb300 import cases
from suli_gb300._abi import PREC_FP64, PREC_MIXED

pytestmark = pytest.mark.gpu


def _mms_errors(gpu_lib, n, precision, steps):
    c = cases.mms_case(n, precision=precision)
    g = gpu_lib.SuliGPU(c.params)
    g.start(c.fields)
    g.step(steps)
    e = g.mms_error()
    g.close()
    return e


def test_mms_converges_and_forms_agree(gpu_lib):
    errs = {}
    for n in (16, 32):
        # 100 steps: past the start-up transient, the error is the
        # discretisation's (after 10-20 steps it is not)
        steps = 100
        e64 = _mms_errors(gpu_lib, n, PREC_FP64, steps)
        em = _mms_errors(gpu_lib, n, PREC_MIXED, steps)
        errs[n] = e64
        for a, b in zip(em[:3], e64[:3]):        # u, v, w errors
            assert abs(a - b) <= 1e-3 * b + 1e-12, (n, em, e64)
    # observed order of the velocity error between 16^3 and 32^3
    order = math.log(errs[16][0] / errs[32][0], 2)
    assert order > 0.5, errs
