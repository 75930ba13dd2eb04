"""The failure paths of the C ABI, none of them a GPU fault: the CG
iteration cap (the reference's "pulou pressao", 9_grad.f90:393-398,590), the
cap of the volume-correction loop (unbounded upstream, 14_level_set.f90:243),
a NaN in a host buffer before upload, a truncated or foreign restart file
(SULI_BAD_CONFIG, the handle left as it was), and a bounded device wait that
runs out (SULI_DEVICE_TIMEOUT: a wait on an mbarrier that no copy completes,
given up after one second)."""
import os
import time

import numpy as np
import pytest

from suli_gb300 import cases
from suli_gb300._abi import (PREC_FP64, PREC_MIXED, SULI_BAD_CONFIG, SULI_CG_MAXITER, SULI_DEVICE_TIMEOUT,
                             SULI_NONFINITE, SULI_VOL_LOOP_CAP)

pytestmark = pytest.mark.gpu


def _start(gpu_lib, case):
    g = gpu_lib.SuliGPU(case.params)
    g.start(case.fields)
    return g


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_MIXED])
def test_cg_cap_warns(gpu_lib, precision):
    case = cases.dam_break(24, 12, 12, precision=precision)
    case.params.cg_max_iter = 1
    g = _start(gpu_lib, case)
    g.set_stage(1)
    for name in ("visco", "convdiff", "complementos", "tempo"):
        getattr(g, name)()
    g.contorno(2)
    it = g.graddin()                         # returns the warning, not an error
    assert it >= 1
    assert g.warnings & (1 << SULI_CG_MAXITER)
    g.step(1)                                # the step goes on after the warning, as upstream
    assert g.diag().status_flags & (1 << SULI_CG_MAXITER)
    g.close()


def test_volume_loop_cap(gpu_lib):
    case = cases.dam_break(24, 12, 12)
    case.params.vol_loop_max = 0
    g = _start(gpu_lib, case)
    g.set_scalar("VOL_INI", 1.5 * g.scalar("VOL_INS"))   # 33 % volume error: the loop must run
    g.level_set()
    d = g.diag()
    assert d.vol_loops == 0
    assert d.status_flags & (1 << SULI_VOL_LOOP_CAP)
    g.close()
    # with passes allowed the same state runs the loop (and stays bounded)
    case = cases.dam_break(24, 12, 12)
    case.params.vol_loop_max = 3
    g = _start(gpu_lib, case)
    g.set_scalar("VOL_INI", 1.5 * g.scalar("VOL_INS"))
    g.level_set()
    assert 1 <= g.diag().vol_loops <= 3
    g.close()


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_MIXED])
def test_nan_in_host_buffer_is_reported(gpu_lib, precision):
    case = cases.dam_break(24, 12, 12, precision=precision)
    u = case.fields["U"].copy(order="F")
    u[10, 6, 3] = np.nan
    case.fields["U"] = u
    g = _start(gpu_lib, case)
    with pytest.raises(gpu_lib.SuliError) as ei:
        g.step(2)
    assert ei.value.code == SULI_NONFINITE
    g.close()
    # a clean state steps without the status
    g = _start(gpu_lib, cases.dam_break(24, 12, 12, precision=precision))
    g.step(2)
    assert np.isfinite(g.conmassa())
    g.close()


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_MIXED])
def test_tma_wait_timeout_is_reported(gpu_lib, monkeypatch, precision):
    """SULI_TEST_TMA_SHORTFALL=1 (read at handle creation) arms the last
    plane of each unit of the TMA-staged convdiff with 16 bytes more than its
    copies deliver, while the case has no timeout recorded: the bounded
    waits run out after a second, the kernel marks the case and returns, and
    the step reports SULI_DEVICE_TIMEOUT -- no fault, no hang.  The context
    stays usable: a fresh handle of the same case steps, twice to the same
    bits."""
    monkeypatch.setenv("SULI_TEST_TMA_SHORTFALL", "1")
    g = _start(gpu_lib, cases.dam_break(40, 16, 24, precision=precision))
    monkeypatch.delenv("SULI_TEST_TMA_SHORTFALL")
    t0 = time.time()
    with pytest.raises(gpu_lib.SuliError) as ei:
        g.step(1)
    assert ei.value.code == SULI_DEVICE_TIMEOUT
    assert time.time() - t0 < 120
    g.close()
    out = []
    for _ in range(2):
        g = _start(gpu_lib, cases.dam_break(40, 16, 24, precision=precision))
        g.step(2)
        out.append(g.download("PRD1"))
        g.close()
    assert np.isfinite(out[0]).all()
    assert np.array_equal(out[0], out[1])


def test_bad_restart_files_leave_the_handle(gpu_lib, tmp_path):
    case = cases.dam_break(24, 12, 12)
    g = _start(gpu_lib, case)
    g.step(1)
    good = tmp_path / "good.bin"
    g.restart_save(str(good))
    u_before = g.download("U")
    raw = good.read_bytes()
    # truncated in the middle of the last record, then in the middle of the first
    for cut in (len(raw) - 100, 200):
        bad = tmp_path / ("cut%d.bin" % cut)
        bad.write_bytes(raw[:cut])
        with pytest.raises(gpu_lib.SuliError) as ei:
            g.restart_load(str(bad))
        assert ei.value.code == SULI_BAD_CONFIG
        assert np.array_equal(g.download("U"), u_before)
    # not a restart file at all
    junk = tmp_path / "junk.bin"
    junk.write_bytes(os.urandom(4096))
    with pytest.raises(gpu_lib.SuliError) as ei:
        g.restart_load(str(junk))
    assert ei.value.code == SULI_BAD_CONFIG
    # written for another batch
    other = _start(gpu_lib, cases.dam_break(16, 8, 8))
    with pytest.raises(gpu_lib.SuliError) as ei:
        other.restart_load(str(good))
    assert ei.value.code == SULI_BAD_CONFIG
    other.close()
    # the intact file still loads
    g.restart_load(str(good))
    assert np.array_equal(g.download("U"), u_before)
    g.close()
