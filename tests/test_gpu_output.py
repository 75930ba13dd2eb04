"""Field output (PRTSCR, 4_plot.f90:501-635) and restart (restart_salva /
restart_ini, 11_diversos.f90:500-599) through the C ABI on the GPU."""
import numpy as np
import pytest

from helpers import copy_state, model_fields, oracle_for
from suli_gb300 import cases
from suli_gb300._abi import PREC_FP64, PREC_MIXED, SULI_BAD_CONFIG
from test_output import read_fortran_record, split_record

pytestmark = pytest.mark.gpu


def _case(kind, precision):
    if kind == "dam_break":
        return cases.dam_break(24, 12, 10, precision=precision)
    if kind == "k_les":      # nut and ka in the record
        return cases.k_channel(24, 6, 12, m_turb=2, precision=precision)
    if kind == "ipa":        # prd0 + prd1 in the record
        return cases.ipa_tank(16, 6, 12, precision=precision)
    return cases.open_channel(32, 12, 12, dt=2e-3, radius=0.25, periodic=True, precision=precision)


@pytest.mark.parametrize("t_plot", [0, 1])
@pytest.mark.parametrize("precision", [PREC_FP64, PREC_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["dam_break", "channel_ibm", "k_les", "ipa"])
def test_write_fields_matches_oracle(gpu_lib, tmp_path, kind, precision, t_plot):
    """The device-formed record equals the oracle's for the same state: same
    framing and sizes, the same float32 values up to one rounding of values
    that agree to FP64 round-off (the mixed form reads its FP64 masters)."""
    case = _case(kind, PREC_FP64)
    o = oracle_for(case, warm_steps=2)
    gc = _case(kind, precision)
    g = gpu_lib.SuliGPU(gc.params)
    g.start(gc.fields)
    copy_state(o, g)
    o.prtscr_write(tmp_path / "oracle", t_plot)
    g.write_fields(tmp_path / "gpu", 0, t_plot)
    g.close()
    ro = read_fortran_record(tmp_path / "oracle")
    rg = read_fortran_record(tmp_path / "gpu")
    assert ro.size == rg.size
    for n, (a, b) in enumerate(zip(split_record(rg, case.params, t_plot), split_record(ro, case.params, t_plot))):
        scale = max(1e-30, float(np.abs(b).max()))
        assert np.allclose(a, b, rtol=1e-6, atol=1e-6 * scale), (n, float(np.abs(a - b).max()), scale)
    assert np.array_equal(rg[:3 * (gc.params.nx + 1) * (gc.params.ny + 1) * (gc.params.nz + 1)],
                          ro[:3 * (gc.params.nx + 1) * (gc.params.ny + 1) * (gc.params.nz + 1)])   # coordinates


@pytest.mark.parametrize("precision", [PREC_FP64, PREC_MIXED], ids=["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["dam_break", "batch", "k_les", "ipa"])
def test_restart_continues_exactly(gpu_lib, tmp_path, kind, precision):
    """N steps, save, a new handle with the same parameters loads the file and
    runs M steps: the fields, t and it equal those of N + M uninterrupted
    steps (the reference's restart resets t and it)."""
    def mk():
        if kind == "dam_break":
            return [cases.dam_break(24, 12, 12, precision=precision)]
        if kind in ("k_les", "ipa"):
            return [_case(kind, precision)]
        dims, hcol, amp = cases.ensemble_dims(2, seed=9, lo=14, hi=24)
        return [cases.ensemble_case(i, dims, hcol, amp, precision=precision) for i in range(2)]

    cs = mk()
    names = ["U", "V", "W", "PRD1", "LS", "HS", "RHO"] + model_fields(cs[0].params)
    ga = gpu_lib.SuliGPU([c.params for c in cs])
    ga.start([c.fields for c in cs])
    ga.step(4)
    want = {(n, i): ga.download(n, i) for i in range(len(cs)) for n in names}
    t_want, it_want = ga.scalar("T"), ga.scalar("IT")
    ga.close()

    cs = mk()
    gb = gpu_lib.SuliGPU([c.params for c in cs])
    gb.start([c.fields for c in cs])
    gb.step(2)
    gb.restart_save(tmp_path / "restart.bin")
    gb.close()
    gc = gpu_lib.SuliGPU([c.params for c in mk()])
    gc.restart_load(tmp_path / "restart.bin")
    assert gc.scalar("IT") == 2
    gc.step(2)
    for (n, i), a in want.items():
        assert np.array_equal(gc.download(n, i), a), (n, i)
    assert gc.scalar("T") == t_want and gc.scalar("IT") == it_want
    gc.close()


def test_restart_rejects_another_batch(gpu_lib, tmp_path):
    a = cases.dam_break(16, 8, 8)
    g = gpu_lib.SuliGPU(a.params)
    g.start(a.fields)
    g.restart_save(tmp_path / "r.bin")
    g.close()
    b = cases.dam_break(16, 8, 10)
    h = gpu_lib.SuliGPU(b.params)
    with pytest.raises(gpu_lib.SuliError) as ei:
        h.restart_load(tmp_path / "r.bin")
    assert ei.value.code == SULI_BAD_CONFIG
    h.close()
