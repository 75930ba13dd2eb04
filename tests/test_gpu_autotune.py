"""The autotuner (suli_autotune): every launch shape it may choose gives the
same bits -- the planes per unit of the TMA-staged convdiff, the one-block
coarse end of the V-cycle, the blocks per SM of the level-0 sweep -- and the
tuner keeps the fastest of the shapes it timed, once per device and workload
shape (a second handle of the same shape takes the cached choice)."""
import numpy as np
import pytest

from suli_gb300 import cases
from suli_gb300._abi import PREC_MIXED

pytestmark = pytest.mark.gpu

FIELDS = ("U", "V", "W", "LS", "PRD1")
KNOBS = ("SULI_TUNE", "SULI_TUNE_CD", "SULI_TUNE_SWEEP", "SULI_MG_CTA_CELLS")


def _batch():
    dims, hcol, amp = cases.ensemble_dims(4, seed=5, lo=24, hi=80)
    return [cases.ensemble_case(i, dims, hcol, amp, precision=PREC_MIXED) for i in range(4)]


def _run(gpu_lib, monkeypatch, env, steps=3):
    for k in KNOBS:
        monkeypatch.delenv(k, raising=False)
    for k, v in env.items():
        monkeypatch.setenv(k, str(v))
    cs = _batch()
    g = gpu_lib.SuliGPU([c.params for c in cs])      # the shapes are read at creation
    for k in KNOBS:
        monkeypatch.delenv(k, raising=False)
    g.start([c.fields for c in cs])
    g.step(steps)
    out = [{n: g.download(n, case=q) for n in FIELDS} for q in range(len(cs))]
    tun = g.tuning()
    g.close()
    return out, tun


def test_every_tuned_shape_gives_the_same_bits(gpu_lib, monkeypatch):
    ref, t0 = _run(gpu_lib, monkeypatch, {"SULI_TUNE": 0})
    assert t0["tuned"] == 0 and t0["convdiff_planes"] == 16
    for env in ({"SULI_TUNE_CD": 0}, {"SULI_TUNE_CD": 2}, {"SULI_TUNE_SWEEP": 2},
                {"SULI_TUNE_SWEEP": 3, "SULI_MG_CTA_CELLS": 0}, {"SULI_TUNE_CD": 0, "SULI_MG_CTA_CELLS": 65536}):
        got, t = _run(gpu_lib, monkeypatch, env)
        assert t["tuned"] == 0
        for q, (a, b) in enumerate(zip(got, ref)):
            for n in FIELDS:
                assert np.array_equal(a[n], b[n]), (env, q, n, float(np.abs(a[n] - b[n]).max()))


def test_tuner_keeps_the_fastest_and_caches_it(gpu_lib, monkeypatch):
    out, t = _run(gpu_lib, monkeypatch, {}, steps=1)     # tunes after the first step
    assert t["tuned"] == 1
    assert t["convdiff_planes"] in (8, 16, 32)
    assert t["mg_block_cells"] in (0, 4096, 16384, 65536)
    assert t["sweep_blocks_per_sm"] in (0, 2, 3)
    assert 0.0 < t["tuned_ms"] <= t["default_ms"]
    # a second handle of the same shape: the cached choice, no new timing
    cs = _batch()
    g = gpu_lib.SuliGPU([c.params for c in cs])
    g.start([c.fields for c in cs])
    t2 = g.autotune()
    g.close()
    assert t2["tuned"] == 1
    for k in ("convdiff_planes", "mg_block_cells", "sweep_blocks_per_sm", "default_ms", "tuned_ms"):
        assert t2[k] == t[k], k
