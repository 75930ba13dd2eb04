"""The oracle against golden vectors of the reference itself.

tests/golden/*.npz hold the state of small cases after each of two full
time steps of SuLi-IC's own Fortran routines (1_principal.f90:69-111),
executed in this container by tests/golden/f90sub.py (a runner for the
Fortran 90 subset the hot-path files use; there is no Fortran compiler on
either machine) through tests/golden/make_golden.py, which also sets each
case up the way the reference's program starts a run.  Here the oracle
runs the same cases from the same start and must reproduce every field and
the volume integral: on this toolchain bit for bit; the bound below is a
few units in the last place of each field's largest value.  (The GPU path
is held to the oracle by the GPU parity tests.)"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _cases():
    import sys
    sys.path.insert(0, GOLDEN)
    import make_golden
    return make_golden, {name: (case, n) for name, case, n in make_golden.cases()}


MG, CASES = _cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_the_reference(name, tmp_path):
    import pyoracle
    path = os.path.join(GOLDEN, name + ".npz")
    assert os.path.exists(path), "fixture missing: run tests/golden/make_golden.py"
    g = np.load(path)
    case, nsteps = CASES[name]
    assert int(g["steps"]) == nsteps
    pyoracle.Oracle.set_threads(1)
    o = MG.oracle_setup(case)
    fields = list(MG.FIELDS) + list(MG.model_fields(case.params))
    for s in range(nsteps + 1):
        if s:
            o.step()
            o.conmassa()        # the divergence field of PLOT's CONMASSA, as the reference run after each step
        tag = "s%d" % s
        for f in fields:
            key = "%s_%s" % (tag, f)
            if f in MG.STATIC and s > 0:
                continue            # kept at the start only (the obstacle does not change)
            ref = g[key]
            got = o.field(f)
            assert got.shape == ref.shape, (tag, f, got.shape, ref.shape)
            assert np.isfinite(ref).all(), (tag, f, "non-finite reference field")
            scale = float(np.abs(ref).max()) or 1.0
            err = float(np.abs(got - ref).max())
            assert err <= 4e-16 * scale, (tag, f, err, scale)
        if s:
            vi = float(g["%s_vol_ins" % tag])
            assert abs(o.scalar("VOL_INS") - vi) <= 4e-16 * abs(vi), (tag, o.scalar("VOL_INS"), vi)
    assert abs(o.scalar("VOL_INI") - float(g["s0_vol_ini"])) <= 4e-16 * abs(float(g["s0_vol_ini"]))
    # the field record of PRTSCR (4_plot.f90:501-620) for the final state,
    # byte for byte (float32 fields, the record's length markers)
    for tp in (0, 1):
        key = "prtscr%d" % tp
        if key not in g.files:
            continue
        path = os.path.join(str(tmp_path), "campos_%d" % tp)
        o.prtscr_write(path, tp)
        got = np.fromfile(path, dtype=np.uint8)
        ref = g[key]
        assert got.size == ref.size, (tp, got.size, ref.size)
        keep = np.ones(ref.size, dtype=bool)
        if case.params.ibm_t == 2:
            # obs_ls, the record's 8th array, is the one known deviation: the
            # reference reinitialises this output-only level set
            # (3_contorno.f90:992), the oracle and the GPU write it as set up
            p = case.params
            n1, n = (p.nx + 1) * (p.ny + 1) * (p.nz + 1), p.nx * p.ny * p.nz
            start = 4 + 4 * (6 * n1 + n)
            keep[start:start + 4 * n1] = False
        assert (got[keep] == ref[keep]).all(), tp


ROUTINES = {name: (case, seed) for name, case, seed in MG.routine_cases()}


@pytest.mark.parametrize("name", sorted(ROUTINES))
def test_oracle_routines_reproduce_the_reference(name):
    """One RK stage routine by routine (contorno(1), visco, convdiff,
    complementos, tempo, contorno(2), posdin) from a seeded random state with
    velocities of both signs everywhere: the oracle's fields after each
    routine against the reference's."""
    import pyoracle
    path = os.path.join(GOLDEN, name + ".npz")
    assert os.path.exists(path), "fixture missing: run tests/golden/make_golden.py"
    g = np.load(path)
    case, _ = ROUTINES[name]
    pyoracle.Oracle.set_threads(1)
    o = MG.oracle_setup(case)
    for f in ("U", "V", "W", "PRD1"):
        o.set_field(f, g["in_%s" % f])
    o.set_stage(1)
    for q, (routine, args, fields) in enumerate(MG.SEQUENCE):
        getattr(o, routine)(*args)
        for f in fields:
            ref = g["r%d_%s" % (q, f)]
            got = o.field(f)
            assert got.shape == ref.shape, (routine, f, got.shape, ref.shape)
            assert np.isfinite(ref).all(), (routine, f)
            scale = float(np.abs(ref).max()) or 1.0
            err = float(np.abs(got - ref).max())
            assert err <= 4e-16 * scale, (routine, f, err, scale)


def test_fixture_regenerates_from_the_reference_sources():
    """Provenance: where the reference's sources are present (the build
    container, not the GPU machine), the generator reproduces a committed fixture
    exactly from them."""
    if not os.path.isdir(os.path.join(MG.REFROOT, "SuLi-IC")):
        pytest.skip("reference sources not present")
    name = "dam_break_12x6x6"
    case, nsteps = CASES[name]
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    prog = MG.load_reference()
    MG.setup(prog, case)
    for s in range(1, nsteps + 1):
        MG.step(prog)
        snap = MG.snapshot(prog, "s%d" % s, case.params)
        for k, v in snap.items():
            assert np.array_equal(np.asarray(v), g[k]), k
