"""GPU parity of the plain FP64 form against the CPU oracle, through the C ABI.

Every reference routine is checked on its own from an identical state (the
oracle's state after a few warm-up steps uploaded into the GPU case), then
whole time steps are checked with the oracle's data-dependent iteration
counts replayed (CG iterations per RK stage, reinitialisation iterations) so
that both sides take the same control path.  Bar: relative L2 <= 1e-10.
"""
import numpy as np
import pytest

from helpers import compare, copy_state, model_compare, oracle_for, rel_l2
from suli_gb300 import cases

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _capped(case, n):
    case.params.cg_max_iter = n
    return case


def _configs():
    return [
        ("dam_break", cases.dam_break(24, 12, 12)),
        # the velocity of a tank near rest is the small difference between the
        # gravity increment and the hydrostatic gradient, which amplifies the
        # CG's stopping error: solve to 1e-12 so it stays below the 1e-10 bar
        ("wave_les", cases.wave_tank(32, 8, 12, dt=5e-4, cg_tol=1e-12)),
        ("mms_periodic", cases.mms_case(16)),
        ("channel_ibm", cases.open_channel(48, 16, 16, dt=2e-3, radius=0.25, cg_tol=1e-10, periodic=True)),
        ("inflow_ibm", cases.open_channel(48, 16, 16, dt=2e-3, radius=0.25, cg_tol=1e-10)),
        # the same inflow channel with the balanced free outflow (outflow_flux
        # = 1): the pressure equation has a solution, so whole steps compare
        ("outflow_ibm", cases.open_channel(64, 16, 16, dt=2e-3, radius=0.25, cg_tol=1e-10, balanced=True)),
        # SuLi-ICdz's stretched z grid (dz_t = 1): dz from 0.6 to 1.4 times
        # the uniform spacing, bed to top.  Its pressure equation has no
        # solution (the operator's z coefficients use dz(k)^2, the divergence
        # and posdin dzz(k): SuLi-ICdz/9_grad.f90:141,166 and 10_pos.f90:41), so
        # the CG runs into round-off chaos after a few thousand iterations;
        # the solve is capped at 40 (the reference's "pulou pressao" path)
        # so that both sides take the same well-defined iterations
        ("dam_break_dz", _capped(cases.dam_break_dz(24, 12, 16), 40)),
        # surface tension (t_tens = 1): weights, curvature, the momentum term
        ("capillary", cases.capillary_column(32, 4, 0.25)),
        # k equation: LES (m_turb = 2) and DES (m_turb = 3), no-slip bed
        ("k_les", cases.k_channel(24, 6, 12, m_turb=2)),
        ("k_des", cases.k_channel(24, 6, 12, m_turb=3)),
        # implicit pressure algorithm (t_press = 2)
        ("ipa", cases.ipa_tank(16, 6, 12)),
        # sponge layer over the last metre (esp_type 1 graded, 2 linear); a
        # tank near rest, solved to 1e-12 like wave_les
        ("sponge1", cases.sponge_tank(32, 4, 16, esp_type=1, cg_tol=1e-12)),
        ("sponge2", cases.sponge_tank(32, 4, 16, esp_type=2, cg_tol=1e-12)),
        # inflow waves (Stokes II, Stokes V) into a flume with a sponge
        ("waves2", cases.wave_flume(24, 4, 16, wave_t=2)),
        ("waves5", cases.wave_flume(24, 4, 16, wave_t=5)),
    ]


def _needs_solvable_pressure(case):
    """Prescribed inflow with free outflow (ccx0 = 3, ccxf = 4) leaves a net
    boundary flux in the all-Neumann pressure equation of graddin: the system
    has no solution, the CG drifts the constant mode of p without bound and
    both sides end in round-off of a huge constant.  Routines downstream of
    the pressure solve are compared on the closed (periodic) channel."""
    if case.params.ccx0 == 3 and case.params.ccxf == 4 and case.params.outflow_flux == 0:
        pytest.skip("pressure equation without a solution (net inflow through an all-Neumann boundary)")


def _warm_steps(case):
    """Steps the oracle takes before the routine tests: none for the wave
    flume, whose incompatible pressure equation diverges the CG (the waves
    are compared routine by routine)."""
    return 0 if case.params.wave_t > 0 else 3


@pytest.fixture(scope="module", params=_configs(), ids=lambda c: c[0])
def pair(request, gpu_lib):
    name, case = request.param
    o = oracle_for(case, warm_steps=_warm_steps(case))
    g = gpu_lib.SuliGPU(case.params)
    g.start(case.fields)
    yield case, o, g
    g.close()


def _sync(o, g):
    copy_state(o, g)


def test_level_set(pair):
    case, o, g = pair
    _sync(o, g)
    g.set_scalar("DT", o.scalar("DT"))
    o.level_set()
    g.set_replay(None, o.diag().reinit_iters)
    g.level_set()
    g.set_replay(None, -1)
    compare(o, g, ["LS", "HS", "RHO", "LS_MU"], TOL)
    if case.params.t_tens:
        compare(o, g, ["HSX", "HSZ", "KURV"], TOL)
        assert np.abs(g.download("KURV")).max() > 0
    assert g.diag().reinit_iters == o.diag().reinit_iters
    assert abs(g.scalar("VOL_INS") - o.scalar("VOL_INS")) <= 1e-12 * abs(o.scalar("VOL_INS"))


def test_level_set_free_running(pair):
    """Without replay the GPU's own signed band-error test picks the same count."""
    case, o, g = pair
    _sync(o, g)
    g.set_scalar("DT", o.scalar("DT"))
    o.level_set()
    g.level_set()
    assert g.diag().reinit_iters == o.diag().reinit_iters
    compare(o, g, ["LS"], TOL)


def test_visco(pair):
    case, o, g = pair
    _sync(o, g)
    o.visco()
    g.visco()
    compare(o, g, ["MU", "visc"], TOL)
    if case.params.m_turb:
        compare(o, g, ["MUT"], TOL)
    if case.params.m_turb >= 2:
        compare(o, g, ["KA", "NUT"], TOL)
        assert g.download("KA").max() > 0


def test_contorno_les(pair):
    """The ghost fills of ka: exact copies (negated for no-slip), edges in the
    reference's plane order."""
    case, o, g = pair
    if case.params.m_turb < 2:
        pytest.skip("no k equation")
    _sync(o, g)
    rng = np.random.default_rng(5)
    ka = rng.random(o.field("KA").shape)
    o.set_field("KA", np.asfortranarray(ka))
    g.upload("KA", np.asfortranarray(ka))
    o.contorno_les()
    g.contorno_les()
    assert np.array_equal(g.download("KA"), o.field("KA"))


def test_boundary_waves(pair):
    """The wave on the inflow planes and ls(1, :, :) at two times, then the
    inflow fill of contorno(2) that reads them (w(0, :, :) = bxz0)."""
    case, o, g = pair
    if case.params.wave_t == 0:
        pytest.skip("no waves")
    _sync(o, g)
    for t in (0.3, 1.7):
        o.set_scalar("T", t)
        g.set_scalar("T", t)
        o.boundary_waves()
        g.boundary_waves()
        compare(o, g, ["LS", "BXX0", "BXX1", "BXZ0"], TOL)
    assert np.abs(g.download("BXZ0")).max() > 0
    o.contorno(2)
    g.contorno(2)
    compare(o, g, ["velocity"], TOL)


def test_exp_press(pair):
    case, o, g = pair
    if case.params.t_press != 2:
        pytest.skip("no IPA")
    _sync(o, g)
    o.exp_press()
    g.exp_press()
    compare(o, g, ["PRD0", "pforce"], TOL)
    assert np.abs(g.download("PZ")).max() > 0


@pytest.mark.parametrize("tt", [1, 2, 3])
def test_convdiff_complementos_tempo(pair, tt):
    case, o, g = pair
    _sync(o, g)
    o.visco()
    g.visco()
    o.set_stage(tt)
    g.set_stage(tt)
    o.convdiff()
    g.convdiff()
    compare(o, g, ["F"], TOL)
    o.complementos()
    g.complementos()
    compare(o, g, ["F"], TOL)
    o.tempo()
    g.tempo()
    compare(o, g, ["velocity"], TOL)


@pytest.mark.parametrize("nlock", [1, 2])
def test_contorno(pair, nlock):
    case, o, g = pair
    _sync(o, g)
    # perturb ghosts so the fills are exercised
    rng = np.random.default_rng(nlock)
    for name in ("U", "V", "W", "PRD1"):
        a = o.field(name)
        a[0, :, :] += rng.standard_normal(a[0].shape)
        a[:, 0, :] += rng.standard_normal(a[:, 0].shape)
        a[:, :, -1] += rng.standard_normal(a[:, :, -1].shape)
        g.upload(name, a)
    o.contorno(nlock)
    g.contorno(nlock)
    for name in ("U", "V", "W", "PRD1"):
        if case.params.ibm_t == 2 and name != "PRD1":
            # image-point values are arithmetic (distance weights), not
            # copies: they agree to round-off, and so do ghosts copied from them
            assert rel_l2(g.download(name), o.field(name)) <= TOL, name
        else:
            d = np.abs(g.download(name) - o.field(name)).max()
            assert d == 0.0, "%s ghost fill differs by %g" % (name, d)


def test_graddin_posdin(pair):
    case, o, g = pair
    _needs_solvable_pressure(case)
    if case.params.mms_t and not case.params.project_under_mms:
        pytest.skip("no projection")
    _sync(o, g)
    for tt in (1, 2):
        o.set_stage(tt)
        g.set_stage(tt)
        o.visco(); g.visco()
        o.convdiff(); g.convdiff()
        o.complementos(); g.complementos()
        o.tempo(); g.tempo()
        o.contorno(2); g.contorno(2)
        it_o = o.graddin()
        g.set_replay([it_o] * 3, -1)
        it_g = g.graddin()
        g.set_replay(None, -1)
        assert it_g == it_o
        compare(o, g, ["PRD1"], TOL)
        if case.params.t_press == 1:   # the IPA step has no posdin
            o.posdin(); g.posdin()
            compare(o, g, ["velocity", "PRD"], TOL)
        o.contorno(1); g.contorno(1)
    m_o = o.conmassa()
    m_g = g.conmassa()
    # max|div| is the CG residual left by the projection: same order, not same bits
    assert abs(m_g - m_o) <= 0.25 * m_o + 1e-12


def test_graddin_free_running_iterations(pair):
    """The GPU's own stopping test lands on the oracle's count (or one off)."""
    case, o, g = pair
    _needs_solvable_pressure(case)
    if case.params.mms_t and not case.params.project_under_mms:
        pytest.skip("no projection")
    _sync(o, g)
    o.set_stage(1)
    g.set_stage(1)
    for x in (o, g):          # predictor, so the solve has a real right-hand side
        x.visco(); x.convdiff(); x.complementos(); x.tempo(); x.contorno(2)
    it_o = o.graddin()
    it_g = g.graddin()
    assert abs(it_g - it_o) <= max(1, int(0.02 * it_o))
    # the Neumann/periodic problem fixes p only up to a constant, which the
    # two iterations drift along differently: compare p minus its mean
    pg = g.download("PRD1")[1:-1, 1:-1, 1:-1]
    po = o.field("PRD1")[1:-1, 1:-1, 1:-1]
    assert rel_l2(pg - pg.mean(), po - po.mean()) <= 1e-8


def test_steps_replayed(pair):
    case, o, g = pair
    _needs_solvable_pressure(case)
    _sync(o, g)
    g.set_scalar("DT", o.scalar("DT"))
    for _ in range(3):
        o.step()
        d = o.diag()
        g.set_replay(list(d.cg_iters), d.reinit_iters)
        g.step(1)
    g.set_replay(None, -1)
    compare(o, g, ["velocity", "PRD1", "LS", "RHO"] + model_compare(case.params), TOL)
    # max|div| after the projection is the CG residual: same order, not same bits
    assert abs(g.diag().maxdiv - o.diag().maxdiv) <= 0.25 * o.diag().maxdiv + 1e-13


def test_ibm_masks_bit_exact(pair):
    case, o, g = pair
    if case.params.ibm_t != 2:
        pytest.skip("no obstacle")
    for name in ("ID_IBMX", "ID_IBMY", "ID_IBMZ", "ID_IBM"):
        a = g.download(name)
        b = o.field(name)
        assert a.sum() > 0
        assert np.array_equal(a, b), "%s differs at %d points" % (name, int((a != b).sum()))
    for name in ("OBS_LSX", "OBS_LSY", "OBS_LSZ", "OBS_LSS"):
        assert rel_l2(g.download(name), o.field(name)) <= TOL


def test_ibm_contorno(pair):
    case, o, g = pair
    if case.params.ibm_t != 2:
        pytest.skip("no obstacle")
    _sync(o, g)
    for nlock in (2, 1, 3):
        o.contorno(nlock)
        g.contorno(nlock)
        compare(o, g, ["velocity", "LS"], TOL)
