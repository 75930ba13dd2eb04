"""The variable-z-spacing variant (SuLi-ICdz, dz_t = 1) in the oracle: the
spacing arrays of dz_dist and, as a known answer, the uniform limit -- with
dzmin = dzmax every ICdz stencil (spacing-weighted interpolations, dz(k)
and dzz(k) differences, the WENO z spacing) reduces in exact arithmetic to
SuLi-IC's, so the two oracles agree to round-off over whole steps.  One
upstream quirk does not reduce: SuLi-ICdz divides the z-interpolated face
viscosities of the Fu and Fv terms by dz(k) only over i <= nx, j <= ny, k <=
nz (SuLi-ICdz/6_convdiff.f90:118-126), so the top face and the last x / y
face keep undivided values.  The limit is therefore checked on an inviscid
flow (mu = 0 in both fluids), where those terms vanish, and the viscous
difference is checked to be confined to that quirk's size."""
import numpy as np
import pytest

import pyoracle
from helpers import oracle_for, rel_l2
from suli_gb300 import cases


def test_z_centres_follow_dz_dist():
    nz, a, b = 10, 0.01, 0.03
    z = cases.z_centres_dz(nz, a, b)
    dz = [a + (b - a) * k / nz for k in range(nz + 2)]
    assert z[0] == pytest.approx(dz[1] / 2)
    for k in range(1, nz):
        assert z[k] - z[k - 1] == pytest.approx((dz[k] + dz[k + 1]) / 2)


def _pair(nx, ny, nz, inviscid):
    h = 1.0 / nx
    ca = cases.dam_break(nx, ny, nz)
    cb = cases.dam_break_dz(nx, ny, nz, dzmin=h, dzmax=h)
    assert cb.params.dz_t == 1
    if inviscid:
        for c in (ca, cb):
            c.params.mu_f1 = 0.0
            c.params.mu_f2 = 0.0
    return oracle_for(ca), oracle_for(cb)


def test_uniform_limit_matches_the_uniform_oracle():
    pyoracle.Oracle.set_threads(1)     # serial reductions: the same bits every run
    a, b = _pair(24, 12, 12, inviscid=True)
    for _ in range(3):
        a.step()
        d = a.diag()
        b.set_replay(list(d.cg_iters), d.reinit_iters)   # the same control path on both sides
        b.step()
    vel = [np.concatenate([o.field(n).ravel() for n in ("U", "V", "W")]) for o in (a, b)]
    assert rel_l2(vel[1], vel[0]) <= 1e-9
    assert rel_l2(b.field("LS"), a.field("LS")) <= 1e-12
    pa, pb = a.field("PRD1")[1:-1, 1:-1, 1:-1], b.field("PRD1")[1:-1, 1:-1, 1:-1]
    assert rel_l2(pb - pb.mean(), pa - pa.mean()) <= 1e-9


def test_stretched_grid_differs_and_conserves_volume():
    pyoracle.Oracle.set_threads(1)     # serial reductions: the same bits every run
    c = cases.dam_break_dz(24, 12, 12)
    o = oracle_for(c)
    v0 = o.scalar("VOL_INI")
    o.step(3)
    assert abs(o.scalar("VOL_INS") - v0) <= 0.01 * v0
    assert np.abs(o.field("W")).max() > 0


def test_uniform_limit_viscous_difference_is_the_face_quirk():
    """With viscosity the two oracles part by the undivided top / last-face
    viscous flux of SuLi-ICdz (measured 1.6e-7 in velocity after a step of
    the 24 x 12 x 12 dam break): small, but far above round-off."""
    pyoracle.Oracle.set_threads(1)     # serial reductions: the same bits every run
    a, b = _pair(24, 12, 12, inviscid=False)
    a.step()
    d = a.diag()
    b.set_replay(list(d.cg_iters), d.reinit_iters)
    b.step()
    vel = [np.concatenate([o.field(n).ravel() for n in ("U", "V", "W")]) for o in (a, b)]
    e = rel_l2(vel[1], vel[0])
    assert 1e-9 < e < 1e-5, e
