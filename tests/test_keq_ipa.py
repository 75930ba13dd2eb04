"""The k-equation model (m_turb = 2 LES, 3 DES; 5_viscosidade.f90:91-145,
6_convdiff.f90:171-205, 3_contorno.f90:666-790, 11_diversos.f90:300-351 and
the kinetic-energy term of complementos :403-444) and the implicit pressure
algorithm (t_press = 2: exp_press 11_diversos.f90:455-495, graddin with the
density rho_f1, 1_principal.f90:82,111) in the oracle, on CPU.  The
reference's tests hold no golden values for either, so the restatement is
pinned on known answers: without flow the k equation reduces to the ODE
dk/dt = -des k^1.5 / lcar, whose exact solution the RK3 sub-stages follow to
O(dt^3); the ghost rules of contorno_les; exp_press on a linear pressure."""
import math

import numpy as np
import pytest

import pyoracle
from suli_gb300 import cases
from suli_gb300._abi import CG_TOL_REL, default_params


def _still_box(m_turb, k0=0.01, lcar=0.1, n=16, dt=1e-3):
    """Water everywhere (ls far above the band), no gravity, free-slip walls:
    no flow, uniform ka = k0."""
    h = 1.0 / n
    p = default_params(nx=n, ny=n, nz=n, dx=h, dy=h, dz=h, dt=dt, ccx0=1, ccxf=1, ccy0=1, ccyf=1,
                       ccz0=1, cczf=1, gx=0.0, gz=0.0, m_turb=m_turb, cg_tol_mode=CG_TOL_REL, cg_tol=1e-10)
    p.lcar = lcar
    o = pyoracle.Oracle(p)
    o.set_field("LS", np.full((n, n, n), 10.0, order="F"))
    ka = np.zeros((n + 2, n + 2, n + 2), order="F")
    ka[1:-1, 1:-1, 1:-1] = k0
    o.set_field("KA", ka)
    o.contorno_les()
    o.heaviside_init()
    for nl in (1, 2, 3):
        o.contorno(nl)
    return p, o


@pytest.mark.parametrize("m_turb,lcar", [(2, 0.1), (3, 0.1), (3, 0.02)])
def test_k_decay_follows_the_ode(m_turb, lcar):
    k0, steps, dt = 0.01, 40, 1e-3
    p, o = _still_box(m_turb, k0=k0, lcar=lcar, dt=dt)
    for _ in range(steps):
        o.step()
    delta = p.dx
    des = 1.0
    if m_turb == 3:
        des = max(1.0, lcar / (p.cdes * delta))     # ka^1.5 / (cdes delta ka^1.5 / lcar)
    c = des / lcar
    t = steps * dt
    exact = 1.0 / (1.0 / math.sqrt(k0) + 0.5 * c * t) ** 2
    ka = o.field("KA")[1:-1, 1:-1, 1:-1]
    assert np.ptp(ka) == 0.0                        # stays uniform
    assert abs(ka[0, 0, 0] - exact) <= 1e-7 * exact, (ka[0, 0, 0], exact)
    assert k0 - ka[0, 0, 0] > 0.03 * k0            # and did decay
    # nut = cmu sqrt(ka) delta, mut = nut rho (:143-144)
    nut = o.field("NUT")
    assert np.allclose(nut, p.cmu * np.sqrt(ka) * delta, rtol=1e-14, atol=0)
    assert np.allclose(o.field("MUT"), nut * o.field("RHO"), rtol=1e-14, atol=0)


def test_contorno_les_ghost_rules():
    case = cases.k_channel(16, 6, 10, m_turb=2)
    p = case.params
    o = pyoracle.Oracle(p)
    rng = np.random.default_rng(3)
    ka = rng.random((p.nx + 2, p.ny + 2, p.nz + 2))
    o.set_field("KA", np.asfortranarray(ka))
    o.contorno_les()
    k = o.field("KA")
    nx, ny, nz = p.nx, p.ny, p.nz
    # x periodic (ccx0 = ccxf = 0), the last fill: whole planes
    assert np.array_equal(k[0], k[nx]) and np.array_equal(k[nx + 1], k[1])
    # y free-slip: copies; z no-slip bed: negated copy; free-slip lid: copy
    s = np.s_[1:nx + 1]
    assert np.array_equal(k[s, 0, :], k[s, 1, :]) and np.array_equal(k[s, ny + 1, :], k[s, ny, :])
    assert np.array_equal(k[s, 1:ny + 1, 0], -k[s, 1:ny + 1, 1])
    assert np.array_equal(k[s, 1:ny + 1, nz + 1], k[s, 1:ny + 1, nz])
    # the interior is untouched
    assert np.array_equal(k[1:-1, 1:-1, 1:-1], ka[1:-1, 1:-1, 1:-1])


def test_k_channel_stays_physical():
    """Sheared channel flow: ka stays finite and non-negative in the cells,
    and the no-slip bed produces more of it than the free stream has."""
    case = cases.k_channel(32, 6, 16, m_turb=2)
    o = pyoracle.Oracle(case.params)
    for k, v in case.fields.items():
        o.set_field(k, v)
    o.contorno_les()
    o.heaviside_init()
    for nl in (1, 2, 3):
        o.contorno(nl)
    for _ in range(10):
        o.step()
    ka = o.field("KA")[1:-1, 1:-1, 1:-1]
    assert np.all(np.isfinite(ka)) and ka.min() >= 0.0
    assert ka[:, :, 0].mean() > ka[:, :, 5].mean()


def test_exp_press_linear_pressure():
    """prd0 += prd1; px = -d(prd0 + prd1)/dx / rho_face: a linear pressure in
    a uniform fluid gives a uniform force."""
    case = cases.ipa_tank(12, 6, 8)
    p = case.params
    o = pyoracle.Oracle(p)
    o.set_field("LS", np.full((p.nx, p.ny, p.nz), 10.0, order="F"))
    o.heaviside_init()
    i = np.arange(p.nx + 2)[:, None, None]
    k = np.arange(p.nz + 2)[None, None, :]
    prd1 = np.asfortranarray(np.broadcast_to(2.0 * i + 0.0 * k, (p.nx + 2, p.ny + 2, p.nz + 2)))
    prd0 = np.asfortranarray(np.broadcast_to(0.0 * i + 3.0 * k, (p.nx + 2, p.ny + 2, p.nz + 2)))
    o.set_field("PRD1", prd1)
    o.set_field("PRD0", prd0)
    o.exp_press()
    rho = p.rho_f2
    assert np.allclose(o.field("PRD0"), prd0 + prd1, rtol=0, atol=1e-12)
    assert np.allclose(o.field("PX"), -2.0 * 2.0 / p.dx / rho, rtol=1e-13)    # prdaux = prd0 + 2 prd1
    assert np.allclose(o.field("PY"), 0.0, atol=1e-15)
    assert np.allclose(o.field("PZ"), -3.0 / p.dz / rho, rtol=1e-13)


def test_ipa_tank_builds_hydrostatic_pressure():
    """Under the IPA the pressure accumulates in prd0: after some steps it
    rises with depth in the water column, and the fall of the water stays
    below free fall."""
    case = cases.ipa_tank(24, 6, 16)
    p = case.params
    o = pyoracle.Oracle(p)
    for k, v in case.fields.items():
        o.set_field(k, v)
    o.heaviside_init()
    for nl in (1, 2, 3):
        o.contorno(nl)
    steps = 20
    for _ in range(steps):
        o.step()
    col = o.field("PRD0")[1:-1, 1:-1, 1:-1].mean(axis=(0, 1))
    water = int(0.45 / p.dz)                        # cells below the surface
    assert np.all(np.diff(col[:water]) < 0), col[:water]
    assert np.abs(o.field("W")).max() < p.gz * steps * p.dt


@pytest.mark.parametrize("esp_type", [1, 2])
def test_sponge_layer_profile(esp_type):
    """sponge_layer (3_contorno.f90:1011-1103) through complementos: Fw loses
    w epis_z, epis_z = 30 a over the last metre for esp_type 2 and 60 a^2
    times the relative depth (water) or height (air) for esp_type 1, with a
    the distance into the layer in metres."""
    case = cases.sponge_tank(32, 4, 16, esp_type=esp_type)
    p = case.params
    o = pyoracle.Oracle(p)
    flat = np.empty((p.nx, p.ny, p.nz), order="F")
    z = (np.arange(1, p.nz + 1) - 0.5) * p.dz
    flat[...] = 0.5 - z[None, None, :]
    o.set_field("LS", flat)
    o.heaviside_init()
    rng = np.random.default_rng(1)
    w = np.asfortranarray(rng.standard_normal(o.field("W").shape))
    o.set_field("W", w)
    fw0 = np.asfortranarray(rng.standard_normal(o.field("FW").shape))
    p0 = p.copy()
    p0.esp_type = 0
    o0 = pyoracle.Oracle(p0)
    o0.set_field("LS", flat)
    o0.heaviside_init()
    o0.set_field("W", w)
    o0.set_field("FW", fw0)
    o0.complementos()
    o.set_field("FW", fw0)
    o.complementos()
    d = o0.field("FW") - o.field("FW")                 # = w epis_z (w faces 1..nz1)
    xc = (np.arange(1, p.nx + 1) - 0.5) * p.dx
    a = np.maximum(xc - (p.nx * p.dx - 1.0), 0.0)[:, None, None]
    zx = ((np.arange(1, p.nz + 1) - 1) * p.dz)[None, None, :]
    if esp_type == 2:
        ep = 30.0 * a * np.ones((1, p.ny, p.nz))
    else:
        zpfs, zpt = 0.5, p.dz * p.nz
        water = flat >= 0
        ep = np.where(water, 60.0 * a * a * zx / zpfs, 60.0 * a * a * (zx - zpt) / (zpfs - zpt))
    ep[xc <= p.nx * p.dx - 1.0] = 0.0
    want = w[1:p.nx + 1, 1:p.ny + 1, 1:p.nz + 1] * ep
    assert np.allclose(d[:, :, :p.nz], want, rtol=1e-9, atol=1e-12)
    assert np.all(d[:, :, p.nz] == 0.0)
    assert np.abs(want).max() > 1.0
