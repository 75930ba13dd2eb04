"""Inflow waves (wave_t = 1 Stokes I, 2 Stokes II, 5 Stokes V;
boundary_waves 3_contorno.f90:1189-1319 with waves_coef :1323-1445) in the
oracle and in the host set-up, on CPU.  The reference's tests hold no golden
values for them, so they are pinned on the wave theory they restate: the
linear dispersion relation, the Stokes V first harmonic against the
amplitude, and the inflow planes against the closed-form Stokes I fields."""
import math

import numpy as np
import pytest

import pyoracle
from suli_gb300 import cases


def test_linear_dispersion_relation():
    g = 9.80665
    w = cases.waves_coef(g, 1)
    k, om, h = w["n_w"], w["f_w"], w["h0_f"]
    assert abs(om * om - g * k * math.tanh(k * h)) <= 1e-12 * om * om


def test_stokes5_first_harmonic():
    """The surface's first harmonic is the amplitude to within the weak
    nonlinearity (k a ~ 0.03), and the wave is a little longer than the
    linear one (amplitude dispersion)."""
    w5 = cases.waves_coef(9.80665, 5)
    w1 = cases.waves_coef(9.80665, 1)
    assert abs(w5["aeta"][0] - w5["a_w"]) < 0.01 * w5["a_w"]
    assert w5["n_w"] < w1["n_w"] and (w1["n_w"] - w5["n_w"]) / w1["n_w"] < 0.01
    assert all(abs(w5["aeta"][m + 1]) < abs(w5["aeta"][m]) for m in range(4))


@pytest.mark.parametrize("t", [0.0, 0.37, 1.9])
def test_stokes1_inflow_planes(t):
    case = cases.wave_flume(24, 4, 16, wave_t=1)
    p = case.params
    o = pyoracle.Oracle(p)
    for k_, v in case.fields.items():
        o.set_field(k_, v)
    o.set_scalar("T", t)
    o.boundary_waves()
    kp = (np.arange(0, p.nz + 2) - 0.5) * p.dz
    a, om, k, h = p.a_w, p.f_w, p.n_w, p.h0_f

    def field(i):
        eta = h + a * math.cos(k * p.dx * (i - 0.5) - om * t)
        wet = eta - kp >= 0
        u = np.where(wet, a * om * np.cosh(k * kp) / math.sinh(k * h) * math.cos(k * p.dx * (i - 1.0) - om * t), 0.0)
        w = np.where(wet, a * om * np.sinh(k * (kp - 0.5 * p.dz)) / math.sinh(k * h) * math.sin(k * p.dx * (i - 0.5) - om * t), 0.0)
        return eta, u, w

    eta0, u0, w0 = field(0)
    eta1, u1, _ = field(1)
    bxx0 = o.field("BXX0")[:, :, 0]
    assert np.allclose(bxx0, np.broadcast_to(u0, bxx0.shape), rtol=1e-13, atol=1e-15)
    assert np.allclose(o.field("BXZ0")[:, :, 0], np.broadcast_to(w0, bxx0.shape), rtol=1e-13, atol=1e-15)
    assert np.allclose(o.field("BXX1")[:, :, 0], np.broadcast_to(u1, bxx0.shape), rtol=1e-13, atol=1e-15)
    ls1 = o.field("LS")[0]
    assert np.allclose(ls1, np.broadcast_to(eta1 - kp[1:-1], ls1.shape), rtol=0, atol=1e-14)
    assert np.abs(bxx0).max() > 0.1 * a * om * math.cosh(k * h) / math.sinh(k * h)


def test_wave_inflow_fill():
    """contorno(2) with ccx0 = 3 after boundary_waves: the inflow face takes
    the wave (iturb = 0: no perturbation) where the water is, w(0, :, :) the
    plane bxz0 and v(0, :, :) zero (3_contorno.f90:301-330).  Whole steps of
    the flume are not run here: the wave's net inflow through the
    all-Neumann pressure equation has no solution, and the CG diverges on it
    in the oracle and the library alike."""
    case = cases.wave_flume(24, 4, 16, wave_t=2)
    p = case.params
    o = pyoracle.Oracle(p)
    for k_, v in case.fields.items():
        o.set_field(k_, v)
    o.heaviside_init()
    o.set_scalar("T", 0.4)
    o.boundary_waves()
    o.contorno(2)
    w0 = o.field("W")[0]
    bz = o.field("BXZ0")[:, :, 0]
    assert np.array_equal(w0[:, :p.nz + 2], bz) and np.all(w0[:, p.nz + 2] == 0.0)
    assert np.all(o.field("V")[0] == 0.0)
    u = o.field("U")
    bx = o.field("BXX1")[:, :, 0]
    wet = o.field("LS")[0, :, :] >= 0            # ls(1, :, :) = blx1: the still level
    assert np.abs(u[1, 1:p.ny + 1, 1:p.nz + 1][wet] - bx[1:p.ny + 1, 1:p.nz + 1][wet]).max() == 0.0
    assert np.abs(bz).max() > 0
