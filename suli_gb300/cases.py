"""Synthetic workloads of the SuLi hot path and their initial conditions.

Host-side set-up only (the reference runs it once on the host too:
iniciais() 2_iniciais.f90:127-274 and level_set_ini() 14_level_set.f90:10-200).
Each builder returns a Case: the suli_params of the run plus the initial
fields in the reference layout (Fortran order, reference lower bounds), ready
for upload.  No public dataset is involved: every input is generated here
from the workload's stated shapes and seeded distributions.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from ._abi import CG_TOL_ABS, CG_TOL_REL, PREC_FP64, SuliParams, default_params, field_shape


@dataclasses.dataclass
class Case:
    name: str
    params: SuliParams
    fields: dict            # name -> np.ndarray (Fortran order)
    steps: int              # steps the workload is quoted on
    obstacle: dict | None = None   # cylinder description for IBM set-up

    @property
    def cells(self) -> int:
        return self.params.nx * self.params.ny * self.params.nz


def _centres(n, h):
    return (np.arange(1, n + 1) - 0.5) * h


def _zeros(p, name):
    return np.zeros(field_shape(p, name), order="F")


def level_set_tipo(p: SuliParams, tipo: int, ampl=0.0, lambdax=0.0, lambday=0.0, prof=0.0, m=30.0):
    """level_set_ini() 14_level_set.f90:56-129 for tipo 1 (wave), 3 (dam), 4 (drop)."""
    x = _centres(p.nx, p.dx)[:, None, None]
    y = _centres(p.ny, p.dy)[None, :, None]
    z = _centres(p.nz, p.dz)[None, None, :]
    if tipo == 1:
        if lambday != 0.0:
            d = np.cos(2.0 * math.pi / lambday * y) + 0.0 * x
        elif lambdax == 0.0:
            d = np.zeros((1, 1, 1))
        else:
            d = np.ones((1, 1, 1))
        if lambdax != 0.0:
            d = -ampl * d * np.cos(2.0 * math.pi / lambdax * x)
        ls = d - z + prof
    elif tipo == 3:
        lsaux = np.power(z - prof, m) + np.power(x - lambdax, m) + np.power(y - lambday, m) / np.power(10.0, m)
        ls = -np.power(lsaux, 1.0 / m) + ampl
    elif tipo == 4:
        lsaux = np.power(x - lambdax, m) / 2.0 + np.power(y - lambday, m) / 2.0 + np.power(z - prof, m) / 2.0
        ls = -np.power(lsaux, 1.0 / m) + ampl
    else:
        raise ValueError(f"tipo {tipo} not supported")
    out = np.empty((p.nx, p.ny, p.nz), order="F")
    out[...] = ls
    return out


def _base_fields(p: SuliParams, ls: np.ndarray) -> dict:
    """iniciais() 2_iniciais.f90:294-399: v = w = prd = 0, u = uinicial."""
    f = {"LS": np.asfortranarray(ls)}
    u = _zeros(p, "U")
    u[...] = p.uinicial
    f["U"] = u
    f["V"] = _zeros(p, "V")
    f["W"] = _zeros(p, "W")
    f["PRD1"] = _zeros(p, "PRD1")
    bx = _zeros(p, "BXX0")
    bx[...] = p.uinicial
    f["BXX0"] = bx
    f["BXX1"] = bx.copy()
    f["BLX1"] = np.asfortranarray(ls[0, :, :].reshape(p.ny, p.nz, 1))
    return f


def dam_break(nx=64, ny=32, nz=32, precision=PREC_FP64, reinit_iters=5, cg_tol=1e-10) -> Case:
    """Plain FP64 3-D dam break: 1.0 x 0.5 x 0.5 m box, water column x<0.25,
    z<0.25 (tipo 3, ampl 0.25, m 30), rho 1000/1.2, mu 1e-3/1.8e-5, g 9.81,
    no-slip walls, dt 1e-4, no LES, no IBM; 200 steps."""
    lx = 1.0
    h = lx / nx
    p = default_params(nx=nx, ny=ny, nz=nz, dx=h, dy=h, dz=h, dt=1e-4,
                       ccx0=2, ccxf=2, ccy0=2, ccyf=2, ccz0=2, cczf=2,
                       gx=0.0, gz=9.81, rho_f1=1.2, mu_f1=1.8e-5, rho_f2=1000.0, mu_f2=1e-3,
                       m_turb=0, reinit_max_iter=reinit_iters, cg_tol_mode=CG_TOL_REL,
                       cg_tol=cg_tol, precision=precision)
    ls = level_set_tipo(p, 3, ampl=0.25, lambdax=0.0, lambday=0.0, prof=0.0, m=30.0)
    return Case("dam_break_%dx%dx%d" % (nx, ny, nz), p, _base_fields(p, ls), steps=200)


def z_centres_dz(nz, dzmin, dzmax):
    """Cell-centre heights of the variable z spacing of SuLi-ICdz (dz_dist,
    SuLi-ICdz/2_iniciais.f90:326-406, dz_t = 1): dz(k) = dzmin + (dzmax -
    dzmin) k / nz, z(1) = dz(1) / 2, z(k) = z(k-1) + (dz(k-1) + dz(k)) / 2."""
    dz = [dzmin + (dzmax - dzmin) * k / nz for k in range(nz + 2)]
    z = np.empty(nz)
    z[0] = dz[1] * 0.5
    for k in range(2, nz + 1):
        z[k - 1] = z[k - 2] + (dz[k - 1] + dz[k]) * 0.5
    return z


def dam_break_dz(nx=64, ny=32, nz=32, dzmin=None, dzmax=None, precision=PREC_FP64, reinit_iters=5,
                 cg_tol=1e-10) -> Case:
    """The dam break on SuLi-ICdz's stretched z grid (dz_t = 1): x, y as the
    uniform dam break (1.0 x 0.5 m), dz growing linearly from dzmin at the
    bed to dzmax at the top (defaults 0.6 and 1.4 times the uniform 0.5/nz:
    the same height), water column x < 0.25, z < 0.25 (tipo 3 with the
    variable grid's cell heights)."""
    h = 1.0 / nx
    dzmin = 0.6 * 0.5 / nz if dzmin is None else dzmin
    dzmax = 1.4 * 0.5 / nz if dzmax is None else dzmax
    p = default_params(nx=nx, ny=ny, nz=nz, dx=h, dy=h, dz=dzmin, dt=1e-4,
                       ccx0=2, ccxf=2, ccy0=2, ccyf=2, ccz0=2, cczf=2,
                       gx=0.0, gz=9.81, rho_f1=1.2, mu_f1=1.8e-5, rho_f2=1000.0, mu_f2=1e-3,
                       m_turb=0, reinit_max_iter=reinit_iters, cg_tol_mode=CG_TOL_REL,
                       cg_tol=cg_tol, precision=precision, dz_t=1, dzmin=dzmin, dzmax=dzmax)
    x = _centres(nx, h)[:, None, None]
    y = _centres(ny, h)[None, :, None]
    z = z_centres_dz(nz, dzmin, dzmax)[None, None, :]
    m = 30.0
    lsaux = np.power(z, m) + np.power(x, m) + np.power(y, m) / np.power(10.0, m)
    ls = np.empty((nx, ny, nz), order="F")
    ls[...] = -np.power(lsaux, 1.0 / m) + 0.25
    return Case("dam_break_dz_%dx%dx%d" % (nx, ny, nz), p, _base_fields(p, ls), steps=200)


def wave_tank(nx=1024, ny=256, nz=256, precision=PREC_FP64, dt=2e-4, cg_tol=1e-8) -> Case:
    """Large wave tank: 8 x 2 x 2 m, depth 1.0 m, eta = 0.05 sin(2 pi x / 2),
    still water, Smagorinsky LES (Cs 0.1), closed free-slip tank; 1000 steps."""
    h = 8.0 / nx
    p = default_params(nx=nx, ny=ny, nz=nz, dx=h, dy=h, dz=h, dt=dt,
                       ccx0=1, ccxf=1, ccy0=1, ccyf=1, ccz0=1, cczf=1,
                       gz=9.80665, m_turb=1, csmag=0.1, reinit_max_iter=3,
                       cg_tol_mode=CG_TOL_REL, cg_tol=cg_tol, precision=precision)
    x = _centres(nx, h)[:, None, None]
    z = _centres(nz, h)[None, None, :]
    eta = 0.05 * np.sin(2.0 * math.pi * x / 2.0)
    ls = np.empty((nx, ny, nz), order="F")
    ls[...] = eta - z + 1.0
    return Case("wave_tank_%dx%dx%d" % (nx, ny, nz), p, _base_fields(p, ls), steps=1000)


def mms_case(n=32, precision=PREC_FP64, dt=None, project=True) -> Case:
    """Steady manufactured solution (13_mms.f90:39-114, a = 0, h0 = 2) on a
    2 pi x 2 pi x 2 box, periodic in x and y (the sin x cos y fields are
    2 pi-periodic), no-slip bed, free-slip top, gravity off; 100 steps."""
    L = 2.0 * math.pi
    dxy = L / n
    dz = 2.0 / n
    if dt is None:
        dt = 0.002 * 32.0 / n
    p = default_params(nx=n, ny=n, nz=n, dx=dxy, dy=dxy, dz=dz, dt=dt,
                       ccx0=0, ccxf=0, ccy0=0, ccyf=0, ccz0=2, cczf=1,
                       gx=0.0, gz=0.0, mms_t=1, project_under_mms=1 if project else 0,
                       rho_f2=998.0, mu_f2=0.00100798, cg_tol_mode=CG_TOL_ABS, cg_tol=1e-4,
                       precision=precision)
    a, h0 = 0.0, 2.0
    f = {}
    x = _centres(n, dxy)[:, None, None]
    y = _centres(n, dxy)[None, :, None]
    z = _centres(n, dz)[None, None, :]
    ls = np.empty((n, n, n), order="F")
    ls[...] = a * np.sin(x) * np.sin(y) + h0 - z
    f = _base_fields(p, ls)
    u = f["U"]
    xf = (np.arange(1, n + 2) - 1.0) * dxy
    yc = _centres(n, dxy)
    zc = _centres(n, dz)
    X, Y, Z = np.meshgrid(xf, yc, zc, indexing="ij")
    hh = a * np.sin(X) * np.sin(Y) + h0
    u[1:n + 2, 1:n + 1, 1:n + 1] = np.sin(X) * np.cos(Y) * np.sin(math.pi * 0.5 * Z / hh) - \
        np.cos(X) * np.sin(Y) * (np.cos(math.pi * 2.0 * Z / hh) - 1.0)
    v = f["V"]
    X, Y, Z = np.meshgrid(_centres(n, dxy), (np.arange(1, n + 2) - 1.0) * dxy, zc, indexing="ij")
    hh = a * np.sin(X) * np.sin(Y) + h0
    v[1:n + 1, 1:n + 2, 1:n + 1] = -np.cos(X) * np.sin(Y) * np.sin(math.pi * 0.5 * Z / hh) + \
        np.sin(X) * np.cos(Y) * (np.cos(math.pi * 2.0 * Z / hh) - 1.0)
    return Case("mms_%d" % n, p, f, steps=100)


def cylinder_obstacle(p: SuliParams, xc: float, yc: float, radius: float) -> dict:
    """Vertical cylinder as an obstacle level set (positive inside):
    phi_s = R - sqrt((x-xc)^2 + (y-yc)^2) on the half-cell sub-grid of
    obstaculo() (x = (i-1) dx/2, 3_contorno.f90:829-841) sampled at the
    staggered locations as 3_contorno.f90:951-989 does."""
    nx, ny, nz = p.nx, p.ny, p.nz

    def phi(ii, jj):
        x = (ii - 1.0) * p.dx * 0.5
        y = (jj - 1.0) * p.dy * 0.5
        return radius - np.sqrt(np.power(x - xc, 2.0) + np.power(y - yc, 2.0))

    def field(ni, nj, nk, fi, fj):
        i = np.arange(1, ni + 1)[:, None, None]
        j = np.arange(1, nj + 1)[None, :, None]
        out = np.empty((ni, nj, nk), order="F")
        out[...] = phi(fi(i), fj(j))
        return out

    # obs_ls at the cell corners for the field output: the sub-grid's odd
    # points 2i-1 (3_contorno.f90:905-911)

    return {
        "OBS_LSX": field(nx + 1, ny, nz, lambda i: 2 * i - 1, lambda j: 2 * j),
        "OBS_LSY": field(nx, ny + 1, nz, lambda i: 2 * i, lambda j: 2 * j - 1),
        "OBS_LSZ": field(nx, ny, nz + 1, lambda i: 2 * i, lambda j: 2 * j),
        "OBS_LSS": field(nx, ny, nz, lambda i: 2 * i, lambda j: 2 * j),
        "OBS_LS": field(nx + 1, ny + 1, nz + 1, lambda i: 2 * i - 1, lambda j: 2 * j - 1),
    }


def inflow_profile(p: SuliParams, ls: np.ndarray, seed: int) -> np.ndarray:
    """Initial u of iniciais() for ccx0 = 0 or 3 (2_iniciais.f90:189-210):
    u = uinicial (1 + r iturb), r uniform in [-1, 1), on x faces where the
    face level set is >= -2 dz, and above that the tanh decay
    u(i,j,iik) (1 + tanh(pi (iik - k - 1) / 2)) from the last such level iik
    (loop order k, j, i as upstream).  random_number is replaced by a seeded
    numpy generator."""
    nx, ny, nz = p.nx, p.ny, p.nz
    # interpx_cf: face average, end faces from the two nearest cells (periodic: wrap)
    lsx = np.empty((nx + 1, ny, nz))
    lsx[1:nx] = 0.5 * (ls[1:] + ls[:-1])
    if p.ccx0 == 0:
        lsx[0] = lsx[nx] = 0.5 * (ls[0] + ls[nx - 1])
    else:
        lsx[0] = 0.5 * (ls[1] + ls[0])
        lsx[nx] = 0.5 * (ls[nx - 1] + ls[nx - 2])
    rng = np.random.default_rng(seed)
    u = _zeros(p, "U")
    iik = 0
    for k in range(1, nz + 1):
        r = 2.0 * (rng.random((nx + 1, ny)) - 0.5)
        for j in range(1, ny + 1):
            water = lsx[:, j - 1, k - 1] >= -2 * p.dz
            # air faces before the row's first water face still see the old
            # iik; from it on iik = k and u(i,j,k) itself (still 0) is scaled
            seen = np.cumsum(water) > 0
            air_old = u[1:nx + 2, j, iik] * (1.0 + math.tanh(math.pi * (iik - k - 1) / 2.0))
            col = np.where(water, p.uinicial * (1.0 + r[:, j - 1] * p.iturb), np.where(seen, 0.0, air_old))
            if water.any():
                iik = k
            u[1:nx + 2, j, k] = col
    return u


def open_channel(nx=512, ny=128, nz=128, precision=PREC_FP64, dt=1e-3, seed=1234, radius=0.05,
                 cg_tol=1e-8, periodic=False, balanced=False) -> Case:
    """Open channel, 4 x 1 x 1 m, depth 0.6 m flat surface, inflow u = 0.5 m/s
    with a seeded uniform 5 % perturbation (ccx0 = 3), free outflow, no-slip
    bed, Smagorinsky LES Cs = 0.1, vertical cylinder D = 0.1 m at x = 1.0
    through image-point IBM; 2000 steps.  The start is the reference's
    inflow profile (water at uinicial, air decaying to rest).

    periodic=True closes the channel in x (ccx0 = ccxf = 0): the pressure
    equation then has a solution (zero net boundary flux), where prescribed
    inflow with free outflow leaves the all-Neumann system of graddin with
    a net flux that its CG cannot remove.  balanced=True keeps the inflow
    and the free outflow but has contorno(2) correct the outflow faces to the
    inflow's flux (outflow_flux = 1), which makes the pressure equation
    solvable too."""
    h = 4.0 / nx
    cx = (0, 0) if periodic else (3, 4)
    p = default_params(nx=nx, ny=ny, nz=nz, dx=h, dy=h, dz=h, dt=dt,
                       ccx0=cx[0], ccxf=cx[1], ccy0=1, ccyf=1, ccz0=2, cczf=1,
                       gz=9.80665, m_turb=1, csmag=0.1, uinicial=0.5, iturb=0.05,
                       ibm_t=2, obst_t=4, reinit_max_iter=3, cg_tol_mode=CG_TOL_REL, cg_tol=cg_tol,
                       precision=precision, seed=seed, outflow_flux=1 if (balanced and not periodic) else 0)
    ls = level_set_tipo(p, 1, ampl=0.0, lambdax=0.0, lambday=0.0, prof=0.6)
    f = _base_fields(p, ls)
    f["U"] = inflow_profile(p, ls, seed)
    f.update(cylinder_obstacle(p, 1.0, 0.5, radius))
    name = "periodic_channel" if periodic else ("balanced_channel" if balanced else "open_channel")
    return Case("%s_%dx%dx%d" % (name, nx, ny, nz), p, f, steps=2000,
                obstacle={"kind": "cylinder", "xc": 1.0, "yc": 0.5, "radius": radius})


def ensemble_dims(ncases=256, seed=0, lo=32, hi=96):
    """Grid dims drawn per axis uniformly from {lo..hi} (seeded)."""
    rng = np.random.default_rng(seed)
    dims = rng.integers(lo, hi + 1, size=(ncases, 3))
    hcol = rng.uniform(0.2, 0.6, size=ncases)
    amp = rng.uniform(0.0, 0.05, size=ncases)
    return dims, hcol, amp


def ensemble_case(i, dims, hcol, amp, precision=PREC_FP64, dt=1e-4, cg_tol=1e-10) -> Case:
    """One member of the sloshing / dam-break ensemble: dx = 1/64; a water
    column of height hcol*lz (tipo 3 form) united with a sloshing layer of
    depth 0.25 lz and cosine amplitude amp*lz (tipo 1 form); the union of the
    two water regions is the max of the two level sets (a build-side
    composition of two reference tipos)."""
    nx, ny, nz = (int(d) for d in dims[i])
    h = 1.0 / 64.0
    p = default_params(nx=nx, ny=ny, nz=nz, dx=h, dy=h, dz=h, dt=dt,
                       ccx0=2, ccxf=2, ccy0=2, ccyf=2, ccz0=2, cczf=2,
                       gz=9.81, rho_f1=1.2, mu_f1=1.8e-5, rho_f2=1000.0, mu_f2=1e-3,
                       reinit_max_iter=3, cg_tol_mode=CG_TOL_REL, cg_tol=cg_tol, precision=precision)
    lx, lz = nx * h, nz * h
    col = level_set_tipo(p, 3, ampl=float(hcol[i]) * lz, m=30.0)
    layer = level_set_tipo(p, 1, ampl=float(amp[i]) * lz, lambdax=2.0 * lx, prof=0.25 * lz)
    ls = np.maximum(col, layer)
    return Case("ensemble_%d" % i, p, _base_fields(p, ls), steps=500)


def capillary_column(n=48, ny=4, radius=0.25, precision=PREC_FP64, dt=2e-4) -> Case:
    """A water column of circular section (axis along y) at rest in air, with
    surface tension (t_tens = 1, 14_level_set.f90:519-567, :660-704): ls =
    R - |(x, z) - centre| on a 1 x 1 x-z box, walls all round (y periodic),
    gravity off.  Its curvature is -1/R; the Laplace pressure jump sigma/R
    drives the flow."""
    h = 1.0 / n
    p = default_params(nx=n, ny=ny, nz=n, dx=h, dy=h, dz=h, dt=dt, ccy0=0, ccyf=0,
                       gx=0.0, gz=0.0, precision=precision, cg_tol_mode=CG_TOL_REL, cg_tol=1e-10)
    p.t_tens = 1
    x = _centres(n, h)[:, None, None]
    z = _centres(n, h)[None, None, :]
    ls = np.empty((n, ny, n), order="F")
    ls[...] = radius - np.sqrt((x - 0.5) ** 2 + (z - 0.5) ** 2)
    return Case("capillary_%d" % n, p, _base_fields(p, ls), steps=20)


def k_channel(nx=32, ny=8, nz=16, m_turb=2, precision=PREC_FP64, dt=2e-4, seed=7) -> Case:
    """Open-channel flow with the k-equation model (m_turb = 2, LES with the
    turbulent kinetic energy equation, or 3, DES; 5_viscosidade.f90:91-145):
    a 2 x 0.5 x 1 m box periodic in x, water below z = 0.6 m, no-slip bed,
    free-slip side walls and lid, driven by a bed slope of 0.01 (gx).  The initial state
    is iniciais() for m_turb >= 2 (2_iniciais.f90:216-235): u = uinicial = 0.5
    m/s, ka = 1.5 iturb^2 (uinicial^2 + 1e-6) in every cell and each velocity
    component perturbed by sqrt(ka) times a uniform draw (seeded here, as
    random_number is upstream); the ghost values of ka come from
    contorno_les, which the caller applies once (suli_contorno_les)."""
    lx = 2.0
    h = lx / nx
    slope = 0.01
    g = 9.80665
    p = default_params(nx=nx, ny=ny, nz=nz, dx=h, dy=h, dz=h, dt=dt,
                       ccx0=0, ccxf=0, ccy0=1, ccyf=1, ccz0=2, cczf=1,
                       gx=g * math.sin(math.atan(slope)), gz=g * math.cos(math.atan(slope)),
                       m_turb=m_turb, uinicial=0.5, iturb=0.05, reinit_max_iter=3,
                       cg_tol_mode=CG_TOL_REL, cg_tol=1e-10, precision=precision)
    p.lcar = 0.6
    z = _centres(nz, h)[None, None, :]
    ls = np.empty((nx, ny, nz), order="F")
    ls[...] = 0.6 - z
    f = _base_fields(p, ls)
    aux1 = p.iturb * p.iturb * (p.uinicial * p.uinicial + 1e-6) * 1.5
    rng = np.random.default_rng(seed)
    ka = _zeros(p, "KA")
    ka[1:nx + 1, 1:ny + 1, 1:nz + 1] = aux1
    f["KA"] = ka
    for name in ("U", "V", "W"):
        a = f[name]
        a[1:nx + 1, 1:ny + 1, 1:nz + 1] += math.sqrt(aux1) * rng.random((nx, ny, nz))
    return Case("k_channel_m%d_%dx%dx%d" % (m_turb, nx, ny, nz), p, f, steps=200)


def ipa_tank(nx=24, ny=8, nz=16, precision=PREC_FP64, dt=1e-4) -> Case:
    """Still water in a closed tank under the implicit pressure algorithm
    (t_press = 2: exp_press before visco, graddin with the density rho_f1
    after the RK loop and no posdin; 1_principal.f90:82,111, 11_diversos.f90:
    455-495, 9_grad.f90:103-115): a 1.5 x 0.5 x 1 m box with a slightly
    tilted free surface (eta = 0.02 (x - 0.75)) at 0.5 m depth, free-slip
    walls.  The pressure accumulates in prd0 towards the hydrostatic one."""
    h = 1.5 / nx
    p = default_params(nx=nx, ny=ny, nz=nz, dx=h, dy=h, dz=h, dt=dt,
                       ccx0=1, ccxf=1, ccy0=1, ccyf=1, ccz0=1, cczf=1,
                       gz=9.80665, t_press=2, reinit_max_iter=3,
                       cg_tol_mode=CG_TOL_REL, cg_tol=1e-10, precision=precision)
    x = _centres(nx, h)[:, None, None]
    z = _centres(nz, h)[None, None, :]
    ls = np.empty((nx, ny, nz), order="F")
    ls[...] = 0.5 + 0.02 * (x - 0.75) - z
    f = _base_fields(p, ls)
    f["PRD0"] = _zeros(p, "PRD0")
    return Case("ipa_tank_%dx%dx%d" % (nx, ny, nz), p, f, steps=200)


def sponge_tank(nx=32, ny=4, nz=16, esp_type=1, precision=PREC_FP64, dt=2e-4, cg_tol=1e-10) -> Case:
    """Sloshing in a 2 x 0.25 x 1 m tank with a sponge layer over its last
    metre (esp_type 1: graded with the depth below the interface, 2: linear;
    3_contorno.f90:1011-1103): water 0.5 m deep under a cosine surface of
    amplitude 0.05 m, free-slip walls."""
    lx = 2.0
    h = lx / nx
    p = default_params(nx=nx, ny=ny, nz=nz, dx=h, dy=h, dz=1.0 / nz, dt=dt,
                       ccx0=1, ccxf=1, ccy0=1, ccyf=1, ccz0=1, cczf=1,
                       gz=9.80665, reinit_max_iter=3, cg_tol_mode=CG_TOL_REL, cg_tol=cg_tol,
                       precision=precision)
    p.esp_type = esp_type
    x = _centres(nx, h)[:, None, None]
    z = _centres(nz, p.dz)[None, None, :]
    ls = np.empty((nx, ny, nz), order="F")
    ls[...] = 0.5 + 0.05 * np.cos(math.pi * x / lx) - z
    return Case("sponge_tank_%dx%dx%d" % (nx, ny, nz), p, _base_fields(p, ls), steps=200)


def waves_coef(gz: float, wave_t: int) -> dict:
    """waves_coef (3_contorno.f90:1323-1445), the host set-up of the inflow
    waves that iniciais runs once (2_iniciais.f90:241-245): amplitude 0.03 m,
    period 2.5 s, still depth 1 m as upstream; the wave length from the
    linear dispersion relation by 1000 fixed-point steps (Stokes I, II), or
    for Stokes V the length and the expansion parameter lambda where the two
    fixed-point estimates of lambda agree best over 10000 trial lengths
    (10000 steps each, vectorised over the trials).  Returns the suli_params
    fields a_w, f_w, n_w, h0_f, aeta, avel."""
    pi = math.pi
    a_w, p_w, h0_f = 0.03, 2.5, 1.0
    l0_w = gz * p_w * p_w / (2.0 * pi)
    out = {"a_w": a_w, "h0_f": h0_f, "aeta": [0.0] * 5, "avel": [0.0] * 5}
    if wave_t <= 2:
        l_w = gz * p_w * p_w / (2.0 * pi)
        for _ in range(1000):
            l_w = gz * p_w * p_w / (2.0 * pi) * math.tanh(2.0 * pi * h0_f / l_w)
        out.update(f_w=2.0 * pi / p_w, n_w=2.0 * pi / l_w)
        return out

    def coefs(s, c):
        b33 = 3.0 * (8.0 * c ** 6.0 + 1.0) / (64.0 * s ** 6.0)
        b35 = (88128.0 * c ** 14.0 - 208224.0 * c ** 12 + 70848.0 * c ** 10.0 + 54000.0 * c ** 8.0
               - 21816.0 * c ** 6.0 + 6264.0 * c ** 4.0 - 54.0 * c * c - 81.0) / (12288.0 * s ** 12.0 * (6.0 * c * c - 1.0))
        b55 = (192000.0 * c ** 16.0 - 262720.0 * c ** 14.0 + 83680.0 * c ** 12 + 20160.0 * c ** 10.0
               - 7280.0 * c ** 8.0 + 7160.0 * c ** 6.0 - 1800.0 * c ** 4.0 - 1050.0 * c * c + 225.0) / \
            (12288 * s ** 10.0 * (6.0 * c * c - 1.0) * (8.0 * c ** 4.0 - 11.0 * c * c + 3.0))
        c1 = (8.0 * c ** 4.0 - 8.0 * c * c + 9.0) / (8.0 * s ** 4.0)
        c2 = (3840.0 * c ** 12.0 - 4096.0 * c ** 10.0 + 2592.0 * c ** 8.0 - 1008.0 * c ** 6.0 + 5944.0 * c ** 4.0
              - 1830.0 * c * c + 147.0) / (512.0 * s ** 10.0 * (6.0 * c * c - 1.0))
        return b33, b35, b55, c1, c2

    ii = np.arange(1, 10001, dtype=np.float64)
    l_w1 = l0_w * 0.5 + l0_w * (ii / 10000) * 2.5
    s = np.sinh(2.0 * pi * h0_f / l_w1)
    c = np.cosh(2.0 * pi * h0_f / l_w1)
    b33, b35, b55, c1, c2 = coefs(s, c)
    with np.errstate(all="ignore"):
        lamb1 = np.zeros_like(l_w1)
        for _ in range(10000):
            lamb1 = pi * a_w * 2.0 / l_w1 - lamb1 ** 3.0 * b33 - lamb1 ** 5.0 * (b35 + b55)
        lamb2 = np.zeros_like(l_w1)
        for _ in range(10000):
            lamb2 = np.sqrt((l_w1 / (l0_w * np.tanh(2.0 * pi * h0_f / l_w1)) - 1.0) / (c1 + lamb2 ** 2.0 * c2))
        erro = np.abs(lamb1 - lamb2)
    best = int(np.nanargmin(erro))      # the first of the smallest, as the strict < of the search
    lamb, l_w = float(lamb1[best]), float(l_w1[best])
    f_w, n_w = 2.0 * pi / p_w, 2.0 * pi / l_w
    s = math.sinh(2.0 * pi * h0_f / l_w)
    c = math.cosh(2.0 * pi * h0_f / l_w)
    b33, b35, b55, c1, c2 = coefs(s, c)
    a11 = 1.0 / s
    a13 = -c * c * (5.0 * c * c + 1.0) / (8.0 * s ** 5.0)
    a15 = -(1184.0 * c ** 10.0 - 1440.0 * c ** 8.0 - 1992.0 * c ** 6.0 + 2641.0 * c ** 4.0 - 249.0 * c ** 2.0 + 18.0) \
        / (1536.0 * s ** 11.0)
    a22 = 3.0 / (8.0 * s ** 4.0)
    a24 = (192.0 * c ** 8.0 - 424.0 * c ** 6.0 - 312.0 * c ** 4.0 + 480.0 * c * c - 17.0) / (768.0 * s ** 10.0)
    a33 = (13.0 - 4.0 * c * c) / (64.0 * s ** 7.0)
    a35 = (512.0 * c ** 12.0 + 4224.0 * c ** 10.0 - 6800.0 * c ** 8.0 - 12808.0 * c ** 6.0 + 16704.0 * c ** 4.0
           - 3154.0 * c * c + 107.0) / (4096.0 * s ** 13.0 * (6.0 * c * c - 1.0))
    a44 = (80.0 * c ** 6.0 - 816.0 * c ** 4.0 + 1338.0 * c * c - 197.0) / (1536.0 * s ** 10.0 * (6.0 * c * c - 1.0))
    a55 = -(2880.0 * c ** 10.0 - 72480.0 * c ** 8.0 + 324000.0 * c ** 6.0 - 432000.0 * c ** 4.0 + 163470.0 * c * c
            - 16245.0) / (61440.0 * s ** 11.0 * (6.0 * c * c - 1.0) * (8.0 * c ** 4.0 - 11.0 * c * c + 3.0))
    b22 = c * (2.0 * c * c + 1.0) / (4.0 * s ** 3.0)
    b24 = c * (272.0 * c ** 8.0 - 504.0 * c ** 6.0 - 192.0 * c ** 4.0 + 322 * c * c + 21.0) / (384.0 * s ** 9.0)
    b44 = c * (768.0 * c ** 10.0 - 448.0 * c ** 8.0 - 48.0 * c ** 6.0 + 48.0 * c ** 4.0 + 106.0 * c * c - 21.0) / \
        (384.0 * s ** 9.0 * (6.0 * c * c - 1.0))
    aeta = [lamb / n_w,
            (lamb * lamb * b22 + lamb ** 4.0 * b24) / n_w,
            (lamb ** 3.0 * b33 + lamb ** 5.0 * b35) / n_w,
            lamb ** 4.0 * b44 / n_w,
            lamb ** 5.0 * b55 / n_w]
    k0 = 2.0 * pi / (p_w * n_w)
    avel = [1.0 * k0 * (lamb * a11 + lamb ** 3.0 * a13 + lamb ** 5.0 * a15),
            2.0 * k0 * (lamb ** 2.0 * a22 + lamb ** 4.0 * a24),
            3.0 * k0 * (lamb ** 3.0 * a33 + lamb ** 5.0 * a35),
            4.0 * k0 * (lamb ** 4.0 * a44),
            5.0 * k0 * (lamb ** 5.0 * a55)]
    out.update(f_w=f_w, n_w=n_w, aeta=aeta, avel=avel, lamb=lamb)
    return out


def set_waves(p: SuliParams, wave_t: int) -> dict:
    """waves_coef's results into the suli_params of a case."""
    w = waves_coef(p.gz, wave_t)
    p.wave_t = wave_t
    p.a_w, p.f_w, p.n_w, p.h0_f = w["a_w"], w["f_w"], w["n_w"], w["h0_f"]
    for m in range(5):
        p.aeta[m] = w["aeta"][m]
        p.avel[m] = w["avel"][m]
    return w


def wave_flume(nx=48, ny=4, nz=24, wave_t=1, precision=PREC_FP64, dt=2e-4, esp_type=1) -> Case:
    """A wave flume: still water 1 m deep (waves_coef's h0_f) in a 6 x 0.5 x
    1.5 m box, waves entering through the prescribed inflow face (ccx0 = 3,
    boundary_waves, 3_contorno.f90:1189-1319) and absorbed by the sponge
    layer over the last metre (esp_type 1) before the free outflow at x = 6 m
    (ccxf = 4).  The wave's net inflow makes the all-Neumann pressure
    equation incompatible, as upstream: the reference's absolute stopping
    test (1e-4) ends each solve at the compatible part."""
    h = 6.0 / nx
    p = default_params(nx=nx, ny=ny, nz=nz, dx=h, dy=0.5 / ny, dz=1.5 / nz, dt=dt,
                       ccx0=3, ccxf=4, ccy0=1, ccyf=1, ccz0=1, cczf=1, gz=9.80665,
                       uinicial=0.0, iturb=0.0, reinit_max_iter=3, cg_tol_mode=CG_TOL_ABS, cg_tol=1e-4,
                       precision=precision)
    p.esp_type = esp_type
    set_waves(p, wave_t)
    z = _centres(nz, p.dz)[None, None, :]
    ls = np.empty((nx, ny, nz), order="F")
    ls[...] = p.h0_f - z
    return Case("wave_flume_s%d_%dx%dx%d" % (wave_t, nx, ny, nz), p, _base_fields(p, ls), steps=2000)
