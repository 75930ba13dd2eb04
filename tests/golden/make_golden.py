"""Golden vectors from the reference itself: SuLi-IC's own Fortran routines,
executed by the Fortran-subset runner f90sub.py (this container has no
Fortran compiler), on small seeded cases, written to tests/golden/*.npz.

Each case is set up the way the reference's program starts a run
(1_principal.f90:28-55): the module parameters of parametros()
(2_iniciais.f90:11-122, set here from the case's suli_params instead of
read from 00_suli3d.prm, with the reference's own derived quantities),
init_variables1..7, the body of iniciais() (2_iniciais.f90:126-271) with the
case's initial velocity and level set in place of the generated ones,
coef_tempo, then contorno(1), (2), (3).  Each step is the body of the time
loop (1_principal.f90:69-111), followed by PLOT's CONMASSA.  After every
step the fixture keeps the fields and scalars the oracle is compared on;
some cases add PRTSCR's field records, and three more run one RK stage
routine by routine from a seeded random state.  Every subscript is
bounds-checked by the runner; the one undefined read a case may carry (the
inflow fill's ls_x(0, j, k)) is resolved as the oracle resolves it
(oob_policy).  SuLi-ICdz cases run on SuLi-ICdz's own sources.

Run from the repository root:  python tests/golden/make_golden.py [case ...]
(reads the reference's sources from REFERENCE_DIR or /root/reference).
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

import f90sub  # noqa: E402

REFROOT = os.environ.get("REFERENCE_DIR", "/root/reference")
FILES = ["0_modules.f90", "2_iniciais.f90", "3_contorno.f90", "5_viscosidade.f90", "6_convdiff.f90",
         "7_advectivo.f90", "8_derivadas.f90", "9_grad.f90", "10_pos.f90", "11_diversos.f90",
         "14_level_set.f90", "15_ibm.f90", "13_mms.f90", "4_plot.f90"]

# the fields kept per step: fixture name -> reference module array (plus
# the model's own fields, model_fields())
FIELDS = {"U": "u", "V": "v", "W": "w", "PRD1": "prd1", "LS": "ls", "HS": "hs", "RHO": "rho",
          "LS_MU": "ls_mu", "MU": "mu", "XMU": "xmu", "YMU": "ymu", "ZMU": "zmu", "DIV": "div"}
# case fields a run starts from, beyond the level set and the velocity
START = {"PRD1": "prd1", "PRD0": "prd0", "KA": "ka"}


def model_fields(p):
    f = {}
    if p.m_turb >= 2:
        f.update({"KA": "ka", "NUT": "nut"})
    if p.t_press == 2:
        f.update({"PRD0": "prd0", "PX": "px", "PY": "py", "PZ": "pz"})
    if p.t_tens == 1:
        f.update({"KURV": "kurv", "HSX": "hsx", "HSY": "hsy", "HSZ": "hsz"})
    if p.ibm_t == 2:
        f.update({"OBS_LSX": "obs_lsx", "OBS_LSY": "obs_lsy", "OBS_LSZ": "obs_lsz", "OBS_LSS": "obs_lss",
                  "ID_IBMX": "id_ibmx", "ID_IBMY": "id_ibmy", "ID_IBMZ": "id_ibmz", "ID_IBM": "id_ibm"})
    return f

# suli_params fields that are module variables of the reference under the same name
PARAMS = ["nx", "ny", "nz", "dx", "dy", "dz", "t_tempo", "der", "adv_type", "ibm_t", "obst_t", "m_turb",
          "esp_type", "wave_t", "t_press", "mms_t", "t_tens", "ccx0", "ccxf", "ccy0", "ccyf", "ccz0",
          "cczf", "csmag", "cmu", "cdes", "alpha1", "rho_f1", "mu_f1", "rho_f2", "mu_f2", "sigma",
          "uinicial", "iturb", "omp_t", "gx", "gz"]


def load_reference(tree="SuLi-IC"):
    """The hot-path files of one of the reference's programs (SuLi-IC, or
    SuLi-ICdz with its variable z spacing), translated."""
    return f90sub.load([os.path.join(REFROOT, tree, f) for f in FILES])


def call(prog, name, *args):
    return f90sub.call(prog, name, *args)


def oob_policy(p):
    """The one undefined read a case may carry, replaced by the oracle's
    documented choice: with a prescribed inflow (ccx0 = 3) contorno fills the
    plane i = 0 from ls_x(0, j, k), below the face array that starts at 1
    (3_contorno.f90:315); face 1 is taken, as the oracle and the GPU do."""
    f90sub.OOB_READS.clear()
    if p.ccx0 == 3:
        f90sub.OOB_READS["ls_x"] = lambda idx: (1,) + idx[1:] if idx[0] == 0 else idx


def setup(prog, case):
    """The reference's start of a run for `case` (see the module docstring)."""
    M = prog.M
    p = case.params
    oob_policy(p)
    dzvar = p.dz_t == 1
    for k in PARAMS:
        if dzvar and k == "dz":
            continue                # SuLi-ICdz: dz(k) comes from dz_dist
        cur = getattr(M, k)
        setattr(M, k, int(getattr(p, k)) if isinstance(cur, int) else np.float64(getattr(p, k)))
    M.numb_threads = 1
    M.dt0 = np.float64(p.dt)
    # parametros(): the derived quantities, as the reference forms them
    M.dt = M.dt0
    M.nx1, M.ny1, M.nz1 = M.nx + 1, M.ny + 1, M.nz + 1
    M.ts = 10 ** 6
    third = np.float64(1.0) / np.float64(3.0)
    if dzvar:
        # SuLi-ICdz/2_iniciais.f90:104-124
        M.dzmin, M.dzmax, M.dz_t = np.float64(p.dzmin), np.float64(p.dzmax), 1
        M.nxx, M.nyy, M.nzz = M.nx1 * 2, M.ny1 * 2, M.nz1 * 2
        call(prog, "init_disc")
        call(prog, "dz_dist")
        M.lx, M.ly = M.dx * M.nx, M.dy * M.ny
        M.lz = f90sub._fsum(M.dz.d[1:M.nz + 1])
        M.delta = f90sub._max(M.dx, M.dy, M.dza)
        M.deltai.d[...] = f90sub._rpow(M.dx * M.dy * M.dz.d, third)
    else:
        M.lx, M.ly, M.lz = M.dx * M.nx, M.dy * M.ny, M.dz * M.nz
        M.delta = f90sub._max(M.dx, M.dy, M.dz)
        M.deltai = f90sub._rpow(M.dx * M.dy * M.dz, third)
    M.tipo = 0           # no generated level set: the case's own is used
    if p.m_turb >= 2:
        # visco's characteristic length is max(prof, ampl) of the initial
        # level set's parameters (5_viscosidade.f90:103); suli_params carries
        # it as lcar
        M.prof = np.float64(p.lcar)
        M.ampl = np.float64(0.0)
    M.irest = np.float64(0.0)
    M.interv_rest = np.float64(1e30)
    for n in range(1, 8):
        call(prog, "init_variables%d" % n)
    # iniciais(), 2_iniciais.f90:165-271, with the case's initial fields
    M.t = np.float64(0.0)
    for a in ("v", "w", "prd0", "prd1", "px", "py", "pz", "ub", "vb", "wb"):
        getattr(M, a).d[...] = 0.0
    M.d_max = M.d_min = np.float64(0.0)
    for a in ("hsx", "hsy", "hsz"):
        getattr(M, a).d[...] = 0.0
    M.ls.d[...] = case.fields["LS"]
    call(prog, "level_set_ini")
    for name in ("U", "V", "W"):
        getattr(M, name.lower()).d[...] = case.fields[name]
    for name, arr in START.items():
        if name in case.fields:
            getattr(M, arr).d[...] = case.fields[name]
    if M.m_turb >= 2:
        call(prog, "contorno_les")
    if M.ibm_t == 2:
        # the reference's obstacles are not cylinders: the case's obstacle
        # level sets go in where obstaculo() samples its sub-grid, then the
        # rest of obstaculo()'s ibm_t = 2 branch (3_contorno.f90:991-1003)
        for name in ("OBS_LS", "OBS_LSX", "OBS_LSY", "OBS_LSZ", "OBS_LSS"):
            getattr(M, name.lower()).d[...] = case.fields[name]
        nx, ny, nz, nx1, ny1, nz1 = M.nx, M.ny, M.nz, M.nx1, M.ny1, M.nz1
        call(prog, "reinic_weno", M.obs_ls, nx1, ny1, nz1)
        call(prog, "reinic_weno", M.obs_lsx, nx1, ny, nz)
        call(prog, "reinic_weno", M.obs_lsy, nx, ny1, nz)
        call(prog, "reinic_weno", M.obs_lsz, nx, ny, nz1)
        call(prog, "reinic_weno", M.obs_lss, nx, ny, nz)
        call(prog, "ibm_posicoes", M.id_ibmx, M.obs_lsx, nx1, ny, nz)
        call(prog, "ibm_posicoes", M.id_ibmy, M.obs_lsy, nx, ny1, nz)
        call(prog, "ibm_posicoes", M.id_ibmz, M.obs_lsz, nx, ny, nz1)
        call(prog, "ibm_posicoes", M.id_ibm, M.obs_lss, nx, ny, nz)
        mod_ls = f90sub.FArr.alloc([(1, nx), (1, ny), (1, nz)], "r")
        call(prog, "mod_ls1", M.obs_lss, mod_ls, M.norm_xx, M.norm_yy, M.norm_zz, nx, ny, nz)
    else:
        call(prog, "obstaculo")
    if M.wave_t > 0:
        call(prog, "waves_coef")
    else:
        M.bxx1.d[...] = M.uinicial
        M.bxx0.d[...] = M.uinicial
        M.bxy0.d[...] = 0.0
        M.bxz0.d[...] = 0.0
    for a in ("tf_p", "tf_u", "tf_v", "tf_w"):
        getattr(M, a).d[...] = 0.0
    M.it = 0
    M.cont = 10
    call(prog, "coef_tempo")
    for n in (1, 2, 3):
        call(prog, "contorno", n)
    if M.mms_t > 0:
        call(prog, "mms")


def step(prog):
    """One pass of the time loop's body (1_principal.f90:69-111)."""
    M = prog.M
    M.it = M.it + 1
    M.t = M.t + M.dt
    if M.mms_t == 1 and M.it == 1:
        call(prog, "termo_fonte1")
    call(prog, "level_set")
    call(prog, "contorno", 3)
    if M.t_press == 2 and M.mms_t == 0:
        call(prog, "exp_press")
    call(prog, "visco")
    for tt in range(1, M.ntt + 1):
        M.tt = tt
        M.dt = M.a_dt.d[tt - 1]
        call(prog, "convdiff")
        call(prog, "complementos")
        call(prog, "tempo")
        if M.wave_t > 0:
            call(prog, "boundary_waves")
        call(prog, "contorno", 2)
        if M.mms_t == 0:
            if M.t_press == 1:
                call(prog, "graddin")
                call(prog, "posdin")
            call(prog, "contorno", 1)
    if M.t_press == 2 and M.mms_t == 0:
        call(prog, "graddin")
    if M.mms_t > 0:
        call(prog, "mms")
    # PLOT's mass-conservation check (4_plot.f90:370-392): the divergence field
    call(prog, "conmassa")


STATIC = ("OBS_LSX", "OBS_LSY", "OBS_LSZ", "OBS_LSS", "ID_IBMX", "ID_IBMY", "ID_IBMZ", "ID_IBM")


def snapshot(prog, tag, p):
    M = prog.M
    out = {}
    for name, arr in list(FIELDS.items()) + list(model_fields(p).items()):
        if name in STATIC and tag != "s0":
            continue            # the obstacle does not change after the start
        a = getattr(M, arr)
        out["%s_%s" % (tag, name)] = np.array(a.d)
        out["lb_%s" % name] = np.array(a.l)
    for s in ("vol_ini", "vol_ins", "t", "dt"):
        out["%s_%s" % (tag, s)] = np.float64(getattr(M, s))
    return out


def sphere_tank(n=20):
    """A submerged sphere through the image-point IBM (ibm_t = 2) in a closed
    1 m cube, water below z = 0.8 m moving at 0.1 m/s, Smagorinsky LES.  The
    reference's own obstacles (obstaculo(), obst_t 1..3) and the product's
    cylinder all reach a wall, where the image stencil of ibm_images
    (15_ibm.f90:240-270) reads past its arrays (x(ii+1), id_ibm(.., kk+1)) --
    memory the Fortran does not define; an interior sphere keeps every image
    stencil inside them.  Obstacle level sets are sampled on obstaculo()'s
    half-cell sub-grid (x = (ii-1) dx/2, 3_contorno.f90:829-841) at the
    staggered points it takes them from (:905-989)."""
    from suli_gb300 import cases as C
    from suli_gb300._abi import default_params
    h = 1.0 / n
    p = default_params(nx=n, ny=n, nz=n, dx=h, dy=h, dz=h, dt=5e-4, ccx0=1, ccxf=1, ccy0=1, ccyf=1,
                       ccz0=2, cczf=1, gz=9.80665, m_turb=1, csmag=0.1, uinicial=0.1, ibm_t=2, obst_t=4)
    z = (np.arange(1, n + 1) - 0.5) * h
    ls = np.empty((n, n, n), order="F")
    ls[...] = 0.8 - z[None, None, :]
    f = C._base_fields(p, ls)
    xc, yc, zc, rad = 0.5, 0.5, 0.4, 0.15

    def field(ni, nj, nk, fi, fj, fk):
        i = np.arange(1, ni + 1)[:, None, None]
        j = np.arange(1, nj + 1)[None, :, None]
        k = np.arange(1, nk + 1)[None, None, :]
        x = (fi(i) - 1.0) * h * 0.5
        y = (fj(j) - 1.0) * h * 0.5
        zz = (fk(k) - 1.0) * h * 0.5
        out = np.empty((ni, nj, nk), order="F")
        out[...] = rad - np.sqrt((x - xc) * (x - xc) + (y - yc) * (y - yc) + (zz - zc) * (zz - zc))
        return out

    odd, even = (lambda a: 2 * a - 1), (lambda a: 2 * a)
    f.update({"OBS_LSX": field(n + 1, n, n, odd, even, even), "OBS_LSY": field(n, n + 1, n, even, odd, even),
              "OBS_LSZ": field(n, n, n + 1, even, even, odd), "OBS_LSS": field(n, n, n, even, even, even),
              "OBS_LS": field(n + 1, n + 1, n + 1, odd, odd, odd)})
    return C.Case("sphere_ibm_les_%d" % n, p, f, steps=2, obstacle={"kind": "fields"})


def oracle_setup(case):
    """The oracle started as tests/helpers.oracle_for does, the obstacle
    level sets of a "fields" obstacle taken as uploaded (reinitialised and
    marked by the oracle's obstaculo() tail)."""
    import pyoracle
    if not (case.obstacle and case.obstacle.get("kind") == "fields"):
        from helpers import oracle_for
        return oracle_for(case)
    o = pyoracle.Oracle(case.params)
    for k, v in case.fields.items():
        o.set_field(k, v)
    o.heaviside_init()
    o.ibm_setup()
    for n in (1, 2, 3):
        o.contorno(n)
    return o


def cases():
    from suli_gb300 import cases as C
    from suli_gb300._abi import CG_TOL_ABS

    def ref_defaults(c):
        # the reference's fixed choices: CG stop r.r <= 1e-4 / N (absolute) or
        # 10000 iterations (9_grad.f90:393-398), three reinitialisation
        # iterations (14_level_set.f90:389), serial sums (omp_t = 0)
        c.params.cg_tol_mode = CG_TOL_ABS
        c.params.cg_tol = 1e-4
        c.params.cg_max_iter = 10000
        c.params.reinit_max_iter = 3
        c.params.omp_t = 0
        return c

    kles = C.k_channel(16, 4, 8, m_turb=2)
    kdes = C.k_channel(16, 4, 8, m_turb=3)
    smag = C.k_channel(16, 4, 8, m_turb=2)
    smag.params.m_turb = 1
    del smag.fields["KA"]
    schemes = []
    for tt, nm in ((0, "euler"), (1, "rk2"), (3, "ab2"), (4, "ab3")):
        c = ref_defaults(C.dam_break(12, 6, 6))
        c.params.t_tempo = tt
        schemes.append(("dam_break_%s_12x6x6" % nm, c, 3))
    return [("dam_break_12x6x6", ref_defaults(C.dam_break(12, 6, 6)), 2)] + schemes + [
            ("sphere_ibm_les_20", ref_defaults(sphere_tank(20)), 1),
            ("dam_break_dz_12x6x8", ref_defaults(C.dam_break_dz(12, 6, 8)), 2),
            ("wave_flume_stokes1_16x4x8", ref_defaults(C.wave_flume(16, 4, 8, wave_t=1)), 1),
            ("wave_flume_stokes2_16x4x8", ref_defaults(C.wave_flume(16, 4, 8, wave_t=2)), 1),
            ("wave_flume_stokes5_16x4x8", ref_defaults(C.wave_flume(16, 4, 8, wave_t=5)), 1),
            ("wave_tank_les_16x4x8", ref_defaults(C.wave_tank(16, 4, 8, dt=5e-4)), 2),
            ("channel_smagorinsky_16x4x8", ref_defaults(smag), 2),
            ("channel_keq_les_16x4x8", ref_defaults(kles), 2),
            ("channel_keq_des_16x4x8", ref_defaults(kdes), 2),
            ("ipa_tank_12x4x8", ref_defaults(C.ipa_tank(12, 4, 8)), 2),
            ("capillary_16x4", ref_defaults(C.capillary_column(16, 4, 0.25)), 2),
            ("sponge1_16x4x8", ref_defaults(C.sponge_tank(16, 4, 8, esp_type=1)), 2),
            ("sponge2_16x4x8", ref_defaults(C.sponge_tank(16, 4, 8, esp_type=2)), 2)]


# routine by routine from a seeded random state: every routine of the RK
# stage on velocities of both signs everywhere (all upwind branches, every
# boundary plane); (routine, args, fields compared after it)
SEQUENCE = [("contorno", (1,), ("U", "V", "W", "PRD1")),
            ("visco", (), ("MU", "XMU", "YMU", "ZMU")),
            ("convdiff", (), ("FU", "FV", "FW")),
            ("complementos", (), ("FU", "FV", "FW")),
            ("tempo", (), ("U", "V", "W")),
            ("contorno", (2,), ("U", "V", "W")),
            ("posdin", (), ("U", "V", "W"))]
ARR = {"U": "u", "V": "v", "W": "w", "PRD1": "prd1", "MU": "mu", "XMU": "xmu", "YMU": "ymu", "ZMU": "zmu",
       "FU": "fu", "FV": "fv", "FW": "fw"}


def random_state(case, seed):
    """Seeded random velocities (both signs, ghosts included) and pressure in
    the case's own array shapes."""
    rng = np.random.default_rng(seed)
    out = {}
    for name in ("U", "V", "W", "PRD1"):
        a = case.fields[name] if name in case.fields else None
        shape = a.shape if a is not None else None
        if shape is None:
            from suli_gb300 import cases as C
            shape = C._zeros(case.params, name).shape
        scale = 0.3 if name != "PRD1" else 50.0
        out[name] = np.asfortranarray(scale * rng.standard_normal(shape))
    return out


def routine_cases():
    from suli_gb300 import cases as C
    smag = C.k_channel(16, 4, 8, m_turb=2)
    smag.params.m_turb = 1
    del smag.fields["KA"]
    return [("routines_channel_les_16x4x8", smag, 11),
            ("routines_dam_break_12x6x6", C.dam_break(12, 6, 6), 12),
            ("routines_wave_flume_16x4x8", C.wave_flume(16, 4, 8, wave_t=1), 13)]


def run_routines(prog, case, seed):
    setup(prog, case)
    M = prog.M
    rs = random_state(case, seed)
    data = {"in_%s" % k: v for k, v in rs.items()}
    for k, v in rs.items():
        getattr(M, ARR[k]).d[...] = v
    M.it = 1
    M.t = M.t + M.dt
    M.tt = 1
    M.dt = M.a_dt.d[0]
    for q, (name, args, fields) in enumerate(SEQUENCE):
        call(prog, name, *args)
        for f in fields:
            data["r%d_%s" % (q, f)] = np.array(getattr(M, ARR[f]).d)
    return data


# cases whose final state is also written by PRTSCR (4_plot.f90:501-620)
PRTSCR_CASES = ("dam_break_12x6x6", "channel_keq_les_16x4x8")


def prtscr_records(prog):
    """The field records PRTSCR writes for t_plot = 0 and 1 (each an
    unformatted sequential record: length, data, length), as bytes."""
    M = prog.M
    out = {}
    saved = M.t_plot
    M.dt_frame = np.float64(0.0)        # every call writes a frame
    for tp in (0, 1):
        M.t_plot = tp
        f90sub.FILES.clear()
        call(prog, "prtscr")
        (unit, recs), = f90sub.FILES.items()
        assert len(recs) == 1, recs
        out["prtscr%d" % tp] = np.frombuffer(recs[0], dtype=np.uint8).copy()
    M.t_plot = saved
    return out


def main():
    t0 = time.time()
    prog = load_reference()
    print("translated %d subroutines in %.1f s" % (len(prog.units), time.time() - t0), flush=True)
    only = set(sys.argv[1:])            # optional: the case names to (re)generate
    for name, case, nsteps in cases():
        if only and name not in only:
            continue
        prog = load_reference("SuLi-ICdz" if case.params.dz_t == 1 else "SuLi-IC")   # fresh state per case
        setup(prog, case)
        data = snapshot(prog, "s0", case.params)
        for s in range(1, nsteps + 1):
            t1 = time.time()
            step(prog)
            data.update(snapshot(prog, "s%d" % s, case.params))
            print("%s step %d: %.1f s" % (name, s, time.time() - t1), flush=True)
        data["steps"] = np.int64(nsteps)
        if name in PRTSCR_CASES:
            data.update(prtscr_records(prog))
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **data)
        print("wrote", path, os.path.getsize(path), "bytes", flush=True)
    for name, case, seed in routine_cases():
        if only and name not in only:
            continue
        prog = load_reference()
        data = run_routines(prog, case, seed)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **data)
        print("wrote", path, os.path.getsize(path), "bytes", flush=True)


if __name__ == "__main__":
    main()
