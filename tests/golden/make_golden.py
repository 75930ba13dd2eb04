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
loop (1_principal.f90:69-111).  After every step the fixture keeps the
fields and scalars the oracle is compared on.

Run from the repository root:  python tests/golden/make_golden.py
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

REF = os.path.join(os.environ.get("REFERENCE_DIR", "/root/reference"), "SuLi-IC")
FILES = ["0_modules.f90", "2_iniciais.f90", "3_contorno.f90", "5_viscosidade.f90", "6_convdiff.f90",
         "7_advectivo.f90", "8_derivadas.f90", "9_grad.f90", "10_pos.f90", "11_diversos.f90",
         "14_level_set.f90", "15_ibm.f90", "13_mms.f90"]

# the fields kept per step: fixture name -> reference module array (plus
# the model's own fields, model_fields())
FIELDS = {"U": "u", "V": "v", "W": "w", "PRD1": "prd1", "LS": "ls", "HS": "hs", "RHO": "rho",
          "LS_MU": "ls_mu", "MU": "mu", "XMU": "xmu", "YMU": "ymu", "ZMU": "zmu"}
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
    return f

# suli_params fields that are module variables of the reference under the same name
PARAMS = ["nx", "ny", "nz", "dx", "dy", "dz", "t_tempo", "der", "adv_type", "ibm_t", "obst_t", "m_turb",
          "esp_type", "wave_t", "t_press", "mms_t", "t_tens", "ccx0", "ccxf", "ccy0", "ccyf", "ccz0",
          "cczf", "csmag", "cmu", "cdes", "alpha1", "rho_f1", "mu_f1", "rho_f2", "mu_f2", "sigma",
          "uinicial", "iturb", "omp_t", "gx", "gz"]


def load_reference():
    return f90sub.load([os.path.join(REF, f) for f in FILES])


def call(prog, name, *args):
    return f90sub.call(prog, name, *args)


def setup(prog, case):
    """The reference's start of a run for `case` (see the module docstring)."""
    M = prog.M
    p = case.params
    for k in PARAMS:
        cur = getattr(M, k)
        setattr(M, k, int(getattr(p, k)) if isinstance(cur, int) else np.float64(getattr(p, k)))
    M.numb_threads = 1
    M.dt0 = np.float64(p.dt)
    # parametros(): the derived quantities, as the reference forms them
    M.dt = M.dt0
    M.lx, M.ly, M.lz = M.dx * M.nx, M.dy * M.ny, M.dz * M.nz
    M.nx1, M.ny1, M.nz1 = M.nx + 1, M.ny + 1, M.nz + 1
    M.ts = 10 ** 6
    M.delta = f90sub._max(M.dx, M.dy, M.dz)
    M.deltai = f90sub._rpow(M.dx * M.dy * M.dz, np.float64(1.0) / np.float64(3.0))
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
    call(prog, "obstaculo")
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


def step(prog):
    """One pass of the time loop's body (1_principal.f90:69-111)."""
    M = prog.M
    M.it = M.it + 1
    M.t = M.t + M.dt
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


def snapshot(prog, tag, p):
    M = prog.M
    out = {}
    for name, arr in list(FIELDS.items()) + list(model_fields(p).items()):
        a = getattr(M, arr)
        out["%s_%s" % (tag, name)] = np.array(a.d)
        out["lb_%s" % name] = np.array(a.l)
    for s in ("vol_ini", "vol_ins", "t", "dt"):
        out["%s_%s" % (tag, s)] = np.float64(getattr(M, s))
    return out


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
    return [("dam_break_12x6x6", ref_defaults(C.dam_break(12, 6, 6)), 2),
            ("wave_tank_les_16x4x8", ref_defaults(C.wave_tank(16, 4, 8, dt=5e-4)), 2),
            ("channel_smagorinsky_16x4x8", ref_defaults(smag), 2),
            ("channel_keq_les_16x4x8", ref_defaults(kles), 2),
            ("channel_keq_des_16x4x8", ref_defaults(kdes), 2),
            ("ipa_tank_12x4x8", ref_defaults(C.ipa_tank(12, 4, 8)), 2),
            ("capillary_16x4", ref_defaults(C.capillary_column(16, 4, 0.25)), 2),
            ("sponge1_16x4x8", ref_defaults(C.sponge_tank(16, 4, 8, esp_type=1)), 2),
            ("sponge2_16x4x8", ref_defaults(C.sponge_tank(16, 4, 8, esp_type=2)), 2)]


def main():
    t0 = time.time()
    prog = load_reference()
    print("translated %d subroutines in %.1f s" % (len(prog.units), time.time() - t0), flush=True)
    for name, case, nsteps in cases():
        prog = load_reference()         # fresh module state per case
        setup(prog, case)
        data = snapshot(prog, "s0", case.params)
        for s in range(1, nsteps + 1):
            t1 = time.time()
            step(prog)
            data.update(snapshot(prog, "s%d" % s, case.params))
            print("%s step %d: %.1f s" % (name, s, time.time() - t1), flush=True)
        data["steps"] = np.int64(nsteps)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **data)
        print("wrote", path, os.path.getsize(path), "bytes", flush=True)


if __name__ == "__main__":
    main()
