"""Shared helpers of the parity tests: build an oracle/GPU pair on the same
initial state, copy oracle state to the GPU, compare fields."""
import numpy as np

import pyoracle

STATE_FIELDS = ["U", "V", "W", "PRD1", "PRD", "LS", "HS", "RHO", "LS_MU", "MU", "MUT", "XMU", "YMU", "ZMU",
                "FU", "FV", "FW", "U0", "V0", "W0", "FU0", "FV0", "FW0", "FU1", "FV1", "FW1",
                "TF_U", "TF_V", "TF_W", "HSX", "HSY", "HSZ", "KURV", "BXX0", "BXX1", "BXZ0", "BLX1"]


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    n = np.linalg.norm(b.ravel())
    d = np.linalg.norm((a - b).ravel())
    return d / n if n > 0 else d


def oracle_for(case, warm_steps=0):
    o = pyoracle.Oracle(case.params)
    for k, v in case.fields.items():
        o.set_field(k, v)
    if case.params.mms_t:
        o.termo_fonte1()
    if case.params.m_turb >= 2:
        o.contorno_les()             # iniciais, 2_iniciais.f90:216-235
    o.heaviside_init()
    if case.params.ibm_t == 2:
        ob = case.obstacle
        o.obstaculo_cylinder(ob["xc"], ob["yc"], ob["radius"])
        o.ibm_setup()
    for n in (1, 2, 3):
        o.contorno(n)
    for _ in range(warm_steps):
        o.step()
    return o


KEQ_FIELDS = ["KA", "NUT"]
IPA_FIELDS = ["PRD0", "PX", "PY", "PZ"]


def model_fields(p):
    """The fields of the k equation / the IPA, stored for those cases only."""
    return (KEQ_FIELDS if p.m_turb >= 2 else []) + (IPA_FIELDS if p.t_press == 2 else [])


def model_compare(p):
    """The same fields as compare() names: the IPA force as one vector (its
    y component is round-off in a y-uniform flow)."""
    return (KEQ_FIELDS if p.m_turb >= 2 else []) + (["PRD0", "pforce"] if p.t_press == 2 else [])


def copy_state(o, g, case=0):
    for name in STATE_FIELDS + model_fields(g.params[case]):
        g.upload(name, o.field(name), case=case)
    g.set_scalar("VOL_INI", o.scalar("VOL_INI"), case=case)
    g.set_scalar("VOL_INS", o.scalar("VOL_INS"), case=case)
    g.set_scalar("T", o.scalar("T"))
    g.set_scalar("IT", o.scalar("IT"))
    g.set_scalar("RNG", o.scalar("RNG"))


VECTORS = {"velocity": ("U", "V", "W"), "F": ("FU", "FV", "FW"), "visc": ("XMU", "YMU", "ZMU"),
           "pforce": ("PX", "PY", "PZ")}


def compare(o, g, names, tol, case=0):
    """Relative L2 per field; a name from VECTORS compares its components as
    one vector field (a component that is only round-off, such as v in a
    y-uniform flow, is then measured against the size of the whole field)."""
    out = {}
    for name in names:
        if name in VECTORS:
            a = np.concatenate([g.download(n, case=case).ravel() for n in VECTORS[name]])
            b = np.concatenate([o.field(n).ravel() for n in VECTORS[name]])
            out[name] = rel_l2(a, b)
        else:
            out[name] = rel_l2(g.download(name, case=case), o.field(name))
    bad = {k: v for k, v in out.items() if not v <= tol}
    assert not bad, "rel L2 above %g: %s (all: %s)" % (tol, bad, out)
    return out
