"""ctypes mirror of include/suli_gpu.h (structs, ids, field shapes).

The shapes follow the reference allocations in SuLi-IC/0_modules.f90:121-347:
every array keeps its Fortran lower/upper bounds and column-major order.
"""
from __future__ import annotations

import ctypes as C

SULI_OK = 0
SULI_CG_MAXITER = 1
SULI_VOL_LOOP_CAP = 2
SULI_DEVICE_TIMEOUT = 3
SULI_BAD_CONFIG = 4
SULI_BAD_ARG = 5
SULI_CUDA_ERROR = 6
SULI_NO_DEVICE = 7
SULI_OUT_OF_MEMORY = 8
SULI_CG_STALLED = 9
SULI_NONFINITE = 10

PREC_FP64 = 0
PREC_MIXED = 1
CG_TOL_ABS = 0
CG_TOL_REL = 1


class SuliParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
        ("dx", C.c_double), ("dy", C.c_double), ("dz", C.c_double),
        ("dt", C.c_double),
        ("t_tempo", C.c_int32), ("der", C.c_int32), ("adv_type", C.c_int32),
        ("ibm_t", C.c_int32), ("obst_t", C.c_int32), ("m_turb", C.c_int32),
        ("t_press", C.c_int32), ("mms_t", C.c_int32),
        ("ccx0", C.c_int32), ("ccxf", C.c_int32), ("ccy0", C.c_int32),
        ("ccyf", C.c_int32), ("ccz0", C.c_int32), ("cczf", C.c_int32),
        ("gx", C.c_double), ("gz", C.c_double),
        ("csmag", C.c_double),
        ("alpha1", C.c_double),
        ("rho_f1", C.c_double), ("mu_f1", C.c_double),
        ("rho_f2", C.c_double), ("mu_f2", C.c_double),
        ("uinicial", C.c_double), ("iturb", C.c_double),
        ("omp_t", C.c_int32),
        ("reinit_max_iter", C.c_int32),
        ("cg_max_iter", C.c_int32),
        ("cg_tol_mode", C.c_int32),
        ("cg_tol", C.c_double),
        ("precision", C.c_int32),
        ("project_under_mms", C.c_int32),
        ("vol_loop_max", C.c_int32),
        ("mixed_precond", C.c_int32),
        ("seed", C.c_uint64),
        ("t_tens", C.c_int32),
        ("sigma", C.c_double),
        ("cmu", C.c_double),
        ("cdes", C.c_double),
        ("lcar", C.c_double),
        ("esp_type", C.c_int32),
        ("wave_t", C.c_int32),
        ("a_w", C.c_double),
        ("f_w", C.c_double),
        ("n_w", C.c_double),
        ("h0_f", C.c_double),
        ("aeta", C.c_double * 5),
        ("avel", C.c_double * 5),
        ("outflow_flux", C.c_int32),
        ("dz_t", C.c_int32),
        ("dzmin", C.c_double),
        ("dzmax", C.c_double),
    ]

    def copy(self) -> "SuliParams":
        out = SuliParams()
        C.pointer(out)[0] = self
        return out

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class SuliDiag(C.Structure):
    _fields_ = [
        ("vol_ini", C.c_double), ("vol_ins", C.c_double),
        ("maxdiv", C.c_double), ("t", C.c_double),
        ("cg_res", C.c_double * 3),
        ("cg_iters", C.c_int32 * 3),
        ("cg_outer", C.c_int32 * 3),
        ("reinit_iters", C.c_int32),
        ("vol_loops", C.c_int32),
        ("it", C.c_int32),
        ("status_flags", C.c_int32),
    ]


class SuliTuning(C.Structure):
    """suli_tuning: the autotuner's launch shapes and the timed gain."""
    _fields_ = [("convdiff_planes", C.c_int32), ("mg_block_cells", C.c_int32),
                ("sweep_blocks_per_sm", C.c_int32), ("tuned", C.c_int32),
                ("default_ms", C.c_double), ("tuned_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


def default_params(**kw) -> SuliParams:
    """Reference defaults (00_suli3d.prm / 2_iniciais.f90) plus build knobs."""
    p = SuliParams()
    p.t_tempo = 2
    p.der = 3
    p.adv_type = 1
    p.t_press = 1
    p.ccx0 = p.ccxf = p.ccy0 = p.ccyf = p.ccz0 = p.cczf = 1
    p.gx = 0.0
    p.gz = 9.80665
    p.csmag = 0.13
    p.alpha1 = 1.5
    p.rho_f1, p.mu_f1 = 1.204, 0.000018253
    p.rho_f2, p.mu_f2 = 998.0, 0.00100798
    p.omp_t = 1
    p.reinit_max_iter = 3
    p.cg_max_iter = 10000
    p.cg_tol_mode = CG_TOL_ABS
    p.cg_tol = 1e-4
    p.precision = PREC_FP64
    p.vol_loop_max = 1000
    p.t_tens = 0
    p.sigma = 0.0728
    p.cmu = 0.05
    p.cdes = 0.65
    p.lcar = 0.05715
    p.esp_type = 0
    p.wave_t = 0
    p.mixed_precond = 1
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError(f"suli_params has no field {k!r}")
        setattr(p, k, v)
    return p


# field ids, in the order of enum suli_field
FIELDS = [
    "U", "V", "W", "PRD1", "PRD", "LS", "HS", "RHO", "LS_MU", "MU", "MUT",
    "XMU", "YMU", "ZMU", "FU", "FV", "FW", "U0", "V0", "W0", "FU0", "FV0",
    "FW0", "FU1", "FV1", "FW1", "DIV", "TF_U", "TF_V", "TF_W",
    "OBS_LSX", "OBS_LSY", "OBS_LSZ", "OBS_LSS",
    "ID_IBMX", "ID_IBMY", "ID_IBMZ", "ID_IBM",
    "BXX0", "BXX1", "BLX1", "OBS_LS", "HSX", "HSY", "HSZ", "KURV",
    "KA", "NUT", "PRD0", "PX", "PY", "PZ", "BXZ0",
]
FIELD_ID = {name: i for i, name in enumerate(FIELDS)}
INT_FIELDS = {"ID_IBMX", "ID_IBMY", "ID_IBMZ", "ID_IBM"}

SCALARS = ["T", "DT", "VOL_INI", "VOL_INS", "MAXDIV", "IT", "TT", "RNG"]
SCALAR_ID = {name: i for i, name in enumerate(SCALARS)}


def field_bounds(p: SuliParams, name: str):
    """(lo, hi) Fortran bounds of a field, as in 0_modules.f90."""
    nx, ny, nz = p.nx, p.ny, p.nz
    nx1, ny1, nz1 = nx + 1, ny + 1, nz + 1
    xface = ((1, 1, 1), (nx1, ny, nz))
    yface = ((1, 1, 1), (nx, ny1, nz))
    zface = ((1, 1, 1), (nx, ny, nz1))
    cell = ((1, 1, 1), (nx, ny, nz))
    table = {
        "U": ((0, 0, 0), (nx1 + 1, ny + 1, nz + 1)),
        "V": ((0, 0, 0), (nx + 1, ny1 + 1, nz + 1)),
        "W": ((0, 0, 0), (nx + 1, ny + 1, nz1 + 1)),
        "PRD1": ((0, 0, 0), (nx + 1, ny + 1, nz + 1)),
        "PRD": ((0, 0, 0), (nx + 1, ny + 1, nz + 1)),
        "KA": ((0, 0, 0), (nx + 1, ny + 1, nz + 1)),
        "PRD0": ((0, 0, 0), (nx + 1, ny + 1, nz + 1)),
        "BXX0": ((0, 0, 0), (ny + 1, nz + 1, 0)),
        "BXX1": ((0, 0, 0), (ny + 1, nz + 1, 0)),
        "BXZ0": ((0, 0, 0), (ny + 1, nz + 1, 0)),
        "BLX1": ((1, 1, 0), (ny, nz, 0)),
        "OBS_LS": ((1, 1, 1), (nx1, ny1, nz1)),
    }
    if name in table:
        return table[name]
    if name in ("LS", "HS", "RHO", "LS_MU", "MU", "MUT", "DIV", "OBS_LSS", "ID_IBM", "HSX", "HSY", "HSZ", "KURV",
                "NUT"):
        return cell
    if name in ("XMU", "FU", "U0", "FU0", "FU1", "TF_U", "OBS_LSX", "ID_IBMX", "PX"):
        return xface
    if name in ("YMU", "FV", "V0", "FV0", "FV1", "TF_V", "OBS_LSY", "ID_IBMY", "PY"):
        return yface
    if name in ("ZMU", "FW", "W0", "FW0", "FW1", "TF_W", "OBS_LSZ", "ID_IBMZ", "PZ"):
        return zface
    raise KeyError(name)


def field_shape(p: SuliParams, name: str):
    """numpy shape (Fortran order: pass order='F') of a field."""
    lo, hi = field_bounds(p, name)
    return tuple(h - l + 1 for l, h in zip(lo, hi))
