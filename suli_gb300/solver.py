"""Host-side interface of the GPU hot path (ctypes over libsuli_gpu.so).

Mirrors the reference's subroutine interface: one method per hot routine
(level_set, contorno, visco, convdiff, complementos, tempo, graddin, posdin,
conmassa), plus step() for the whole body of the time loop of
SuLi-IC/1_principal.f90:69-124.  Errors come back as SuliError carrying the
library's status code and message; there is no CPU fallback -- if
libsuli_gpu.so or a CUDA device is missing, construction fails.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ._abi import (FIELD_ID, INT_FIELDS, SCALAR_ID, SULI_CG_MAXITER, SuliDiag,
                   SuliParams, SuliTuning, field_shape)

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libsuli_gpu.so")

# every entry point declared in include/suli_gpu.h
EXPORTS = [
    "suli_default_params", "suli_field_shape", "suli_create", "suli_create_batch", "suli_num_cases",
    "suli_destroy", "suli_upload_field", "suli_download_field", "suli_set_scalar", "suli_get_scalar",
    "suli_set_replay", "suli_heaviside_init", "suli_level_set", "suli_contorno", "suli_visco",
    "suli_convdiff", "suli_complementos", "suli_tempo", "suli_graddin", "suli_posdin", "suli_conmassa",
    "suli_mms_error", "suli_set_stage", "suli_step", "suli_diagnostics", "suli_synchronize",
    "suli_last_error", "suli_device_info", "suli_get_stream", "suli_profile", "suli_profile_read",
    "suli_ibm_setup", "suli_conmassa_noalloc", "suli_time_kernel", "suli_upload_fields",
    "suli_download_fields", "suli_write_fields", "suli_restart_save", "suli_restart_load",
    "suli_exp_press", "suli_contorno_les", "suli_boundary_waves", "suli_autotune", "suli_get_tuning",
]


class SuliProfile(C.Structure):
    _fields_ = [("launches", C.c_uint64), ("cg_ms", C.c_double), ("cg_cell_iters", C.c_double),
                ("cg_bytes_per_cell_iter", C.c_double)]

_lib = None


class SuliError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("suli status %d: %s" % (code, msg))
        self.code = code


def load_library(path: str = LIB_PATH):
    """Load libsuli_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libsuli_gpu.so not built (%s); run __graft_entry__.build()" % path)
    L = C.CDLL(path)
    P = C.POINTER
    i32 = C.c_int32
    L.suli_default_params.argtypes = [P(SuliParams)]
    L.suli_default_params.restype = None
    L.suli_field_shape.argtypes = [P(SuliParams), C.c_int, P(C.c_int), P(C.c_int)]
    L.suli_create.argtypes = [P(SuliParams), P(C.c_void_p)]
    L.suli_create_batch.argtypes = [P(SuliParams), C.c_int, P(C.c_void_p)]
    L.suli_num_cases.argtypes = [C.c_void_p, P(C.c_int)]
    L.suli_destroy.argtypes = [C.c_void_p]
    L.suli_upload_field.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    L.suli_download_field.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p]
    L.suli_set_scalar.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double]
    L.suli_get_scalar.argtypes = [C.c_void_p, C.c_int, C.c_int, P(C.c_double)]
    L.suli_set_replay.argtypes = [C.c_void_p, P(i32), i32]
    for name in ("suli_heaviside_init", "suli_ibm_setup", "suli_level_set", "suli_visco", "suli_convdiff",
                 "suli_complementos", "suli_tempo", "suli_posdin", "suli_synchronize", "suli_exp_press",
                 "suli_contorno_les", "suli_boundary_waves"):
        getattr(L, name).argtypes = [C.c_void_p]
    L.suli_contorno.argtypes = [C.c_void_p, C.c_int]
    L.suli_graddin.argtypes = [C.c_void_p, P(i32)]
    L.suli_conmassa.argtypes = [C.c_void_p, P(C.c_double)]
    L.suli_mms_error.argtypes = [C.c_void_p, P(C.c_double)]
    L.suli_set_stage.argtypes = [C.c_void_p, C.c_int]
    L.suli_step.argtypes = [C.c_void_p, C.c_int]
    L.suli_diagnostics.argtypes = [C.c_void_p, C.c_int, P(SuliDiag)]
    L.suli_last_error.argtypes = [C.c_char_p, C.c_size_t]
    L.suli_device_info.argtypes = [P(C.c_int), C.c_char_p, C.c_size_t]
    L.suli_get_stream.argtypes = [C.c_void_p, P(C.c_void_p)]
    L.suli_profile.argtypes = [C.c_void_p, C.c_int]
    L.suli_profile_read.argtypes = [C.c_void_p, P(SuliProfile)]
    L.suli_upload_fields.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    L.suli_download_fields.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    L.suli_time_kernel.argtypes = [C.c_void_p, C.c_int, C.c_int, P(C.c_double), P(C.c_double)]
    L.suli_write_fields.argtypes = [C.c_void_p, C.c_int, C.c_char_p, C.c_int]
    L.suli_restart_save.argtypes = [C.c_void_p, C.c_char_p]
    L.suli_restart_load.argtypes = [C.c_void_p, C.c_char_p]
    L.suli_conmassa_noalloc.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, i32, i32, i32, C.c_double,
                                        C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    L.suli_autotune.argtypes = [C.c_void_p, P(SuliTuning)]
    L.suli_get_tuning.argtypes = [C.c_void_p, P(SuliTuning)]
    _lib = L
    return L


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    load_library().suli_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def _check(rc: int, allow=()):
    if rc != 0 and rc not in allow:
        raise SuliError(rc, last_error())
    return rc


def device_info():
    n = C.c_int(0)
    name = C.create_string_buffer(256)
    _check(load_library().suli_device_info(C.byref(n), name, len(name)))
    return n.value, name.value.decode()


class SuliGPU:
    """A batch of device-resident cases (one case = the Fortran drop-in)."""

    def __init__(self, params):
        if isinstance(params, SuliParams):
            params = [params]
        self.params = [p.copy() for p in params]
        L = load_library()
        arr = (SuliParams * len(self.params))(*self.params)
        h = C.c_void_p()
        _check(L.suli_create_batch(arr, len(self.params), C.byref(h)))
        self._h = h
        self.warnings = 0

    @property
    def ncases(self):
        return len(self.params)

    def close(self):
        if getattr(self, "_h", None):
            load_library().suli_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- fields ---------------------------------------------------------
    def upload(self, name: str, arr, case: int = 0):
        p = self.params[case]
        dt = np.int32 if name in INT_FIELDS else np.float64
        a = np.asfortranarray(np.asarray(arr, dtype=dt).reshape(field_shape(p, name), order="F"))
        _check(load_library().suli_upload_field(self._h, case, FIELD_ID[name], a.ctypes.data))

    def download(self, name: str, case: int = 0) -> np.ndarray:
        p = self.params[case]
        dt = np.int32 if name in INT_FIELDS else np.float64
        a = np.zeros(field_shape(p, name), dtype=dt, order="F")
        _check(load_library().suli_download_field(self._h, case, FIELD_ID[name], a.ctypes.data))
        return a

    def _batch(self, items, up):
        """items: (field name, case, array) with each array already in the
        field's Fortran-order shape and dtype (it is used in place, so a
        pinned buffer stays pinned)."""
        n = len(items)
        cases = (C.c_int32 * n)()
        fields = (C.c_int32 * n)()
        ptrs = (C.c_void_p * n)()
        for q, (name, case, a) in enumerate(items):
            p = self.params[case]
            dt = np.int32 if name in INT_FIELDS else np.float64
            if a.dtype != dt or tuple(a.shape) != tuple(field_shape(p, name)) or not a.flags.f_contiguous:
                raise ValueError("%s of case %d: need a Fortran-order %s array of shape %s"
                                 % (name, case, np.dtype(dt).name, field_shape(p, name)))
            cases[q] = case
            fields[q] = FIELD_ID[name]
            ptrs[q] = a.ctypes.data
        fn = load_library().suli_upload_fields if up else load_library().suli_download_fields
        _check(fn(self._h, n, cases, fields, ptrs))

    def upload_many(self, items):
        """Upload (field name, case, array) triples in one call (one sync)."""
        self._batch(items, True)

    def download_many(self, items):
        """Download into (field name, case, array) triples in one call."""
        self._batch(items, False)

    def scalar(self, name: str, case: int = 0) -> float:
        v = C.c_double()
        _check(load_library().suli_get_scalar(self._h, case, SCALAR_ID[name], C.byref(v)))
        return v.value

    def set_scalar(self, name: str, value: float, case: int = 0):
        _check(load_library().suli_set_scalar(self._h, case, SCALAR_ID[name], float(value)))

    def set_replay(self, cg_iters=None, reinit_iters=-1):
        arr = (C.c_int32 * 3)(*(cg_iters if cg_iters is not None else (-1, -1, -1)))
        _check(load_library().suli_set_replay(self._h, arr, int(reinit_iters)))

    # ---- reference routines ---------------------------------------------------
    def heaviside_init(self):
        _check(load_library().suli_heaviside_init(self._h))

    def ibm_setup(self):
        _check(load_library().suli_ibm_setup(self._h))

    def level_set(self):
        _check(load_library().suli_level_set(self._h))

    def contorno(self, nlock: int):
        _check(load_library().suli_contorno(self._h, nlock))

    def visco(self):
        _check(load_library().suli_visco(self._h))

    def convdiff(self):
        _check(load_library().suli_convdiff(self._h))

    def complementos(self):
        _check(load_library().suli_complementos(self._h))

    def tempo(self):
        _check(load_library().suli_tempo(self._h))

    def set_stage(self, tt: int):
        _check(load_library().suli_set_stage(self._h, tt))

    def graddin(self) -> int:
        it = C.c_int32()
        rc = _check(load_library().suli_graddin(self._h, C.byref(it)), allow=(SULI_CG_MAXITER,))
        if rc:
            self.warnings |= 1 << rc
        return it.value

    def posdin(self):
        _check(load_library().suli_posdin(self._h))

    def exp_press(self):
        """exp_press (11_diversos.f90:455-495), t_press = 2."""
        _check(load_library().suli_exp_press(self._h))

    def contorno_les(self):
        """contorno_les (3_contorno.f90:666-790) on the m_turb >= 2 cases."""
        _check(load_library().suli_contorno_les(self._h))

    def boundary_waves(self):
        """boundary_waves (3_contorno.f90:1189-1319) on the wave_t > 0 cases."""
        _check(load_library().suli_boundary_waves(self._h))

    def conmassa(self) -> float:
        m = C.c_double()
        _check(load_library().suli_conmassa(self._h, C.byref(m)))
        return m.value

    def mms_error(self):
        e = (C.c_double * 4)()
        _check(load_library().suli_mms_error(self._h, e))
        return list(e)

    def step(self, n: int = 1):
        _check(load_library().suli_step(self._h, int(n)))

    def synchronize(self):
        _check(load_library().suli_synchronize(self._h))

    def stream_handle(self) -> int:
        """The cudaStream_t all of this handle's kernels run on."""
        p = C.c_void_p()
        _check(load_library().suli_get_stream(self._h, C.byref(p)))
        return p.value or 0

    def profile(self, enable: bool = True):
        _check(load_library().suli_profile(self._h, 1 if enable else 0))

    def profile_read(self) -> SuliProfile:
        out = SuliProfile()
        _check(load_library().suli_profile_read(self._h, C.byref(out)))
        return out

    def time_kernel(self, kernel: int, reps: int = 20):
        """(ms per launch, algorithmic bytes per launch) of one kernel timed
        alone over every case: 0 CG matrix-vector product, 1 multigrid
        smoother half-sweep on the case grid, 2 CG direction update."""
        ms, by = C.c_double(), C.c_double()
        _check(load_library().suli_time_kernel(self._h, kernel, reps, C.byref(ms), C.byref(by)))
        return ms.value, by.value

    # ---- autotuner -------------------------------------------------------------
    def autotune(self) -> dict:
        """Tune the launch shapes now (or apply the cached choice for this
        device and workload shape); returns suli_tuning as a dict."""
        t = SuliTuning()
        _check(load_library().suli_autotune(self._h, C.byref(t)))
        return t.as_dict()

    def tuning(self) -> dict:
        t = SuliTuning()
        _check(load_library().suli_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    # ---- output and restart --------------------------------------------------
    def write_fields(self, path, case: int = 0, t_plot: int = 0):
        """PRTSCR's field record of one case (4_plot.f90:501-635) as a
        Fortran unformatted file at `path`."""
        _check(load_library().suli_write_fields(self._h, case, str(path).encode(), int(t_plot)))

    def restart_save(self, path):
        """Every field, t, it and the counters of the batch (restart_salva)."""
        _check(load_library().suli_restart_save(self._h, str(path).encode()))

    def restart_load(self, path):
        """Restore a restart_save file into this handle (restart_ini, with t
        and it kept)."""
        _check(load_library().suli_restart_load(self._h, str(path).encode()))

    def diag(self, case: int = 0) -> SuliDiag:
        d = SuliDiag()
        _check(load_library().suli_diagnostics(self._h, case, C.byref(d)))
        return d

    # ---- set-up ------------------------------------------------------------
    def start(self, fields_per_case):
        """Upload initial fields and run the start-up of 1_principal.f90:50-53:
        heaviside + vol_ini, then contorno(1), (2), (3); with the k equation
        (m_turb >= 2) first the ghost values of ka, as iniciais does
        (2_iniciais.f90:216-235)."""
        if isinstance(fields_per_case, dict):
            fields_per_case = [fields_per_case]
        for c, fields in enumerate(fields_per_case):
            for name, arr in fields.items():
                self.upload(name, arr, case=c)
        if any(p.m_turb >= 2 for p in self.params):
            self.contorno_les()
        self.heaviside_init()
        if any(p.ibm_t == 2 for p in self.params):
            self.ibm_setup()          # obstaculo(): reinit obstacle level sets, image masks
        for n in (1, 2, 3):
            self.contorno(n)
