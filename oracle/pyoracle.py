"""ctypes binding of the CPU oracle (test infrastructure only).

Loads oracle/_build/libsuli_oracle.so (built by oracle/Makefile or
__graft_entry__.build()).  Only tests/, __graft_entry__.smoke() and the
cpu-baseline / --impl reference legs of bench.py import this module; the
suli_gb300 package never does.

Parity: pinned against outputs of the reference itself (golden vectors of
its own Fortran routines, tests/golden/; bit for bit) and by analytic
known-answer tests (see oracle/suli_oracle.h).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from suli_gb300._abi import (FIELD_ID, INT_FIELDS, SCALAR_ID, SuliDiag,
                             SuliParams, field_shape)

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libsuli_oracle.so")
_lib = None


def build_oracle(force: bool = False) -> str:
    src = os.path.join(_HERE, "suli_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", _HERE])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = C.CDLL(_LIB_PATH)
        L.or_create.restype = C.c_void_p
        L.or_create.argtypes = [C.POINTER(SuliParams)]
        L.or_destroy.argtypes = [C.c_void_p]
        L.or_field.restype = C.c_void_p
        L.or_field.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.or_set_scalar.argtypes = [C.c_void_p, C.c_int, C.c_double]
        L.or_get_scalar.restype = C.c_double
        L.or_get_scalar.argtypes = [C.c_void_p, C.c_int]
        L.or_level_set_ini.argtypes = [C.c_void_p, C.c_int] + [C.c_double] * 5
        for name in ("or_heaviside_init", "or_iniciais_velocity", "or_mms_init", "or_termo_fonte1",
                     "or_ibm_setup", "or_level_set", "or_visco", "or_convdiff", "or_complementos",
                     "or_tempo", "or_posdin", "or_step", "or_exp_press", "or_contorno_les",
                     "or_boundary_waves"):
            getattr(L, name).argtypes = [C.c_void_p]
            getattr(L, name).restype = None
        L.or_obstaculo_cylinder.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
        L.or_contorno.argtypes = [C.c_void_p, C.c_int]
        L.or_graddin.argtypes = [C.c_void_p]
        L.or_graddin.restype = C.c_int
        L.or_conmassa.argtypes = [C.c_void_p]
        L.or_conmassa.restype = C.c_double
        L.or_prtscr_write.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
        L.or_prtscr_write.restype = C.c_int
        L.or_mms_error.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        L.or_set_stage.argtypes = [C.c_void_p, C.c_int]
        L.or_diag.argtypes = [C.c_void_p, C.POINTER(SuliDiag)]
        L.or_set_replay.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_int]
        L.or_set_threads.argtypes = [C.c_int]
        L.or_weno_line.argtypes = [C.POINTER(C.c_double), C.c_long, C.c_int, C.c_double, C.c_int,
                                   C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib = L
    return _lib


def weno_line(a: np.ndarray, h: float, ihs: int):
    """WENO5 (phi+, phi-) of a 1-D line, 8_derivadas.f90:675-811."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    dp = np.zeros_like(a)
    dn = np.zeros_like(a)
    P = C.POINTER(C.c_double)
    lib().or_weno_line(a.ctypes.data_as(P), 1, a.size, h, ihs, dp.ctypes.data_as(P), dn.ctypes.data_as(P))
    return dp, dn


class Oracle:
    """One reference case on the CPU, fields exposed as numpy views."""

    def __init__(self, params: SuliParams):
        self.p = params.copy()
        self._h = lib().or_create(C.byref(self.p))
        if not self._h:
            raise RuntimeError("or_create failed")

    def close(self):
        if self._h:
            lib().or_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def field(self, name: str) -> np.ndarray:
        """Writable Fortran-ordered view of the oracle's array."""
        lo = (C.c_int * 3)()
        hi = (C.c_int * 3)()
        ptr = lib().or_field(self._h, FIELD_ID[name], lo, hi)
        shape = field_shape(self.p, name)
        ctype = C.c_int32 if name in INT_FIELDS else C.c_double
        n = int(np.prod(shape))
        buf = (ctype * n).from_address(ptr)
        arr = np.frombuffer(buf, dtype=np.int32 if name in INT_FIELDS else np.float64)
        return arr.reshape(shape, order="F")

    def set_field(self, name: str, value):
        self.field(name)[...] = value

    def scalar(self, name: str) -> float:
        return lib().or_get_scalar(self._h, SCALAR_ID[name])

    def set_scalar(self, name: str, v: float):
        lib().or_set_scalar(self._h, SCALAR_ID[name], float(v))

    # initial conditions
    def level_set_ini(self, tipo, ampl=0.0, lambdax=0.0, lambday=0.0, prof=0.0, m=30.0):
        lib().or_level_set_ini(self._h, tipo, ampl, lambdax, lambday, prof, m)

    def heaviside_init(self):
        lib().or_heaviside_init(self._h)

    def iniciais_velocity(self):
        lib().or_iniciais_velocity(self._h)

    def mms_init(self):
        lib().or_mms_init(self._h)

    def termo_fonte1(self):
        lib().or_termo_fonte1(self._h)

    def obstaculo_cylinder(self, xc, yc, radius):
        lib().or_obstaculo_cylinder(self._h, xc, yc, radius)

    def ibm_setup(self):
        lib().or_ibm_setup(self._h)

    # hot path
    def level_set(self):
        lib().or_level_set(self._h)

    def contorno(self, nlock):
        lib().or_contorno(self._h, nlock)

    def visco(self):
        lib().or_visco(self._h)

    def convdiff(self):
        lib().or_convdiff(self._h)

    def complementos(self):
        lib().or_complementos(self._h)

    def tempo(self):
        lib().or_tempo(self._h)

    def graddin(self) -> int:
        return lib().or_graddin(self._h)

    def posdin(self):
        lib().or_posdin(self._h)

    def exp_press(self):
        lib().or_exp_press(self._h)

    def contorno_les(self):
        lib().or_contorno_les(self._h)

    def boundary_waves(self):
        lib().or_boundary_waves(self._h)

    def conmassa(self) -> float:
        return lib().or_conmassa(self._h)

    def prtscr_write(self, path: str, t_plot: int = 0):
        """The PRTSCR field record (4_plot.f90:547-615) as a Fortran
        unformatted file."""
        if lib().or_prtscr_write(self._h, str(path).encode(), int(t_plot)) != 0:
            raise OSError("or_prtscr_write failed for %s" % path)

    def mms_error(self):
        e = (C.c_double * 4)()
        lib().or_mms_error(self._h, e)
        return list(e)

    def set_stage(self, tt):
        lib().or_set_stage(self._h, tt)

    def step(self, n: int = 1):
        for _ in range(n):
            lib().or_step(self._h)

    def diag(self) -> SuliDiag:
        d = SuliDiag()
        lib().or_diag(self._h, C.byref(d))
        return d

    def set_replay(self, cg_iters=None, reinit_iters=-1):
        arr = (C.c_int * 3)(*(cg_iters if cg_iters is not None else (-1, -1, -1)))
        lib().or_set_replay(self._h, arr, int(reinit_iters))

    @staticmethod
    def set_threads(n: int):
        lib().or_set_threads(int(n))
